// ArgmaxEvaluator (src/argmax.{h,cpp}): tournament maximum over `len` slots
// with the sign polynomial and a bootstrap after every round, then the
// one-hot indicator sgn(x - max) + 1.  Same call sequence as NEXUS's.
#pragma once
#include "bootstrap.h"
#include "nexus_ops.h"

namespace nexus {

template <class EV, class CT>
class ArgmaxEvaluatorT {
public:
    CKKSEvaluatorT<EV, CT> *ckks;

    ArgmaxEvaluatorT(CKKSEvaluatorT<EV, CT> &ck, BootstrapperT<EV, CT> &bs) : ckks(&ck), bootstrapper_(&bs) {}
    void argmax(CT &x, CT &res, int len);
    void bootstrap(CT &x);

private:
    BootstrapperT<EV, CT> *bootstrapper_;
};

using ArgmaxEvaluator = ArgmaxEvaluatorT<Evaluator, Ciphertext>;

}  // namespace nexus
