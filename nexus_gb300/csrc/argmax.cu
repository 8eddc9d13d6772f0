// ArgmaxEvaluator on the engine (src/argmax.cpp:9-81).
#include <cmath>

#include "argmax.h"

namespace nexus {

template <class EV, class CT>
void ArgmaxEvaluatorT<EV, CT>::argmax(CT &x, CT &res, int len)
{
    EV &ev = *ckks->evaluator;
    CT tmp, a, b, sign, a_plus_b, a_minus_b, a_minus_b_sgn;
    Plaintext one, half;
    const int log_step = (int)std::log2(len);

    // x = [a_0 .. a_n, 0 ..] -> [a_0 .. a_n, a_0 .. a_n, 0 ..]
    ev.rotate_vector(x, -len, tmp);
    ev.add_inplace(x, tmp);

    a = x;
    for (int i = 0; i < log_step; ++i) {
        ev.rotate_vector(a, 1 << i, b);
        ev.add(a, b, a_plus_b);
        ev.sub(a, b, a_minus_b);
        sign = ckks->sgn_eval(a_minus_b, 2, 2);

        // (a - b) * sgn(a - b) / 2
        ev.mod_switch_to_inplace(a_minus_b, sign.limbs());
        ev.multiply(a_minus_b, sign, a_minus_b_sgn);
        ev.relinearize_inplace(a_minus_b_sgn);
        ev.rescale_to_next_inplace(a_minus_b_sgn);

        // (a + b) / 2
        ev.encode(0.5, a_plus_b.limbs(), a_plus_b.scale(), half);
        ev.multiply_plain_inplace(a_plus_b, half);
        ev.rescale_to_next_inplace(a_plus_b);

        // a = max(a, b)
        a_plus_b.scale() = a_minus_b_sgn.scale();
        ev.mod_switch_to_inplace(a_plus_b, a_minus_b_sgn.limbs());
        ev.add(a_plus_b, a_minus_b_sgn, a);

        bootstrap(a);
    }

    x.scale() = a.scale();
    ev.mod_switch_to_inplace(x, a.limbs());
    ev.sub(x, a, res);
    res = ckks->sgn_eval(res, 2, 2, 1.0);
    ev.encode(1.0, res.limbs(), res.scale(), one);
    ev.add_plain_inplace(res, one);
}

// ArgmaxEvaluator::bootstrap (src/argmax.cpp:83-106): drop to the lowest
// level, keep the scale, refresh
template <class EV, class CT>
void ArgmaxEvaluatorT<EV, CT>::bootstrap(CT &x)
{
    EV &ev = *ckks->evaluator;
    while (x.limbs() > 1) ev.mod_switch_to_next_inplace(x);
    CT x_0 = x;
    bootstrapper_->set_final_scale(x.scale());
    bootstrapper_->bootstrap_3(x, x_0);
}

template class ArgmaxEvaluatorT<Evaluator, Ciphertext>;
template class ArgmaxEvaluatorT<BatchEvaluator, CtBatch>;

}  // namespace nexus
