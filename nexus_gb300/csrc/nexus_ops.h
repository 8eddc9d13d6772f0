// NEXUS's operators on the GB300 engine: the CKKSEvaluator primitives of
// src/ckks_evaluator.{h,cpp} and GeLUEvaluator / SoftmaxEvaluator /
// LNEvaluator (src/gelu.cpp, src/softmax.cpp, src/layer_norm.cpp) with the
// same class and method names, arguments, defaults and scale bookkeeping, so
// they produce SEAL's output words for the same keys and inputs.
#pragma once
#include <utility>
#include <vector>

#include "batch.h"
#include "ckks.h"

namespace nexus {

// EV / CT: Evaluator / Ciphertext, or BatchEvaluator / CtBatch to run the
// same operator on several ciphertexts in lockstep (one launch per step for
// the whole batch); the call sequence is NEXUS's in both cases.
template <class EV, class CT>
class CKKSEvaluatorT {
public:
    // constants of src/ckks_evaluator.h:14-27
    std::vector<double> F4_COEFFS = {0, 315, 0, -420, 0, 378, 0, -180, 0, 35};
    int f4_scale = (1 << 7);
    std::vector<double> G4_COEFFS = {0, 5850, 0, -34974, 0, 97015, 0, -113492, 0, 46623};
    int g4_scale = (1 << 10);

    EV *evaluator;
    double scale;
    size_t slot_count;
    size_t degree;

    CKKSEvaluatorT(EV &ev, double scale);

    std::vector<double> init_vec_with_value(size_t n, double value) const { return std::vector<double>(n, value); }
    uint64_t get_modulus(const CT &x, int k) const;
    void eval_odd_deg9_poly(const std::vector<double> &a, CT &x, CT &dest);

    CT sgn_eval(CT x, int d_g, int d_f, double sgn_factor = 0.5);
    CT invert_sqrt(CT x, int d_newt = 5, int d_gold = 2);
    CT exp(CT x);
    CT inverse(CT x, int iter = 4);

    CT newtonIter(CT x, CT res, int iter = 4);
    std::pair<CT, CT> goldSchmidtIter(CT v, CT y, int d = 1);
    CT initGuess(CT x);
    CT evalLine(CT x, Plaintext m, Plaintext c);
};

template <class EV, class CT>
class GeLUEvaluatorT {
public:
    explicit GeLUEvaluatorT(CKKSEvaluatorT<EV, CT> &ckks) : ckks(&ckks) {}
    void gelu(CT &x, CT &res);

private:
    CKKSEvaluatorT<EV, CT> *ckks;
};

template <class EV, class CT>
class SoftmaxEvaluatorT {
public:
    explicit SoftmaxEvaluatorT(CKKSEvaluatorT<EV, CT> &ckks) : ckks(&ckks) {}
    void softmax(CT &x, CT &res, int len);

private:
    CKKSEvaluatorT<EV, CT> *ckks;
};

template <class EV, class CT>
class LNEvaluatorT {
public:
    explicit LNEvaluatorT(CKKSEvaluatorT<EV, CT> &ckks) : ckks(&ckks) {}
    void layer_norm(CT &x, CT &res, int len);

private:
    CKKSEvaluatorT<EV, CT> *ckks;
};

using CKKSEvaluator = CKKSEvaluatorT<Evaluator, Ciphertext>;
using GeLUEvaluator = GeLUEvaluatorT<Evaluator, Ciphertext>;
using GELUEvaluator = GeLUEvaluator;  // name of the CUDA build (cuda/src/gelu.cuh)
using SoftmaxEvaluator = SoftmaxEvaluatorT<Evaluator, Ciphertext>;
using LNEvaluator = LNEvaluatorT<Evaluator, Ciphertext>;

// MMEvaluator (src/matrix_mul.{h,cpp}): ct x pt MatMul through the ciphertext
// expansion tree; see matmul.cu for the GPU form.
class MMEvaluator {
public:
    explicit MMEvaluator(CKKSEvaluator &ckks);
    std::vector<uint32_t> rots;  // ckks->rots: Galois elements (N + 2^i) / 2^i

    void multiply_power_of_x(Ciphertext &encrypted, Ciphertext &destination, int index);
    std::vector<Ciphertext> expand_ciphertext(const Ciphertext &encrypted, uint32_t m);
    // res[r] = sum_k leaf(r*cols + k) * pts[k] over the expanded compressed
    // ciphertexts, scale *= factor, rescaled to one prime
    void matrix_mul(const std::vector<Ciphertext> &compressed, const std::vector<Plaintext> &pts, int rows, int cols,
                    double factor, std::vector<Ciphertext> &res, int subtree_depth = 6);
    // the same with the plaintexts already stacked on the device, d_pts[cols][l][N] at pt_scale
    void matrix_mul(const std::vector<const Ciphertext *> &compressed, const uint64_t *d_pts, double pt_scale,
                    int rows, int cols, double factor, std::vector<Ciphertext> &res, int subtree_depth = 6);
    // optional bias: res[r] += encode(bias) at the output level and scale
    void add_bias(std::vector<Ciphertext> &res, const std::vector<double> &bias);

private:
    const uint64_t *key_for(uint32_t elt) const;
    CKKSEvaluator *ckks;
};

}  // namespace nexus
