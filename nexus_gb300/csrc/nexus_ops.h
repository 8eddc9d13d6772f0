// NEXUS's operators on the GB300 engine: the CKKSEvaluator primitives of
// src/ckks_evaluator.{h,cpp} and GeLUEvaluator / SoftmaxEvaluator /
// LNEvaluator (src/gelu.cpp, src/softmax.cpp, src/layer_norm.cpp) with the
// same class and method names, arguments, defaults and scale bookkeeping, so
// they produce SEAL's output words for the same keys and inputs.
#pragma once
#include <utility>
#include <vector>

#include "ckks.h"

namespace nexus {

class CKKSEvaluator {
public:
    // constants of src/ckks_evaluator.h:14-27
    std::vector<double> F4_COEFFS = {0, 315, 0, -420, 0, 378, 0, -180, 0, 35};
    int f4_scale = (1 << 7);
    std::vector<double> G4_COEFFS = {0, 5850, 0, -34974, 0, 97015, 0, -113492, 0, 46623};
    int g4_scale = (1 << 10);

    Evaluator *evaluator;
    double scale;
    size_t slot_count;
    size_t degree;

    CKKSEvaluator(Evaluator &ev, double scale);

    std::vector<double> init_vec_with_value(size_t n, double value) const { return std::vector<double>(n, value); }
    uint64_t get_modulus(const Ciphertext &x, int k) const;
    void eval_odd_deg9_poly(const std::vector<double> &a, Ciphertext &x, Ciphertext &dest);

    Ciphertext sgn_eval(Ciphertext x, int d_g, int d_f, double sgn_factor = 0.5);
    Ciphertext invert_sqrt(Ciphertext x, int d_newt = 5, int d_gold = 2);
    Ciphertext exp(Ciphertext x);
    Ciphertext inverse(Ciphertext x, int iter = 4);

    Ciphertext newtonIter(Ciphertext x, Ciphertext res, int iter = 4);
    std::pair<Ciphertext, Ciphertext> goldSchmidtIter(Ciphertext v, Ciphertext y, int d = 1);
    Ciphertext initGuess(Ciphertext x);
    Ciphertext evalLine(Ciphertext x, Plaintext m, Plaintext c);
};

class GeLUEvaluator {
public:
    explicit GeLUEvaluator(CKKSEvaluator &ckks) : ckks(&ckks) {}
    void gelu(Ciphertext &x, Ciphertext &res);

private:
    CKKSEvaluator *ckks;
};
using GELUEvaluator = GeLUEvaluator;  // name of the CUDA build (cuda/src/gelu.cuh)

class SoftmaxEvaluator {
public:
    explicit SoftmaxEvaluator(CKKSEvaluator &ckks) : ckks(&ckks) {}
    void softmax(Ciphertext &x, Ciphertext &res, int len);

private:
    CKKSEvaluator *ckks;
};

class LNEvaluator {
public:
    explicit LNEvaluator(CKKSEvaluator &ckks) : ckks(&ckks) {}
    void layer_norm(Ciphertext &x, Ciphertext &res, int len);

private:
    CKKSEvaluator *ckks;
};

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
