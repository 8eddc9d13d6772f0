// Lockstep evaluation of B ciphertexts that undergo the same operation
// sequence (the ciphertexts of one bootstrap step, of one layer's rows, ...).
//
// A CtBatch keeps B ciphertexts of one size, level and scale back to back,
// [B][size][limbs][N].  BatchEvaluator offers the Evaluator operations the
// bootstrapper uses on whole batches, each as one launch over all B
// ciphertexts; key switching reads each key once per batch
// (switch_key_batch).  Every word equals what the Evaluator computes for each
// ciphertext on its own.
#pragma once
#include <complex>
#include <vector>

#include "ckks.h"

namespace nexus {

class CtBatch {
public:
    CtBatch() = default;
    CtBatch(const CtBatch &o) { *this = o; }
    CtBatch &operator=(const CtBatch &o);
    CtBatch(CtBatch &&) noexcept = default;
    CtBatch &operator=(CtBatch &&) noexcept = default;

    // allocate for batch x size x limbs (contents undefined)
    void resize(const Context &c, int batch, int size, int limbs, cudaStream_t s);
    // same batch, new shape
    void resize(const Context &c, int size, int limbs, cudaStream_t s) { resize(c, batch_, size, limbs, s); }
    uint64_t *data() const { return buf_.get(); }
    uint64_t *ct(int b) const { return buf_.get() + (size_t)b * words_per_ct(); }
    size_t words_per_ct() const { return (size_t)size_ * limbs_ * n_; }
    int batch() const { return batch_; }
    int size() const { return size_; }
    int limbs() const { return limbs_; }
    size_t n() const { return n_; }
    double &scale() { return scale_; }
    double scale() const { return scale_; }
    bool empty() const { return size_ == 0; }

private:
    DeviceBuffer buf_;
    int batch_ = 1, size_ = 0, limbs_ = 0;
    size_t n_ = 0;
    double scale_ = 1.0;
    cudaStream_t s_ = nullptr;
};

class BatchEvaluator {
public:
    explicit BatchEvaluator(Evaluator &base) : ev_(base), c_(base.context()) {}
    Evaluator &base() { return ev_; }
    Context &context() { return c_; }
    cudaStream_t stream() const { return ev_.stream(); }
    size_t slot_count() const { return ev_.slot_count(); }
    int top_limbs() const { return ev_.top_limbs(); }
    uint64_t modulus(int i) const { return ev_.modulus(i); }

    // encoding (shared by the whole batch)
    void encode(const std::vector<std::complex<double>> &v, int limbs, double scale, Plaintext &out)
    {
        ev_.encode(v, limbs, scale, out);
    }
    void encode_then_drop(const std::vector<std::complex<double>> &v, int limbs, double scale, Plaintext &out)
    {
        ev_.encode_then_drop(v, limbs, scale, out);
    }
    void encode(const std::vector<double> &v, int limbs, double scale, Plaintext &out)
    {
        ev_.encode(v, limbs, scale, out);
    }
    void encode(double value, int limbs, double scale, Plaintext &out) { ev_.encode(value, limbs, scale, out); }
    void encode(double value, double scale, Plaintext &out) { ev_.encode(value, scale, out); }
    void mod_switch_to_inplace(Plaintext &pt, int limbs) { ev_.mod_switch_to_inplace(pt, limbs); }

    // level management
    void mod_switch_to_inplace(CtBatch &ct, int limbs);
    void mod_switch_to_next_inplace(CtBatch &ct) { mod_switch_to_inplace(ct, ct.limbs() - 1); }
    void rescale_to_next_inplace(CtBatch &ct);

    // arithmetic
    void multiply_inplace(CtBatch &a, const CtBatch &b);
    void multiply(const CtBatch &a, const CtBatch &b, CtBatch &dest);
    void square_inplace(CtBatch &a) { multiply_inplace(a, a); }
    void square(const CtBatch &a, CtBatch &dest) { multiply(a, a, dest); }
    void relinearize_inplace(CtBatch &ct);
    void add_inplace(CtBatch &a, const CtBatch &b);
    void add(const CtBatch &a, const CtBatch &b, CtBatch &dest);
    void sub_inplace(CtBatch &a, const CtBatch &b);
    void sub(const CtBatch &a, const CtBatch &b, CtBatch &dest);
    void double_inplace(CtBatch &ct) { add_inplace(ct, ct); }
    void negate_inplace(CtBatch &ct);
    void negate(const CtBatch &ct, CtBatch &dest);
    void add_plain_inplace(CtBatch &ct, const Plaintext &pt) { plain_arith(ct, pt, false); }
    void sub_plain_inplace(CtBatch &ct, const Plaintext &pt) { plain_arith(ct, pt, true); }
    void add_plain(const CtBatch &ct, const Plaintext &pt, CtBatch &dest);
    void sub_plain(const CtBatch &ct, const Plaintext &pt, CtBatch &dest);
    void multiply_plain_inplace(CtBatch &ct, const Plaintext &pt);
    void multiply_plain(const CtBatch &ct, const Plaintext &pt, CtBatch &dest);
    void multiply_plain_accumulate(const std::vector<const CtBatch *> &cts, const std::vector<const Plaintext *> &pts,
                                   CtBatch &dest);

    // fork ops
    void add_const_inplace(CtBatch &ct, double value);
    void multiply_const_inplace(CtBatch &ct, double value);
    void multiply_const(const CtBatch &ct, double value, CtBatch &dest);
    void multiply_const_rescale(const CtBatch &ct, double value, CtBatch &dest, double set_scale = 0.0);
    void multiply_const_rescale_add(const CtBatch &x, double value, CtBatch &acc);
    void multiply_vector_reduced_error(const CtBatch &ct, const std::vector<std::complex<double>> &values,
                                       CtBatch &dest);
    void add_inplace_reduced_error(CtBatch &a, const CtBatch &b);
    void sub_inplace_reduced_error(CtBatch &a, const CtBatch &b);
    void multiply_inplace_reduced_error(CtBatch &a, const CtBatch &b);
    void add_reduced_error(const CtBatch &a, const CtBatch &b, CtBatch &dest);
    void sub_reduced_error(const CtBatch &a, const CtBatch &b, CtBatch &dest);
    void multiply_reduced_error(const CtBatch &a, const CtBatch &b, CtBatch &dest);

    // rotations
    void apply_galois_inplace(CtBatch &ct, uint32_t elt);
    void rotate_vector_inplace(CtBatch &ct, int steps);
    void rotate_vector(const CtBatch &ct, int steps, CtBatch &dest);
    void complex_conjugate_inplace(CtBatch &ct) { apply_galois_inplace(ct, ev_.galois_elt(0)); }
    // outs[i] = rotate_vector(ct, steps[i]); the steps with their own key share
    // one ModUp of the batch's c1 polynomials when that is exact
    void rotate_vector_many(const CtBatch &ct, const std::vector<int> &steps, std::vector<CtBatch> &outs);

private:
    void plain_arith(CtBatch &ct, const Plaintext &pt, bool sub);
    void apply_galois(const CtBatch &ct, uint32_t elt, const uint64_t *key, CtBatch &out);
    CtBatch adjust_down(const CtBatch &hi, const CtBatch &lo);
    Evaluator &ev_;
    Context &c_;
};

}  // namespace nexus
