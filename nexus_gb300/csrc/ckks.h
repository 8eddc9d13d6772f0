// C++ host layer over the engine's kernels: ciphertext / plaintext objects in
// device memory and an evaluator with SEAL's semantics (scale bookkeeping,
// level dropping, NAF rotations, the same error conditions), so NEXUS's
// operators can be written against it call for call.
//
// Levels are identified by their number of data limbs (SEAL's parms_id).
// Every operation is enqueued on the evaluator's stream; device memory comes
// from the stream-ordered allocator (cudaMallocAsync pool).
#pragma once
#include <complex>
#include <cstdint>
#include <map>
#include <tuple>
#include <utility>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "context.h"

namespace nexus {

class Encoder;

// Device buffer owned by one object, freed stream-ordered.
class DeviceBuffer {
public:
    DeviceBuffer() = default;
    ~DeviceBuffer() { release(); }
    DeviceBuffer(const DeviceBuffer &) = delete;
    DeviceBuffer &operator=(const DeviceBuffer &) = delete;
    DeviceBuffer(DeviceBuffer &&o) noexcept { swap(o); }
    DeviceBuffer &operator=(DeviceBuffer &&o) noexcept
    {
        if (this != &o) {
            release();
            swap(o);
        }
        return *this;
    }
    void reserve(size_t words, cudaStream_t s);
    void release();
    uint64_t *get() const { return p_; }
    size_t capacity() const { return words_; }
    cudaStream_t stream() const { return s_; }
    // true while a CUDA-graph capture is under way on this buffer's stream
    // and the buffer was allocated outside it: the capture may read and
    // write it but cannot free it (a graph frees only its own allocations)
    bool predates_capture() const;

private:
    void swap(DeviceBuffer &o) noexcept
    {
        std::swap(p_, o.p_);
        std::swap(words_, o.words_);
        std::swap(s_, o.s_);
        std::swap(cap_, o.cap_);
    }
    uint64_t *p_ = nullptr;
    size_t words_ = 0;
    cudaStream_t s_ = nullptr;
    unsigned long long cap_ = 0;   // id of the capture the buffer was allocated in, 0 outside any
};

class Ciphertext {
public:
    Ciphertext() = default;
    Ciphertext(const Ciphertext &o);
    Ciphertext &operator=(const Ciphertext &o);
    Ciphertext(Ciphertext &&) noexcept = default;
    // Takes o's words.  Outside a graph capture this moves o's buffer in.
    // While a capture is under way on this ciphertext's stream and its
    // buffer was allocated before the capture (a caller's handle), the
    // buffer is kept and o's words are copied into it when they fit, so an
    // in-place operation on a captured input leaves the handle's memory in
    // place for the caller to reload before each launch.
    Ciphertext &operator=(Ciphertext &&o) noexcept;

    // allocate for size x limbs (contents undefined)
    void resize(const Context &c, int size, int limbs, cudaStream_t s);
    uint64_t *data() const { return buf_.get(); }
    uint64_t *poly(int i) const { return buf_.get() + (size_t)i * limbs_ * n_; }
    int size() const { return size_; }
    int limbs() const { return limbs_; }
    size_t n() const { return n_; }
    double &scale() { return scale_; }
    double scale() const { return scale_; }
    cudaStream_t stream() const { return s_; }
    bool empty() const { return size_ == 0; }

private:
    DeviceBuffer buf_;
    int size_ = 0, limbs_ = 0;
    size_t n_ = 0;
    double scale_ = 1.0;
    cudaStream_t s_ = nullptr;
};

// A vector-encoded plaintext lives on the device ([limbs][N], NTT form); a
// scalar-encoded one (SEAL's encode(double)) is one residue per limb, which
// SEAL stores in every coefficient of its NTT form.
class Plaintext {
public:
    Plaintext() = default;
    Plaintext(const Plaintext &o);
    Plaintext &operator=(const Plaintext &o);
    Plaintext(Plaintext &&) noexcept = default;
    Plaintext &operator=(Plaintext &&) noexcept = default;
    bool is_scalar() const { return scalar_; }
    int limbs() const { return limbs_; }
    double &scale() { return scale_; }
    double scale() const { return scale_; }
    const uint64_t *data() const { return buf_.get(); }
    const std::vector<uint64_t> &residues() const { return res_; }

    void set_scalar(std::vector<uint64_t> r, double scale);
    void set_vector(const Context &c, int limbs, double scale, cudaStream_t s);  // allocates; caller fills data
    uint64_t *mutable_data() { return buf_.get(); }
    // keep the first `limbs` limbs (mod_switch_to for a plaintext)
    void drop_to(int limbs, cudaStream_t s, const Context &c);

private:
    bool scalar_ = true;
    int limbs_ = 0;
    double scale_ = 1.0;
    std::vector<uint64_t> res_;
    DeviceBuffer buf_;
    size_t n_ = 0;
    cudaStream_t s_ = nullptr;
};

class Evaluator {
public:
    Evaluator(Context &c, cudaStream_t s = nullptr);
    ~Evaluator();
    Context &context() { return c_; }
    cudaStream_t stream() const { return s_; }
    void set_stream(cudaStream_t s)
    {
        s_ = s;
        const_cache_.clear();   // cached encodings are copied on the stream they were made on
        const_cache_words_ = 0;
        monomials_.clear();
    }
    size_t slot_count() const { return c_.n / 2; }
    int top_limbs() const { return c_.k - 1; }
    uint64_t modulus(int i) const { return c_.q[i]; }

    // keys (device pointers owned by the caller, SEAL layout [K-1][2][K][N])
    const uint64_t *relin_key = nullptr;
    std::map<uint32_t, const uint64_t *> galois_keys;
    // set (or replace) the key of a Galois element; drops the element's
    // hoisting data, which is derived from the key
    void set_galois_key(uint32_t elt, const uint64_t *key);

    // CKKSEncoder
    void encode(const std::vector<double> &values, int limbs, double scale, Plaintext &out);
    void encode(double value, int limbs, double scale, Plaintext &out);  // scalar path
    void encode(double value, double scale, Plaintext &out) { encode(value, top_limbs(), scale, out); }
    void encode(const std::vector<std::complex<double>> &values, int limbs, double scale, Plaintext &out);
    // outs[i] = encode(*values[i], limbs, scale): the host FFTs run on up to
    // `threads` threads (0: every core), then one upload and NTT per plaintext
    void encode_many(const std::vector<const std::vector<std::complex<double>> *> &values, int limbs, double scale,
                     const std::vector<Plaintext *> &outs, unsigned threads = 0);
    // SEAL's encode(..., scale) at the top level followed by mod_switch_to(limbs)
    void encode_then_drop(const std::vector<std::complex<double>> &values, int limbs, double scale, Plaintext &out);
    void encode_then_drop(double value, int limbs, double scale, Plaintext &out);
    std::vector<double> decode(const Plaintext &pt);

    // level management
    void mod_switch_to_inplace(Ciphertext &ct, int limbs);
    void mod_switch_to_inplace(Plaintext &pt, int limbs);
    void mod_switch_to_next_inplace(Ciphertext &ct) { mod_switch_to_inplace(ct, ct.limbs() - 1); }
    void rescale_to_next_inplace(Ciphertext &ct);

    // arithmetic
    void multiply_inplace(Ciphertext &a, const Ciphertext &b);
    void multiply(const Ciphertext &a, const Ciphertext &b, Ciphertext &dest);
    void square_inplace(Ciphertext &a) { multiply_inplace(a, a); }
    void square(const Ciphertext &a, Ciphertext &dest) { multiply(a, a, dest); }
    void relinearize_inplace(Ciphertext &ct);
    void add_inplace(Ciphertext &a, const Ciphertext &b);
    void add(const Ciphertext &a, const Ciphertext &b, Ciphertext &dest);
    void sub_inplace(Ciphertext &a, const Ciphertext &b);
    void sub(const Ciphertext &a, const Ciphertext &b, Ciphertext &dest);
    void negate_inplace(Ciphertext &a);
    void negate(const Ciphertext &a, Ciphertext &dest);
    void add_plain_inplace(Ciphertext &ct, const Plaintext &pt);
    void add_plain(const Ciphertext &ct, const Plaintext &pt, Ciphertext &dest);
    void sub_plain_inplace(Ciphertext &ct, const Plaintext &pt);
    void sub_plain(const Ciphertext &ct, const Plaintext &pt, Ciphertext &dest);
    void multiply_plain_inplace(Ciphertext &ct, const Plaintext &pt);
    void multiply_plain(const Ciphertext &ct, const Plaintext &pt, Ciphertext &dest);
    // sum_j multiply_plain(cts[j], pts[j]) for size-2 ciphertexts at one level,
    // as repeated add_inplace_reduced_error of the products does at one
    // level (the result takes the last product's scale); one fused kernel
    void multiply_plain_accumulate(const std::vector<const Ciphertext *> &cts,
                                   const std::vector<const Plaintext *> &pts, Ciphertext &dest);

    // constant / vector ops of the bootstrapping fork of SEAL (evaluator.cpp:395-418)
    void add_const_inplace(Ciphertext &ct, double value);
    void multiply_const_inplace(Ciphertext &ct, double value);
    void multiply_const(const Ciphertext &ct, double value, Ciphertext &dest);
    // multiply_const then rescale_to_next_inplace, same words and checks, with
    // the constant applied inside the rescale; set_scale > 0 replaces the
    // product's scale before the rescale (as the reduced-error level matching does)
    void multiply_const_rescale(const Ciphertext &ct, double value, Ciphertext &dest, double set_scale = 0.0);
    // multiply_const_rescale(x, value, tmp) then add_inplace_reduced_error(acc, tmp)
    void multiply_const_rescale_add(const Ciphertext &x, double value, Ciphertext &acc);
    void multiply_vector_inplace_reduced_error(Ciphertext &ct, const std::vector<std::complex<double>> &values);
    void multiply_vector_reduced_error(const Ciphertext &ct, const std::vector<std::complex<double>> &values,
                                       Ciphertext &dest);
    // reduced-error level matching (Kim et al., CT-RSA'22; evaluator.cpp:420-590)
    void add_inplace_reduced_error(Ciphertext &a, const Ciphertext &b);
    void sub_inplace_reduced_error(Ciphertext &a, const Ciphertext &b);
    void multiply_inplace_reduced_error(Ciphertext &a, const Ciphertext &b);
    void add_reduced_error(const Ciphertext &a, const Ciphertext &b, Ciphertext &dest);
    void sub_reduced_error(const Ciphertext &a, const Ciphertext &b, Ciphertext &dest);
    void multiply_reduced_error(const Ciphertext &a, const Ciphertext &b, Ciphertext &dest);
    void double_inplace(Ciphertext &ct) { add_inplace(ct, ct); }

    // rotations
    void apply_galois_inplace(Ciphertext &ct, uint32_t elt);
    void rotate_vector_inplace(Ciphertext &ct, int steps);
    void rotate_vector(const Ciphertext &ct, int steps, Ciphertext &dest);
    void complex_conjugate_inplace(Ciphertext &ct);
    // the NTT form of the monomial X^power at `limbs` limbs, scale 1 (made
    // once per evaluator, then cached): multiply_plain by it multiplies the
    // message by X^power exactly and leaves the scale and level as they are
    const Plaintext &monomial(int power, int limbs);
    uint32_t galois_elt(int step) const;
    // outs[i] = rotate_vector(ct, steps[i]) for every i, word for word; the
    // steps that have their own Galois key share one ModUp of c1 (hoisted
    // rotations, ops.h) when that is exact.  ct must not be one of outs.
    void rotate_vector_many(const Ciphertext &ct, const std::vector<int> &steps, std::vector<Ciphertext> &outs);

    // Hoisting data of a Galois element, built on first use and kept until
    // its key is replaced: the key with its rows permuted (the size of the
    // key) and, per level, a [2][limbs+1][N] correction.
    const uint64_t *hoist_key(uint32_t elt);
    const uint64_t *hoist_corr(uint32_t elt, int limbs);
    // count device ints for hoist_decompose's per-ciphertext zero flags
    int *hoist_flags(int count);
    // hoisting pays when at least two rotations share the decomposition and
    // the level is high enough for the ModUp to dominate the key switch
    static bool hoist_pays(int direct_steps, int limbs) { return direct_steps >= 2 && limbs >= 8; }
    // hoisting on (default) or off; off, or when its data cannot be
    // allocated, every step is switched on its own (the same words)
    bool hoisting = true;
    // the permuted keys and corrections for these rotations, or false when
    // they cannot be allocated (the allocation error is cleared)
    bool hoist_prepare(const std::vector<uint32_t> &elts, int limbs);

    int total_bits(int limbs) const;
    // is_scale_within_bounds (evaluator.cpp:29-47)
    void check_scale(double scale, int limbs) const;

private:
    void plain_arith(Ciphertext &ct, const Plaintext &pt, bool sub);
    // the scale adjustment shared by the *_reduced_error ops: bring the higher
    // ciphertext `hi` down to lo's level at lo's scale
    Ciphertext adjust_down(const Ciphertext &hi, const Ciphertext &lo);
    Context &c_;
    cudaStream_t s_;
    Encoder *enc_ = nullptr;
    std::vector<int> bits_;
    std::map<uint32_t, DeviceBuffer> hoist_keys_, hoist_masks_;
    std::map<std::pair<uint32_t, int>, DeviceBuffer> hoist_corrs_;
    DeviceBuffer hoist_flag_;
    // Encodings of constant vectors (every slot the same value), the kind of
    // vector NEXUS's operators encode on every call: the first encode of a
    // (value, slot count, limbs, scale, form) runs the FFT and the upload,
    // later ones copy the cached device words.  Encoding is a pure function
    // of those, so the words are the same; it also keeps repeated operator
    // calls free of host waits, so they can be captured in a CUDA graph.
    struct ConstKey {
        uint64_t re, im, scale;
        size_t count;
        int limbs, form;   // form 0: encode, 1: encode_then_drop
        bool operator<(const ConstKey &o) const
        {
            return std::tie(re, im, scale, count, limbs, form) < std::tie(o.re, o.im, o.scale, o.count, o.limbs, o.form);
        }
    };
    bool const_lookup(const ConstKey &k, Plaintext &out) const;
    void const_store(const ConstKey &k, const Plaintext &pt);
    std::map<ConstKey, Plaintext> const_cache_;
    size_t const_cache_words_ = 0;
    std::map<std::pair<int, int>, Plaintext> monomials_;
};

bool are_close(double a, double b);
std::vector<int> naf(int value);

}  // namespace nexus
