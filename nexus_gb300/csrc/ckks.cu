// C++ evaluator with SEAL's semantics over the engine's kernels (see ckks.h).
// Error conditions and their messages follow SEAL's Evaluator
// (evaluator.cpp in SEAL-4.1-bs) so NEXUS's code paths fail where SEAL's do.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <string>
#include <thread>

#include "ckks.h"
#include "encoder.h"
#include "ntt.h"
#include "ops.h"

namespace nexus {

static void ck(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// ---------------------------------------------------------------- buffers

// the id of the graph capture under way on `s`, or 0 (the legacy default
// stream is never captured and is not queried)
static unsigned long long capture_id(cudaStream_t s)
{
    if (!s) return 0;
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    unsigned long long id = 0;
    if (cudaStreamGetCaptureInfo(s, &st, &id) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return st == cudaStreamCaptureStatusActive ? id : 0;
}

void DeviceBuffer::reserve(size_t words, cudaStream_t s)
{
    if (words <= words_ && p_) return;
    release();
    ck(cudaMallocAsync(&p_, words * sizeof(uint64_t), s), "cudaMallocAsync");
    words_ = words;
    s_ = s;
    cap_ = capture_id(s);
}

void DeviceBuffer::release()
{
    if (p_) cudaFreeAsync(p_, s_);
    p_ = nullptr;
    words_ = 0;
    cap_ = 0;
}

bool DeviceBuffer::predates_capture() const
{
    if (!p_) return false;
    const unsigned long long id = capture_id(s_);
    return id != 0 && id != cap_;
}

Ciphertext &Ciphertext::operator=(Ciphertext &&o) noexcept
{
    if (this == &o) return *this;
    const size_t words = (size_t)o.size_ * o.limbs_ * o.n_;
    if (o.buf_.get() && words <= buf_.capacity() && buf_.predates_capture()) {
        cudaMemcpyAsync(buf_.get(), o.buf_.get(), words * 8, cudaMemcpyDeviceToDevice, buf_.stream());
        size_ = o.size_;
        limbs_ = o.limbs_;
        n_ = o.n_;
        scale_ = o.scale_;
        o.buf_.release();
        o.size_ = o.limbs_ = 0;
        return *this;
    }
    buf_ = std::move(o.buf_);
    size_ = o.size_;
    limbs_ = o.limbs_;
    n_ = o.n_;
    scale_ = o.scale_;
    s_ = o.s_;
    return *this;
}

void Ciphertext::resize(const Context &c, int size, int limbs, cudaStream_t s)
{
    n_ = c.n;
    s_ = s;
    buf_.reserve((size_t)size * limbs * c.n, s);
    size_ = size;
    limbs_ = limbs;
}

Ciphertext::Ciphertext(const Ciphertext &o) { *this = o; }

Ciphertext &Ciphertext::operator=(const Ciphertext &o)
{
    if (this == &o) return *this;
    if (o.empty()) {
        buf_.release();
        size_ = limbs_ = 0;
        scale_ = o.scale_;
        return *this;
    }
    n_ = o.n_;
    s_ = o.s_;
    buf_.reserve((size_t)o.size_ * o.limbs_ * o.n_, s_);
    size_ = o.size_;
    limbs_ = o.limbs_;
    scale_ = o.scale_;
    ck(cudaMemcpyAsync(buf_.get(), o.buf_.get(), (size_t)size_ * limbs_ * n_ * 8, cudaMemcpyDeviceToDevice, s_),
       "copy ciphertext");
    return *this;
}

Plaintext::Plaintext(const Plaintext &o) { *this = o; }

Plaintext &Plaintext::operator=(const Plaintext &o)
{
    if (this == &o) return *this;
    scalar_ = o.scalar_;
    limbs_ = o.limbs_;
    scale_ = o.scale_;
    res_ = o.res_;
    n_ = o.n_;
    s_ = o.s_;
    if (o.scalar_ || !o.buf_.get()) {
        buf_.release();
    } else {
        buf_.reserve((size_t)limbs_ * n_, s_);
        ck(cudaMemcpyAsync(buf_.get(), o.buf_.get(), (size_t)limbs_ * n_ * 8, cudaMemcpyDeviceToDevice, s_),
           "copy plaintext");
    }
    return *this;
}

void Plaintext::set_scalar(std::vector<uint64_t> r, double scale)
{
    scalar_ = true;
    res_ = std::move(r);
    limbs_ = (int)res_.size();
    scale_ = scale;
    buf_.release();
}

void Plaintext::set_vector(const Context &c, int limbs, double scale, cudaStream_t s)
{
    scalar_ = false;
    limbs_ = limbs;
    scale_ = scale;
    res_.clear();
    n_ = c.n;
    s_ = s;
    buf_.reserve((size_t)limbs * c.n, s);
}

void Plaintext::drop_to(int limbs, cudaStream_t s, const Context &c)
{
    if (limbs > limbs_) throw std::invalid_argument("cannot switch to higher level modulus");
    if (limbs == limbs_) return;
    if (scalar_) {
        res_.resize(limbs);
    } else {
        DeviceBuffer nb;
        nb.reserve((size_t)limbs * c.n, s);
        ck(cudaMemcpyAsync(nb.get(), buf_.get(), (size_t)limbs * c.n * 8, cudaMemcpyDeviceToDevice, s), "drop limbs");
        buf_ = std::move(nb);
    }
    limbs_ = limbs;
}

// ---------------------------------------------------------------- helpers

bool are_close(double a, double b)
{
    // util::are_close (util/common.h:569-573)
    double sf = std::max(std::max(std::fabs(a), std::fabs(b)), 1.0);
    return std::fabs(a - b) < std::numeric_limits<double>::epsilon() * sf;
}

std::vector<int> naf(int value)
{
    // util::naf (util/numth.h:22-42)
    std::vector<int> res;
    bool sign = value < 0;
    value = std::abs(value);
    for (int i = 0; value; ++i) {
        int zi = (value & 1) ? 2 - (value & 3) : 0;
        value = (value - zi) >> 1;
        if (zi) res.push_back((sign ? -zi : zi) * (1 << i));
    }
    return res;
}

Evaluator::Evaluator(Context &c, cudaStream_t s) : c_(c), s_(s)
{
    enc_ = new Encoder(c);
    bits_.assign(c.k + 1, 0);
    for (int l = 1; l <= c.k; ++l) {
        // bit count of prod_{i<l} q_i (ContextData::total_coeff_modulus_bit_count)
        std::vector<uint64_t> p(l + 1, 0);
        p[0] = 1;
        for (int i = 0; i < l; ++i) {
            unsigned __int128 carry = 0;
            for (auto &w : p) {
                unsigned __int128 t = (unsigned __int128)w * c.q[i] + carry;
                w = (uint64_t)t;
                carry = t >> 64;
            }
        }
        int b = 0;
        for (int w = l; w >= 0; --w)
            if (p[w]) {
                b = w * 64 + (64 - __builtin_clzll(p[w]));
                break;
            }
        bits_[l] = b;
    }
}

Evaluator::~Evaluator() { delete enc_; }

int Evaluator::total_bits(int limbs) const { return bits_.at(limbs); }

void Evaluator::check_scale(double scale, int limbs) const
{
    // is_scale_within_bounds (evaluator.cpp:29-47)
    if (scale <= 0 || (int)std::log2(scale) >= total_bits(limbs)) throw std::invalid_argument("scale out of bounds");
}

uint32_t Evaluator::galois_elt(int step) const
{
    // GaloisTool::get_elt_from_step (util/galois.cpp:53-90)
    const uint32_t n = (uint32_t)c_.n;
    const uint64_t m = 2ull * n;
    if (step == 0) return (uint32_t)(m - 1);
    bool neg = step < 0;
    uint32_t pos = (uint32_t)std::abs(step);
    if (pos >= (n >> 1)) throw std::invalid_argument("step count too large");
    int e = neg ? (int)(n >> 1) - (int)pos : (int)pos;
    uint64_t g = 1;
    while (e--) g = (g * 5) & (m - 1);
    return (uint32_t)g;
}

// ---------------------------------------------------------------- encoding

namespace {

uint64_t bits_of(double v)
{
    uint64_t b;
    std::memcpy(&b, &v, sizeof b);
    return b;
}

// the value every entry of `v` holds, or false (empty, NaN or differing entries)
template <class T>
bool constant_value(const std::vector<T> &v, std::complex<double> &c)
{
    if (v.empty()) return false;
    for (const T &x : v)
        if (!(x == v[0])) return false;
    c = std::complex<double>(v[0]);
    return true;
}

// at most this many words (8 GiB) of cached constant encodings per evaluator
constexpr size_t kConstCacheWords = (size_t)1 << 30;

}  // namespace

bool Evaluator::const_lookup(const ConstKey &k, Plaintext &out) const
{
    auto it = const_cache_.find(k);
    if (it == const_cache_.end()) return false;
    out = it->second;
    return true;
}

void Evaluator::const_store(const ConstKey &k, const Plaintext &pt)
{
    const size_t words = (size_t)pt.limbs() * c_.n;
    if (const_cache_words_ + words > kConstCacheWords) return;
    const_cache_[k] = pt;
    const_cache_words_ += words;
}

void Evaluator::encode(const std::vector<double> &values, int limbs, double scale, Plaintext &out)
{
    if (limbs < 1 || limbs > top_limbs()) throw std::invalid_argument("parms_id is not valid for encryption parameters");
    std::complex<double> cv;
    const bool constant = constant_value(values, cv);
    const ConstKey key{bits_of(cv.real()), bits_of(cv.imag()), bits_of(scale), values.size(), limbs, 0};
    if (constant && const_lookup(key, out)) return;
    std::vector<std::complex<double>> v(values.size());
    for (size_t i = 0; i < values.size(); ++i) v[i] = values[i];
    std::vector<uint64_t> host((size_t)limbs * c_.n);
    enc_->encode(v.data(), v.size(), scale, limbs, host.data());
    out.set_vector(c_, limbs, scale, s_);
    ck(cudaMemcpyAsync(out.mutable_data(), host.data(), host.size() * 8, cudaMemcpyHostToDevice, s_), "upload");
    ck(cudaStreamSynchronize(s_), "encode");  // host buffer lifetime
    ntt_forward(c_, out.mutable_data(), 1, 0, limbs, s_);
    if (constant) const_store(key, out);
}

void Evaluator::encode(const std::vector<std::complex<double>> &values, int limbs, double scale, Plaintext &out)
{
    if (limbs < 1 || limbs > top_limbs()) throw std::invalid_argument("parms_id is not valid for encryption parameters");
    std::complex<double> cv;
    const bool constant = constant_value(values, cv);
    const ConstKey key{bits_of(cv.real()), bits_of(cv.imag()), bits_of(scale), values.size(), limbs, 0};
    if (constant && const_lookup(key, out)) return;
    std::vector<uint64_t> host((size_t)limbs * c_.n);
    enc_->encode(values.data(), values.size(), scale, limbs, host.data());
    out.set_vector(c_, limbs, scale, s_);
    ck(cudaMemcpyAsync(out.mutable_data(), host.data(), host.size() * 8, cudaMemcpyHostToDevice, s_), "upload");
    ck(cudaStreamSynchronize(s_), "encode");
    ntt_forward(c_, out.mutable_data(), 1, 0, limbs, s_);
    if (constant) const_store(key, out);
}

void Evaluator::encode_many(const std::vector<const std::vector<std::complex<double>> *> &values, int limbs,
                            double scale, const std::vector<Plaintext *> &outs, unsigned threads)
{
    if (limbs < 1 || limbs > top_limbs()) throw std::invalid_argument("parms_id is not valid for encryption parameters");
    if (values.size() != outs.size()) throw std::invalid_argument("encode_many: one output per value vector");
    const size_t m = values.size(), words = (size_t)limbs * c_.n;
    if (m == 0) return;
    if (threads == 0) threads = std::max(1u, std::thread::hardware_concurrency());
    threads = (unsigned)std::min<size_t>(threads, m);
    std::vector<uint64_t> host(m * words);
    std::vector<std::string> errors(threads);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < threads; ++t)
        th.emplace_back([&, t] {
            try {
                for (size_t i = t; i < m; i += threads)
                    enc_->encode(values[i]->data(), values[i]->size(), scale, limbs, host.data() + i * words);
            } catch (const std::exception &e) {
                errors[t] = e.what();
            }
        });
    for (auto &t : th) t.join();
    for (auto &e : errors)
        if (!e.empty()) throw std::invalid_argument(e);
    for (size_t i = 0; i < m; ++i) {
        outs[i]->set_vector(c_, limbs, scale, s_);
        ck(cudaMemcpyAsync(outs[i]->mutable_data(), host.data() + i * words, words * 8, cudaMemcpyHostToDevice, s_),
           "upload");
    }
    ck(cudaStreamSynchronize(s_), "encode");  // host buffer lifetime
    for (size_t i = 0; i < m; ++i) ntt_forward(c_, outs[i]->mutable_data(), 1, 0, limbs, s_);
}

void Evaluator::encode_then_drop(const std::vector<std::complex<double>> &values, int limbs, double scale,
                                 Plaintext &out)
{
    if (limbs < 1 || limbs > top_limbs()) throw std::invalid_argument("cannot switch to higher level modulus");
    std::complex<double> cv;
    const bool constant = constant_value(values, cv);
    const ConstKey key{bits_of(cv.real()), bits_of(cv.imag()), bits_of(scale), values.size(), limbs, 1};
    if (constant && const_lookup(key, out)) return;
    std::vector<uint64_t> host((size_t)limbs * c_.n);
    enc_->encode(values.data(), values.size(), scale, limbs, host.data(), top_limbs());
    out.set_vector(c_, limbs, scale, s_);
    ck(cudaMemcpyAsync(out.mutable_data(), host.data(), host.size() * 8, cudaMemcpyHostToDevice, s_), "upload");
    ck(cudaStreamSynchronize(s_), "encode");
    ntt_forward(c_, out.mutable_data(), 1, 0, limbs, s_);
    if (constant) const_store(key, out);
}

void Evaluator::encode_then_drop(double value, int limbs, double scale, Plaintext &out)
{
    if (limbs < 1 || limbs > top_limbs()) throw std::invalid_argument("cannot switch to higher level modulus");
    std::vector<uint64_t> r(limbs);
    enc_->encode_scalar(value, scale, limbs, r.data(), top_limbs());
    out.set_scalar(std::move(r), scale);
}

void Evaluator::encode(double value, int limbs, double scale, Plaintext &out)
{
    if (limbs < 1 || limbs > top_limbs()) throw std::invalid_argument("parms_id is not valid for encryption parameters");
    std::vector<uint64_t> r(limbs);
    enc_->encode_scalar(value, scale, limbs, r.data());
    out.set_scalar(std::move(r), scale);
}

std::vector<double> Evaluator::decode(const Plaintext &pt)
{
    if (pt.is_scalar()) throw std::invalid_argument("decode of a scalar plaintext");
    const size_t n = c_.n;
    std::vector<uint64_t> host((size_t)pt.limbs() * n);
    uint64_t *tmp = c_.get_scratch(host.size());
    ck(cudaMemcpyAsync(tmp, pt.data(), host.size() * 8, cudaMemcpyDeviceToDevice, s_), "copy");
    ntt_inverse(c_, tmp, 1, 0, pt.limbs(), s_);
    ck(cudaMemcpyAsync(host.data(), tmp, host.size() * 8, cudaMemcpyDeviceToHost, s_), "download");
    ck(cudaStreamSynchronize(s_), "decode");
    std::vector<std::complex<double>> v(n / 2);
    enc_->decode(host.data(), pt.limbs(), pt.scale(), v.data(), n / 2, 0);
    std::vector<double> out(n / 2);
    for (size_t i = 0; i < n / 2; ++i) out[i] = v[i].real();
    return out;
}

// ---------------------------------------------------------------- levels

void Evaluator::mod_switch_to_inplace(Ciphertext &ct, int limbs)
{
    // mod_switch_to_inplace / mod_switch_drop_to_next (evaluator.cpp:1483-1546, 1630)
    if (limbs > ct.limbs()) throw std::invalid_argument("cannot switch to higher level modulus");
    if (limbs == ct.limbs()) return;
    if (limbs < 1) throw std::invalid_argument("end of modulus switching chain reached");
    Ciphertext out;
    out.resize(c_, ct.size(), limbs, s_);
    out.scale() = ct.scale();
    const size_t row = c_.n * 8;
    ck(cudaMemcpy2DAsync(out.data(), limbs * row, ct.data(), ct.limbs() * row, limbs * row, ct.size(),
                         cudaMemcpyDeviceToDevice, s_),
       "drop limbs");
    ct = std::move(out);
}

void Evaluator::mod_switch_to_inplace(Plaintext &pt, int limbs) { pt.drop_to(limbs, s_, c_); }

void Evaluator::rescale_to_next_inplace(Ciphertext &ct)
{
    // rescale_to_next -> mod_switch_scale_to_next (evaluator.cpp:1402-1480, 1682)
    if (ct.limbs() < 2) throw std::invalid_argument("end of modulus switching chain reached");
    const double scale = ct.scale() / (double)c_.q[ct.limbs() - 1];
    check_scale(scale, ct.limbs() - 1);
    Ciphertext out;
    out.resize(c_, ct.size(), ct.limbs() - 1, s_);
    rescale(c_, ct.data(), ct.size(), ct.limbs(), out.data(), s_);
    out.scale() = scale;
    ct = std::move(out);
}

// ---------------------------------------------------------------- arithmetic

void Evaluator::multiply_inplace(Ciphertext &a, const Ciphertext &b)
{
    // multiply_inplace -> ckks_multiply (evaluator.cpp:770-850)
    if (a.limbs() != b.limbs()) throw std::invalid_argument("encrypted1 and encrypted2 parameter mismatch");
    if (a.size() != 2 || b.size() != 2) throw std::invalid_argument("multiply expects size-2 ciphertexts");
    const double scale = a.scale() * b.scale();
    check_scale(scale, a.limbs());
    Ciphertext out;
    out.resize(c_, 3, a.limbs(), s_);
    tensor(c_, a.data(), b.data(), a.limbs(), out.data(), s_);
    out.scale() = scale;
    a = std::move(out);
}

void Evaluator::multiply(const Ciphertext &a, const Ciphertext &b, Ciphertext &dest)
{
    if (&b == &dest) {
        multiply_inplace(dest, a);
    } else {
        if (&a != &dest) dest = a;
        multiply_inplace(dest, b);
    }
}

void Evaluator::relinearize_inplace(Ciphertext &ct)
{
    // relinearize_internal (evaluator.cpp:1345-1400)
    if (ct.size() == 2) return;
    if (!relin_key) throw std::invalid_argument("relin_keys is not valid for encryption parameters");
    Ciphertext out;
    out.resize(c_, 2, ct.limbs(), s_);
    relinearize(c_, ct.data(), ct.limbs(), relin_key, out.data(), s_);
    out.scale() = ct.scale();
    ct = std::move(out);
}

static void check_same(const Ciphertext &a, const Ciphertext &b)
{
    if (a.limbs() != b.limbs()) throw std::invalid_argument("encrypted1 and encrypted2 parameter mismatch");
    if (!are_close(a.scale(), b.scale())) throw std::invalid_argument("scale mismatch");
    if (a.size() != b.size()) throw std::invalid_argument("ciphertext sizes differ");
}

void Evaluator::add_inplace(Ciphertext &a, const Ciphertext &b)
{
    check_same(a, b);
    poly_add(c_, a.data(), b.data(), a.size(), a.limbs(), a.data(), s_);
}

void Evaluator::add(const Ciphertext &a, const Ciphertext &b, Ciphertext &dest)
{
    if (&b == &dest) {
        add_inplace(dest, a);
    } else {
        if (&a != &dest) dest = a;
        add_inplace(dest, b);
    }
}

void Evaluator::sub_inplace(Ciphertext &a, const Ciphertext &b)
{
    check_same(a, b);
    poly_sub(c_, a.data(), b.data(), a.size(), a.limbs(), a.data(), s_);
}

void Evaluator::sub(const Ciphertext &a, const Ciphertext &b, Ciphertext &dest)
{
    if (&b == &dest) {
        sub_inplace(dest, a);
        negate_inplace(dest);
    } else {
        if (&a != &dest) dest = a;
        sub_inplace(dest, b);
    }
}

void Evaluator::negate_inplace(Ciphertext &a) { poly_negate(c_, a.data(), a.size(), a.limbs(), a.data(), s_); }

void Evaluator::negate(const Ciphertext &a, Ciphertext &dest)
{
    if (&a != &dest) dest = a;
    negate_inplace(dest);
}

void Evaluator::plain_arith(Ciphertext &ct, const Plaintext &pt, bool sub)
{
    // add_plain_inplace / sub_plain_inplace (evaluator.cpp:1938, 2046)
    if (ct.limbs() != pt.limbs()) throw std::invalid_argument("encrypted and plain parameter mismatch");
    if (!are_close(ct.scale(), pt.scale())) throw std::invalid_argument("scale mismatch");
    if (pt.is_scalar())
        poly_add_scalar(c_, ct.data(), ct.limbs(), pt.residues().data(), sub ? 1 : 0, ct.data(), s_);
    else
        poly_add_plain(c_, ct.data(), 1, ct.limbs(), pt.data(), sub ? 1 : 0, ct.data(), s_);
}

void Evaluator::add_plain_inplace(Ciphertext &ct, const Plaintext &pt) { plain_arith(ct, pt, false); }
void Evaluator::sub_plain_inplace(Ciphertext &ct, const Plaintext &pt) { plain_arith(ct, pt, true); }

void Evaluator::add_plain(const Ciphertext &ct, const Plaintext &pt, Ciphertext &dest)
{
    if (&ct != &dest) dest = ct;
    add_plain_inplace(dest, pt);
}

void Evaluator::sub_plain(const Ciphertext &ct, const Plaintext &pt, Ciphertext &dest)
{
    if (&ct != &dest) dest = ct;
    sub_plain_inplace(dest, pt);
}

void Evaluator::multiply_plain_inplace(Ciphertext &ct, const Plaintext &pt)
{
    // multiply_plain_inplace -> multiply_plain_ntt (evaluator.cpp:2154, 2336-2373)
    if (ct.limbs() != pt.limbs()) throw std::invalid_argument("encrypted and plain parameter mismatch");
    const double scale = ct.scale() * pt.scale();
    check_scale(scale, ct.limbs());
    if (pt.is_scalar())
        poly_mul_scalar(c_, ct.data(), ct.size(), ct.limbs(), pt.residues().data(), ct.data(), s_);
    else
        poly_mul_plain(c_, ct.data(), ct.size(), ct.limbs(), pt.data(), ct.data(), s_);
    ct.scale() = scale;
}

void Evaluator::multiply_plain(const Ciphertext &ct, const Plaintext &pt, Ciphertext &dest)
{
    if (&ct == &dest) {
        multiply_plain_inplace(dest, pt);
        return;
    }
    // out of place: the product is written straight into dest
    if (ct.limbs() != pt.limbs()) throw std::invalid_argument("encrypted and plain parameter mismatch");
    const double scale = ct.scale() * pt.scale();
    check_scale(scale, ct.limbs());
    dest.resize(c_, ct.size(), ct.limbs(), s_);
    if (pt.is_scalar())
        poly_mul_scalar(c_, ct.data(), ct.size(), ct.limbs(), pt.residues().data(), dest.data(), s_);
    else
        poly_mul_plain(c_, ct.data(), ct.size(), ct.limbs(), pt.data(), dest.data(), s_);
    dest.scale() = scale;
}

void Evaluator::multiply_plain_accumulate(const std::vector<const Ciphertext *> &cts,
                                          const std::vector<const Plaintext *> &pts, Ciphertext &dest)
{
    const size_t m = cts.size();
    if (m == 0 || pts.size() != m) throw std::invalid_argument("multiply_plain_accumulate: bad term count");
    const int limbs = cts[0]->limbs();
    double scale = 0.0;
    std::vector<const uint64_t *> cp(m), pp(m);
    for (size_t j = 0; j < m; ++j) {
        const Ciphertext &ct = *cts[j];
        const Plaintext &pt = *pts[j];
        if (ct.size() != 2 || ct.limbs() != limbs || &ct == &dest)
            throw std::invalid_argument("multiply_plain_accumulate: ciphertexts must be distinct, size 2, one level");
        if (pt.is_scalar() || pt.limbs() != limbs) throw std::invalid_argument("encrypted and plain parameter mismatch");
        scale = ct.scale() * pt.scale();
        check_scale(scale, limbs);
        cp[j] = ct.data();
        pp[j] = pt.data();
    }
    dest.resize(c_, 2, limbs, s_);
    size_t done = 0;
    while (done < m) {
        const int take = (int)std::min<size_t>(16, m - done);
        if (done == 0) {
            poly_mac_plain(c_, cp.data(), pp.data(), take, limbs, dest.data(), s_);
        } else {
            Ciphertext part;
            part.resize(c_, 2, limbs, s_);
            poly_mac_plain(c_, cp.data() + done, pp.data() + done, take, limbs, part.data(), s_);
            poly_add(c_, dest.data(), part.data(), 2, limbs, dest.data(), s_);
        }
        done += take;
    }
    dest.scale() = scale;
}

// ---------------------------------------------------------------- fork ops

// add_const_inplace / multiply_const_inplace / multiply_vector_inplace
// (evaluator.cpp:395-418): encode at the ciphertext's scale on the top level,
// drop to its level, then add / multiply
void Evaluator::add_const_inplace(Ciphertext &ct, double value)
{
    Plaintext p;
    encode_then_drop(value, ct.limbs(), ct.scale(), p);
    add_plain_inplace(ct, p);
}

void Evaluator::multiply_const_inplace(Ciphertext &ct, double value)
{
    Plaintext p;
    encode_then_drop(value, ct.limbs(), ct.scale(), p);
    multiply_plain_inplace(ct, p);
}

void Evaluator::multiply_const(const Ciphertext &ct, double value, Ciphertext &dest)
{
    Plaintext p;
    encode_then_drop(value, ct.limbs(), ct.scale(), p);
    multiply_plain(ct, p, dest);
}

void Evaluator::multiply_vector_inplace_reduced_error(Ciphertext &ct, const std::vector<std::complex<double>> &values)
{
    Plaintext p;
    encode_then_drop(values, ct.limbs(), ct.scale(), p);
    multiply_plain_inplace(ct, p);
}

void Evaluator::multiply_vector_reduced_error(const Ciphertext &ct, const std::vector<std::complex<double>> &values,
                                              Ciphertext &dest)
{
    if (&ct != &dest) dest = ct;
    multiply_vector_inplace_reduced_error(dest, values);
}

// The level matching of add/sub/multiply_inplace_reduced_error
// (evaluator.cpp:420-590): the higher ciphertext is multiplied by
// lo.scale * q_top / hi.scale^2, given scale lo.scale * q_top, rescaled and
// dropped to lo's level.
Ciphertext Evaluator::adjust_down(const Ciphertext &hi, const Ciphertext &lo)
{
    const double q_top = (double)c_.q[hi.limbs() - 1];
    const double scale_adjust = lo.scale() * q_top / (hi.scale() * hi.scale());
    Ciphertext adj;
    multiply_const_rescale(hi, scale_adjust, adj, lo.scale() * q_top);
    mod_switch_to_inplace(adj, lo.limbs());
    return adj;
}

void Evaluator::multiply_const_rescale_add(const Ciphertext &x, double value, Ciphertext &acc)
{
    // the rescaled product lands on acc's level: add_inplace_reduced_error's
    // equal-level case (acc takes the product's scale, then acc += product),
    // done by the rescale's finishing kernel
    if (&x != &acc && x.limbs() >= 2 && acc.limbs() == x.limbs() - 1 && acc.size() == x.size()) {
        Plaintext p;
        encode_then_drop(value, x.limbs(), x.scale(), p);
        const double prod = x.scale() * p.scale();
        check_scale(prod, x.limbs());
        const double scale = prod / (double)c_.q[x.limbs() - 1];
        check_scale(scale, x.limbs() - 1);
        rescale_scaled(c_, x.data(), x.size(), x.limbs(), p.residues().data(), acc.data(), s_, true);
        acc.scale() = scale;
        return;
    }
    Ciphertext tmp;
    multiply_const_rescale(x, value, tmp);
    add_inplace_reduced_error(acc, tmp);
}

void Evaluator::multiply_const_rescale(const Ciphertext &ct, double value, Ciphertext &dest, double set_scale)
{
    Plaintext p;
    encode_then_drop(value, ct.limbs(), ct.scale(), p);
    const double prod = ct.scale() * p.scale();
    check_scale(prod, ct.limbs());
    if (ct.limbs() < 2) throw std::invalid_argument("end of modulus switching chain reached");
    const double scale = (set_scale > 0.0 ? set_scale : prod) / (double)c_.q[ct.limbs() - 1];
    check_scale(scale, ct.limbs() - 1);
    Ciphertext out;
    out.resize(c_, ct.size(), ct.limbs() - 1, s_);
    rescale_scaled(c_, ct.data(), ct.size(), ct.limbs(), p.residues().data(), out.data(), s_);
    out.scale() = scale;
    dest = std::move(out);
}

void Evaluator::add_inplace_reduced_error(Ciphertext &a, const Ciphertext &b)
{
    if (a.limbs() == b.limbs()) {
        a.scale() = b.scale();
        add_inplace(a, b);
    } else if (a.limbs() < b.limbs()) {
        Ciphertext adj = adjust_down(b, a);
        a.scale() = adj.scale();
        add_inplace(a, adj);
    } else {
        Ciphertext adj = adjust_down(a, b);
        adj.scale() = b.scale();
        add(adj, b, a);
    }
}

void Evaluator::sub_inplace_reduced_error(Ciphertext &a, const Ciphertext &b)
{
    if (a.limbs() == b.limbs()) {
        a.scale() = b.scale();
        sub_inplace(a, b);
    } else if (a.limbs() < b.limbs()) {
        Ciphertext adj = adjust_down(b, a);
        a.scale() = adj.scale();
        sub_inplace(a, adj);
    } else {
        Ciphertext adj = adjust_down(a, b);
        adj.scale() = b.scale();
        sub(adj, b, a);
    }
}

void Evaluator::multiply_inplace_reduced_error(Ciphertext &a, const Ciphertext &b)
{
    if (a.limbs() == b.limbs()) {
        a.scale() = b.scale();
        multiply_inplace(a, b);
    } else if (a.limbs() < b.limbs()) {
        Ciphertext adj = adjust_down(b, a);
        a.scale() = adj.scale();
        multiply_inplace(a, adj);
    } else {
        Ciphertext adj = adjust_down(a, b);
        adj.scale() = b.scale();
        multiply(adj, b, a);
    }
    relinearize_inplace(a);
}

void Evaluator::add_reduced_error(const Ciphertext &a, const Ciphertext &b, Ciphertext &dest)
{
    if (&b == &dest) {
        add_inplace_reduced_error(dest, a);
    } else {
        if (&a != &dest) dest = a;
        add_inplace_reduced_error(dest, b);
    }
}

void Evaluator::sub_reduced_error(const Ciphertext &a, const Ciphertext &b, Ciphertext &dest)
{
    Ciphertext bb = b;  // b may alias dest
    if (&a != &dest) dest = a;
    sub_inplace_reduced_error(dest, bb);
}

void Evaluator::multiply_reduced_error(const Ciphertext &a, const Ciphertext &b, Ciphertext &dest)
{
    if (&b == &dest) {
        multiply_inplace_reduced_error(dest, a);
    } else {
        if (&a != &dest) dest = a;
        multiply_inplace_reduced_error(dest, b);
    }
}

// ---------------------------------------------------------------- rotations

void Evaluator::apply_galois_inplace(Ciphertext &ct, uint32_t elt)
{
    // apply_galois_inplace (evaluator.cpp:2563-2665)
    auto it = galois_keys.find(elt);
    if (it == galois_keys.end()) throw std::invalid_argument("Galois key not present");
    if (ct.size() != 2) throw std::invalid_argument("encrypted size must be 2");
    Ciphertext out;
    out.resize(c_, 2, ct.limbs(), s_);
    apply_galois(c_, ct.data(), ct.limbs(), elt, it->second, out.data(), s_);
    out.scale() = ct.scale();
    ct = std::move(out);
}

void Evaluator::rotate_vector_inplace(Ciphertext &ct, int steps)
{
    // rotate_internal with the NAF fallback (evaluator.cpp:2667-2722)
    if (steps == 0) return;
    const uint32_t elt = galois_elt(steps);
    if (galois_keys.count(elt)) {
        apply_galois_inplace(ct, elt);
        return;
    }
    std::vector<int> parts = naf(steps);
    if (parts.size() == 1) throw std::invalid_argument("Galois key not present");
    for (int st : parts)
        if ((size_t)std::abs(st) != (c_.n >> 1)) rotate_vector_inplace(ct, st);
}

void Evaluator::rotate_vector(const Ciphertext &ct, int steps, Ciphertext &dest)
{
    if (&ct != &dest && steps != 0) {
        // a direct key: permute and key-switch straight into dest
        const uint32_t elt = galois_elt(steps);
        auto it = galois_keys.find(elt);
        if (it != galois_keys.end()) {
            if (ct.size() != 2) throw std::invalid_argument("encrypted size must be 2");
            dest.resize(c_, 2, ct.limbs(), s_);
            apply_galois(c_, ct.data(), ct.limbs(), elt, it->second, dest.data(), s_);
            dest.scale() = ct.scale();
            return;
        }
    }
    if (&ct != &dest) dest = ct;
    rotate_vector_inplace(dest, steps);
}

void Evaluator::complex_conjugate_inplace(Ciphertext &ct) { apply_galois_inplace(ct, galois_elt(0)); }

const Plaintext &Evaluator::monomial(int power, int limbs)
{
    if (power < 0 || power >= (int)c_.n) throw std::invalid_argument("monomial: power out of range");
    if (limbs < 1 || limbs > top_limbs()) throw std::invalid_argument("monomial: limbs out of range");
    const auto key = std::make_pair(power, limbs);
    auto it = monomials_.find(key);
    if (it != monomials_.end()) return it->second;
    std::vector<uint64_t> host((size_t)limbs * c_.n, 0);
    for (int l = 0; l < limbs; ++l) host[(size_t)l * c_.n + (size_t)power] = 1;
    Plaintext p;
    p.set_vector(c_, limbs, 1.0, s_);
    ck(cudaMemcpyAsync(p.mutable_data(), host.data(), host.size() * 8, cudaMemcpyHostToDevice, s_), "upload");
    ck(cudaStreamSynchronize(s_), "monomial");  // host buffer lifetime
    ntt_forward(c_, p.mutable_data(), 1, 0, limbs, s_);
    return monomials_.emplace(key, std::move(p)).first->second;
}

// ------------------------------------------------------- hoisted rotations

void Evaluator::set_galois_key(uint32_t elt, const uint64_t *key)
{
    galois_keys[elt] = key;
    hoist_keys_.erase(elt);
    for (auto it = hoist_corrs_.begin(); it != hoist_corrs_.end();)
        it = (it->first.first == elt) ? hoist_corrs_.erase(it) : std::next(it);
}

const uint64_t *Evaluator::hoist_key(uint32_t elt)
{
    auto it = hoist_keys_.find(elt);
    if (it != hoist_keys_.end()) return it->second.get();
    auto k = galois_keys.find(elt);
    if (k == galois_keys.end()) throw std::invalid_argument("Galois key not present");
    DeviceBuffer b;
    b.reserve((size_t)(c_.k - 1) * 2 * c_.k * c_.n, s_);
    hoist_permute_key(c_, k->second, elt, b.get(), s_);
    return (hoist_keys_[elt] = std::move(b)).get();
}

const uint64_t *Evaluator::hoist_corr(uint32_t elt, int limbs)
{
    auto it = hoist_corrs_.find({elt, limbs});
    if (it != hoist_corrs_.end()) return it->second.get();
    auto k = galois_keys.find(elt);
    if (k == galois_keys.end()) throw std::invalid_argument("Galois key not present");
    auto m = hoist_masks_.find(elt);
    if (m == hoist_masks_.end()) {
        DeviceBuffer mb;
        mb.reserve((size_t)c_.k * c_.n, s_);
        hoist_galois_mask_ntt(c_, elt, mb.get(), s_);
        m = hoist_masks_.emplace(elt, std::move(mb)).first;
    }
    DeviceBuffer b;
    b.reserve((size_t)2 * (limbs + 1) * c_.n, s_);
    hoist_correction(c_, k->second, m->second.get(), limbs, b.get(), s_);
    return (hoist_corrs_[{elt, limbs}] = std::move(b)).get();
}

bool Evaluator::hoist_prepare(const std::vector<uint32_t> &elts, int limbs)
{
    try {
        hoist_flags(1);
        for (uint32_t e : elts) {
            hoist_key(e);
            hoist_corr(e, limbs);
        }
    } catch (const std::runtime_error &) {
        cudaGetLastError();   // an out-of-memory allocation is not sticky
        return false;
    }
    return true;
}

int *Evaluator::hoist_flags(int count)
{
    hoist_flag_.reserve(((size_t)count + 1) / 2, s_);
    return reinterpret_cast<int *>(hoist_flag_.get());
}

void Evaluator::rotate_vector_many(const Ciphertext &ct, const std::vector<int> &steps, std::vector<Ciphertext> &outs)
{
    outs.resize(steps.size());
    for (const Ciphertext &o : outs)
        if (&o == &ct) throw std::invalid_argument("rotate_vector_many: ct must not be one of the outputs");
    const int l = ct.limbs();
    std::vector<bool> done(steps.size(), false);
    std::vector<size_t> direct;
    for (size_t i = 0; i < steps.size(); ++i)
        if (steps[i] != 0 && galois_keys.count(galois_elt(steps[i]))) direct.push_back(i);
    std::vector<uint32_t> elts;
    for (size_t i : direct) elts.push_back(galois_elt(steps[i]));
    if (hoisting && ct.size() == 2 && hoist_pays((int)direct.size(), l) && hoist_prepare(elts, l)) {
        const size_t N = c_.n;
        DeviceBuffer t, D;
        t.reserve((size_t)l * N, s_);
        D.reserve((size_t)l * (l + 1) * N, s_);
        int *flags = hoist_flags(1);
        hoist_decompose(c_, ct.data() + (size_t)l * N, 2 * (size_t)l * N, 1, l, t.get(), D.get(), flags, s_);
        std::vector<HoistRotation> rots;
        for (size_t i : direct) {
            const uint32_t elt = galois_elt(steps[i]);
            const uint64_t *pk = hoist_key(elt), *corr = hoist_corr(elt, l);
            outs[i].resize(c_, 2, l, s_);
            outs[i].scale() = ct.scale();
            hoist_rotate(c_, D.get(), 1, l, elt, pk, corr, ct.data(), 0, outs[i].data(), s_);
            rots.push_back({elt, galois_keys.at(elt), outs[i].data()});
            done[i] = true;
        }
        hoist_fix(c_, t.get(), ct.data(), 0, flags, 1, l, rots, s_);
    }
    for (size_t i = 0; i < steps.size(); ++i)
        if (!done[i]) rotate_vector(ct, steps[i], outs[i]);
}

}  // namespace nexus
