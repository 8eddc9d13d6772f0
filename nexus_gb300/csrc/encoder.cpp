// CKKS encoder on the host: the FP64 special FFT of SEAL's CKKSEncoder
// (ckks.cpp:13-70, ckks.h:457-640 and 640-760, util/croots.cpp,
// util/dwthandler.h in SEAL-4.1-bs), with the same root table, slot order,
// butterfly order and rounding, so an encoded plaintext equals SEAL's word for
// word.  This file is compiled with -ffp-contract=off: a fused multiply-add
// would change the rounding of the FFT.
//
// The coefficient-domain result is reduced into every prime here and then
// uploaded and transformed by the GPU NTT.
#include <cmath>
#include <complex>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "encoder.h"

namespace nexus {

namespace {

constexpr double kPi = 3.1415926535897932384626433832795028842;

uint32_t rev_bits(uint64_t x, int bits)
{
    uint64_t r = 0;
    for (int i = 0; i < bits; ++i) {
        r = (r << 1) | (x & 1);
        x >>= 1;
    }
    return (uint32_t)r;
}

// ComplexRoots (util/croots.cpp): 1/8 of the m-th roots from std::polar, the
// rest by the 8-fold symmetry.
struct Roots {
    size_t m;
    std::vector<std::complex<double>> r;
    explicit Roots(size_t m_) : m(m_), r(m_ / 8 + 1)
    {
        for (size_t i = 0; i <= m / 8; ++i) r[i] = std::polar<double>(1.0, 2 * kPi * (double)i / (double)m);
    }
    std::complex<double> get(size_t index) const
    {
        index &= m - 1;
        if (index <= m / 8) return r[index];
        if (index <= m / 4) {
            auto a = r[m / 4 - index];
            return {a.imag(), a.real()};
        }
        if (index <= m / 2) return -std::conj(get(m / 2 - index));
        if (index <= 3 * m / 4) return -get(index - m / 2);
        return std::conj(get(m - index));
    }
};

}  // namespace

Encoder::Encoder(const Context &c) : ctx_(c)
{
    const size_t n = c.n;
    slots_ = n / 2;
    const uint64_t m = (uint64_t)n << 1;
    index_map_.resize(n);
    uint64_t pos = 1;
    for (size_t i = 0; i < slots_; ++i) {
        uint64_t i1 = (pos - 1) >> 1, i2 = (m - pos - 1) >> 1;
        index_map_[i] = rev_bits(i1, c.logn);
        index_map_[slots_ | i] = rev_bits(i2, c.logn);
        pos = (pos * 5) & (m - 1);
    }
    Roots roots(m);
    root_powers_.resize(n);
    inv_root_powers_.resize(n);
    for (size_t i = 1; i < n; ++i) {
        root_powers_[i] = roots.get(rev_bits(i, c.logn));
        inv_root_powers_[i] = std::conj(roots.get(rev_bits(i - 1, c.logn) + 1));
    }
}

// DWTHandler::transform_from_rev over complex<double> with the scalar merged
// into the last stage (util/dwthandler.h:200-290)
static void fft_from_rev(std::complex<double> *v, int logn, const std::complex<double> *roots, double scalar)
{
    const size_t n = (size_t)1 << logn;
    size_t gap = 1, m = n >> 1;
    const std::complex<double> *rt = roots;
    for (; m > 1; m >>= 1) {
        size_t off = 0;
        for (size_t i = 0; i < m; ++i) {
            const std::complex<double> r = *++rt;
            std::complex<double> *x = v + off, *y = x + gap;
            for (size_t j = 0; j < gap; ++j) {
                std::complex<double> u = x[j], w = y[j];
                x[j] = u + w;
                y[j] = (u - w) * r;
            }
            off += gap << 1;
        }
        gap <<= 1;
    }
    const std::complex<double> r = *++rt;
    const std::complex<double> sr = r * scalar;
    for (size_t j = 0; j < gap; ++j) {
        std::complex<double> u = v[j], w = v[j + gap];
        v[j] = (u + w) * scalar;
        v[j + gap] = (u - w) * sr;
    }
}

// DWTHandler::transform_to_rev over complex<double> (util/dwthandler.h:94-190)
static void fft_to_rev(std::complex<double> *v, int logn, const std::complex<double> *roots)
{
    const size_t n = (size_t)1 << logn;
    size_t gap = n >> 1, m = 1;
    const std::complex<double> *rt = roots;
    for (; m < (n >> 1); m <<= 1) {
        size_t off = 0;
        for (size_t i = 0; i < m; ++i) {
            const std::complex<double> r = *++rt;
            std::complex<double> *x = v + off, *y = x + gap;
            for (size_t j = 0; j < gap; ++j) {
                std::complex<double> u = x[j], w = y[j] * r;
                x[j] = u + w;
                y[j] = u - w;
            }
            off += gap << 1;
        }
        gap >>= 1;
    }
    for (size_t i = 0; i < m; ++i) {
        const std::complex<double> r = *++rt;
        std::complex<double> u = v[0], w = v[1] * r;
        v[0] = u + w;
        v[1] = u - w;
        v += 2;
    }
}

// exact bit count of the product of the first `limbs` primes
// (ContextData::total_coeff_modulus_bit_count)
static int total_bits(const Context &c, int limbs)
{
    std::vector<uint64_t> p(limbs + 1, 0);
    p[0] = 1;
    for (int i = 0; i < limbs; ++i) {
        unsigned __int128 carry = 0;
        for (auto &w : p) {
            unsigned __int128 t = (unsigned __int128)w * c.q[i] + carry;
            w = (uint64_t)t;
            carry = t >> 64;
        }
    }
    for (int w = limbs; w >= 0; --w)
        if (p[w]) return w * 64 + (64 - __builtin_clzll(p[w]));
    return 0;
}

// Reduce a non-negative integer given as little-endian 64-bit words mod q.
static uint64_t reduce_words(const uint64_t *w, int count, uint64_t q)
{
    unsigned __int128 r = 0;
    for (int i = count - 1; i >= 0; --i) r = ((r << 64) | w[i]) % q;
    return (uint64_t)r;
}

void Encoder::encode(const std::complex<double> *values, size_t nvals, double scale, int limbs, uint64_t *out,
                     int check_limbs) const
{
    const Context &c = ctx_;
    const size_t n = c.n;
    if (nvals > slots_) throw std::invalid_argument("values_size is too large");
    if (limbs < 1 || limbs > c.k - 1) throw std::invalid_argument("limbs out of range");
    const int tb = total_bits(c, check_limbs > 0 ? check_limbs : limbs);
    if (scale <= 0 || ((int)std::log2(scale) + 1 >= tb)) throw std::invalid_argument("scale out of bounds");
    std::vector<std::complex<double>> v(n, std::complex<double>(0, 0));
    for (size_t i = 0; i < nvals; ++i) {
        v[index_map_[i]] = values[i];
        v[index_map_[i + slots_]] = std::conj(values[i]);
    }
    const double fix = scale / (double)n;
    fft_from_rev(v.data(), c.logn, inv_root_powers_.data(), fix);
    double max_coeff = 0;
    for (size_t i = 0; i < n; ++i) max_coeff = std::max(max_coeff, std::fabs(v[i].real()));
    const int max_bits = (int)std::ceil(std::log2(std::max(max_coeff, 1.0))) + 1;
    if (max_bits >= tb) throw std::invalid_argument("encoded values are too large");
    const double two64 = std::pow(2.0, 64);
    for (size_t i = 0; i < n; ++i) {
        double cd = std::round(v[i].real());
        const bool neg = std::signbit(cd);
        cd = std::fabs(cd);
        uint64_t words[40];
        int count = 0;
        if (max_bits <= 64) {
            words[0] = (uint64_t)cd;
            count = 1;
        } else if (max_bits <= 128) {
            words[0] = (uint64_t)std::fmod(cd, two64);
            words[1] = (uint64_t)(cd / two64);
            count = 2;
        } else {
            while (cd >= 1 && count < 40) {
                words[count++] = (uint64_t)std::fmod(cd, two64);
                cd /= two64;
            }
        }
        for (int j = 0; j < limbs; ++j) {
            const uint64_t q = c.q[j];
            uint64_t r = count ? reduce_words(words, count, q) : 0;
            if (neg && r) r = q - r;
            out[(size_t)j * n + i] = r;
        }
    }
}

// CKKSEncoder::encode_internal(double) (ckks.cpp:75-205): the constant
// polynomial round(value*scale); in NTT form every coefficient of limb j holds
// the same residue, returned here per limb.
void Encoder::encode_scalar(double value, double scale, int limbs, uint64_t *per_limb, int check_limbs) const
{
    const Context &c = ctx_;
    const int tb = total_bits(c, check_limbs > 0 ? check_limbs : limbs);
    if (scale <= 0 || ((int)std::log2(scale) >= tb)) throw std::invalid_argument("scale out of bounds");
    value *= scale;
    const int cb = (int)std::log2(std::fabs(value)) + 2;
    if (cb >= tb) throw std::invalid_argument("encoded value is too large");
    const double two64 = std::pow(2.0, 64);
    double cd = std::round(value);
    const bool neg = std::signbit(cd);
    cd = std::fabs(cd);
    uint64_t words[40];
    int count = 0;
    if (cb <= 64) {
        words[0] = (uint64_t)std::fabs(cd);
        count = 1;
    } else if (cb <= 128) {
        words[0] = (uint64_t)std::fmod(cd, two64);
        words[1] = (uint64_t)(cd / two64);
        count = 2;
    } else {
        while (cd >= 1 && count < 40) {
            words[count++] = (uint64_t)std::fmod(cd, two64);
            cd /= two64;
        }
    }
    for (int j = 0; j < limbs; ++j) {
        const uint64_t q = c.q[j];
        uint64_t r = count ? reduce_words(words, count, q) : 0;
        if (neg && r) r = q - r;
        per_limb[j] = r;
    }
}

// CKKSEncoder::decode_internal (ckks.h:640-760) from coefficient-form
// residues coeffs[limbs][N] (already inverse transformed).  CRT composition is
// exact multi-precision; the conversion to double follows SEAL's word order.
void Encoder::decode(const uint64_t *coeffs, int limbs, double scale, std::complex<double> *out, size_t nvals,
                     size_t sparse_slots) const
{
    const Context &c = ctx_;
    const size_t n = c.n;
    if (nvals > slots_) nvals = slots_;
    // Q = prod q_i as little-endian words, punctured products and inverses
    const int W = limbs;  // words needed for Q (each prime < 2^64)
    std::vector<uint64_t> Q(W + 1, 0);
    Q[0] = 1;
    auto mul_small = [](std::vector<uint64_t> &a, uint64_t b) {
        unsigned __int128 carry = 0;
        for (auto &w : a) {
            unsigned __int128 t = (unsigned __int128)w * b + carry;
            w = (uint64_t)t;
            carry = t >> 64;
        }
    };
    for (int i = 0; i < limbs; ++i) mul_small(Q, c.q[i]);
    std::vector<std::vector<uint64_t>> punct(limbs);
    std::vector<uint64_t> inv_punct(limbs);
    for (int i = 0; i < limbs; ++i) {
        std::vector<uint64_t> p(W + 1, 0);
        p[0] = 1;
        uint64_t pm = 1;
        for (int j = 0; j < limbs; ++j)
            if (j != i) {
                mul_small(p, c.q[j]);
                pm = host_mulmod(pm, c.q[j] % c.q[i], c.q[i]);
            }
        punct[i] = p;
        inv_punct[i] = host_invmod(pm, c.q[i]);
    }
    // upper half threshold = ceil(Q / 2)
    std::vector<uint64_t> half(W + 1, 0);
    {
        uint64_t carry = 0;
        for (int w = W; w >= 0; --w) {
            uint64_t v = Q[w];
            half[w] = (v >> 1) | (carry << 63);
            carry = v & 1;
        }
        if (carry) {  // ceil
            for (int w = 0; w <= W; ++w) {
                if (++half[w]) break;
            }
        }
    }
    auto geq = [&](const std::vector<uint64_t> &a, const std::vector<uint64_t> &b) {
        for (int w = W; w >= 0; --w) {
            if (a[w] != b[w]) return a[w] > b[w];
        }
        return true;
    };
    const double inv_scale = 1.0 / scale;
    const double two64 = std::pow(2.0, 64);
    std::vector<std::complex<double>> res(n);
    std::vector<uint64_t> x(W + 1);
    for (size_t t = 0; t < n; ++t) {
        // x = sum_i (c_i * inv_punct_i mod q_i) * punct_i  mod Q
        std::fill(x.begin(), x.end(), 0);
        for (int i = 0; i < limbs; ++i) {
            uint64_t f = host_mulmod(coeffs[(size_t)i * n + t], inv_punct[i], c.q[i]);
            unsigned __int128 carry = 0;
            for (int w = 0; w <= W; ++w) {
                unsigned __int128 s = (unsigned __int128)punct[i][w] * f + x[w] + carry;
                x[w] = (uint64_t)s;
                carry = s >> 64;
            }
        }
        // reduce mod Q (x < limbs * Q): subtract Q while x >= Q
        while (geq(x, Q)) {
            uint64_t borrow = 0;
            for (int w = 0; w <= W; ++w) {
                unsigned __int128 d = (unsigned __int128)x[w] - Q[w] - borrow;
                x[w] = (uint64_t)d;
                borrow = (uint64_t)(d >> 64) ? 1 : 0;
            }
        }
        if (sparse_slots && sparse_slots != slots_) {
            const size_t sparsity = slots_ / sparse_slots;
            if (((t - 1) & (sparsity - 1)) != sparsity - 1) std::fill(x.begin(), x.end(), 0);
        }
        double acc = 0.0;
        double sc = inv_scale;
        if (geq(x, half)) {
            for (int w = 0; w < W; ++w, sc *= two64) {
                if (x[w] > Q[w]) {
                    uint64_t d = x[w] - Q[w];
                    acc += d ? (double)d * sc : 0.0;
                } else {
                    uint64_t d = Q[w] - x[w];
                    acc -= d ? (double)d * sc : 0.0;
                }
            }
        } else {
            for (int w = 0; w < W; ++w, sc *= two64) {
                acc += x[w] ? (double)x[w] * sc : 0.0;
            }
        }
        res[t] = acc;
    }
    fft_to_rev(res.data(), c.logn, root_powers_.data());
    for (size_t i = 0; i < nvals; ++i) out[i] = res[index_map_[i]];
}

}  // namespace nexus
