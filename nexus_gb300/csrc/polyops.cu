// Element-wise RNS kernels, rescale and the NTT-domain automorphism.
//
// Every result is the fully reduced residue SEAL produces for the same
// operation (references are to the SEAL-4.1-bs tree bundled with NEXUS).
#include <algorithm>
#include <stdexcept>

#include "context.h"
#include "ntt.h"
#include "ops.h"

namespace nexus {

namespace {

constexpr int kBlock = 256;
constexpr int kMacTerms = 16;

inline unsigned grid_for(size_t pairs)
{
    size_t g = (pairs + kBlock - 1) / kBlock;
    return (unsigned)(g > 1048576 ? 1048576 : g);
}

// Iterate residue pairs (2 consecutive coefficients of one limb) over
// [rows][N]; `limb` is the limb index of the row within its polynomial.
#define FOR_PAIRS(total_pairs)                                                            \
    for (size_t pi = (size_t)blockIdx.x * blockDim.x + threadIdx.x; pi < (total_pairs);  \
         pi += (size_t)gridDim.x * blockDim.x)

__device__ __forceinline__ uint64_t add_mod(uint64_t a, uint64_t b, uint64_t q) { return csub(a + b, q); }
__device__ __forceinline__ uint64_t sub_mod(uint64_t a, uint64_t b, uint64_t q) { return csub(a + q - b, q); }

__global__ void k_add_sub(const ulonglong2 *__restrict__ a, const ulonglong2 *__restrict__ b, ulonglong2 *out,
                          const PrimeConst *__restrict__ pc, int limbs, int logn, size_t pairs, int sub)
{
    FOR_PAIRS(pairs)
    {
        const int limb = (int)((pi >> (logn - 1)) % (size_t)limbs);
        const uint64_t q = pc[limb].q;
        ulonglong2 x = a[pi], y = b[pi];
        if (sub) {
            x.x = sub_mod(x.x, y.x, q);
            x.y = sub_mod(x.y, y.y, q);
        } else {
            x.x = add_mod(x.x, y.x, q);
            x.y = add_mod(x.y, y.y, q);
        }
        out[pi] = x;
    }
}

__global__ void k_negate(const ulonglong2 *__restrict__ a, ulonglong2 *out, const PrimeConst *__restrict__ pc,
                         int limbs, int logn, size_t pairs)
{
    FOR_PAIRS(pairs)
    {
        const int limb = (int)((pi >> (logn - 1)) % (size_t)limbs);
        const uint64_t q = pc[limb].q;
        ulonglong2 x = a[pi];
        x.x = x.x ? q - x.x : 0;
        x.y = x.y ? q - x.y : 0;
        out[pi] = x;
    }
}

// out[p][l] = ct[p][l] (*|+|-) pt[l]
__global__ void k_plain(const ulonglong2 *__restrict__ ct, const ulonglong2 *__restrict__ pt, ulonglong2 *out,
                        const PrimeConst *__restrict__ pc, int limbs, int logn, size_t pairs, int op)
{
    const size_t pt_pairs = ((size_t)limbs << logn) >> 1;
    FOR_PAIRS(pairs)
    {
        const int limb = (int)((pi >> (logn - 1)) % (size_t)limbs);
        const PrimeConst P = pc[limb];
        ulonglong2 x = ct[pi], y = pt[pi % pt_pairs];
        if (op == 0) {
            x.x = mul_mod(x.x, y.x, P.q, P.r0, P.r1);
            x.y = mul_mod(x.y, y.y, P.q, P.r0, P.r1);
        } else if (op == 1) {
            x.x = add_mod(x.x, y.x, P.q);
            x.y = add_mod(x.y, y.y, P.q);
        } else {
            x.x = sub_mod(x.x, y.x, P.q);
            x.y = sub_mod(x.y, y.y, P.q);
        }
        out[pi] = x;
    }
}

// out[p] = sum_j ct_j[p] * pt_j mod q over `count` ciphertext / plaintext
// pairs, for both polynomials, accumulated exactly in 128 bits and reduced once
struct MacTerms {
    const uint64_t *ct[kMacTerms];
    const uint64_t *pt[kMacTerms];
};

__device__ __forceinline__ void mac128p(uint64_t &lo, uint64_t &hi, uint64_t a, uint64_t b)
{
    asm("mad.lo.cc.u64 %0, %2, %3, %0;\n\tmadc.hi.u64 %1, %2, %3, %1;" : "+l"(lo), "+l"(hi) : "l"(a), "l"(b));
}

// (ct_j and out hold `total / (limbs N)` ciphertexts back to back, [batch][2][limbs][N])
__global__ void k_mac_plain(MacTerms t, int count, uint64_t *__restrict__ out, const PrimeConst *__restrict__ pc,
                            int limbs, int logn, size_t total)
{
    const size_t poly = (size_t)limbs << logn;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const size_t b = x / poly, e = x - b * poly;  // ciphertext, limb * N + coefficient
        const size_t at = b * 2 * poly + e;
        const int limb = (int)(e >> logn);
        uint64_t lo0 = 0, hi0 = 0, lo1 = 0, hi1 = 0;
        for (int j = 0; j < count; ++j) {
            const uint64_t w = t.pt[j][e];
            mac128p(lo0, hi0, t.ct[j][at], w);
            mac128p(lo1, hi1, t.ct[j][at + poly], w);
        }
        const PrimeConst P = pc[limb];
        out[at] = barrett_128(lo0, hi0, P.q, P.r0, P.r1);
        out[at + poly] = barrett_128(lo1, hi1, P.q, P.r0, P.r1);
    }
}

struct LimbScalars {
    ulonglong2 w[64];  // {scalar mod q_l, Shoup quotient}
};

__global__ void k_mul_scalar(const ulonglong2 *__restrict__ ct, const LimbScalars sc, ulonglong2 *out,
                             const PrimeConst *__restrict__ pc, int limbs, int logn, size_t pairs)
{
    FOR_PAIRS(pairs)
    {
        const int limb = (int)((pi >> (logn - 1)) % (size_t)limbs);
        const uint64_t q = pc[limb].q;
        const ulonglong2 w = sc.w[limb];
        ulonglong2 x = ct[pi];
        x.x = mul_shoup(x.x, w.x, w.y, q);
        x.y = mul_shoup(x.y, w.x, w.y, q);
        out[pi] = x;
    }
}

// out[l] = in[l] (+|-) sc[l] over `batch` polynomials [limbs][N] that start
// every `stride` pairs (component 0 of each ciphertext of a batch)
__global__ void k_add_scalar(const ulonglong2 *__restrict__ in, const LimbScalars sc, ulonglong2 *out,
                             const PrimeConst *__restrict__ pc, int logn, size_t poly_pairs, int sub, size_t stride,
                             size_t total)
{
    FOR_PAIRS(total)
    {
        const size_t b = pi / poly_pairs, e = pi - b * poly_pairs;
        const size_t at = b * stride + e;
        const int limb = (int)(e >> (logn - 1));
        const uint64_t q = pc[limb].q, w = sc.w[limb].x;
        ulonglong2 x = in[at];
        if (sub) {
            x.x = sub_mod(x.x, w, q);
            x.y = sub_mod(x.y, w, q);
        } else {
            x.x = add_mod(x.x, w, q);
            x.y = add_mod(x.y, w, q);
        }
        out[at] = x;
    }
}

// (x0 y0, x0 y1 + x1 y0, x1 y1) mod q from three 128-bit products: the cross
// term is (x0 + x1)(y0 + y1) - x0 y0 - x1 y1, exact in 128 bits (below 2^123
// for q < 2^61), then one reduction each
__device__ __forceinline__ void tensor3(uint64_t x0, uint64_t x1, uint64_t y0, uint64_t y1, const PrimeConst &P,
                                        uint64_t &o0, uint64_t &o1, uint64_t &o2)
{
    const uint64_t l00 = x0 * y0, h00 = __umul64hi(x0, y0);
    const uint64_t l11 = x1 * y1, h11 = __umul64hi(x1, y1);
    const uint64_t sx = x0 + x1, sy = y0 + y1;
    const uint64_t ls = sx * sy, hs = __umul64hi(sx, sy);
    const uint64_t m1 = ls - l00;
    uint64_t mh = hs - h00 - (ls < l00);
    const uint64_t m2 = m1 - l11;
    mh = mh - h11 - (m1 < l11);
    o0 = barrett_128(l00, h00, P.q, P.r0, P.r1);
    o1 = barrett_128(m2, mh, P.q, P.r0, P.r1);
    o2 = barrett_128(l11, h11, P.q, P.r0, P.r1);
}

// ckks_multiply (evaluator.cpp:770-850): out3 = (a0 b0, a0 b1 + a1 b0, a1 b1)
// over `batch` ciphertext pairs laid out back to back ([batch][2] in, [batch][3] out)
__global__ void k_tensor(const ulonglong2 *__restrict__ a_, const ulonglong2 *__restrict__ b_, ulonglong2 *out_,
                         const PrimeConst *__restrict__ pc, int limbs, int logn, size_t total)
{
    const size_t poly_pairs = ((size_t)limbs << logn) >> 1;
    FOR_PAIRS(total)
    {
        const size_t bt = pi / poly_pairs, e = pi - bt * poly_pairs;
        const ulonglong2 *a = a_ + bt * 2 * poly_pairs, *b = b_ + bt * 2 * poly_pairs;
        ulonglong2 *out = out_ + bt * 3 * poly_pairs;
        const int limb = (int)(e >> (logn - 1));
        const PrimeConst P = pc[limb];
        const ulonglong2 x0 = a[e], x1 = a[e + poly_pairs], y0 = b[e], y1 = b[e + poly_pairs];
        uint64_t r[6];
        tensor3(x0.x, x1.x, y0.x, y1.x, P, r[0], r[1], r[2]);
        tensor3(x0.y, x1.y, y0.y, y1.y, P, r[3], r[4], r[5]);
        const ulonglong2 o0 = make_ulonglong2(r[0], r[3]), o1 = make_ulonglong2(r[1], r[4]),
                         o2 = make_ulonglong2(r[2], r[5]);
        out[e] = o0;
        out[e + poly_pairs] = o1;
        out[e + 2 * poly_pairs] = o2;
    }
}

// copy limb `which` of each of `polys` polynomials ([polys][limbs][N]) into dst[polys][N]
__global__ void k_gather_limb(const ulonglong2 *__restrict__ src, ulonglong2 *dst, int limbs, int which, int logn,
                              size_t pairs)
{
    const size_t half = (size_t)1 << (logn - 1);
    FOR_PAIRS(pairs)
    {
        const size_t p = pi / half, i = pi % half;
        dst[pi] = src[(p * limbs + which) * half + i];
    }
}

// out[p][i] = (in[p][i] - t[p][i]) * q_last^{-1} mod q_i   (t in [0, q_i))
__global__ void k_rescale_finish(const ulonglong2 *__restrict__ in, const ulonglong2 *__restrict__ t,
                                 ulonglong2 *out, const PrimeConst *__restrict__ pc,
                                 const ulonglong2 *__restrict__ inv_row, int limbs, int logn, size_t pairs)
{
    const size_t half = (size_t)1 << (logn - 1);
    const int ol = limbs - 1;
    FOR_PAIRS(pairs)
    {
        const size_t row = pi / half, i = pi % half;
        const size_t p = row / ol;
        const int l = (int)(row % ol);
        const uint64_t q = pc[l].q;
        const ulonglong2 w = inv_row[l];
        const ulonglong2 x = in[(p * limbs + l) * half + i], y = t[pi];
        ulonglong2 r;
        r.x = mul_shoup(x.x + q - y.x, w.x, w.y, q);
        r.y = mul_shoup(x.y + q - y.y, w.x, w.y, q);
        out[pi] = r;
    }
}

// k_gather_limb / k_rescale_finish of in * c (c a per-limb scalar, Shoup
// pairs in sc): the product is formed where each is read instead of by a
// separate pass, with the same residues
__global__ void k_gather_limb_scaled(const ulonglong2 *__restrict__ in, ulonglong2 *__restrict__ out, const LimbScalars sc,
                                     const PrimeConst *__restrict__ pc, int limbs, int which, int logn, size_t pairs)
{
    const size_t half = (size_t)1 << (logn - 1);
    const uint64_t q = pc[which].q;
    const ulonglong2 w = sc.w[which];
    FOR_PAIRS(pairs)
    {
        const size_t p = pi / half, i = pi % half;
        ulonglong2 x = in[(p * limbs + which) * half + i];
        x.x = mul_shoup(x.x, w.x, w.y, q);
        x.y = mul_shoup(x.y, w.x, w.y, q);
        out[pi] = x;
    }
}

// ACC: out += the rescaled value (mod q) instead of out = it
template <bool ACC>
__global__ void k_rescale_finish_scaled(const ulonglong2 *__restrict__ in, const ulonglong2 *__restrict__ t,
                                        ulonglong2 *out, const LimbScalars sc, const PrimeConst *__restrict__ pc,
                                        const ulonglong2 *__restrict__ inv_row, int limbs, int logn, size_t pairs)
{
    const size_t half = (size_t)1 << (logn - 1);
    const int ol = limbs - 1;
    FOR_PAIRS(pairs)
    {
        const size_t row = pi / half, i = pi % half;
        const size_t p = row / ol;
        const int l = (int)(row % ol);
        const uint64_t q = pc[l].q;
        const ulonglong2 w = inv_row[l], c = sc.w[l];
        const ulonglong2 x = in[(p * limbs + l) * half + i], y = t[pi];
        const uint64_t x0 = mul_shoup(x.x, c.x, c.y, q), x1 = mul_shoup(x.y, c.x, c.y, q);
        ulonglong2 r;
        r.x = mul_shoup(x0 + q - y.x, w.x, w.y, q);
        r.y = mul_shoup(x1 + q - y.y, w.x, w.y, q);
        if (ACC) {
            const ulonglong2 a = out[pi];
            r.x = csub(r.x + a.x, q);
            r.y = csub(r.y + a.y, q);
        }
        out[pi] = r;
    }
}

__global__ void k_permute(const uint64_t *__restrict__ in, uint64_t *__restrict__ out,
                          const uint32_t *__restrict__ tab, int logn, size_t total)
{
    const size_t mask = ((size_t)1 << logn) - 1;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t base = t & ~mask;
        out[t] = in[base + tab[t & mask]];
    }
}

}  // namespace

static size_t pairs_of(const Context &c, int polys, int limbs) { return ((size_t)polys * limbs * c.n) >> 1; }

void poly_add(const Context &c, const uint64_t *a, const uint64_t *b, int polys, int limbs, uint64_t *out,
              cudaStream_t s)
{
    size_t pr = pairs_of(c, polys, limbs);
    k_add_sub<<<grid_for(pr), kBlock, 0, s>>>((const ulonglong2 *)a, (const ulonglong2 *)b, (ulonglong2 *)out, c.d_pc,
                                               limbs, c.logn, pr, 0); NEXUS_LAUNCHED();
}

void poly_sub(const Context &c, const uint64_t *a, const uint64_t *b, int polys, int limbs, uint64_t *out,
              cudaStream_t s)
{
    size_t pr = pairs_of(c, polys, limbs);
    k_add_sub<<<grid_for(pr), kBlock, 0, s>>>((const ulonglong2 *)a, (const ulonglong2 *)b, (ulonglong2 *)out, c.d_pc,
                                               limbs, c.logn, pr, 1); NEXUS_LAUNCHED();
}

void poly_negate(const Context &c, const uint64_t *a, int polys, int limbs, uint64_t *out, cudaStream_t s)
{
    size_t pr = pairs_of(c, polys, limbs);
    k_negate<<<grid_for(pr), kBlock, 0, s>>>((const ulonglong2 *)a, (ulonglong2 *)out, c.d_pc, limbs, c.logn, pr); NEXUS_LAUNCHED();
}

void poly_mul_plain(const Context &c, const uint64_t *ct, int polys, int limbs, const uint64_t *pt, uint64_t *out,
                    cudaStream_t s)
{
    size_t pr = pairs_of(c, polys, limbs);
    k_plain<<<grid_for(pr), kBlock, 0, s>>>((const ulonglong2 *)ct, (const ulonglong2 *)pt, (ulonglong2 *)out, c.d_pc,
                                             limbs, c.logn, pr, 0); NEXUS_LAUNCHED();
}

void poly_mac_plain(const Context &c, const uint64_t *const *cts, const uint64_t *const *pts, int count, int limbs,
                    uint64_t *out, cudaStream_t s, int batch)
{
    if (count < 1 || count > kMacTerms) throw std::invalid_argument("poly_mac_plain: 1..16 terms");
    MacTerms t{};
    for (int j = 0; j < count; ++j) {
        t.ct[j] = cts[j];
        t.pt[j] = pts[j];
    }
    const size_t total = ((size_t)limbs << c.logn) * (size_t)batch;
    const unsigned grid = (unsigned)std::min<size_t>((total + kBlock - 1) / kBlock, 152 * 8);
    k_mac_plain<<<grid, kBlock, 0, s>>>(t, count, out, c.d_pc, limbs, c.logn, total); NEXUS_LAUNCHED();
}

void poly_add_plain(const Context &c, const uint64_t *ct, int polys, int limbs, const uint64_t *pt, int sub,
                    uint64_t *out, cudaStream_t s)
{
    size_t pr = pairs_of(c, polys, limbs);
    k_plain<<<grid_for(pr), kBlock, 0, s>>>((const ulonglong2 *)ct, (const ulonglong2 *)pt, (ulonglong2 *)out, c.d_pc,
                                             limbs, c.logn, pr, sub ? 2 : 1); NEXUS_LAUNCHED();
}

void poly_mul_scalar(const Context &c, const uint64_t *ct, int polys, int limbs, const uint64_t *scalars,
                     uint64_t *out, cudaStream_t s)
{
    // host scalars (already reduced mod q_l) travel as a kernel parameter
    if (limbs > 64) throw std::invalid_argument("at most 64 limbs");
    LimbScalars w;
    for (int l = 0; l < limbs; ++l) w.w[l] = make_ulonglong2(scalars[l], host_shoup(scalars[l], c.q[l]));
    size_t pr = pairs_of(c, polys, limbs);
    k_mul_scalar<<<grid_for(pr), kBlock, 0, s>>>((const ulonglong2 *)ct, w, (ulonglong2 *)out, c.d_pc, limbs, c.logn,
                                                  pr); NEXUS_LAUNCHED();
}

void poly_add_scalar(const Context &c, const uint64_t *in, int limbs, const uint64_t *scalars, int sub, uint64_t *out,
                     cudaStream_t s, int batch, size_t stride_words)
{
    if (limbs > 64) throw std::invalid_argument("at most 64 limbs");
    LimbScalars w;
    for (int l = 0; l < limbs; ++l) w.w[l] = make_ulonglong2(scalars[l], 0);
    const size_t pp = pairs_of(c, 1, limbs);
    const size_t stride = stride_words ? stride_words / 2 : pp;
    const size_t total = pp * (size_t)batch;
    k_add_scalar<<<grid_for(total), kBlock, 0, s>>>((const ulonglong2 *)in, w, (ulonglong2 *)out, c.d_pc, c.logn, pp,
                                                     sub, stride, total); NEXUS_LAUNCHED();
}

void tensor(const Context &c, const uint64_t *a, const uint64_t *b, int limbs, uint64_t *out3, cudaStream_t s,
            int batch)
{
    size_t pr = pairs_of(c, batch, limbs);
    k_tensor<<<grid_for(pr), kBlock, 0, s>>>((const ulonglong2 *)a, (const ulonglong2 *)b, (ulonglong2 *)out3, c.d_pc,
                                              limbs, c.logn, pr); NEXUS_LAUNCHED();
}

void rescale(const Context &c_in, const uint64_t *in, int size, int limbs, uint64_t *out, cudaStream_t s)
{
    if (limbs < 2) throw std::invalid_argument("rescale needs at least two limbs");
    Context &c = const_cast<Context &>(c_in);
    const size_t n = c.n;
    uint64_t *last = c.get_scratch((size_t)size * n * limbs);
    uint64_t *t = last + (size_t)size * n;
    size_t pr = ((size_t)size * n) >> 1;
    k_gather_limb<<<grid_for(pr), kBlock, 0, s>>>((const ulonglong2 *)in, (ulonglong2 *)last, limbs, limbs - 1, c.logn,
                                                   pr); NEXUS_LAUNCHED();
    ntt_inverse(c, last, size, LimbMap{1, limbs - 1, -1}, s);
    // rounding spread fused into the first pass of the forward NTT
    NttLoader ld;
    ld.kind = 2;
    ld.src = last;
    ld.group = limbs - 1;
    ld.special = limbs - 1;
    ntt_forward_loaded(c, t, size, LimbMap{limbs - 1, 0, -1}, ld, s);
    pr = pairs_of(c, size, limbs - 1);
    k_rescale_finish<<<grid_for(pr), kBlock, 0, s>>>((const ulonglong2 *)in, (const ulonglong2 *)t, (ulonglong2 *)out,
                                                      c.d_pc, c.d_inv_q + (size_t)(limbs - 1) * c.k, limbs, c.logn,
                                                      pr); NEXUS_LAUNCHED();
}

void rescale_scaled(const Context &c_in, const uint64_t *in, int size, int limbs, const uint64_t *scalars,
                    uint64_t *out, cudaStream_t s, bool accumulate)
{
    if (limbs < 2) throw std::invalid_argument("rescale needs at least two limbs");
    if (limbs > 64) throw std::invalid_argument("at most 64 limbs");
    Context &c = const_cast<Context &>(c_in);
    LimbScalars w;
    for (int l = 0; l < limbs; ++l) w.w[l] = make_ulonglong2(scalars[l], host_shoup(scalars[l], c.q[l]));
    const size_t n = c.n;
    uint64_t *last = c.get_scratch((size_t)size * n * limbs);
    uint64_t *t = last + (size_t)size * n;
    size_t pr = ((size_t)size * n) >> 1;
    k_gather_limb_scaled<<<grid_for(pr), kBlock, 0, s>>>((const ulonglong2 *)in, (ulonglong2 *)last, w, c.d_pc, limbs,
                                                          limbs - 1, c.logn, pr); NEXUS_LAUNCHED();
    ntt_inverse(c, last, size, LimbMap{1, limbs - 1, -1}, s);
    NttLoader ld;
    ld.kind = 2;
    ld.src = last;
    ld.group = limbs - 1;
    ld.special = limbs - 1;
    ntt_forward_loaded(c, t, size, LimbMap{limbs - 1, 0, -1}, ld, s);
    pr = pairs_of(c, size, limbs - 1);
    if (accumulate)
        k_rescale_finish_scaled<true><<<grid_for(pr), kBlock, 0, s>>>(
            (const ulonglong2 *)in, (const ulonglong2 *)t, (ulonglong2 *)out, w, c.d_pc,
            c.d_inv_q + (size_t)(limbs - 1) * c.k, limbs, c.logn, pr);
    else
        k_rescale_finish_scaled<false><<<grid_for(pr), kBlock, 0, s>>>(
            (const ulonglong2 *)in, (const ulonglong2 *)t, (ulonglong2 *)out, w, c.d_pc,
            c.d_inv_q + (size_t)(limbs - 1) * c.k, limbs, c.logn, pr);
    NEXUS_LAUNCHED();
}

void galois_permute(Context &c, const uint64_t *in, int polys, int limbs, uint32_t elt, uint64_t *out,
                    cudaStream_t s)
{
    const uint32_t *tab = c.galois_table(elt);
    size_t tot = (size_t)polys * limbs * c.n;
    k_permute<<<grid_for(tot), kBlock, 0, s>>>(in, out, tab, c.logn, tot); NEXUS_LAUNCHED();
}

}  // namespace nexus
