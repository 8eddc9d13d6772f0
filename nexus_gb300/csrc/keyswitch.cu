// Key switching with one special prime and one digit per data prime, the
// decomposition of SEAL's Evaluator::switch_key_inplace (evaluator.cpp:2724-3022
// in SEAL-4.1-bs), so the output words equal SEAL's.
//
//   1. INTT of the target's l limbs (coefficient form, each in [0, q_j)).
//   2. ModUp: digit j is reduced into every prime of {q_0..q_{l-1}, p} and
//      transformed: D[j][i] = NTT_i(t_j mod q_i).  For i == j this is the
//      target limb itself, which SEAL reuses; it is copied, not transformed.
//   3. Inner product with the key, 128-bit accumulation, one Barrett
//      reduction: P[k][i] = sum_j D[j][i] * key[j][k][i] mod q_i.
//   4. ModDown with rounding: ct[k][i] += (P[k][i] - NTT_i(((INTT_p(P[k][p]) + p/2)
//      mod p) - p/2)) * p^{-1} mod q_i.
#include <cstdint>
#include <algorithm>
#include <stdexcept>
#include <string>
#include <vector>
#include <cooperative_groups.h>

#include "context.h"
#include "ntt.h"
#include "ops.h"

namespace nexus {

namespace {

constexpr int kBlock = 256;

inline unsigned grid_for(size_t n)
{
    size_t g = (n + kBlock - 1) / kBlock;
    return (unsigned)(g > 1048576 ? 1048576 : g);
}

// D[b][j][j] = t[b][j] for the rows of t (B*l rows, row = b*l + j): digit j's
// own limb of the ModUp is the NTT-form target limb, as in SEAL
__global__ void k_modup_diag(const ulonglong2 *__restrict__ t, ulonglong2 *__restrict__ D, int l, int logn,
                             size_t total)
{
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const size_t row = x >> (logn - 1);
        const size_t n2 = x & (((size_t)1 << (logn - 1)) - 1);
        const size_t j = row % (size_t)l;
        D[((row * (size_t)(l + 1) + j) << (logn - 1)) + n2] = t[x];
    }
}

__device__ __forceinline__ void mac128(uint64_t &lo, uint64_t &hi, uint64_t a, uint64_t b)
{
    asm("mad.lo.cc.u64 %0, %2, %3, %0;\n\tmadc.hi.u64 %1, %2, %3, %1;" : "+l"(lo), "+l"(hi) : "l"(a), "l"(b));
}


// P[b][k][i'][n] = sum_j D[b][j][i'][n] * key[j][k][kidx(i')][n] mod q(i')
// One CTA covers 512 coefficients (two per thread, 16-byte loads) of one
// (b, i') pair; CTAs run prime-major, then by ciphertext, with the coefficient
// chunk fastest: neighbouring CTAs read neighbouring 4 KB pieces of the same
// D rows (few pages in flight), and a prime's key rows (2l limbs) are read
// by the B ciphertexts one after another while they are still in L2.  The
// kernel is bound by its D stream and its 32 x 32 -> 64 multiplies together
// (three per product on the small-prime path); the register cap keeps four
// CTAs (32 warps) per SM in flight there, three with 128-bit accumulators.
constexpr int kInnerCoeffs = 2 * kBlock;

template <bool SPLIT>
__global__ void __launch_bounds__(kBlock, SPLIT ? 4 : 3)
    k_ks_inner(const uint64_t *__restrict__ D, const uint64_t *__restrict__ key, uint64_t *__restrict__ P,
               const PrimeConst *__restrict__ pc, int l, int K, int logn, int B, unsigned nblocks)
{
    const int log_chunks = logn - 9;
    for (unsigned blk = blockIdx.x; blk < nblocks; blk += gridDim.x) {
        const unsigned chunk = blk & ((1u << log_chunks) - 1), rest = blk >> log_chunks;
        const unsigned b = rest % (unsigned)B;
        const int i = (int)(rest / (unsigned)B);
        const size_t n = ((size_t)chunk * kInnerCoeffs) + 2 * threadIdx.x;
        const int kidx = (i == l) ? K - 1 : i;
        const PrimeConst P0 = pc[kidx];
        const ulonglong2 *d =
            reinterpret_cast<const ulonglong2 *>(D + (((size_t)b * l * (l + 1) + i) << logn) + n);
        const ulonglong2 *k0 = reinterpret_cast<const ulonglong2 *>(key + ((size_t)kidx << logn) + n);
        const size_t dstride = ((size_t)(l + 1) << logn) >> 1;   // in ulonglong2
        const size_t kstride = ((size_t)2 * K << logn) >> 1;
        const size_t kcomp = ((size_t)K << logn) >> 1;
        uint64_t *pb = P + (((size_t)b * 2 * (l + 1)) << logn) + n;
        ulonglong2 r0, r1;
        if (SPLIT) {
            // every residue below 2^52: each product from three 32 x 32 -> 64
            // products of its 26-bit halves (mac_split), summed exactly in
            // three 64-bit accumulators, one reduction at the end; the
            // inner product is bound by these wide multiplies
            uint64_t h[4] = {0, 0, 0, 0}, x[4] = {0, 0, 0, 0}, w[4] = {0, 0, 0, 0};
            // D is read once: streaming loads keep the key rows in L2
#pragma unroll 2
            for (int j = 0; j < l; ++j) {
                const ulonglong2 dv = __ldcs(d + j * dstride);
                const ulonglong2 ka = k0[j * kstride], kb = k0[j * kstride + kcomp];
                const uint64_t dd[2] = {dv.x, dv.y}, aa[4] = {ka.x, ka.y, kb.x, kb.y};
#pragma unroll
                for (int e = 0; e < 4; ++e) mac_split(h[e], x[e], w[e], dd[e & 1], aa[e]);
            }
            r0 = make_ulonglong2(reduce_karatsuba(h[0], x[0], w[0], P0), reduce_karatsuba(h[1], x[1], w[1], P0));
            r1 = make_ulonglong2(reduce_karatsuba(h[2], x[2], w[2], P0), reduce_karatsuba(h[3], x[3], w[3], P0));
        } else {
            uint64_t lo[4] = {0, 0, 0, 0}, hi[4] = {0, 0, 0, 0};
#pragma unroll 2
            for (int j = 0; j < l; ++j) {
                const ulonglong2 dv = d[j * dstride];
                const ulonglong2 ka = k0[j * kstride], kb = k0[j * kstride + kcomp];
                mac128(lo[0], hi[0], dv.x, ka.x);
                mac128(lo[1], hi[1], dv.y, ka.y);
                mac128(lo[2], hi[2], dv.x, kb.x);
                mac128(lo[3], hi[3], dv.y, kb.y);
            }
            r0 = make_ulonglong2(barrett_128(lo[0], hi[0], P0.q, P0.r0, P0.r1),
                                 barrett_128(lo[1], hi[1], P0.q, P0.r0, P0.r1));
            r1 = make_ulonglong2(barrett_128(lo[2], hi[2], P0.q, P0.r0, P0.r1),
                                 barrett_128(lo[3], hi[3], P0.q, P0.r0, P0.r1));
        }
        *reinterpret_cast<ulonglong2 *>(pb + ((size_t)i << logn)) = r0;
        *reinterpret_cast<ulonglong2 *>(pb + ((size_t)(l + 1 + i) << logn)) = r1;
    }
}

// launch of k_ks_inner over B ciphertexts at l limbs
void launch_ks_inner(const Context &c, const uint64_t *D, const uint64_t *key, uint64_t *P, int l, int B,
                     cudaStream_t s)
{
    static_assert(kInnerCoeffs == 512, "k_ks_inner maps 512 coefficients to a CTA");
    if (c.logn < 9) throw std::invalid_argument("key switching needs N >= 512");
    const unsigned nb = (unsigned)((size_t)B * (l + 1) << (c.logn - 9));
    unsigned grid = nb;
    if (c.tune.ks_inner_ctas_per_sm > 0 && c.sm_count > 0)
        grid = std::min(nb, (unsigned)(c.tune.ks_inner_ctas_per_sm * c.sm_count));
    if (c.small_primes && l <= 31)
        k_ks_inner<true><<<grid, kBlock, 0, s>>>(D, key, P, c.d_pc, l, c.k, c.logn, B, nb);
    else
        k_ks_inner<false><<<grid, kBlock, 0, s>>>(D, key, P, c.d_pc, l, c.k, c.logn, B, nb);
    NEXUS_LAUNCHED();
}

// ct[kb][i] += (P[kb][i] - T[kb][i]) * p^{-1} mod q_i with kb = 2*b + k over the
// batch; T[kb][i] in [0, q_i)
__global__ void k_moddown_finish(uint64_t *__restrict__ ct, const uint64_t *__restrict__ P,
                                 const uint64_t *__restrict__ T, const PrimeConst *__restrict__ pc,
                                 const ulonglong2 *__restrict__ inv_p, int l, int logn, size_t total)
{
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const size_t row = x >> logn;             // k*l + i
        const size_t n = x & (((size_t)1 << logn) - 1);
        const int k = (int)(row / l), i = (int)(row % l);
        const uint64_t q = pc[i].q;
        const ulonglong2 w = inv_p[i];
        const uint64_t pv = P[(((size_t)k * (l + 1) + i) << logn) + n];
        const uint64_t v = mul_shoup(pv + q - T[x], w.x, w.y, q);
        ct[x] = csub(ct[x] + v, q);
    }
}

// the key-switch targets of a Galois automorphism: t[b][j][n] = ct[b][1][j][tab[n]]
__global__ void k_galois_target(const uint64_t *__restrict__ ct, const uint32_t *__restrict__ tab,
                                uint64_t *__restrict__ t, int l, int logn, size_t total)
{
    const size_t N = (size_t)1 << logn, poly = (size_t)l << logn;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const size_t b = x / poly, r = x - b * poly;
        t[x] = ct[(2 * b + 1) * poly + (r & ~(N - 1)) + tab[r & (N - 1)]];
    }
}

// the automorphism's result: out[b][k][i][n] = (k == 0 ? ct[b][0][i][tab[n]] : 0)
//   + (P[b][k][i][n] - T[b][k][i][n]) * p^{-1} mod q_i
__global__ void k_galois_finish(const uint64_t *__restrict__ ct, const uint32_t *__restrict__ tab,
                                const uint64_t *__restrict__ P, const uint64_t *__restrict__ T,
                                const PrimeConst *__restrict__ pc, const ulonglong2 *__restrict__ inv_p, int l,
                                int logn, size_t total, uint64_t *__restrict__ out)
{
    const size_t N = (size_t)1 << logn;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const size_t row = x >> logn, n = x & (N - 1);     // (b * 2 + k) * l + i
        const size_t bk = row / (size_t)l;
        const int i = (int)(row - bk * (size_t)l);
        const uint64_t q = pc[i].q;
        const ulonglong2 w = inv_p[i];
        const uint64_t pv = P[((bk * (size_t)(l + 1) + (size_t)i) << logn) + n];
        uint64_t v = mul_shoup(pv + q - T[x], w.x, w.y, q);
        if ((bk & 1) == 0) v = csub(v + ct[((bk * (size_t)l + (size_t)i) << logn) + tab[n]], q);
        out[x] = v;
    }
}

// relinearisation's result: out[b][k][i][n] = ct3[b][k][i][n]
//   + (P[b][k][i][n] - T[b][k][i][n]) * p^{-1} mod q_i
__global__ void k_relin_finish(const uint64_t *__restrict__ ct3, const uint64_t *__restrict__ P,
                               const uint64_t *__restrict__ T, const PrimeConst *__restrict__ pc,
                               const ulonglong2 *__restrict__ inv_p, int l, int logn, size_t total,
                               uint64_t *__restrict__ out)
{
    const size_t N = (size_t)1 << logn;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const size_t row = x >> logn, n = x & (N - 1);     // (b * 2 + k) * l + i
        const size_t bk = row / (size_t)l;
        const int i = (int)(row - bk * (size_t)l);
        const size_t b = bk >> 1, k = bk & 1;
        const uint64_t q = pc[i].q;
        const ulonglong2 w = inv_p[i];
        const uint64_t pv = P[((bk * (size_t)(l + 1) + (size_t)i) << logn) + n];
        const uint64_t v = mul_shoup(pv + q - T[x], w.x, w.y, q);
        out[x] = csub(v + ct3[(((b * 3 + k) * (size_t)l + (size_t)i) << logn) + n], q);
    }
}

}  // namespace

// Stage 1 (ModUp + inner product) of a batched key switch.  t [B][l][N]
// holds the targets in NTT form and is overwritten (inverse-transformed in
// place); D is scratch of B*l*(l+1) limbs; P [B][2][l+1][N] receives the
// inner products.
void ks_modup_inner(Context &c, uint64_t *t, int B, int l, const uint64_t *key, uint64_t *D, uint64_t *P,
                    cudaStream_t s)
{
    const size_t N = c.n, Bs = (size_t)B;
    const int sp = c.k - 1;
    // digit j's limb j is the target limb itself (SEAL reuses it for CKKS):
    // copy it across and leave it out of the forward transform
    const size_t pairs = Bs * l * N / 2;
    k_modup_diag<<<grid_for(pairs), kBlock, 0, s>>>(reinterpret_cast<const ulonglong2 *>(t),
                                                    reinterpret_cast<ulonglong2 *>(D), l, c.logn, pairs);
    NEXUS_LAUNCHED();
    ntt_inverse(c, t, Bs, LimbMap{l, 0, -1}, s);
    // ModUp spread fused into the first pass of the forward NTT
    NttLoader ld;
    ld.kind = 1;
    ld.src = t;
    ld.group = l;
    ld.src_limbs = l;
    ntt_forward_loaded(c, D, Bs * l, LimbMap{l, 0, sp, 1}, ld, s);
    launch_ks_inner(c, D, key, P, l, B, s);
}

// The ModDown rounding terms T [B][2][l][N] from the special limbs already
// gathered into `last` [B][2][N] (inverse-transformed in place).
static void ks_moddown_terms_from_last(Context &c, int B, int l, uint64_t *T, uint64_t *last, cudaStream_t s)
{
    const size_t Bs = (size_t)B;
    const int sp = c.k - 1;
    ntt_inverse(c, last, 2 * Bs, LimbMap{1, sp, -1}, s);
    // rounding spread fused into the first pass of the forward NTT
    NttLoader ld;
    ld.kind = 2;
    ld.src = last;
    ld.group = l;
    ld.special = sp;
    ntt_forward_loaded(c, T, 2 * Bs, LimbMap{l, 0, -1}, ld, s);
}

// Stage 2: the rounding terms T [B][2][l][N] of the ModDown from the special
// limbs of P; `last` is scratch of 2B limbs.
void ks_moddown_terms(Context &c, const uint64_t *P, int B, int l, uint64_t *T, uint64_t *last, cudaStream_t s)
{
    const size_t N = c.n, Bs = (size_t)B;
    cudaMemcpy2DAsync(last, N * 8, P + (size_t)l * N, (size_t)(l + 1) * N * 8, N * 8, 2 * Bs,
                      cudaMemcpyDeviceToDevice, s);
    ks_moddown_terms_from_last(c, B, l, T, last, s);
}

void switch_key_batch(Context &c, uint64_t *ct, int batch, int l, const uint64_t *target, const uint64_t *key,
                      cudaStream_t s, size_t target_pitch)
{
    if (l < 1 || l > c.k - 1) throw std::invalid_argument("switch_key: level out of range");
    if (batch < 1) return;
    if (reinterpret_cast<uintptr_t>(key) & 15) throw std::invalid_argument("switch_key: the key must be 16-byte aligned");
    const size_t N = c.n, B = (size_t)batch;
    const int sp = c.k - 1;
    // scratch per ciphertext: t[l] | D[l][l+1] | P[2][l+1] | T[2][l] | last[2]
    const size_t words = B * N * ((size_t)l + (size_t)l * (l + 1) + 2 * (size_t)(l + 1) + 2 * (size_t)l + 2);
    uint64_t *t = c.get_scratch(words);
    uint64_t *D = t + B * l * N;
    uint64_t *P = D + B * l * (l + 1) * N;
    uint64_t *T = P + B * 2 * (l + 1) * N;
    uint64_t *last = T + B * 2 * l * N;

    if (target_pitch == 0 || target_pitch == (size_t)l * N)
        cudaMemcpyAsync(t, target, sizeof(uint64_t) * B * l * N, cudaMemcpyDeviceToDevice, s);
    else
        cudaMemcpy2DAsync(t, sizeof(uint64_t) * l * N, target, sizeof(uint64_t) * target_pitch,
                          sizeof(uint64_t) * l * N, B, cudaMemcpyDeviceToDevice, s);
    ks_modup_inner(c, t, batch, l, key, D, P, s);
    ks_moddown_terms(c, P, batch, l, T, last, s);
    const size_t tot = B * 2 * l * N;
    k_moddown_finish<<<grid_for(tot), kBlock, 0, s>>>(ct, P, T, c.d_pc, c.d_inv_q + (size_t)sp * c.k, l, c.logn, tot); NEXUS_LAUNCHED();
}

void switch_key(Context &c, uint64_t *ct, int l, const uint64_t *target, const uint64_t *key, cudaStream_t s)
{
    switch_key_batch(c, ct, 1, l, target, key, s);
}

void relinearize_batch(Context &c, const uint64_t *ct3, int B, int l, const uint64_t *key, uint64_t *out2,
                       cudaStream_t s)
{
    if (l < 1 || l > c.k - 1) throw std::invalid_argument("relinearize: level out of range");
    if (B < 1) return;
    if (reinterpret_cast<uintptr_t>(key) & 15) throw std::invalid_argument("relinearize: the key must be 16-byte aligned");
    const size_t N = c.n, Bs = (size_t)B, poly = (size_t)l * N;
    const int sp = c.k - 1;
    // scratch per ciphertext: t[l] | D[l][l+1] | P[2][l+1] | T[2][l] | last[2]
    const size_t words = Bs * N * ((size_t)l + (size_t)l * (l + 1) + 2 * (size_t)(l + 1) + 2 * (size_t)l + 2);
    uint64_t *t = c.get_scratch(words);
    uint64_t *D = t + Bs * l * N;
    uint64_t *P = D + Bs * l * (l + 1) * N;
    uint64_t *T = P + Bs * 2 * (l + 1) * N;
    uint64_t *last = T + Bs * 2 * l * N;
    // c2 of every ciphertext is the key-switch target
    cudaMemcpy2DAsync(t, sizeof(uint64_t) * poly, ct3 + 2 * poly, sizeof(uint64_t) * 3 * poly, sizeof(uint64_t) * poly,
                      Bs, cudaMemcpyDeviceToDevice, s);
    ks_modup_inner(c, t, B, l, key, D, P, s);
    ks_moddown_terms(c, P, B, l, T, last, s);
    const size_t tot = Bs * 2 * poly;
    k_relin_finish<<<grid_for(tot), kBlock, 0, s>>>(ct3, P, T, c.d_pc, c.d_inv_q + (size_t)sp * c.k, l, c.logn, tot,
                                                     out2);
    NEXUS_LAUNCHED();
}

void relinearize(Context &c, const uint64_t *ct3, int l, const uint64_t *key, uint64_t *out2, cudaStream_t s)
{
    const size_t words = (size_t)2 * l * c.n;
    if (out2 + words <= ct3 || ct3 + 3 * (size_t)l * c.n <= out2) {
        relinearize_batch(c, ct3, 1, l, key, out2, s);
        return;
    }
    // in place (out2 overlaps ct3): the finishing kernel reads ct3, so it
    // writes a temporary that is copied back
    uint64_t *tmp = nullptr;
    if (cudaMallocAsync(&tmp, sizeof(uint64_t) * words, s) != cudaSuccess) throw std::runtime_error("cudaMallocAsync");
    relinearize_batch(c, ct3, 1, l, key, tmp, s);
    cudaMemcpyAsync(out2, tmp, sizeof(uint64_t) * words, cudaMemcpyDeviceToDevice, s);
    cudaFreeAsync(tmp, s);
}

void apply_galois_batch(Context &c, const uint64_t *ct, int B, int l, uint32_t elt, const uint64_t *key,
                        uint64_t *out, cudaStream_t s)
{
    if (l < 1 || l > c.k - 1) throw std::invalid_argument("apply_galois: level out of range");
    if (B < 1) return;
    if (reinterpret_cast<uintptr_t>(key) & 15) throw std::invalid_argument("apply_galois: the key must be 16-byte aligned");
    const size_t N = c.n, Bs = (size_t)B;
    const int sp = c.k - 1;
    // scratch per ciphertext: t[l] | D[l][l+1] | P[2][l+1] | T[2][l] | last[2]
    const size_t words = Bs * N * ((size_t)l + (size_t)l * (l + 1) + 2 * (size_t)(l + 1) + 2 * (size_t)l + 2);
    uint64_t *t = c.get_scratch(words);
    uint64_t *D = t + Bs * l * N;
    uint64_t *P = D + Bs * l * (l + 1) * N;
    uint64_t *T = P + Bs * 2 * (l + 1) * N;
    uint64_t *last = T + Bs * 2 * l * N;
    const uint32_t *tab = c.galois_table(elt);
    size_t tot = Bs * l * N;
    k_galois_target<<<grid_for(tot), kBlock, 0, s>>>(ct, tab, t, l, c.logn, tot);
    NEXUS_LAUNCHED();
    ks_modup_inner(c, t, B, l, key, D, P, s);
    ks_moddown_terms(c, P, B, l, T, last, s);
    tot = Bs * 2 * l * N;
    k_galois_finish<<<grid_for(tot), kBlock, 0, s>>>(ct, tab, P, T, c.d_pc, c.d_inv_q + (size_t)sp * c.k, l, c.logn,
                                                      tot, out);
    NEXUS_LAUNCHED();
}

void apply_galois(Context &c, const uint64_t *ct, int l, uint32_t elt, const uint64_t *key, uint64_t *out,
                  cudaStream_t s)
{
    apply_galois_batch(c, ct, 1, l, elt, key, out, s);
}

}  // namespace nexus

// ---------------------------------------------------------------------------
// Hoisted rotations: several Galois elements applied to one batch of
// ciphertexts share one ModUp of c1.
//
// For the automorphism sigma_g the key-switch target of a rotation is
// pi_g(c1) (pi_g the NTT-domain permutation), whose coefficient form is the
// signed permutation of t_j = INTT_j(c1_j): a coefficient that lands on a
// negated position becomes q_j - a.  Reduced into another prime q_i that is
// (q_j mod q_i) - (a mod q_i), so when no coefficient of t is zero
//
//   ModUp(pi_g(c1))[j][i] = pi_g(D[j][i]) + (q_j mod q_i) * M_g[i],
//
// with D the ModUp of c1 itself and M_g[i] the NTT of the 0/1 polynomial of
// negated positions.  The key inner product of a rotation is then
//
//   P[k][i][n] = Ptil[k][i][pi_g(n)] + Corr_g[k][i][n],
//   Ptil = sum_j D[j][i] * Kperm[j][k][i],   Kperm[..][pi_g(n)] = K_g[..][n],
//   Corr_g[k][i] = M_g[i] * sum_j (q_j mod q_i) * K_g[j][k][i]   (mod q_i),
//
// the same residues as the inner product of the rotated target, so the
// ModDown and the output words are the ones apply_galois gives.  A zero
// coefficient in t (probability about l*N/q per ciphertext for random data,
// certain for a trivial c1) breaks the identity: a negated zero is 0, not
// q_j.  hoist_decompose marks each ciphertext that has one in a device flag,
// and hoist_fix, one cooperative launch after the group's hoisted rotations,
// recomputes every rotation of the marked ciphertexts by the ordinary key
// switch; when nothing is marked its CTAs return at once.  Nothing waits on
// the host.

namespace nexus {

namespace {

// flag[b] = 1 when member b's rows of t (`per` words each) hold a zero
__global__ void k_any_zero(const uint64_t *__restrict__ t, size_t total, size_t per, int *flag)
{
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x)
        if (t[x] == 0) flag[x / per] = 1;
}

// out[p][pos] = 1 where the automorphism X -> X^elt negates the coefficient
// it moves to pos, else 0; the same 0/1 polynomial in each of the `limbs` rows
__global__ void k_galois_mask(uint64_t *__restrict__ out, uint32_t elt, int logn, int limbs)
{
    const size_t N = (size_t)1 << logn;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < N; x += (size_t)gridDim.x * blockDim.x) {
        const uint64_t raw = (x * (uint64_t)elt) & (2 * N - 1);
        if (raw >= N)
            for (int p = 0; p < limbs; ++p) out[p * N + (raw - N)] = 1;
    }
}

// out[row][tab[n]] = in[row][n] for every N-word row
__global__ void k_scatter_rows(const uint64_t *__restrict__ in, uint64_t *__restrict__ out,
                               const uint32_t *__restrict__ tab, int logn, size_t total)
{
    const size_t mask = ((size_t)1 << logn) - 1;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x)
        out[(x & ~mask) + tab[x & mask]] = in[x];
}

// Corr[k][i][n] = M[kidx(i)][n] * sum_{j<l} (q_j mod q_kidx) * key[j][k][kidx(i)][n] mod q_kidx
__global__ void k_hoist_corr(const uint64_t *__restrict__ key, const uint64_t *__restrict__ M,
                             const PrimeConst *__restrict__ pc, int l, int K, int logn, uint64_t *__restrict__ out)
{
    const size_t N = (size_t)1 << logn, total = (size_t)2 * (l + 1) * N;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const size_t row = x >> logn, n = x & (N - 1);
        const int k = (int)(row / (size_t)(l + 1)), i = (int)(row % (size_t)(l + 1));
        const int kidx = (i == l) ? K - 1 : i;
        const PrimeConst P = pc[kidx];
        uint64_t lo = 0, hi = 0;
        for (int j = 0; j < l; ++j) {
            const uint64_t qj = pc[j].q;
            const uint64_t c = (qj >= P.q) ? barrett_64(qj, P.q, P.r1) : qj;
            mac128(lo, hi, c, key[(((size_t)j * 2 + k) * K + kidx) * N + n]);
        }
        const uint64_t s = barrett_128(lo, hi, P.q, P.r0, P.r1);
        out[x] = mul_mod(s, M[(size_t)kidx * N + n], P.q, P.r0, P.r1);
    }
}

// last[b][k][n] = Ptil[b][k][l][tab[n]] + Corr[k][l][n] mod p: the special
// limbs of the rotation's inner product, which the ModDown's INTT needs first
__global__ void k_hoist_special(const uint64_t *__restrict__ Pt, const uint64_t *__restrict__ corr,
                                const uint32_t *__restrict__ tab, const PrimeConst *__restrict__ pc, int l, int K,
                                int logn, size_t total, uint64_t *__restrict__ last)
{
    const size_t N = (size_t)1 << logn;
    const uint64_t p = pc[K - 1].q;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const size_t row = x >> logn, n = x & (N - 1);     // b * 2 + k
        const size_t k = row & 1;
        const size_t prow = row * (size_t)(l + 1) + (size_t)l;
        last[x] = csub(Pt[(prow << logn) + tab[n]] + corr[((k * (size_t)(l + 1) + (size_t)l) << logn) + n], p);
    }
}

// The rotation's ModDown finish with the hoisted inner product read in
// place: out[b][k][i][n] = (k == 0 ? c0[b][i][tab[n]] : 0)
//   + (Ptil[b][k][i][tab[n]] + Corr[k][i][n] - T[b][k][i][n]) * p^{-1} mod q_i
__global__ void k_hoist_finish(const uint64_t *__restrict__ Pt, const uint64_t *__restrict__ corr,
                               const uint64_t *__restrict__ T, const uint64_t *__restrict__ ct, size_t ct_pitch,
                               const uint32_t *__restrict__ tab, const PrimeConst *__restrict__ pc,
                               const ulonglong2 *__restrict__ inv_p, int l, int logn, size_t total,
                               uint64_t *__restrict__ out)
{
    const size_t N = (size_t)1 << logn;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const size_t row = x >> logn, n = x & (N - 1);     // (b * 2 + k) * l + i
        const size_t bk = row / (size_t)l;
        const int i = (int)(row - bk * (size_t)l);
        const size_t b = bk >> 1, k = bk & 1;
        const uint64_t q = pc[i].q;
        const ulonglong2 w = inv_p[i];
        const size_t tn = tab[n];
        const uint64_t pv = csub(Pt[((bk * (size_t)(l + 1) + (size_t)i) << logn) + tn] +
                                     corr[((k * (size_t)(l + 1) + (size_t)i) << logn) + n], q);
        uint64_t v = mul_shoup(pv + q - T[x], w.x, w.y, q);
        if (k == 0) v = csub(v + ct[b * ct_pitch + ((size_t)i << logn) + tn], q);
        out[x] = v;
    }
}

}  // namespace

void hoist_decompose(Context &c, const uint64_t *c1, size_t c1_pitch, int B, int l, uint64_t *t, uint64_t *D,
                     int *d_flags, cudaStream_t s)
{
    const size_t N = c.n, Bs = (size_t)B;
    const int sp = c.k - 1;
    if (c1_pitch == 0 || c1_pitch == (size_t)l * N)
        cudaMemcpyAsync(t, c1, sizeof(uint64_t) * Bs * l * N, cudaMemcpyDeviceToDevice, s);
    else
        cudaMemcpy2DAsync(t, sizeof(uint64_t) * l * N, c1, sizeof(uint64_t) * c1_pitch, sizeof(uint64_t) * l * N, Bs,
                          cudaMemcpyDeviceToDevice, s);
    const size_t pairs = Bs * l * N / 2;
    k_modup_diag<<<grid_for(pairs), kBlock, 0, s>>>(reinterpret_cast<const ulonglong2 *>(t),
                                                    reinterpret_cast<ulonglong2 *>(D), l, c.logn, pairs);
    NEXUS_LAUNCHED();
    ntt_inverse(c, t, Bs, LimbMap{l, 0, -1}, s);
    cudaMemsetAsync(d_flags, 0, sizeof(int) * Bs, s);
    const size_t words = Bs * l * N;
    k_any_zero<<<grid_for(words), kBlock, 0, s>>>(t, words, (size_t)l * N, d_flags);
    NEXUS_LAUNCHED();
    NttLoader ld;
    ld.kind = 1;
    ld.src = t;
    ld.group = l;
    ld.src_limbs = l;
    ntt_forward_loaded(c, D, Bs * l, LimbMap{l, 0, sp, 1}, ld, s);
}

void hoist_galois_mask_ntt(Context &c, uint32_t elt, uint64_t *M, cudaStream_t s)
{
    const size_t N = c.n;
    cudaMemsetAsync(M, 0, sizeof(uint64_t) * c.k * N, s);
    k_galois_mask<<<grid_for(N), kBlock, 0, s>>>(M, elt, c.logn, c.k);
    NEXUS_LAUNCHED();
    ntt_forward(c, M, 1, LimbMap{c.k, 0, -1}, s);
}

void hoist_permute_key(Context &c, const uint64_t *key, uint32_t elt, uint64_t *out, cudaStream_t s)
{
    const size_t total = (size_t)(c.k - 1) * 2 * c.k * c.n;
    k_scatter_rows<<<grid_for(total), kBlock, 0, s>>>(key, out, c.galois_table(elt), c.logn, total);
    NEXUS_LAUNCHED();
}

void hoist_correction(Context &c, const uint64_t *key, const uint64_t *M, int l, uint64_t *out, cudaStream_t s)
{
    const size_t total = (size_t)2 * (l + 1) * c.n;
    k_hoist_corr<<<grid_for(total), kBlock, 0, s>>>(key, M, c.d_pc, l, c.k, c.logn, out);
    NEXUS_LAUNCHED();
}

void hoist_rotate(Context &c, const uint64_t *D, int B, int l, uint32_t elt, const uint64_t *perm_key,
                  const uint64_t *corr, const uint64_t *ct, size_t ct_pitch, uint64_t *out, cudaStream_t s)
{
    if (reinterpret_cast<uintptr_t>(perm_key) & 15) throw std::invalid_argument("hoist_rotate: unaligned key");
    const size_t N = c.n, Bs = (size_t)B;
    const int sp = c.k - 1;
    const size_t poly = (size_t)l * N;
    if (ct_pitch == 0) ct_pitch = 2 * poly;
    // scratch per ciphertext: Ptil[2][l+1] | T[2][l] | last[2]
    const size_t words = Bs * N * (2 * (size_t)(l + 1) + 2 * (size_t)l + 2);
    uint64_t *Pt = c.get_scratch(words);
    uint64_t *T = Pt + Bs * 2 * (l + 1) * N;
    uint64_t *last = T + Bs * 2 * l * N;
    launch_ks_inner(c, D, perm_key, Pt, l, B, s);
    const uint32_t *tab = c.galois_table(elt);
    const size_t tot_sp = Bs * 2 * N;
    k_hoist_special<<<grid_for(tot_sp), kBlock, 0, s>>>(Pt, corr, tab, c.d_pc, l, c.k, c.logn, tot_sp, last);
    NEXUS_LAUNCHED();
    ks_moddown_terms_from_last(c, B, l, T, last, s);
    const size_t tot = Bs * 2 * poly;
    k_hoist_finish<<<grid_for(tot), kBlock, 0, s>>>(Pt, corr, T, ct, ct_pitch, tab, c.d_pc,
                                                     c.d_inv_q + (size_t)sp * c.k, l, c.logn, tot, out);
    NEXUS_LAUNCHED();
}

// ---------------------------------------------------------------------------
// The exact fallback of a hoisted group, for the ciphertexts whose INTT(c1)
// has a zero coefficient.  One cooperative launch covers up to kFixMaxRot
// rotations of the group; its CTAs read the flags written by
// hoist_decompose and return when none is set.  Otherwise, for each marked
// ciphertext and each element, the grid runs the key switch of
// switch_key_inplace on the rotated target with grid-wide barriers between
// the steps: digit j of the target is the signed permutation of t_j (a
// negated zero stays 0), reduced into the l+1 primes, transformed by a
// radix-2 negacyclic NTT, multiplied into P with the unpermuted key; then
// the ModDown with rounding, and the permuted c0 added to the first
// polynomial.  Slow, rare, and word for word apply_galois.

namespace {

namespace cg = cooperative_groups;

constexpr int kFixMaxRot = 48;

struct HoistFixArgs {
    const uint64_t *t;        // [B][l][N], INTT of the c1 polynomials
    const uint64_t *ct;       // c0 of ciphertext b at ct + b * pitch
    size_t pitch;
    const int *flags;         // [B]
    const PrimeConst *pc;
    const ulonglong2 *tw_fwd, *tw_inv;
    const ulonglong2 *inv_p;  // p^{-1} mod q_i with its Shoup quotient
    uint64_t *U, *P, *V;      // scratch [l+1][N], [2][l+1][N], [N]
    int B, l, K, logn, R;
    uint32_t elt[kFixMaxRot];
    const uint64_t *key[kFixMaxRot];   // [K-1][2][K][N], as generated
    const uint32_t *tab[kFixMaxRot];   // NTT-domain permutation of elt
    uint64_t *out[kFixMaxRot];         // [B][2][l][N]
};

// prime of row r: fixed when >= 0, else the ModUp order q_0..q_{l-1}, p
__device__ __forceinline__ int fix_prime(int r, int fixed, int l, int K)
{
    return fixed >= 0 ? fixed : (r == l ? K - 1 : r);
}

// forward negacyclic NTT of `rows` rows of a, radix 2, one stage between
// grid barriers; input and output in [0, q)
__device__ void fix_ntt_forward(cg::grid_group &g, const HoistFixArgs &a, uint64_t *d, int rows, int fixed)
{
    const size_t N = (size_t)1 << a.logn, half = N >> 1;
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    for (int lm = 0; lm < a.logn; ++lm) {
        const size_t m = (size_t)1 << lm, t = half >> lm;
        for (size_t x = tid; x < (size_t)rows * half; x += stride) {
            const int r = (int)(x >> (a.logn - 1));
            const size_t b = x & (half - 1), i = b >> (a.logn - 1 - lm);
            const size_t idx = 2 * i * t + (b & (t - 1));
            const int p = fix_prime(r, fixed, a.l, a.K);
            const uint64_t q = a.pc[p].q;
            const ulonglong2 w = a.tw_fwd[(size_t)p * N + m + i];
            uint64_t *row = d + ((size_t)r << a.logn);
            const uint64_t X = row[idx], Y = mul_shoup(row[idx + t], w.x, w.y, q);
            row[idx] = csub(X + Y, q);
            row[idx + t] = csub(X + q - Y, q);
        }
        g.sync();
    }
}

// inverse of fix_ntt_forward (Gentleman-Sande stages, then n^{-1})
__device__ void fix_ntt_inverse(cg::grid_group &g, const HoistFixArgs &a, uint64_t *d, int rows, int fixed)
{
    const size_t N = (size_t)1 << a.logn, half = N >> 1;
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    for (int lm = a.logn - 1; lm >= 0; --lm) {
        const size_t m = (size_t)1 << lm, t = half >> lm;
        for (size_t x = tid; x < (size_t)rows * half; x += stride) {
            const int r = (int)(x >> (a.logn - 1));
            const size_t b = x & (half - 1), i = b >> (a.logn - 1 - lm);
            const size_t idx = 2 * i * t + (b & (t - 1));
            const int p = fix_prime(r, fixed, a.l, a.K);
            const uint64_t q = a.pc[p].q;
            const ulonglong2 w = a.tw_inv[(size_t)p * N + m + i];
            uint64_t *row = d + ((size_t)r << a.logn);
            const uint64_t X = row[idx], Y = row[idx + t];
            row[idx] = csub(X + Y, q);
            row[idx + t] = mul_shoup(X + q - Y, w.x, w.y, q);
        }
        g.sync();
    }
    for (size_t x = tid; x < ((size_t)rows << a.logn); x += stride) {
        const PrimeConst P = a.pc[fix_prime((int)(x >> a.logn), fixed, a.l, a.K)];
        d[x] = mul_shoup(d[x], P.inv_n, P.inv_n_q, P.q);
    }
    g.sync();
}

__global__ void __launch_bounds__(kBlock) k_hoist_fix(const HoistFixArgs a)
{
    bool any = false;
    for (int b = 0; b < a.B; ++b) any |= a.flags[b] != 0;
    if (!any) return;   // the same answer in every CTA: the flags were written by an earlier launch
    cg::grid_group g = cg::this_grid();
    const int l = a.l, K = a.K, logn = a.logn;
    const size_t N = (size_t)1 << logn;
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    const PrimeConst Psp = a.pc[K - 1];
    for (int b = 0; b < a.B; ++b) {
        if (!a.flags[b]) continue;
        const uint64_t *tb = a.t + (size_t)b * l * N;
        const uint64_t *c0 = a.ct + (size_t)b * a.pitch;
        for (int r = 0; r < a.R; ++r) {
            const uint64_t elt = a.elt[r];
            const uint64_t *key = a.key[r];
            for (size_t x = tid; x < (size_t)2 * (l + 1) * N; x += stride) a.P[x] = 0;
            g.sync();
            for (int j = 0; j < l; ++j) {
                // digit j of the rotated target: coefficient n of t_j moves to
                // n * elt mod 2N, negated (mod q_j) past N; reduced into every prime
                const uint64_t qj = a.pc[j].q;
                for (size_t n = tid; n < N; n += stride) {
                    const uint64_t raw = (n * elt) & (2 * N - 1), v0 = tb[(size_t)j * N + n];
                    const size_t dst = raw < N ? raw : raw - N;
                    const uint64_t v = raw < N ? v0 : (v0 ? qj - v0 : 0);
                    for (int i = 0; i <= l; ++i) {
                        const PrimeConst Q = a.pc[fix_prime(i, -1, l, K)];
                        a.U[((size_t)i << logn) + dst] = Q.q < qj ? barrett_64(v, Q.q, Q.r1) : v;
                    }
                }
                g.sync();
                fix_ntt_forward(g, a, a.U, l + 1, -1);
                for (size_t x = tid; x < ((size_t)(l + 1) << logn); x += stride) {
                    const int i = (int)(x >> logn);
                    const int kidx = fix_prime(i, -1, l, K);
                    const size_t n = x & (N - 1);
                    const PrimeConst Q = a.pc[kidx];
                    const uint64_t u = a.U[x];
#pragma unroll
                    for (int k = 0; k < 2; ++k) {
                        const uint64_t kv = key[((((size_t)j * 2 + k) * K + kidx) << logn) + n];
                        uint64_t &acc = a.P[(((size_t)k * (l + 1) + i) << logn) + n];
                        acc = csub(acc + mul_mod(u, kv, Q.q, Q.r0, Q.r1), Q.q);
                    }
                }
                g.sync();
            }
            const uint32_t *tab = a.tab[r];
            uint64_t *out = a.out[r] + (size_t)b * 2 * l * N;
            for (int k = 0; k < 2; ++k) {
                const uint64_t *Pk = a.P + (((size_t)k * (l + 1)) << logn);
                for (size_t n = tid; n < N; n += stride) a.V[n] = Pk[((size_t)l << logn) + n];
                g.sync();
                fix_ntt_inverse(g, a, a.V, 1, K - 1);
                // rounding: ((x + p/2) mod p) mod q_i - (p/2 mod q_i)
                const uint64_t h = Psp.q >> 1;
                for (size_t x = tid; x < ((size_t)l << logn); x += stride) {
                    const PrimeConst Q = a.pc[(int)(x >> logn)];
                    const uint64_t u = csub(a.V[x & (N - 1)] + h, Psp.q);
                    const uint64_t ui = Q.q < Psp.q ? barrett_64(u, Q.q, Q.r1) : u;
                    const uint64_t hi = Q.q < Psp.q ? barrett_64(h, Q.q, Q.r1) : h;
                    a.U[x] = csub(ui + Q.q - hi, Q.q);
                }
                g.sync();
                fix_ntt_forward(g, a, a.U, l, -1);
                for (size_t x = tid; x < ((size_t)l << logn); x += stride) {
                    const int i = (int)(x >> logn);
                    const size_t n = x & (N - 1);
                    const uint64_t q = a.pc[i].q;
                    const ulonglong2 w = a.inv_p[i];
                    uint64_t v = mul_shoup(Pk[((size_t)i << logn) + n] + q - a.U[x], w.x, w.y, q);
                    if (k == 0) v = csub(v + c0[((size_t)i << logn) + tab[n]], q);
                    out[((size_t)k * l << logn) + x] = v;
                }
                g.sync();
            }
        }
    }
}

}  // namespace

void hoist_fix(Context &c, const uint64_t *t, const uint64_t *ct, size_t ct_pitch, const int *d_flags, int B, int l,
               const std::vector<HoistRotation> &rots, cudaStream_t s)
{
    const size_t N = c.n;
    if (ct_pitch == 0) ct_pitch = 2 * (size_t)l * N;
    // co-resident CTAs per SM (a cooperative launch must not exceed them)
    static const int blocks_per_sm = [] {
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_hoist_fix, kBlock, 0) != cudaSuccess || nb < 1)
            throw std::runtime_error("hoist_fix: occupancy query failed");
        return nb;
    }();
    // scratch U | P | V; hoist_rotate's arena (B*N*(4l+4) words) already holds it
    uint64_t *U = c.get_scratch(N * (3 * (size_t)(l + 1) + 1));
    HoistFixArgs a{};
    a.t = t;
    a.ct = ct;
    a.pitch = ct_pitch;
    a.flags = d_flags;
    a.pc = c.d_pc;
    a.tw_fwd = c.d_tw_fwd;
    a.tw_inv = c.d_tw_inv;
    a.inv_p = c.d_inv_q + (size_t)(c.k - 1) * c.k;
    a.U = U;
    a.P = U + (size_t)(l + 1) * N;
    a.V = a.P + 2 * (size_t)(l + 1) * N;
    a.B = B;
    a.l = l;
    a.K = c.k;
    a.logn = c.logn;
    const unsigned grid = (unsigned)(blocks_per_sm * c.sm_count);
    for (size_t first = 0; first < rots.size(); first += kFixMaxRot) {
        a.R = (int)std::min(rots.size() - first, (size_t)kFixMaxRot);
        for (int r = 0; r < a.R; ++r) {
            const HoistRotation &h = rots[first + r];
            a.elt[r] = h.elt;
            a.key[r] = h.key;
            a.tab[r] = c.galois_table(h.elt);
            a.out[r] = h.out;
        }
        void *args[] = {&a};
        if (cudaLaunchCooperativeKernel((const void *)k_hoist_fix, dim3(grid), dim3(kBlock), args, 0, s) !=
            cudaSuccess)
            throw std::runtime_error("hoist_fix: cooperative launch failed");
        NEXUS_LAUNCHED();
    }
}

}  // namespace nexus

// ---------------------------------------------------------------------------
// Key switching that allocates nothing.
//
// nexus_switch_key takes its temporaries from the context's scratch arena,
// which is allocated (and regrown) with cudaMalloc/cudaFree on first use.
// Some callers cannot allow that: a host program whose device memory is
// entirely owned by another runtime's pool, or a serving loop in which the
// implicit device-wide synchronisation of cudaMalloc/cudaFree would stall
// other streams.  nexus_switch_key_noalloc gives them the same operation with
// its temporaries in a fixed device array that is part of the library image:
// every GPU that loads the library reserves kNoAllocWords * 8 bytes (16 MiB)
// for it until the process exits.  The caller still passes the ciphertext,
// the target and the key.  The array holds N * (l^2 + 6l + 4) words for
// ring degree N and l data limbs; larger requests are rejected.
using namespace nexus;

namespace {

constexpr size_t kNoAllocWords = size_t(1) << 21;
static __device__ __align__(256) uint64_t g_noalloc_scratch[kNoAllocWords];

// Device address of g_noalloc_scratch in the current context.  It is looked
// up on every call (a host-side query, no allocation): an address cached once
// per device would go stale if the module were reloaded, for instance after
// cudaDeviceReset.
uint64_t *noalloc_scratch_on_current_device()
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) throw std::runtime_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    return static_cast<uint64_t *>(p);
}

}  // namespace

extern "C" int nexus_switch_key_noalloc(nexus_context *ctx, uint64_t *ct, int l, const uint64_t *target,
                                        const uint64_t *key, void *stream)
{
    static const char *fn = "nexus_switch_key_noalloc";
    if (!ctx || !ct || !target || !key) {
        set_error(std::string(fn) + ": null argument");
        return -1;
    }
    Context &c = ctx->c;
    if (l < 1 || l > c.k - 1) {
        set_error(std::string(fn) + ": limbs must be in [1, n_moduli-1]");
        return -1;
    }
    const size_t N = c.n;
    const size_t words = N * ((size_t)l * l + 6 * (size_t)l + 4);
    if (words > kNoAllocWords) {
        set_error(std::string(fn) + ": needs " + std::to_string(words) + " scratch words (N*(l^2+6l+4)), the fixed " +
                  "device buffer holds " + std::to_string(kNoAllocWords));
        return -1;
    }
    if (reinterpret_cast<uintptr_t>(key) & 15) {
        set_error(std::string(fn) + ": the key must be 16-byte aligned");
        return -1;
    }
    try {
        int dev = -1;
        if (cudaGetDevice(&dev) != cudaSuccess || dev != c.device)
            throw std::runtime_error("the context's device must be current");
        uint64_t *t = noalloc_scratch_on_current_device();
        // the fused sequence of switch_key_batch for one ciphertext, with its
        // scratch t[l] | D[l][l+1] | P[2][l+1] | T[2][l] | last[2] in the
        // fixed array instead of the context's arena
        cudaStream_t s = (cudaStream_t)stream;
        const int sp = c.k - 1;
        uint64_t *D = t + (size_t)l * N;
        uint64_t *P = D + (size_t)l * (l + 1) * N;
        uint64_t *T = P + 2 * (size_t)(l + 1) * N;
        uint64_t *last = T + 2 * (size_t)l * N;
        cudaMemcpyAsync(t, target, sizeof(uint64_t) * l * N, cudaMemcpyDeviceToDevice, s);
        ks_modup_inner(c, t, 1, l, key, D, P, s);
        ks_moddown_terms(c, P, 1, l, T, last, s);
        const size_t tot = (size_t)2 * l * N;
        k_moddown_finish<<<grid_for(tot), kBlock, 0, s>>>(ct, P, T, c.d_pc, c.d_inv_q + (size_t)sp * c.k, l, c.logn,
                                                           tot); NEXUS_LAUNCHED();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
    } catch (const std::exception &e) {
        set_error(std::string(fn) + ": " + e.what());
        return -1;
    }
    return 0;
}
