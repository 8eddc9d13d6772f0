// Batched negacyclic RNS NTT / INTT over [poly][limb][N] uint64 residues.
//
// The transform is the one SEAL computes in ntt_negacyclic_harvey /
// inverse_ntt_negacyclic_harvey (util/ntt.cpp:394-470, util/dwthandler.h:94-290
// in SEAL-4.1-bs): input in natural order, output in bit-reversed order, with
// psi the minimal primitive 2N-th root.  Because the transform is a linear map
// over Z_q and both sides reduce to [0, q), any exact evaluation of it gives
// SEAL's words; this file evaluates it as two passes over an n1 x n2 view of
// each limb (row index r = i / n2, column c = i % n2):
//
//   pass 1 (columns): the first log2(n1) Cooley-Tukey stages only pair rows of
//     one column, and the stage with m blocks uses twiddle W[m + block];
//   pass 2 (rows): the remaining log2(n2) stages stay inside one contiguous
//     row r, and the local stage with m blocks uses W[(n1 + r) * m + block].
//
// Each thread holds 16 residues in registers; 4 butterfly stages run in
// registers, the thread group exchanges through shared memory, and the next
// log2(T) stages run in registers again.  Butterflies are Harvey's lazy
// Shoup butterflies (values in [0,4q) forward, [0,2q) inverse).
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>
#include <cooperative_groups.h>

#include "context.h"
#include "ntt.h"

namespace nexus {

namespace {

constexpr int kE = 16;          // residues per thread
constexpr int kThreads = 256;   // threads per CTA

// Every CTA of either pass covers kThreads * kE residues (32 KB): 256 lines of
// 128 bytes.  Before its own work each CTA asks L2 for the tile of the CTA one
// residency wave ahead (the CTA that will take its slot), one line per thread,
// so that CTA's loads find their data in L2 instead of waiting on HBM.  A
// prefetch is only a hint: nothing waits for it.
__device__ __forceinline__ void prefetch_l2(const void *p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__device__ __forceinline__ unsigned sm_count()
{
    unsigned n;
    asm("mov.u32 %0, %%nsmid;" : "=r"(n));
    return n;
}

// the tile of CTA fb in a columns pass: S rows of C residues, row stride n2
template <int S, int C>
__device__ __forceinline__ void prefetch_cols_tile(const uint64_t *data, unsigned fb, int logn, int n2, int tiles,
                                                   const LimbMap &lm)
{
    const uint32_t pl = fb / (uint32_t)tiles;
    const int col0 = (int)(fb - pl * (uint32_t)tiles) * C;
    size_t lrow;
    int prime;
    lm.locate(pl, lrow, prime);
    constexpr int kLinesPerRow = C / 16;
    const int row = threadIdx.x / kLinesPerRow, sub = threadIdx.x % kLinesPerRow;
    prefetch_l2(data + (lrow << logn) + col0 + (size_t)row * n2 + sub * 16);
}

// the tile of CTA fb in a rows pass: R contiguous rows of S residues
template <int S, int R>
__device__ __forceinline__ void prefetch_rows_tile(const uint64_t *data, unsigned fb, int logn, int log_n1,
                                                   const LimbMap &lm)
{
    const size_t grow = (size_t)fb * R;
    const uint32_t pl = (uint32_t)(grow >> log_n1);
    const uint64_t r = grow & ((1u << log_n1) - 1);
    size_t lrow;
    int prime;
    lm.locate(pl, lrow, prime);
    prefetch_l2(data + (lrow << logn) + r * S + (size_t)threadIdx.x * 16);
}

__device__ __forceinline__ void ct_bfly(uint64_t &x, uint64_t &y, ulonglong2 w, uint64_t q, uint64_t q2)
{
    uint64_t u = csub(x, q2);
    uint64_t v = mul_shoup_lazy(y, w.x, w.y, q);
    x = u + v;
    y = u + q2 - v;
}

// Lazy product for primes below 2^52: the Shoup quotient estimate
// floor(y * wq / 2^64) from the high halves of the three upper 32-bit partial
// products of y * wq.  Each dropped low half (and the dropped low x low
// product) is below one unit of the estimate, so it is at most two below the
// exact Shoup quotient, which is itself at most one below floor(y*w/q): the
// result is congruent to y*w and lies in [0, 4q).
__device__ __forceinline__ uint64_t mul_shoup_lazy4(uint64_t y, uint64_t w, uint64_t wq, uint64_t q)
{
    const uint32_t y0 = (uint32_t)y, y1 = (uint32_t)(y >> 32), b0 = (uint32_t)wq, b1 = (uint32_t)(wq >> 32);
    const uint64_t hi = (uint64_t)y1 * b1 + __umulhi(y1, b0) + __umulhi(y0, b1);
    return y * w - hi * q;
}

// Cooley-Tukey butterfly without reductions for primes below 2^52: each stage
// adds less than 4q to the largest value, so 16 stages from below 2^53 stay
// below 2^53 + 64q < 2^59.
__device__ __forceinline__ void ct_bfly_small(uint64_t &x, uint64_t &y, ulonglong2 w, uint64_t q, uint64_t q4)
{
    const uint64_t v = mul_shoup_lazy4(y, w.x, w.y, q);
    const uint64_t u = x;
    x = u + v;
    y = u + q4 - v;
}

template <bool SMALL>
__device__ __forceinline__ void fwd_bfly(uint64_t &x, uint64_t &y, ulonglong2 w, uint64_t q, uint64_t q2)
{
    if (SMALL)
        ct_bfly_small(x, y, w, q, q2 << 1);
    else
        ct_bfly(x, y, w, q, q2);
}

__device__ __forceinline__ void gs_bfly(uint64_t &x, uint64_t &y, ulonglong2 w, uint64_t q, uint64_t q2)
{
    uint64_t u = x, v = y;
    x = csub(u + v, q2);
    y = mul_shoup_lazy(u + q2 - v, w.x, w.y, q);
}

// Forward stages whose pairs are (k, k+h) inside the thread, residues at
// sub-transform positions s = t + T*k.  Stage with pair distance h has
// m = E/(2h) blocks and block index k/(2h).
template <bool SMALL>
__device__ __forceinline__ void fwd_regs_strided(uint64_t (&x)[kE], const ulonglong2 *__restrict__ W, uint64_t B,
                                                 uint64_t q, uint64_t q2)
{
#pragma unroll
    for (int h = kE / 2; h >= 1; h >>= 1) {
        const int m = kE / (2 * h);
#pragma unroll
        for (int k = 0; k < kE; ++k) {
            if (k & h) continue;
            ulonglong2 w = __ldg(&W[B * m + k / (2 * h)]);
            fwd_bfly<SMALL>(x[k], x[k + h], w, q, q2);
        }
    }
}

// Forward stages with gaps T/2 .. 1 on residues at s = E*t + k.
template <int T, bool SMALL>
__device__ __forceinline__ void fwd_regs_blocked(uint64_t (&x)[kE], const ulonglong2 *__restrict__ W, uint64_t B,
                                                 int t, uint64_t q, uint64_t q2)
{
    static_assert(T <= kE, "the blocked stages pair residues inside one thread: at most kE * kE points per pass");
    constexpr int S = kE * T;
#pragma unroll
    for (int g = T / 2; g >= 1; g >>= 1) {
        const int m = S / (2 * g);
        const uint64_t base = B * m + (uint64_t)(kE * t) / (2 * g);
#pragma unroll
        for (int k = 0; k < kE; ++k) {
            if (k & g) continue;
            ulonglong2 w = __ldg(&W[base + k / (2 * g)]);
            fwd_bfly<SMALL>(x[k], x[k + g], w, q, q2);
        }
    }
}

// Inverse of fwd_regs_blocked: gaps 1 .. T/2, Gentleman-Sande butterflies.
template <int T>
__device__ __forceinline__ void inv_regs_blocked(uint64_t (&x)[kE], const ulonglong2 *__restrict__ W, uint64_t B,
                                                 int t, uint64_t q, uint64_t q2)
{
    static_assert(T <= kE, "the blocked stages pair residues inside one thread: at most kE * kE points per pass");
    constexpr int S = kE * T;
#pragma unroll
    for (int g = 1; g <= T / 2; g <<= 1) {
        const int m = S / (2 * g);
        const uint64_t base = B * m + (uint64_t)(kE * t) / (2 * g);
#pragma unroll
        for (int k = 0; k < kE; ++k) {
            if (k & g) continue;
            ulonglong2 w = __ldg(&W[base + k / (2 * g)]);
            gs_bfly(x[k], x[k + g], w, q, q2);
        }
    }
}

// Inverse of fwd_regs_strided: pair distances 1 .. E/2.
__device__ __forceinline__ void inv_regs_strided(uint64_t (&x)[kE], const ulonglong2 *__restrict__ W, uint64_t B,
                                                 uint64_t q, uint64_t q2)
{
#pragma unroll
    for (int h = 1; h <= kE / 2; h <<= 1) {
        const int m = kE / (2 * h);
#pragma unroll
        for (int k = 0; k < kE; ++k) {
            if (k & h) continue;
            ulonglong2 w = __ldg(&W[B * m + k / (2 * h)]);
            gs_bfly(x[k], x[k + h], w, q, q2);
        }
    }
}

__device__ __forceinline__ int swz(int s) { return s + (s >> 4); }

// ---------------------------------------------------------------- forward

// Pass 1: size-2^LOGS transforms down the columns.  Output stays in [0,4q).
// KIND selects the input (NttLoader): 0 the data itself, 1 the ModUp spread,
// 2 the ModDown rounding spread of a key switch.
template <int LOGS, int KIND, bool SMALL>
__global__ void __launch_bounds__(kThreads, 3) k_fwd_cols(uint64_t *__restrict__ data, const ulonglong2 *__restrict__ tw,
                                                       const PrimeConst *__restrict__ pc, int logn, LimbMap lm,
                                                       NttLoader ld)
{
    constexpr int S = 1 << LOGS, T = S / kE, C = kThreads / T;
    __shared__ uint64_t sm[S * C];
    const int n2 = 1 << (logn - LOGS);
    const int tiles = n2 / C;
    const uint32_t pl = blockIdx.x / (uint32_t)tiles;
    const int col0 = (int)(blockIdx.x - pl * (uint32_t)tiles) * C;
    size_t lrow;
    int prime;
    lm.locate(pl, lrow, prime);
    const uint64_t q = pc[prime].q, q2 = q << 1;
    const ulonglong2 *W = tw + ((size_t)prime << logn);
    uint64_t *p = data + (lrow << logn) + col0;
    const int c = threadIdx.x % C, t = threadIdx.x / C;

    uint64_t x[kE];
    if (KIND == 0) {
#pragma unroll
        for (int k = 0; k < kE; ++k) x[k] = p[(size_t)(t + T * k) * n2 + c];
    } else {
        const uint32_t srow = pl / (uint32_t)ld.group;
        const uint64_t *sp = ld.src + ((size_t)srow << logn) + col0;
        const uint64_t r1 = pc[prime].r1;
        // On the small-prime path the spread values enter unreduced: they are
        // below 2^53, the reduction-free stages add less than 4q each (below
        // 2^59 after all 16) and the final Barrett step of the rows pass
        // returns the canonical residue, so the output words are the same.
        if (KIND == 1) {
            const uint64_t qj = pc[(int)(srow % (uint32_t)ld.src_limbs)].q;
#pragma unroll
            for (int k = 0; k < kE; ++k) {
                const uint64_t v = sp[(size_t)(t + T * k) * n2 + c];
                x[k] = (!SMALL && q < qj) ? barrett_64(v, q, r1) : v;
            }
        } else {
            const uint64_t P = pc[ld.special].q, h = P >> 1;
            const uint64_t hr = (q < P) ? barrett_64(h, q, r1) : h;
#pragma unroll
            for (int k = 0; k < kE; ++k) {
                const uint64_t v = csub(sp[(size_t)(t + T * k) * n2 + c] + h, P);
                x[k] = ((!SMALL && q < P) ? barrett_64(v, q, r1) : v) + (q - hr);
            }
        }
    }
    fwd_regs_strided<SMALL>(x, W, 1, q, q2);
#pragma unroll
    for (int k = 0; k < kE; ++k) sm[(t + T * k) * C + c] = x[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kE; ++k) x[k] = sm[(kE * t + k) * C + c];
    fwd_regs_blocked<T, SMALL>(x, W, 1, t, q, q2);
#pragma unroll
    for (int k = 0; k < kE; ++k) p[(size_t)(kE * t + k) * n2 + c] = x[k];
}

// The rows-pass CTA of a limb-grouped launch: row r of the R launch limbs
// (chunk*R + rr) * count + m, rr < R -- the same position m in R consecutive
// polynomials, which use one prime (with skip_diag all but the digit whose
// diagonal is left out), so the CTA's R row groups read the same twiddles.
// A row group past the last polynomial repeats the chunk's first limb and
// stores nothing.
struct GroupedRow {
    uint32_t pl;
    uint64_t r;
    bool active;
};

template <int R>
__device__ __forceinline__ GroupedRow grouped_row(unsigned blk, int rr, int log_n1, const LimbMap &lm,
                                                  uint32_t n_polys)
{
    const uint32_t chunks = (n_polys + R - 1) / R;
    GroupedRow g;
    g.r = blk & ((1u << log_n1) - 1);
    const uint32_t mc = blk >> log_n1;            // m * chunks + chunk
    const uint32_t m = mc / chunks, chunk = mc - m * chunks;
    uint32_t poly = chunk * R + (uint32_t)rr;
    g.active = poly < n_polys;
    if (!g.active) poly = chunk * R;
    g.pl = poly * (uint32_t)lm.count + m;
    return g;
}

// Pass 2: size-2^LOGS transforms along contiguous rows, then the final
// reduction to [0,q) (from [0,4q), or from below 2^59 on the small-prime path).
// GROUPED: the CTA takes one row of R limbs of one prime (grouped_row)
// instead of R rows of one limb.
template <int LOGS, bool SMALL, bool GROUPED>
__global__ void __launch_bounds__(kThreads, 3) k_fwd_rows(uint64_t *__restrict__ data, const ulonglong2 *__restrict__ tw,
                                                       const PrimeConst *__restrict__ pc, int logn, LimbMap lm, int pf,
                                                       uint32_t n_polys)
{
    constexpr int S = 1 << LOGS, T = S / kE, R = kThreads / T, SP = S + S / 16;
    // the T threads of a row sit in one warp and share only their row's
    // slice of shared memory, so warp barriers order the exchanges
    static_assert(32 % T == 0, "a row's threads must lie inside one warp");
    __shared__ uint64_t sm[R * SP];
    const int log_n1 = logn - LOGS;
    const int rr = threadIdx.x / T, t = threadIdx.x % T;
    uint32_t pl;
    uint64_t r;
    bool active = true;
    if (GROUPED) {
        const GroupedRow g = grouped_row<R>(blockIdx.x, rr, log_n1, lm, n_polys);
        pl = g.pl;
        r = g.r;
        active = g.active;
    } else {
        const size_t grow = (size_t)blockIdx.x * R + rr;
        pl = (uint32_t)(grow >> log_n1);
        r = grow & ((1u << log_n1) - 1);
    }
    size_t lrow;
    int prime;
    lm.locate(pl, lrow, prime);
    const uint64_t q = pc[prime].q, q2 = q << 1;
    const ulonglong2 *W = tw + ((size_t)prime << logn);
    uint64_t *p = data + (lrow << logn) + r * S;
    uint64_t *srow = sm + rr * SP;
    const uint64_t B = (1ull << log_n1) + r;
    if (pf) {
        const unsigned fb = blockIdx.x + (unsigned)pf * 3 * sm_count();
        if (fb < gridDim.x) {
            if (GROUPED) {
                const GroupedRow g = grouped_row<R>(fb, rr, log_n1, lm, n_polys);
                size_t frow;
                int fprime;
                lm.locate(g.pl, frow, fprime);
                prefetch_l2(data + (frow << logn) + g.r * S + (size_t)t * 16);
            } else {
                prefetch_rows_tile<S, R>(data, fb, logn, log_n1, lm);
            }
        }
    }

    uint64_t x[kE];
#pragma unroll
    for (int k = 0; k < kE; ++k) x[k] = p[t + T * k];
    fwd_regs_strided<SMALL>(x, W, B, q, q2);
#pragma unroll
    for (int k = 0; k < kE; ++k) srow[swz(t + T * k)] = x[k];
    __syncwarp();
#pragma unroll
    for (int k = 0; k < kE; ++k) x[k] = srow[swz(kE * t + k)];
    fwd_regs_blocked<T, SMALL>(x, W, B, t, q, q2);
    if (SMALL) {
        const uint64_t r1 = pc[prime].r1;
        if (r1 >> 32) {
#pragma unroll
            for (int k = 0; k < kE; ++k) srow[swz(kE * t + k)] = barrett_64(x[k], q, r1);
        } else {
#pragma unroll
            for (int k = 0; k < kE; ++k) srow[swz(kE * t + k)] = barrett_64_r32(x[k], q, (uint32_t)r1);
        }
    } else {
#pragma unroll
        for (int k = 0; k < kE; ++k) srow[swz(kE * t + k)] = csub(csub(x[k], q2), q);
    }
    __syncwarp();
    if (active) {
#pragma unroll
        for (int k = 0; k < kE; ++k) p[t + T * k] = srow[swz(t + T * k)];
    }
}

// ------------------------------------------------- forward, one pass per cluster
//
// The same two passes in one launch: a cluster of CS = N / 4096 CTAs holds
// one limb in its shared memory.  CTA rank cr first runs the columns pass on
// column tile cr (the tile of k_fwd_cols, loaders included) and keeps the
// result in its own shared memory; after a cluster barrier it reads its R
// rows from the CS tiles through distributed shared memory (the row's
// column col lives in CTA col / C at column col % C) into registers, runs
// the rows pass's first stages there, waits until every peer has read its
// own tile, reuses that tile for the rows pass's exchange and writes the
// rows to global memory.  A limb crosses HBM
// once each way instead of twice.  Each CTA needs only its 32 KB tile, so
// the cluster scheduler is limited by registers (3 CTAs per SM), not by
// shared memory.
template <int L1, int L2>
struct ClusterShape {
    static constexpr int T1 = (1 << L1) / kE, C = kThreads / T1;          // columns pass
    static constexpr int S2 = 1 << L2, T2 = S2 / kE, R = kThreads / T2;   // rows pass
    static constexpr int CS = (1 << (L1 + L2)) / (kThreads * kE);        // CTAs per limb
    static constexpr size_t smem_words = (size_t)kThreads * kE;          // one tile
    static_assert((1 << L2) / C == CS && (1 << L1) / R == CS, "tiles must cover the limb once");
    static_assert((size_t)R * S2 == smem_words && (size_t)(1 << L1) * C == smem_words, "the exchanges share one tile");
};

// a cluster-wide barrier with release/acquire ordering of shared memory
__device__ __forceinline__ void cluster_barrier()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// the 64-bit word at shared-memory offset `addr` of CTA `rank` of this cluster
__device__ __forceinline__ uint64_t ld_cluster(uint32_t addr, uint32_t rank)
{
    uint32_t remote;
    uint64_t v;
    asm("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(addr), "r"(rank));
    asm volatile("ld.shared::cluster.u64 %0, [%1];" : "=l"(v) : "r"(remote));
    return v;
}

// The rows exchange without padding: word s of a row sits at
// s ^ ((s >> 4) & 15), which keeps both access patterns free of bank
// conflicts.  For s = t + T*k (t < T <= 16) that is s ^ ((T*k) >> 4), a
// constant per register k; for s = kE*t + k it is kE*t + (k ^ t).
template <int T>
__device__ __forceinline__ int swx_strided(int t, int k) { return (t + T * k) ^ ((T * k) >> 4); }
__device__ __forceinline__ int swx_blocked(int t, int k) { return kE * t + (k ^ t); }

template <int L1, int L2, int KIND, bool SMALL>
__global__ void __launch_bounds__(kThreads, 3)
    k_fwd_cluster(uint64_t *__restrict__ data, const ulonglong2 *__restrict__ tw, const PrimeConst *__restrict__ pc,
                  int logn, LimbMap lm, NttLoader ld)
{
    using Sh = ClusterShape<L1, L2>;
    constexpr int T1 = Sh::T1, C = Sh::C, S2 = Sh::S2, T2 = Sh::T2;
    // the T2 threads of a row sit in one warp (warp barriers order the row exchange)
    static_assert(32 % T2 == 0, "a row's threads must lie inside one warp");
    extern __shared__ uint64_t tile[];   // [2^L1][C] after pass 1, then [R][S2] for the rows exchange
    const unsigned cr = blockIdx.x % (unsigned)Sh::CS;   // rank in the cluster (clusters run along x)
    const uint32_t pl = blockIdx.x / (unsigned)Sh::CS;
    size_t lrow;
    int prime;
    lm.locate(pl, lrow, prime);
    const uint64_t q = pc[prime].q, q2 = q << 1;
    const ulonglong2 *W = tw + ((size_t)prime << logn);
    const int n2 = S2;

    // pass 1: columns cr * C .. cr * C + C - 1
    {
        const int col0 = (int)cr * C;
        const uint64_t *p = data + (lrow << logn) + col0;
        const int c = threadIdx.x % C, t = threadIdx.x / C;
        uint64_t x[kE];
        if (KIND == 0) {
#pragma unroll
            for (int k = 0; k < kE; ++k) x[k] = p[(size_t)(t + T1 * k) * n2 + c];
        } else {
            const uint32_t srow = pl / (uint32_t)ld.group;
            const uint64_t *sp = ld.src + ((size_t)srow << logn) + col0;
            const uint64_t r1 = pc[prime].r1;
            if (KIND == 1) {
                const uint64_t qj = pc[(int)(srow % (uint32_t)ld.src_limbs)].q;
#pragma unroll
                for (int k = 0; k < kE; ++k) {
                    const uint64_t v = sp[(size_t)(t + T1 * k) * n2 + c];
                    x[k] = (!SMALL && q < qj) ? barrett_64(v, q, r1) : v;
                }
            } else {
                const uint64_t P = pc[ld.special].q, h = P >> 1;
                const uint64_t hr = (q < P) ? barrett_64(h, q, r1) : h;
#pragma unroll
                for (int k = 0; k < kE; ++k) {
                    const uint64_t v = csub(sp[(size_t)(t + T1 * k) * n2 + c] + h, P);
                    x[k] = ((!SMALL && q < P) ? barrett_64(v, q, r1) : v) + (q - hr);
                }
            }
        }
        fwd_regs_strided<SMALL>(x, W, 1, q, q2);
#pragma unroll
        for (int k = 0; k < kE; ++k) tile[(t + T1 * k) * C + c] = x[k];
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kE; ++k) x[k] = tile[(kE * t + k) * C + c];
        fwd_regs_blocked<T1, SMALL>(x, W, 1, t, q, q2);
        // each thread writes back the words it alone read
#pragma unroll
        for (int k = 0; k < kE; ++k) tile[(kE * t + k) * C + c] = x[k];
    }
    cluster_barrier();

    // pass 2: rows cr * R .. cr * R + R - 1, gathered from the cluster's tiles
    const int rr = threadIdx.x / T2, t = threadIdx.x % T2;
    const uint64_t r = (uint64_t)cr * Sh::R + rr;
    uint64_t x[kE];
    {
        const uint32_t row_base = (uint32_t)__cvta_generic_to_shared(tile) + (uint32_t)(r * C) * 8u;
#pragma unroll
        for (int k = 0; k < kE; ++k) {
            const int col = t + T2 * k;
            x[k] = ld_cluster(row_base + (uint32_t)(col % C) * 8u, (uint32_t)(col / C));
        }
    }
    const uint64_t B = (1ull << (logn - L2)) + r;
    fwd_regs_strided<SMALL>(x, W, B, q, q2);
    // every peer has read this CTA's tile: it becomes the rows exchange
    cluster_barrier();
    uint64_t *srow = tile + rr * S2;
#pragma unroll
    for (int k = 0; k < kE; ++k) srow[swx_strided<T2>(t, k)] = x[k];
    __syncwarp();
#pragma unroll
    for (int k = 0; k < kE; ++k) x[k] = srow[swx_blocked(t, k)];
    fwd_regs_blocked<T2, SMALL>(x, W, B, t, q, q2);
    if (SMALL) {
        const uint64_t r1 = pc[prime].r1;
        if (r1 >> 32) {
#pragma unroll
            for (int k = 0; k < kE; ++k) srow[swx_blocked(t, k)] = barrett_64(x[k], q, r1);
        } else {
#pragma unroll
            for (int k = 0; k < kE; ++k) srow[swx_blocked(t, k)] = barrett_64_r32(x[k], q, (uint32_t)r1);
        }
    } else {
#pragma unroll
        for (int k = 0; k < kE; ++k) srow[swx_blocked(t, k)] = csub(csub(x[k], q2), q);
    }
    __syncwarp();
    uint64_t *p = data + (lrow << logn) + r * S2;
#pragma unroll
    for (int k = 0; k < kE; ++k) p[t + T2 * k] = srow[swx_strided<T2>(t, k)];
}

// ---------------------------------------------------------------- inverse

// Inverse pass A: rows first (undoing pass 2).  Output in [0,2q).
template <int LOGS>
__global__ void __launch_bounds__(kThreads, 3) k_inv_rows(uint64_t *__restrict__ data, const ulonglong2 *__restrict__ tw,
                                                       const PrimeConst *__restrict__ pc, int logn, LimbMap lm, int pf)
{
    constexpr int S = 1 << LOGS, T = S / kE, R = kThreads / T, SP = S + S / 16;
    // the T threads of a row sit in one warp and share only their row's
    // slice of shared memory, so warp barriers order the exchanges
    static_assert(32 % T == 0, "a row's threads must lie inside one warp");
    __shared__ uint64_t sm[R * SP];
    const int log_n1 = logn - LOGS;
    const int rr = threadIdx.x / T, t = threadIdx.x % T;
    const size_t grow = (size_t)blockIdx.x * R + rr;
    const uint32_t pl = (uint32_t)(grow >> log_n1);
    const uint64_t r = grow & ((1u << log_n1) - 1);
    size_t lrow;
    int prime;
    lm.locate(pl, lrow, prime);
    const uint64_t q = pc[prime].q, q2 = q << 1;
    const ulonglong2 *W = tw + ((size_t)prime << logn);
    uint64_t *p = data + (lrow << logn) + r * S;
    uint64_t *srow = sm + rr * SP;
    const uint64_t B = (1ull << log_n1) + r;
    if (pf) {
        const unsigned fb = blockIdx.x + (unsigned)pf * 3 * sm_count();
        if (fb < gridDim.x) prefetch_rows_tile<S, R>(data, fb, logn, log_n1, lm);
    }

    uint64_t x[kE];
#pragma unroll
    for (int k = 0; k < kE; ++k) srow[swz(t + T * k)] = p[t + T * k];
    __syncwarp();
#pragma unroll
    for (int k = 0; k < kE; ++k) x[k] = srow[swz(kE * t + k)];
    inv_regs_blocked<T>(x, W, B, t, q, q2);
#pragma unroll
    for (int k = 0; k < kE; ++k) srow[swz(kE * t + k)] = x[k];
    __syncwarp();
#pragma unroll
    for (int k = 0; k < kE; ++k) x[k] = srow[swz(t + T * k)];
    inv_regs_strided(x, W, B, q, q2);
#pragma unroll
    for (int k = 0; k < kE; ++k) p[t + T * k] = x[k];
}

// Inverse pass B: columns (undoing pass 1), then n^{-1} and reduction to [0,q).
template <int LOGS>
__global__ void __launch_bounds__(kThreads, 3) k_inv_cols(uint64_t *__restrict__ data, const ulonglong2 *__restrict__ tw,
                                                       const PrimeConst *__restrict__ pc, int logn, LimbMap lm, int pf)
{
    constexpr int S = 1 << LOGS, T = S / kE, C = kThreads / T;
    __shared__ uint64_t sm[S * C];
    const int n2 = 1 << (logn - LOGS);
    const int tiles = n2 / C;
    const uint32_t pl = blockIdx.x / (uint32_t)tiles;
    const int col0 = (int)(blockIdx.x - pl * (uint32_t)tiles) * C;
    size_t lrow;
    int prime;
    lm.locate(pl, lrow, prime);
    const PrimeConst P = pc[prime];
    const uint64_t q = P.q, q2 = q << 1;
    const ulonglong2 *W = tw + ((size_t)prime << logn);
    uint64_t *p = data + (lrow << logn) + col0;
    const int c = threadIdx.x % C, t = threadIdx.x / C;

    if (pf) {
        const unsigned fb = blockIdx.x + (unsigned)pf * 3 * sm_count();
        if (fb < gridDim.x) prefetch_cols_tile<S, C>(data, fb, logn, n2, tiles, lm);
    }

    uint64_t x[kE];
#pragma unroll
    for (int k = 0; k < kE; ++k) x[k] = p[(size_t)(kE * t + k) * n2 + c];
    inv_regs_blocked<T>(x, W, 1, t, q, q2);
#pragma unroll
    for (int k = 0; k < kE; ++k) sm[(kE * t + k) * C + c] = x[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kE; ++k) x[k] = sm[(t + T * k) * C + c];
    inv_regs_strided(x, W, 1, q, q2);
#pragma unroll
    for (int k = 0; k < kE; ++k) p[(size_t)(t + T * k) * n2 + c] = mul_shoup(x[k], P.inv_n, P.inv_n_q, q);
}

// one cluster of ClusterShape::CS CTAs per limb
template <int L1, int L2, int KIND, bool SMALL>
void launch_cluster_k(const Context &c, uint64_t *d, size_t limbs, LimbMap lm, NttLoader ld, cudaStream_t s)
{
    using Sh = ClusterShape<L1, L2>;
    auto kern = k_fwd_cluster<L1, L2, KIND, SMALL>;
    const size_t smem = Sh::smem_words * sizeof(uint64_t);
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        (Sh::CS > 8 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess))
        throw std::runtime_error("NTT cluster form: kernel attributes refused");
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(limbs * Sh::CS));
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = Sh::CS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, d, c.d_tw_fwd, c.d_pc, c.logn, lm, ld);
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw std::runtime_error(std::string("NTT cluster form: launch failed: ") + cudaGetErrorString(e));
    }
    NEXUS_LAUNCHED();
}

template <int L1, int L2, bool SMALL>
void launch_fwd_t(const Context &c, uint64_t *d, size_t n_polys, LimbMap lm, cudaStream_t s, NttLoader ld)
{
    const size_t limbs = n_polys * (size_t)lm.count;
    if (c.tune.ntt_cluster) {
        if (ld.kind == 1)
            launch_cluster_k<L1, L2, 1, SMALL>(c, d, limbs, lm, ld, s);
        else if (ld.kind == 2)
            launch_cluster_k<L1, L2, 2, SMALL>(c, d, limbs, lm, ld, s);
        else
            launch_cluster_k<L1, L2, 0, SMALL>(c, d, limbs, lm, ld, s);
        return;
    }
    constexpr int C = kThreads / ((1 << L1) / kE);
    constexpr int R = kThreads / ((1 << L2) / kE);
    const unsigned g1 = (unsigned)(limbs * ((1u << L2) / C));
    const unsigned g2 = (unsigned)(limbs * ((1u << L1) / R));
    if (ld.kind == 1)
        k_fwd_cols<L1, 1, SMALL><<<g1, kThreads, 0, s>>>(d, c.d_tw_fwd, c.d_pc, c.logn, lm, ld);
    else if (ld.kind == 2)
        k_fwd_cols<L1, 2, SMALL><<<g1, kThreads, 0, s>>>(d, c.d_tw_fwd, c.d_pc, c.logn, lm, ld);
    else
        k_fwd_cols<L1, 0, SMALL><<<g1, kThreads, 0, s>>>(d, c.d_tw_fwd, c.d_pc, c.logn, lm, ld);
    NEXUS_LAUNCHED();
    if (c.tune.ntt_rows_grouped && n_polys >= (size_t)R) {
        // one row of R limbs of one prime per CTA (the CTA reads its
        // twiddles once); idle row groups only past the last polynomial
        const unsigned chunks = (unsigned)((n_polys + R - 1) / R);
        const unsigned gg = (unsigned)lm.count * chunks << (c.logn - L2);
        k_fwd_rows<L2, SMALL, true><<<gg, kThreads, 0, s>>>(d, c.d_tw_fwd, c.d_pc, c.logn, lm,
                                                             c.tune.ntt_prefetch_waves, (uint32_t)n_polys);
    } else {
        k_fwd_rows<L2, SMALL, false><<<g2, kThreads, 0, s>>>(d, c.d_tw_fwd, c.d_pc, c.logn, lm,
                                                              c.tune.ntt_prefetch_waves, (uint32_t)n_polys);
    }
    NEXUS_LAUNCHED();
}

template <int L1, int L2>
void launch_fwd(const Context &c, uint64_t *d, size_t n_polys, LimbMap lm, cudaStream_t s, NttLoader ld = NttLoader())
{
    if (c.small_primes)
        launch_fwd_t<L1, L2, true>(c, d, n_polys, lm, s, ld);
    else
        launch_fwd_t<L1, L2, false>(c, d, n_polys, lm, s, ld);
}

template <int L1, int L2>
void launch_inv(const Context &c, uint64_t *d, size_t n_polys, LimbMap lm, cudaStream_t s)
{
    const size_t limbs = n_polys * (size_t)lm.count;
    constexpr int C = kThreads / ((1 << L1) / kE);
    constexpr int R = kThreads / ((1 << L2) / kE);
    const unsigned g1 = (unsigned)(limbs * ((1u << L2) / C));
    const unsigned g2 = (unsigned)(limbs * ((1u << L1) / R));
    k_inv_rows<L2><<<g2, kThreads, 0, s>>>(d, c.d_tw_inv, c.d_pc, c.logn, lm, c.tune.ntt_prefetch_waves);
    NEXUS_LAUNCHED();
    k_inv_cols<L1><<<g1, kThreads, 0, s>>>(d, c.d_tw_inv, c.d_pc, c.logn, lm, c.tune.ntt_prefetch_waves);
    NEXUS_LAUNCHED();
}

}  // namespace

static void timing_mark(const Context &c, cudaStream_t s)
{
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, s);
    c.ntt_events.push_back(e);
}

// every launch indexes its limbs and CTAs with 32-bit integers
static void check_launch_size(const Context &c, size_t n_polys, const LimbMap &lm)
{
    const size_t blocks_per_limb = c.n / ((size_t)kThreads * kE);   // CTAs per limb of either pass
    if (n_polys * (size_t)lm.count * (blocks_per_limb ? blocks_per_limb : 1) >= (size_t)1 << 31)
        throw std::invalid_argument("NTT: too many limbs in one call");
}

void ntt_forward_loaded(const Context &c, uint64_t *d, size_t n_polys, LimbMap lm, NttLoader ld, cudaStream_t s)
{
    if (n_polys == 0 || lm.count == 0) return;
    check_launch_size(c, n_polys, lm);
    if (c.ntt_timing) {
        timing_mark(c, s);
        c.ntt_limbs.push_back(n_polys * lm.count);
    }
    switch (c.logn) {
    case 12: launch_fwd<6, 6>(c, d, n_polys, lm, s, ld); break;
    case 13: launch_fwd<6, 7>(c, d, n_polys, lm, s, ld); break;
    case 14: launch_fwd<7, 7>(c, d, n_polys, lm, s, ld); break;
    case 15: launch_fwd<7, 8>(c, d, n_polys, lm, s, ld); break;
    case 16: launch_fwd<8, 8>(c, d, n_polys, lm, s, ld); break;
    default: throw std::invalid_argument("unsupported log_n");
    }
    if (c.ntt_timing) timing_mark(c, s);
}

void ntt_forward(const Context &c, uint64_t *d, size_t n_polys, LimbMap lm, cudaStream_t s)
{
    ntt_forward_loaded(c, d, n_polys, lm, NttLoader(), s);
}

void ntt_inverse(const Context &c, uint64_t *d, size_t n_polys, LimbMap lm, cudaStream_t s)
{
    if (n_polys == 0 || lm.count == 0) return;
    check_launch_size(c, n_polys, lm);
    if (c.ntt_timing) {
        timing_mark(c, s);
        c.ntt_limbs.push_back(n_polys * lm.count);
    }
    switch (c.logn) {
    case 12: launch_inv<6, 6>(c, d, n_polys, lm, s); break;
    case 13: launch_inv<6, 7>(c, d, n_polys, lm, s); break;
    case 14: launch_inv<7, 7>(c, d, n_polys, lm, s); break;
    case 15: launch_inv<7, 8>(c, d, n_polys, lm, s); break;
    case 16: launch_inv<8, 8>(c, d, n_polys, lm, s); break;
    default: throw std::invalid_argument("unsupported log_n");
    }
    if (c.ntt_timing) timing_mark(c, s);
}

void ntt_forward(const Context &c, uint64_t *d, size_t n_polys, int limb_begin, int limb_end, cudaStream_t s)
{
    ntt_forward(c, d, n_polys, LimbMap{limb_end - limb_begin, limb_begin, -1}, s);
}

void ntt_inverse(const Context &c, uint64_t *d, size_t n_polys, int limb_begin, int limb_end, cudaStream_t s)
{
    ntt_inverse(c, d, n_polys, LimbMap{limb_end - limb_begin, limb_begin, -1}, s);
}

// ------------------------------------------------------------------ butterfly rate

namespace {

// The compute ceiling of the butterflies above: every thread runs `rounds`
// rounds of the four radix-2 stages over its 16 register residues (32
// butterflies a round) with per-stage twiddles in registers, no memory
// traffic in the loop.  mode 0: ct_bfly, 1: ct_bfly_small, 2: gs_bfly.
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_bfly_rate(const ulonglong2 *__restrict__ W, const uint64_t *__restrict__ in,
                                                        uint64_t *out, uint64_t q, int rounds)
{
    const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
    uint64_t x[kE];
#pragma unroll
    for (int k = 0; k < kE; ++k) x[k] = in[(t * kE + k) & 1023];
    ulonglong2 w[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) w[s] = W[(threadIdx.x + 37 * s) & 255];
    const uint64_t q2 = q << 1;
    for (int r = 0; r < rounds; ++r) {
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const int h = 8 >> s;
#pragma unroll
            for (int k = 0; k < kE; ++k)
                if ((k & h) == 0) {
                    if (MODE == 0) ct_bfly(x[k], x[k + h], w[s], q, q2);
                    else if (MODE == 1) ct_bfly_small(x[k], x[k + h], w[s], q, q2 << 1);
                    else gs_bfly(x[k], x[k + h], w[s], q, q2);
                }
        }
    }
    uint64_t acc = 0;
#pragma unroll
    for (int k = 0; k < kE; ++k) acc ^= x[k];
    out[t] = acc;
}

}  // namespace

double butterfly_rate(int mode, uint64_t q, int rounds, int blocks_per_sm, double *ms_out)
{
    if (mode < 0 || mode > 2) throw std::invalid_argument("mode must be 0, 1 or 2");
    if (q < 3 || q >= (1ull << 61) || rounds < 1 || blocks_per_sm < 1) throw std::invalid_argument("bad arguments");
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        throw std::runtime_error("device query failed");
    const unsigned blocks = (unsigned)(sms * blocks_per_sm);
    std::vector<ulonglong2> hw(256);
    std::vector<uint64_t> hin(1024);
    uint64_t st = 0x9E3779B97F4A7C15ull;
    auto next = [&]() {
        st ^= st << 13;
        st ^= st >> 7;
        st ^= st << 17;
        return st;
    };
    for (auto &w : hw) {
        const uint64_t v = next() % q;
        w.x = v;
        w.y = (uint64_t)(((unsigned __int128)v << 64) / q);
    }
    for (auto &v : hin) v = next() % q;
    ulonglong2 *dW = nullptr;
    uint64_t *din = nullptr, *dout = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto release = [&]() {
        cudaFree(dW);
        cudaFree(din);
        cudaFree(dout);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    if (cudaMalloc(&dW, 256 * sizeof(ulonglong2)) != cudaSuccess || cudaMalloc(&din, 1024 * 8) != cudaSuccess ||
        cudaMalloc(&dout, (size_t)blocks * kThreads * 8) != cudaSuccess) {
        release();
        throw std::runtime_error("allocation failed");
    }
    cudaMemcpy(dW, hw.data(), 256 * sizeof(ulonglong2), cudaMemcpyHostToDevice);
    cudaMemcpy(din, hin.data(), 1024 * 8, cudaMemcpyHostToDevice);
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto launch = [&]() {
        if (mode == 0) k_bfly_rate<0><<<blocks, kThreads>>>(dW, din, dout, q, rounds);
        else if (mode == 1) k_bfly_rate<1><<<blocks, kThreads>>>(dW, din, dout, q, rounds);
        else k_bfly_rate<2><<<blocks, kThreads>>>(dW, din, dout, q, rounds);
        NEXUS_LAUNCHED();
    };
    launch();  // warm-up
    cudaEventRecord(e0);
    const int reps = 5;
    for (int i = 0; i < reps; ++i) launch();
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    release();
    if (err != cudaSuccess) throw std::runtime_error(cudaGetErrorString(err));
    const double per = ms / reps;
    if (ms_out) *ms_out = per;
    return (double)blocks * kThreads * rounds * 32.0 / (per * 1e-3);
}

}  // namespace nexus
