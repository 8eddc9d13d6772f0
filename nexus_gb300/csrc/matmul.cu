// NEXUS's ct x pt MatMul (MMEvaluator, src/matrix_mul.cpp) on the GPU.
//
// The encrypted operand arrives coefficient-packed (enc_compress_ciphertext)
// and is expanded by NEXUS's Galois tree (expand_ciphertext): at level i every
// node T becomes T + rot(T) and T*X^(2N-2^i) + rot(T)*X^idx_i, rot being the
// automorphism X -> X^(N/2^i + 1) with its key switch.  Leaf t of the tree
// encrypts N times coefficient t; output row r is sum_k leaf(r*K + k) * P_k.
//
// GPU form, word-for-word equal to the reference:
//  * all nodes of a level share one Galois key, so their key switches run as
//    one batched key switch (the key is read once per level, not per node);
//  * the automorphism's permutation is folded into the gather of the key
//    switch target and into the epilogue, which forms both children at once:
//    the rotated ciphertext is never written;
//  * multiply_power_of_x is a pointwise product with NTT(X^k), whose slot j
//    is psi^(k (2 bitrev(j) + 1)) read from the forward twiddle table (no
//    INTT/shift/NTT round trip and no host copy as in the reference's GPU
//    build);
//  * leaves are never all materialised: the tree is split into 2^d subtrees
//    whose leaves are multiplied by their plaintexts and accumulated into the
//    output rows straight away (modular sums are exact, so the order of the
//    accumulation does not change a word).
#include <stdexcept>
#include <vector>

#include "ckks.h"
#include "nexus_ops.h"
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

// psi_p^(k * (2 bitrev(j) + 1)) as {value, Shoup quotient, negate?}
__device__ __forceinline__ ulonglong2 monomial_slot(const ulonglong2 *__restrict__ W, uint32_t k, uint32_t j, int logn,
                                                    bool &neg)
{
    const uint32_t n = 1u << logn;
    const uint32_t e = 2u * (__brev(j) >> (32 - logn)) + 1u;
    const uint32_t t = (uint32_t)(((uint64_t)k * e) & (2ull * n - 1));
    neg = (t & n) != 0;
    return W[__brev(t & (n - 1)) >> (32 - logn)];
}

// key-switch target of the automorphism: tgt[a][j][i] = nodes[a][1][j][tab[i]]
__global__ void k_galois_c1(const uint64_t *__restrict__ nodes, const uint32_t *__restrict__ tab, uint64_t *tgt,
                            int l, int logn, size_t total)
{
    const size_t N = (size_t)1 << logn, mask = N - 1;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const size_t row = x >> logn;  // a*l + j
        const size_t a = row / (size_t)l, j = row % (size_t)l;
        tgt[x] = nodes[((a * 2 + 1) * l + j) * N + tab[x & mask]];
    }
}

// One expansion level after the key switch's inner products P and ModDown
// terms T: R = apply_galois(T_a) = (perm(c0) | 0) + (P - T) * p^{-1}, then
// left = node + R and right = node * X^k1 + R * X^k2, without writing R.
__global__ void k_expand_fused(const uint64_t *__restrict__ nodes, const uint32_t *__restrict__ tab,
                               const uint64_t *__restrict__ P, const uint64_t *__restrict__ T,
                               const ulonglong2 *__restrict__ inv_p, uint64_t *left, uint64_t *right,
                               const PrimeConst *__restrict__ pc, const ulonglong2 *__restrict__ tw, int l, int logn,
                               uint32_t k1, uint32_t k2, size_t total)
{
    const size_t N = (size_t)1 << logn, mask = N - 1;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const size_t row = x >> logn;          // (a*2 + comp)*l + limb
        const int limb = (int)(row % (size_t)l);
        const size_t ac = row / (size_t)l;     // a*2 + comp
        const int comp = (int)(ac & 1);
        const uint32_t j = (uint32_t)(x & mask);
        const uint64_t q = pc[limb].q;
        const ulonglong2 w = inv_p[limb];
        uint64_t r = mul_shoup(P[(ac * (l + 1) + limb) * N + j] + q - T[x], w.x, w.y, q);
        if (comp == 0) r = csub(r + nodes[((ac * l) + limb) * N + tab[j]], q);
        const uint64_t a = nodes[x];
        left[x] = csub(a + r, q);
        const ulonglong2 *W = tw + ((size_t)limb << logn);
        bool n1, n2;
        const ulonglong2 w1 = monomial_slot(W, k1, j, logn, n1);
        const ulonglong2 w2 = monomial_slot(W, k2, j, logn, n2);
        uint64_t u = mul_shoup(a, w1.x, w1.y, q);
        uint64_t v = mul_shoup(r, w2.x, w2.y, q);
        if (n1 && u) u = q - u;
        if (n2 && v) v = q - v;
        right[x] = csub(u + v, q);
    }
}

// ct[p] *= X^k for polys [polys][l][N] (NTT domain), out may alias in
__global__ void k_mul_monomial(const uint64_t *in, uint64_t *out, const PrimeConst *__restrict__ pc,
                               const ulonglong2 *__restrict__ tw, int l, int logn, uint32_t k, size_t total)
{
    const size_t mask = ((size_t)1 << logn) - 1;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const int limb = (int)((x >> logn) % (size_t)l);
        const uint64_t q = pc[limb].q;
        bool neg;
        const ulonglong2 w = monomial_slot(tw + ((size_t)limb << logn), k, (uint32_t)(x & mask), logn, neg);
        uint64_t v = mul_shoup(in[x], w.x, w.y, q);
        out[x] = (neg && v) ? q - v : v;
    }
}

// out[r] += sum of leaf(u) * pt[k] over the leaves u of one subtree that
// belong to row r.  Leaf u of subtree s is tree leaf t = s + u * 2^d of
// compressed ciphertext c, i.e. element e = c*N + t = r*K + k.
__global__ void k_mm_accumulate(const uint64_t *__restrict__ leaves, const uint64_t *__restrict__ pts,
                                uint64_t *out, const PrimeConst *__restrict__ pc, int l, int logn, int d, int s,
                                int c, int K, int r0, int rows_here, size_t total)
{
    const size_t N = (size_t)1 << logn;
    const size_t mask = N - 1;
    const size_t per_leaf = (size_t)2 * l << logn;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const size_t n = x & mask;
        const size_t rest = x >> logn;                // ((r - r0) * 2 + comp) * l + limb
        const int limb = (int)(rest % (size_t)l);
        const size_t rc = rest / (size_t)l;
        const int comp = (int)(rc & 1);
        const int r = r0 + (int)(rc >> 1);
        const PrimeConst P = pc[limb];
        // tree leaves t of this row inside ciphertext c
        const long long e_lo = (long long)r * K, e_hi = e_lo + K;
        long long t_lo = e_lo - (long long)c * (long long)N, t_hi = e_hi - (long long)c * (long long)N;
        if (t_lo < 0) t_lo = 0;
        if (t_hi > (long long)N) t_hi = (long long)N;
        uint64_t acc = 0;
        if (t_lo < t_hi) {
            // u with s + u*2^d in [t_lo, t_hi)
            const long long step = 1ll << d;
            long long u_lo = (t_lo - s + step - 1) >> d;
            if (u_lo < 0) u_lo = 0;
            const long long u_hi = (t_hi - 1 - s) >= 0 ? ((t_hi - 1 - s) >> d) + 1 : 0;
            for (long long u = u_lo; u < u_hi; ++u) {
                const long long t = s + (u << d);
                const int k = (int)((long long)c * (long long)N + t - e_lo);
                const uint64_t lv = leaves[(size_t)u * per_leaf + (((size_t)comp * l + limb) << logn) + n];
                const uint64_t pv = pts[(((size_t)k * l + limb) << logn) + n];
                acc = csub(acc + mul_mod(lv, pv, P.q, P.r0, P.r1), P.q);
            }
        }
        const size_t oi = ((((size_t)r * 2 + comp) * l + limb) << logn) + n;
        out[oi] = csub(out[oi] + acc, P.q);
    }
}

}  // namespace

// One expansion level for `count` nodes: nodes[count][2][l][N] -> next[2*count][2][l][N]
// (left children first, then right children, the order of expand_ciphertext).
// The automorphism's permutation is folded into the key-switch target gather
// and into the epilogue, which also forms both children.
static void expand_level(Context &c, const uint64_t *nodes, int count, int l, int level, const uint64_t *key,
                         uint64_t *next, cudaStream_t s)
{
    const size_t N = c.n, per = (size_t)2 * l * N, B = (size_t)count;
    const uint32_t n = (uint32_t)N;
    const uint32_t elt = (n + (1u << level)) / (1u << level);
    const uint32_t idx_raw = 2 * n - (1u << level);
    const uint32_t idx = (uint32_t)(((uint64_t)idx_raw * elt) % (2ull * n));
    const uint32_t *tab = c.galois_table(elt);
    // scratch: tgt[B][l] | D[B][l][l+1] | P[B][2][l+1] | T[B][2][l] | last[B][2]
    const size_t words = B * N * ((size_t)l + (size_t)l * (l + 1) + 2 * (size_t)(l + 1) + 2 * (size_t)l + 2);
    uint64_t *tgt = c.get_scratch(words);
    uint64_t *D = tgt + B * l * N;
    uint64_t *P = D + B * l * (l + 1) * N;
    uint64_t *T = P + B * 2 * (l + 1) * N;
    uint64_t *last = T + B * 2 * l * N;
    size_t total = B * l * N;
    k_galois_c1<<<grid_for(total), kBlock, 0, s>>>(nodes, tab, tgt, l, c.logn, total); NEXUS_LAUNCHED();
    ks_modup_inner(c, tgt, count, l, key, D, P, s);
    ks_moddown_terms(c, P, count, l, T, last, s);
    total = B * per;
    k_expand_fused<<<grid_for(total), kBlock, 0, s>>>(nodes, tab, P, T, c.d_inv_q + (size_t)(c.k - 1) * c.k, next,
                                                       next + B * per, c.d_pc, c.d_tw_fwd, l, c.logn, idx_raw, idx,
                                                       total); NEXUS_LAUNCHED();
}

// ---------------------------------------------------------------- MMEvaluator

MMEvaluator::MMEvaluator(CKKSEvaluator &ck) : ckks(&ck)
{
    const size_t n = ck.degree;
    int logn = 0;
    while ((1ull << logn) < n) ++logn;
    for (int i = 0; i < logn; ++i) rots.push_back((uint32_t)((n + (1ull << i)) / (1ull << i)));
}

const uint64_t *MMEvaluator::key_for(uint32_t elt) const
{
    auto &gk = ckks->evaluator->galois_keys;
    auto it = gk.find(elt);
    if (it == gk.end()) throw std::invalid_argument("Galois key not present");
    return it->second;
}

// multiply_power_of_x (src/matrix_mul.cpp:131-172): destination = encrypted * X^index
void MMEvaluator::multiply_power_of_x(Ciphertext &encrypted, Ciphertext &destination, int index)
{
    Evaluator &ev = *ckks->evaluator;
    Context &c = ev.context();
    const uint32_t k = (uint32_t)(((long long)index % (long long)(2 * c.n) + 2 * c.n) % (2 * c.n));
    Ciphertext out;
    out.resize(c, encrypted.size(), encrypted.limbs(), ev.stream());
    out.scale() = encrypted.scale();
    const size_t total = (size_t)encrypted.size() * encrypted.limbs() * c.n;
    k_mul_monomial<<<grid_for(total), kBlock, 0, ev.stream()>>>(encrypted.data(), out.data(), c.d_pc, c.d_tw_fwd,
                                                                 encrypted.limbs(), c.logn, k, total); NEXUS_LAUNCHED();
    destination = std::move(out);
}

// expand_ciphertext (src/matrix_mul.cpp:101-129), all m leaves materialised
std::vector<Ciphertext> MMEvaluator::expand_ciphertext(const Ciphertext &encrypted, uint32_t m)
{
    Evaluator &ev = *ckks->evaluator;
    Context &c = ev.context();
    cudaStream_t s = ev.stream();
    if (encrypted.size() != 2) throw std::invalid_argument("encrypted size must be 2");
    int logm = 0;
    while ((1u << logm) < m) ++logm;
    const int l = encrypted.limbs();
    const size_t per = (size_t)2 * l * c.n;
    DeviceBuffer cur, next;
    cur.reserve(per, s);
    cudaMemcpyAsync(cur.get(), encrypted.data(), per * 8, cudaMemcpyDeviceToDevice, s);
    int count = 1;
    for (int i = 0; i < logm; ++i) {
        next.reserve(per * 2 * count, s);
        expand_level(c, cur.get(), count, l, i, key_for(rots[i]), next.get(), s);
        std::swap(cur, next);
        count *= 2;
    }
    std::vector<Ciphertext> out(count);
    for (int a = 0; a < count; ++a) {
        out[a].resize(c, 2, l, s);
        out[a].scale() = encrypted.scale();
        cudaMemcpyAsync(out[a].data(), cur.get() + (size_t)a * per, per * 8, cudaMemcpyDeviceToDevice, s);
    }
    return out;
}

// matrix_mul after the compression (src/matrix_mul.cpp:174-246, generalised):
// the compressed ciphertexts hold an rows x cols matrix flattened row-major
// (element r*cols + k is coefficient (r*cols + k) mod N of ciphertext
// (r*cols + k) / N); res[r] = sum_k leaf(r*cols + k) * pts[k], its scale
// multiplied by `factor`, then rescaled down to one prime as in the reference.
void MMEvaluator::matrix_mul(const std::vector<Ciphertext> &compressed, const std::vector<Plaintext> &pts, int rows,
                             int cols, double factor, std::vector<Ciphertext> &res, int subtree_depth)
{
    Evaluator &ev = *ckks->evaluator;
    Context &c = ev.context();
    cudaStream_t s = ev.stream();
    if (compressed.empty()) throw std::invalid_argument("no compressed ciphertexts");
    if ((int)pts.size() != cols) throw std::invalid_argument("one plaintext per column is required");
    const int l = compressed[0].limbs();
    DeviceBuffer P;
    P.reserve((size_t)cols * l * c.n, s);
    for (int k = 0; k < cols; ++k) {
        if (pts[k].is_scalar() || pts[k].limbs() != l) throw std::invalid_argument("plaintext level mismatch");
        cudaMemcpyAsync(P.get() + (size_t)k * l * c.n, pts[k].data(), (size_t)l * c.n * 8, cudaMemcpyDeviceToDevice,
                        s);
    }
    std::vector<const Ciphertext *> cp;
    for (auto &ct : compressed) cp.push_back(&ct);
    matrix_mul(cp, P.get(), pts[0].scale(), rows, cols, factor, res, subtree_depth);
}

void MMEvaluator::matrix_mul(const std::vector<const Ciphertext *> &compressed, const uint64_t *d_pts,
                             double pt_scale, int rows, int cols, double factor, std::vector<Ciphertext> &res,
                             int subtree_depth)
{
    Evaluator &ev = *ckks->evaluator;
    Context &c = ev.context();
    cudaStream_t s = ev.stream();
    const size_t N = c.n;
    if (compressed.empty()) throw std::invalid_argument("no compressed ciphertexts");
    if (rows < 1 || cols < 1) throw std::invalid_argument("empty matrix");
    if ((size_t)rows * cols > compressed.size() * N) throw std::invalid_argument("matrix larger than the packing");
    const int l = compressed[0]->limbs();
    for (auto *ct : compressed)
        if (ct->limbs() != l || ct->size() != 2 || ct->scale() != compressed[0]->scale())
            throw std::invalid_argument("compressed ciphertexts differ in level or scale");
    const size_t per = (size_t)2 * l * N;
    DeviceBuffer out;
    out.reserve((size_t)rows * per, s);
    cudaMemsetAsync(out.get(), 0, (size_t)rows * per * 8, s);

    const int logn = c.logn;
    const int d = std::min(subtree_depth, logn);
    DeviceBuffer roots, next, cur;
    for (size_t ci = 0; ci < compressed.size(); ++ci) {
        // rows touched by this ciphertext
        const long long e0 = (long long)ci * N, e1 = e0 + N;
        const int r_first = (int)(e0 / cols);
        int r_last = (int)((e1 - 1) / cols);
        if (r_last >= rows) r_last = rows - 1;
        if (r_first > r_last) continue;
        // levels 0..d-1: 2^d subtree roots
        roots.reserve(per, s);
        cudaMemcpyAsync(roots.get(), compressed[ci]->data(), per * 8, cudaMemcpyDeviceToDevice, s);
        int count = 1;
        for (int i = 0; i < d; ++i) {
            next.reserve(per * 2 * count, s);
            expand_level(c, roots.get(), count, l, i, key_for(rots[i]), next.get(), s);
            std::swap(roots, next);
            count *= 2;
        }
        // each subtree: levels d..logn-1, then accumulate its leaves
        for (int sidx = 0; sidx < (1 << d); ++sidx) {
            cur.reserve(per, s);
            cudaMemcpyAsync(cur.get(), roots.get() + (size_t)sidx * per, per * 8, cudaMemcpyDeviceToDevice, s);
            int cnt = 1;
            for (int i = d; i < logn; ++i) {
                next.reserve(per * 2 * cnt, s);
                expand_level(c, cur.get(), cnt, l, i, key_for(rots[i]), next.get(), s);
                std::swap(cur, next);
                cnt *= 2;
            }
            const int rows_here = r_last - r_first + 1;
            const size_t total = (size_t)rows_here * per;
            k_mm_accumulate<<<grid_for(total), kBlock, 0, s>>>(cur.get(), d_pts, out.get(), c.d_pc, l, logn, d,
                                                                sidx, (int)ci, cols, r_first, rows_here, total); NEXUS_LAUNCHED();
        }
    }
    const double scale = compressed[0]->scale() * pt_scale * factor;
    res.clear();
    res.resize(rows);
    for (int r = 0; r < rows; ++r) {
        res[r].resize(c, 2, l, s);
        cudaMemcpyAsync(res[r].data(), out.get() + (size_t)r * per, per * 8, cudaMemcpyDeviceToDevice, s);
        res[r].scale() = scale;
        while (res[r].limbs() > 1) ev.rescale_to_next_inplace(res[r]);
    }
}

void MMEvaluator::add_bias(std::vector<Ciphertext> &res, const std::vector<double> &bias)
{
    if (res.empty() || bias.empty()) return;
    Evaluator &ev = *ckks->evaluator;
    Plaintext b;
    ev.encode(bias, res[0].limbs(), res[0].scale(), b);
    for (auto &ct : res) ev.add_plain_inplace(ct, b);
}

}  // namespace nexus
