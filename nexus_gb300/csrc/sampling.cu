// Key generation, symmetric encryption and decryption on the GPU.
//
// The structure follows SEAL-4.1-bs: ternary (or sparse ternary, the NEXUS
// fork's secret_key_hamming_weight) secret keys, centered-binomial noise of
// standard deviation 3.2 (util/rlwe.cpp:99-135), and key-switching keys made
// as in KeyGenerator::generate_one_kswitch_key (keygenerator.cpp:303-336): for
// every data prime j, a symmetric encryption of zero at the key level whose
// component 0, limb j, also carries (p mod q_j) * new_key_j.
//
// Randomness comes from a counter-based hash of (seed, stream, index).  It is
// reproducible and statistically sound but NOT a cryptographic generator:
// keys made here are for tests and benchmarks.  Deployed keys are generated
// by the client (SEAL) and imported in SEAL's layout.
#include <algorithm>
#include <random>
#include <stdexcept>
#include <vector>

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

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ uint64_t rnd(uint64_t seed, uint64_t stream, uint64_t idx)
{
    return mix64(mix64(seed ^ mix64(stream)) + idx * 0xD1B54A32D192ED03ull);
}

// uniform residues: out[p][l][n] for primes lm.prime(l); 128 random bits
// reduced mod q (bias below 2^-60)
__global__ void k_uniform(uint64_t *out, const PrimeConst *__restrict__ pc, LimbMap lm, int logn, size_t total,
                          uint64_t seed, uint64_t stream)
{
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const int l = (int)((x >> logn) % (size_t)lm.count);
        const PrimeConst P = pc[lm.prime(l)];
        const uint64_t lo = rnd(seed, stream, 2 * x), hi = rnd(seed, stream, 2 * x + 1);
        out[x] = barrett_128(lo, hi, P.q, P.r0, P.r1);
    }
}

// centered binomial noise (21 + 21 bits, sd 3.2) written into every limb
__global__ void k_cbd(uint64_t *out, const PrimeConst *__restrict__ pc, LimbMap lm, int logn, size_t n_coeffs,
                      uint64_t seed, uint64_t stream)
{
    const size_t N = (size_t)1 << logn;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < n_coeffs; x += (size_t)gridDim.x * blockDim.x) {
        const uint64_t r = rnd(seed, stream, x);
        const int e = __popcll(r & 0x1FFFFFull) - __popcll((r >> 21) & 0x1FFFFFull);
        const size_t p = x / N, n = x % N;
        for (int l = 0; l < lm.count; ++l) {
            const uint64_t q = pc[lm.prime(l)].q;
            out[(p * lm.count + l) * N + n] = e < 0 ? q - (uint64_t)(-e) : (uint64_t)e;
        }
    }
}

// small signed coefficients (host-sampled secret) into residues of every limb
__global__ void k_small_to_rns(const int8_t *__restrict__ v, uint64_t *out, const PrimeConst *__restrict__ pc,
                               int limbs, int logn)
{
    const size_t N = (size_t)1 << logn;
    for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (size_t)gridDim.x * blockDim.x) {
        const int s = v[n];
        for (int l = 0; l < limbs; ++l) {
            const uint64_t q = pc[l].q;
            out[(size_t)l * N + n] = s < 0 ? q - (uint64_t)(-s) : (uint64_t)s;
        }
    }
}

// b = e - a*s (+ factor * nk on limb `digit`), all NTT form over K limbs
__global__ void k_kswitch_row(uint64_t *b, const uint64_t *__restrict__ a, const uint64_t *__restrict__ e,
                              const uint64_t *__restrict__ s, const uint64_t *__restrict__ nk,
                              const PrimeConst *__restrict__ pc, int K, int digit, uint64_t factor, int logn)
{
    const size_t total = (size_t)K << logn;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const int l = (int)(x >> logn);
        const PrimeConst P = pc[l];
        uint64_t v = mul_mod(a[x], s[x], P.q, P.r0, P.r1);
        v = csub(e[x] + P.q - v, P.q);
        if (l == digit && nk) v = csub(v + mul_mod(nk[x], factor, P.q, P.r0, P.r1), P.q);
        b[x] = v;
    }
}

// c0 = e + m - a*s over `limbs` limbs (c1 = a already written)
__global__ void k_encrypt_sym(uint64_t *c0, const uint64_t *__restrict__ a, const uint64_t *__restrict__ e,
                              const uint64_t *__restrict__ m, const uint64_t *__restrict__ s,
                              const PrimeConst *__restrict__ pc, int limbs, int logn)
{
    const size_t total = (size_t)limbs << logn;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const PrimeConst P = pc[x >> logn];
        const uint64_t as = mul_mod(a[x], s[x], P.q, P.r0, P.r1);
        uint64_t v = csub(e[x] + (m ? m[x] : 0), P.q);
        c0[x] = csub(v + P.q - as, P.q);
    }
}

// m = c0 + c1*s (+ c2*s^2) over `limbs` limbs; s given at the key level
__global__ void k_decrypt(uint64_t *m, const uint64_t *__restrict__ ct, int size, const uint64_t *__restrict__ s,
                          const PrimeConst *__restrict__ pc, int limbs, int logn)
{
    const size_t per = (size_t)limbs << logn;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < per; x += (size_t)gridDim.x * blockDim.x) {
        const PrimeConst P = pc[x >> logn];
        const uint64_t sv = s[x];
        uint64_t acc = ct[x], sp = sv;
        for (int c = 1; c < size; ++c) {
            acc = csub(acc + mul_mod(ct[c * per + x], sp, P.q, P.r0, P.r1), P.q);
            sp = mul_mod(sp, sv, P.q, P.r0, P.r1);
        }
        m[x] = acc;
    }
}

__global__ void k_square(uint64_t *out, const uint64_t *__restrict__ in, const PrimeConst *__restrict__ pc, int logn,
                         size_t total)
{
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const PrimeConst P = pc[x >> logn];
        out[x] = mul_mod(in[x], in[x], P.q, P.r0, P.r1);
    }
}

}  // namespace

// Ternary secret (uniform in {-1,0,1}, or exactly `hamming_weight` nonzeros
// of random sign) in NTT form over all K primes.
void keygen_secret(Context &c, uint64_t seed, int hamming_weight, uint64_t *sk, cudaStream_t s)
{
    const size_t N = c.n;
    std::vector<int8_t> v(N, 0);
    std::mt19937_64 g(seed);
    if (hamming_weight > 0) {
        if ((size_t)hamming_weight > N) throw std::invalid_argument("hamming weight exceeds N");
        std::vector<uint32_t> idx(N);
        for (size_t i = 0; i < N; ++i) idx[i] = (uint32_t)i;
        for (int i = 0; i < hamming_weight; ++i) {
            size_t j = i + (size_t)(g() % (N - i));
            std::swap(idx[i], idx[j]);
            v[idx[i]] = (g() & 1) ? 1 : -1;
        }
    } else {
        for (size_t i = 0; i < N; ++i) v[i] = (int8_t)((int)(g() % 3) - 1);
    }
    int8_t *d = nullptr;
    if (cudaMalloc(&d, N) != cudaSuccess) throw std::runtime_error("cudaMalloc");
    cudaMemcpy(d, v.data(), N, cudaMemcpyHostToDevice);
    k_small_to_rns<<<grid_for(N), kBlock, 0, s>>>(d, sk, c.d_pc, c.k, c.logn); NEXUS_LAUNCHED();
    ntt_forward(c, sk, 1, 0, c.k, s);
    cudaStreamSynchronize(s);
    cudaFree(d);
}

// generate_one_kswitch_key for new_key (NTT form, K limbs): key[K-1][2][K][N]
void keygen_kswitch(Context &c, const uint64_t *sk, const uint64_t *new_key, uint64_t seed, uint64_t *key,
                    cudaStream_t s)
{
    const size_t N = c.n;
    const int K = c.k;
    uint64_t *e = c.get_scratch((size_t)K * N);
    const uint64_t p = c.q[K - 1];
    for (int j = 0; j < K - 1; ++j) {
        uint64_t *b = key + (size_t)j * 2 * K * N;
        uint64_t *a = b + (size_t)K * N;
        size_t tot = (size_t)K * N;
        k_uniform<<<grid_for(tot), kBlock, 0, s>>>(a, c.d_pc, LimbMap{K, 0, -1}, c.logn, tot, seed, 2 * j + 1); NEXUS_LAUNCHED();
        k_cbd<<<grid_for(N), kBlock, 0, s>>>(e, c.d_pc, LimbMap{K, 0, -1}, c.logn, N, seed, 2 * j + 2); NEXUS_LAUNCHED();
        ntt_forward(c, e, 1, 0, K, s);
        const uint64_t factor = p % c.q[j];
        k_kswitch_row<<<grid_for(tot), kBlock, 0, s>>>(b, a, e, sk, new_key, c.d_pc, K, j, factor, c.logn); NEXUS_LAUNCHED();
    }
}

void keygen_relin(Context &c, const uint64_t *sk, uint64_t seed, uint64_t *key, cudaStream_t s)
{
    uint64_t *sq = nullptr;
    const size_t words = (size_t)c.k * c.n;
    if (cudaMallocAsync(&sq, words * 8, s) != cudaSuccess) throw std::runtime_error("cudaMallocAsync");
    k_square<<<grid_for(words), kBlock, 0, s>>>(sq, sk, c.d_pc, c.logn, words); NEXUS_LAUNCHED();
    keygen_kswitch(c, sk, sq, seed, key, s);
    cudaFreeAsync(sq, s);
}

void keygen_galois(Context &c, const uint64_t *sk, uint32_t elt, uint64_t seed, uint64_t *key, cudaStream_t s)
{
    uint64_t *rot = nullptr;
    const size_t words = (size_t)c.k * c.n;
    if (cudaMallocAsync(&rot, words * 8, s) != cudaSuccess) throw std::runtime_error("cudaMallocAsync");
    galois_permute(c, sk, 1, c.k, elt, rot, s);
    keygen_kswitch(c, sk, rot, seed ^ ((uint64_t)elt << 32), key, s);
    cudaFreeAsync(rot, s);
}

// symmetric encryption of the NTT-form plaintext m [limbs][N] (m may be null
// for an encryption of zero); ct [2][limbs][N]
void encrypt_symmetric(Context &c, const uint64_t *sk, const uint64_t *m, int limbs, uint64_t seed, uint64_t *ct,
                       cudaStream_t s)
{
    const size_t N = c.n;
    uint64_t *e = c.get_scratch((size_t)limbs * N);
    uint64_t *a = ct + (size_t)limbs * N;
    size_t tot = (size_t)limbs * N;
    k_uniform<<<grid_for(tot), kBlock, 0, s>>>(a, c.d_pc, LimbMap{limbs, 0, -1}, c.logn, tot, seed, 1ull << 40); NEXUS_LAUNCHED();
    k_cbd<<<grid_for(N), kBlock, 0, s>>>(e, c.d_pc, LimbMap{limbs, 0, -1}, c.logn, N, seed, (1ull << 40) + 1); NEXUS_LAUNCHED();
    ntt_forward(c, e, 1, 0, limbs, s);
    k_encrypt_sym<<<grid_for(tot), kBlock, 0, s>>>(ct, a, e, m, sk, c.d_pc, limbs, c.logn); NEXUS_LAUNCHED();
}

void decrypt(Context &c, const uint64_t *sk, const uint64_t *ct, int size, int limbs, uint64_t *m, cudaStream_t s)
{
    size_t tot = (size_t)limbs * c.n;
    k_decrypt<<<grid_for(tot), kBlock, 0, s>>>(m, ct, size, sk, c.d_pc, limbs, c.logn); NEXUS_LAUNCHED();
}

}  // namespace nexus
