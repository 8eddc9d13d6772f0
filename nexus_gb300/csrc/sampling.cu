// Key generation, symmetric encryption and decryption on the GPU.
//
// The structure follows SEAL-4.1-bs: ternary (or sparse ternary, the NEXUS
// fork's secret_key_hamming_weight) secret keys, centered-binomial noise of
// standard deviation 3.2 (util/rlwe.cpp:99-135), and key-switching keys made
// as in KeyGenerator::generate_one_kswitch_key (keygenerator.cpp:303-336): for
// every data prime j, a symmetric encryption of zero at the key level whose
// component 0, limb j, also carries (p mod q_j) * new_key_j.
//
// Two sources of randomness.  keygen_* / encrypt_symmetric draw from a
// counter-based hash of (seed, stream, index): reproducible and
// statistically sound but NOT a cryptographic generator, for tests and
// benchmarks.  seal_* draw from SEAL's own Blake2xbPRNG streams and samplers
// (seal_prng.cpp) and give SEAL's words for the same seeds.
#include <algorithm>
#include <random>
#include <stdexcept>
#include <vector>

#include "context.h"
#include "ntt.h"
#include "ops.h"
#include "seal_prng.h"

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

// raw uniform words [rows][N] to residues mod the prime of each row (in place allowed)
__global__ void k_reduce_rows(const uint64_t *raw, uint64_t *out, const PrimeConst *__restrict__ pc, int logn,
                              size_t total)
{
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const PrimeConst P = pc[x >> logn];
        out[x] = barrett_128(raw[x], 0, P.q, P.r0, P.r1);
    }
}

// c0 = -(s a + e) (+ m) over `limbs` limbs, and on limb `digit` also
// + nk * factor: encrypt_zero_symmetric's c0 (util/rlwe.cpp:387-422), the
// plaintext added by Encryptor::encrypt_internal (encryptor.cpp:232-236) and
// the key term of generate_one_kswitch_key (keygenerator.cpp:324-329)
__global__ void k_seal_c0(uint64_t *c0, const uint64_t *__restrict__ a, const uint64_t *__restrict__ e,
                          const uint64_t *__restrict__ s, const uint64_t *__restrict__ m,
                          const uint64_t *__restrict__ nk, int digit, uint64_t factor,
                          const PrimeConst *__restrict__ pc, int limbs, int logn)
{
    const size_t total = (size_t)limbs << logn;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const int l = (int)(x >> logn);
        const PrimeConst P = pc[l];
        uint64_t v = csub(mul_mod(s[x], a[x], P.q, P.r0, P.r1) + e[x], P.q);
        v = v ? P.q - v : 0;
        if (m) v = csub(v + m[x], P.q);
        if (l == digit) v = csub(v + mul_mod(nk[x], factor, P.q, P.r0, P.r1), P.q);
        c0[x] = v;
    }
}

// c[j] = u pk[j] + e[j], j = 0, 1, over `limbs` limbs (encrypt_zero_asymmetric,
// util/rlwe.cpp:224-309); pk components are pk_pitch words apart
__global__ void k_seal_asym(uint64_t *c, const uint64_t *__restrict__ u, const uint64_t *__restrict__ e,
                            const uint64_t *__restrict__ pk, size_t pk_pitch, const PrimeConst *__restrict__ pc,
                            int limbs, int logn)
{
    const size_t per = (size_t)limbs << logn;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < 2 * per; x += (size_t)gridDim.x * blockDim.x) {
        const size_t j = x / per, y = x - j * per;
        const PrimeConst P = pc[y >> logn];
        c[x] = csub(mul_mod(u[y], pk[j * pk_pitch + y], P.q, P.r0, P.r1) + e[x], P.q);
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

// ---------------------------------------------------------------------------
// Key generation and encryption with SEAL's own randomness: every seed is the
// 64-byte seed that one UniformRandomGeneratorFactory::create() call gives a
// Blake2xbPRNG (a factory built with a default seed gives that seed to every
// call).  The uniform samples' streams run on the GPU (seal_prng_gpu.cu), the
// short ones (secret, noise, ternary u) on the host (seal_prng.cpp), the NTTs
// and the modular arithmetic here.

namespace {

struct DeviceTemp {
    void *p = nullptr;
    cudaStream_t s;
    DeviceTemp(size_t bytes, cudaStream_t st) : s(st)
    {
        if (cudaMallocAsync(&p, bytes, s) != cudaSuccess) throw std::runtime_error("cudaMallocAsync failed");
    }
    ~DeviceTemp() { cudaFreeAsync(p, s); }
    template <class T> T *as(size_t byte_offset = 0) { return reinterpret_cast<T *>((char *)p + byte_offset); }
};

// small signed values (int8 on the host) as residues [limbs][N] on the device
void upload_small(Context &c, const std::vector<int8_t> &v, int8_t *d_tmp, uint64_t *out, int limbs, cudaStream_t s)
{
    cudaMemcpyAsync(d_tmp, v.data(), v.size(), cudaMemcpyHostToDevice, s);
    k_small_to_rns<<<grid_for(c.n), kBlock, 0, s>>>(d_tmp, out, c.d_pc, limbs, c.logn); NEXUS_LAUNCHED();
}

// encrypt_zero_symmetric(secret_key, level of `limbs` primes, is_ntt_form,
// no saved seed) (util/rlwe.cpp:311-441) into ct [2][limbs][N], with the
// plaintext m and the key-switching term folded into c0.  `e` [limbs][N] and
// `e8` [N] are device scratch; with reuse_noise the noise already in `e`
// and the c1 already in ct (same seed as the call before) are kept.
void seal_zero_symmetric(Context &c, const uint64_t seed[8], const uint64_t *sk, const uint64_t *m, int limbs,
                         const uint64_t *nk, int digit, uint64_t factor, uint64_t *ct, uint64_t *e, int8_t *e8,
                         bool reuse_noise, cudaStream_t s)
{
    const size_t N = c.n, words = (size_t)limbs * N;
    uint64_t *c1 = ct + words;
    if (!reuse_noise) {
        sealrng::Stream boot(seed);
        uint64_t pub[sealrng::kSeedWords];
        boot.bytes(reinterpret_cast<uint8_t *>(pub), sizeof(pub));
        sealrng::sample_uniform_raw_device(pub, c.logn, c.q.data(), limbs, c1, s);
        std::vector<int8_t> noise(N);
        sealrng::sample_cbd(boot, N, noise.data());
        k_reduce_rows<<<grid_for(words), kBlock, 0, s>>>(c1, c1, c.d_pc, c.logn, words); NEXUS_LAUNCHED();
        upload_small(c, noise, e8, e, limbs, s);
        ntt_forward(c, e, 1, 0, limbs, s);
    }
    k_seal_c0<<<grid_for(words), kBlock, 0, s>>>(ct, c1, e, sk, m, nk, digit, factor, c.d_pc, limbs, c.logn);
    NEXUS_LAUNCHED();
}

void check_level(const Context &c, int limbs)
{
    if (limbs < 1 || limbs > c.k) throw std::invalid_argument("parms_id is not valid for encryption parameters");
}

}  // namespace

void seal_keygen_secret(Context &c, const uint64_t seed[8], int hamming_weight, uint64_t *sk, cudaStream_t s)
{
    const size_t N = c.n, words = (size_t)c.k * N;
    if (hamming_weight < 0 || (size_t)hamming_weight > N) throw std::invalid_argument("invalid hamming weight");
    sealrng::Stream st(seed);
    if (hamming_weight > 0) {
        std::vector<uint64_t> v(words);
        sealrng::sample_sparse_ternary(st, N, c.q.data(), c.k, (size_t)hamming_weight, v.data());
        // A draw at position N leaves q_{r-1} - 1 at coefficient 0 of row r.
        // SEAL's forward NTT takes inputs below 4 q_r to the canonical
        // transform of their residue; from 4 q_r up its output words are out
        // of range and SEAL rejects the key (is_valid_for) when it is used.
        for (int r = 1; r < c.k; ++r) {
            uint64_t &x = v[(size_t)r * N];
            if (x >= c.q[r]) {
                if (x / 4 >= c.q[r]) throw std::invalid_argument("secret key is not valid for encryption parameters");
                x %= c.q[r];
            }
        }
        cudaMemcpyAsync(sk, v.data(), words * sizeof(uint64_t), cudaMemcpyHostToDevice, s);
    } else {
        std::vector<int8_t> v(N);
        sealrng::sample_ternary(st, N, v.data());
        DeviceTemp t(N, s);
        upload_small(c, v, t.as<int8_t>(), sk, c.k, s);
    }
    ntt_forward(c, sk, 1, 0, c.k, s);
    cudaStreamSynchronize(s);
}

void seal_encrypt_zero_symmetric(Context &c, const uint64_t seed[8], const uint64_t *sk, const uint64_t *m,
                                 int limbs, uint64_t *ct, cudaStream_t s)
{
    check_level(c, limbs);
    const size_t words = (size_t)limbs * c.n;
    DeviceTemp t(words * sizeof(uint64_t) + c.n, s);
    seal_zero_symmetric(c, seed, sk, m, limbs, nullptr, -1, 0, ct, t.as<uint64_t>(),
                        t.as<int8_t>(words * sizeof(uint64_t)), false, s);
    cudaStreamSynchronize(s);
}

void seal_keygen_kswitch(Context &c, const uint64_t *seeds, const uint64_t *sk, const uint64_t *new_key,
                         uint64_t *key, cudaStream_t s)
{
    const size_t N = c.n, K = (size_t)c.k, words = K * N;
    DeviceTemp t(words * sizeof(uint64_t) + N, s);
    uint64_t *e = t.as<uint64_t>();
    int8_t *e8 = t.as<int8_t>(words * sizeof(uint64_t));
    const uint64_t p = c.q[K - 1];
    for (size_t j = 0; j + 1 < K; ++j) {
        const uint64_t *sd = seeds + j * sealrng::kSeedWords;
        uint64_t *kj = key + j * 2 * words;
        const bool same = j > 0 && std::equal(sd, sd + sealrng::kSeedWords, sd - sealrng::kSeedWords);
        if (same)   // same seed: the same c1 and noise as the digit before
            cudaMemcpyAsync(kj + words, kj - words, words * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s);
        seal_zero_symmetric(c, sd, sk, nullptr, (int)K, new_key, (int)j, p % c.q[j], kj, e, e8, same, s);
    }
    cudaStreamSynchronize(s);
}

void seal_keygen_relin(Context &c, const uint64_t *seeds, const uint64_t *sk, uint64_t *key, cudaStream_t s)
{
    const size_t words = (size_t)c.k * c.n;
    DeviceTemp sq(words * sizeof(uint64_t), s);
    k_square<<<grid_for(words), kBlock, 0, s>>>(sq.as<uint64_t>(), sk, c.d_pc, c.logn, words); NEXUS_LAUNCHED();
    seal_keygen_kswitch(c, seeds, sk, sq.as<uint64_t>(), key, s);
}

void seal_keygen_galois(Context &c, const uint64_t *seeds, const uint64_t *sk, uint32_t elt, uint64_t *key,
                        cudaStream_t s)
{
    const size_t words = (size_t)c.k * c.n;
    DeviceTemp rot(words * sizeof(uint64_t), s);
    galois_permute(c, sk, 1, c.k, elt, rot.as<uint64_t>(), s);
    seal_keygen_kswitch(c, seeds, sk, rot.as<uint64_t>(), key, s);
}

// Encryptor::encrypt with the public key (encryptor.cpp:88-174, 176-237): an
// asymmetric encryption of zero one level up (the key level for the first
// data level), divided and rounded by that level's last prime, plus m.
void seal_encrypt_asymmetric(Context &c, const uint64_t seed[8], const uint64_t *pk, const uint64_t *m, int limbs,
                             uint64_t *ct, cudaStream_t s)
{
    check_level(c, limbs);
    const size_t N = c.n;
    const int up = limbs < c.k ? limbs + 1 : limbs;
    const size_t words = (size_t)up * N;
    sealrng::Stream st(seed);
    std::vector<int8_t> u(N), e0(N), e1(N);
    sealrng::sample_ternary(st, N, u.data());
    sealrng::sample_cbd(st, N, e0.data());
    sealrng::sample_cbd(st, N, e1.data());
    // u [up][N] | e [2][up][N] | c [2][up][N] | int8 staging [3][N]
    DeviceTemp t(5 * words * sizeof(uint64_t) + 3 * N, s);
    uint64_t *du = t.as<uint64_t>(), *de = du + words, *dc = de + 2 * words;
    int8_t *d8 = t.as<int8_t>(5 * words * sizeof(uint64_t));
    upload_small(c, u, d8, du, up, s);
    upload_small(c, e0, d8 + N, de, up, s);
    upload_small(c, e1, d8 + 2 * N, de + words, up, s);
    ntt_forward(c, du, 1, 0, up, s);
    ntt_forward(c, de, 2, 0, up, s);
    k_seal_asym<<<grid_for(2 * words), kBlock, 0, s>>>(dc, du, de, pk, (size_t)c.k * N, c.d_pc, up, c.logn);
    NEXUS_LAUNCHED();
    if (up > limbs)
        rescale(c, dc, 2, up, ct, s);
    else
        cudaMemcpyAsync(ct, dc, 2 * words * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s);
    if (m) poly_add(c, ct, m, 1, limbs, ct, s);
    cudaStreamSynchronize(s);
}

}  // namespace nexus
