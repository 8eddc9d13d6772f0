// SEAL's seeded randomness on the host: BLAKE2b / BLAKE2Xb, the byte stream
// of Blake2xbPRNG and the samplers of util/rlwe.cpp (declarations and
// references in seal_prng.h).
#include "seal_prng.h"

#include <algorithm>
#include <cstring>
#include <stdexcept>
#include <thread>
#include <vector>

#if !defined(__BYTE_ORDER__) || __BYTE_ORDER__ != __ORDER_LITTLE_ENDIAN__
#error "the stream is read as little-endian words"
#endif

namespace nexus {
namespace sealrng {

namespace {

// RFC 7693, section 2.6: the SHA-512 initial value
constexpr uint64_t kIV[8] = {0x6a09e667f3bcc908ull, 0xbb67ae8584caa73bull, 0x3c6ef372fe94f82bull,
                             0xa54ff53a5f1d36f1ull, 0x510e527fade682d1ull, 0x9b05688c2b3e6c1full,
                             0x1f83d9abfb41bd6bull, 0x5be0cd19137e2179ull};

// RFC 7693, section 2.7: message word schedule of the ten distinct rounds
constexpr uint8_t kSigma[10][16] = {
    {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15}, {14, 10, 4, 8, 9, 15, 13, 6, 1, 12, 0, 2, 11, 7, 5, 3},
    {11, 8, 12, 0, 5, 2, 15, 13, 10, 14, 3, 6, 7, 1, 9, 4}, {7, 9, 3, 1, 13, 12, 11, 14, 2, 6, 5, 10, 4, 0, 15, 8},
    {9, 0, 5, 7, 2, 4, 10, 15, 14, 1, 11, 12, 6, 8, 3, 13}, {2, 12, 6, 10, 0, 11, 8, 3, 4, 13, 7, 5, 15, 14, 1, 9},
    {12, 5, 1, 15, 14, 13, 4, 10, 0, 7, 6, 3, 9, 2, 8, 11}, {13, 11, 7, 14, 12, 1, 3, 9, 5, 0, 15, 4, 8, 6, 2, 10},
    {6, 15, 14, 9, 11, 3, 0, 8, 12, 2, 13, 7, 1, 4, 10, 5}, {10, 2, 8, 4, 7, 6, 1, 5, 15, 11, 9, 14, 3, 12, 13, 0}};

inline uint64_t rotr(uint64_t x, int r) { return (x >> r) | (x << (64 - r)); }

// RFC 7693, section 3.1: the mixing function G
inline void mix(uint64_t v[16], int a, int b, int c, int d, uint64_t x, uint64_t y)
{
    v[a] += v[b] + x;
    v[d] = rotr(v[d] ^ v[a], 32);
    v[c] += v[d];
    v[b] = rotr(v[b] ^ v[c], 24);
    v[a] += v[b] + y;
    v[d] = rotr(v[d] ^ v[a], 16);
    v[c] += v[d];
    v[b] = rotr(v[b] ^ v[c], 63);
}

// RFC 7693, section 3.2: compression of one 128-byte block m with byte
// count t (below 2^64 here) and the final-block flag
void compress(uint64_t h[8], const uint64_t m[16], uint64_t t, bool last)
{
    uint64_t v[16];
    for (int i = 0; i < 8; ++i) {
        v[i] = h[i];
        v[i + 8] = kIV[i];
    }
    v[12] ^= t;
    if (last) v[14] = ~v[14];
    for (int r = 0; r < 12; ++r) {
        const uint8_t *s = kSigma[r % 10];
        mix(v, 0, 4, 8, 12, m[s[0]], m[s[1]]);
        mix(v, 1, 5, 9, 13, m[s[2]], m[s[3]]);
        mix(v, 2, 6, 10, 14, m[s[4]], m[s[5]]);
        mix(v, 3, 7, 11, 15, m[s[6]], m[s[7]]);
        mix(v, 0, 5, 10, 15, m[s[8]], m[s[9]]);
        mix(v, 1, 6, 11, 12, m[s[10]], m[s[11]]);
        mix(v, 2, 7, 8, 13, m[s[12]], m[s[13]]);
        mix(v, 3, 4, 9, 14, m[s[14]], m[s[15]]);
    }
    for (int i = 0; i < 8; ++i) h[i] ^= v[i] ^ v[i + 8];
}

// BLAKE2b parameter block, first three words (the rest is zero here):
// digest length, key length, fanout, depth, leaf length | node offset, XOF
// length | node depth, inner length
inline void init_param(uint64_t h[8], unsigned digest, unsigned key, unsigned fanout, unsigned depth, uint32_t leaf,
                       uint32_t node_offset, uint32_t xof_len, unsigned node_depth, unsigned inner)
{
    for (int i = 0; i < 8; ++i) h[i] = kIV[i];
    h[0] ^= (uint64_t)digest | ((uint64_t)key << 8) | ((uint64_t)fanout << 16) | ((uint64_t)depth << 24) |
            ((uint64_t)leaf << 32);
    h[1] ^= (uint64_t)node_offset | ((uint64_t)xof_len << 32);
    h[2] ^= (uint64_t)node_depth | ((uint64_t)inner << 8);
}

unsigned worker_count(size_t blocks)
{
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    return (unsigned)std::min<size_t>({(size_t)hw, (size_t)32, std::max<size_t>(1, blocks / 16)});
}

}  // namespace

void blake2xb_refill(const uint64_t seed[kSeedWords], uint64_t counter, uint8_t out[kRefillBytes])
{
    // root: keyed BLAKE2b-512 of the counter with the XOF length in the
    // parameter block; the key fills the first block, the message the second
    uint64_t h[8], m[16];
    init_param(h, 64, 64, 1, 1, 0, 0, (uint32_t)kRefillBytes, 0, 0);
    for (int i = 0; i < 8; ++i) {
        m[i] = seed[i];
        m[i + 8] = 0;
    }
    compress(h, m, 128, false);
    m[0] = counter;
    for (int i = 1; i < 16; ++i) m[i] = 0;
    compress(h, m, 128 + 8, true);
    // output block i: unkeyed BLAKE2b-512 of the root with node offset i
    uint64_t root[16];
    for (int i = 0; i < 8; ++i) {
        root[i] = h[i];
        root[i + 8] = 0;
    }
    for (uint32_t i = 0; i < kRefillBytes / 64; ++i) {
        uint64_t g[8];
        init_param(g, 64, 0, 0, 0, 64, i, (uint32_t)kRefillBytes, 0, 64);
        compress(g, root, 64, true);
        std::memcpy(out + 64 * i, g, 64);
    }
}

Stream::Stream(const uint64_t seed[kSeedWords]) { std::memcpy(seed_, seed, sizeof(seed_)); }

void Stream::refill()
{
    blake2xb_refill(seed_, next_++, buf_);
    head_ = 0;
}

void Stream::seek(uint64_t pos)
{
    next_ = pos / kRefillBytes;
    head_ = kRefillBytes;
    if (pos % kRefillBytes) {
        refill();
        head_ = (size_t)(pos % kRefillBytes);
    }
}

void Stream::bytes(uint8_t *dst, size_t n)
{
    while (n) {
        if (head_ == kRefillBytes) refill();
        const size_t take = std::min(n, kRefillBytes - head_);
        std::memcpy(dst, buf_ + head_, take);
        head_ += take;
        dst += take;
        n -= take;
    }
}

uint32_t Stream::u32()
{
    uint32_t v;
    bytes(reinterpret_cast<uint8_t *>(&v), sizeof(v));
    return v;
}

uint64_t Stream::u64()
{
    uint64_t v;
    bytes(reinterpret_cast<uint8_t *>(&v), sizeof(v));
    return v;
}

void Stream::bytes_parallel(uint8_t *dst, size_t n)
{
    const size_t first = std::min(n, kRefillBytes - head_);
    bytes(dst, first);
    dst += first;
    n -= first;
    const size_t blocks = n / kRefillBytes;
    const uint64_t base = next_;
    const unsigned workers = worker_count(blocks);
    auto run = [&](unsigned w) {
        for (size_t b = w; b < blocks; b += workers) blake2xb_refill(seed_, base + b, dst + b * kRefillBytes);
    };
    if (workers <= 1) {
        run(0);
    } else {
        std::vector<std::thread> pool;
        for (unsigned w = 1; w < workers; ++w) pool.emplace_back(run, w);
        run(0);
        for (auto &t : pool) t.join();
    }
    next_ = base + blocks;
    bytes(dst + blocks * kRefillBytes, n - blocks * kRefillBytes);
}

uint64_t uniform_int(Stream &s, uint64_t lo, uint64_t hi)
{
    const uint64_t range = hi - lo + 1;
    if (hi < lo || range > 0xFFFFFFFFull) throw std::invalid_argument("uniform_int: range must fit 32 bits");
    const uint32_t r = (uint32_t)range;
    uint64_t product = (uint64_t)s.u32() * r;
    uint32_t low = (uint32_t)product;
    if (low < r) {
        const uint32_t threshold = (uint32_t)(0u - r) % r;
        while (low < threshold) {
            product = (uint64_t)s.u32() * r;
            low = (uint32_t)product;
        }
    }
    return lo + (product >> 32);
}

void sample_ternary(Stream &s, size_t n, int8_t *out)
{
    for (size_t i = 0; i < n; ++i) out[i] = (int8_t)((int)uniform_int(s, 0, 2) - 1);
}

void sample_cbd(Stream &s, size_t n, int8_t *out)
{
    for (size_t i = 0; i < n; ++i) {
        uint8_t x[6];
        s.bytes(x, 6);
        x[2] &= 0x1F;
        x[5] &= 0x1F;
        out[i] = (int8_t)(__builtin_popcount(x[0]) + __builtin_popcount(x[1]) + __builtin_popcount(x[2]) -
                          __builtin_popcount(x[3]) - __builtin_popcount(x[4]) - __builtin_popcount(x[5]));
    }
}

void sample_sparse_ternary(Stream &s, size_t n, const uint64_t *q, int k, size_t hw, uint64_t *out)
{
    if (k < 1) throw std::invalid_argument("sample_sparse_ternary: no primes");
    if (hw > n) throw std::invalid_argument("sample_sparse_ternary: hamming weight exceeds the degree");
    const size_t words = (size_t)k * n;
    std::vector<uint64_t> a(words + 1, 0);      // one word past the rows, as written by position n
    size_t weight = 0;
    while (weight < hw) {
        const size_t index = (size_t)uniform_int(s, 0, n);
        if (a[index] != 0) continue;
        const bool neg = uniform_int(s, 0, 1) == 0;     // 2 * {0, 1} - 1
        for (int i = 0; i < k; ++i) a[index + (size_t)i * n] = neg ? q[i] - 1 : 1;
        ++weight;
    }
    std::memcpy(out, a.data(), words * sizeof(uint64_t));
}

uint64_t uniform_bound(uint64_t q) { return ~0ull - (~0ull % q) - 1; }

void sample_uniform_raw(Stream &s, size_t n, const uint64_t *q, int k, uint64_t *raw)
{
    const size_t words = (size_t)k * n;
    s.bytes_parallel(reinterpret_cast<uint8_t *>(raw), words * sizeof(uint64_t));
    for (int j = 0; j < k; ++j) {
        const uint64_t bound = uniform_bound(q[j]);
        uint64_t *row = raw + (size_t)j * n;
        for (size_t i = 0; i < n; ++i)
            while (row[i] >= bound) row[i] = s.u64();
    }
}

}  // namespace sealrng
}  // namespace nexus
