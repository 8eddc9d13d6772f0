// SEAL's seeded randomness on the host: the byte stream of Blake2xbPRNG
// (BLAKE2Xb refills from blake2b.h) and the samplers of util/rlwe.cpp
// (declarations and references in seal_prng.h).
#include "seal_prng.h"
#include "blake2b.h"

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

unsigned worker_count(size_t blocks)
{
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    return (unsigned)std::min<size_t>({(size_t)hw, (size_t)32, std::max<size_t>(1, blocks / 16)});
}

}  // namespace

void blake2xb_refill(const uint64_t seed[kSeedWords], uint64_t counter, uint8_t out[kRefillBytes])
{
    uint64_t root[8];
    blake2b::xof_root(seed, counter, (uint32_t)kRefillBytes, root);
    for (uint32_t i = 0; i < kRefillBytes / 64; ++i) {
        uint64_t g[8];
        blake2b::xof_block(root, i, (uint32_t)kRefillBytes, g);
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
