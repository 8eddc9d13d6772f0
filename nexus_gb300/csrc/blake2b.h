// BLAKE2b (RFC 7693) compression and the BLAKE2X parameter blocks used by
// Blake2xbPRNG, shared by the host stream (seal_prng.cpp) and the device
// refills (seal_prng_gpu.cu).
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define NEXUS_HD __host__ __device__ __forceinline__
#else
#define NEXUS_HD inline
#endif

namespace nexus {
namespace blake2b {

// RFC 7693, section 2.6: the SHA-512 initial value
NEXUS_HD constexpr uint64_t iv(int i)
{
    constexpr uint64_t t[8] = {0x6a09e667f3bcc908ull, 0xbb67ae8584caa73bull, 0x3c6ef372fe94f82bull,
                               0xa54ff53a5f1d36f1ull, 0x510e527fade682d1ull, 0x9b05688c2b3e6c1full,
                               0x1f83d9abfb41bd6bull, 0x5be0cd19137e2179ull};
    return t[i];
}

// RFC 7693, section 2.7: message word schedule of the ten distinct rounds
// (a constexpr function, so that with the rounds unrolled every index folds
// to a constant and the message words stay in registers on the GPU)
NEXUS_HD constexpr int sigma(int r, int i)
{
    constexpr uint8_t t[10][16] = {
        {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15}, {14, 10, 4, 8, 9, 15, 13, 6, 1, 12, 0, 2, 11, 7, 5, 3},
        {11, 8, 12, 0, 5, 2, 15, 13, 10, 14, 3, 6, 7, 1, 9, 4}, {7, 9, 3, 1, 13, 12, 11, 14, 2, 6, 5, 10, 4, 0, 15, 8},
        {9, 0, 5, 7, 2, 4, 10, 15, 14, 1, 11, 12, 6, 8, 3, 13}, {2, 12, 6, 10, 0, 11, 8, 3, 4, 13, 7, 5, 15, 14, 1, 9},
        {12, 5, 1, 15, 14, 13, 4, 10, 0, 7, 6, 3, 9, 2, 8, 11}, {13, 11, 7, 14, 12, 1, 3, 9, 5, 0, 15, 4, 8, 6, 2, 10},
        {6, 15, 14, 9, 11, 3, 0, 8, 12, 2, 13, 7, 1, 4, 10, 5}, {10, 2, 8, 4, 7, 6, 1, 5, 15, 11, 9, 14, 3, 12, 13, 0}};
    return t[r % 10][i];
}

NEXUS_HD uint64_t rotr(uint64_t x, int r) { return (x >> r) | (x << (64 - r)); }

// RFC 7693, section 3.1: the mixing function G
NEXUS_HD void mix(uint64_t v[16], int a, int b, int c, int d, uint64_t x, uint64_t y)
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
// count t (below 2^64 here) and the final-block flag.  Fully unrolled, so
// every message index is a constant and m stays in registers on the GPU.
NEXUS_HD void compress(uint64_t h[8], const uint64_t m[16], uint64_t t, bool last)
{
    uint64_t v[16];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        v[i] = h[i];
        v[i + 8] = iv(i);
    }
    v[12] ^= t;
    if (last) v[14] = ~v[14];
#pragma unroll
    for (int r = 0; r < 12; ++r) {
        mix(v, 0, 4, 8, 12, m[sigma(r, 0)], m[sigma(r, 1)]);
        mix(v, 1, 5, 9, 13, m[sigma(r, 2)], m[sigma(r, 3)]);
        mix(v, 2, 6, 10, 14, m[sigma(r, 4)], m[sigma(r, 5)]);
        mix(v, 3, 7, 11, 15, m[sigma(r, 6)], m[sigma(r, 7)]);
        mix(v, 0, 5, 10, 15, m[sigma(r, 8)], m[sigma(r, 9)]);
        mix(v, 1, 6, 11, 12, m[sigma(r, 10)], m[sigma(r, 11)]);
        mix(v, 2, 7, 8, 13, m[sigma(r, 12)], m[sigma(r, 13)]);
        mix(v, 3, 4, 9, 14, m[sigma(r, 14)], m[sigma(r, 15)]);
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) h[i] ^= v[i] ^ v[i + 8];
}

// initial state for a parameter block whose first three words carry digest
// length, key length, fanout, depth, leaf length | node offset, XOF length |
// node depth, inner length (the rest zero)
NEXUS_HD void init_param(uint64_t h[8], unsigned digest, unsigned key, unsigned fanout, unsigned depth, uint32_t leaf,
                         uint32_t node_offset, uint32_t xof_len, unsigned node_depth, unsigned inner)
{
#pragma unroll
    for (int i = 0; i < 8; ++i) h[i] = iv(i);
    h[0] ^= (uint64_t)digest | ((uint64_t)key << 8) | ((uint64_t)fanout << 16) | ((uint64_t)depth << 24) |
            ((uint64_t)leaf << 32);
    h[1] ^= (uint64_t)node_offset | ((uint64_t)xof_len << 32);
    h[2] ^= (uint64_t)node_depth | ((uint64_t)inner << 8);
}

// BLAKE2Xb with a 64-byte key, an 8-byte message and `xof_len` bytes of
// output: the root is keyed BLAKE2b-512 of the message with the XOF length
// in the parameter block (the key fills the first block, the message the
// second) ...
NEXUS_HD void xof_root(const uint64_t key[8], uint64_t message, uint32_t xof_len, uint64_t root[8])
{
    uint64_t m[16];
    init_param(root, 64, 64, 1, 1, 0, 0, xof_len, 0, 0);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        m[i] = key[i];
        m[i + 8] = 0;
    }
    compress(root, m, 128, false);
    m[0] = message;
#pragma unroll
    for (int i = 1; i < 16; ++i) m[i] = 0;
    compress(root, m, 128 + 8, true);
}

// ... and output block i is unkeyed BLAKE2b-512 of the root with node offset
// i, leaf and inner length 64 (whole 64-byte blocks only)
NEXUS_HD void xof_block(const uint64_t root[8], uint32_t i, uint32_t xof_len, uint64_t out[8])
{
    uint64_t m[16];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        m[k] = root[k];
        m[k + 8] = 0;
    }
    init_param(out, 64, 0, 0, 0, 64, i, xof_len, 0, 64);
    compress(out, m, 64, true);
}

}  // namespace blake2b
}  // namespace nexus
