// SEAL's seeded randomness on the host, for key generation and encryption
// that reproduce SEAL-4.1-bs word for word from the same seeds.
//
// The stream is Blake2xbPRNG's (randomgen.h:504-530, randomgen.cpp:197-207):
// refill r of the 4096-byte buffer is BLAKE2Xb with the 64-byte seed as key,
// the 8-byte little-endian counter r as message and 4096 bytes of output;
// bytes are handed out in order (UniformRandomGenerator::generate,
// randomgen.cpp:174-190).  BLAKE2b follows RFC 7693 and BLAKE2Xb the BLAKE2X
// specification (Aumasson, Neves, Wilcox-O'Hearn, Winnerlein, 2016); the
// NEXUS tree carries the BLAKE2 reference package for these
// (thirdparty/SEAL-4.1-bs/native/src/seal/util/blake2b.c, blake2xb.c).
//
// The samplers are those of util/rlwe.cpp:21-165 with SEAL's default noise
// sampler (centered binomial) and the NEXUS fork's sparse ternary secret.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace nexus {
namespace sealrng {

constexpr size_t kSeedWords = 8;       // prng_seed_type: 8 x uint64, the BLAKE2b key
constexpr size_t kRefillBytes = 4096;  // UniformRandomGenerator::buffer_size_

// One refill of Blake2xbPRNG: BLAKE2Xb(key = seed, message = counter, 4096 bytes).
void blake2xb_refill(const uint64_t seed[kSeedWords], uint64_t counter, uint8_t out[kRefillBytes]);

// The byte stream of one Blake2xbPRNG instance.
class Stream {
public:
    explicit Stream(const uint64_t seed[kSeedWords]);
    void bytes(uint8_t *dst, size_t n);      // UniformRandomGenerator::generate(n, dst)
    uint32_t u32();                           // generate() (RandomToStandardAdapter)
    uint64_t u64();                           // 8 bytes into a uint64_t
    // `n` bytes in order, whole refills computed by several host threads
    void bytes_parallel(uint8_t *dst, size_t n);
    // continue at byte `pos` of the stream
    void seek(uint64_t pos);

private:
    void refill();
    uint64_t seed_[kSeedWords];
    uint64_t next_ = 0;                       // counter of the next refill
    size_t head_ = kRefillBytes;              // buffer starts empty
    uint8_t buf_[kRefillBytes];
};

// std::uniform_int_distribution<uint64_t>(lo, hi) drawing 32-bit values, as
// libstdc++ (GCC 11 and later) computes it for a generator of exactly 32
// bits: Lemire's nearly divisionless method ("Fast Random Integer
// Generation in an Interval", ACM TOMACS 29(1), 2019).
uint64_t uniform_int(Stream &s, uint64_t lo, uint64_t hi);

// sample_poly_ternary (rlwe.cpp:21-37): values in {-1, 0, 1}
void sample_ternary(Stream &s, size_t n, int8_t *out);
// sample_poly_cbd (rlwe.cpp:99-135): centered binomial of 21 + 21 bits
void sample_cbd(Stream &s, size_t n, int8_t *out);
// sample_poly_sparse_ternary (rlwe.cpp:39-69): exactly hw nonzero +-1 over
// k residue rows out[k][n].  The fork draws positions from [0, n] inclusive;
// position n addresses coefficient 0 of rows 1..k-1 (each taking the residue
// of the row before) and one word past the array, which is dropped here.
void sample_sparse_ternary(Stream &s, size_t n, const uint64_t *q, int k, size_t hw, uint64_t *out);
// sample_poly_uniform (rlwe.cpp:137-165) before its reduction: raw[k][n]
// words, each redrawn while >= the largest multiple bound of its prime; the
// residue is raw mod q_j.
void sample_uniform_raw(Stream &s, size_t n, const uint64_t *q, int k, uint64_t *raw);
// the bound of sample_poly_uniform: 2^64 - 1 - ((2^64 - 1) mod q) - 1
uint64_t uniform_bound(uint64_t q);

// sample_uniform_raw of a fresh stream of `seed` into d_raw [k][2^logn] on
// the device (seal_prng_gpu.cu): the bulk refills on the GPU, the redraws
// from the stream after the bulk on the host.  Returns after the device work.
void sample_uniform_raw_device(const uint64_t seed[kSeedWords], int logn, const uint64_t *q, int k, uint64_t *d_raw,
                               cudaStream_t s);

}  // namespace sealrng
}  // namespace nexus
