// Device-side modular arithmetic on 64-bit RNS residues (primes < 2^61).
//
// Every operation is exact integer math.  Lazy ranges follow the Harvey
// butterfly conventions used by SEAL's NTT (util/ntt.h:21-67 in the SEAL-4.1-bs
// tree): a value "in [0, kq)" is congruent to the true residue and below kq.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace nexus {

#if defined(__CUDACC__)
// Shoup multiplication: w < q, wq = floor(w * 2^64 / q).  For any x < 2^64
// the result is congruent to x*w mod q and lies in [0, 2q).
__device__ __forceinline__ uint64_t mul_shoup_lazy(uint64_t x, uint64_t w, uint64_t wq, uint64_t q)
{
    uint64_t hi = __umul64hi(x, wq);
    return x * w - hi * q;
}

__device__ __forceinline__ uint64_t csub(uint64_t x, uint64_t m) { return x >= m ? x - m : x; }

__device__ __forceinline__ uint64_t mul_shoup(uint64_t x, uint64_t w, uint64_t wq, uint64_t q)
{
    return csub(mul_shoup_lazy(x, w, wq, q), q);
}

// Barrett reduction of a 128-bit value (hi:lo) by q < 2^61 with
// ratio = floor(2^128 / q) given as (r1:r0).  Returns the residue in [0, q).
__device__ __forceinline__ uint64_t barrett_128(uint64_t lo, uint64_t hi, uint64_t q, uint64_t r0, uint64_t r1)
{
    // estimate floor(x * ratio / 2^128) using the top words only
    uint64_t c1 = __umul64hi(lo, r0);
    uint64_t a_lo = lo * r1, a_hi = __umul64hi(lo, r1);
    uint64_t b_lo = hi * r0, b_hi = __umul64hi(hi, r0);
    // sum of middle terms: c1 + a_lo + b_lo, carries into top
    uint64_t s = c1 + a_lo;
    uint64_t carry = s < c1;
    uint64_t s2 = s + b_lo;
    carry += s2 < s;
    uint64_t top = hi * r1 + a_hi + b_hi + carry;
    uint64_t r = lo - top * q;
    // top is the quotient estimate mod 2^64; it undershoots floor(x/q) by
    // at most 2, so the wrapped difference is the remainder plus < 2q
    r = csub(r, q);
    return csub(r, q);
}

// Full product a*b mod q for a, b < 2^64 via Barrett.
__device__ __forceinline__ uint64_t mul_mod(uint64_t a, uint64_t b, uint64_t q, uint64_t r0, uint64_t r1)
{
    return barrett_128(a * b, __umul64hi(a, b), q, r0, r1);
}

// Barrett reduction of a 64-bit value: r1 = floor(2^128/q) >> 64 = floor(2^64/q).
__device__ __forceinline__ uint64_t barrett_64(uint64_t x, uint64_t q, uint64_t r1)
{
    uint64_t t = __umul64hi(x, r1);
    return csub(x - t * q, q);
}

// barrett_64 for q > 2^32, where r1 = floor(2^64/q) fits in 32 bits: the
// same quotient floor(x * r1 / 2^64), formed exactly from two 32 x 32-bit
// products (x * r1 = x1 * r1 * 2^32 + x0 * r1), so the same result.
__device__ __forceinline__ uint64_t barrett_64_r32(uint64_t x, uint64_t q, uint32_t r1)
{
    const uint32_t x0 = (uint32_t)x, x1 = (uint32_t)(x >> 32);
    const uint64_t lo = (uint64_t)x0 * r1;
    const uint32_t t = (uint32_t)(((uint64_t)x1 * r1 + (lo >> 32)) >> 32);
    return csub(x - (uint64_t)t * q, q);
}

#endif  // __CUDACC__

// Per-prime constants stored on the device.
struct PrimeConst {
    uint64_t q;
    uint64_t r0, r1;      // floor(2^128 / q) = r1 * 2^64 + r0
    uint64_t inv_n, inv_n_q; // n^{-1} mod q and its Shoup quotient
};

#ifdef __CUDACC__

// Exact sums of products a * b with a, b < 2^52 from 32 x 32 -> 64 products
// of their 26-bit halves (Karatsuba): h += ah*bh, w += al*bl and
// x += (ah+al)*(bh+bl), each term below 2^54, so up to 32 terms stay below
// 2^59.  The middle term sum(ah*bl + al*bh) = x - h - w (below 2^58).
__device__ __forceinline__ void mac_split(uint64_t &h, uint64_t &x, uint64_t &w, uint64_t a, uint64_t b)
{
    const uint32_t ah = (uint32_t)(a >> 26), al = (uint32_t)a & 0x3ffffffu;
    const uint32_t bh = (uint32_t)(b >> 26), bl = (uint32_t)b & 0x3ffffffu;
    h += (uint64_t)ah * bh;
    w += (uint64_t)al * bl;
    x += (uint64_t)(ah + al) * (bh + bl);
}

// hh * 2^52 + mid * 2^26 + ll as a 128-bit value, reduced mod q
__device__ __forceinline__ uint64_t reduce_split(uint64_t hh, uint64_t mid, uint64_t ll, const PrimeConst &P)
{
    const uint64_t a = hh << 52, b = mid << 26;
    const uint64_t lo = a + b;
    uint64_t hi = (hh >> 12) + (mid >> 38) + (lo < a);
    const uint64_t lo2 = lo + ll;
    hi += lo2 < lo;
    return barrett_128(lo2, hi, P.q, P.r0, P.r1);
}

// the sum accumulated by mac_split, reduced mod q
__device__ __forceinline__ uint64_t reduce_karatsuba(uint64_t h, uint64_t x, uint64_t w, const PrimeConst &P)
{
    return reduce_split(h, x - h - w, w, P);
}

#endif  // __CUDACC__

}  // namespace nexus
