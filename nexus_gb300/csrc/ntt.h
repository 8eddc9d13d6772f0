// Internal launchers of the batched negacyclic NTT (see ntt.cu).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "context.h"

namespace nexus {

// Which prime each limb of a polynomial uses: limb l < count-1 (or every
// limb when special_last < 0) uses prime begin + l; with special_last >= 0 the
// last limb uses prime special_last (the ModUp layout q_0..q_{l-1}, p).
struct LimbMap {
    int count;
    int begin;
    int special_last;
    __host__ __device__ int prime(int l) const
    {
        return (special_last >= 0 && l == count - 1) ? special_last : begin + l;
    }
};

// Where the forward NTT's first pass reads its input.  Besides the in-place
// transform it can fuse the two element-wise steps of a key switch that feed
// an NTT: the ModUp spread (limb p of the output is row p / group of `src`,
// a coefficient-form residue of prime (p / group) % src_limbs, reduced into the
// output prime) and the ModDown rounding spread (row p / group of `src` is
// the coefficient-form special limb x; the input is ((x + h) mod P) mod q
// + (q - h mod q) with h = P/2 and P the prime `special`).
struct NttLoader {
    int kind = 0;                   // 0 in place, 1 ModUp spread, 2 rounding spread
    const uint64_t *src = nullptr;
    int group = 1;
    int src_limbs = 1;
    int special = 0;
};

void ntt_forward(const Context &c, uint64_t *data, size_t n_polys, LimbMap lm, cudaStream_t s);
void ntt_forward_loaded(const Context &c, uint64_t *data, size_t n_polys, LimbMap lm, NttLoader ld, cudaStream_t s);
void ntt_inverse(const Context &c, uint64_t *data, size_t n_polys, LimbMap lm, cudaStream_t s);

// data: [n_polys][limb_end - limb_begin][N]; limb l of each polynomial uses
// prime limb_begin + l.  Input residues in [0, q), output in [0, q).
void ntt_forward(const Context &c, uint64_t *data, size_t n_polys, int limb_begin, int limb_end, cudaStream_t s);
void ntt_inverse(const Context &c, uint64_t *data, size_t n_polys, int limb_begin, int limb_end, cudaStream_t s);

}  // namespace nexus
