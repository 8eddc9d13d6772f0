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

void ntt_forward(const Context &c, uint64_t *data, size_t n_polys, LimbMap lm, cudaStream_t s);
void ntt_inverse(const Context &c, uint64_t *data, size_t n_polys, LimbMap lm, cudaStream_t s);

// data: [n_polys][limb_end - limb_begin][N]; limb l of each polynomial uses
// prime limb_begin + l.  Input residues in [0, q), output in [0, q).
void ntt_forward(const Context &c, uint64_t *data, size_t n_polys, int limb_begin, int limb_end, cudaStream_t s);
void ntt_inverse(const Context &c, uint64_t *data, size_t n_polys, int limb_begin, int limb_end, cudaStream_t s);

}  // namespace nexus
