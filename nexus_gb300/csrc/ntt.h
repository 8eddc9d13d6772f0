// Internal launchers of the batched negacyclic NTT (see ntt.cu).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "context.h"

namespace nexus {

// data: [n_polys][limb_end - limb_begin][N]; limb l of each polynomial uses
// prime limb_begin + l.  Input residues in [0, q), output in [0, q).
void ntt_forward(const Context &c, uint64_t *data, size_t n_polys, int limb_begin, int limb_end, cudaStream_t s);
void ntt_inverse(const Context &c, uint64_t *data, size_t n_polys, int limb_begin, int limb_end, cudaStream_t s);

}  // namespace nexus
