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
//
// skip_diag: the polynomials are the digits of a ModUp, stored with count + 1
// limbs each ([B][count digits][count + 1][N], the last limb on special_last)
// and digit j's limb j is left out of the transform (it is the NTT-form
// target limb itself).  The transform then covers count limbs per digit:
// launch limb m of digit j is stored limb m + (m >= j).
struct LimbMap {
    int count;
    int begin;
    int special_last;
    int skip_diag = 0;
    __host__ __device__ int prime(int l) const
    {
        return (special_last >= 0 && l == count - 1) ? special_last : begin + l;
    }
    // Memory row (limb index from the start of the buffer) and prime of
    // launch limb pl; launches hold fewer than 2^32 limbs.
    __host__ __device__ void locate(uint32_t pl, size_t &row, int &p) const
    {
        const uint32_t cnt = (uint32_t)count;
        const uint32_t poly = pl / cnt, m = pl - poly * cnt;
        if (!skip_diag) {
            row = pl;
            p = prime((int)m);
            return;
        }
        const uint32_t j = poly % cnt, i = m + (m >= j ? 1u : 0u);
        row = (size_t)poly * (cnt + 1) + i;
        p = (i == cnt) ? special_last : begin + (int)i;
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

// Butterflies per second of the NTT's own butterfly (mode 0: forward, 1:
// forward for primes below 2^52, 2: inverse) on register data over the whole
// GPU: the compute ceiling of the transform.  Synchronous; *ms receives the
// duration of one launch.
double butterfly_rate(int mode, uint64_t q, int rounds, int blocks_per_sm, double *ms);

}  // namespace nexus
