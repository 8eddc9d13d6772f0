// CKKS encoder (host FP64 special FFT, bit-identical to SEAL's CKKSEncoder).
#pragma once
#include <complex>
#include <cstdint>
#include <vector>

#include "context.h"

namespace nexus {

class Encoder {
public:
    explicit Encoder(const Context &c);
    // values[nvals] (nvals <= N/2) at `scale` into coefficient-form residues
    // out[limbs][N] (the caller applies the forward NTT)
    // check_limbs > 0: bound checks as for an encode at that level (SEAL's
    // encode at the top level followed by mod_switch_to keeps the top-level
    // checks while only the first `limbs` residues survive)
    void encode(const std::complex<double> *values, size_t nvals, double scale, int limbs, uint64_t *out,
                int check_limbs = 0) const;
    // residue of round(value * scale) in each of the first `limbs` primes
    void encode_scalar(double value, double scale, int limbs, uint64_t *per_limb, int check_limbs = 0) const;
    // coefficient-form residues coeffs[limbs][N] -> nvals slot values;
    // sparse_slots (0 = all) zeroes coefficients as the fork's sparse decode does
    void decode(const uint64_t *coeffs, int limbs, double scale, std::complex<double> *out, size_t nvals,
                size_t sparse_slots) const;
    size_t slots() const { return slots_; }

private:
    const Context &ctx_;
    size_t slots_ = 0;
    std::vector<uint32_t> index_map_;
    std::vector<std::complex<double>> root_powers_, inv_root_powers_;
};

}  // namespace nexus
