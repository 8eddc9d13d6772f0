// NEXUS's CKKS bootstrapping on the engine: Bootstrapper
// (src/bootstrapping/Bootstrapper.{h,cpp}, the three-level BSGS "_3" path)
// and ModularReducer (src/bootstrapping/ModularReducer.{h,cpp}) with the
// heap-based polynomial evaluation of common/Polynomial.cpp:255-485.  Same
// member names, arguments and call order, so the ciphertext words equal the
// reference's for the same keys, input and EvalMod polynomial heap.
//
// Differences from the reference, none of which changes a result word:
//  * the EvalMod polynomial (minimax cosine + heap split) is computed once
//    offline in high precision and passed in as the doubles the reference
//    encodes (the reference runs its NTL Remez in prepare_mod_polynomial);
//  * every LT diagonal, once encoded at a given level and scale, is kept on
//    the device and reused by later bootstraps (the reference re-encodes it
//    each time; encoding is a pure function of values, scale and level).
#pragma once
#include <complex>
#include <cstdint>
#include <map>
#include <tuple>
#include <vector>

#include "batch.h"
#include "ckks.h"

namespace nexus {

using CVec = std::vector<std::complex<double>>;

// giantstep (common/func.cpp:204-214)
int giantstep(int m);
// rotation (common/func.cpp:216-225)
void rotation(int logslot, int nh, int shiftcount, const CVec &vec, CVec &rtnvec);
// genorigcoeff + genfftcoeff_3 + geninvfftcoeff_3 for one slot count 2^logn:
// out = {fftcoeff1, fftcoeff2, fftcoeff3, invfftcoeff1, invfftcoeff2, invfftcoeff3}
void lt_coefficients_3(long logn, long logNh, long boundary_K, std::vector<CVec> out[6]);

// EV / CT: Evaluator / Ciphertext (one ciphertext) or BatchEvaluator / CtBatch
// (ciphertexts in lockstep); the code is the same call sequence for both.
template <class EV, class CT>
class ModularReducerT {
public:
    long boundary_K;
    double log_width;
    long deg;
    long num_double_formula;
    long inverse_deg;
    double scale_inverse_coeff = 1.0;

    // Polynomial heap of the cosine (generate_poly_heap; scaled when
    // inverse_deg == 1): node i holds its Chebyshev coefficients; an empty
    // node is absent.
    long heap_k = 0, heap_m = 0;
    std::vector<std::vector<double>> heap;

    // The inverse-sine polynomial of inverse_deg > 1 (generate_inverse_sine_
    // polynomial, ModularReducer.cpp:38-47): its power-basis coefficients,
    // which the direct forms of degree <= 3 read, and above degree 3 its odd
    // heap (generate_poly_heap_odd).
    struct InversePoly {
        std::vector<double> power;
        long heap_k = 0, heap_m = 0;
        std::vector<std::vector<double>> heap;
    } inverse;

    ModularReducerT(EV &ev, long boundary_K, double log_width, long deg, long num_double_formula, long inverse_deg);
    void set_polynomial_heap(long k, long m, std::vector<std::vector<double>> nodes, double scale_inverse_coeff);
    void set_inverse_polynomial(InversePoly p);
    template <class EV2, class CT2>
    void adopt_polynomials(const ModularReducerT<EV2, CT2> &o)
    {
        set_polynomial_heap(o.heap_k, o.heap_m, o.heap, o.scale_inverse_coeff);
        inverse.power = o.inverse.power;
        inverse.heap_k = o.inverse.heap_k;
        inverse.heap_m = o.inverse.heap_m;
        inverse.heap = o.inverse.heap;
    }

    void double_angle_formula(CT &cipher);
    void double_angle_formula_scaled(CT &cipher, double scale_coeff);
    // Polynomial::homomorphic_poly_evaluation of the cosine heap
    void homomorphic_poly_evaluation(CT &rtn, const CT &cipher);
    // the same routine for any heap of degree >= 4 ...
    void evaluate_heap(CT &rtn, const CT &cipher, long k, long m, const std::vector<std::vector<double>> &nodes);
    // ... and its direct forms for degree 1-3 on power-basis coefficients
    void evaluate_power(CT &rtn, const CT &cipher, const std::vector<double> &coeff);
    void modular_reduction(CT &rtn, const CT &cipher);

private:
    EV *ev_;
};

template <class EV, class CT>
class BootstrapperT {
public:
    long loge, logn, n, logNh, Nh, L;
    double initial_scale = 0.0, final_scale;
    long boundary_K, sin_cos_deg, scale_factor, inverse_deg;

    std::vector<long> slot_vec;
    long slot_index = 0;
    // per slot_vec entry: the LT diagonals of the three levels
    std::vector<std::vector<CVec>> fftcoeff1, fftcoeff2, fftcoeff3;
    std::vector<std::vector<CVec>> invfftcoeff1, invfftcoeff2, invfftcoeff3;

    ModularReducerT<EV, CT> mod_reducer;

    BootstrapperT(EV &ev, long loge, long logn, long logNh, long L, double final_scale, long boundary_K,
                  long sin_cos_deg, long scale_factor, long inverse_deg);
    // take the EvalMod heap and LT diagonals of another bootstrapper with the
    // same parameters (the batched form reuses the single form's setup)
    template <class EV2, class CT2>
    void adopt_setup(const BootstrapperT<EV2, CT2> &o)
    {
        slot_vec = o.slot_vec;
        slot_index = o.slot_index;
        fftcoeff1 = o.fftcoeff1;
        fftcoeff2 = o.fftcoeff2;
        fftcoeff3 = o.fftcoeff3;
        invfftcoeff1 = o.invfftcoeff1;
        invfftcoeff2 = o.invfftcoeff2;
        invfftcoeff3 = o.invfftcoeff3;
        final_scale = o.final_scale;
        mod_reducer.adopt_polynomials(o.mod_reducer);
        cache_.clear();
    }

    void set_final_scale(double s) { final_scale = s; }
    void prepare_mod_polynomial(long heap_k, long heap_m, std::vector<std::vector<double>> nodes,
                                double scale_inverse_coeff);
    void addLeftRotKeys_Linear_to_vector_3(std::vector<int> &gal_steps_vector) const;
    void generate_LT_coefficient_3();
    void change_logn(long new_logn);

    void bsgs_linear_transform(CT &rtncipher, const CT &cipher, int totlen, int basicstep,
                               int coeff_logn, const std::vector<CVec> &fftcoeff, int tag);
    void rotated_bsgs_linear_transform(CT &rtncipher, const CT &cipher, int totlen, int basicstep,
                                       int coeff_logn, const std::vector<CVec> &fftcoeff, int tag);

    void sfl_3(CT &rtncipher, const CT &cipher);
    void sfl_full_3(CT &rtncipher, const CT &cipher);
    void sflinv_3(CT &rtncipher, const CT &cipher);
    void sflinv_full_3(CT &rtncipher, const CT &cipher);
    void coefftoslot_3(CT &rtncipher, const CT &cipher);
    void slottocoeff_3(CT &rtncipher, const CT &cipher);
    void coefftoslot_full_3(CT &rtncipher1, CT &rtncipher2, const CT &cipher);
    void slottocoeff_full_3(CT &rtncipher, const CT &cipher1, const CT &cipher2);
    void modraise_inplace(CT &cipher);

    void bootstrap_sparse_3(CT &rtncipher, CT &cipher);
    void bootstrap_full_3(CT &rtncipher, CT &cipher);
    void bootstrap_3(CT &rtncipher, CT &cipher);
    void bootstrap_inplace_3(CT &cipher);

    // device copies of encoded diagonals kept between bootstraps
    size_t cached_plaintexts() const { return cache_.size(); }
    void clear_cache() { cache_.clear(); }

private:
    // the plaintext multiply_vector_reduced_error(ct, rotation(coeff_logn, Nh,
    // shift, v)) encodes, taken from (or put into) the cache
    const Plaintext &diagonal(const CT &ct, int tag, int index, int shift, int coeff_logn, const CVec &v,
                              uint64_t salt);
    const Plaintext &unit_plain(bool plus_i, int limbs);
    EV *ev_;
    using Key = std::tuple<int, int, int, int, uint64_t, uint64_t>;
    std::map<Key, Plaintext> cache_;
    uint64_t salt_ = 0;  // distinguishes diagonals that depend on the scales of the call
};

using ModularReducer = ModularReducerT<Evaluator, Ciphertext>;
using Bootstrapper = BootstrapperT<Evaluator, Ciphertext>;
using BatchBootstrapper = BootstrapperT<BatchEvaluator, CtBatch>;

}  // namespace nexus
