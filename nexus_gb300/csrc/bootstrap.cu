// NEXUS's bootstrapping (src/bootstrapping/Bootstrapper.cpp,
// ModularReducer.cpp, common/Polynomial.cpp, common/func.cpp) on the engine.
//
// The LT diagonals are computed on the host with std::complex<double> in the
// reference's operation order (the translation unit is compiled with FP
// contraction off), so each diagonal is the same double vector the reference
// encodes.  Ciphertext work runs through the Evaluator's kernels; the one
// kernel of its own here is the modulus raise.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>

#include "bootstrap.h"
#include "modarith.cuh"
#include "ntt.h"

namespace nexus {

namespace {
inline int batch_of(const Ciphertext &) { return 1; }
inline int batch_of(const CtBatch &c) { return c.batch(); }
}  // namespace

int giantstep(int m)
{
    int minval = m, mink = 1;
    for (int k = 1; k <= 3 * std::sqrt((double)m); k++) {
        int cur = (int)std::ceil((m + 0.0) / (k + 0.0)) + k - 1;
        if (cur < minval) {
            minval = cur;
            mink = k;
        }
    }
    return mink;
}

void rotation(int logslot, int nh, int shiftcount, const CVec &vec, CVec &rtnvec)
{
    const int slotlen = 1 << logslot;
    const int repeat = nh / slotlen;
    rtnvec.clear();
    rtnvec.reserve(nh);
    for (int j = 0; j < repeat; j++)
        for (int i = 0; i < slotlen; i++) {
            const int idx = slotlen + i + shiftcount;
            if (idx < 0) throw std::logic_error("rotation: negative index");
            rtnvec.push_back(vec[idx % slotlen]);
        }
}

// ------------------------------------------------------------------ EvalMod

template <class EV, class CT>
ModularReducerT<EV, CT>::ModularReducerT(EV &ev, long K, double lw, long d, long ndf, long ideg)
    : boundary_K(K), log_width(lw), deg(d), num_double_formula(ndf), inverse_deg(ideg), ev_(&ev)
{
}

template <class EV, class CT>
void ModularReducerT<EV, CT>::set_polynomial_heap(long k, long m, std::vector<std::vector<double>> nodes, double sic)
{
    if (k < 2 || m < 1 || nodes.size() != (size_t)((1 << (m + 1)) - 1) || nodes[0].empty())
        throw std::invalid_argument("malformed polynomial heap");
    // the evaluation reads coefficients 0 and 1 of every leaf and at most
    // k + 1 of them (T_k is the first giant step)
    for (size_t i = (size_t)(1 << m) - 1; i < nodes.size(); i++)
        if (!nodes[i].empty() && (nodes[i].size() < 2 || nodes[i].size() > (size_t)k + 1))
            throw std::invalid_argument("malformed polynomial heap");
    heap_k = k;
    heap_m = m;
    heap = std::move(nodes);
    scale_inverse_coeff = sic;
}

template <class EV, class CT>
void ModularReducerT<EV, CT>::set_inverse_polynomial(InversePoly p)
{
    const long d = (long)p.power.size() - 1;
    if (d < 1) throw std::invalid_argument("inverse-sine polynomial: no coefficients");
    if (d > 3) {
        const long k = p.heap_k, m = p.heap_m;
        if (k < 2 || m < 1 || p.heap.size() != (size_t)((1 << (m + 1)) - 1) || p.heap[0].empty())
            throw std::invalid_argument("inverse-sine polynomial: malformed heap");
        for (size_t i = (size_t)(1 << m) - 1; i < p.heap.size(); i++)
            if (!p.heap[i].empty() && (p.heap[i].size() < 2 || p.heap[i].size() > (size_t)k + 1))
                throw std::invalid_argument("inverse-sine polynomial: malformed heap");
    }
    inverse = std::move(p);
}

template <class EV, class CT>
void ModularReducerT<EV, CT>::double_angle_formula(CT &cipher)
{
    ev_->square_inplace(cipher);
    ev_->relinearize_inplace(cipher);
    ev_->rescale_to_next_inplace(cipher);
    ev_->double_inplace(cipher);
    ev_->add_const_inplace(cipher, -1.0);
}

template <class EV, class CT>
void ModularReducerT<EV, CT>::double_angle_formula_scaled(CT &cipher, double scale_coeff)
{
    ev_->square_inplace(cipher);
    ev_->relinearize_inplace(cipher);
    ev_->rescale_to_next_inplace(cipher);
    ev_->double_inplace(cipher);
    ev_->add_const_inplace(cipher, -scale_coeff);
}

// Polynomial::homomorphic_poly_evaluation (common/Polynomial.cpp:255-485)
// over the heap: Chebyshev baby steps T_1..T_{k-1}, giant steps
// T_k, T_2k, ..., leaves as sums of constant multiples, then the heap
// combined bottom-up with the giant steps.
template <class EV, class CT>
void ModularReducerT<EV, CT>::homomorphic_poly_evaluation(CT &rtn, const CT &cipher)
{
    evaluate_heap(rtn, cipher, heap_k, heap_m, heap);
}

// The direct forms of Polynomial::homomorphic_poly_evaluation for degree
// 1, 2 and 3 (common/Polynomial.cpp:257-325), on the power-basis
// coefficients; a term whose coefficient is below 1 / scale is left out
// where the reference leaves it out.
template <class EV, class CT>
void ModularReducerT<EV, CT>::evaluate_power(CT &rtn, const CT &cipher, const std::vector<double> &coeff)
{
    EV &ev = *ev_;
    const double zero = 1. / cipher.scale();
    const size_t d = coeff.size() - 1;
    if (d == 1) {
        ev.multiply_const_rescale(cipher, coeff[1], rtn);
        ev.add_const_inplace(rtn, coeff[0]);
        return;
    }
    if (d == 2) {
        CT squared;
        ev.square(cipher, squared);
        ev.relinearize_inplace(squared);
        ev.rescale_to_next_inplace(squared);
        ev.multiply_const_rescale(squared, coeff[2], squared);
        if (std::fabs(coeff[1]) >= zero) {
            ev.multiply_const_rescale(cipher, coeff[1], rtn);
            ev.add_inplace_reduced_error(rtn, squared);
        } else {
            rtn = std::move(squared);
        }
        ev.add_const_inplace(rtn, coeff[0]);
        return;
    }
    if (d != 3) throw std::invalid_argument("evaluate_power: degree 1, 2 or 3 expected");
    CT squared, cubic;
    ev.square(cipher, squared);
    ev.relinearize_inplace(squared);
    ev.rescale_to_next_inplace(squared);
    ev.multiply_const_rescale(cipher, coeff[3], cubic);
    ev.multiply_inplace_reduced_error(cubic, squared);
    ev.rescale_to_next_inplace(cubic);
    if (std::fabs(coeff[1]) >= zero) {
        ev.multiply_const_rescale(cipher, coeff[1], rtn);
        ev.add_inplace_reduced_error(rtn, cubic);
    } else {
        rtn = std::move(cubic);
    }
    if (std::fabs(coeff[2]) >= zero) {
        ev.multiply_const_rescale(squared, coeff[2], squared);
        ev.add_inplace_reduced_error(rtn, squared);
    }
    ev.add_const_inplace(rtn, coeff[0]);
}

template <class EV, class CT>
void ModularReducerT<EV, CT>::evaluate_heap(CT &rtn, const CT &cipher, long k, long m,
                                            const std::vector<std::vector<double>> &heap)
{
    EV &ev = *ev_;
    const double zero = 1. / cipher.scale();
    if (heap.empty() || (long)heap[0].size() - 1 < 4 || m < 1)
        throw std::invalid_argument("homomorphic_poly_evaluation: polynomial heap of degree >= 4 expected");
    std::vector<CT> baby(k);
    std::vector<bool> have(k, false);
    baby[1] = cipher;
    have[1] = true;
    for (long i = 2; i < k; i *= 2) {
        ev.square(baby[i / 2], baby[i]);
        ev.relinearize_inplace(baby[i]);
        ev.rescale_to_next_inplace(baby[i]);
        ev.double_inplace(baby[i]);
        ev.add_const_inplace(baby[i], -1.0);
        have[i] = true;
    }
    for (long i = 1; i < k; i++) {
        if (have[i]) continue;
        const long lpow2 = 1L << (int)std::floor(std::log((double)i) / std::log(2.0));
        const long res = i - lpow2;
        const long diff = std::labs(lpow2 - res);
        ev.multiply_reduced_error(baby[lpow2], baby[res], baby[i]);
        ev.rescale_to_next_inplace(baby[i]);
        ev.double_inplace(baby[i]);
        ev.sub_inplace_reduced_error(baby[i], baby[diff]);
        have[i] = true;
    }
    std::vector<CT> giant(m);
    {
        const long lpow2 = 1L << ((int)std::ceil(std::log((double)k) / std::log(2.0)) - 1);
        const long res = k - lpow2;
        const long diff = std::labs(lpow2 - res);
        if (res == 0) {
            giant[0] = baby[lpow2];
        } else if (diff == 0) {
            ev.square(baby[lpow2], giant[0]);
            ev.relinearize_inplace(giant[0]);
            ev.rescale_to_next_inplace(giant[0]);
            ev.double_inplace(giant[0]);
            ev.add_const_inplace(giant[0], -1.0);
        } else {
            ev.multiply_reduced_error(baby[lpow2], baby[res], giant[0]);
            ev.rescale_to_next_inplace(giant[0]);
            ev.double_inplace(giant[0]);
            ev.sub_inplace_reduced_error(giant[0], baby[diff]);
        }
    }
    for (long i = 1; i < m; i++) {
        ev.square(giant[i - 1], giant[i]);
        ev.relinearize_inplace(giant[i]);
        ev.rescale_to_next_inplace(giant[i]);
        ev.double_inplace(giant[i]);
        ev.add_const_inplace(giant[i], -1.0);
    }

    const long len = (1L << (m + 1)) - 1;
    std::vector<CT> ch(len);
    std::vector<bool> chb(len, false);
    for (long i = (1L << m) - 1; i < len; i++) {
        const std::vector<double> &cf = heap[i];
        if (cf.empty()) continue;
        chb[i] = true;
        ev.multiply_const_rescale(baby[1], cf[1], ch[i]);
        if (!(std::fabs(cf[1]) <= zero)) ev.add_const_inplace(ch[i], cf[0]);
        for (size_t j = 2; j < cf.size(); j++) {
            if (std::fabs(cf[j]) <= zero) continue;
            ev.multiply_const_rescale_add((long)j < k ? baby[j] : giant[0], cf[j], ch[i]);
        }
    }
    long depth = m, gindex = 0;
    while (depth != 0) {
        depth--;
        for (long i = (1L << depth) - 1; i < (1L << (depth + 1)) - 1; i++) {
            if (heap[i].empty()) continue;
            chb[i] = true;
            const long l = 2 * (i + 1) - 1, r = 2 * (i + 1);
            if (!chb[l]) {
                ch[i] = ch[r];
            } else {
                ev.multiply_reduced_error(ch[l], giant[gindex], ch[i]);
                ev.rescale_to_next_inplace(ch[i]);
                ev.add_inplace_reduced_error(ch[i], ch[r]);
            }
        }
        gindex++;
    }
    rtn = std::move(ch[0]);
}

template <class EV, class CT>
void ModularReducerT<EV, CT>::modular_reduction(CT &rtn, const CT &cipher)
{
    if (heap.empty()) throw std::logic_error("prepare_mod_polynomial has not been called");
    CT tmp2;
    homomorphic_poly_evaluation(tmp2, cipher);
    if (inverse_deg == 1) {
        double curr_scale = scale_inverse_coeff;
        for (long i = 0; i < num_double_formula; i++) {
            curr_scale = curr_scale * curr_scale;
            double_angle_formula_scaled(tmp2, curr_scale);
        }
        rtn = std::move(tmp2);
        return;
    }
    if ((long)inverse.power.size() != inverse_deg + 1)
        throw std::logic_error("the inverse-sine polynomial has not been set for this inverse_deg");
    for (long i = 0; i < num_double_formula; i++) double_angle_formula(tmp2);
    if (inverse_deg <= 3)
        evaluate_power(rtn, tmp2, inverse.power);
    else
        evaluate_heap(rtn, tmp2, inverse.heap_k, inverse.heap_m, inverse.heap);
}

// ------------------------------------------------------------ Bootstrapper

template <class EV, class CT>
BootstrapperT<EV, CT>::BootstrapperT(EV &ev, long loge_, long logn_, long logNh_, long L_, double fs, long K, long scd,
                           long sf, long ideg)
    : loge(loge_), logn(logn_), logNh(logNh_), L(L_), final_scale(fs), boundary_K(K), sin_cos_deg(scd),
      scale_factor(sf), inverse_deg(ideg), mod_reducer(ev, K, (double)loge_, scd, sf, ideg), ev_(&ev)
{
    if (logn_ < 0 || logn_ > logNh_ || (1L << logNh_) != (long)ev.slot_count())
        throw std::invalid_argument("logn / logNh do not match the context");
    n = 1L << logn;
    Nh = 1L << logNh;
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::prepare_mod_polynomial(long heap_k, long heap_m, std::vector<std::vector<double>> nodes,
                                          double scale_inverse_coeff)
{
    mod_reducer.set_polynomial_heap(heap_k, heap_m, std::move(nodes), scale_inverse_coeff);
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::change_logn(long new_logn)
{
    logn = new_logn;
    n = 1L << logn;
    slot_index = -1;
    for (size_t i = 0; i < slot_vec.size(); i++)
        if (slot_vec[i] == logn) {
            slot_index = (long)i;
            break;
        }
    if (slot_index == -1) throw std::invalid_argument("LT coefficients were not generated for this logn");
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::addLeftRotKeys_Linear_to_vector_3(std::vector<int> &v) const
{
    auto push = [&](int s) {
        for (int x : v)
            if (x == s) return;
        v.push_back(s);
    };
    const int d1 = (int)std::floor(logn / 3.0);
    const int d2 = (int)std::floor((logn - d1) / 2.0);
    const int d3 = (int)logn - d1 - d2;
    const int t1 = (1 << d1) - 1, t2 = (1 << d2) - 1, t3 = (1 << d3) - 1;
    const int bs1 = 1 << (logn - d1), bs2 = 1 << (logn - d1 - d2), bs3 = 1;
    const int nh = (int)Nh;
    const int gs1 = giantstep(t1 + 1);
    const int gs1_e = logn != logNh ? giantstep(2 * t1 + 1) : 0;
    const int gs2 = giantstep(2 * t2 + 1), gs3 = giantstep(2 * t3 + 1);
    const int start1 = -t1 + gs1 * (t1 / gs1), gfirst1 = -(t1 / gs1), glast1 = (2 * t1) / gs1 + gfirst1;
    const int glast1_e = logn != logNh ? t1 / gs1 : 0;
    const int start2 = -t2 + gs2 * (t2 / gs2), gfirst2 = -(t2 / gs2), glast2 = (2 * t2) / gs2 + gfirst2;
    const int start3 = -t3 + gs3 * (t3 / gs3), gfirst3 = -(t3 / gs3), glast3 = (2 * t3) / gs3 + gfirst3;
    for (int i = start1; i < start1 + gs1; i++)
        if (i) push((nh + i * bs1) % nh);
    for (int i = 1; i < gs1_e; i++) push(i * bs1);
    for (int i = start2; i < start2 + gs2; i++)
        if (i) push((nh + i * bs2) % nh);
    for (int i = start3; i < start3 + gs3; i++)
        if (i) push((nh + i * bs3) % nh);
    for (int i = gfirst1; i <= glast1; i++)
        if (i) push((nh + i * gs1 * bs1) % nh);
    for (int i = 1; i <= glast1_e; i++) push(i * gs1_e * bs1);
    for (int i = gfirst2; i <= glast2; i++)
        if (i) push((nh + i * gs2 * bs2) % nh);
    for (int i = gfirst3; i <= glast3; i++)
        if (i) push((nh + i * gs3 * bs3) % nh);
}

namespace {

using Orig = std::vector<std::vector<CVec>>;  // [level][3][n]

// genorigcoeff (Bootstrapper.cpp:522-602) for one slot count
void gen_orig(long lg, Orig &orig, Orig &inv)
{
    const long nn = 1L << lg;
    orig.assign(lg, std::vector<CVec>(3, CVec(nn)));
    inv.assign(lg, std::vector<CVec>(3, CVec(nn)));
    double theta0 = M_PI / (2 * nn);
    long blocklen = 1, blockcount = nn;
    for (long i = 0; i < lg; i++) {
        blocklen <<= 1;
        blockcount >>= 1;
        const double theta = theta0 * (1 << (lg - 1 - i));
        long power = 1;
        std::complex<double> zeta = std::polar(1.0, theta * power);
        for (long j = 0; j < blocklen / 2; j++) {
            for (long k = 0; k < blockcount; k++) {
                orig[i][1][k * blocklen + j] = 1;
                orig[i][1][k * blocklen + j + blocklen / 2] = -zeta;
                orig[i][0][k * blocklen + j] = 0;
                orig[i][0][k * blocklen + j + blocklen / 2] = 1;
                orig[i][2][k * blocklen + j] = zeta;
                orig[i][2][k * blocklen + j + blocklen / 2] = 0;
            }
            power = (5 * power) % (1L << (i + 3));
            zeta = std::polar(1.0, theta * power);
        }
    }
    theta0 = -M_PI / (2 * nn);
    blocklen = nn;
    blockcount = 1;
    for (long i = 0; i < lg; i++) {
        const double theta = theta0 * (1 << i);
        long power = 1;
        std::complex<double> zeta = std::polar(1.0, theta * power);
        for (long j = 0; j < blocklen / 2; j++) {
            for (long k = 0; k < blockcount; k++) {
                inv[i][1][k * blocklen + j] = 0.5;
                inv[i][1][k * blocklen + j + blocklen / 2] = -0.5 * zeta;
                inv[i][0][k * blocklen + j] = 0;
                inv[i][0][k * blocklen + j + blocklen / 2] = 0.5 * zeta;
                inv[i][2][k * blocklen + j] = 0.5;
                inv[i][2][k * blocklen + j + blocklen / 2] = 0;
            }
            power = (5 * power) % (1L << ((lg - 1 - i) + 3));
            zeta = std::polar(1.0, theta * power);
        }
        blocklen >>= 1;
        blockcount <<= 1;
    }
}

// One level of genfftcoeff_3 / geninvfftcoeff_3: for each of the 3^d paths
// through d radix-2 butterfly levels, the product of the d rotated
// butterfly diagonals, added into the diagonal of the path's net shift.
// `msb_first` selects the inverse transform's shift weights 2^(d-1-p).
void merge_level(const Orig &orig, int offset, int d, long basicstep, long nn, bool msb_first, std::vector<CVec> &out,
                 int nslots, int (*slot_of)(int pos, int totlen), int totlen)
{
    out.assign(nslots, CVec(nn, 0));
    CVec tmp(nn);
    std::vector<int> cnt(d);
    long all = 1;
    for (int p = 0; p < d; p++) all *= 3;
    for (long j = 0; j < all; j++) {
        long ind = j;
        int pos = 0;
        for (int p = 0; p < d; p++) {
            const int r = (int)(ind % 3);
            pos += (r - 1) * (1 << (msb_first ? d - 1 - p : p));
            cnt[p] = r;
            ind = (ind - r) / 3;
        }
        int cur = pos;
        for (long k = 0; k < nn; k++) tmp[k] = 1.0;
        for (int p = 0; p < d; p++) {
            cur = cur - (cnt[p] - 1) * (1 << (msb_first ? d - 1 - p : p));
            const CVec &o = orig[p + offset][cnt[p]];
            for (long k = 0; k < nn; k++) tmp[k] = tmp[k] * o[(k + basicstep * (nn + cur)) % nn];
        }
        CVec &dst = out[slot_of(pos, totlen)];
        for (long k = 0; k < nn; k++) dst[k] += tmp[k];
    }
}

int slot_centered(int pos, int t) { return pos + t; }
int slot_wrapped(int pos, int t) { return (pos + t + 1) % (t + 1); }

}  // namespace

void lt_coefficients_3(long cl, long logNh, long boundary_K, std::vector<CVec> out[6])
{
    const long cn = 1L << cl;
    Orig orig, inv;
    gen_orig(cl, orig, inv);
    std::vector<CVec> &f1 = out[0], &f2 = out[1], &f3 = out[2], &i1 = out[3], &i2 = out[4], &i3 = out[5];
    {  // genfftcoeff_3 (Bootstrapper.cpp:1144-1550)
        const int d3 = (int)std::floor(cl / 3.0);
        const int d2 = (int)std::floor((cl - d3) / 2.0);
        const int d1 = (int)cl - d3 - d2;
        const int t1 = (1 << d1) - 1, t2 = (1 << d2) - 1, t3 = (1 << d3) - 1;
        merge_level(orig, 0, d1, 1, cn, false, f1, 2 * t1 + 1, slot_centered, t1);
        merge_level(orig, d1, d2, 1L << d1, cn, false, f2, 2 * t2 + 1, slot_centered, t2);
        if (cl == logNh) {
            merge_level(orig, d1 + d2, d3, 1L << (d1 + d2), cn, false, f3, t3 + 1, slot_wrapped, t3);
        } else {
            merge_level(orig, d1 + d2, d3, 1L << (d1 + d2), cn, false, f3, 2 * t3 + 1, slot_centered, t3);
            // second half: a copy (levels 1, 2) or i times the first half (level 3)
            for (auto *lvl : {&f1, &f2})
                for (CVec &v : *lvl) {
                    v.resize(2 * cn);
                    for (long j = 0; j < cn; j++) v[j + cn] = v[j];
                }
            for (CVec &v : f3) {
                v.resize(2 * cn);
                for (long j = 0; j < cn; j++) v[j + cn] = std::complex<double>(0, 1) * v[j];
            }
        }
    }
    {  // geninvfftcoeff_3 (Bootstrapper.cpp:1552-1954)
        const int d1 = (int)std::floor(cl / 3.0);
        const int d2 = (int)std::floor((cl - d1) / 2.0);
        const int d3 = (int)cl - d1 - d2;
        const int t1 = (1 << d1) - 1, t2 = (1 << d2) - 1, t3 = (1 << d3) - 1;
        merge_level(inv, 0, d1, 1L << (cl - d1), cn, true, i1, t1 + 1, slot_wrapped, t1);
        merge_level(inv, d1, d2, 1L << (cl - d1 - d2), cn, true, i2, 2 * t2 + 1, slot_centered, t2);
        merge_level(inv, d1 + d2, d3, 1, cn, true, i3, 2 * t3 + 1, slot_centered, t3);
        if (cl == logNh) {
            for (CVec &v : i1)
                for (auto &x : v) x *= 1.0 / boundary_K;
            for (CVec &v : i3)
                for (auto &x : v) x *= 0.5;
        } else {
            for (CVec &v : i1)
                for (auto &x : v) x *= 1.0 / (boundary_K * (1 << (logNh - cl)));
            for (CVec &v : i3) {
                v.resize(2 * cn);
                for (long j = 0; j < cn; j++) {
                    v[j] *= 0.5;
                    v[j + cn] = std::complex<double>(0, -1) * v[j];
                }
            }
        }
    }
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::generate_LT_coefficient_3()
{
    if (slot_vec.empty()) slot_vec.push_back(logn);
    const size_t U = slot_vec.size();
    fftcoeff1.assign(U, {});
    fftcoeff2.assign(U, {});
    fftcoeff3.assign(U, {});
    invfftcoeff1.assign(U, {});
    invfftcoeff2.assign(U, {});
    invfftcoeff3.assign(U, {});
    for (size_t u = 0; u < U; u++) {
        std::vector<CVec> out[6];
        lt_coefficients_3(slot_vec[u], logNh, boundary_K, out);
        fftcoeff1[u] = std::move(out[0]);
        fftcoeff2[u] = std::move(out[1]);
        fftcoeff3[u] = std::move(out[2]);
        invfftcoeff1[u] = std::move(out[3]);
        invfftcoeff2[u] = std::move(out[4]);
        invfftcoeff3[u] = std::move(out[5]);
    }
    slot_index = -1;
    for (size_t i = 0; i < slot_vec.size(); i++)
        if (slot_vec[i] == logn) slot_index = (long)i;
    if (slot_index < 0) throw std::invalid_argument("slot_vec does not contain logn");
    cache_.clear();
}

template <class EV, class CT>
const Plaintext &BootstrapperT<EV, CT>::diagonal(const CT &ct, int tag, int index, int shift, int coeff_logn,
                                        const CVec &v, uint64_t salt)
{
    const double scale = ct.scale();
    uint64_t sbits;
    std::memcpy(&sbits, &scale, 8);
    const Key key{tag | (int)(slot_index << 8), index, shift, ct.limbs(), sbits, salt};
    auto it = cache_.find(key);
    if (it == cache_.end()) {
        CVec rot;
        rotation(coeff_logn, (int)Nh, shift, v, rot);
        Plaintext p;
        ev_->encode_then_drop(rot, ct.limbs(), ct.scale(), p);
        it = cache_.emplace(key, std::move(p)).first;
    }
    return it->second;
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::bsgs_linear_transform(CT &rtncipher, const CT &cipher, int totlen, int basicstep,
                                         int coeff_logn, const std::vector<CVec> &fftcoeff, int tag)
{
    EV &ev = *ev_;
    const int nh = (int)Nh;
    const int gs1 = giantstep(2 * totlen + 1);
    const int start = -totlen + gs1 * (int)std::floor((totlen + 0.0) / (gs1 + 0.0));
    const int gfirst = -(int)std::floor((totlen + 0.0) / (gs1 + 0.0));
    const int glast = (int)std::floor((2 * totlen + 0.0) / (gs1 + 0.0)) + gfirst;
    // the baby steps rotate one ciphertext: they share its decomposition
    std::vector<CT> baby(gs1);
    {
        std::vector<int> steps;
        std::vector<int> slot;
        for (int i = start; i < start + gs1; i++) {
            if (i == 0) {
                baby[i - start] = cipher;
            } else {
                steps.push_back((nh + i * basicstep) % nh);
                slot.push_back(i - start);
            }
        }
        std::vector<CT> rotated;
        ev.rotate_vector_many(cipher, steps, rotated);
        for (size_t r = 0; r < slot.size(); r++) baby[slot[r]] = std::move(rotated[r]);
    }
    CT giant, acc, t;
    bool have_acc = false;
    std::vector<const CT *> terms;
    std::vector<const Plaintext *> diags;
    for (int i = gfirst; i <= glast; i++) {
        // giant = sum_j baby_j * diag_ij: the products and their
        // add_inplace_reduced_error chain at one level, fused
        terms.clear();
        diags.clear();
        const int jend = i != glast ? start + gs1 - 1 : totlen - i * gs1;
        for (int j = start; j <= jend; j++) {
            const int idx = i * gs1 + j + totlen;
            terms.push_back(&baby[j - start]);
            diags.push_back(&diagonal(baby[j - start], tag, idx, -i * gs1 * basicstep, coeff_logn, fftcoeff[idx], salt_));
        }
        ev.multiply_plain_accumulate(terms, diags, giant);
        if (i != 0) {
            ev.rotate_vector(giant, (nh + i * gs1 * basicstep) % nh, t);
            if (!have_acc) {
                acc = std::move(t);
                have_acc = true;
            } else {
                ev.add_inplace_reduced_error(acc, t);
            }
        } else {
            if (!have_acc) {
                acc = std::move(giant);
                have_acc = true;
            } else {
                ev.add_inplace_reduced_error(acc, giant);
            }
        }
    }
    rtncipher = std::move(acc);
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::rotated_bsgs_linear_transform(CT &rtncipher, const CT &cipher, int totlen,
                                                 int basicstep, int coeff_logn, const std::vector<CVec> &fftcoeff,
                                                 int tag)
{
    EV &ev = *ev_;
    const int nh = (int)Nh;
    const int gs2 = giantstep(totlen + 1);
    const int glast = (int)std::floor((totlen + 0.0) / (gs2 + 0.0));
    // the baby steps rotate one ciphertext: they share its decomposition
    std::vector<CT> baby(gs2);
    {
        std::vector<int> steps;
        for (int i = 1; i < gs2; i++) steps.push_back((nh + i * basicstep) % nh);
        std::vector<CT> rotated;
        ev.rotate_vector_many(cipher, steps, rotated);
        baby[0] = cipher;
        for (int i = 1; i < gs2; i++) baby[i] = std::move(rotated[i - 1]);
    }
    CT giant, acc, t;
    bool have_acc = false;
    std::vector<const CT *> terms;
    std::vector<const Plaintext *> diags;
    for (int i = 0; i <= glast; i++) {
        terms.clear();
        diags.clear();
        const int jend = i != glast ? gs2 - 1 : totlen - i * gs2;
        for (int j = 0; j <= jend; j++) {
            const int idx = i * gs2 + j;
            terms.push_back(&baby[j]);
            diags.push_back(&diagonal(baby[j], tag, idx, -i * gs2 * basicstep, coeff_logn, fftcoeff[idx], salt_));
        }
        ev.multiply_plain_accumulate(terms, diags, giant);
        if (i != 0) {
            ev.rotate_vector(giant, (nh + i * gs2 * basicstep) % nh, t);
            if (!have_acc) {
                acc = std::move(t);
                have_acc = true;
            } else {
                ev.add_inplace_reduced_error(acc, t);
            }
        } else {
            if (!have_acc) {
                acc = std::move(giant);
                have_acc = true;
            } else {
                ev.add_inplace_reduced_error(acc, giant);
            }
        }
    }
    rtncipher = std::move(acc);
}

namespace {

enum Tag { kInv1 = 1, kInv2, kInv3, kFwd1, kFwd2, kFwd3 };

uint64_t bits_of(double x)
{
    uint64_t b;
    std::memcpy(&b, &x, 8);
    return b;
}

// the fftcoeff3 scaling of sfl_3 / sfl_full_3:
// v * curr_mod * mod_zero * final_scale / (scale * scale * initial_scale)
std::vector<CVec> scale_level3(const std::vector<CVec> &c3, size_t count, size_t len, double curr_mod, double mod_zero,
                               double final_scale, double scale, double initial_scale)
{
    std::vector<CVec> out(c3.size());
    for (size_t i = 0; i < count; i++) {
        out[i].resize(len);
        for (size_t j = 0; j < len; j++)
            out[i][j] = c3[i][j] * curr_mod * mod_zero * final_scale / (scale * scale * initial_scale);
    }
    return out;
}

}  // namespace

template <class EV, class CT>
void BootstrapperT<EV, CT>::sflinv_full_3(CT &rtncipher, const CT &cipher)
{
    const int d1 = (int)std::floor(logn / 3.0);
    const int d2 = (int)std::floor((logn - d1) / 2.0);
    const int d3 = (int)logn - d1 - d2;
    const int t1 = (1 << d1) - 1, t2 = (1 << d2) - 1, t3 = (1 << d3) - 1;
    CT tmpct, tmpct2;
    salt_ = 0;
    rotated_bsgs_linear_transform(tmpct, cipher, t1, 1 << (logn - d1), (int)logn, invfftcoeff1[slot_index], kInv1);
    ev_->rescale_to_next_inplace(tmpct);
    bsgs_linear_transform(tmpct2, tmpct, t2, 1 << (logn - d1 - d2), (int)logn, invfftcoeff2[slot_index], kInv2);
    ev_->rescale_to_next_inplace(tmpct2);
    bsgs_linear_transform(rtncipher, tmpct2, t3, 1, (int)logn, invfftcoeff3[slot_index], kInv3);
    ev_->rescale_to_next_inplace(rtncipher);
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::sflinv_3(CT &rtncipher, const CT &cipher)
{
    const int d1 = (int)std::floor(logn / 3.0);
    const int d2 = (int)std::floor((logn - d1) / 2.0);
    const int d3 = (int)logn - d1 - d2;
    const int t1 = (1 << d1) - 1, t2 = (1 << d2) - 1, t3 = (1 << d3) - 1;
    CT tmpct, tmpct2;
    salt_ = 0;
    rotated_bsgs_linear_transform(tmpct, cipher, t1, 1 << (logn - d1), (int)logn, invfftcoeff1[slot_index], kInv1);
    ev_->rescale_to_next_inplace(tmpct);
    bsgs_linear_transform(tmpct2, tmpct, t2, 1 << (logn - d1 - d2), (int)logn, invfftcoeff2[slot_index], kInv2);
    ev_->rescale_to_next_inplace(tmpct2);
    bsgs_linear_transform(rtncipher, tmpct2, t3, 1, (int)logn + 1, invfftcoeff3[slot_index], kInv3);
    ev_->rescale_to_next_inplace(rtncipher);
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::sfl_full_3(CT &rtncipher, const CT &cipher)
{
    const int d3 = (int)std::floor(logn / 3.0);
    const int d2 = (int)std::floor((logn - d3) / 2.0);
    const int d1 = (int)logn - d3 - d2;
    const int t1 = (1 << d1) - 1, t2 = (1 << d2) - 1, t3 = (1 << d3) - 1;
    // the reference scales totlen2 + 1 level-3 diagonals and reads
    // totlen3 + 1 of them: defined only when the two agree
    if (t2 != t3) throw std::invalid_argument("sfl_full_3 needs logn % 3 != 2");
    CT tmpct, tmpct2;
    salt_ = 0;
    bsgs_linear_transform(tmpct, cipher, t1, 1, (int)logn, fftcoeff1[slot_index], kFwd1);
    ev_->rescale_to_next_inplace(tmpct);
    bsgs_linear_transform(tmpct2, tmpct, t2, 1 << d1, (int)logn, fftcoeff2[slot_index], kFwd2);
    ev_->rescale_to_next_inplace(tmpct2);
    const double mod_zero = (double)ev_->modulus(0);
    const double curr_mod = (double)ev_->modulus(tmpct2.limbs() - 1);
    const std::vector<CVec> sc = scale_level3(fftcoeff3[slot_index], (size_t)t2 + 1, (size_t)n, curr_mod, mod_zero,
                                              final_scale, tmpct2.scale(), initial_scale);
    salt_ = bits_of(initial_scale) * 0x9E3779B97F4A7C15ull ^ bits_of(final_scale);
    rotated_bsgs_linear_transform(rtncipher, tmpct2, t3, 1 << (d1 + d2), (int)logn, sc, kFwd3);
    salt_ = 0;
    ev_->rescale_to_next_inplace(rtncipher);
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::sfl_3(CT &rtncipher, const CT &cipher)
{
    const int d3 = (int)std::floor(logn / 3.0);
    const int d2 = (int)std::floor((logn - d3) / 2.0);
    const int d1 = (int)logn - d3 - d2;
    const int t1 = (1 << d1) - 1, t2 = (1 << d2) - 1, t3 = (1 << d3) - 1;
    CT tmpct, tmpct2;
    salt_ = 0;
    bsgs_linear_transform(tmpct, cipher, t1, 1, (int)logn + 1, fftcoeff1[slot_index], kFwd1);
    ev_->rescale_to_next_inplace(tmpct);
    bsgs_linear_transform(tmpct2, tmpct, t2, 1 << d1, (int)logn + 1, fftcoeff2[slot_index], kFwd2);
    ev_->rescale_to_next_inplace(tmpct2);
    const double mod_zero = (double)ev_->modulus(0);
    const double curr_mod = (double)ev_->modulus(tmpct2.limbs() - 1);
    const std::vector<CVec> sc = scale_level3(fftcoeff3[slot_index], (size_t)(2 * t3 + 1), (size_t)(2 * n), curr_mod,
                                              mod_zero, final_scale, tmpct2.scale(), initial_scale);
    salt_ = bits_of(initial_scale) * 0x9E3779B97F4A7C15ull ^ bits_of(final_scale);
    bsgs_linear_transform(rtncipher, tmpct2, t3, 1 << (d1 + d2), (int)logn + 1, sc, kFwd3);
    salt_ = 0;
    ev_->rescale_to_next_inplace(rtncipher);
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::coefftoslot_3(CT &rtncipher, const CT &cipher)
{
    CT t1, t2;
    sflinv_3(t1, cipher);
    t2 = t1;
    ev_->complex_conjugate_inplace(t2);
    ev_->add_reduced_error(t1, t2, rtncipher);
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::slottocoeff_3(CT &rtncipher, const CT &cipher)
{
    CT t1, t2;
    sfl_3(t1, cipher);
    ev_->rotate_vector(t1, (int)n, t2);
    ev_->add_reduced_error(t1, t2, rtncipher);
}

// encode(vector of +-i, 1.0) at the top level, then mod_switch_to(limbs): the
// constant plaintexts of coefftoslot_full_3 / slottocoeff_full_3, kept on the device
template <class EV, class CT>
const Plaintext &BootstrapperT<EV, CT>::unit_plain(bool plus_i, int limbs)
{
    const Key key{plus_i ? -1 : -2, 0, 0, limbs, 0, 0};
    auto it = cache_.find(key);
    if (it == cache_.end()) {
        CVec v(Nh, 0);
        const std::complex<double> iunit(0.0, 1.0);
        for (long i = 0; i < Nh; i++) {
            if (plus_i)
                v[i] += iunit;
            else
                v[i] -= iunit;
        }
        Plaintext p;
        ev_->encode(v, ev_->top_limbs(), 1.0, p);
        ev_->mod_switch_to_inplace(p, limbs);
        it = cache_.emplace(key, std::move(p)).first;
    }
    return it->second;
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::coefftoslot_full_3(CT &rtncipher1, CT &rtncipher2, const CT &cipher)
{
    CT t1, t2, t3, t4;
    sflinv_full_3(t1, cipher);
    ev_->multiply_plain(t1, unit_plain(false, t1.limbs()), t2);
    t3 = t2;
    ev_->complex_conjugate_inplace(t3);
    t4 = t1;
    ev_->complex_conjugate_inplace(t4);
    ev_->add_reduced_error(t1, t4, rtncipher1);
    ev_->add_reduced_error(t2, t3, rtncipher2);
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::slottocoeff_full_3(CT &rtncipher, const CT &cipher1, const CT &cipher2)
{
    CT t1, t3;
    ev_->multiply_plain(cipher2, unit_plain(true, cipher2.limbs()), t1);
    ev_->add_reduced_error(cipher1, t1, t3);
    sfl_full_3(rtncipher, t3);
}

// ------------------------------------------------------------ modulus raise

namespace {

// out[p][j][i] = centred lift of the q0 residue src[p][i] into prime j
__global__ void k_modraise(const uint64_t *__restrict__ src, uint64_t *__restrict__ out,
                           const PrimeConst *__restrict__ pc, int limbs, int logn, size_t total)
{
    const uint64_t q0 = pc[0].q;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t i = t & ((1ull << logn) - 1);
        const size_t row = t >> logn;
        const int j = (int)(row % (size_t)limbs);
        const size_t p = row / (size_t)limbs;
        const uint64_t v = src[(p << logn) + i];
        const uint64_t q = pc[j].q;
        uint64_t r = barrett_64(v, q, pc[j].r1);
        if (v > (q0 >> 1)) {
            const uint64_t minus_q0 = j == 0 ? 0 : q - barrett_64(q0, q, pc[j].r1);
            r += minus_q0;
            r = r >= q ? r - q : r;
        }
        out[t] = r;
    }
}

}  // namespace

template <class EV, class CT>
void BootstrapperT<EV, CT>::modraise_inplace(CT &cipher)
{
    if (cipher.size() != 2) throw std::invalid_argument("Ciphertexts of size 2 are supported only!");
    if (cipher.limbs() != 1) throw std::invalid_argument("Ciphertexts in the lowest level are supported only!");
    Context &c = ev_->context();
    cudaStream_t s = ev_->stream();
    const int top = ev_->top_limbs();
    const int polys = 2 * batch_of(cipher);
    CT src = cipher;  // [polys][1][N], inverse-transformed below
    ntt_inverse(c, src.data(), polys, 0, 1, s);
    const double scale = cipher.scale();
    cipher.resize(c, 2, top, s);
    cipher.scale() = scale;
    const size_t total = (size_t)polys * top * c.n;
    const unsigned grid = (unsigned)std::min<size_t>((total + 255) / 256, 152 * 16);
    k_modraise<<<grid, 256, 0, s>>>(src.data(), cipher.data(), c.d_pc, top, c.logn, total);
    NEXUS_LAUNCHED();
    ntt_forward(c, cipher.data(), polys, 0, top, s);
}

// ------------------------------------------------------------------ drivers

// EvalMod of the two halves of a full-slot bootstrap, one after the other
template <class EV, class CT>
static void evalmod_halves(ModularReducerT<EV, CT> &mr, EV &, CT &m1, CT &m2, const CT &r1, const CT &r2)
{
    mr.modular_reduction(m1, r1);
    mr.modular_reduction(m2, r2);
}

// In lockstep the two halves take the same operation sequence (same level
// and scale), so they run as one batch of twice the size: every ciphertext
// gets the words it gets on its own, with half the launches and key reads
// per ciphertext.
static void evalmod_halves(ModularReducerT<BatchEvaluator, CtBatch> &mr, BatchEvaluator &ev, CtBatch &m1,
                           CtBatch &m2, const CtBatch &r1, const CtBatch &r2)
{
    if (r1.batch() != r2.batch() || r1.size() != r2.size() || r1.limbs() != r2.limbs() || r1.scale() != r2.scale()) {
        mr.modular_reduction(m1, r1);
        mr.modular_reduction(m2, r2);
        return;
    }
    Context &c = ev.context();
    cudaStream_t s = ev.stream();
    const size_t half = (size_t)r1.batch() * r1.words_per_ct() * 8;
    CtBatch both, m;
    both.resize(c, 2 * r1.batch(), r1.size(), r1.limbs(), s);
    both.scale() = r1.scale();
    if (cudaMemcpyAsync(both.data(), r1.data(), half, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(both.ct(r1.batch()), r2.data(), half, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        throw std::runtime_error("EvalMod: batch copy failed");
    mr.modular_reduction(m, both);
    const size_t out_half = (size_t)r1.batch() * m.words_per_ct() * 8;
    for (CtBatch *dst : {&m1, &m2}) {
        dst->resize(c, r1.batch(), m.size(), m.limbs(), s);
        dst->scale() = m.scale();
    }
    if (cudaMemcpyAsync(m1.data(), m.data(), out_half, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(m2.data(), m.ct(r1.batch()), out_half, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        throw std::runtime_error("EvalMod: batch copy failed");
}

// The single-ciphertext bootstrap's two halves likewise run as a lockstep
// batch of two: the same words as two modular_reduction calls.
static void evalmod_halves(ModularReducerT<Evaluator, Ciphertext> &mr, Evaluator &ev, Ciphertext &m1,
                           Ciphertext &m2, const Ciphertext &r1, const Ciphertext &r2)
{
    if (r1.size() != r2.size() || r1.limbs() != r2.limbs() || r1.scale() != r2.scale()) {
        mr.modular_reduction(m1, r1);
        mr.modular_reduction(m2, r2);
        return;
    }
    Context &c = ev.context();
    cudaStream_t s = ev.stream();
    BatchEvaluator bev(ev);
    ModularReducerT<BatchEvaluator, CtBatch> bmr(bev, mr.boundary_K, mr.log_width, mr.deg, mr.num_double_formula,
                                                 mr.inverse_deg);
    bmr.adopt_polynomials(mr);
    const size_t words = (size_t)r1.size() * r1.limbs() * c.n;
    CtBatch both, m;
    both.resize(c, 2, r1.size(), r1.limbs(), s);
    both.scale() = r1.scale();
    if (cudaMemcpyAsync(both.ct(0), r1.data(), words * 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(both.ct(1), r2.data(), words * 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        throw std::runtime_error("EvalMod: batch copy failed");
    bmr.modular_reduction(m, both);
    const size_t out_words = m.words_per_ct();
    for (Ciphertext *dst : {&m1, &m2}) {
        dst->resize(c, m.size(), m.limbs(), s);
        dst->scale() = m.scale();
    }
    if (cudaMemcpyAsync(m1.data(), m.ct(0), out_words * 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(m2.data(), m.ct(1), out_words * 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        throw std::runtime_error("EvalMod: batch copy failed");
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::bootstrap_full_3(CT &rtncipher, CT &cipher)
{
    modraise_inplace(cipher);
    cipher.scale() = (double)ev_->modulus(0);
    CT rtn1, rtn2, m1, m2;
    coefftoslot_full_3(rtn1, rtn2, cipher);
    evalmod_halves(mod_reducer, *ev_, m1, m2, rtn1, rtn2);
    slottocoeff_full_3(rtncipher, m1, m2);
    rtncipher.scale() = final_scale;
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::bootstrap_sparse_3(CT &rtncipher, CT &cipher)
{
    EV &ev = *ev_;
    modraise_inplace(cipher);
    cipher.scale() = (double)ev.modulus(0);
    CT rot;
    for (long i = logn; i < logNh; ++i) {
        ev.rotate_vector(cipher, (int)(1L << i), rot);
        ev.add_inplace(cipher, rot);
    }
    CT rtn;
    if (logn == 0) {
        CVec cts(Nh, 0);
        for (long i = 0; i < Nh; i++) {
            if (i % 2 == 0)
                cts[i] = 1.0 / (2.0 * boundary_K * (1 << logNh));
            else
                cts[i] = -std::complex<double>(0, 1.0) / (2.0 * boundary_K * (1 << logNh));
        }
        ev.multiply_vector_reduced_error(cipher, cts, rtn);
        ev.rescale_to_next_inplace(rtn);
        CT conj = rtn;
        ev.complex_conjugate_inplace(conj);
        ev.add_inplace_reduced_error(rtn, conj);
    } else {
        coefftoslot_3(rtn, cipher);
    }
    CT modrtn;
    mod_reducer.modular_reduction(modrtn, rtn);
    if (logn == 0) {
        const double mod_zero = (double)ev.modulus(0);
        const double curr_mod = (double)ev.modulus(modrtn.limbs() - 1);
        const double scale_adj = curr_mod * mod_zero * final_scale / (modrtn.scale() * modrtn.scale() * initial_scale);
        CVec stc(Nh, 0);
        for (long i = 0; i < Nh; i++) {
            if (i % 2 == 0)
                stc[i] = scale_adj;
            else
                stc[i] = std::complex<double>(0, 1.0) * scale_adj;
        }
        ev.multiply_vector_reduced_error(modrtn, stc, rtncipher);
        ev.rescale_to_next_inplace(rtncipher);
        CT r;
        ev.rotate_vector(rtncipher, 1, r);
        ev.add_inplace_reduced_error(rtncipher, r);
    } else {
        slottocoeff_3(rtncipher, modrtn);
    }
    rtncipher.scale() = final_scale;
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::bootstrap_3(CT &rtncipher, CT &cipher)
{
    if (fftcoeff1.empty()) throw std::logic_error("generate_LT_coefficient_3 has not been called");
    initial_scale = cipher.scale();
    if (logn == logNh)
        bootstrap_full_3(rtncipher, cipher);
    else
        bootstrap_sparse_3(rtncipher, cipher);
}

template <class EV, class CT>
void BootstrapperT<EV, CT>::bootstrap_inplace_3(CT &cipher)
{
    CT r;
    bootstrap_3(r, cipher);
    cipher = std::move(r);
}

template class ModularReducerT<Evaluator, Ciphertext>;
template class ModularReducerT<BatchEvaluator, CtBatch>;
template class BootstrapperT<Evaluator, Ciphertext>;
template class BootstrapperT<BatchEvaluator, CtBatch>;

}  // namespace nexus
