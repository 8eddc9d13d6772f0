// NEXUS operators over the engine's Evaluator.  The call sequence of each
// operator is NEXUS's own (cited per function, src/ in the NEXUS tree): it
// fixes every intermediate scale and level, and through them the output words.
#include <cmath>

#include "nexus_ops.h"

namespace nexus {

template <class EV, class CT>
CKKSEvaluatorT<EV, CT>::CKKSEvaluatorT(EV &ev, double scale_) : evaluator(&ev), scale(scale_)
{
    slot_count = ev.slot_count();
    degree = slot_count * 2;
}

// get_modulus (src/ckks_evaluator.cpp:511-515): q[limbs - k] of x's level
template <class EV, class CT>
uint64_t CKKSEvaluatorT<EV, CT>::get_modulus(const CT &x, int k) const
{
    const int idx = x.limbs() - k;
    if (idx < 0) throw std::invalid_argument("level too low for the degree-9 evaluation");
    return evaluator->modulus(idx);
}

// sgn_eval (src/ckks_evaluator.cpp:181-212): g-polynomials then f-polynomials,
// the last of each scaled by sgn_factor
template <class EV, class CT>
CT CKKSEvaluatorT<EV, CT>::sgn_eval(CT x, int d_g, int d_f, double sgn_factor)
{
    std::vector<double> f4 = F4_COEFFS, g4 = G4_COEFFS, f4_last(10), g4_last(10);
    for (int i = 0; i <= 9; ++i) {
        f4[i] /= f4_scale;
        f4_last[i] = f4[i] * sgn_factor;
        g4[i] /= g4_scale;
        g4_last[i] = g4[i] * sgn_factor;
    }
    CT dest = x;
    for (int i = 0; i < d_g; ++i) eval_odd_deg9_poly(i == d_g - 1 ? g4_last : g4, dest, dest);
    for (int i = 0; i < d_f; ++i) eval_odd_deg9_poly(i == d_f - 1 ? f4_last : f4, dest, dest);
    return dest;
}

// eval_odd_deg9_poly (src/ckks_evaluator.cpp:214-364): P = T1 + T2 + T3 with
// T1 = (a3 + a5 x^2) x^3, T2 = (a7 x + a9 x^3) x^6, T3 = a1 x, each
// coefficient encoded at the scale that makes the three terms meet.
template <class EV, class CT>
void CKKSEvaluatorT<EV, CT>::eval_odd_deg9_poly(const std::vector<double> &a, CT &x_in, CT &dest)
{
    EV &ev = *evaluator;
    CT x = x_in;
    const double D = x.scale();
    const uint64_t p = get_modulus(x, 2), q = get_modulus(x, 3), r = get_modulus(x, 4);

    CT x2, x3, x6;
    ev.square(x, x2);
    ev.relinearize_inplace(x2);
    ev.rescale_to_next_inplace(x2);
    ev.mod_switch_to_next_inplace(x);
    ev.multiply(x2, x, x3);
    ev.relinearize_inplace(x3);
    ev.rescale_to_next_inplace(x3);
    ev.square(x3, x6);
    ev.relinearize_inplace(x6);
    ev.rescale_to_next_inplace(x6);

    Plaintext a1, a3, a5, a7, a9;
    CT T1;
    const double a5_scale = D / x2.scale() * (double)p / x3.scale() * (double)q;
    ev.encode(a[5], x2.limbs(), a5_scale, a5);
    ev.multiply_plain(x2, a5, T1);
    ev.rescale_to_next_inplace(T1);
    ev.encode(a[3], T1.limbs(), T1.scale(), a3);
    ev.add_plain_inplace(T1, a3);
    ev.multiply_inplace(T1, x3);
    ev.relinearize_inplace(T1);
    ev.rescale_to_next_inplace(T1);

    CT T2, a7x;
    const double a9_scale = D / x3.scale() * (double)r / x6.scale() * (double)q;
    ev.encode(a[9], x3.limbs(), a9_scale, a9);
    ev.multiply_plain(x3, a9, T2);
    ev.rescale_to_next_inplace(T2);
    const double a7_scale = T2.scale() / x.scale() * (double)p;
    ev.encode(a[7], x.limbs(), a7_scale, a7);
    ev.multiply_plain(x, a7, a7x);
    ev.rescale_to_next_inplace(a7x);
    ev.mod_switch_to_inplace(a7x, T2.limbs());
    const double mid = (T2.scale() + a7x.scale()) / 2;
    T2.scale() = a7x.scale() = mid;
    ev.add_inplace(T2, a7x);
    ev.multiply_inplace(T2, x6);
    ev.relinearize_inplace(T2);
    ev.rescale_to_next_inplace(T2);

    CT T3;
    ev.encode(a[1], x.limbs(), (double)p, a1);
    ev.multiply_plain(x, a1, T3);
    ev.rescale_to_next_inplace(T3);

    const double mid3 = (T1.scale() + T2.scale() + T3.scale()) / 3;
    T1.scale() = T2.scale() = T3.scale() = mid3;
    dest = T2;
    ev.mod_switch_to_inplace(T1, dest.limbs());
    ev.add_inplace(dest, T1);
    ev.mod_switch_to_inplace(T3, dest.limbs());
    ev.add_inplace(dest, T3);
}

// newtonIter (src/ckks_evaluator.cpp:366-422): res <- 1.5 res - 0.5 x res^3
template <class EV, class CT>
CT CKKSEvaluatorT<EV, CT>::newtonIter(CT x, CT res, int iter)
{
    EV &ev = *evaluator;
    for (int i = 0; i < iter; ++i) {
        Plaintext three_half, neg_half;
        ev.encode(1.5, scale, three_half);
        ev.encode(-0.5, scale, neg_half);
        CT res_sq, res_x;
        ev.square(res, res_sq);
        ev.relinearize_inplace(res_sq);
        ev.rescale_to_next_inplace(res_sq);
        ev.mod_switch_to_inplace(neg_half, x.limbs());
        ev.multiply_plain(x, neg_half, res_x);
        ev.rescale_to_next_inplace(res_x);
        if (res.limbs() < res_x.limbs())
            ev.mod_switch_to_inplace(res_x, res.limbs());
        else
            ev.mod_switch_to_inplace(res, res_x.limbs());
        ev.multiply_inplace(res_x, res);
        ev.relinearize_inplace(res_x);
        ev.rescale_to_next_inplace(res_x);
        ev.mod_switch_to_inplace(res_sq, res_x.limbs());
        ev.multiply_inplace(res_x, res_sq);
        ev.relinearize_inplace(res_x);
        ev.rescale_to_next_inplace(res_x);
        ev.mod_switch_to_inplace(three_half, res.limbs());
        ev.multiply_plain_inplace(res, three_half);
        ev.rescale_to_next_inplace(res);
        ev.mod_switch_to_inplace(res, res_x.limbs());
        res_x.scale() = scale;
        res.scale() = scale;
        ev.add_inplace(res, res_x);
    }
    return res;
}

// goldSchmidtIter (src/ckks_evaluator.cpp:424-478)
template <class EV, class CT>
std::pair<CT, CT> CKKSEvaluatorT<EV, CT>::goldSchmidtIter(CT v, CT y, int d)
{
    EV &ev = *evaluator;
    CT x, h, r, temp;
    Plaintext constant;
    ev.encode(0.5, scale, constant);
    ev.mod_switch_to_inplace(v, y.limbs());
    ev.multiply(v, y, x);
    ev.relinearize_inplace(x);
    ev.rescale_to_next_inplace(x);
    ev.mod_switch_to_inplace(constant, y.limbs());
    ev.multiply_plain(y, constant, h);
    ev.rescale_to_next_inplace(h);
    for (int i = 0; i < d; ++i) {
        ev.encode(0.5, scale, constant);
        ev.multiply(x, h, r);
        ev.relinearize_inplace(r);
        ev.rescale_to_next_inplace(r);
        r.scale() = scale;
        ev.negate(r, temp);
        ev.mod_switch_to_inplace(constant, temp.limbs());
        ev.add_plain(temp, constant, r);
        ev.mod_switch_to_inplace(x, r.limbs());
        ev.multiply(x, r, temp);
        ev.relinearize_inplace(temp);
        ev.rescale_to_next_inplace(temp);
        x.scale() = scale;
        temp.scale() = scale;
        ev.mod_switch_to_inplace(x, temp.limbs());
        ev.add_inplace(x, temp);
        ev.mod_switch_to_inplace(h, r.limbs());
        ev.multiply(h, r, temp);
        ev.relinearize_inplace(temp);
        ev.rescale_to_next_inplace(temp);
        h.scale() = scale;
        temp.scale() = scale;
        ev.mod_switch_to_inplace(h, temp.limbs());
        ev.add_inplace(h, temp);
    }
    ev.encode(2.0, scale, constant);
    ev.mod_switch_to_inplace(constant, h.limbs());
    ev.multiply_plain_inplace(h, constant);
    ev.rescale_to_next_inplace(h);
    return {x, h};
}

// invert_sqrt (src/ckks_evaluator.cpp:480-485): line guess, Newton, Goldschmidt
template <class EV, class CT>
CT CKKSEvaluatorT<EV, CT>::invert_sqrt(CT x, int d_newt, int d_gold)
{
    CT res = initGuess(x);
    CT y = newtonIter(x, res, d_newt);
    return goldSchmidtIter(x, y, d_gold).second;
}

// inverse (src/ckks_evaluator.cpp:487-509): prod_i (1 + (1-x)^(2^i))
template <class EV, class CT>
CT CKKSEvaluatorT<EV, CT>::inverse(CT x, int iter)
{
    EV &ev = *evaluator;
    CT y, tmp, res;
    Plaintext one;
    ev.encode(1.0, x.limbs(), x.scale(), one);
    ev.sub_plain(x, one, y);
    ev.negate_inplace(y);
    ev.add_plain(y, one, tmp);
    res = tmp;
    for (int i = 0; i < iter; ++i) {
        ev.square_inplace(y);
        ev.relinearize_inplace(y);
        ev.rescale_to_next_inplace(y);
        ev.encode(1.0, y.limbs(), y.scale(), one);
        ev.add_plain(y, one, tmp);
        ev.mod_switch_to_inplace(res, tmp.limbs());
        ev.multiply_inplace(res, tmp);
        ev.relinearize_inplace(res);
        ev.rescale_to_next_inplace(res);
    }
    return res;
}

// initGuess / evalLine (src/ckks_evaluator.cpp:517-532)
template <class EV, class CT>
CT CKKSEvaluatorT<EV, CT>::initGuess(CT x)
{
    Plaintext A, B;
    evaluator->encode(-1.29054537e-04, scale, A);
    evaluator->encode(1.29054537e-01, scale, B);
    return evalLine(x, A, B);
}

template <class EV, class CT>
CT CKKSEvaluatorT<EV, CT>::evalLine(CT x, Plaintext m, Plaintext c)
{
    EV &ev = *evaluator;
    ev.mod_switch_to_inplace(m, x.limbs());
    ev.multiply_plain_inplace(x, m);
    ev.rescale_to_next_inplace(x);
    ev.mod_switch_to_inplace(c, x.limbs());
    x.scale() = scale;
    ev.add_plain_inplace(x, c);
    return x;
}

// exp (src/ckks_evaluator.cpp:534-548): (1 + x/128)^128
template <class EV, class CT>
CT CKKSEvaluatorT<EV, CT>::exp(CT x)
{
    EV &ev = *evaluator;
    Plaintext one, inverse_128;
    ev.encode(0.0078125, x.limbs(), x.scale(), inverse_128);
    ev.multiply_plain_inplace(x, inverse_128);
    ev.rescale_to_next_inplace(x);
    ev.encode(1.0, x.limbs(), x.scale(), one);
    ev.add_plain_inplace(x, one);
    for (int i = 0; i < 7; ++i) {
        ev.square_inplace(x);
        ev.relinearize_inplace(x);
        ev.rescale_to_next_inplace(x);
    }
    return x;
}

// GeLUEvaluator::gelu (src/gelu.cpp:5-111); like the original, x is mod-switched in place
template <class EV, class CT>
void GeLUEvaluatorT<EV, CT>::gelu(CT &x, CT &res)
{
    EV &ev = *ckks->evaluator;
    const size_t sc = ckks->slot_count;
    CT b0, b1;
    Plaintext p0, p1, delta;
    ev.encode(ckks->init_vec_with_value(sc, -3.5), x.limbs(), x.scale(), p0);
    ev.encode(ckks->init_vec_with_value(sc, 3.5), x.limbs(), x.scale(), p1);
    ev.encode(ckks->init_vec_with_value(sc, 1.0 / 8.5), x.limbs(), x.scale(), delta);
    ev.sub_plain(x, p0, b0);
    ev.multiply_plain_inplace(b0, delta);
    ev.rescale_to_next_inplace(b0);
    ev.sub_plain(x, p1, b1);
    ev.multiply_plain_inplace(b1, delta);
    ev.rescale_to_next_inplace(b1);
    b0 = ckks->sgn_eval(b0, 2, 2);
    b1 = ckks->sgn_eval(b1, 2, 2);

    Plaintext zero_point_five;
    ev.encode(ckks->init_vec_with_value(sc, 0.5), b1.limbs(), b1.scale(), zero_point_five);
    CT a1, a2;
    ev.sub(b0, b1, a1);
    ev.add_plain(b1, zero_point_five, a2);

    CT x_2, x_4, x_6, x_8, x_10, x_12;
    ev.square(x, x_2);
    ev.relinearize_inplace(x_2);
    ev.rescale_to_next_inplace(x_2);
    ev.square(x_2, x_4);
    ev.relinearize_inplace(x_4);
    ev.rescale_to_next_inplace(x_4);
    ev.mod_switch_to_inplace(x_2, x_4.limbs());
    ev.multiply(x_2, x_4, x_6);
    ev.relinearize_inplace(x_6);
    ev.rescale_to_next_inplace(x_6);
    ev.square(x_4, x_8);
    ev.relinearize_inplace(x_8);
    ev.rescale_to_next_inplace(x_8);
    ev.mod_switch_to_inplace(x_2, x_8.limbs());
    ev.multiply(x_2, x_8, x_10);
    ev.relinearize_inplace(x_10);
    ev.rescale_to_next_inplace(x_10);
    ev.square(x_6, x_12);
    ev.relinearize_inplace(x_12);
    ev.rescale_to_next_inplace(x_12);

    const double A[] = {2.25775755e-04, 0.5, 3.96880960e-01, -6.37042698e-02, 8.38841647e-03, -7.17830961e-04,
                        3.49617829e-05, -7.26059653e-07};
    std::vector<Plaintext> coeff_A(8);
    for (size_t i = 0; i < 8; ++i) ev.encode(A[i], ckks->scale, coeff_A[i]);
    std::vector<CT> cts(8);
    cts[1] = x;
    cts[2] = x_2;
    cts[3] = x_4;
    cts[4] = x_6;
    cts[5] = x_8;
    cts[6] = x_10;
    cts[7] = x_12;
    for (size_t i = 1; i < 8; ++i) {
        ev.mod_switch_to_inplace(coeff_A[i], cts[i].limbs());
        ev.multiply_plain_inplace(cts[i], coeff_A[i]);
        ev.rescale_to_next_inplace(cts[i]);
        cts[i].scale() = ckks->scale;
    }
    CT Ax = cts[7];
    for (size_t i = 1; i < 7; ++i) {
        ev.mod_switch_to_inplace(cts[i], Ax.limbs());
        ev.add_inplace(Ax, cts[i]);
    }
    ev.mod_switch_to_inplace(coeff_A[0], Ax.limbs());
    ev.add_plain_inplace(Ax, coeff_A[0]);

    CT s1, s2;
    ev.mod_switch_to_inplace(Ax, a1.limbs());
    ev.multiply(Ax, a1, s1);
    ev.relinearize_inplace(s1);
    ev.rescale_to_next_inplace(s1);
    ev.mod_switch_to_inplace(x, a2.limbs());
    ev.multiply(x, a2, s2);
    ev.relinearize_inplace(s2);
    ev.rescale_to_next_inplace(s2);
    s1.scale() = ckks->scale;
    s2.scale() = ckks->scale;
    ev.mod_switch_to_inplace(s2, s1.limbs());
    ev.add(s1, s2, res);
}

// SoftmaxEvaluator::softmax (src/softmax.cpp:6-42); x is updated in place as in the original
template <class EV, class CT>
void SoftmaxEvaluatorT<EV, CT>::softmax(CT &x, CT &res, int len)
{
    EV &ev = *ckks->evaluator;
    CT tmp, exp_x;
    const int log_step = (int)std::log2(len);
    ev.rotate_vector(x, -len, tmp);
    ev.add_inplace(x, tmp);
    exp_x = ckks->exp(x);
    tmp = exp_x;
    for (int i = 0; i < log_step; ++i) {
        ev.rotate_vector(tmp, 1 << i, res);
        ev.add_inplace(res, tmp);
        tmp = res;
    }
    Plaintext delta;
    ev.encode(0.01, res.limbs(), res.scale(), delta);
    ev.multiply_plain_inplace(res, delta);
    ev.rescale_to_next_inplace(res);
    res = ckks->inverse(res);
    ev.encode(0.01, res.limbs(), res.scale(), delta);
    ev.multiply_plain_inplace(res, delta);
    ev.rescale_to_next_inplace(res);
    ev.mod_switch_to_inplace(exp_x, res.limbs());
    ev.multiply(res, exp_x, res);
    ev.relinearize_inplace(res);
    ev.rescale_to_next_inplace(res);
}

// LNEvaluator::layer_norm (src/layer_norm.cpp:6-33); x is updated in place as in the original
template <class EV, class CT>
void LNEvaluatorT<EV, CT>::layer_norm(CT &x, CT &res, int len)
{
    EV &ev = *ckks->evaluator;
    CT tmp, x2;
    const int log_step = (int)std::log2(len);
    ev.rotate_vector(x, -len, tmp);
    ev.add_inplace(x, tmp);
    ev.square(x, x2);
    ev.relinearize_inplace(x2);
    ev.rescale_to_next_inplace(x2);
    tmp = x2;
    for (int i = 0; i < log_step; ++i) {
        ev.rotate_vector(tmp, 1 << i, res);
        ev.add_inplace(res, tmp);
        tmp = res;
    }
    Plaintext delta;
    ev.encode(1.0 / 768, res.limbs(), res.scale(), delta);
    ev.multiply_plain_inplace(res, delta);
    ev.rescale_to_next_inplace(res);
    res = ckks->invert_sqrt(res, 4, 2);
    ev.mod_switch_to_inplace(x, res.limbs());
    ev.multiply(res, x, res);
    ev.relinearize_inplace(res);
    ev.rescale_to_next_inplace(res);
}

template class CKKSEvaluatorT<Evaluator, Ciphertext>;
template class CKKSEvaluatorT<BatchEvaluator, CtBatch>;
template class GeLUEvaluatorT<Evaluator, Ciphertext>;
template class GeLUEvaluatorT<BatchEvaluator, CtBatch>;
template class SoftmaxEvaluatorT<Evaluator, Ciphertext>;
template class SoftmaxEvaluatorT<BatchEvaluator, CtBatch>;
template class LNEvaluatorT<Evaluator, Ciphertext>;
template class LNEvaluatorT<BatchEvaluator, CtBatch>;

}  // namespace nexus
