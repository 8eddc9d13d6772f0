// Batched (lockstep) evaluation: see batch.h.  Each operation mirrors the
// Evaluator's (ckks.cu) checks, scale bookkeeping and error messages, with
// one launch over the whole batch where the Evaluator has one per ciphertext.
#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>

#include "batch.h"
#include "ops.h"

namespace nexus {

namespace {

void ck(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

void check_same(const CtBatch &a, const CtBatch &b)
{
    if (a.limbs() != b.limbs()) throw std::invalid_argument("encrypted1 and encrypted2 parameter mismatch");
    if (!are_close(a.scale(), b.scale())) throw std::invalid_argument("scale mismatch");
    if (a.size() != b.size()) throw std::invalid_argument("ciphertext sizes differ");
    if (a.batch() != b.batch()) throw std::invalid_argument("batch sizes differ");
}

}  // namespace

// ------------------------------------------------------------------ CtBatch

void CtBatch::resize(const Context &c, int batch, int size, int limbs, cudaStream_t s)
{
    if (batch < 1) throw std::invalid_argument("batch must be positive");
    n_ = c.n;
    s_ = s;
    buf_.reserve((size_t)batch * size * limbs * c.n, s);
    batch_ = batch;
    size_ = size;
    limbs_ = limbs;
}

CtBatch &CtBatch::operator=(const CtBatch &o)
{
    if (this == &o) return *this;
    batch_ = o.batch_;
    scale_ = o.scale_;
    if (o.empty()) {
        buf_.release();
        size_ = limbs_ = 0;
        return *this;
    }
    n_ = o.n_;
    s_ = o.s_;
    buf_.reserve((size_t)o.batch_ * o.words_per_ct(), s_);
    size_ = o.size_;
    limbs_ = o.limbs_;
    ck(cudaMemcpyAsync(buf_.get(), o.buf_.get(), (size_t)batch_ * words_per_ct() * 8, cudaMemcpyDeviceToDevice, s_),
       "copy batch");
    return *this;
}

// ----------------------------------------------------------- level management

void BatchEvaluator::mod_switch_to_inplace(CtBatch &ct, int limbs)
{
    if (limbs > ct.limbs()) throw std::invalid_argument("cannot switch to higher level modulus");
    if (limbs == ct.limbs()) return;
    if (limbs < 1) throw std::invalid_argument("end of modulus switching chain reached");
    CtBatch out;
    out.resize(c_, ct.batch(), ct.size(), limbs, stream());
    out.scale() = ct.scale();
    const size_t row = c_.n * 8;
    ck(cudaMemcpy2DAsync(out.data(), limbs * row, ct.data(), ct.limbs() * row, limbs * row,
                         (size_t)ct.size() * ct.batch(), cudaMemcpyDeviceToDevice, stream()),
       "drop limbs");
    ct = std::move(out);
}

void BatchEvaluator::rescale_to_next_inplace(CtBatch &ct)
{
    if (ct.limbs() < 2) throw std::invalid_argument("end of modulus switching chain reached");
    const double scale = ct.scale() / (double)c_.q[ct.limbs() - 1];
    ev_.check_scale(scale, ct.limbs() - 1);
    CtBatch out;
    out.resize(c_, ct.batch(), ct.size(), ct.limbs() - 1, stream());
    rescale(c_, ct.data(), ct.size() * ct.batch(), ct.limbs(), out.data(), stream());
    out.scale() = scale;
    ct = std::move(out);
}

// ----------------------------------------------------------------- arithmetic

void BatchEvaluator::multiply_inplace(CtBatch &a, const CtBatch &b)
{
    if (a.limbs() != b.limbs()) throw std::invalid_argument("encrypted1 and encrypted2 parameter mismatch");
    if (a.size() != 2 || b.size() != 2) throw std::invalid_argument("multiply expects size-2 ciphertexts");
    if (a.batch() != b.batch()) throw std::invalid_argument("batch sizes differ");
    const double scale = a.scale() * b.scale();
    ev_.check_scale(scale, a.limbs());
    CtBatch out;
    out.resize(c_, a.batch(), 3, a.limbs(), stream());
    tensor(c_, a.data(), b.data(), a.limbs(), out.data(), stream(), a.batch());
    out.scale() = scale;
    a = std::move(out);
}

void BatchEvaluator::multiply(const CtBatch &a, const CtBatch &b, CtBatch &dest)
{
    if (&b == &dest) {
        multiply_inplace(dest, a);
    } else {
        if (&a != &dest) dest = a;
        multiply_inplace(dest, b);
    }
}

void BatchEvaluator::relinearize_inplace(CtBatch &ct)
{
    if (ct.size() == 2) return;
    if (!ev_.relin_key) throw std::invalid_argument("relin_keys is not valid for encryption parameters");
    const int l = ct.limbs();
    CtBatch out;
    out.resize(c_, ct.batch(), 2, l, stream());
    out.scale() = ct.scale();
    relinearize_batch(c_, ct.data(), ct.batch(), l, ev_.relin_key, out.data(), stream());
    ct = std::move(out);
}

void BatchEvaluator::add_inplace(CtBatch &a, const CtBatch &b)
{
    check_same(a, b);
    poly_add(c_, a.data(), b.data(), a.size() * a.batch(), a.limbs(), a.data(), stream());
}

void BatchEvaluator::add(const CtBatch &a, const CtBatch &b, CtBatch &dest)
{
    if (&b == &dest) {
        add_inplace(dest, a);
    } else {
        if (&a != &dest) dest = a;
        add_inplace(dest, b);
    }
}

void BatchEvaluator::sub_inplace(CtBatch &a, const CtBatch &b)
{
    check_same(a, b);
    poly_sub(c_, a.data(), b.data(), a.size() * a.batch(), a.limbs(), a.data(), stream());
}

void BatchEvaluator::sub(const CtBatch &a, const CtBatch &b, CtBatch &dest)
{
    CtBatch bb = b;
    if (&a != &dest) dest = a;
    sub_inplace(dest, bb);
}

void BatchEvaluator::plain_arith(CtBatch &ct, const Plaintext &pt, bool sub)
{
    if (ct.limbs() != pt.limbs()) throw std::invalid_argument("encrypted and plain parameter mismatch");
    if (!are_close(ct.scale(), pt.scale())) throw std::invalid_argument("scale mismatch");
    if (pt.is_scalar()) {
        poly_add_scalar(c_, ct.data(), ct.limbs(), pt.residues().data(), sub ? 1 : 0, ct.data(), stream(), ct.batch(),
                        ct.words_per_ct());
    } else {
        for (int b = 0; b < ct.batch(); ++b)
            poly_add_plain(c_, ct.ct(b), 1, ct.limbs(), pt.data(), sub ? 1 : 0, ct.ct(b), stream());
    }
}

void BatchEvaluator::add_plain(const CtBatch &ct, const Plaintext &pt, CtBatch &dest)
{
    if (&ct != &dest) dest = ct;
    add_plain_inplace(dest, pt);
}

void BatchEvaluator::sub_plain(const CtBatch &ct, const Plaintext &pt, CtBatch &dest)
{
    if (&ct != &dest) dest = ct;
    sub_plain_inplace(dest, pt);
}

void BatchEvaluator::negate_inplace(CtBatch &ct)
{
    poly_negate(c_, ct.data(), ct.size() * ct.batch(), ct.limbs(), ct.data(), stream());
}

void BatchEvaluator::negate(const CtBatch &ct, CtBatch &dest)
{
    if (&ct != &dest) dest = ct;
    negate_inplace(dest);
}

void BatchEvaluator::multiply_plain_inplace(CtBatch &ct, const Plaintext &pt)
{
    multiply_plain(ct, pt, ct);
}

void BatchEvaluator::multiply_plain(const CtBatch &ct, const Plaintext &pt, CtBatch &dest)
{
    if (ct.limbs() != pt.limbs()) throw std::invalid_argument("encrypted and plain parameter mismatch");
    const double scale = ct.scale() * pt.scale();
    ev_.check_scale(scale, ct.limbs());
    if (&ct != &dest) dest.resize(c_, ct.batch(), ct.size(), ct.limbs(), stream());
    const int polys = ct.size() * ct.batch();
    if (pt.is_scalar())
        poly_mul_scalar(c_, ct.data(), polys, ct.limbs(), pt.residues().data(), dest.data(), stream());
    else
        poly_mul_plain(c_, ct.data(), polys, ct.limbs(), pt.data(), dest.data(), stream());
    dest.scale() = scale;
}

void BatchEvaluator::multiply_plain_accumulate(const std::vector<const CtBatch *> &cts,
                                               const std::vector<const Plaintext *> &pts, CtBatch &dest)
{
    const size_t m = cts.size();
    if (m == 0 || pts.size() != m) throw std::invalid_argument("multiply_plain_accumulate: bad term count");
    const int limbs = cts[0]->limbs(), B = cts[0]->batch();
    double scale = 0.0;
    std::vector<const uint64_t *> cp(m), pp(m);
    for (size_t j = 0; j < m; ++j) {
        const CtBatch &ct = *cts[j];
        const Plaintext &pt = *pts[j];
        if (ct.size() != 2 || ct.limbs() != limbs || ct.batch() != B || &ct == &dest)
            throw std::invalid_argument("multiply_plain_accumulate: ciphertexts must be distinct, size 2, one level");
        if (pt.is_scalar() || pt.limbs() != limbs) throw std::invalid_argument("encrypted and plain parameter mismatch");
        scale = ct.scale() * pt.scale();
        ev_.check_scale(scale, limbs);
        cp[j] = ct.data();
        pp[j] = pt.data();
    }
    dest.resize(c_, B, 2, limbs, stream());
    size_t done = 0;
    while (done < m) {
        const int take = (int)std::min<size_t>(16, m - done);
        if (done == 0) {
            poly_mac_plain(c_, cp.data(), pp.data(), take, limbs, dest.data(), stream(), B);
        } else {
            CtBatch part;
            part.resize(c_, B, 2, limbs, stream());
            poly_mac_plain(c_, cp.data() + done, pp.data() + done, take, limbs, part.data(), stream(), B);
            poly_add(c_, dest.data(), part.data(), 2 * B, limbs, dest.data(), stream());
        }
        done += take;
    }
    dest.scale() = scale;
}

// ------------------------------------------------------------------- fork ops

void BatchEvaluator::add_const_inplace(CtBatch &ct, double value)
{
    Plaintext p;
    ev_.encode_then_drop(value, ct.limbs(), ct.scale(), p);
    add_plain_inplace(ct, p);
}

void BatchEvaluator::multiply_const_inplace(CtBatch &ct, double value)
{
    Plaintext p;
    ev_.encode_then_drop(value, ct.limbs(), ct.scale(), p);
    multiply_plain_inplace(ct, p);
}

void BatchEvaluator::multiply_const(const CtBatch &ct, double value, CtBatch &dest)
{
    Plaintext p;
    ev_.encode_then_drop(value, ct.limbs(), ct.scale(), p);
    multiply_plain(ct, p, dest);
}

void BatchEvaluator::multiply_vector_reduced_error(const CtBatch &ct, const std::vector<std::complex<double>> &values,
                                                   CtBatch &dest)
{
    Plaintext p;
    ev_.encode_then_drop(values, ct.limbs(), ct.scale(), p);
    multiply_plain(ct, p, dest);
}

CtBatch BatchEvaluator::adjust_down(const CtBatch &hi, const CtBatch &lo)
{
    const double q_top = (double)c_.q[hi.limbs() - 1];
    const double scale_adjust = lo.scale() * q_top / (hi.scale() * hi.scale());
    CtBatch adj;
    multiply_const_rescale(hi, scale_adjust, adj, lo.scale() * q_top);
    mod_switch_to_inplace(adj, lo.limbs());
    return adj;
}

void BatchEvaluator::multiply_const_rescale_add(const CtBatch &x, double value, CtBatch &acc)
{
    // the rescaled product lands on acc's level: add_inplace_reduced_error's
    // equal-level case (acc takes the product's scale, then acc += product),
    // done by the rescale's finishing kernel
    if (&x != &acc && x.limbs() >= 2 && acc.limbs() == x.limbs() - 1 && acc.size() == x.size() && acc.batch() == x.batch()) {
        Plaintext p;
        ev_.encode_then_drop(value, x.limbs(), x.scale(), p);
        const double prod = x.scale() * p.scale();
        ev_.check_scale(prod, x.limbs());
        const double scale = prod / (double)c_.q[x.limbs() - 1];
        ev_.check_scale(scale, x.limbs() - 1);
        rescale_scaled(c_, x.data(), x.size() * x.batch(), x.limbs(), p.residues().data(), acc.data(), stream(), true);
        acc.scale() = scale;
        return;
    }
    CtBatch tmp;
    multiply_const_rescale(x, value, tmp);
    add_inplace_reduced_error(acc, tmp);
}

void BatchEvaluator::multiply_const_rescale(const CtBatch &ct, double value, CtBatch &dest, double set_scale)
{
    Plaintext p;
    ev_.encode_then_drop(value, ct.limbs(), ct.scale(), p);
    const double prod = ct.scale() * p.scale();
    ev_.check_scale(prod, ct.limbs());
    if (ct.limbs() < 2) throw std::invalid_argument("end of modulus switching chain reached");
    const double scale = (set_scale > 0.0 ? set_scale : prod) / (double)c_.q[ct.limbs() - 1];
    ev_.check_scale(scale, ct.limbs() - 1);
    CtBatch out;
    out.resize(c_, ct.batch(), ct.size(), ct.limbs() - 1, stream());
    rescale_scaled(c_, ct.data(), ct.size() * ct.batch(), ct.limbs(), p.residues().data(), out.data(), stream());
    out.scale() = scale;
    dest = std::move(out);
}

void BatchEvaluator::add_inplace_reduced_error(CtBatch &a, const CtBatch &b)
{
    if (a.limbs() == b.limbs()) {
        a.scale() = b.scale();
        add_inplace(a, b);
    } else if (a.limbs() < b.limbs()) {
        CtBatch adj = adjust_down(b, a);
        a.scale() = adj.scale();
        add_inplace(a, adj);
    } else {
        CtBatch adj = adjust_down(a, b);
        adj.scale() = b.scale();
        add(adj, b, a);
    }
}

void BatchEvaluator::sub_inplace_reduced_error(CtBatch &a, const CtBatch &b)
{
    if (a.limbs() == b.limbs()) {
        a.scale() = b.scale();
        sub_inplace(a, b);
    } else if (a.limbs() < b.limbs()) {
        CtBatch adj = adjust_down(b, a);
        a.scale() = adj.scale();
        sub_inplace(a, adj);
    } else {
        CtBatch adj = adjust_down(a, b);
        adj.scale() = b.scale();
        sub(adj, b, a);
    }
}

void BatchEvaluator::multiply_inplace_reduced_error(CtBatch &a, const CtBatch &b)
{
    if (a.limbs() == b.limbs()) {
        a.scale() = b.scale();
        multiply_inplace(a, b);
    } else if (a.limbs() < b.limbs()) {
        CtBatch adj = adjust_down(b, a);
        a.scale() = adj.scale();
        multiply_inplace(a, adj);
    } else {
        CtBatch adj = adjust_down(a, b);
        adj.scale() = b.scale();
        multiply(adj, b, a);
    }
    relinearize_inplace(a);
}

void BatchEvaluator::add_reduced_error(const CtBatch &a, const CtBatch &b, CtBatch &dest)
{
    if (&b == &dest) {
        add_inplace_reduced_error(dest, a);
    } else {
        if (&a != &dest) dest = a;
        add_inplace_reduced_error(dest, b);
    }
}

void BatchEvaluator::sub_reduced_error(const CtBatch &a, const CtBatch &b, CtBatch &dest)
{
    CtBatch bb = b;
    if (&a != &dest) dest = a;
    sub_inplace_reduced_error(dest, bb);
}

void BatchEvaluator::multiply_reduced_error(const CtBatch &a, const CtBatch &b, CtBatch &dest)
{
    if (&b == &dest) {
        multiply_inplace_reduced_error(dest, a);
    } else {
        if (&a != &dest) dest = a;
        multiply_inplace_reduced_error(dest, b);
    }
}

// ------------------------------------------------------------------ rotations

// out = apply_galois of every ciphertext, one batched key switch
void BatchEvaluator::apply_galois(const CtBatch &ct, uint32_t elt, const uint64_t *key, CtBatch &out)
{
    CtBatch res;
    res.resize(c_, ct.batch(), 2, ct.limbs(), stream());
    res.scale() = ct.scale();
    apply_galois_batch(c_, ct.data(), ct.batch(), ct.limbs(), elt, key, res.data(), stream());
    out = std::move(res);
}

void BatchEvaluator::apply_galois_inplace(CtBatch &ct, uint32_t elt)
{
    auto it = ev_.galois_keys.find(elt);
    if (it == ev_.galois_keys.end()) throw std::invalid_argument("Galois key not present");
    if (ct.size() != 2) throw std::invalid_argument("encrypted size must be 2");
    CtBatch out;
    apply_galois(ct, elt, it->second, out);
    ct = std::move(out);
}

void BatchEvaluator::rotate_vector_inplace(CtBatch &ct, int steps)
{
    if (steps == 0) return;
    const uint32_t elt = ev_.galois_elt(steps);
    if (ev_.galois_keys.count(elt)) {
        apply_galois_inplace(ct, elt);
        return;
    }
    std::vector<int> parts = naf(steps);
    if (parts.size() == 1) throw std::invalid_argument("Galois key not present");
    for (int st : parts)
        if ((size_t)std::abs(st) != (c_.n >> 1)) rotate_vector_inplace(ct, st);
}

void BatchEvaluator::rotate_vector_many(const CtBatch &ct, const std::vector<int> &steps, std::vector<CtBatch> &outs)
{
    outs.resize(steps.size());
    for (const CtBatch &o : outs)
        if (&o == &ct) throw std::invalid_argument("rotate_vector_many: ct must not be one of the outputs");
    const int l = ct.limbs(), B = ct.batch();
    std::vector<bool> done(steps.size(), false);
    std::vector<size_t> direct;
    for (size_t i = 0; i < steps.size(); ++i)
        if (steps[i] != 0 && ev_.galois_keys.count(ev_.galois_elt(steps[i]))) direct.push_back(i);
    std::vector<uint32_t> elts;
    for (size_t i : direct) elts.push_back(ev_.galois_elt(steps[i]));
    if (ev_.hoisting && ct.size() == 2 && Evaluator::hoist_pays((int)direct.size(), l) && ev_.hoist_prepare(elts, l)) {
        const size_t N = c_.n, pitch = ct.words_per_ct();
        DeviceBuffer t, D;
        t.reserve((size_t)B * l * N, stream());
        D.reserve((size_t)B * l * (l + 1) * N, stream());
        int *flags = ev_.hoist_flags(B);
        hoist_decompose(c_, ct.data() + (size_t)l * N, pitch, B, l, t.get(), D.get(), flags, stream());
        std::vector<HoistRotation> rots;
        for (size_t i : direct) {
            const uint32_t elt = ev_.galois_elt(steps[i]);
            const uint64_t *pk = ev_.hoist_key(elt), *corr = ev_.hoist_corr(elt, l);
            outs[i].resize(c_, B, 2, l, stream());
            outs[i].scale() = ct.scale();
            hoist_rotate(c_, D.get(), B, l, elt, pk, corr, ct.data(), pitch, outs[i].data(), stream());
            rots.push_back({elt, ev_.galois_keys.at(elt), outs[i].data()});
            done[i] = true;
        }
        hoist_fix(c_, t.get(), ct.data(), pitch, flags, B, l, rots, stream());
    }
    for (size_t i = 0; i < steps.size(); ++i)
        if (!done[i]) rotate_vector(ct, steps[i], outs[i]);
}

void BatchEvaluator::rotate_vector(const CtBatch &ct, int steps, CtBatch &dest)
{
    if (&ct != &dest && steps != 0) {
        const uint32_t elt = ev_.galois_elt(steps);
        auto it = ev_.galois_keys.find(elt);
        if (it != ev_.galois_keys.end()) {
            if (ct.size() != 2) throw std::invalid_argument("encrypted size must be 2");
            apply_galois(ct, elt, it->second, dest);
            return;
        }
    }
    if (&ct != &dest) dest = ct;
    rotate_vector_inplace(dest, steps);
}

}  // namespace nexus
