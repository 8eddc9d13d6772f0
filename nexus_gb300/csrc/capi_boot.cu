// C ABI of the bootstrapper (declared in include/nexus_gb300.h).
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>

#include "../../include/nexus_gb300.h"
#include "argmax.h"
#include "bert.h"
#include "bootstrap.h"
#include "capi_types.h"

using namespace nexus;

struct nexus_bootstrapper {
    nexus_evaluator *ev;
    Bootstrapper bs;
    // the lockstep form, built from bs's setup on the first batched call
    std::unique_ptr<BatchEvaluator> bev;
    std::unique_ptr<BatchBootstrapper> bbs;
};

namespace {

int fail(const char *fn, const std::string &msg)
{
    set_error(std::string(fn) + ": " + msg);
    return -1;
}

template <class F>
int guarded(const char *fn, F &&f)
{
    try {
        f();
    } catch (const std::exception &e) {
        return fail(fn, e.what());
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(fn, cudaGetErrorString(e));
    return 0;
}

// the lockstep form of bs, built from its setup on first use
BatchBootstrapper &lockstep_form(nexus_bootstrapper *bs)
{
    Bootstrapper &S = bs->bs;
    if (S.fftcoeff1.empty()) throw std::logic_error("generate_LT_coefficient_3 has not been called");
    if (!bs->bbs) {
        bs->bev.reset(new BatchEvaluator(bs->ev->ev));
        bs->bbs.reset(new BatchBootstrapper(*bs->bev, S.loge, S.logn, S.logNh, S.L, S.final_scale, S.boundary_K,
                                            S.sin_cos_deg, S.scale_factor, S.inverse_deg));
        bs->bbs->adopt_setup(S);
    }
    bs->bbs->set_final_scale(S.final_scale);
    return *bs->bbs;
}

}  // namespace

extern "C" int nexus_bootstrapper_create(nexus_evaluator *ev, long loge, long logn, long logNh, long L,
                                         double final_scale, long boundary_K, long sin_cos_deg, long scale_factor,
                                         long inverse_deg, nexus_bootstrapper **out)
{
    static const char *fn = "nexus_bootstrapper_create";
    if (!ev || !out) return fail(fn, "null argument");
    *out = nullptr;
    return guarded(fn, [&] {
        *out = new nexus_bootstrapper{ev,
                                      Bootstrapper(ev->ev, loge, logn, logNh, L, final_scale, boundary_K, sin_cos_deg,
                                                   scale_factor, inverse_deg),
                                      nullptr, nullptr};
    });
}

extern "C" int nexus_bootstrapper_destroy(nexus_bootstrapper *bs)
{
    delete bs;
    return 0;
}

extern "C" int nexus_bootstrapper_prepare_mod_polynomial(nexus_bootstrapper *bs, int heap_k, int heap_m,
                                                         const int *node_len, const double *coeffs,
                                                         double scale_inverse_coeff)
{
    static const char *fn = "nexus_bootstrapper_prepare_mod_polynomial";
    if (!bs || !node_len || !coeffs) return fail(fn, "null argument");
    if (heap_m < 0 || heap_m > 16) return fail(fn, "heap_m out of range");
    return guarded(fn, [&] {
        const int len = (1 << (heap_m + 1)) - 1;
        std::vector<std::vector<double>> nodes(len);
        size_t off = 0;
        for (int i = 0; i < len; i++) {
            if (node_len[i] < 0) throw std::invalid_argument("negative node length");
            nodes[i].assign(coeffs + off, coeffs + off + node_len[i]);
            off += (size_t)node_len[i];
        }
        bs->bs.prepare_mod_polynomial(heap_k, heap_m, std::move(nodes), scale_inverse_coeff);
        bs->bbs.reset();
    });
}

extern "C" int nexus_bootstrapper_set_inverse_polynomial(nexus_bootstrapper *bs, int deg, const double *power,
                                                         int heap_k, int heap_m, const int *node_len,
                                                         const double *coeffs)
{
    static const char *fn = "nexus_bootstrapper_set_inverse_polynomial";
    if (!bs || !power) return fail(fn, "null argument");
    if (deg < 1 || deg > 255) return fail(fn, "deg out of range");
    if (deg > 3 && (!node_len || !coeffs)) return fail(fn, "null argument");
    if (deg > 3 && (heap_m < 1 || heap_m > 16)) return fail(fn, "heap_m out of range");
    if (bs->bs.inverse_deg != deg) return fail(fn, "deg differs from the bootstrapper's inverse_deg");
    return guarded(fn, [&] {
        ModularReducerT<Evaluator, Ciphertext>::InversePoly p;
        p.power.assign(power, power + deg + 1);
        if (deg > 3) {
            const int len = (1 << (heap_m + 1)) - 1;
            p.heap_k = heap_k;
            p.heap_m = heap_m;
            p.heap.resize(len);
            size_t off = 0;
            for (int i = 0; i < len; i++) {
                if (node_len[i] < 0) throw std::invalid_argument("negative node length");
                p.heap[i].assign(coeffs + off, coeffs + off + node_len[i]);
                off += (size_t)node_len[i];
            }
        }
        bs->bs.mod_reducer.set_inverse_polynomial(std::move(p));
        bs->bbs.reset();
    });
}

extern "C" int nexus_bootstrapper_add_rot_steps(const nexus_bootstrapper *bs, int *steps, int *count, int capacity)
{
    static const char *fn = "nexus_bootstrapper_add_rot_steps";
    if (!bs || !steps || !count) return fail(fn, "null argument");
    if (*count < 0 || *count > capacity) return fail(fn, "count out of range");
    return guarded(fn, [&] {
        std::vector<int> v(steps, steps + *count);
        bs->bs.addLeftRotKeys_Linear_to_vector_3(v);
        if ((int)v.size() > capacity) throw std::length_error("capacity too small");
        for (size_t i = 0; i < v.size(); i++) steps[i] = v[i];
        *count = (int)v.size();
    });
}

extern "C" int nexus_bootstrapper_generate_lt(nexus_bootstrapper *bs)
{
    static const char *fn = "nexus_bootstrapper_generate_lt";
    if (!bs) return fail(fn, "null argument");
    return guarded(fn, [&] {
        bs->bs.generate_LT_coefficient_3();
        bs->bbs.reset();
    });
}

extern "C" int nexus_lt_coefficients_3(int logn, int logNh, long boundary_K, int which, double *out, int *count,
                                       int *len)
{
    static const char *fn = "nexus_lt_coefficients_3";
    if (!count || !len) return fail(fn, "null argument");
    if (which < 0 || which > 5) return fail(fn, "which must be 0..5");
    if (logn < 1 || logn > logNh || logNh > 16) return fail(fn, "bad logn / logNh");
    if (boundary_K < 1) return fail(fn, "boundary_K must be positive");
    try {
        std::vector<CVec> v[6];
        lt_coefficients_3(logn, logNh, boundary_K, v);
        const std::vector<CVec> &d = v[which];
        *count = (int)d.size();
        *len = 0;
        for (const CVec &x : d)
            if ((int)x.size() > *len) *len = (int)x.size();
        if (!out) return 0;
        for (size_t i = 0; i < d.size(); i++)
            for (int j = 0; j < *len; j++) {
                const std::complex<double> z = j < (int)d[i].size() ? d[i][j] : std::complex<double>(0, 0);
                out[((size_t)i * *len + j) * 2] = z.real();
                out[((size_t)i * *len + j) * 2 + 1] = z.imag();
            }
    } catch (const std::exception &e) {
        return fail(fn, e.what());
    }
    return 0;
}

extern "C" int nexus_bootstrap(nexus_bootstrapper *bs, nexus_ciphertext *ct, nexus_ciphertext *rtn)
{
    static const char *fn = "nexus_bootstrap";
    if (!bs || !ct || !rtn) return fail(fn, "null argument");
    if (ct == rtn) return fail(fn, "rtn must be a different ciphertext");
    if (const char *e = input_problem(bs->ev->ctx, ct)) return fail(fn, e);
    return guarded(fn, [&] { bs->bs.bootstrap_3(rtn->ct, ct->ct); });
}

extern "C" int nexus_bootstrap_batch(nexus_bootstrapper *bs, nexus_ciphertext *const *cts, int count,
                                     nexus_ciphertext *const *rtn)
{
    static const char *fn = "nexus_bootstrap_batch";
    if (!bs || !cts || !rtn || count < 1) return fail(fn, "null argument");
    for (int b = 0; b < count; ++b) {
        if (!cts[b] || !rtn[b]) return fail(fn, "null ciphertext");
        if (const char *e = input_problem(bs->ev->ctx, cts[b])) return fail(fn, e);
        for (int j = 0; j < count; ++j)
            if (rtn[b] == cts[j]) return fail(fn, "rtn must not alias an input");
    }
    return guarded(fn, [&] {
        BatchBootstrapper &BB = lockstep_form(bs);
        const Ciphertext &first = cts[0]->ct;
        for (int b = 0; b < count; ++b) {
            const Ciphertext &c = cts[b]->ct;
            if (c.size() != 2) throw std::invalid_argument("Ciphertexts of size 2 are supported only!");
            if (c.limbs() != 1) throw std::invalid_argument("Ciphertexts in the lowest level are supported only!");
            if (c.scale() != first.scale()) throw std::invalid_argument("the ciphertexts of a batch must share one scale");
        }
        Context &ctx = bs->ev->ctx->c;
        cudaStream_t s = bs->ev->ev.stream();
        CtBatch in, out;
        in.resize(ctx, count, 2, 1, s);
        in.scale() = first.scale();
        for (int b = 0; b < count; ++b)
            if (cudaMemcpyAsync(in.ct(b), cts[b]->ct.data(), in.words_per_ct() * 8, cudaMemcpyDeviceToDevice, s) !=
                cudaSuccess)
                throw std::runtime_error("copy failed");
        BB.bootstrap_3(out, in);
        for (int b = 0; b < count; ++b) {
            Ciphertext &r = rtn[b]->ct;
            r.resize(ctx, out.size(), out.limbs(), s);
            r.scale() = out.scale();
            if (cudaMemcpyAsync(r.data(), out.ct(b), out.words_per_ct() * 8, cudaMemcpyDeviceToDevice, s) !=
                cudaSuccess)
                throw std::runtime_error("copy failed");
        }
    });
}

extern "C" int nexus_argmax(nexus_bootstrapper *bs, nexus_ciphertext *x, int len, nexus_ciphertext *res)
{
    static const char *fn = "nexus_argmax";
    if (!bs || !x || !res) return fail(fn, "null argument");
    if (len < 1 || (len & (len - 1))) return fail(fn, "len must be a power of two");
    if (x == res) return fail(fn, "res must be a different ciphertext");
    if (const char *e = input_problem(bs->ev->ctx, x)) return fail(fn, e);
    return guarded(fn, [&] {
        if (bs->bs.fftcoeff1.empty()) throw std::logic_error("generate_LT_coefficient_3 has not been called");
        ArgmaxEvaluator am(bs->ev->ck, bs->bs);
        am.argmax(x->ct, res->ct, len);
    });
}

extern "C" int nexus_argmax_batch(nexus_bootstrapper *bs, nexus_ciphertext *const *x, int count, int len,
                                  nexus_ciphertext *const *res)
{
    static const char *fn = "nexus_argmax_batch";
    if (!bs || !x || !res || count < 1) return fail(fn, "null argument");
    if (len < 1 || (len & (len - 1))) return fail(fn, "len must be a power of two");
    for (int k = 0; k < count; ++k) {
        if (!x[k] || !res[k]) return fail(fn, "null ciphertext");
        if (const char *e = input_problem(bs->ev->ctx, x[k])) return fail(fn, e);
        for (int j = 0; j < count; ++j)
            if (res[k] == x[j] || (j != k && (res[k] == res[j] || x[k] == x[j])))
                return fail(fn, "results and inputs must be distinct ciphertexts");
    }
    return guarded(fn, [&] {
        BatchBootstrapper &BB = lockstep_form(bs);
        CKKSEvaluatorT<BatchEvaluator, CtBatch> ck(*bs->bev, bs->ev->ck.scale);
        ArgmaxEvaluatorT<BatchEvaluator, CtBatch> am(ck, BB);
        CtBatch xb = gather_batch(bs->ev, x, count), out;
        am.argmax(xb, out, len);
        scatter_batch(bs->ev, xb, x);   // the inputs are updated as the single form updates its input
        scatter_batch(bs->ev, out, res);
    });
}

extern "C" int nexus_bootstrap_real_batch(nexus_bootstrapper *bs, nexus_ciphertext *const *cts, int count,
                                          nexus_ciphertext *const *rtn)
{
    static const char *fn = "nexus_bootstrap_real_batch";
    if (!bs || !cts || !rtn || count < 1) return fail(fn, "null argument");
    for (int b = 0; b < count; ++b) {
        if (!cts[b] || !rtn[b]) return fail(fn, "null ciphertext");
        if (const char *e = input_problem(bs->ev->ctx, cts[b])) return fail(fn, e);
        for (int j = 0; j < count; ++j)
            if (rtn[b] == cts[j]) return fail(fn, "rtn must not alias an input");
    }
    return guarded(fn, [&] {
        BatchBootstrapper &BB = lockstep_form(bs);
        BatchEvaluator &ev = *bs->bev;
        const Ciphertext &first = cts[0]->ct;
        for (int b = 0; b < count; ++b) {
            const Ciphertext &c = cts[b]->ct;
            if (c.size() != 2) throw std::invalid_argument("Ciphertexts of size 2 are supported only!");
            if (c.limbs() != 1) throw std::invalid_argument("Ciphertexts in the lowest level are supported only!");
            if (c.scale() != first.scale()) throw std::invalid_argument("the ciphertexts of a batch must share one scale");
        }
        Context &ctx = bs->ev->ctx->c;
        cudaStream_t s = bs->ev->ev.stream();
        const int pairs = count / 2, odd = count % 2;
        auto gather = [&](CtBatch &dst, int first_index, int step, int n) {
            dst.resize(ctx, n, 2, 1, s);
            dst.scale() = first.scale();
            for (int b = 0; b < n; ++b)
                if (cudaMemcpyAsync(dst.ct(b), cts[first_index + step * b]->ct.data(), dst.words_per_ct() * 8,
                                    cudaMemcpyDeviceToDevice, s) != cudaSuccess)
                    throw std::runtime_error("copy failed");
        };
        auto scatter = [&](const CtBatch &src, int first_index, int step) {
            for (int b = 0; b < src.batch(); ++b) {
                Ciphertext &r = rtn[first_index + step * b]->ct;
                r.resize(ctx, src.size(), src.limbs(), s);
                r.scale() = src.scale();
                if (cudaMemcpyAsync(r.data(), src.ct(b), src.words_per_ct() * 8, cudaMemcpyDeviceToDevice, s) !=
                    cudaSuccess)
                    throw std::runtime_error("copy failed");
            }
        };
        Evaluator &base = bs->ev->ev;
        const int half = (int)(ctx.n / 2);
        if (pairs) {
            // z = c0 + X^(N/2) c1 holds c0 + i c1; its scale doubled, the
            // refreshed z holds (c0 + i c1) / 2
            CtBatch c0, c1, t, z, out;
            gather(c0, 0, 2, pairs);
            gather(c1, 1, 2, pairs);
            ev.multiply_plain(c1, base.monomial(half, 1), t);
            ev.add(c0, t, z);
            z.scale() *= 2.0;
            BB.bootstrap_3(out, z);
            CtBatch conj = out, re, im;
            ev.complex_conjugate_inplace(conj);
            ev.add(out, conj, re);
            ev.sub(conj, out, im);
            ev.multiply_plain_inplace(im, base.monomial(half, im.limbs()));
            scatter(re, 0, 2);
            scatter(im, 1, 2);
        }
        if (odd) {
            CtBatch one, out;
            gather(one, count - 1, 1, 1);
            BB.bootstrap_3(out, one);
            scatter(out, count - 1, 1);
        }
    });
}

extern "C" int nexus_bootstrapper_stage(nexus_bootstrapper *bs, int stage, nexus_ciphertext *a,
                                        const nexus_ciphertext *b, nexus_ciphertext *r1, nexus_ciphertext *r2)
{
    static const char *fn = "nexus_bootstrapper_stage";
    if (!bs || !a) return fail(fn, "null argument");
    if (const char *e = input_problem(bs->ev->ctx, a)) return fail(fn, e);
    if (b) {
        if (const char *e = input_problem(bs->ev->ctx, b)) return fail(fn, e);
    }
    return guarded(fn, [&] {
        Bootstrapper &B = bs->bs;
        switch (stage) {
        case NEXUS_BOOT_MODRAISE:
            B.modraise_inplace(a->ct);
            break;
        case NEXUS_BOOT_COEFFTOSLOT:
            if (!r1 || !r2) throw std::invalid_argument("null result");
            B.coefftoslot_full_3(r1->ct, r2->ct, a->ct);
            break;
        case NEXUS_BOOT_MODULAR_REDUCTION:
            if (!r1) throw std::invalid_argument("null result");
            B.mod_reducer.modular_reduction(r1->ct, a->ct);
            break;
        case NEXUS_BOOT_SLOTTOCOEFF:
            if (!b || !r1) throw std::invalid_argument("null argument");
            B.slottocoeff_full_3(r1->ct, a->ct, b->ct);
            break;
        case NEXUS_BOOT_SET_INITIAL_SCALE:
            B.initial_scale = a->ct.scale();
            break;
        default:
            throw std::invalid_argument("unknown stage");
        }
    });
}

extern "C" int nexus_bootstrapper_stage_batch(nexus_bootstrapper *bs, int stage, nexus_ciphertext *const *a,
                                              const nexus_ciphertext *const *b, int count, nexus_ciphertext *const *r1,
                                              nexus_ciphertext *const *r2)
{
    static const char *fn = "nexus_bootstrapper_stage_batch";
    if (!bs || !a || count < 1) return fail(fn, "null argument");
    for (int k = 0; k < count; ++k) {
        if (!a[k]) return fail(fn, "null ciphertext");
        if (const char *e = input_problem(bs->ev->ctx, a[k])) return fail(fn, e);
        if (b) {
            if (!b[k]) return fail(fn, "null ciphertext");
            if (const char *e = input_problem(bs->ev->ctx, b[k])) return fail(fn, e);
        }
        for (int j = 0; j < count; ++j) {
            if ((r1 && r1[k] && (r1[k] == a[j] || (b && r1[k] == b[j]))) ||
                (r2 && r2[k] && (r2[k] == a[j] || (b && r2[k] == b[j]))))
                return fail(fn, "results must not alias inputs");
        }
    }
    auto all = [&](nexus_ciphertext *const *r) {
        if (!r) return false;
        for (int k = 0; k < count; ++k)
            if (!r[k]) return false;
        return true;
    };
    return guarded(fn, [&] {
        BatchBootstrapper &BB = lockstep_form(bs);
        nexus_evaluator *ev = bs->ev;
        CtBatch x = gather_batch(ev, a, count), o1, o2;
        switch (stage) {
        case NEXUS_BOOT_MODRAISE:
            BB.modraise_inplace(x);
            scatter_batch(ev, x, a);
            break;
        case NEXUS_BOOT_COEFFTOSLOT:
            if (!all(r1) || !all(r2)) throw std::invalid_argument("null result");
            BB.coefftoslot_full_3(o1, o2, x);
            scatter_batch(ev, o1, r1);
            scatter_batch(ev, o2, r2);
            break;
        case NEXUS_BOOT_MODULAR_REDUCTION:
            if (!all(r1)) throw std::invalid_argument("null result");
            BB.mod_reducer.modular_reduction(o1, x);
            scatter_batch(ev, o1, r1);
            break;
        case NEXUS_BOOT_SLOTTOCOEFF: {
            if (!b || !all(r1)) throw std::invalid_argument("null argument");
            CtBatch y = gather_batch(ev, b, count);
            BB.slottocoeff_full_3(o1, x, y);
            scatter_batch(ev, o1, r1);
            break;
        }
        case NEXUS_BOOT_SET_INITIAL_SCALE:
            BB.initial_scale = x.scale();
            break;
        default:
            throw std::invalid_argument("unknown stage");
        }
    });
}

extern "C" int nexus_bootstrapper_cached_plaintexts(const nexus_bootstrapper *bs, uint64_t *count)
{
    if (!bs || !count) return fail("nexus_bootstrapper_cached_plaintexts", "null argument");
    *count = bs->bs.cached_plaintexts() + (bs->bbs ? bs->bbs->cached_plaintexts() : 0);
    return 0;
}

// ------------------------------------------------------------------ BERT layer

struct nexus_bert_layer {
    nexus_bootstrapper *bs;
    BertShape shape;
    BertWeights w;
    std::shared_ptr<BertPlaintexts> plain;
    std::vector<std::unique_ptr<BertLayer>> single;  // one per lane
    std::unique_ptr<BatchBertLayer> lockstep;        // every lane, built on first use
    bool timing = false;
};

extern "C" int nexus_bert_layer_create(nexus_bootstrapper *bs, int hidden, int heads, int head_dim, int ffn, int T,
                                       int n_lanes, const int *lane_requests, const int *requests,
                                       double boot_shrink, const double *weights, nexus_bert_layer **out)
{
    static const char *fn = "nexus_bert_layer_create";
    if (!bs || !lane_requests || !requests || !weights || !out) return fail(fn, "null argument");
    if (n_lanes < 1) return fail(fn, "at least one lane is required");
    *out = nullptr;
    return guarded(fn, [&] {
        if (bs->bs.fftcoeff1.empty()) throw std::logic_error("generate_LT_coefficient_3 has not been called");
        std::unique_ptr<nexus_bert_layer> L(new nexus_bert_layer());
        L->bs = bs;
        BertShape &sh = L->shape;
        sh.hidden = hidden;
        sh.heads = heads;
        sh.head_dim = head_dim;
        sh.ffn = ffn;
        sh.T = T;
        sh.boot_shrink = boot_shrink;
        size_t r = 0;
        for (int l = 0; l < n_lanes; ++l) {
            if (lane_requests[l] < 1) throw std::invalid_argument("a lane needs at least one request");
            std::vector<std::pair<int, int>> lane;
            for (int j = 0; j < lane_requests[l]; ++j, ++r) lane.emplace_back(requests[2 * r], requests[2 * r + 1]);
            sh.lanes.push_back(lane);
        }
        sh.derive(bs->ev->ev.slot_count());
        const size_t d = hidden, f = ffn;
        const double *p = weights;
        auto take = [&](std::vector<double> &v, size_t n) {
            v.assign(p, p + n);
            p += n;
        };
        BertWeights &w = L->w;
        take(w.wq, d * d);
        take(w.wk, d * d);
        take(w.wv, d * d);
        take(w.wo, d * d);
        take(w.w1, d * f);
        take(w.w2, f * d);
        take(w.bq, d);
        take(w.bk, d);
        take(w.bv, d);
        take(w.bo, d);
        take(w.b1, f);
        take(w.b2, d);
        L->plain = std::make_shared<BertPlaintexts>();
        for (int l = 0; l < n_lanes; ++l)
            L->single.emplace_back(new BertLayer(bs->ev->ev, bs->bs, sh, w, {l}, L->plain));
        *out = L.release();
    });
}

extern "C" int nexus_bert_layer_destroy(nexus_bert_layer *layer)
{
    delete layer;
    return 0;
}

extern "C" int nexus_bert_layer_info(const nexus_bert_layer *layer, int *n_lanes, int *n_hidden_cts, int *n_head_cts,
                                     int *n_ffn_cts, uint64_t *cached_plaintexts)
{
    if (!layer) return fail("nexus_bert_layer_info", "null argument");
    if (n_lanes) *n_lanes = (int)layer->shape.lanes.size();
    if (n_hidden_cts) *n_hidden_cts = layer->shape.n_hid;
    if (n_head_cts) *n_head_cts = layer->shape.n_head;
    if (n_ffn_cts) *n_ffn_cts = layer->shape.n_ffn;
    if (cached_plaintexts) *cached_plaintexts = layer->plain ? layer->plain->count() : 0;
    return 0;
}

extern "C" int nexus_bert_layer_rotation_steps(const nexus_bert_layer *layer, int *steps, int *count, int capacity)
{
    static const char *fn = "nexus_bert_layer_rotation_steps";
    if (!layer || !count) return fail(fn, "null argument");
    return guarded(fn, [&] {
        const std::vector<int> v = layer->shape.rotation_steps();
        if (steps) {
            if ((int)v.size() > capacity) throw std::length_error("capacity too small");
            for (size_t i = 0; i < v.size(); ++i) steps[i] = v[i];
        }
        *count = (int)v.size();
    });
}

namespace {

BatchBertLayer &bert_lockstep(nexus_bert_layer *L)
{
    if (!L->lockstep) {
        BatchBootstrapper &BB = lockstep_form(L->bs);
        std::vector<int> lanes;
        for (size_t l = 0; l < L->shape.lanes.size(); ++l) lanes.push_back((int)l);
        L->lockstep.reset(new BatchBertLayer(*L->bs->bev, BB, L->shape, L->w, lanes, L->plain));
        L->lockstep->timing = L->timing;
    }
    return *L->lockstep;
}

// run `body` on the lanes' ciphertexts: in[count_in] per lane (lane-major
// handles) -> out[count_out] per lane
template <class F1, class F2>
void bert_run(nexus_bert_layer *L, int lockstep, nexus_ciphertext *const *in, int count_in,
              nexus_ciphertext *const *out, int count_out, F1 &&single_body, F2 &&batch_body)
{
    const int lanes = (int)L->shape.lanes.size();
    nexus_evaluator *ev = L->bs->ev;
    for (int i = 0; i < lanes * count_in; ++i) {
        if (!in[i]) throw std::invalid_argument("null ciphertext");
        if (const char *e = input_problem(ev->ctx, in[i])) throw std::invalid_argument(e);
    }
    for (int i = 0; i < lanes * count_out; ++i)
        if (!out[i]) throw std::invalid_argument("null result");
    if (!lockstep) {
        for (int l = 0; l < lanes; ++l) {
            std::vector<Ciphertext> x(count_in), y;
            for (int c = 0; c < count_in; ++c) x[c] = in[l * count_in + c]->ct;
            single_body(*L->single[l], x, y);
            if ((int)y.size() != count_out) throw std::logic_error("unexpected output count");
            for (int c = 0; c < count_out; ++c) out[l * count_out + c]->ct = std::move(y[c]);
        }
        return;
    }
    BatchBertLayer &B = bert_lockstep(L);
    std::vector<CtBatch> x(count_in), y;
    std::vector<const nexus_ciphertext *> col(lanes);
    for (int c = 0; c < count_in; ++c) {
        for (int l = 0; l < lanes; ++l) col[l] = in[l * count_in + c];
        x[c] = gather_batch(ev, col.data(), lanes);
    }
    batch_body(B, x, y);
    if ((int)y.size() != count_out) throw std::logic_error("unexpected output count");
    std::vector<nexus_ciphertext *> dst(lanes);
    for (int c = 0; c < count_out; ++c) {
        for (int l = 0; l < lanes; ++l) dst[l] = out[l * count_out + c];
        scatter_batch(ev, y[c], dst.data());
    }
}

}  // namespace

extern "C" int nexus_bert_layer_forward(nexus_bert_layer *layer, int lockstep, nexus_ciphertext *const *x,
                                        nexus_ciphertext *const *out)
{
    static const char *fn = "nexus_bert_layer_forward";
    if (!layer || !x || !out) return fail(fn, "null argument");
    return guarded(fn, [&] {
        const int n = layer->shape.n_hid;
        bert_run(
            layer, lockstep, x, n, out, n,
            [](BertLayer &L, std::vector<Ciphertext> &a, std::vector<Ciphertext> &b) { L.forward(a, b); },
            [](BatchBertLayer &L, std::vector<CtBatch> &a, std::vector<CtBatch> &b) { L.forward(a, b); });
    });
}

extern "C" int nexus_bert_layer_stage(nexus_bert_layer *layer, int lockstep, int stage, int which,
                                      nexus_ciphertext *const *in, int count_in, nexus_ciphertext *const *out,
                                      int count_out)
{
    static const char *fn = "nexus_bert_layer_stage";
    if (!layer || !in || !out) return fail(fn, "null argument");
    return guarded(fn, [&] {
        const BertShape &sh = layer->shape;
        switch (stage) {
        case NEXUS_BERT_PROJECT: {
            const bool lower = (which & NEXUS_BERT_LOWER_HALF) != 0;
            const int map = which & ~NEXUS_BERT_LOWER_HALF;
            if (map < 0 || map > 5) throw std::invalid_argument("unknown linear map");
            const int n_in = map == 3 ? sh.n_head : map == 5 ? sh.n_ffn : sh.n_hid;
            const int n_out = map <= 2 ? sh.n_head : map == 4 ? sh.n_ffn : sh.n_hid;
            if (count_in != n_in || count_out != n_out) throw std::invalid_argument("wrong ciphertext count");
            bert_run(
                layer, lockstep, in, n_in, out, n_out,
                [&](BertLayer &L, std::vector<Ciphertext> &a, std::vector<Ciphertext> &b) {
                    L.project(a, map, b, lower);
                },
                [&](BatchBertLayer &L, std::vector<CtBatch> &a, std::vector<CtBatch> &b) {
                    L.project(a, map, b, lower);
                });
            break;
        }
        case NEXUS_BERT_FOLD:
        case NEXUS_BERT_UNFOLD: {
            const bool fold = stage == NEXUS_BERT_FOLD;
            const int halves = fold ? count_in : count_out, folded = fold ? count_out : count_in;
            if (halves < 1 || folded != (halves + 1) / 2) throw std::invalid_argument("wrong ciphertext count");
            if (which != 0 && (fold || which != 1)) throw std::invalid_argument("FOLD takes which = 0, UNFOLD 0 or 1");
            const bool copies = which == 1;
            bert_run(
                layer, lockstep, in, count_in, out, count_out,
                [&](BertLayer &L, std::vector<Ciphertext> &a, std::vector<Ciphertext> &b) {
                    if (fold) L.fold_halves(a);
                    else if (copies) L.unfold_copies(a, count_out);
                    else L.unfold_halves(a, count_out);
                    b = std::move(a);
                },
                [&](BatchBertLayer &L, std::vector<CtBatch> &a, std::vector<CtBatch> &b) {
                    if (fold) L.fold_halves(a);
                    else if (copies) L.unfold_copies(a, count_out);
                    else L.unfold_halves(a, count_out);
                    b = std::move(a);
                });
            break;
        }
        case NEXUS_BERT_ATTENTION: {
            const int nh = sh.n_head;
            if (count_in != 3 * nh || count_out != nh) throw std::invalid_argument("wrong ciphertext count");
            auto split = [nh](auto &a, auto &q, auto &k, auto &v) {
                for (int i = 0; i < nh; ++i) {
                    q.push_back(std::move(a[i]));
                    k.push_back(std::move(a[nh + i]));
                    v.push_back(std::move(a[2 * nh + i]));
                }
            };
            bert_run(
                layer, lockstep, in, 3 * nh, out, nh,
                [&](BertLayer &L, std::vector<Ciphertext> &a, std::vector<Ciphertext> &b) {
                    std::vector<Ciphertext> q, k, v;
                    split(a, q, k, v);
                    L.attention(q, k, v, b);
                },
                [&](BatchBertLayer &L, std::vector<CtBatch> &a, std::vector<CtBatch> &b) {
                    std::vector<CtBatch> q, k, v;
                    split(a, q, k, v);
                    L.attention(q, k, v, b);
                });
            break;
        }
        case NEXUS_BERT_LAYER_NORM:
        case NEXUS_BERT_BOOTSTRAP: {
            if (count_in != count_out || count_in < 1) throw std::invalid_argument("wrong ciphertext count");
            const bool ln = stage == NEXUS_BERT_LAYER_NORM;
            if (ln && which != 0 && which != 1) throw std::invalid_argument("LAYER_NORM takes which = 0 or 1");
            bert_run(
                layer, lockstep, in, count_in, out, count_out,
                [&](BertLayer &L, std::vector<Ciphertext> &a, std::vector<Ciphertext> &b) {
                    if (ln) L.layer_norm(a, which == 1);
                    else L.bootstrap_all(a);
                    b = std::move(a);
                },
                [&](BatchBertLayer &L, std::vector<CtBatch> &a, std::vector<CtBatch> &b) {
                    if (ln) L.layer_norm(a, which == 1);
                    else L.bootstrap_all(a);
                    b = std::move(a);
                });
            break;
        }
        default:
            throw std::invalid_argument("unknown stage");
        }
    });
}

extern "C" int nexus_bert_layer_set_timing(nexus_bert_layer *layer, int enable)
{
    if (!layer) return fail("nexus_bert_layer_set_timing", "null argument");
    for (auto &l : layer->single) l->timing = enable != 0;
    if (layer->lockstep) layer->lockstep->timing = enable != 0;
    layer->timing = enable != 0;
    return 0;
}

extern "C" int nexus_bert_layer_set_boot_pack(nexus_bert_layer *layer, int enable)
{
    if (!layer) return fail("nexus_bert_layer_set_boot_pack", "null argument");
    layer->shape.boot_pack = enable != 0;
    for (auto &l : layer->single) l->set_boot_pack(enable != 0);
    if (layer->lockstep) layer->lockstep->set_boot_pack(enable != 0);
    return 0;
}

extern "C" int nexus_bert_layer_set_token_fold(nexus_bert_layer *layer, int enable)
{
    if (!layer) return fail("nexus_bert_layer_set_token_fold", "null argument");
    layer->shape.token_fold = enable != 0;
    for (auto &l : layer->single) l->set_token_fold(enable != 0);
    if (layer->lockstep) layer->lockstep->set_token_fold(enable != 0);
    return 0;
}

extern "C" int nexus_bert_layer_stage_times(nexus_bert_layer *layer, int lockstep, int lane, double *ms, char *names,
                                            size_t names_capacity, int *count, int capacity)
{
    static const char *fn = "nexus_bert_layer_stage_times";
    if (!layer || !count) return fail(fn, "null argument");
    return guarded(fn, [&] {
        std::vector<std::pair<std::string, double>> t;
        if (lockstep) {
            if (!layer->lockstep) throw std::logic_error("the lockstep form has not run");
            t = layer->lockstep->stage_times();
        } else {
            if (lane < 0 || lane >= (int)layer->single.size()) throw std::invalid_argument("lane out of range");
            t = layer->single[lane]->stage_times();
        }
        if (ms) {
            if ((int)t.size() > capacity) throw std::length_error("capacity too small");
            std::string joined;
            for (size_t i = 0; i < t.size(); ++i) {
                ms[i] = t[i].second;
                joined += t[i].first + "\n";
            }
            if (names) {
                if (joined.size() + 1 > names_capacity) throw std::length_error("names capacity too small");
                std::memcpy(names, joined.c_str(), joined.size() + 1);
            }
        }
        *count = (int)t.size();
    });
}
