// C ABI of the NEXUS operator layer: ciphertext handles, an evaluator bound
// to caller-owned keys, and the CKKSEvaluator / GELU / softmax / LayerNorm
// operators (declared in include/nexus_gb300.h).
#include <stdexcept>
#include <string>

#include "../../include/nexus_gb300.h"
#include "batch.h"
#include "capi_types.h"

using namespace nexus;

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

}  // namespace

extern "C" int nexus_evaluator_create(nexus_context *ctx, double scale, const uint64_t *d_relin_key, void *stream,
                                      nexus_evaluator **out)
{
    static const char *fn = "nexus_evaluator_create";
    if (!ctx || !out) return fail(fn, "null argument");
    *out = nullptr;
    return guarded(fn, [&] {
        auto *e = new nexus_evaluator(ctx, scale);
        e->ev.set_stream((cudaStream_t)stream);
        e->ev.relin_key = d_relin_key;
        *out = e;
    });
}

extern "C" int nexus_evaluator_destroy(nexus_evaluator *ev)
{
    delete ev;
    return 0;
}

extern "C" int nexus_evaluator_add_galois_key(nexus_evaluator *ev, uint32_t galois_elt, const uint64_t *d_key)
{
    static const char *fn = "nexus_evaluator_add_galois_key";
    if (!ev || !d_key) return fail(fn, "null argument");
    if (!(galois_elt & 1) || galois_elt >= 2 * ev->ctx->c.n) return fail(fn, "Galois element is not valid");
    ev->ev.set_galois_key(galois_elt, d_key);
    return 0;
}

extern "C" int nexus_ciphertext_create(nexus_context *ctx, nexus_ciphertext **out)
{
    if (!ctx || !out) return fail("nexus_ciphertext_create", "null argument");
    *out = new nexus_ciphertext{ctx, Ciphertext()};
    return 0;
}

extern "C" int nexus_ciphertext_destroy(nexus_ciphertext *ct)
{
    delete ct;
    return 0;
}

extern "C" int nexus_ciphertext_load(nexus_ciphertext *ct, const uint64_t *src, int size, int limbs, double scale,
                                     int from_host, void *stream)
{
    static const char *fn = "nexus_ciphertext_load";
    if (!ct || !src) return fail(fn, "null argument");
    if (size < 2 || size > 3 || limbs < 1 || limbs > ct->ctx->c.k - 1) return fail(fn, "bad size or limbs");
    return guarded(fn, [&] {
        cudaStream_t s = (cudaStream_t)stream;
        ct->ct.resize(ct->ctx->c, size, limbs, s);
        ct->ct.scale() = scale;
        const size_t bytes = (size_t)size * limbs * ct->ctx->c.n * 8;
        if (cudaMemcpyAsync(ct->ct.data(), src, bytes, from_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                            s) != cudaSuccess)
            throw std::runtime_error("copy failed");
    });
}

extern "C" int nexus_ciphertext_info(const nexus_ciphertext *ct, int *size, int *limbs, double *scale,
                                     uint64_t **d_data)
{
    if (!ct) return fail("nexus_ciphertext_info", "null argument");
    if (size) *size = ct->ct.size();
    if (limbs) *limbs = ct->ct.limbs();
    if (scale) *scale = ct->ct.scale();
    if (d_data) *d_data = ct->ct.data();
    return 0;
}

extern "C" int nexus_ciphertext_store(const nexus_ciphertext *ct, uint64_t *dst, int to_host, void *stream)
{
    static const char *fn = "nexus_ciphertext_store";
    if (!ct || !dst) return fail(fn, "null argument");
    return guarded(fn, [&] {
        cudaStream_t s = (cudaStream_t)stream;
        const size_t bytes = (size_t)ct->ct.size() * ct->ct.limbs() * ct->ctx->c.n * 8;
        if (cudaMemcpyAsync(dst, ct->ct.data(), bytes, to_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                            s) != cudaSuccess)
            throw std::runtime_error("copy failed");
        if (to_host && cudaStreamSynchronize(s) != cudaSuccess) throw std::runtime_error("synchronize failed");
    });
}

extern "C" int nexus_gelu(nexus_evaluator *ev, nexus_ciphertext *x, nexus_ciphertext *res)
{
    static const char *fn = "nexus_gelu";
    if (!ev || !x || !res) return fail(fn, "null argument");
    if (const char *e = input_problem(ev->ctx, x)) return fail(fn, e);
    return guarded(fn, [&] {
        GeLUEvaluator g(ev->ck);
        g.gelu(x->ct, res->ct);
    });
}

extern "C" int nexus_softmax(nexus_evaluator *ev, nexus_ciphertext *x, int len, nexus_ciphertext *res)
{
    static const char *fn = "nexus_softmax";
    if (!ev || !x || !res) return fail(fn, "null argument");
    if (const char *e = input_problem(ev->ctx, x)) return fail(fn, e);
    if (len < 1 || (len & (len - 1))) return fail(fn, "len must be a power of two");
    return guarded(fn, [&] {
        SoftmaxEvaluator sm(ev->ck);
        sm.softmax(x->ct, res->ct, len);
    });
}

extern "C" int nexus_layer_norm(nexus_evaluator *ev, nexus_ciphertext *x, int len, nexus_ciphertext *res)
{
    static const char *fn = "nexus_layer_norm";
    if (!ev || !x || !res) return fail(fn, "null argument");
    if (const char *e = input_problem(ev->ctx, x)) return fail(fn, e);
    if (len < 1 || (len & (len - 1))) return fail(fn, "len must be a power of two");
    return guarded(fn, [&] {
        LNEvaluator ln(ev->ck);
        ln.layer_norm(x->ct, res->ct, len);
    });
}

extern "C" int nexus_ckks_op(nexus_evaluator *ev, int op, const nexus_ciphertext *x, int a1, int a2, double f,
                             nexus_ciphertext *res)
{
    static const char *fn = "nexus_ckks_op";
    if (!ev || !x || !res) return fail(fn, "null argument");
    if (const char *e = input_problem(ev->ctx, x)) return fail(fn, e);
    return guarded(fn, [&] {
        switch (op) {
        case NEXUS_OP_SGN_EVAL: res->ct = ev->ck.sgn_eval(x->ct, a1, a2, f); break;
        case NEXUS_OP_EXP: res->ct = ev->ck.exp(x->ct); break;
        case NEXUS_OP_INVERSE: res->ct = ev->ck.inverse(x->ct, a1); break;
        case NEXUS_OP_INVERT_SQRT: res->ct = ev->ck.invert_sqrt(x->ct, a1, a2); break;
        default: throw std::invalid_argument("unknown op");
        }
    });
}

extern "C" int nexus_evaluator_set_hoisting(nexus_evaluator *ev, int enable)
{
    if (!ev) return fail("nexus_evaluator_set_hoisting", "null argument");
    ev->ev.hoisting = enable != 0;
    return 0;
}

extern "C" int nexus_rotate_vector_many(nexus_evaluator *ev, const nexus_ciphertext *x, const int *steps, int count,
                                        nexus_ciphertext *const *res)
{
    static const char *fn = "nexus_rotate_vector_many";
    if (!ev || !x || !res || (count > 0 && !steps) || count < 0) return fail(fn, "null argument");
    if (const char *e = input_problem(ev->ctx, x)) return fail(fn, e);
    for (int i = 0; i < count; ++i) {
        if (!res[i]) return fail(fn, "null result");
        if (res[i] == x) return fail(fn, "results must not alias the input");
        for (int j = 0; j < i; ++j)
            if (res[j] == res[i]) return fail(fn, "results must be distinct");
    }
    return guarded(fn, [&] {
        std::vector<Ciphertext> outs;
        ev->ev.rotate_vector_many(x->ct, std::vector<int>(steps, steps + count), outs);
        for (int i = 0; i < count; ++i) res[i]->ct = std::move(outs[i]);
    });
}

// ------------------------------------------------------------ lockstep forms

namespace {

using BatchCKKS = CKKSEvaluatorT<BatchEvaluator, CtBatch>;

int check_batch(const char *fn, nexus_evaluator *ev, nexus_ciphertext *const *cts, int count,
                nexus_ciphertext *const *res)
{
    if (!ev || !cts || !res || count < 1) return fail(fn, "null argument");
    for (int b = 0; b < count; ++b) {
        if (!cts[b] || !res[b]) return fail(fn, "null ciphertext");
        if (const char *e = input_problem(ev->ctx, cts[b])) return fail(fn, e);
        for (int j = 0; j < count; ++j)
            if (res[b] == cts[j]) return fail(fn, "results must not alias inputs");
    }
    return 0;
}

}  // namespace

extern "C" int nexus_rotate_vector_many_batch(nexus_evaluator *ev, nexus_ciphertext *const *cts, int count,
                                              const int *steps, int n_steps, nexus_ciphertext *const *res)
{
    static const char *fn = "nexus_rotate_vector_many_batch";
    if (!ev || !cts || !res || count < 1 || n_steps < 0 || (n_steps > 0 && !steps)) return fail(fn, "null argument");
    const size_t total = (size_t)count * n_steps;
    for (int b = 0; b < count; ++b) {
        if (!cts[b]) return fail(fn, "null ciphertext");
        if (const char *e = input_problem(ev->ctx, cts[b])) return fail(fn, e);
    }
    for (size_t i = 0; i < total; ++i) {
        if (!res[i]) return fail(fn, "null result");
        for (int b = 0; b < count; ++b)
            if (res[i] == cts[b]) return fail(fn, "results must not alias inputs");
        for (size_t j = 0; j < i; ++j)
            if (res[j] == res[i]) return fail(fn, "results must be distinct");
    }
    return guarded(fn, [&] {
        BatchEvaluator bev(ev->ev);
        CtBatch x = gather_batch(ev, cts, count);
        std::vector<CtBatch> outs;
        bev.rotate_vector_many(x, std::vector<int>(steps, steps + n_steps), outs);
        for (int i = 0; i < n_steps; ++i) scatter_batch(ev, outs[i], res + (size_t)i * count);
    });
}

extern "C" int nexus_gelu_batch(nexus_evaluator *ev, nexus_ciphertext *const *cts, int count,
                                nexus_ciphertext *const *res)
{
    static const char *fn = "nexus_gelu_batch";
    if (check_batch(fn, ev, cts, count, res)) return -1;
    return guarded(fn, [&] {
        BatchEvaluator bev(ev->ev);
        BatchCKKS ck(bev, ev->ck.scale);
        GeLUEvaluatorT<BatchEvaluator, CtBatch> g(ck);
        CtBatch x = gather_batch(ev, cts, count), out;
        g.gelu(x, out);
        scatter_batch(ev, out, res);
    });
}

extern "C" int nexus_softmax_batch(nexus_evaluator *ev, nexus_ciphertext *const *cts, int count, int len,
                                   nexus_ciphertext *const *res)
{
    static const char *fn = "nexus_softmax_batch";
    if (check_batch(fn, ev, cts, count, res)) return -1;
    if (len < 1 || (len & (len - 1))) return fail(fn, "len must be a power of two");
    return guarded(fn, [&] {
        BatchEvaluator bev(ev->ev);
        BatchCKKS ck(bev, ev->ck.scale);
        SoftmaxEvaluatorT<BatchEvaluator, CtBatch> sm(ck);
        CtBatch x = gather_batch(ev, cts, count), out;
        sm.softmax(x, out, len);
        scatter_batch(ev, out, res);
    });
}

extern "C" int nexus_layer_norm_batch(nexus_evaluator *ev, nexus_ciphertext *const *cts, int count, int len,
                                      nexus_ciphertext *const *res)
{
    static const char *fn = "nexus_layer_norm_batch";
    if (check_batch(fn, ev, cts, count, res)) return -1;
    if (len < 1 || (len & (len - 1))) return fail(fn, "len must be a power of two");
    return guarded(fn, [&] {
        BatchEvaluator bev(ev->ev);
        BatchCKKS ck(bev, ev->ck.scale);
        LNEvaluatorT<BatchEvaluator, CtBatch> ln(ck);
        CtBatch x = gather_batch(ev, cts, count), out;
        ln.layer_norm(x, out, len);
        scatter_batch(ev, out, res);
    });
}

extern "C" int nexus_ckks_op_batch(nexus_evaluator *ev, int op, nexus_ciphertext *const *cts, int count, int a1,
                                   int a2, double f, nexus_ciphertext *const *res)
{
    static const char *fn = "nexus_ckks_op_batch";
    if (check_batch(fn, ev, cts, count, res)) return -1;
    return guarded(fn, [&] {
        BatchEvaluator bev(ev->ev);
        BatchCKKS ck(bev, ev->ck.scale);
        CtBatch x = gather_batch(ev, cts, count), out;
        switch (op) {
        case NEXUS_OP_SGN_EVAL: out = ck.sgn_eval(x, a1, a2, f); break;
        case NEXUS_OP_EXP: out = ck.exp(x); break;
        case NEXUS_OP_INVERSE: out = ck.inverse(x, a1); break;
        case NEXUS_OP_INVERT_SQRT: out = ck.invert_sqrt(x, a1, a2); break;
        default: throw std::invalid_argument("unknown op");
        }
        scatter_batch(ev, out, res);
    });
}

extern "C" int nexus_mm_power_of_x(nexus_evaluator *ev, nexus_ciphertext *x, int index, nexus_ciphertext *res)
{
    static const char *fn = "nexus_mm_power_of_x";
    if (!ev || !x || !res) return fail(fn, "null argument");
    if (const char *e = input_problem(ev->ctx, x)) return fail(fn, e);
    return guarded(fn, [&] {
        MMEvaluator mm(ev->ck);
        mm.multiply_power_of_x(x->ct, res->ct, index);
    });
}

extern "C" int nexus_mm_expand(nexus_evaluator *ev, const nexus_ciphertext *x, uint32_t m, uint64_t *d_out)
{
    static const char *fn = "nexus_mm_expand";
    if (!ev || !x || !d_out) return fail(fn, "null argument");
    if (const char *e = input_problem(ev->ctx, x)) return fail(fn, e);
    if (m < 1 || (m & (m - 1)) || m > ev->ctx->c.n) return fail(fn, "m must be a power of two <= N");
    return guarded(fn, [&] {
        MMEvaluator mm(ev->ck);
        auto leaves = mm.expand_ciphertext(x->ct, m);
        const size_t per = (size_t)2 * x->ct.limbs() * ev->ctx->c.n;
        for (size_t i = 0; i < leaves.size(); ++i)
            cudaMemcpyAsync(d_out + i * per, leaves[i].data(), per * 8, cudaMemcpyDeviceToDevice, ev->ev.stream());
    });
}

extern "C" int nexus_matrix_mul(nexus_evaluator *ev, nexus_ciphertext *const *compressed, int n_compressed,
                                const uint64_t *d_pts, double pt_scale, int rows, int cols, double factor,
                                const double *bias, int bias_len, nexus_ciphertext *const *res)
{
    static const char *fn = "nexus_matrix_mul";
    if (!ev || !compressed || !d_pts || !res || n_compressed < 1) return fail(fn, "null argument");
    for (int i = 0; i < n_compressed; ++i) {
        if (!compressed[i]) return fail(fn, "null compressed ciphertext");
        if (const char *e = input_problem(ev->ctx, compressed[i])) return fail(fn, e);
    }
    for (int r = 0; r < rows; ++r)
        if (!res[r]) return fail(fn, "null result handle");
    return guarded(fn, [&] {
        MMEvaluator mm(ev->ck);
        std::vector<const Ciphertext *> cp;
        for (int i = 0; i < n_compressed; ++i) cp.push_back(&compressed[i]->ct);
        std::vector<Ciphertext> out;
        mm.matrix_mul(cp, d_pts, pt_scale, rows, cols, factor, out);
        if (bias && bias_len > 0) mm.add_bias(out, std::vector<double>(bias, bias + bias_len));
        for (int r = 0; r < rows; ++r) res[r]->ct = std::move(out[r]);
    });
}
