// C ABI entry points (declared in include/nexus_gb300.h).  Each validates
// its arguments, converts C++ exceptions to a status code and records the
// message for nexus_last_error().
#include <stdexcept>
#include <string>

#include "../../include/nexus_gb300.h"
#include "context.h"
#include "ntt.h"
#include "ops.h"
#include "encoder.h"

#include <cmath>
#include <complex>
#include <vector>

using namespace nexus;

namespace {

int fail(const char *fn, const std::string &msg)
{
    set_error(std::string(fn) + ": " + msg);
    return -1;
}

int check_launch(const char *fn)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(fn, cudaGetErrorString(e));
    return 0;
}

int check_limbs(const char *fn, const nexus_context *ctx, const void *d, int lb, int le)
{
    if (!ctx || !d) return fail(fn, "null argument");
    if (lb < 0 || le > ctx->c.k || lb >= le) return fail(fn, "limb range must satisfy 0 <= begin < end <= n_moduli");
    return 0;
}

}  // namespace

extern "C" int nexus_ntt_forward(nexus_context *ctx, uint64_t *d_data, size_t n_polys, int limb_begin, int limb_end,
                                 void *stream)
{
    static const char *fn = "nexus_ntt_forward";
    if (check_limbs(fn, ctx, d_data, limb_begin, limb_end)) return -1;
    try {
        ntt_forward(ctx->c, d_data, n_polys, limb_begin, limb_end, (cudaStream_t)stream);
    } catch (const std::exception &e) {
        return fail(fn, e.what());
    }
    return check_launch(fn);
}

extern "C" int nexus_ntt_inverse(nexus_context *ctx, uint64_t *d_data, size_t n_polys, int limb_begin, int limb_end,
                                 void *stream)
{
    static const char *fn = "nexus_ntt_inverse";
    if (check_limbs(fn, ctx, d_data, limb_begin, limb_end)) return -1;
    try {
        ntt_inverse(ctx->c, d_data, n_polys, limb_begin, limb_end, (cudaStream_t)stream);
    } catch (const std::exception &e) {
        return fail(fn, e.what());
    }
    return check_launch(fn);
}

namespace {

int check_ct(const char *fn, const nexus_context *ctx, int limbs, int min_limbs = 1)
{
    if (!ctx) return fail(fn, "null context");
    if (limbs < min_limbs || limbs > ctx->c.k - 1)
        return fail(fn, "limbs must be in [" + std::to_string(min_limbs) + ", n_moduli-1]");
    return 0;
}

template <class F>
int guarded(const char *fn, F &&f)
{
    try {
        f();
    } catch (const std::exception &e) {
        return fail(fn, e.what());
    }
    return check_launch(fn);
}

}  // namespace

extern "C" int nexus_multiply(nexus_context *ctx, const uint64_t *a, const uint64_t *b, int limbs, uint64_t *out3,
                              void *stream)
{
    static const char *fn = "nexus_multiply";
    if (check_ct(fn, ctx, limbs)) return -1;
    if (!a || !b || !out3) return fail(fn, "null argument");
    return guarded(fn, [&] { tensor(ctx->c, a, b, limbs, out3, (cudaStream_t)stream); });
}

extern "C" int nexus_rescale(nexus_context *ctx, const uint64_t *in, int size, int limbs, uint64_t *out, void *stream)
{
    static const char *fn = "nexus_rescale";
    if (check_ct(fn, ctx, limbs, 2)) return -1;
    if (!in || !out || size < 1) return fail(fn, "null argument or size < 1");
    const size_t n = ctx->c.n;
    if (out < in + (size_t)size * limbs * n && in < out + (size_t)size * (limbs - 1) * n)
        return fail(fn, "d_out must not overlap d_in");
    return guarded(fn, [&] { rescale(ctx->c, in, size, limbs, out, (cudaStream_t)stream); });
}

extern "C" int nexus_switch_key(nexus_context *ctx, uint64_t *ct, int limbs, const uint64_t *target,
                                const uint64_t *key, void *stream)
{
    static const char *fn = "nexus_switch_key";
    if (check_ct(fn, ctx, limbs)) return -1;
    if (!ct || !target || !key) return fail(fn, "null argument");
    return guarded(fn, [&] { switch_key(ctx->c, ct, limbs, target, key, (cudaStream_t)stream); });
}

extern "C" int nexus_switch_key_batch(nexus_context *ctx, uint64_t *ct, int batch, int limbs, const uint64_t *target,
                                      const uint64_t *key, void *stream)
{
    static const char *fn = "nexus_switch_key_batch";
    if (check_ct(fn, ctx, limbs)) return -1;
    if (batch < 0) return fail(fn, "batch must be >= 0");
    if (batch == 0) return 0;
    if (!ct || !target || !key) return fail(fn, "null argument");
    const size_t ct_words = (size_t)batch * 2 * limbs * ctx->c.n, t_words = (size_t)batch * limbs * ctx->c.n;
    if (ct < target + t_words && target < ct + ct_words) return fail(fn, "d_target must not overlap d_ct");
    return guarded(fn, [&] { switch_key_batch(ctx->c, ct, batch, limbs, target, key, (cudaStream_t)stream); });
}

extern "C" int nexus_relinearize(nexus_context *ctx, const uint64_t *ct3, int limbs, const uint64_t *key,
                                 uint64_t *out2, void *stream)
{
    static const char *fn = "nexus_relinearize";
    if (check_ct(fn, ctx, limbs)) return -1;
    if (!ct3 || !key || !out2) return fail(fn, "null argument");
    return guarded(fn, [&] { relinearize(ctx->c, ct3, limbs, key, out2, (cudaStream_t)stream); });
}

extern "C" int nexus_apply_galois(nexus_context *ctx, const uint64_t *ct, int limbs, uint32_t elt, const uint64_t *key,
                                  uint64_t *out, void *stream)
{
    static const char *fn = "nexus_apply_galois";
    if (check_ct(fn, ctx, limbs)) return -1;
    if (!ct || !key || !out) return fail(fn, "null argument");
    if (!(elt & 1) || elt >= 2 * ctx->c.n) return fail(fn, "Galois element is not valid");
    const size_t words = (size_t)2 * limbs * ctx->c.n;
    if (out < ct + words && ct < out + words) return fail(fn, "d_out must not overlap d_ct");
    return guarded(fn, [&] { apply_galois(ctx->c, ct, limbs, elt, key, out, (cudaStream_t)stream); });
}

// GaloisTool::get_elt_from_step (util/galois.cpp:53-90), generator 5
extern "C" int nexus_galois_elt_from_step(int log_n, int step, uint32_t *out)
{
    static const char *fn = "nexus_galois_elt_from_step";
    if (!out || log_n < 1 || log_n > 17) return fail(fn, "bad arguments");
    const uint32_t n = 1u << log_n;
    const uint64_t m = 2ull * n;
    if (step == 0) {
        *out = (uint32_t)(m - 1);
        return 0;
    }
    const bool neg = step < 0;
    uint32_t pos = (uint32_t)(neg ? -(int64_t)step : step);
    if (pos >= (n >> 1)) return fail(fn, "step count too large");
    int e = neg ? (int)(n >> 1) - (int)pos : (int)pos;
    uint64_t g = 1;
    while (e--) g = (g * 5) & (m - 1);
    *out = (uint32_t)g;
    return 0;
}

extern "C" int nexus_add(nexus_context *ctx, const uint64_t *a, const uint64_t *b, int polys, int limbs, uint64_t *out,
                         void *stream)
{
    static const char *fn = "nexus_add";
    if (check_ct(fn, ctx, limbs)) return -1;
    if (!a || !b || !out || polys < 1) return fail(fn, "null argument");
    return guarded(fn, [&] { poly_add(ctx->c, a, b, polys, limbs, out, (cudaStream_t)stream); });
}

extern "C" int nexus_sub(nexus_context *ctx, const uint64_t *a, const uint64_t *b, int polys, int limbs, uint64_t *out,
                         void *stream)
{
    static const char *fn = "nexus_sub";
    if (check_ct(fn, ctx, limbs)) return -1;
    if (!a || !b || !out || polys < 1) return fail(fn, "null argument");
    return guarded(fn, [&] { poly_sub(ctx->c, a, b, polys, limbs, out, (cudaStream_t)stream); });
}

extern "C" int nexus_negate(nexus_context *ctx, const uint64_t *a, int polys, int limbs, uint64_t *out, void *stream)
{
    static const char *fn = "nexus_negate";
    if (check_ct(fn, ctx, limbs)) return -1;
    if (!a || !out || polys < 1) return fail(fn, "null argument");
    return guarded(fn, [&] { poly_negate(ctx->c, a, polys, limbs, out, (cudaStream_t)stream); });
}

extern "C" int nexus_plain_op(nexus_context *ctx, const uint64_t *ct, int size, int limbs, const uint64_t *pt, int op,
                              uint64_t *out, void *stream)
{
    static const char *fn = "nexus_plain_op";
    if (check_ct(fn, ctx, limbs)) return -1;
    if (!ct || !pt || !out || size < 1) return fail(fn, "null argument");
    if (op < 0 || op > 2) return fail(fn, "op must be 0 (multiply), 1 (add) or 2 (sub)");
    return guarded(fn, [&] {
        if (op == 0) poly_mul_plain(ctx->c, ct, size, limbs, pt, out, (cudaStream_t)stream);
        else poly_add_plain(ctx->c, ct, size, limbs, pt, op == 2, out, (cudaStream_t)stream);
    });
}

namespace {

Encoder &encoder_of(nexus_context *ctx)
{
    if (!ctx->enc) ctx->enc = new Encoder(ctx->c);
    return *ctx->enc;
}

}  // namespace

extern "C" int nexus_encode(nexus_context *ctx, const double *re, const double *im, size_t nvals, double scale,
                            int limbs, uint64_t *d_out, void *stream)
{
    static const char *fn = "nexus_encode";
    if (check_ct(fn, ctx, limbs)) return -1;
    if ((!re && nvals) || !d_out) return fail(fn, "null argument");
    return guarded(fn, [&] {
        Encoder &e = encoder_of(ctx);
        std::vector<std::complex<double>> v(nvals);
        for (size_t i = 0; i < nvals; ++i) v[i] = {re[i], im ? im[i] : 0.0};
        std::vector<uint64_t> host((size_t)limbs * ctx->c.n);
        e.encode(v.data(), nvals, scale, limbs, host.data());
        cudaStream_t s = (cudaStream_t)stream;
        if (cudaMemcpyAsync(d_out, host.data(), host.size() * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
            throw std::runtime_error("upload failed");
        ntt_forward(ctx->c, d_out, 1, 0, limbs, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) throw std::runtime_error("stream synchronize failed");
    });
}

extern "C" int nexus_encode_scalar(nexus_context *ctx, double value, double scale, int limbs, uint64_t *per_limb)
{
    static const char *fn = "nexus_encode_scalar";
    if (check_ct(fn, ctx, limbs)) return -1;
    if (!per_limb) return fail(fn, "null argument");
    try {
        encoder_of(ctx).encode_scalar(value, scale, limbs, per_limb);
    } catch (const std::exception &e) {
        return fail(fn, e.what());
    }
    return 0;
}

extern "C" int nexus_multiply_scalar(nexus_context *ctx, const uint64_t *in, int polys, int limbs,
                                     const uint64_t *per_limb, uint64_t *out, void *stream)
{
    static const char *fn = "nexus_multiply_scalar";
    if (check_ct(fn, ctx, limbs)) return -1;
    if (!in || !per_limb || !out || polys < 1) return fail(fn, "null argument");
    for (int l = 0; l < limbs; ++l)
        if (per_limb[l] >= ctx->c.q[l]) return fail(fn, "scalar not reduced mod q_l");
    return guarded(fn, [&] { poly_mul_scalar(ctx->c, in, polys, limbs, per_limb, out, (cudaStream_t)stream); });
}

extern "C" int nexus_decode(nexus_context *ctx, const uint64_t *d_pt, int limbs, double scale, double *re,
                            double *im, size_t nvals, size_t sparse_slots, void *stream)
{
    static const char *fn = "nexus_decode";
    if (check_ct(fn, ctx, limbs)) return -1;
    if (!d_pt || !re) return fail(fn, "null argument");
    if (scale <= 0) return fail(fn, "scale out of bounds");
    return guarded(fn, [&] {
        Encoder &e = encoder_of(ctx);
        const size_t n = ctx->c.n;
        cudaStream_t s = (cudaStream_t)stream;
        uint64_t *tmp = ctx->c.get_scratch((size_t)limbs * n);
        cudaMemcpyAsync(tmp, d_pt, (size_t)limbs * n * 8, cudaMemcpyDeviceToDevice, s);
        ntt_inverse(ctx->c, tmp, 1, 0, limbs, s);
        std::vector<uint64_t> host((size_t)limbs * n);
        if (cudaMemcpyAsync(host.data(), tmp, host.size() * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            throw std::runtime_error("download failed");
        std::vector<std::complex<double>> v(nvals);
        e.decode(host.data(), limbs, scale, v.data(), nvals, sparse_slots);
        for (size_t i = 0; i < nvals; ++i) {
            re[i] = v[i].real();
            if (im) im[i] = v[i].imag();
        }
    });
}

extern "C" int nexus_keygen_secret(nexus_context *ctx, uint64_t seed, int hamming_weight, uint64_t *d_sk,
                                   void *stream)
{
    static const char *fn = "nexus_keygen_secret";
    if (!ctx || !d_sk) return fail(fn, "null argument");
    if (hamming_weight < 0) return fail(fn, "hamming_weight must be >= 0");
    return guarded(fn, [&] { keygen_secret(ctx->c, seed, hamming_weight, d_sk, (cudaStream_t)stream); });
}

extern "C" int nexus_keygen_relin(nexus_context *ctx, const uint64_t *d_sk, uint64_t seed, uint64_t *d_key,
                                  void *stream)
{
    static const char *fn = "nexus_keygen_relin";
    if (!ctx || !d_sk || !d_key) return fail(fn, "null argument");
    return guarded(fn, [&] { keygen_relin(ctx->c, d_sk, seed, d_key, (cudaStream_t)stream); });
}

extern "C" int nexus_keygen_galois(nexus_context *ctx, const uint64_t *d_sk, uint32_t elt, uint64_t seed,
                                   uint64_t *d_key, void *stream)
{
    static const char *fn = "nexus_keygen_galois";
    if (!ctx || !d_sk || !d_key) return fail(fn, "null argument");
    if (!(elt & 1) || elt >= 2 * ctx->c.n) return fail(fn, "Galois element is not valid");
    return guarded(fn, [&] { keygen_galois(ctx->c, d_sk, elt, seed, d_key, (cudaStream_t)stream); });
}

extern "C" int nexus_encrypt_symmetric(nexus_context *ctx, const uint64_t *d_sk, const uint64_t *d_pt, int limbs,
                                       uint64_t seed, uint64_t *d_ct, void *stream)
{
    static const char *fn = "nexus_encrypt_symmetric";
    if (check_ct(fn, ctx, limbs)) return -1;
    if (!d_sk || !d_ct) return fail(fn, "null argument");
    return guarded(fn, [&] { encrypt_symmetric(ctx->c, d_sk, d_pt, limbs, seed, d_ct, (cudaStream_t)stream); });
}

extern "C" int nexus_decrypt(nexus_context *ctx, const uint64_t *d_sk, const uint64_t *d_ct, int size, int limbs,
                             uint64_t *d_pt, void *stream)
{
    static const char *fn = "nexus_decrypt";
    if (check_ct(fn, ctx, limbs)) return -1;
    if (!d_sk || !d_ct || !d_pt || size < 2 || size > 3) return fail(fn, "null argument or size not 2 or 3");
    return guarded(fn, [&] { decrypt(ctx->c, d_sk, d_ct, size, limbs, d_pt, (cudaStream_t)stream); });
}

// coefficient packing of MMEvaluator::enc_compress_ciphertext (src/matrix_mul.cpp:72-96)
extern "C" int nexus_encode_coefficients(nexus_context *ctx, const double *values, size_t n, double scale, int limbs,
                                         uint64_t *d_out, void *stream)
{
    static const char *fn = "nexus_encode_coefficients";
    if (check_ct(fn, ctx, limbs)) return -1;
    if ((!values && n) || !d_out) return fail(fn, "null argument");
    if (n > ctx->c.n) return fail(fn, "more values than coefficients");
    return guarded(fn, [&] {
        const size_t N = ctx->c.n;
        std::vector<uint64_t> host((size_t)limbs * N, 0);
        for (size_t i = 0; i < n; ++i) {
            const double cd = std::round(values[i] * scale);
            const bool neg = std::signbit(cd);
            const double mag = std::fabs(cd);
            if (mag >= 18446744073709551616.0) throw std::invalid_argument("coefficient does not fit in 64 bits");
            const uint64_t cu = (uint64_t)mag;
            for (int j = 0; j < limbs; ++j) {
                uint64_t r = cu % ctx->c.q[j];
                host[(size_t)j * N + i] = (neg && r) ? ctx->c.q[j] - r : r;
            }
        }
        cudaStream_t s = (cudaStream_t)stream;
        if (cudaMemcpyAsync(d_out, host.data(), host.size() * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
            throw std::runtime_error("upload failed");
        ntt_forward(ctx->c, d_out, 1, 0, limbs, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) throw std::runtime_error("stream synchronize failed");
    });
}

extern "C" int nexus_ntt_timing_begin(nexus_context *ctx)
{
    if (!ctx) return fail("nexus_ntt_timing_begin", "null context");
    for (auto e : ctx->c.ntt_events) cudaEventDestroy(e);
    ctx->c.ntt_events.clear();
    ctx->c.ntt_limbs.clear();
    ctx->c.ntt_timing = true;
    return 0;
}

extern "C" int nexus_ntt_timing_end(nexus_context *ctx, double *total_ms, uint64_t *calls, uint64_t *limbs)
{
    static const char *fn = "nexus_ntt_timing_end";
    if (!ctx) return fail(fn, "null context");
    Context &c = ctx->c;
    c.ntt_timing = false;
    double ms = 0;
    uint64_t nl = 0;
    const size_t n = c.ntt_events.size() / 2;
    for (size_t i = 0; i < n; ++i) {
        float t = 0;
        if (cudaEventSynchronize(c.ntt_events[2 * i + 1]) != cudaSuccess ||
            cudaEventElapsedTime(&t, c.ntt_events[2 * i], c.ntt_events[2 * i + 1]) != cudaSuccess)
            return fail(fn, "event timing failed");
        ms += t;
        nl += c.ntt_limbs[i];
    }
    for (auto e : c.ntt_events) cudaEventDestroy(e);
    c.ntt_events.clear();
    c.ntt_limbs.clear();
    if (total_ms) *total_ms = ms;
    if (calls) *calls = n;
    if (limbs) *limbs = nl;
    return 0;
}

extern "C" int nexus_autotune(nexus_context *ctx, int limbs, int batch, int reps, int *ntt_prefetch_waves,
                              int *ks_inner_ctas_per_sm, double *best_ms)
{
    static const char *fn = "nexus_autotune";
    if (!ctx) return fail(fn, "null context");
    try {
        const double ms = nexus::autotune_keyswitch(ctx->c, limbs, batch, nullptr, reps < 1 ? 3 : reps);
        if (best_ms) *best_ms = ms;
    } catch (const std::exception &e) {
        return fail(fn, e.what());
    }
    if (ntt_prefetch_waves) *ntt_prefetch_waves = ctx->c.tune.ntt_prefetch_waves;
    if (ks_inner_ctas_per_sm) *ks_inner_ctas_per_sm = ctx->c.tune.ks_inner_ctas_per_sm;
    return 0;
}

extern "C" int nexus_set_tuning(nexus_context *ctx, int ntt_prefetch_waves, int ks_inner_ctas_per_sm)
{
    static const char *fn = "nexus_set_tuning";
    if (!ctx) return fail(fn, "null context");
    if (ntt_prefetch_waves < 0 || ntt_prefetch_waves > 64 || ks_inner_ctas_per_sm < 0 || ks_inner_ctas_per_sm > 64)
        return fail(fn, "tuning value out of range");
    ctx->c.tune.ntt_prefetch_waves = ntt_prefetch_waves;
    ctx->c.tune.ks_inner_ctas_per_sm = ks_inner_ctas_per_sm;
    return 0;
}

extern "C" int nexus_get_tuning(const nexus_context *ctx, int *ntt_prefetch_waves, int *ks_inner_ctas_per_sm)
{
    if (!ctx) return fail("nexus_get_tuning", "null context");
    if (ntt_prefetch_waves) *ntt_prefetch_waves = ctx->c.tune.ntt_prefetch_waves;
    if (ks_inner_ctas_per_sm) *ks_inner_ctas_per_sm = ctx->c.tune.ks_inner_ctas_per_sm;
    return 0;
}

extern "C" int nexus_set_ntt_form(nexus_context *ctx, int form)
{
    static const char *fn = "nexus_set_ntt_form";
    if (!ctx) return fail(fn, "null context");
    if (form < 0 || form > 2)
        return fail(fn, "form must be 0 (two passes), 1 (one cluster pass) or 2 (two passes, limb-grouped rows)");
    ctx->c.tune.ntt_cluster = form == 1;
    ctx->c.tune.ntt_rows_grouped = form == 2;
    return 0;
}

extern "C" int nexus_get_ntt_form(const nexus_context *ctx, int *form)
{
    if (!ctx || !form) return fail("nexus_get_ntt_form", "null argument");
    *form = ctx->c.tune.ntt_cluster ? 1 : (ctx->c.tune.ntt_rows_grouped ? 2 : 0);
    return 0;
}

extern "C" int nexus_butterfly_rate(int mode, uint64_t q, int rounds, int blocks_per_sm, double *butterflies_per_s,
                                    double *ms)
{
    static const char *fn = "nexus_butterfly_rate";
    if (!butterflies_per_s) return fail(fn, "null argument");
    try {
        *butterflies_per_s = nexus::butterfly_rate(mode, q, rounds, blocks_per_sm, ms);
    } catch (const std::exception &e) {
        return fail(fn, e.what());
    }
    return 0;
}
