// C ABI of key generation and encryption with SEAL's own randomness
// (declared in include/nexus_gb300.h; sampling.cu and seal_prng.cpp).
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/nexus_gb300.h"
#include "context.h"
#include "ops.h"
#include "seal_prng.h"

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

// host-only entry points: no CUDA state to check afterwards
template <class F>
int guarded_host(const char *fn, F &&f)
{
    try {
        f();
    } catch (const std::exception &e) {
        return fail(fn, e.what());
    }
    return 0;
}

bool moduli_in_range(const uint64_t *moduli, int k)
{
    for (int i = 0; i < k; ++i)
        if (moduli[i] < 2 || moduli[i] >= (1ull << 61)) return false;
    return true;
}

}  // namespace

extern "C" int nexus_seal_prng_bytes(const uint64_t *seed, uint64_t offset, size_t n, uint8_t *out)
{
    static const char *fn = "nexus_seal_prng_bytes";
    if (!seed || (!out && n)) return fail(fn, "null argument");
    return guarded_host(fn, [&] {
        sealrng::Stream st(seed);
        st.seek(offset);
        st.bytes_parallel(out, n);
    });
}

extern "C" int nexus_seal_sample_poly(const uint64_t *seed, uint64_t offset, int kind, int log_n,
                                      const uint64_t *moduli, int k, int hamming_weight, uint64_t *out)
{
    static const char *fn = "nexus_seal_sample_poly";
    if (!seed || !moduli || !out) return fail(fn, "null argument");
    if (log_n < 1 || log_n > 17) return fail(fn, "log_n must be in [1, 17]");
    if (k < 1 || !moduli_in_range(moduli, k)) return fail(fn, "moduli must be k >= 1 values in [2, 2^61)");
    const size_t n = (size_t)1 << log_n;
    if (kind == 1 && (hamming_weight < 1 || (size_t)hamming_weight > n))
        return fail(fn, "hamming_weight must be in [1, N] for the sparse ternary sampler");
    if (kind < 0 || kind > 3) return fail(fn, "kind must be 0 (ternary), 1 (sparse ternary), 2 (cbd) or 3 (uniform)");
    return guarded_host(fn, [&] {
        sealrng::Stream st(seed);
        st.seek(offset);
        if (kind == 1) {
            sealrng::sample_sparse_ternary(st, n, moduli, k, (size_t)hamming_weight, out);
            return;
        }
        if (kind == 3) {
            sealrng::sample_uniform_raw(st, n, moduli, k, out);
            for (int j = 0; j < k; ++j)
                for (size_t i = 0; i < n; ++i) out[(size_t)j * n + i] %= moduli[j];
            return;
        }
        std::vector<int8_t> v(n);
        if (kind == 0)
            sealrng::sample_ternary(st, n, v.data());
        else
            sealrng::sample_cbd(st, n, v.data());
        for (int j = 0; j < k; ++j)
            for (size_t i = 0; i < n; ++i)
                out[(size_t)j * n + i] = v[i] < 0 ? moduli[j] - (uint64_t)(-v[i]) : (uint64_t)v[i];
    });
}

extern "C" int nexus_seal_keygen_secret(nexus_context *ctx, const uint64_t *seed, int hamming_weight, uint64_t *d_sk,
                                        void *stream)
{
    static const char *fn = "nexus_seal_keygen_secret";
    if (!ctx || !seed || !d_sk) return fail(fn, "null argument");
    if (hamming_weight < 0 || (size_t)hamming_weight > ctx->c.n) return fail(fn, "hamming_weight must be in [0, N]");
    return guarded(fn, [&] { seal_keygen_secret(ctx->c, seed, hamming_weight, d_sk, (cudaStream_t)stream); });
}

extern "C" int nexus_seal_keygen_public(nexus_context *ctx, const uint64_t *seed, const uint64_t *d_sk,
                                        uint64_t *d_pk, void *stream)
{
    static const char *fn = "nexus_seal_keygen_public";
    if (!ctx || !seed || !d_sk || !d_pk) return fail(fn, "null argument");
    return guarded(fn, [&] {
        seal_encrypt_zero_symmetric(ctx->c, seed, d_sk, nullptr, ctx->c.k, d_pk, (cudaStream_t)stream);
    });
}

extern "C" int nexus_seal_keygen_relin(nexus_context *ctx, const uint64_t *seeds, const uint64_t *d_sk,
                                       uint64_t *d_key, void *stream)
{
    static const char *fn = "nexus_seal_keygen_relin";
    if (!ctx || !seeds || !d_sk || !d_key) return fail(fn, "null argument");
    return guarded(fn, [&] { seal_keygen_relin(ctx->c, seeds, d_sk, d_key, (cudaStream_t)stream); });
}

extern "C" int nexus_seal_keygen_galois(nexus_context *ctx, const uint64_t *seeds, const uint64_t *d_sk,
                                        uint32_t galois_elt, uint64_t *d_key, void *stream)
{
    static const char *fn = "nexus_seal_keygen_galois";
    if (!ctx || !seeds || !d_sk || !d_key) return fail(fn, "null argument");
    if (!(galois_elt & 1) || galois_elt >= 2 * ctx->c.n) return fail(fn, "Galois element is not valid");
    return guarded(fn, [&] { seal_keygen_galois(ctx->c, seeds, d_sk, galois_elt, d_key, (cudaStream_t)stream); });
}

extern "C" int nexus_seal_encrypt(nexus_context *ctx, const uint64_t *seed, const uint64_t *d_pk,
                                  const uint64_t *d_pt, int limbs, uint64_t *d_ct, void *stream)
{
    static const char *fn = "nexus_seal_encrypt";
    if (!ctx || !seed || !d_pk || !d_ct) return fail(fn, "null argument");
    if (limbs < 1 || limbs > ctx->c.k - 1) return fail(fn, "limbs must be in [1, n_moduli-1]");
    return guarded(fn, [&] { seal_encrypt_asymmetric(ctx->c, seed, d_pk, d_pt, limbs, d_ct, (cudaStream_t)stream); });
}

extern "C" int nexus_seal_encrypt_symmetric(nexus_context *ctx, const uint64_t *seed, const uint64_t *d_sk,
                                            const uint64_t *d_pt, int limbs, uint64_t *d_ct, void *stream)
{
    static const char *fn = "nexus_seal_encrypt_symmetric";
    if (!ctx || !seed || !d_sk || !d_ct) return fail(fn, "null argument");
    if (limbs < 1 || limbs > ctx->c.k - 1) return fail(fn, "limbs must be in [1, n_moduli-1]");
    return guarded(fn, [&] {
        seal_encrypt_zero_symmetric(ctx->c, seed, d_sk, d_pt, limbs, d_ct, (cudaStream_t)stream);
    });
}
