// Autotuner of the launch parameters (Context::Tuning): the form of the
// forward NTT (two passes with per-limb or limb-grouped rows, or one pass
// of thread-block clusters), the L2
// prefetch distance of the NTT passes and the grid of the key inner product.
//
// Both only change how work maps to CTAs and when tiles reach L2, never a
// result word.  The tuner times a batched key switch -- a ModUp NTT over
// l(l+1) limbs per ciphertext, the inner product, the ModDown NTTs, the
// shape that dominates the bootstrap and the layer -- on uniform random
// residues for every candidate, with CUDA events after one warm-up,
// and keeps the fastest in the context.
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "context.h"
#include "ops.h"

namespace nexus {

namespace {

// uniform residues of prime pc[prime(r)] for rows r of N words
__global__ void k_fill_random(uint64_t *out, const PrimeConst *__restrict__ pc, int rows_per_prime_cycle, int k,
                              int logn, uint64_t seed, size_t total)
{
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const size_t row = x >> logn;
        const int p = (int)(row % (size_t)rows_per_prime_cycle) % k;
        uint64_t z = seed + x * 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        out[x] = z % pc[p].q;
    }
}

void fill(Context &c, uint64_t *d, size_t rows, int cycle, uint64_t seed, cudaStream_t s)
{
    const size_t total = rows << c.logn;
    const unsigned blocks = (unsigned)std::min<size_t>((total + 255) / 256, (size_t)c.sm_count * 32);
    k_fill_random<<<blocks, 256, 0, s>>>(d, c.d_pc, cycle, c.k, c.logn, seed, total);
    NEXUS_LAUNCHED();
}

}  // namespace

double autotune_keyswitch(Context &c, int l, int B, cudaStream_t s, int reps)
{
    if (l < 1 || l > c.k - 1 || B < 1 || reps < 1) throw std::invalid_argument("autotune: bad shape");
    const size_t N = c.n, K = (size_t)c.k;
    uint64_t *key = nullptr, *ct = nullptr, *tg = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto release = [&]() {
        cudaFree(key);
        cudaFree(ct);
        cudaFree(tg);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    const size_t key_words = (K - 1) * 2 * K * N, ct_words = (size_t)B * 2 * l * N, tg_words = (size_t)B * l * N;
    if (cudaMalloc(&key, key_words * 8) != cudaSuccess || cudaMalloc(&ct, ct_words * 8) != cudaSuccess ||
        cudaMalloc(&tg, tg_words * 8) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
        release();
        cudaGetLastError();
        throw std::runtime_error("autotune: allocation failed");
    }
    // key rows cycle through all K primes; ciphertext and target rows through the first l
    fill(c, key, (K - 1) * 2 * K, (int)K, 1, s);
    fill(c, ct, (size_t)B * 2 * l, l, 2, s);
    fill(c, tg, (size_t)B * l, l, 3, s);
    const Context::Tuning saved = c.tune;
    Context::Tuning best = saved;
    double best_ms = 1e300;
    const int waves[] = {0, 1, 2, 3, 4};
    const int ctas[] = {0, 4, 8, 16};
    // milliseconds per call of the current tuning, after one warm-up call
    auto trial = [&]() {
        switch_key_batch(c, ct, B, l, tg, key, s);
        cudaEventRecord(e0, s);
        for (int r = 0; r < reps; ++r) switch_key_batch(c, ct, B, l, tg, key, s);
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess) throw std::runtime_error("autotune: timing failed");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        return (double)ms / reps;
    };
    try {
        for (int form = 0; form < 3; ++form) {
            c.tune.ntt_cluster = form == 1;
            c.tune.ntt_rows_grouped = form == 2;
            if (form == 1) {
                // the cluster form needs clusters of N/4096 CTAs; where the
                // device refuses them the two-pass form is kept
                try {
                    switch_key_batch(c, ct, B, l, tg, key, s);
                } catch (const std::runtime_error &) {
                    cudaGetLastError();
                    break;
                }
            }
            for (int w : waves)
                for (int g : ctas) {
                    c.tune.ntt_prefetch_waves = w;
                    c.tune.ks_inner_ctas_per_sm = g;
                    const double per = trial();
                    if (per < best_ms) {
                        best_ms = per;
                        best = c.tune;
                    }
                }
        }
    } catch (...) {
        c.tune = saved;
        release();
        throw;
    }
    c.tune = best;
    release();
    return best_ms;
}

}  // namespace nexus
