// Engine context: the RNS prime chain of one CKKS parameter set and the
// device tables every kernel reads (twiddles, Barrett ratios, n^{-1}).
//
// Prime order follows SEAL's key level (context.cpp): indices 0..k-2 are the
// data primes q_0..q_{L-1}; index k-1 is the special prime used only inside
// key switching.
#pragma once
#include <atomic>
#include <cstddef>
#include <cstdint>
#include <string>
#include <map>
#include <vector>
#include <cuda_runtime.h>

#include "modarith.cuh"

namespace nexus {

struct Context {
    int logn = 0;
    uint64_t n = 0;
    int k = 0;                       // primes including the special prime
    int device = 0;
    std::vector<uint64_t> q;         // host copy of the primes
    std::vector<uint64_t> psi;       // minimal primitive 2N-th roots
    std::vector<PrimeConst> pc;      // host copy of the per-prime constants

    PrimeConst *d_pc = nullptr;      // [k]
    // Forward twiddles: tw_fwd[j*n + i] = {psi_j^{bitrev(i)}, Shoup quotient}.
    // This is the power table of SEAL's NTTTables (util/ntt.cpp:270-278).
    ulonglong2 *d_tw_fwd = nullptr;  // [k][n]
    // Inverse twiddles indexed like the forward table:
    // tw_inv[j*n + i] = {psi_j^{-bitrev(i)}, Shoup quotient}.
    ulonglong2 *d_tw_inv = nullptr;  // [k][n]

    // Split of the two-pass NTT: n = n1 * n2 (rows x columns).
    int log_n1 = 0, log_n2 = 0;
    // every prime below 2^52: the forward NTT may skip its per-stage
    // conditional subtractions (values stay below 2^58 over 16 stages)
    bool small_primes = false;

    // inv_q[a*k + b] = {q_a^{-1} mod q_b, Shoup quotient} (0 on the diagonal);
    // rescale divides by q_{l-1}, ModDown by the special prime q_{k-1}.
    ulonglong2 *d_inv_q = nullptr;   // [k][k]
    std::vector<ulonglong2> inv_q;   // host copy

    // Galois permutation tables in the NTT domain, one per element, built on
    // first use (GaloisTool::generate_table_ntt, util/galois.cpp:18-52).
    std::map<uint32_t, uint32_t *> galois_tables;

    // Scratch arena reused by every multi-kernel operation; operations on one
    // context are stream-ordered and must not run concurrently.
    uint64_t *scratch = nullptr;
    size_t scratch_words = 0;
    uint64_t *get_scratch(size_t words);
    const uint32_t *galois_table(uint32_t elt);

    // Launch parameters the autotuner (autotune.cu) chooses per context; they
    // change how work maps to CTAs, never a result word.
    struct Tuning {
        // NTT passes: each CTA asks L2 for the tile of the CTA this many
        // residency waves (3 CTAs per SM) ahead; 0 turns the prefetch off
        int ntt_prefetch_waves = 3;
        // key inner product: CTAs per SM of its grid-stride loop; 0 launches
        // one CTA per 512-coefficient chunk
        int ks_inner_ctas_per_sm = 0;
        // forward NTT: 0 two launches (columns pass, rows pass), 1 one launch
        // of thread-block clusters that keep each limb in distributed shared
        // memory between the passes
        int ntt_cluster = 0;
        // forward NTT rows pass: 0 a CTA takes R rows of one limb, 1 one row
        // of R limbs of one prime (the R row groups share their twiddles)
        int ntt_rows_grouped = 0;
    } tune;
    int sm_count = 0;                // multiprocessors of `device`

    // Optional CUDA-event timing of every NTT launch (nexus_ntt_timing_*):
    // each forward/inverse call records an event pair on its stream.
    mutable bool ntt_timing = false;
    mutable std::vector<cudaEvent_t> ntt_events;   // start, stop, start, stop, ...
    mutable std::vector<size_t> ntt_limbs;        // limbs per recorded call
};

// Count of kernels this library has launched (process-wide); read through
// nexus_kernel_launches() so benchmarks can report their own launches.
extern std::atomic<uint64_t> g_kernel_launches;
#define NEXUS_LAUNCHED() (nexus::g_kernel_launches.fetch_add(1, std::memory_order_relaxed))

// Host helpers shared by the translation units.
uint64_t host_mulmod(uint64_t a, uint64_t b, uint64_t q);
uint64_t host_powmod(uint64_t a, uint64_t e, uint64_t q);
uint64_t host_invmod(uint64_t a, uint64_t q);
uint64_t host_shoup(uint64_t w, uint64_t q);

// Thread-local error text behind nexus_last_error().
void set_error(const std::string &msg);

}  // namespace nexus

namespace nexus {
class Encoder;
}

struct nexus_context {
    nexus::Context c;
    nexus::Encoder *enc = nullptr;  // built on first encode/decode
};
