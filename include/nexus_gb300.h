/*
 * nexus_gb300.h -- C ABI of the GB300 CKKS evaluation engine.
 *
 * Conventions (after SEAL's C API, native/src/seal/c/defines.h:35-47 in the
 * SEAL-4.1-bs tree): every entry point returns an int status, 0 on success and
 * a negative value on failure; nexus_last_error() returns the calling
 * thread's last failure message.  No C++ exception crosses this boundary.
 *
 * Data are plain device pointers to uint64 residues laid out exactly as SEAL
 * stores them: a polynomial in RNS form is [limbs][N], a ciphertext is
 * [size][limbs][N], in NTT form.  Streams are passed as void* (a
 * cudaStream_t; NULL means the legacy default stream).
 */
#ifndef NEXUS_GB300_H
#define NEXUS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nexus_context nexus_context;

/* Message of the calling thread's last failed call ("" if none). */
const char *nexus_last_error(void);

/*
 * Primes for a coefficient modulus: out[i] is a prime of bit_sizes[i] bits,
 * congruent to 1 mod 2*poly_degree, chosen exactly as SEAL chooses them.
 * Replaces: CoeffModulus::Create(poly_modulus_degree, bit_sizes)
 *   (native/src/seal/modulus.cpp:143; C API native/src/seal/c/modulus.h:54
 *   CoeffModulus_Create1).
 */
int nexus_create_coeff_modulus(uint64_t poly_degree, const int *bit_sizes, int count, uint64_t *out);

/*
 * Create a context for ring degree N = 2^log_n over the primes `moduli`
 * (n_moduli >= 2): moduli[0..n_moduli-2] are the data primes q_0..q_{L-1},
 * moduli[n_moduli-1] is the special prime (SEAL's key level order).  Builds
 * the NTT tables of every prime on the current CUDA device.
 * Replaces: SEALContext construction + CreateNTTTables
 *   (native/src/seal/c/sealcontext.h:16 SEALContext_Create;
 *    native/src/seal/util/ntt.cpp:241 NTTTables::initialize),
 *   and PhantomContext's DNTTTable setup in the CUDA build.
 */
int nexus_context_create(int log_n, const uint64_t *moduli, int n_moduli, nexus_context **out);
int nexus_context_destroy(nexus_context *ctx);

/* Copy the minimal primitive 2N-th root of every prime into psi_out[n_moduli]. */
int nexus_context_get_psi(const nexus_context *ctx, uint64_t *psi_out);

/*
 * In-place forward negacyclic NTT of n_polys polynomials d_data[n_polys][limbs][N]
 * whose limb l uses prime limb_begin + l (limbs = limb_end - limb_begin).
 * Input residues in [0, q), output in [0, q) in SEAL's bit-reversed order.
 * Replaces: ntt_negacyclic_harvey(PolyIter, size, tables)
 *   (native/src/seal/util/ntt.h:250, util/ntt.cpp:408) and Phantom's
 *   nwt_2d_radix8_forward_inplace (cuda/thirdparty/phantom-fhe/include/ntt.cuh:47).
 */
int nexus_ntt_forward(nexus_context *ctx, uint64_t *d_data, size_t n_polys, int limb_begin, int limb_end,
                      void *stream);

/*
 * In-place inverse of nexus_ntt_forward (including the n^{-1} factor).
 * Replaces: inverse_ntt_negacyclic_harvey(PolyIter, size, tables)
 *   (native/src/seal/util/ntt.h:323, util/ntt.cpp:445) and Phantom's
 *   nwt_2d_radix8_backward_inplace (cuda/thirdparty/phantom-fhe/include/ntt.cuh:77).
 */
int nexus_ntt_inverse(nexus_context *ctx, uint64_t *d_data, size_t n_polys, int limb_begin, int limb_end,
                      void *stream);

#ifdef __cplusplus
}
#endif

#endif /* NEXUS_GB300_H */
