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

/* Number of GPU kernels this library has launched in the process so far
 * (for benchmarks that report their own launch counts).  No counterpart in
 * the reference. */
uint64_t nexus_kernel_launches(void);

/* Device memory of the current device's stream-ordered pool, which every
 * engine buffer (keys, plaintexts, ciphertexts, temporaries) comes from
 * outside CUDA graphs: bytes in live allocations now, their peak since the
 * process started, and bytes the pool holds (freed blocks stay in the pool
 * for reuse; its release threshold is set to the maximum); and the bytes the
 * device holds for the allocations of instantiated graphs (a graph keeps
 * the memory of its temporaries between launches).  Any pointer may be
 * NULL.  No counterpart in the reference. */
int nexus_memory_info(uint64_t *pool_used, uint64_t *pool_used_high, uint64_t *pool_reserved,
                      uint64_t *graph_reserved);
/* Return the pool's free blocks, and graph memory no instantiated graph
 * uses, to the device (cudaMemPoolTrimTo(pool, 0), cudaDeviceGraphMemTrim);
 * live allocations are untouched.  No counterpart in the reference. */
int nexus_memory_trim(void);

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

/*
 * Measurement hooks: between begin and end every NTT call (forward or
 * inverse, any caller) on this context records a CUDA event pair on its
 * stream; end synchronises and returns the summed device time, the number of
 * calls and the number of limb-NTTs.  No counterpart in the reference.
 */
int nexus_ntt_timing_begin(nexus_context *ctx);
int nexus_ntt_timing_end(nexus_context *ctx, double *total_ms, uint64_t *calls, uint64_t *limbs);

/*
 * The NTT's compute ceiling on this GPU: butterflies per second of its own
 * butterfly (mode 0 the forward Harvey butterfly, 1 the forward butterfly for
 * primes below 2^52, 2 the inverse Gentleman-Sande butterfly), each thread
 * running `rounds` rounds of four radix-2 stages over 16 register residues,
 * blocks_per_sm CTAs of 256 threads per SM, no memory traffic in the loop;
 * *ms receives one launch's duration.  Synchronous.  A measurement aid with
 * no counterpart in the reference.
 */
int nexus_butterfly_rate(int mode, uint64_t q, int rounds, int blocks_per_sm, double *butterflies_per_s,
                         double *ms);

/*
 * Dense rate of this GPU's fifth-generation tensor cores through hand-written
 * tcgen05.mma: one CTA per SM holds a 128 x 256 f32 accumulator in tensor
 * memory and issues `rounds` x 4 MMAs of 128 x 256 x K from shared memory
 * (kind 0: bf16 operands, kind::f16, K = 16; kind 1: e4m3 operands,
 * kind::f8f6f4, K = 32), committed to an mbarrier.  Returns FLOP/s (2 per
 * multiply-add) of the whole GPU; *ms receives one launch's duration.
 * Synchronous.  nexus_tensor_tile runs the same kernel on one CTA and copies
 * the accumulator out: a (128 rows) and b (256 rows) hold 128 bytes of K
 * per row (64 bf16 or 128 e4m3 values, row-major), and d (128 x 256 f32,
 * row-major) receives rounds * a . b^T.  Measurement aids for the tensor-pipe
 * decision, with no counterpart in the reference.
 */
int nexus_tensor_rate(int kind, int rounds, double *flops_per_s, double *ms);
int nexus_tensor_tile(int kind, int rounds, const void *a, const void *b, float *d);

/*
 * Autotuner of the context's launch parameters: the L2 prefetch distance of
 * the NTT passes (in residency waves of 3 CTAs per SM, 0 = none; candidates
 * 0-4) and the grid of the key inner product (CTAs per SM of its grid-stride
 * loop, 0 = one CTA per 512 coefficients; candidates 0, 4, 8, 16).  It times
 * a batched key switch of `batch` ciphertexts at `limbs` limbs on uniform
 * random residues for every pair (one warm-up, then `reps` calls), keeps the
 * fastest in the context and returns it with its milliseconds per call.
 * Synchronous; allocates a key and the ciphertexts for the trial and frees
 * them.  The parameters never change a result word.  set/get read or write
 * them directly.  No counterpart in the reference (Phantom's launch
 * constants are fixed, cuda/thirdparty/phantom-fhe/include/common.h:22-32).
 */
int nexus_autotune(nexus_context *ctx, int limbs, int batch, int reps, int *ntt_prefetch_waves,
                   int *ks_inner_ctas_per_sm, double *best_ms);
int nexus_set_tuning(nexus_context *ctx, int ntt_prefetch_waves, int ks_inner_ctas_per_sm);
int nexus_get_tuning(const nexus_context *ctx, int *ntt_prefetch_waves, int *ks_inner_ctas_per_sm);

/*
 * Form of the forward NTT (every forward transform of the context, the key
 * switch's ModUp and ModDown included): 0 = two launches, a columns pass and
 * a rows pass, each reading and writing the limb in HBM (default); 1 = one
 * launch of thread-block clusters of N/4096 CTAs that keep a limb in their
 * distributed shared memory between the passes, so the limb crosses HBM
 * once each way; 2 = the two launches with the rows pass's CTAs each taking
 * one row of 16 (or 32, 64) limbs of one prime, whose row groups share the
 * row's twiddles (launches of fewer polynomials keep form 0's rows pass).
 * Same words in every form.
 */
int nexus_set_ntt_form(nexus_context *ctx, int form);
int nexus_get_ntt_form(const nexus_context *ctx, int *form);

/* ------------------------------------------------------------------ */
/* CKKS ciphertext arithmetic (NTT form, limbs = data primes 0..limbs-1) */
/* ------------------------------------------------------------------ */

/*
 * Tensor product of two size-2 ciphertexts a, b [2][limbs][N] into the
 * size-3 ciphertext out3 [3][limbs][N] (no relinearization).
 * Replaces: Evaluator::multiply_inplace -> ckks_multiply
 *   (native/src/seal/evaluator.cpp:770-850); Phantom tensor_prod_2x2_rns_poly
 *   (cuda/thirdparty/phantom-fhe/src/polymath.cu:468).
 */
int nexus_multiply(nexus_context *ctx, const uint64_t *d_a, const uint64_t *d_b, int limbs, uint64_t *d_out3,
                   void *stream);

/*
 * Rescale: divide every polynomial of d_in [size][limbs][N] by the last prime
 * with rounding; d_out is [size][limbs-1][N] and must not overlap d_in.
 * Replaces: Evaluator::rescale_to_next -> RNSTool::divide_and_round_q_last_ntt_inplace
 *   (native/src/seal/evaluator.cpp:1682, util/rns.cpp:830-905); Phantom
 *   rescale_to_next (cuda/thirdparty/phantom-fhe/src/rns.cu:1157).
 */
int nexus_rescale(nexus_context *ctx, const uint64_t *d_in, int size, int limbs, uint64_t *d_out, void *stream);

/*
 * Key switching: d_ct [2][limbs][N] += switch(d_target [limbs][N]) under the
 * key-switching key d_key [n_moduli-1][2][n_moduli][N] (SEAL's KSwitchKeys
 * layout: one PublicKey per data prime at the key level).  Every key passed to
 * the key-switching calls (switch, relinearize, Galois) must start on a
 * 16-byte boundary, as any cudaMalloc'd buffer does; others are rejected.
 * Replaces: Evaluator::switch_key_inplace (native/src/seal/evaluator.cpp:2724-3022);
 *   Phantom keyswitch_inplace (cuda/thirdparty/phantom-fhe/src/eval_key_switch.cu:93).
 */
int nexus_switch_key(nexus_context *ctx, uint64_t *d_ct, int limbs, const uint64_t *d_target, const uint64_t *d_key,
                     void *stream);

/*
 * Key switching of `batch` ciphertexts at one level under one key:
 * d_ct [batch][2][limbs][N], d_target [batch][limbs][N] (must not overlap
 * d_ct).  Ciphertext b receives the words nexus_switch_key gives for
 * (d_ct[b], d_target[b]); every kernel runs once over the whole batch and the
 * key is read once per batch.
 * No counterpart in the reference: SEAL's switch_key_inplace
 *   (native/src/seal/evaluator.cpp:2724-3022) takes one ciphertext per call.
 */
int nexus_switch_key_batch(nexus_context *ctx, uint64_t *d_ct, int batch, int limbs, const uint64_t *d_target,
                           const uint64_t *d_key, void *stream);

/*
 * Key switching that allocates nothing: the same operation and output words
 * as nexus_switch_key, for callers that cannot let the library call
 * cudaMalloc/cudaFree (their device memory is owned by another runtime's
 * pool, or the implicit device synchronisation of an allocation is not
 * allowed where they call).  Temporaries live in a fixed device array of
 * 2^21 uint64 words (16 MiB) inside the library, which every GPU that loads
 * the library holds until the process exits; requests needing more than
 * N*(limbs^2 + 6*limbs + 4) > 2^21 words are rejected with an error.  Every
 * call looks up the array's address (cudaGetSymbolAddress, a host query) with
 * the context's device current.  The first call on a device also loads the
 * library's kernel modules (CUDA loads modules lazily), which allocates device
 * memory once: make that first call, or one nexus_switch_key on the same
 * device, before any stream capture or before the other runtime takes over
 * the device's memory.  All calls share the array, so calls whose work
 * overlaps on the GPU (different streams, no ordering) race; every word is
 * written before it is read, so no clearing is needed between calls.
 * No counterpart in the reference: SEAL and Phantom allocate their key-switch
 * temporaries from a memory pool on every call.
 */
int nexus_switch_key_noalloc(nexus_context *ctx, uint64_t *d_ct, int limbs, const uint64_t *d_target,
                             const uint64_t *d_key, void *stream);

/*
 * Relinearize the size-3 ciphertext d_ct3 into d_out2 [2][limbs][N]
 * (d_out2 may equal d_ct3).
 * Replaces: Evaluator::relinearize_inplace -> relinearize_internal
 *   (native/src/seal/evaluator.cpp:1345-1400).
 */
int nexus_relinearize(nexus_context *ctx, const uint64_t *d_ct3, int limbs, const uint64_t *d_relin_key,
                      uint64_t *d_out2, void *stream);

/*
 * Apply the automorphism X -> X^galois_elt and switch back to the secret key.
 * Replaces: Evaluator::apply_galois_inplace (native/src/seal/evaluator.cpp:2563-2665);
 *   rotate_vector / complex_conjugate use it with the element of a step.
 * d_out ([2][limbs][N]) must not overlap d_ct.
 */
int nexus_apply_galois(nexus_context *ctx, const uint64_t *d_ct, int limbs, uint32_t galois_elt,
                       const uint64_t *d_galois_key, uint64_t *d_out, void *stream);

/*
 * Galois element of a slot rotation by `step` (0 = complex conjugation).
 * Replaces: GaloisTool::get_elt_from_step (native/src/seal/util/galois.cpp:53-90).
 */
int nexus_galois_elt_from_step(int log_n, int step, uint32_t *out);

/* out = a + b / a - b / -a over [polys][limbs][N].
 * Replaces: Evaluator::add_inplace / sub_inplace / negate_inplace
 *   (native/src/seal/evaluator.cpp:155, 263, 130). */
int nexus_add(nexus_context *ctx, const uint64_t *d_a, const uint64_t *d_b, int polys, int limbs, uint64_t *d_out,
              void *stream);
int nexus_sub(nexus_context *ctx, const uint64_t *d_a, const uint64_t *d_b, int polys, int limbs, uint64_t *d_out,
              void *stream);
int nexus_negate(nexus_context *ctx, const uint64_t *d_a, int polys, int limbs, uint64_t *d_out, void *stream);

/* Every polynomial of d_ct [size][limbs][N] times (op 0), plus (op 1) or minus
 * (op 2) the plaintext d_pt [limbs][N].
 * Replaces: Evaluator::multiply_plain_inplace -> multiply_plain_ntt
 *   (native/src/seal/evaluator.cpp:2154, 2336-2373), add_plain_inplace (:1938),
 *   sub_plain_inplace (:2046); the plaintext is added to component 0 only,
 *   so callers pass size = 1 for op 1 and 2. */
int nexus_plain_op(nexus_context *ctx, const uint64_t *d_ct, int size, int limbs, const uint64_t *d_pt, int op,
                   uint64_t *d_out, void *stream);

/* ------------------------------------------------------------------ */
/* Keys, encryption, decryption (test/benchmark keys: the sampler is a  */
/* seeded counter hash, not a cryptographic generator; deployed keys are */
/* made by the client with SEAL and imported in the same layout)         */
/* ------------------------------------------------------------------ */

/* Ternary secret key (hamming_weight > 0: exactly that many +-1
 * coefficients, the NEXUS fork's sparse secret) in NTT form, d_sk [n_moduli][N].
 * Replaces: KeyGenerator::generate_sk (native/src/seal/keygenerator.cpp:56). */
int nexus_keygen_secret(nexus_context *ctx, uint64_t seed, int hamming_weight, uint64_t *d_sk, void *stream);

/* Relinearization key for s^2, d_key [n_moduli-1][2][n_moduli][N].
 * Replaces: KeyGenerator::create_relin_keys (native/src/seal/keygenerator.cpp:124)
 *   over generate_one_kswitch_key (:303-336). */
int nexus_keygen_relin(nexus_context *ctx, const uint64_t *d_sk, uint64_t seed, uint64_t *d_key, void *stream);

/* Galois key for X -> X^galois_elt (same layout).
 * Replaces: KeyGenerator::create_galois_keys (native/src/seal/keygenerator.cpp:164). */
int nexus_keygen_galois(nexus_context *ctx, const uint64_t *d_sk, uint32_t galois_elt, uint64_t seed,
                        uint64_t *d_key, void *stream);

/* Symmetric encryption of the NTT-form plaintext d_pt [limbs][N] (NULL:
 * encryption of zero) into d_ct [2][limbs][N].
 * Replaces: Encryptor::encrypt_symmetric -> encrypt_zero_symmetric
 *   (native/src/seal/encryptor.cpp:176, util/rlwe.cpp:311). */
int nexus_encrypt_symmetric(nexus_context *ctx, const uint64_t *d_sk, const uint64_t *d_pt, int limbs, uint64_t seed,
                            uint64_t *d_ct, void *stream);

/* d_pt [limbs][N] = c0 + c1 s (+ c2 s^2 for size 3), NTT form.
 * Replaces: Decryptor::decrypt (native/src/seal/decryptor.cpp:78). */
int nexus_decrypt(nexus_context *ctx, const uint64_t *d_sk, const uint64_t *d_ct, int size, int limbs,
                  uint64_t *d_pt, void *stream);

/* ------------------------------------------------------------------ */
/* Keys and encryption with SEAL's own randomness                       */
/* ------------------------------------------------------------------ */
/*
 * The same words SEAL-4.1-bs produces: every `seed` is 8 words (64 bytes),
 * the seed that one UniformRandomGeneratorFactory::create() call hands to a
 * Blake2xbPRNG (randomgen.h:440-448, 504-567).  A factory made with a default
 * seed (Blake2xbPRNGFactory(seed)) gives that seed to every call; the default
 * factory draws a fresh one per call.  Key-switching keys make one call per
 * data prime, so they take n_moduli-1 seeds back to back, in digit order.
 * The byte streams and samplers run on the host, the NTTs and the modular
 * arithmetic on the GPU; these calls return after the device work is done.
 */

/* Bytes [offset, offset + n) of the Blake2xbPRNG stream of `seed` (host only).
 * Replaces: UniformRandomGenerator::generate (native/src/seal/randomgen.cpp:174-190)
 *   over Blake2xbPRNG::refill_buffer (:197-207). */
int nexus_seal_prng_bytes(const uint64_t *seed, uint64_t offset, size_t n, uint8_t *out);

/* One SEAL sampler on a fresh stream advanced by `offset` bytes, written as
 * residues out [k][2^log_n] (host only): kind 0 sample_poly_ternary, 1
 * sample_poly_sparse_ternary (hamming_weight nonzeros), 2 sample_poly_cbd,
 * 3 sample_poly_uniform.
 * Replaces: native/src/seal/util/rlwe.cpp:21-37, 39-69, 99-135, 137-165. */
int nexus_seal_sample_poly(const uint64_t *seed, uint64_t offset, int kind, int log_n, const uint64_t *moduli, int k,
                           int hamming_weight, uint64_t *out);

/* Secret key d_sk [n_moduli][N] (NTT form); hamming_weight > 0 gives the
 * NEXUS fork's sparse secret.
 * Replaces: KeyGenerator::generate_sk (native/src/seal/keygenerator.cpp:56-93). */
int nexus_seal_keygen_secret(nexus_context *ctx, const uint64_t *seed, int hamming_weight, uint64_t *d_sk,
                             void *stream);

/* Public key d_pk [2][n_moduli][N].
 * Replaces: KeyGenerator::generate_pk (native/src/seal/keygenerator.cpp:95-122)
 *   -> encrypt_zero_symmetric (util/rlwe.cpp:311-441). */
int nexus_seal_keygen_public(nexus_context *ctx, const uint64_t *seed, const uint64_t *d_sk, uint64_t *d_pk,
                             void *stream);

/* Relinearization key for s^2, d_key [n_moduli-1][2][n_moduli][N]; seeds
 * [n_moduli-1][8].
 * Replaces: KeyGenerator::create_relin_keys (native/src/seal/keygenerator.cpp:124-162)
 *   -> generate_one_kswitch_key (:303-336). */
int nexus_seal_keygen_relin(nexus_context *ctx, const uint64_t *seeds, const uint64_t *d_sk, uint64_t *d_key,
                            void *stream);

/* Galois key for X -> X^galois_elt, same layout and seeds.
 * Replaces: KeyGenerator::create_galois_keys (native/src/seal/keygenerator.cpp:164-223). */
int nexus_seal_keygen_galois(nexus_context *ctx, const uint64_t *seeds, const uint64_t *d_sk, uint32_t galois_elt,
                             uint64_t *d_key, void *stream);

/* Public-key encryption of the NTT-form plaintext d_pt [limbs][N] (NULL:
 * zero) into d_ct [2][limbs][N]: an encryption of zero one level up, divided
 * and rounded by that level's last prime.
 * Replaces: Encryptor::encrypt -> encrypt_zero_internal (native/src/seal/encryptor.cpp:88-174,
 *   176-237) -> encrypt_zero_asymmetric (util/rlwe.cpp:224-309). */
int nexus_seal_encrypt(nexus_context *ctx, const uint64_t *seed, const uint64_t *d_pk, const uint64_t *d_pt,
                       int limbs, uint64_t *d_ct, void *stream);

/* Secret-key encryption of d_pt (NULL: zero) into d_ct [2][limbs][N].
 * Replaces: Encryptor::encrypt_symmetric -> encrypt_zero_symmetric
 *   (native/src/seal/encryptor.cpp:176-237, util/rlwe.cpp:311-441). */
int nexus_seal_encrypt_symmetric(nexus_context *ctx, const uint64_t *seed, const uint64_t *d_sk,
                                 const uint64_t *d_pt, int limbs, uint64_t *d_ct, void *stream);

/* ------------------------------------------------------------------ */
/* CKKS encoding                                                        */
/* ------------------------------------------------------------------ */

/*
 * Encode nvals (<= N/2) complex slot values (re[i] + i*im[i]; im may be NULL)
 * at `scale` into the NTT-form plaintext d_out [limbs][N].  The FP64 special
 * FFT runs on the host and reproduces SEAL's rounding; the RNS forward NTT
 * runs on the GPU.  Returns after d_out is written.
 * Replaces: CKKSEncoder::encode(vector<complex<double>>, parms_id, scale, Plaintext&)
 *   -> encode_internal (native/src/seal/ckks.h:457-640); Phantom
 *   PhantomCKKSEncoder::encode (cuda/thirdparty/phantom-fhe/src/ckks.cu:89).
 */
int nexus_encode(nexus_context *ctx, const double *re, const double *im, size_t nvals, double scale, int limbs,
                 uint64_t *d_out, void *stream);

/*
 * Residues of round(value * scale) in each of the first `limbs` primes
 * (host array per_limb[limbs]).  In NTT form SEAL's scalar plaintext holds this
 * residue in every coefficient, so multiplying by it is a per-limb scalar
 * product (nexus_multiply_scalar).
 * Replaces: CKKSEncoder::encode(double, parms_id, scale, Plaintext&)
 *   (native/src/seal/ckks.cpp:75-205).
 */
int nexus_encode_scalar(nexus_context *ctx, double value, double scale, int limbs, uint64_t *per_limb);

/*
 * d_out [polys][limbs][N] = d_in * per_limb[l] mod q_l (host scalars < q_l).
 * Replaces: multiply_plain with a scalar-encoded plaintext
 *   (native/src/seal/evaluator.cpp:2336-2373 with a constant plaintext).
 */
int nexus_multiply_scalar(nexus_context *ctx, const uint64_t *d_in, int polys, int limbs, const uint64_t *per_limb,
                          uint64_t *d_out, void *stream);

/*
 * Decode the NTT-form plaintext d_pt [limbs][N] at `scale` into nvals slot
 * values (re, im host arrays; im may be NULL).  sparse_slots = 0 decodes all
 * N/2 slots; otherwise coefficients outside the sparse subring are zeroed as
 * in the bootstrapping fork of SEAL.
 * Replaces: CKKSEncoder::decode -> decode_internal (native/src/seal/ckks.h:640-760).
 */
int nexus_decode(nexus_context *ctx, const uint64_t *d_pt, int limbs, double scale, double *re, double *im,
                 size_t nvals, size_t sparse_slots, void *stream);

/* ------------------------------------------------------------------ */
/* NEXUS operators (src/ckks_evaluator.cpp, gelu.cpp, softmax.cpp,      */
/* layer_norm.cpp in the NEXUS tree) on the engine                      */
/* ------------------------------------------------------------------ */

typedef struct nexus_evaluator nexus_evaluator;
typedef struct nexus_ciphertext nexus_ciphertext;

/*
 * Evaluator with SEAL's semantics plus NEXUS's CKKSEvaluator at base scale
 * `scale`; d_relin_key (SEAL layout, caller-owned) may be NULL when no
 * multiplication is evaluated.  All work is enqueued on `stream`.
 * Replaces: CKKSEvaluator(SEALContext&, Encryptor&, Decryptor&, CKKSEncoder&,
 *   Evaluator&, double scale, RelinKeys&, GaloisKeys&) (src/ckks_evaluator.h:52-86)
 *   and nexus::CKKSEvaluator (cuda/src/ckks_evaluator.cuh:457-481).
 */
int nexus_evaluator_create(nexus_context *ctx, double scale, const uint64_t *d_relin_key, void *stream,
                           nexus_evaluator **out);
int nexus_evaluator_destroy(nexus_evaluator *ev);
/* Register the Galois key of one element (caller-owned, SEAL layout).
 * Replaces: the GaloisKeys& held by CKKSEvaluator (src/ckks_evaluator.h:42). */
int nexus_evaluator_add_galois_key(nexus_evaluator *ev, uint32_t galois_elt, const uint64_t *d_key);

/* Ciphertext objects owned by the engine ([size][limbs][N] on the device).
 * Replaces: seal::Ciphertext / PhantomCiphertext. */
int nexus_ciphertext_create(nexus_context *ctx, nexus_ciphertext **out);
int nexus_ciphertext_destroy(nexus_ciphertext *ct);
/* copy size x limbs x N words from host (from_host = 1) or device memory */
int nexus_ciphertext_load(nexus_ciphertext *ct, const uint64_t *src, int size, int limbs, double scale, int from_host,
                          void *stream);
int nexus_ciphertext_info(const nexus_ciphertext *ct, int *size, int *limbs, double *scale, uint64_t **d_data);
int nexus_ciphertext_store(const nexus_ciphertext *ct, uint64_t *dst, int to_host, void *stream);

/* GeLUEvaluator::gelu(x, res) (src/gelu.cpp:5-111); x is mod-switched in
 * place as in the original. */
int nexus_gelu(nexus_evaluator *ev, nexus_ciphertext *x, nexus_ciphertext *res);
/* SoftmaxEvaluator::softmax(x, res, len) (src/softmax.cpp:6-42); x is updated in place. */
int nexus_softmax(nexus_evaluator *ev, nexus_ciphertext *x, int len, nexus_ciphertext *res);
/* LNEvaluator::layer_norm(x, res, len) (src/layer_norm.cpp:6-33); x is updated in place. */
int nexus_layer_norm(nexus_evaluator *ev, nexus_ciphertext *x, int len, nexus_ciphertext *res);

/* CKKSEvaluator primitives (src/ckks_evaluator.cpp):
 *   NEXUS_OP_SGN_EVAL     sgn_eval(x, d_g = a1, d_f = a2, sgn_factor = f)   :181-212
 *   NEXUS_OP_EXP          exp(x)                                            :534-548
 *   NEXUS_OP_INVERSE      inverse(x, iter = a1)                             :487-509
 *   NEXUS_OP_INVERT_SQRT  invert_sqrt(x, d_newt = a1, d_gold = a2)          :480-485 */
enum { NEXUS_OP_SGN_EVAL = 0, NEXUS_OP_EXP = 1, NEXUS_OP_INVERSE = 2, NEXUS_OP_INVERT_SQRT = 3 };
int nexus_ckks_op(nexus_evaluator *ev, int op, const nexus_ciphertext *x, int a1, int a2, double f,
                  nexus_ciphertext *res);

/*
 * Rotate one ciphertext by several slot steps: res[i] receives the words
 * Evaluator::rotate_vector(x, steps[i]) gives (NAF decomposition included,
 * evaluator.cpp:2667-2722).  The steps that have their own Galois key share
 * one ModUp of x's c1 (hoisted rotations); when a coefficient of INTT(c1) is
 * zero, where sharing is not exact, the steps are switched on their own by a
 * fallback launch that the device itself enables.  Hoisting keeps, per Galois element, a copy of the key with
 * permuted rows (as large as the key) and a per-level correction.
 * No counterpart in the reference: SEAL rotates one step per call, and the
 * reference's BSGS transforms call rotate_vector once per baby step.
 */
int nexus_rotate_vector_many(nexus_evaluator *ev, const nexus_ciphertext *x, const int *steps, int count,
                             nexus_ciphertext *const *res);

/*
 * The lockstep form of nexus_rotate_vector_many: count ciphertexts of one
 * size, level and scale, each rotated by every step; res[s * count + b]
 * receives rotate_vector(cts[b], steps[s]), word for word the single form.
 * The decomposition is shared by the steps and done once for the batch; a
 * ciphertext whose INTT(c1) has a zero coefficient is recomputed by the
 * ordinary key switch inside the same stream (no host wait).  The BSGS
 * transforms of the lockstep bootstrap and of the encrypted layer run
 * through this path.
 */
int nexus_rotate_vector_many_batch(nexus_evaluator *ev, nexus_ciphertext *const *cts, int count, const int *steps,
                                   int n_steps, nexus_ciphertext *const *res);

/*
 * Hoisted rotations on (enable != 0, the default) or off for this evaluator
 * and every bootstrapper built on it.  Off, every rotation is switched on its
 * own and no permuted key copies are made; the output words are the same
 * either way.  When the copies cannot be allocated the evaluator also falls
 * back to one key switch per step.  No counterpart in the reference.
 */
int nexus_evaluator_set_hoisting(nexus_evaluator *ev, int enable);

/* ------------------------------------------------------------------ */
/* MatMul (src/matrix_mul.cpp in the NEXUS tree)                        */
/* ------------------------------------------------------------------ */

/* Coefficient packing of the MatMul's compressed operand: coefficient i of
 * the plaintext is round(values[i] * scale) (i < n <= N, the rest zero),
 * reduced into the first `limbs` primes and transformed to NTT form.
 * Replaces: the packing loop of MMEvaluator::enc_compress_ciphertext
 *   (src/matrix_mul.cpp:72-96, there with scale 1e10 and two primes). */
int nexus_encode_coefficients(nexus_context *ctx, const double *values, size_t n, double scale, int limbs,
                              uint64_t *d_out, void *stream);

/* The operators above on `count` ciphertexts in lockstep (one size, level
 * and scale): every step runs once over the whole batch, every key is read
 * once per batch, and res[b] receives the words the single form gives for
 * cts[b].  The inputs are left unchanged (the single forms of gelu, softmax
 * and layer_norm mod-switch or update their input in place, as NEXUS's do).
 * No counterpart in the reference. */
int nexus_gelu_batch(nexus_evaluator *ev, nexus_ciphertext *const *cts, int count, nexus_ciphertext *const *res);
int nexus_softmax_batch(nexus_evaluator *ev, nexus_ciphertext *const *cts, int count, int len,
                        nexus_ciphertext *const *res);
int nexus_layer_norm_batch(nexus_evaluator *ev, nexus_ciphertext *const *cts, int count, int len,
                           nexus_ciphertext *const *res);
int nexus_ckks_op_batch(nexus_evaluator *ev, int op, nexus_ciphertext *const *cts, int count, int a1, int a2,
                        double f, nexus_ciphertext *const *res);

/* MMEvaluator::multiply_power_of_x (src/matrix_mul.cpp:131-172): res = x * X^index. */
int nexus_mm_power_of_x(nexus_evaluator *ev, nexus_ciphertext *x, int index, nexus_ciphertext *res);

/* MMEvaluator::expand_ciphertext (src/matrix_mul.cpp:101-129) with the Galois
 * keys of the elements (N + 2^i) / 2^i registered on ev: the m leaves are
 * written to d_out [m][2][limbs][N]. */
int nexus_mm_expand(nexus_evaluator *ev, const nexus_ciphertext *x, uint32_t m, uint64_t *d_out);

/* MMEvaluator::matrix_mul (src/matrix_mul.cpp:174-246), generalised from
 * 768 x 64: the n_compressed ciphertexts hold a rows x cols matrix flattened
 * row-major in their coefficients; d_pts [cols][limbs][N] are NTT-form
 * plaintexts at pt_scale.  res[r] (rows handles, filled) = sum_k
 * leaf(r*cols + k) * pt_k with scale multiplied by `factor` (the expansion
 * multiplies by N), rescaled to one prime; bias (bias_len slot values, may
 * be NULL) is then encoded at the output level and scale and added to every
 * row.  Leaves are accumulated as they are produced and never all held in
 * memory. */
int nexus_matrix_mul(nexus_evaluator *ev, nexus_ciphertext *const *compressed, int n_compressed,
                     const uint64_t *d_pts, double pt_scale, int rows, int cols, double factor, const double *bias,
                     int bias_len, nexus_ciphertext *const *res);

/* ------------------------------------------------------------------------
 * Bootstrapping (src/bootstrapping/Bootstrapper.{h,cpp}, ModularReducer.cpp)
 * ------------------------------------------------------------------------ */
typedef struct nexus_bootstrapper nexus_bootstrapper;

/* Bootstrapper::Bootstrapper (Bootstrapper.h:52-69, Bootstrapper.cpp:3-26):
 * the evaluator's keys must hold the relinearisation key and the Galois keys
 * of nexus_bootstrapper_add_rot_steps. */
int nexus_bootstrapper_create(nexus_evaluator *ev, long loge, long logn, long logNh, long L, double final_scale,
                              long boundary_K, long sin_cos_deg, long scale_factor, long inverse_deg,
                              nexus_bootstrapper **out);
int nexus_bootstrapper_destroy(nexus_bootstrapper *bs);

/* Bootstrapper::prepare_mod_polynomial (Bootstrapper.cpp:1973-1977): the
 * EvalMod polynomial heap (Polynomial::generate_poly_heap,
 * common/Polynomial.cpp:168-214) as doubles.  node_len[i] is the number of
 * Chebyshev coefficients of heap node i (0 = absent) for the 2^(heap_m+1)-1
 * nodes; coeffs holds them back to back.  scale_inverse_coeff as in
 * ModularReducer.cpp:38-46. */
int nexus_bootstrapper_prepare_mod_polynomial(nexus_bootstrapper *bs, int heap_k, int heap_m, const int *node_len,
                                              const double *coeffs, double scale_inverse_coeff);

/* ModularReducer::generate_inverse_sine_polynomial (ModularReducer.cpp:38-47)
 * for inverse_deg > 1: the inverse-sine polynomial that EvalMod evaluates
 * after the unscaled double angles (:62-73).  power holds its deg + 1
 * power-basis coefficients (the direct forms of degree <= 3 read them,
 * common/Polynomial.cpp:257-325); above degree 3 its odd heap
 * (generate_poly_heap_odd, :207-210) follows in the layout of
 * nexus_bootstrapper_prepare_mod_polynomial.  deg must equal the
 * bootstrapper's inverse_deg; the cosine heap given to
 * prepare_mod_polynomial is then the unscaled one. */
int nexus_bootstrapper_set_inverse_polynomial(nexus_bootstrapper *bs, int deg, const double *power, int heap_k,
                                              int heap_m, const int *node_len, const double *coeffs);

/* Bootstrapper::addLeftRotKeys_Linear_to_vector_3 (Bootstrapper.cpp:89-184):
 * appends the missing rotation steps to steps[0..*count) (capacity entries). */
int nexus_bootstrapper_add_rot_steps(const nexus_bootstrapper *bs, int *steps, int *count, int capacity);

/* Bootstrapper::generate_LT_coefficient_3 (Bootstrapper.cpp:1967-1971). */
int nexus_bootstrapper_generate_lt(nexus_bootstrapper *bs);

/* The LT diagonals of genfftcoeff_3 / geninvfftcoeff_3
 * (Bootstrapper.cpp:1144-1954) for 2^logn slots, host-only: which = 0..2
 * fftcoeff1..3, 3..5 invfftcoeff1..3.  out = NULL queries *count diagonals
 * of *len complex values; otherwise out[count][len][2] (re, im), shorter
 * diagonals zero-padded.  No counterpart in the reference (the diagonals are
 * Bootstrapper members there). */
int nexus_lt_coefficients_3(int logn, int logNh, long boundary_K, int which, double *out, int *count, int *len);

/* Bootstrapper::bootstrap_3 (Bootstrapper.cpp:3489-3495): ct (one data
 * limb) is modulus-raised in place as in the reference; rtn receives the
 * refreshed ciphertext at scale final_scale. */
int nexus_bootstrap(nexus_bootstrapper *bs, nexus_ciphertext *ct, nexus_ciphertext *rtn);

/* bootstrap_3 of `count` ciphertexts in lockstep (one scale, one limb each):
 * every operation runs once over the whole batch and every key is read once
 * per batch.  rtn[b] receives the same words nexus_bootstrap gives for
 * cts[b]; the inputs are left unchanged.  No counterpart in the reference
 * (it bootstraps one ciphertext per call). */
int nexus_bootstrap_batch(nexus_bootstrapper *bs, nexus_ciphertext *const *cts, int count,
                          nexus_ciphertext *const *rtn);
/* The ciphertexts of a batch refreshed two per bootstrap, for real slot
 * values: cts[2i] and cts[2i+1] share one lockstep bootstrap_3 of
 * z = cts[2i] + X^(N/2) cts[2i+1] (X^(N/2) multiplies every slot by i) with
 * z's scale doubled, and come back as z + conj(z) and (conj(z) - z) X^(N/2)
 * (one conjugation per pair); an odd last one is refreshed alone.  Each
 * output decrypts to its input's values within an unpacked bootstrap's
 * error, at half the bootstraps; the words are those of that sequence, not
 * of bootstrap_3 on each ciphertext.  Same input rules as
 * nexus_bootstrap_batch.  No counterpart in the reference. */
int nexus_bootstrap_real_batch(nexus_bootstrapper *bs, nexus_ciphertext *const *cts, int count,
                               nexus_ciphertext *const *rtn);

/* The stages of bootstrap_full_3 (Bootstrapper.cpp:3224-3244), for
 * stage-wise checking: MODRAISE a in place (modraise_inplace :2937-2991);
 * COEFFTOSLOT a -> r1, r2 (coefftoslot_full_3 :2741-2757);
 * MODULAR_REDUCTION a -> r1 (ModularReducer::modular_reduction
 * ModularReducer.cpp:58-78); SLOTTOCOEFF a, b -> r1 (slottocoeff_full_3
 * :2759-2775); SET_INITIAL_SCALE from a's scale (bootstrap_3 :3490). */
#define NEXUS_BOOT_MODRAISE 0
#define NEXUS_BOOT_COEFFTOSLOT 1
#define NEXUS_BOOT_MODULAR_REDUCTION 2
#define NEXUS_BOOT_SLOTTOCOEFF 3
#define NEXUS_BOOT_SET_INITIAL_SCALE 4
int nexus_bootstrapper_stage(nexus_bootstrapper *bs, int stage, nexus_ciphertext *a, const nexus_ciphertext *b,
                             nexus_ciphertext *r1, nexus_ciphertext *r2);

/* The same stages run in lockstep over `count` ciphertexts of one size, level
 * and scale: a[k] (and b[k] for SLOTTOCOEFF) in, r1[k] / r2[k] out, each
 * receiving the words nexus_bootstrapper_stage gives for a[k] alone; MODRAISE
 * updates every a[k] in place and SET_INITIAL_SCALE takes the shared scale.
 * The lockstep form keeps its own initial scale (set it with this call before
 * a lockstep SLOTTOCOEFF).  No counterpart in the reference (it has no
 * lockstep form). */
int nexus_bootstrapper_stage_batch(nexus_bootstrapper *bs, int stage, nexus_ciphertext *const *a,
                                   const nexus_ciphertext *const *b, int count, nexus_ciphertext *const *r1,
                                   nexus_ciphertext *const *r2);

/* ArgmaxEvaluator::argmax (src/argmax.cpp:9-81) with the bootstrapper's
 * evaluator and keys: slots 0..len-1 of x -> the one-hot indicator of the
 * maximum (sgn(x - max) + 1), bootstrapping after every round.  x is updated
 * in place as in the reference; len a power of two. */
int nexus_argmax(nexus_bootstrapper *bs, nexus_ciphertext *x, int len, nexus_ciphertext *res);

/* nexus_argmax over `count` ciphertexts of one level and scale in lockstep:
 * res[k] receives the words nexus_argmax gives for x[k], and x[k] is updated
 * as nexus_argmax updates its input.  No counterpart in the reference. */
int nexus_argmax_batch(nexus_bootstrapper *bs, nexus_ciphertext *const *x, int count, int len,
                       nexus_ciphertext *const *res);

/* Number of encoded LT diagonals the bootstrapper keeps on the device. */
int nexus_bootstrapper_cached_plaintexts(const nexus_bootstrapper *bs, uint64_t *count);

/* ------------------------------------------------------------------------
 * Encrypted BERT encoder layer
 * ------------------------------------------------------------------------ */
/*
 * One BERT encoder layer over the bootstrapper's evaluator, keys and chain:
 * Q/K/V projections, multi-head attention (QK^T / sqrt(head_dim), softmax,
 * .V), output projection, residual + LayerNorm, W1 -> GELU -> W2, residual +
 * LayerNorm, bootstrapping (bootstrap_3) between the blocks.  The
 * nonlinearities are NEXUS's CKKSEvaluator::exp / ::inverse (the call
 * sequence of SoftmaxEvaluator::softmax, src/softmax.cpp:6-42),
 * ::invert_sqrt (LNEvaluator::layer_norm, src/layer_norm.cpp:6-33) and
 * GeLUEvaluator::gelu (src/gelu.cpp:5-111).  No counterpart in the
 * reference: its drivers (src/main.cpp:25-27) run one operator at a time and
 * it has no ciphertext x ciphertext product for attention.
 *
 * Packing: slot j*T + t of a ciphertext is feature block j, token slot t;
 * each of n_lanes lanes packs lane_requests[l] requests, request r as
 * requests[2r] = first token slot o and requests[2r+1] = tokens L, its
 * tokens at slots o + i and o + L + i (i < L).  Hidden activations use
 * ceil(hidden / (N/2/T)) ciphertexts, feature f in ciphertext f / (N/2/T),
 * block f % (N/2/T).  weights holds wq, wk, wv, wo [hidden][hidden], w1
 * [hidden][ffn], w2 [ffn][hidden] (row-major [in][out]) then bq, bk, bv, bo,
 * b1, b2.  Values are divided by boot_shrink before each bootstrap (and the
 * scale with them) so the refreshed message stays small.  The bootstrapper
 * must have its EvalMod polynomial and LT coefficients; its evaluator needs
 * the relinearization key, the bootstrapping keys and the Galois keys of
 * nexus_bert_layer_rotation_steps.
 */
typedef struct nexus_bert_layer nexus_bert_layer;
int nexus_bert_layer_create(nexus_bootstrapper *bs, int hidden, int heads, int head_dim, int ffn, int T,
                            int n_lanes, const int *lane_requests, const int *requests, double boot_shrink,
                            const double *weights, nexus_bert_layer **out);
int nexus_bert_layer_destroy(nexus_bert_layer *layer);
/* ciphertexts per lane of the hidden, head-layout and FFN activations, and
 * the plaintexts (encoded diagonals, biases, masks) kept on the device */
int nexus_bert_layer_info(const nexus_bert_layer *layer, int *n_lanes, int *n_hidden_cts, int *n_head_cts,
                          int *n_ffn_cts, uint64_t *cached_plaintexts);
/* the slot rotations the layer performs (steps = NULL only counts them) */
int nexus_bert_layer_rotation_steps(const nexus_bert_layer *layer, int *steps, int *count, int capacity);
/* out[l * n_hidden_cts + c] = the layer applied to x[l * n_hidden_cts + c]
 * (lane-major; x at 4 or more limbs, both token copies filled; the
 * outputs' first token copies hold the result); lockstep = 0
 * runs each lane on its own, one ciphertext at a time (the plain form),
 * lockstep = 1 runs every lane together and bootstraps and evaluates the
 * nonlinearities over all ciphertexts of a step at once, with the same words. */
int nexus_bert_layer_forward(nexus_bert_layer *layer, int lockstep, nexus_ciphertext *const *x,
                             nexus_ciphertext *const *out);
/* One stage of the layer on lane-major ciphertexts, for stage-wise checking:
 * PROJECT linear map `which` (0 Q, 1 K, 2 V, 3 output, 4 W1, 5 W2) plus its
 * bias, written on token slots [0, T/2) only when `which` also carries
 * NEXUS_BERT_LOWER_HALF; ATTENTION q, k, v (head layout, in that order) ->
 * the attention output; LAYER_NORM (which = 1: on folded ciphertexts, two
 * feature sets in the halves of each token block) and BOOTSTRAP return
 * their inputs transformed; FOLD maps count_in ciphertexts to
 * (count_in + 1) / 2 (2i and 2i+1 -> x_2i + rot(x_2i+1, -T/2)), UNFOLD maps
 * (count_out + 1) / 2 back to count_out (2i -> x_i, 2i+1 -> rot(x_i, T/2);
 * which = 1: also rebuilds every request's second token copy where it lies
 * in the upper half, one level down, as K is); see set_token_fold. */
#define NEXUS_BERT_PROJECT 0
#define NEXUS_BERT_ATTENTION 1
#define NEXUS_BERT_LAYER_NORM 2
#define NEXUS_BERT_BOOTSTRAP 3
#define NEXUS_BERT_FOLD 4
#define NEXUS_BERT_UNFOLD 5
#define NEXUS_BERT_LOWER_HALF 16
int nexus_bert_layer_stage(nexus_bert_layer *layer, int lockstep, int stage, int which, nexus_ciphertext *const *in,
                           int count_in, nexus_ciphertext *const *out, int count_out);
/* With timing on, forward records a CUDA event after each of its blocks;
 * stage_times returns the device time of each block of the last forward
 * (lockstep form, or lane `lane` of the single form) in ms[], their names in
 * `names` separated by newlines; ms = NULL only counts them. */
int nexus_bert_layer_set_timing(nexus_bert_layer *layer, int enable);
/* With boot_pack on, each bootstrap of the layer refreshes two ciphertexts:
 * z = c0 + X^(N/2) c1 holds c0 + i c1, its scale doubled, and after
 * bootstrap_3 c0 = z + conj(z), c1 = (conj(z) - z) X^(N/2) (a trailing odd
 * ciphertext is refreshed alone).  Half the bootstraps, one conjugation per
 * pair, the same error per output.  On by default; no counterpart in the
 * reference (NEXUS has no layer). */
int nexus_bert_layer_set_boot_pack(nexus_bert_layer *layer, int enable);
/* With token_fold on, and when every request's tokens lie in token slots
 * [0, T/2), two ciphertexts share one, the second's tokens in the upper half
 * of every token block: Q and K through their bootstrap (K's second token
 * copies rebuilt by masked rotations when unfolded), the attention's scores
 * of offsets 2p and 2p+1 through their exp and the probabilities, and the
 * hidden and FFN activations from the output projection to the layer's
 * output (both residual bootstraps and LayerNorms, the FFN's bootstraps and
 * GELU).  The maps feeding a fold (Q, K, output, W1, W2) and the residual
 * input write the lower half only; a fold is one rotation of -T/2, an
 * unfold gives ciphertext 2i+1 as the folded one rotated by T/2 (Q at the
 * attention's level), and LayerNorm adds the two halves' feature sums with
 * one more rotation.  30 bootstraps per BERT-base layer instead of 54, half
 * the exps, GELUs and LayerNorm products; the rotation steps include +-T/2
 * and the copy shifts (-L for every request length L whose second copy
 * reaches the upper half) whenever the fold applies.  On by default; no
 * counterpart in the reference (NEXUS has no layer). */
int nexus_bert_layer_set_token_fold(nexus_bert_layer *layer, int enable);
int nexus_bert_layer_stage_times(nexus_bert_layer *layer, int lockstep, int lane, double *ms, char *names,
                                 size_t names_capacity, int *count, int capacity);

/* ------------------------------------------------------------------------
 * SEAL byte format of a CKKS ciphertext (host-side, compr_mode_type::none)
 * ------------------------------------------------------------------------ */

/* Ciphertext::save (native/src/seal/ciphertext.cpp:190-248 with the
 * SEALHeader of serialization.h:60-93): words [size][limbs][2^log_n] as SEAL
 * stores them, the caller's parms_id (4 words, the SEALContext's id of the
 * ciphertext's level).  out = NULL only reports the byte count in *written. */
int nexus_seal_ciphertext_save(const uint64_t *words, int size, int limbs, int log_n, double scale,
                               const uint64_t *parms_id, int is_ntt_form, uint8_t *out, size_t capacity,
                               size_t *written);

/* Ciphertext::load (ciphertext.cpp:249-330), structural checks only (the
 * caller validates parms_id against its context): words = NULL only reports
 * the shape. */
int nexus_seal_ciphertext_load(const uint8_t *bytes, size_t len, uint64_t *words, size_t capacity_words, int *size,
                               int *limbs, int *log_n, double *scale, uint64_t *parms_id, int *is_ntt_form);

/* ------------------------------------------------------------------------
 * CUDA-graph capture of engine calls
 * ------------------------------------------------------------------------ */

/*
 * Record the engine calls a thread makes on `stream` (the stream the
 * evaluator was created on; the legacy default stream cannot be captured)
 * between begin and end, and replay them with one nexus_graph_launch.  The
 * calls' host-side work (levels, scales, output sizes) happens once, while
 * capturing; a launch repeats their device work on the same handles, so the
 * caller reloads the captured inputs (nexus_ciphertext_load into the same
 * handles, same size and level) and reads the captured outputs.  Run the
 * calls once before capturing: a call that must wait on the host (an encode
 * of a new vector constant, a cache built for the first time) invalidates
 * the capture, and end refuses a graph that frees device memory allocated
 * before the capture (a buffer that grew inside it), since every launch
 * would free it again; the handles such a refused capture touched are not
 * used again.  An output handle first sized inside the capture keeps a graph
 * allocation that stays valid, at one address, from launch to launch.
 * Launches of one graph must not overlap.  Between launches a captured
 * handle is only reloaded (same size and level): a direct call that gives it
 * a new buffer (an in-place operation outside the graph, a load of a larger
 * size) leaves the graph pointing at freed memory, so keep separate handles
 * for direct calls.  nexus_graph_info returns the graph's node, kernel-node
 * and allocation-node counts.
 * No counterpart in the reference: NEXUS's CUDA path launches every Phantom
 * kernel on its own and synchronises its stream after rotations and at the
 * end of bootstrap_3 (cuda/src/bootstrapping/Bootstrapper.cu:3358-3370).
 */
typedef struct nexus_graph nexus_graph;
int nexus_graph_capture_begin(void *stream);
int nexus_graph_capture_end(void *stream, nexus_graph **out);
int nexus_graph_launch(const nexus_graph *graph, void *stream);
int nexus_graph_info(const nexus_graph *graph, size_t *nodes, size_t *kernel_nodes, size_t *alloc_nodes);
int nexus_graph_destroy(nexus_graph *graph);

#ifdef __cplusplus
}
#endif

#endif /* NEXUS_GB300_H */
