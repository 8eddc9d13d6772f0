// Internal CKKS operations on device arrays in SEAL's layout.  A ciphertext
// with `limbs` limbs uses data primes 0..limbs-1; polynomials are [limbs][N],
// ciphertexts [size][limbs][N], key-switching keys [K-1][2][K][N] with
// K = ctx.k (every prime of the key level).  All functions only enqueue work
// on `s`; multi-kernel operations share the context's scratch arena.
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "context.h"

namespace nexus {

// element-wise, over [polys][limbs][N]
void poly_add(const Context &c, const uint64_t *a, const uint64_t *b, int polys, int limbs, uint64_t *out,
              cudaStream_t s);
void poly_sub(const Context &c, const uint64_t *a, const uint64_t *b, int polys, int limbs, uint64_t *out,
              cudaStream_t s);
void poly_negate(const Context &c, const uint64_t *a, int polys, int limbs, uint64_t *out, cudaStream_t s);
// out[p] = ct[p] * pt for every polynomial p of ct (pt is one [limbs][N] polynomial)
void poly_mul_plain(const Context &c, const uint64_t *ct, int polys, int limbs, const uint64_t *pt, uint64_t *out,
                    cudaStream_t s);
// out[p] = sum_j cts[j][p] * pts[j] for both polynomials p of `count` (<= 16)
// two-polynomial ciphertexts; 128-bit exact accumulation, one reduction
// (batch > 1: each cts[j] and out hold `batch` ciphertexts back to back)
void poly_mac_plain(const Context &c, const uint64_t *const *cts, const uint64_t *const *pts, int count, int limbs,
                    uint64_t *out, cudaStream_t s, int batch = 1);
// out[p] = ct[p] + pt (pt broadcast); used for add_plain
void poly_add_plain(const Context &c, const uint64_t *ct, int polys, int limbs, const uint64_t *pt, int sub,
                    uint64_t *out, cudaStream_t s);
// out[p][l] = ct[p][l] * scalar[l] mod q_l (per-limb scalar from host)
void poly_mul_scalar(const Context &c, const uint64_t *ct, int polys, int limbs, const uint64_t *scalars,
                     uint64_t *out, cudaStream_t s);

// out = in (+|-) per-limb scalar, one polynomial [limbs][N] (add_plain of a scalar plaintext);
// batch > 1: `batch` such polynomials every stride_words words (component 0 of a batch)
void poly_add_scalar(const Context &c, const uint64_t *in, int limbs, const uint64_t *scalars, int sub, uint64_t *out,
                     cudaStream_t s, int batch = 1, size_t stride_words = 0);

// ckks_multiply / ckks_square tensor: out3 = (a0 b0, a0 b1 + a1 b0, a1 b1), over
// `batch` pairs back to back
void tensor(const Context &c, const uint64_t *a, const uint64_t *b, int limbs, uint64_t *out3, cudaStream_t s,
            int batch = 1);

// divide_and_round_q_last_ntt over every polynomial: [size][limbs] -> [size][limbs-1]
void rescale(const Context &c, const uint64_t *in, int size, int limbs, uint64_t *out, cudaStream_t s);

// NTT-domain automorphism of [polys][limbs][N]
void galois_permute(Context &c, const uint64_t *in, int polys, int limbs, uint32_t elt, uint64_t *out,
                    cudaStream_t s);

// rescale of in * c for a per-limb scalar c (host residues, c[l] < q_l):
// the words of poly_mul_scalar followed by rescale, in one pass fewer;
// accumulate: out += that (mod q) instead of out = it
void rescale_scaled(const Context &c, const uint64_t *in, int size, int limbs, const uint64_t *scalars,
                    uint64_t *out, cudaStream_t s, bool accumulate = false);

// switch_key_inplace: ct[2][limbs] += key-switch(target[limbs])
void switch_key(Context &c, uint64_t *ct, int limbs, const uint64_t *target, const uint64_t *key, cudaStream_t s);

// the same for `batch` ciphertexts ct[batch][2][limbs] and targets[batch][limbs]
// sharing one key (the key is read once per launch, not once per ciphertext);
// target_pitch: words between consecutive targets (0 = limbs * N)
void switch_key_batch(Context &c, uint64_t *ct, int batch, int limbs, const uint64_t *target, const uint64_t *key,
                      cudaStream_t s, size_t target_pitch = 0);

// Times a batched key switch of `batch` ciphertexts at `limbs` limbs on
// random data for every candidate Context::Tuning, keeps the fastest in c.tune
// and returns its milliseconds per call (autotune.cu).
double autotune_keyswitch(Context &c, int limbs, int batch, cudaStream_t s, int reps = 3);

// stages of the batched key switch, for callers that fuse their own epilogue:
// ModUp + inner products (t [B][l] NTT-form targets, overwritten; D scratch
// B*l*(l+1) limbs; P [B][2][l+1] out), then the ModDown rounding terms
// (T [B][2][l] out; last scratch 2B limbs).  The result of the key switch is
// (P[b][k][i] - T[b][k][i]) * p^{-1} mod q_i.
void ks_modup_inner(Context &c, uint64_t *t, int B, int l, const uint64_t *key, uint64_t *D, uint64_t *P,
                    cudaStream_t s);
void ks_moddown_terms(Context &c, const uint64_t *P, int B, int l, uint64_t *T, uint64_t *last, cudaStream_t s);

// Hoisted rotations (keyswitch.cu): one ModUp of the c1 polynomials of B
// ciphertexts at l limbs (c1 at c1 + b * c1_pitch) shared by several Galois
// elements.  hoist_decompose fills D [B][l][l+1][N] and t [B][l][N] (the
// INTT of c1) and sets d_flags[b] (B device ints) when a coefficient of
// ciphertext b's INTT(c1) is zero, where the shared decomposition is not
// exact.  Per element: perm_key (hoist_permute_key, the key with every row
// scattered by the element's NTT permutation) and corr [2][l+1][N]
// (hoist_correction from the key and M = hoist_galois_mask_ntt [K][N]) are
// reusable across calls; hoist_rotate writes out [B][2][l][N] (ct at
// ct + b * ct_pitch, 0 = 2 * l * N), and once every element of the group is
// written, hoist_fix rewrites the flagged ciphertexts' outputs by the
// ordinary key switch (one cooperative launch; nothing when no flag is set).
// Together they give the words apply_galois gives, with no host wait.
struct HoistRotation {
    uint32_t elt;
    const uint64_t *key;   // the element's Galois key as generated
    uint64_t *out;         // [B][2][l][N], written by hoist_rotate
};
void hoist_decompose(Context &c, const uint64_t *c1, size_t c1_pitch, int B, int l, uint64_t *t, uint64_t *D,
                     int *d_flags, cudaStream_t s);
void hoist_fix(Context &c, const uint64_t *t, const uint64_t *ct, size_t ct_pitch, const int *d_flags, int B, int l,
               const std::vector<HoistRotation> &rots, cudaStream_t s);
void hoist_galois_mask_ntt(Context &c, uint32_t elt, uint64_t *M, cudaStream_t s);
void hoist_permute_key(Context &c, const uint64_t *key, uint32_t elt, uint64_t *out, cudaStream_t s);
void hoist_correction(Context &c, const uint64_t *key, const uint64_t *M, int l, uint64_t *out, cudaStream_t s);
void hoist_rotate(Context &c, const uint64_t *D, int B, int l, uint32_t elt, const uint64_t *perm_key,
                  const uint64_t *corr, const uint64_t *ct, size_t ct_pitch, uint64_t *out, cudaStream_t s);

// relinearize B size-3 ciphertexts ct3 [B][3][l][N] into out2 [B][2][l][N]
// (no overlap); the ModDown's finishing kernel adds c0 and c1 from ct3
void relinearize_batch(Context &c, const uint64_t *ct3, int B, int limbs, const uint64_t *key, uint64_t *out2,
                       cudaStream_t s);

// relinearize a size-3 ciphertext into out2 (may alias ct3)
void relinearize(Context &c, const uint64_t *ct3, int limbs, const uint64_t *key, uint64_t *out2, cudaStream_t s);

// apply_galois_inplace: permute both polynomials, key-switch the second
// (out must not overlap ct)
void apply_galois(Context &c, const uint64_t *ct, int limbs, uint32_t elt, const uint64_t *key, uint64_t *out,
                  cudaStream_t s);
// the same for B ciphertexts ct/out [B][2][limbs][N] under one key: c1 is
// permuted straight into the key-switch targets and the ModDown's finishing
// kernel adds the permuted c0
void apply_galois_batch(Context &c, const uint64_t *ct, int B, int limbs, uint32_t elt, const uint64_t *key,
                        uint64_t *out, cudaStream_t s);

// key generation / symmetric encryption / decryption (sampling.cu)
void keygen_secret(Context &c, uint64_t seed, int hamming_weight, uint64_t *sk, cudaStream_t s);
void keygen_kswitch(Context &c, const uint64_t *sk, const uint64_t *new_key, uint64_t seed, uint64_t *key,
                    cudaStream_t s);
void keygen_relin(Context &c, const uint64_t *sk, uint64_t seed, uint64_t *key, cudaStream_t s);
void keygen_galois(Context &c, const uint64_t *sk, uint32_t elt, uint64_t seed, uint64_t *key, cudaStream_t s);
void encrypt_symmetric(Context &c, const uint64_t *sk, const uint64_t *m, int limbs, uint64_t seed, uint64_t *ct,
                       cudaStream_t s);
void decrypt(Context &c, const uint64_t *sk, const uint64_t *ct, int size, int limbs, uint64_t *m, cudaStream_t s);

// the same with SEAL's randomness (sampling.cu, seal_prng.cpp): each seed is
// 8 words, the seed of one Blake2xbPRNG; kswitch keys take K-1 seeds (one per
// digit, in order).  These return after the device work is done.
void seal_keygen_secret(Context &c, const uint64_t seed[8], int hamming_weight, uint64_t *sk, cudaStream_t s);
void seal_encrypt_zero_symmetric(Context &c, const uint64_t seed[8], const uint64_t *sk, const uint64_t *m,
                                 int limbs, uint64_t *ct, cudaStream_t s);
void seal_keygen_kswitch(Context &c, const uint64_t *seeds, const uint64_t *sk, const uint64_t *new_key,
                         uint64_t *key, cudaStream_t s);
void seal_keygen_relin(Context &c, const uint64_t *seeds, const uint64_t *sk, uint64_t *key, cudaStream_t s);
void seal_keygen_galois(Context &c, const uint64_t *seeds, const uint64_t *sk, uint32_t elt, uint64_t *key,
                        cudaStream_t s);
void seal_encrypt_asymmetric(Context &c, const uint64_t seed[8], const uint64_t *pk, const uint64_t *m, int limbs,
                             uint64_t *ct, cudaStream_t s);

}  // namespace nexus
