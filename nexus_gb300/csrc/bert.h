// An encrypted BERT encoder layer composed from NEXUS's operators.
//
// The NEXUS tree has no layer driver (its src/main.cpp runs one operator at a
// time) and no ciphertext x ciphertext product for attention; this file
// defines both.  One layer: Q/K/V projections, attention (QK^T / sqrt(d_h),
// softmax, .V), output projection, residual + LayerNorm, FFN (W1, GELU, W2),
// residual + LayerNorm, with bootstraps (Bootstrapper::bootstrap_3) between
// the blocks (Q and K are refreshed; V is projected from the input two levels
// higher, at the level the attention uses it, and is not).  The nonlinearities are NEXUS's: CKKSEvaluator::exp and
// ::inverse inside the softmax (src/softmax.cpp:6-42 call sequence, with the
// row sum taken over diagonals, below), CKKSEvaluator::invert_sqrt inside the
// LayerNorm (src/layer_norm.cpp:6-33, the feature sum taken over blocks), and
// GeLUEvaluator::gelu (src/gelu.cpp:5-111).
//
// Packing.  A ciphertext's S = N/2 slots form NB = S/T blocks of T token
// slots; block j of a ciphertext holds one feature for every token slot.  A
// lane is a set of requests sharing the token slots: request r occupies
// [o_r, o_r + 2 L_r), its tokens at o_r + i and again at o_r + L_r + i (the
// copy lets a rotation by delta < L_r read token (i + delta) mod L_r).
//  * std layout (hidden and FFN activations): feature f in ciphertext f / NB,
//    block f % NB;
//  * head layout (Q, K, V and the attention output): feature h*d_h + k in
//    ciphertext k / KB, block (k % KB) * H2 + h, with H2 the heads rounded up
//    to a power of two and KB = NB / H2, so the sum over k of a head is a sum
//    of ciphertexts plus log2(KB) rotations.
// Every ciphertext op but the attention rotations acts on each token slot on
// its own, so requests never mix.
//
// Linear layers are block-diagonal linear transforms: y_b = sum_a sum_d
// diag(a,b,d) * rot(x_a, d T), baby-step giant-step over the block offset d
// (the baby steps of one input share one ModUp); diag(a,b,d) holds
// W[f_in(a, j + d)][f_out(b, j)] on every token slot of block j.
//
// Attention, per lane, in the diagonal domain: S_delta[i] = Q[i] . K[i + delta]
// (delta < L_max), computed baby-step giant-step over delta
// (S_{G g + b} = rot(fold(sum_c rot(Q_c, -G g) * rot(K_c, b)), G g)), the
// softmax row sum over j becomes the sum over delta, and
// O_c = sum_g rot(sum_b rot(P_{G g + b}, -G g) * rot(V_c, b), G g).
// Pairs with delta >= L_r are masked to -128 before NEXUS's exp, which
// (1 + x/128)^128 maps to 0.
//
// Every value about to be bootstrapped may first be scaled down by
// boot_shrink (folded into the preceding linear map or constant product) and
// its scale divided by the same factor, so the refreshed ciphertext holds the
// value itself while the bootstrap's EvalMod sees a smaller message.  The
// bootstrap's own error grows with the factor (about 2e-4 times it at
// N = 2^16), so it is 1 by default; the softmax row sums, constant over a
// request's token slots (their message concentrates in few coefficients,
// which leave EvalMod's intervals sooner), take rowsum_shrink = 2.
//
// With boot_pack, two ciphertexts share one bootstrap.  The values are real,
// and the full-slot bootstrap refreshes complex slots: z = c0 + X^(N/2) c1
// holds c0 + i c1 (X^(N/2) multiplies every slot by i, exactly, at no
// level), its scale is doubled so that the refreshed z holds (c0 + i c1) / 2,
// and c0 = z + conj(z), c1 = (conj(z) - z) X^(N/2) afterwards (one
// conjugation).  The words EvalMod sees are the two messages' sum, and the
// error of each output is that of an unpacked bootstrap.
//
// With token_fold, two ciphertexts travel as one wherever the upper half of
// the token block carries nothing needed.  Every op but the linear maps'
// block rotations acts on one token slot; only the first token copies of Q
// are read (the scores' mask zeroes every other slot), and past the
// attention only the first copies matter at all.  So when every request's
// tokens lie in the lower half of the token block ([0, T/2)), a map feeding
// a fold writes only that half (its diagonals and bias are zero on the upper
// half; the residual input is masked in the constant product it already
// takes), and ciphertexts 2i and 2i+1 become one: y_2i + rot(y_2i+1, -T/2)
// holds the second's tokens in the upper half of every block.  Unfolding
// gives ciphertext 2i as the folded one itself and 2i+1 as its rotation by
// T/2; each token slot of the lower half then holds the right feature, and
// the upper half, never read for a first copy, holds other tokens' values of
// the same magnitude.  Folded: Q and K through their bootstrap (K, read at
// both token copies, is unfolded with the copies that reach the upper half
// rebuilt from its tokens by masked rotations, one level); the attention's
// scores of offsets 2p and 2p+1 through their exp and the probabilities
// (P is read at the first copies only; each half's row sum takes the other
// half of its own block); and the hidden and FFN activations from the
// output projection to the layer's output (LayerNorm adds the two halves'
// feature sums with one more rotation).
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "batch.h"
#include "bootstrap.h"
#include "ckks.h"
#include "nexus_ops.h"

namespace nexus {

// the level the V projection reads its input at: its output (one level
// lower) is the level the attention's P.V products take V at
constexpr int kVInLimbs = 4;
// the level the attention takes Q and K at (scores 1, mask 1, exp 8, P 1,
// P.V 1, above the output projection's 2 limbs)
constexpr int kQKLimbs = 14;

struct BertShape {
    int hidden = 768, heads = 12, head_dim = 64, ffn = 3072;
    int T = 256;  // token slots per feature block
    // per lane, each request as (first token slot, tokens)
    std::vector<std::vector<std::pair<int, int>>> lanes;
    double boot_shrink = 1.0;
    // the softmax row sums, constant over a request's token slots (their
    // message piles onto few coefficients), are divided by this instead
    double rowsum_shrink = 2.0;
    // refresh two ciphertexts with one bootstrap (c0 + i c1, separated by a
    // conjugation afterwards)
    bool boot_pack = true;
    // fold two Q, and two FFN hidden, ciphertexts into one through their
    // bootstraps (the halves of each token block) when the requests allow
    // it (fold_ok)
    bool token_fold = true;

    // derived by derive()
    int S = 0, NB = 0, H2 = 0, KB = 0, n_head = 0, n_hid = 0, n_ffn = 0, Lmax = 0, G = 0, Glt = 0;
    // every request's tokens in [0, T/2)
    bool fold_ok = false;
    // the distinct lengths of the requests whose second token copy reaches
    // the upper half of the block (o + 2L > T/2): the shifts that rebuild it
    // when K is unfolded
    std::vector<int> copy_shifts;
    void derive(size_t slots);
    bool folding() const { return token_fold && fold_ok; }
    // every rotation step the layer uses (the bootstrapper's are separate)
    std::vector<int> rotation_steps() const;
};

// row-major [in][out] matrices and biases
struct BertWeights {
    std::vector<double> wq, wk, wv, wo, w1, w2;
    std::vector<double> bq, bk, bv, bo, b1, b2;
};

// encoded diagonals, biases and softmax masks, shared by the single-lane and
// lockstep forms of one layer (the words depend only on level and scale)
struct BertPlaintexts {
    using DKey = std::tuple<int, int, int, int, int, uint64_t>;
    std::map<DKey, Plaintext> diag;
    std::map<std::tuple<int, int, int, uint64_t, int>, Plaintext> mask;
    std::map<std::tuple<int, int, int, uint64_t>, Plaintext> bias;
    // a value on the lower or upper half of every token block:
    // (value bits, limbs, scale bits, upper)
    std::map<std::tuple<uint64_t, int, uint64_t, int>, Plaintext> half;
    size_t count() const { return diag.size() + mask.size() + bias.size() + half.size(); }
};

// one layer over ciphertexts that each hold one lane (Evaluator, Ciphertext)
// or every lane in lockstep (BatchEvaluator, CtBatch); `lanes` lists the lane
// of each batch element
template <class EV, class CT>
class BertLayerT {
public:
    BertLayerT(EV &ev, BootstrapperT<EV, CT> &bs, const BertShape &shape, const BertWeights &w,
               std::vector<int> lanes, std::shared_ptr<BertPlaintexts> plain = nullptr);
    // x: n_hid ciphertexts in the std layout (tokens and their copies) at 2
    // or more limbs and at the bootstrapper's final scale; out: n_hid
    // ciphertexts (first copies valid)
    void forward(const std::vector<CT> &x, std::vector<CT> &out);

    // the stages of forward(), public for tests and profiling
    // linear map + bias; lower_half: written on token slots [0, T/2) only
    void project(const std::vector<CT> &x, int which, std::vector<CT> &y, bool lower_half = false);
    void attention(std::vector<CT> &q, std::vector<CT> &k, std::vector<CT> &v, std::vector<CT> &o);
    // folded: x holds two feature sets per ciphertext (the block halves)
    void layer_norm(std::vector<CT> &x, bool folded = false);
    void bootstrap_all(std::vector<CT> &cts);
    // ciphertexts 2i, 2i+1 (lower-half layout) -> one; and back to `count`
    void fold_halves(std::vector<CT> &x);
    void unfold_halves(std::vector<CT> &x, int count);
    // unfold_halves with every request's second token copy rebuilt from its
    // tokens (masks per lane, one rescale): for K, which the attention reads
    // at both copies
    void unfold_copies(std::vector<CT> &x, int count);

    ~BertLayerT();
    BertLayerT(const BertLayerT &) = delete;
    BertLayerT &operator=(const BertLayerT &) = delete;

    // when set, forward() records a CUDA event after each of its blocks;
    // stage_times() then gives each block's device time (ms) in order
    bool timing = false;
    std::vector<std::pair<std::string, double>> stage_times();

    enum { LT_Q = 0, LT_K, LT_V, LT_O, LT_1, LT_2, LT_COUNT };
    double delta() const { return delta_; }
    size_t cached_plaintexts() const { return pt_->count(); }
    const BertShape &shape() const { return sh_; }
    void set_boot_pack(bool on) { sh_.boot_pack = on; }
    void set_token_fold(bool on) { sh_.token_fold = on; }

private:
    int in_count(int which) const;
    int out_count(int which) const;
    int in_features(int which) const;
    int out_features(int which) const;
    const std::vector<double> &weights(int which) const;
    const std::vector<double> &bias(int which) const;
    // feature index at (ciphertext, block) of the input / output, or -1
    int in_feature(int which, int ct, int block) const;
    int out_feature(int which, int ct, int block) const;
    bool diag_nonzero(int which, int a, int b, int d) const;
    std::vector<double> diag_vector(int which, int a, int b, int d, int pre_rotate_blocks, bool lower_half) const;
    const Plaintext &diag(int which, int a, int b, int d, int limbs, double scale, bool lower_half);
    void encode_diagonals(int which, int limbs, double scale, bool lower_half);
    const Plaintext &bias_plain(int which, int ct, int limbs, double scale, bool lower_half);
    void masks(int delta, int kind, int limbs, double scale, std::vector<const Plaintext *> &out);
    // the -128 masks of two offsets folded in one ciphertext (offset 2 pair in
    // the lower half, 2 pair + 1 in the upper), per lane element
    void fold_masks(int pair, int limbs, double scale, std::vector<const Plaintext *> &out);
    // `value` on the lower (or upper) half of every token block, 0 elsewhere
    const Plaintext &half_plain(double value, bool upper, int limbs, double scale);
    // per lane: the lower half of the block (shift 0), or the tokens whose
    // copy lies `shift` slots on in the upper half; encoded at the scale of
    // the prime the rescale drops
    void copy_masks(int shift, int limbs, std::vector<const Plaintext *> &out);
    void shrink_for_bootstrap(std::vector<CT> &cts, bool lower_half = false);
    void begin_marks();
    void mark(const char *name);
    void exact_scale_const(CT &ct, double value, double target_scale, bool lower_half = false);
    Evaluator &base_evaluator();

    EV *ev_;
    BootstrapperT<EV, CT> *bs_;
    CKKSEvaluatorT<EV, CT> ck_;
    BertShape sh_;
    BertWeights w_;
    std::vector<int> lanes_;
    double delta_;
    std::shared_ptr<BertPlaintexts> pt_;
    std::vector<std::pair<std::string, cudaEvent_t>> marks_;
};

using BertLayer = BertLayerT<Evaluator, Ciphertext>;
using BatchBertLayer = BertLayerT<BatchEvaluator, CtBatch>;

}  // namespace nexus
