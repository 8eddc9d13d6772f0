// Encrypted BERT encoder layer (see bert.h for the packing and the method).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <thread>
#include <type_traits>

#include "bert.h"
#include "ops.h"

namespace nexus {

namespace {

int ceil_div(int a, int b) { return (a + b - 1) / b; }

int pow2_ceil(int v)
{
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

uint64_t bits_of(double d)
{
    uint64_t b;
    std::memcpy(&b, &d, 8);
    return b;
}

// apply f to every ciphertext of `cts`: one by one for the single form, as
// lockstep batches of at most `chunk` ciphertexts for the batched form
template <class F>
void each(Evaluator &, std::vector<Ciphertext *> &cts, int, F &&f)
{
    for (auto *c : cts) f(*c);
}

template <class F>
void each(BatchEvaluator &ev, std::vector<CtBatch *> &cts, int chunk, F &&f)
{
    if (cts.empty()) return;
    Context &c = ev.context();
    cudaStream_t s = ev.stream();
    size_t i = 0;
    while (i < cts.size()) {
        size_t j = i, elems = 0;
        while (j < cts.size() && (elems == 0 || (int)(elems + cts[j]->batch()) <= chunk)) elems += cts[j++]->batch();
        const CtBatch &first = *cts[i];
        CtBatch all;
        all.resize(c, (int)elems, first.size(), first.limbs(), s);
        all.scale() = first.scale();
        size_t off = 0;
        for (size_t k = i; k < j; ++k) {
            const CtBatch &x = *cts[k];
            if (x.size() != first.size() || x.limbs() != first.limbs() || x.scale() != first.scale())
                throw std::invalid_argument("lockstep group: ciphertexts differ in size, level or scale");
            cudaMemcpyAsync(all.ct((int)off), x.data(), (size_t)x.batch() * x.words_per_ct() * 8,
                            cudaMemcpyDeviceToDevice, s);
            off += x.batch();
        }
        f(all);
        off = 0;
        for (size_t k = i; k < j; ++k) {
            CtBatch &x = *cts[k];
            const int b = x.batch();
            x.resize(c, b, all.size(), all.limbs(), s);
            x.scale() = all.scale();
            cudaMemcpyAsync(x.data(), all.ct((int)off), (size_t)b * all.words_per_ct() * 8, cudaMemcpyDeviceToDevice,
                            s);
            off += b;
        }
        i = j;
    }
}

// per-element plaintext product / sum: lane b of the batch uses pts[b]
void mul_plain_each(Evaluator &ev, Ciphertext &ct, const std::vector<const Plaintext *> &pts)
{
    ev.multiply_plain_inplace(ct, *pts[0]);
}

void mul_plain_each(BatchEvaluator &ev, CtBatch &ct, const std::vector<const Plaintext *> &pts)
{
    Context &c = ev.context();
    const double scale = ct.scale() * pts[0]->scale();
    for (int b = 0; b < ct.batch(); ++b) {
        const Plaintext &p = *pts[b];
        if (p.limbs() != ct.limbs() || p.is_scalar() || p.scale() != pts[0]->scale())
            throw std::invalid_argument("per-lane plaintexts differ in level or scale");
        poly_mul_plain(c, ct.ct(b), ct.size(), ct.limbs(), p.data(), ct.ct(b), ev.stream());
    }
    ev.base().check_scale(scale, ct.limbs());
    ct.scale() = scale;
}

void add_plain_each(Evaluator &ev, Ciphertext &ct, const std::vector<const Plaintext *> &pts)
{
    ev.add_plain_inplace(ct, *pts[0]);
}

void add_plain_each(BatchEvaluator &ev, CtBatch &ct, const std::vector<const Plaintext *> &pts)
{
    Context &c = ev.context();
    for (int b = 0; b < ct.batch(); ++b) {
        const Plaintext &p = *pts[b];
        if (p.limbs() != ct.limbs() || p.is_scalar() || !are_close(ct.scale(), p.scale()))
            throw std::invalid_argument("per-lane plaintexts differ in level or scale");
        poly_add_plain(c, ct.ct(b), 1, ct.limbs(), p.data(), 0, ct.ct(b), ev.stream());
    }
}

int batch_of(const Ciphertext &) { return 1; }
int batch_of(const CtBatch &c) { return c.batch(); }

}  // namespace

// ------------------------------------------------------------------ shape

void BertShape::derive(size_t slots)
{
    S = (int)slots;
    if (T < 2 || (T & (T - 1)) || T > S) throw std::invalid_argument("T must be a power of two <= the slot count");
    NB = S / T;
    if (hidden < 1 || heads < 1 || head_dim < 1 || ffn < 1 || hidden != heads * head_dim)
        throw std::invalid_argument("hidden must equal heads * head_dim");
    H2 = pow2_ceil(heads);
    if (H2 > NB) throw std::invalid_argument("more heads than blocks per ciphertext");
    KB = NB / H2;
    n_head = ceil_div(head_dim, KB);
    n_hid = ceil_div(hidden, NB);
    n_ffn = ceil_div(ffn, NB);
    if (lanes.empty()) throw std::invalid_argument("no lanes");
    Lmax = 0;
    for (auto &lane : lanes) {
        if (lane.empty()) throw std::invalid_argument("empty lane");
        // the attention's masks key a lane's requests as bits of one 16-bit field
        if (lane.size() > 16) throw std::invalid_argument("more than 16 requests in a lane");
        std::vector<std::pair<int, int>> r = lane;
        std::sort(r.begin(), r.end());
        int end = 0;
        for (auto &q : r) {
            if (q.second < 1 || q.first < end || q.first + 2 * q.second > T)
                throw std::invalid_argument("requests of a lane overlap or leave the token block");
            end = q.first + 2 * q.second;
            Lmax = std::max(Lmax, q.second);
        }
    }
    G = (int)std::ceil(std::sqrt((double)Lmax));
    Glt = (int)std::ceil(std::sqrt((double)NB));
    if (!(boot_shrink >= 1.0)) throw std::invalid_argument("boot_shrink must be >= 1");
    fold_ok = true;
    copy_shifts.clear();
    for (auto &lane : lanes)
        for (auto &q : lane) {
            if (q.first + q.second > T / 2) fold_ok = false;
            if (q.first + 2 * q.second > T / 2 &&
                std::find(copy_shifts.begin(), copy_shifts.end(), q.second) == copy_shifts.end())
                copy_shifts.push_back(q.second);
        }
    std::sort(copy_shifts.begin(), copy_shifts.end());
}

std::vector<int> BertShape::rotation_steps() const
{
    std::vector<int> v;
    auto push = [&](int s) {
        s = ((s % S) + S) % S;
        if (s && std::find(v.begin(), v.end(), s) == v.end()) v.push_back(s);
    };
    for (int b = 1; b < Glt; ++b) push(b * T);
    for (int g = 1; g * Glt < NB; ++g) push(g * Glt * T);
    for (int b = 1; b < G; ++b) push(b);
    for (int g = 1; g * G < Lmax; ++g) {
        push(g * G);
        push(-g * G);
    }
    for (int m = 1; m < KB; m <<= 1) push(H2 * T * m);
    for (int m = 1; m < NB; m <<= 1) push(T * m);
    if (fold_ok) {
        push(T / 2);
        push(-T / 2);
        for (int s : copy_shifts) push(-s);
    }
    return v;
}

// ------------------------------------------------------------------ layer

template <class EV, class CT>
BertLayerT<EV, CT>::BertLayerT(EV &ev, BootstrapperT<EV, CT> &bs, const BertShape &shape, const BertWeights &w,
                               std::vector<int> lanes, std::shared_ptr<BertPlaintexts> plain)
    : ev_(&ev), bs_(&bs), ck_(ev, bs.final_scale), sh_(shape), w_(w), lanes_(std::move(lanes)),
      delta_(bs.final_scale), pt_(plain ? std::move(plain) : std::make_shared<BertPlaintexts>())
{
    sh_.derive(ev.slot_count());
    const size_t d = sh_.hidden, f = sh_.ffn;
    auto need = [](const std::vector<double> &v, size_t n, const char *what) {
        if (v.size() != n) throw std::invalid_argument(std::string("weight ") + what + " has the wrong size");
    };
    need(w_.wq, d * d, "wq");
    need(w_.wk, d * d, "wk");
    need(w_.wv, d * d, "wv");
    need(w_.wo, d * d, "wo");
    need(w_.w1, d * f, "w1");
    need(w_.w2, f * d, "w2");
    need(w_.bq, d, "bq");
    need(w_.bk, d, "bk");
    need(w_.bv, d, "bv");
    need(w_.bo, d, "bo");
    need(w_.b1, f, "b1");
    need(w_.b2, d, "b2");
    for (int l : lanes_)
        if (l < 0 || l >= (int)sh_.lanes.size()) throw std::invalid_argument("lane index out of range");
}

template <class EV, class CT>
int BertLayerT<EV, CT>::in_features(int which) const
{
    return which == LT_2 ? sh_.ffn : sh_.hidden;
}

template <class EV, class CT>
int BertLayerT<EV, CT>::out_features(int which) const
{
    return which == LT_1 ? sh_.ffn : sh_.hidden;
}

template <class EV, class CT>
int BertLayerT<EV, CT>::in_count(int which) const
{
    if (which == LT_O) return sh_.n_head;
    return which == LT_2 ? sh_.n_ffn : sh_.n_hid;
}

template <class EV, class CT>
int BertLayerT<EV, CT>::out_count(int which) const
{
    if (which <= LT_V) return sh_.n_head;
    return which == LT_1 ? sh_.n_ffn : sh_.n_hid;
}

template <class EV, class CT>
const std::vector<double> &BertLayerT<EV, CT>::weights(int which) const
{
    switch (which) {
    case LT_Q: return w_.wq;
    case LT_K: return w_.wk;
    case LT_V: return w_.wv;
    case LT_O: return w_.wo;
    case LT_1: return w_.w1;
    default: return w_.w2;
    }
}

template <class EV, class CT>
const std::vector<double> &BertLayerT<EV, CT>::bias(int which) const
{
    switch (which) {
    case LT_Q: return w_.bq;
    case LT_K: return w_.bk;
    case LT_V: return w_.bv;
    case LT_O: return w_.bo;
    case LT_1: return w_.b1;
    default: return w_.b2;
    }
}

// head layout: feature h*dh + k -> ct k / KB, block (k % KB) * H2 + h
template <class EV, class CT>
int BertLayerT<EV, CT>::in_feature(int which, int ct, int block) const
{
    if (which == LT_O) {
        const int h = block % sh_.H2, k = ct * sh_.KB + block / sh_.H2;
        if (h >= sh_.heads || k >= sh_.head_dim) return -1;
        return h * sh_.head_dim + k;
    }
    const int f = ct * sh_.NB + block;
    return f < in_features(which) ? f : -1;
}

template <class EV, class CT>
int BertLayerT<EV, CT>::out_feature(int which, int ct, int block) const
{
    if (which <= LT_V) {
        const int h = block % sh_.H2, k = ct * sh_.KB + block / sh_.H2;
        if (h >= sh_.heads || k >= sh_.head_dim) return -1;
        return h * sh_.head_dim + k;
    }
    const int f = ct * sh_.NB + block;
    return f < out_features(which) ? f : -1;
}

template <class EV, class CT>
bool BertLayerT<EV, CT>::diag_nonzero(int which, int a, int b, int d) const
{
    for (int j = 0; j < sh_.NB; ++j)
        if (out_feature(which, b, j) >= 0 && in_feature(which, a, (j + d) % sh_.NB) >= 0) return true;
    return false;
}

// diagonal d of the (a -> b) block of map `which`, scaled by 1/boot_shrink,
// rotated right by pre_rotate_blocks blocks: slot s holds the entry of block
// (s / T - pre_rotate_blocks) mod NB (on the lower half of each block only
// when lower_half)
template <class EV, class CT>
std::vector<double> BertLayerT<EV, CT>::diag_vector(int which, int a, int b, int d, int pre_rotate_blocks,
                                                    bool lower_half) const
{
    const auto &W = weights(which);
    const int nout = out_features(which), NB = sh_.NB, T = sh_.T, span = lower_half ? T / 2 : T;
    std::vector<double> v((size_t)sh_.S, 0.0);
    for (int j = 0; j < NB; ++j) {
        const int fo = out_feature(which, b, j), fi = in_feature(which, a, (j + d) % NB);
        if (fo < 0 || fi < 0) continue;
        const double x = W[(size_t)fi * nout + fo] / sh_.boot_shrink;
        const int dst = (j + pre_rotate_blocks) % NB;
        std::fill(v.begin() + (size_t)dst * T, v.begin() + (size_t)dst * T + span, x);
    }
    return v;
}

// encode every nonzero diagonal of map `which` at (limbs, scale) that is not
// cached yet: host FFTs on all cores, one NTT launch per plaintext
template <class EV, class CT>
void BertLayerT<EV, CT>::encode_diagonals(int which, int limbs, double scale, bool lower_half)
{
    std::vector<BertPlaintexts::DKey> keys;
    const uint64_t sb = bits_of(scale);
    const int tag = which + (lower_half ? LT_COUNT : 0);
    for (int a = 0; a < in_count(which); ++a)
        for (int b = 0; b < out_count(which); ++b)
            for (int d = 0; d < sh_.NB; ++d) {
                const BertPlaintexts::DKey key{tag, a, b, d, limbs, sb};
                if (!pt_->diag.count(key) && diag_nonzero(which, a, b, d)) keys.push_back(key);
            }
    Evaluator &base = base_evaluator();
    // host FFTs on every core, in chunks that bound the host staging memory;
    // a chunk enters the cache only once all of it is encoded
    const size_t chunk = 256;
    for (size_t lo = 0; lo < keys.size(); lo += chunk) {
        const size_t hi = std::min(keys.size(), lo + chunk);
        std::vector<std::vector<std::complex<double>>> vecs(hi - lo);
        std::vector<Plaintext> plains(hi - lo);
        std::vector<const std::vector<std::complex<double>> *> vp;
        std::vector<Plaintext *> outs;
        for (size_t i = lo; i < hi; ++i) {
            const int a = std::get<1>(keys[i]), b = std::get<2>(keys[i]), d = std::get<3>(keys[i]);
            const std::vector<double> v = diag_vector(which, a, b, d, (d / sh_.Glt) * sh_.Glt, lower_half);
            vecs[i - lo].assign(v.begin(), v.end());
            vp.push_back(&vecs[i - lo]);
            outs.push_back(&plains[i - lo]);
        }
        base.encode_many(vp, limbs, scale, outs);
        for (size_t i = lo; i < hi; ++i) pt_->diag.emplace(keys[i], std::move(plains[i - lo]));
    }
}

template <class EV, class CT>
const Plaintext &BertLayerT<EV, CT>::diag(int which, int a, int b, int d, int limbs, double scale, bool lower_half)
{
    const BertPlaintexts::DKey key{which + (lower_half ? LT_COUNT : 0), a, b, d, limbs, bits_of(scale)};
    auto it = pt_->diag.find(key);
    if (it == pt_->diag.end()) {
        encode_diagonals(which, limbs, scale, lower_half);
        it = pt_->diag.find(key);
        if (it == pt_->diag.end()) throw std::logic_error("diagonal missing after encoding");
    }
    return it->second;
}

// bias of map `which` for output ciphertext ct: b[f] on every token slot of
// f's block (on the lower half only when lower_half)
template <class EV, class CT>
const Plaintext &BertLayerT<EV, CT>::bias_plain(int which, int ct, int limbs, double scale, bool lower_half)
{
    const auto key = std::make_tuple(which + (lower_half ? LT_COUNT : 0), ct, limbs, bits_of(scale));
    auto it = pt_->bias.find(key);
    if (it != pt_->bias.end()) return it->second;
    const auto &bv = bias(which);
    std::vector<std::complex<double>> v((size_t)sh_.S, 0.0);
    for (int j = 0; j < sh_.NB; ++j) {
        const int f = out_feature(which, ct, j);
        if (f < 0) continue;
        for (int t = 0; t < (lower_half ? sh_.T / 2 : sh_.T); ++t) v[(size_t)j * sh_.T + t] = bv[f];
    }
    Plaintext p;
    ev_->encode(v, limbs, scale, p);
    return pt_->bias.emplace(key, std::move(p)).first->second;
}

// softmax masks for offset delta, per lane element: kind 0 multiplies by
// 1/sqrt(d_h) on the valid slots (a head that exists, a first-copy token of a
// request longer than delta) and by 0 elsewhere (encoded at the scale of the
// prime the rescale drops, so the rescale restores the scale); kind 1 adds
// -128 on the other slots (encoded at `scale`)
template <class EV, class CT>
void BertLayerT<EV, CT>::masks(int delta, int kind, int limbs, double scale, std::vector<const Plaintext *> &out)
{
    out.clear();
    const double sc = kind == 0 ? (double)ev_->modulus(limbs - 1) : scale;
    for (int lane : lanes_) {
        // a mask depends on delta only through the requests longer than it
        int sig = 0;
        const auto &reqs = sh_.lanes[lane];
        for (size_t r = 0; r < reqs.size(); ++r)
            if (delta < reqs[r].second) sig |= 1 << r;
        const auto key = std::make_tuple(lane, sig, limbs, bits_of(sc), kind);
        auto it = pt_->mask.find(key);
        if (it == pt_->mask.end()) {
            std::vector<std::complex<double>> v((size_t)sh_.S, 0.0);
            const double inv_sqrt = 1.0 / std::sqrt((double)sh_.head_dim);
            for (int j = 0; j < sh_.NB; ++j) {
                const bool head_ok = (j % sh_.H2) < sh_.heads;
                for (int t = 0; t < sh_.T; ++t) {
                    bool ok = false;
                    if (head_ok)
                        for (size_t r = 0; r < reqs.size(); ++r)
                            if ((sig >> r & 1) && t >= reqs[r].first && t < reqs[r].first + reqs[r].second) ok = true;
                    v[(size_t)j * sh_.T + t] = kind == 0 ? (ok ? inv_sqrt : 0.0) : (ok ? 0.0 : -128.0);
                }
            }
            Plaintext p;
            ev_->encode(v, limbs, sc, p);
            it = pt_->mask.emplace(key, std::move(p)).first;
        }
        out.push_back(&it->second);
    }
}

// copy-rebuild masks of unfold_copies, per lane element: shift 0 keeps the
// lower half of every block; shift s > 0 selects the token slots of the
// requests of length s whose copy (s slots on) lies in the upper half
template <class EV, class CT>
void BertLayerT<EV, CT>::copy_masks(int shift, int limbs, std::vector<const Plaintext *> &out)
{
    out.clear();
    const double sc = (double)ev_->modulus(limbs - 1);
    const int T = sh_.T, half = T / 2;
    for (int lane : lanes_) {
        const auto key = std::make_tuple(lane, shift, limbs, bits_of(sc), 2);
        auto it = pt_->mask.find(key);
        if (it == pt_->mask.end()) {
            std::vector<double> block((size_t)T, 0.0);
            if (shift == 0) {
                std::fill(block.begin(), block.begin() + half, 1.0);
            } else {
                for (auto &r : sh_.lanes[lane])
                    if (r.second == shift)
                        for (int t = std::max(r.first, half - shift); t < r.first + r.second; ++t) block[t] = 1.0;
            }
            std::vector<double> v((size_t)sh_.S);
            for (int j = 0; j < sh_.NB; ++j) std::copy(block.begin(), block.end(), v.begin() + (size_t)j * T);
            Plaintext p;
            ev_->encode(v, limbs, sc, p);
            it = pt_->mask.emplace(key, std::move(p)).first;
        }
        out.push_back(&it->second);
    }
}

// the kind-1 masks of offsets 2 pair and 2 pair + 1 in the two halves of
// every block (all -128 in the upper half past the last offset)
template <class EV, class CT>
void BertLayerT<EV, CT>::fold_masks(int pair, int limbs, double scale, std::vector<const Plaintext *> &out)
{
    out.clear();
    const int T = sh_.T, half = T / 2, d0 = 2 * pair, d1 = 2 * pair + 1;
    for (int lane : lanes_) {
        const auto &reqs = sh_.lanes[lane];
        auto sig_of = [&](int delta) {
            int sig = 0;
            for (size_t r = 0; r < reqs.size(); ++r)
                if (delta < reqs[r].second) sig |= 1 << r;
            return sig;
        };
        const int s0 = sig_of(d0), s1 = d1 < sh_.Lmax ? sig_of(d1) : 0;
        const auto key = std::make_tuple(lane, s0 * 65536 + s1, limbs, bits_of(scale), 3);
        auto it = pt_->mask.find(key);
        if (it == pt_->mask.end()) {
            std::vector<std::complex<double>> v((size_t)sh_.S, 0.0);
            for (int j = 0; j < sh_.NB; ++j) {
                const bool head_ok = (j % sh_.H2) < sh_.heads;
                for (int t = 0; t < T; ++t) {
                    const int sig = t < half ? s0 : s1, tt = t < half ? t : t - half;
                    bool ok = false;
                    if (head_ok)
                        for (size_t r = 0; r < reqs.size(); ++r)
                            if ((sig >> r & 1) && tt >= reqs[r].first && tt < reqs[r].first + reqs[r].second) ok = true;
                    v[(size_t)j * T + t] = ok ? 0.0 : -128.0;
                }
            }
            Plaintext p;
            ev_->encode(v, limbs, scale, p);
            it = pt_->mask.emplace(key, std::move(p)).first;
        }
        out.push_back(&it->second);
    }
}

// encoded once per level and scale (a graph replays no host encode)
template <class EV, class CT>
const Plaintext &BertLayerT<EV, CT>::half_plain(double value, bool upper, int limbs, double scale)
{
    const auto key = std::make_tuple(bits_of(value), limbs, bits_of(scale), upper ? 1 : 0);
    auto it = pt_->half.find(key);
    if (it == pt_->half.end()) {
        const int half = sh_.T / 2;
        std::vector<double> v((size_t)sh_.S, 0.0);
        for (int j = 0; j < sh_.NB; ++j) {
            const auto b = v.begin() + (size_t)j * sh_.T + (upper ? half : 0);
            std::fill(b, b + half, value);
        }
        Plaintext e;
        ev_->encode(v, limbs, scale, e);
        it = pt_->half.emplace(key, std::move(e)).first;
    }
    return it->second;
}

// ct *= value with the constant encoded so that, after the rescale, the
// scale is target_scale (set exactly); with lower_half the value is on the
// lower half of each token block and 0 on the upper half
template <class EV, class CT>
void BertLayerT<EV, CT>::exact_scale_const(CT &ct, double value, double target_scale, bool lower_half)
{
    const int l = ct.limbs();
    const double q = (double)ev_->modulus(l - 1);
    const double sc = q * target_scale / ct.scale();
    Plaintext scalar;
    const Plaintext *p = &scalar;
    if (lower_half) p = &half_plain(value, false, l, sc);
    else ev_->encode(value, l, sc, scalar);
    ev_->multiply_plain_inplace(ct, *p);
    ev_->rescale_to_next_inplace(ct);
    ct.scale() = target_scale;
}

// y = map(x) + bias, x at >= 2 limbs: y at x.limbs - 1 at scale delta / boot_shrink
template <class EV, class CT>
void BertLayerT<EV, CT>::project(const std::vector<CT> &x, int which, std::vector<CT> &y, bool lower_half)
{
    EV &ev = *ev_;
    const int n_in = in_count(which), n_out = out_count(which);
    if ((int)x.size() != n_in) throw std::invalid_argument("project: wrong number of input ciphertexts");
    const int l = x[0].limbs();
    if (l < 2) throw std::invalid_argument("project: the input needs a level to spend");
    const double in_scale = x[0].scale();
    for (auto &c : x)
        if (c.limbs() != l || c.scale() != in_scale) throw std::invalid_argument("project: inputs differ");
    // diagonals at a scale that brings the product back to delta after the rescale
    const double dscale = (double)ev.modulus(l - 1) * delta_ / in_scale;
    encode_diagonals(which, l, dscale, lower_half);
    const int Glt = sh_.Glt, T = sh_.T, NB = sh_.NB;
    std::vector<std::vector<CT>> baby(n_in);
    std::vector<int> steps;
    for (int b = 1; b < Glt; ++b) steps.push_back(b * T);
    for (int a = 0; a < n_in; ++a) {
        std::vector<CT> rot;
        ev.rotate_vector_many(x[a], steps, rot);
        baby[a].resize(Glt);
        baby[a][0] = x[a];
        for (int b = 1; b < Glt; ++b) baby[a][b] = std::move(rot[b - 1]);
    }
    y.assign(n_out, CT());
    std::vector<const CT *> terms;
    std::vector<const Plaintext *> pts;
    for (int b = 0; b < n_out; ++b) {
        CT acc, giant, t;
        bool have = false;
        for (int g = 0; g * Glt < NB; ++g) {
            terms.clear();
            pts.clear();
            for (int a = 0; a < n_in; ++a)
                for (int bb = 0; bb < Glt && g * Glt + bb < NB; ++bb) {
                    const int d = g * Glt + bb;
                    if (!diag_nonzero(which, a, b, d)) continue;
                    terms.push_back(&baby[a][bb]);
                    pts.push_back(&diag(which, a, b, d, l, dscale, lower_half));
                }
            if (terms.empty()) continue;
            ev.multiply_plain_accumulate(terms, pts, giant);
            if (g) {
                ev.rotate_vector(giant, g * Glt * T, t);
            } else {
                t = std::move(giant);
            }
            if (!have) {
                acc = std::move(t);
                have = true;
            } else {
                ev.add_inplace(acc, t);
            }
        }
        if (!have) throw std::logic_error("project: an output ciphertext has no diagonal");
        ev.rescale_to_next_inplace(acc);
        acc.scale() = delta_ / sh_.boot_shrink;
        ev.add_plain_inplace(acc, bias_plain(which, b, acc.limbs(), acc.scale(), lower_half));
        y[b] = std::move(acc);
    }
}

// out[i] = x[2i] + rot(x[2i+1], -T/2) (x[2i] alone for an odd last one); the
// inputs hold values on the lower half of each token block only
template <class EV, class CT>
void BertLayerT<EV, CT>::fold_halves(std::vector<CT> &x)
{
    EV &ev = *ev_;
    std::vector<CT> out((x.size() + 1) / 2);
    for (size_t i = 0; i < out.size(); ++i) {
        if (2 * i + 1 < x.size()) {
            CT t;
            ev.rotate_vector(x[2 * i + 1], sh_.S - sh_.T / 2, t);
            ev.add(x[2 * i], t, out[i]);
        } else {
            out[i] = std::move(x[2 * i]);
        }
    }
    x = std::move(out);
}

// inverse of fold_halves on the lower half: out[2i] = x[i], out[2i+1] = rot(x[i], T/2)
template <class EV, class CT>
void BertLayerT<EV, CT>::unfold_halves(std::vector<CT> &x, int count)
{
    EV &ev = *ev_;
    if (count < 1 || (int)x.size() != (count + 1) / 2)
        throw std::invalid_argument("unfold_halves: wrong number of ciphertexts");
    std::vector<CT> out(count);
    for (int i = 0; i < count; ++i) {
        if (i % 2) ev.rotate_vector(x[i / 2], sh_.T / 2, out[i]);
        else out[i] = x[i / 2];
    }
    x = std::move(out);
}

// unfold_halves, then on each half: its lower half kept, and for every copy
// shift s the tokens whose second copy lies in the upper half rotated s slots
// on (masks per lane, each product rescaled once: the output is one level
// below the input)
template <class EV, class CT>
void BertLayerT<EV, CT>::unfold_copies(std::vector<CT> &x, int count)
{
    EV &ev = *ev_;
    if (count < 1 || (int)x.size() != (count + 1) / 2)
        throw std::invalid_argument("unfold_copies: wrong number of ciphertexts");
    const int l = x[0].limbs();
    if (l < 2) throw std::invalid_argument("unfold_copies: the input needs a level to spend");
    std::vector<const Plaintext *> keep, mp;
    copy_masks(0, l, keep);
    std::vector<CT> out(count);
    for (int i = 0; i < count; ++i) {
        CT h;
        if (i % 2) ev.rotate_vector(x[i / 2], sh_.T / 2, h);
        else h = x[i / 2];
        CT acc = h;
        mul_plain_each(ev, acc, keep);
        ev.rescale_to_next_inplace(acc);
        for (int s : sh_.copy_shifts) {
            CT t = h, r;
            copy_masks(s, l, mp);
            mul_plain_each(ev, t, mp);
            ev.rescale_to_next_inplace(t);
            ev.rotate_vector(t, sh_.S - s, r);
            ev.add_inplace(acc, r);
        }
        out[i] = std::move(acc);
    }
    x = std::move(out);
}

template <class EV, class CT>
Evaluator &BertLayerT<EV, CT>::base_evaluator()
{
    if constexpr (std::is_same<EV, Evaluator>::value) return *ev_;
    else return ev_->base();
}

template <class EV, class CT>
void BertLayerT<EV, CT>::bootstrap_all(std::vector<CT> &cts)
{
    EV &ev = *ev_;
    for (auto &c : cts) ev.mod_switch_to_inplace(c, 1);
    auto refresh = [&](std::vector<CT> &v) {
        std::vector<CT *> p;
        for (auto &c : v) p.push_back(&c);
        each(ev, p, 16, [&](CT &c) {
            CT r;
            bs_->bootstrap_3(r, c);
            c = std::move(r);
        });
    };
    if (!sh_.boot_pack) {
        refresh(cts);
        return;
    }
    // pairs (2i, 2i + 1) share a bootstrap (see bert.h); a trailing odd one
    // is a pair whose second member is zero, so that every z goes through
    // the same lockstep group
    Evaluator &base = base_evaluator();
    const int half = (int)(base.context().n / 2);
    const size_t pairs = (cts.size() + 1) / 2;
    std::vector<CT> z(pairs);
    for (size_t i = 0; i < pairs; ++i) {
        if (2 * i + 1 < cts.size()) {
            CT t;
            ev.multiply_plain(cts[2 * i + 1], base.monomial(half, 1), t);
            ev.add(cts[2 * i], t, z[i]);
        } else {
            z[i] = std::move(cts[2 * i]);
        }
        z[i].scale() *= 2.0;
    }
    refresh(z);
    for (size_t i = 0; i < pairs; ++i) {
        CT conj = z[i];
        ev.complex_conjugate_inplace(conj);
        ev.add(z[i], conj, cts[2 * i]);
        if (2 * i + 1 < cts.size()) {
            ev.sub(conj, z[i], cts[2 * i + 1]);
            ev.multiply_plain_inplace(cts[2 * i + 1], base.monomial(half, cts[2 * i + 1].limbs()));
        }
    }
}

template <class EV, class CT>
void BertLayerT<EV, CT>::attention(std::vector<CT> &q, std::vector<CT> &k, std::vector<CT> &v, std::vector<CT> &o)
{
    EV &ev = *ev_;
    const int nh = sh_.n_head, G = sh_.G, L = sh_.Lmax, S = sh_.S;
    // levels, counted back from the output projection (2 limbs): PV 1,
    // P = E * I 1, exp 8 (constant + 7 squarings), mask 1, Q.K 1
    const int e_limbs = 4, qk_limbs = kQKLimbs, v_limbs = e_limbs - 1;
    static_assert(kVInLimbs - 1 == 3 && kQKLimbs == 14, "the levels the projections and bootstraps leave");
    for (auto &c : q) ev.mod_switch_to_inplace(c, qk_limbs);
    for (auto &c : k) ev.mod_switch_to_inplace(c, qk_limbs);
    for (auto &c : v) ev.mod_switch_to_inplace(c, v_limbs);
    const int n_g = ceil_div(L, G);
    // hoisted rotations would keep a permuted copy of every key used here
    // (one key's size each); the attention's rotations are switched one by
    // one instead, which leaves that memory to the encoded weights
    Evaluator &base = [&]() -> Evaluator & {
        if constexpr (std::is_same<EV, Evaluator>::value) return ev;
        else return ev.base();
    }();
    struct Restore {
        Evaluator &e;
        bool on;
        ~Restore() { e.hoisting = on; }
    } restore{base, base.hoisting};
    base.hoisting = false;

    // baby steps of K and V, giant pre-rotations of Q
    std::vector<int> baby_steps;
    for (int b = 1; b < G; ++b) baby_steps.push_back(b);
    std::vector<std::vector<CT>> kb(nh), vb(nh), qg(nh);
    for (int c = 0; c < nh; ++c) {
        std::vector<CT> r;
        ev.rotate_vector_many(k[c], baby_steps, r);
        kb[c].resize(G);
        kb[c][0] = k[c];
        for (int b = 1; b < G; ++b) kb[c][b] = std::move(r[b - 1]);
        ev.rotate_vector_many(v[c], baby_steps, r);
        vb[c].resize(G);
        vb[c][0] = v[c];
        for (int b = 1; b < G; ++b) vb[c][b] = std::move(r[b - 1]);
        std::vector<int> gsteps;
        for (int g = 1; g < n_g; ++g) gsteps.push_back(S - g * G);
        ev.rotate_vector_many(q[c], gsteps, r);
        qg[c].resize(n_g);
        qg[c][0] = q[c];
        for (int g = 1; g < n_g; ++g) qg[c][g] = std::move(r[g - 1]);
    }

    // scores S_delta, masked and passed through exp (offsets 2p and 2p+1
    // folded in one ciphertext when folding: the valid slots are first token
    // copies, all in the lower half)
    const bool fold = sh_.folding();
    std::vector<CT> e(L);
    std::vector<const Plaintext *> mp;
    for (int d = 0; d < L; ++d) {
        const int g = d / G, b = d % G;
        CT acc, t;
        for (int c = 0; c < nh; ++c) {
            ev.multiply(qg[c][g], kb[c][b], t);
            if (c == 0) acc = std::move(t);
            else ev.add_inplace(acc, t);
        }
        ev.relinearize_inplace(acc);
        ev.rescale_to_next_inplace(acc);
        if (g) {
            ev.rotate_vector(acc, g * G, t);
            acc = std::move(t);
        }
        masks(d, 0, acc.limbs(), acc.scale(), mp);
        mul_plain_each(ev, acc, mp);
        ev.rescale_to_next_inplace(acc);
        e[d] = std::move(acc);
    }
    // the sum over the KB blocks of each head commutes with the zeroing mask
    // (the same on every block of a head) and with the fold, so it is taken
    // once per ciphertext after both; then the -128 masks
    if (fold) fold_halves(e);
    for (size_t p = 0; p < e.size(); ++p) {
        CT t;
        for (int m = 1; m < sh_.KB; m <<= 1) {
            ev.rotate_vector(e[p], sh_.H2 * sh_.T * m, t);
            ev.add_inplace(e[p], t);
        }
        if (fold) fold_masks((int)p, e[p].limbs(), e[p].scale(), mp);
        else masks((int)p, 1, e[p].limbs(), e[p].scale(), mp);
        add_plain_each(ev, e[p], mp);
    }
    mark("attention scores");
    {
        std::vector<CT *> p;
        for (auto &x : e) p.push_back(&x);
        each(ev, p, 64, [&](CT &x) { x = ck_.exp(x); });
    }
    mark("attention exp");

    // row sums over delta, the inverse after a bootstrap (softmax.cpp:24-35)
    CT sum = e[0];
    for (size_t d = 1; d < e.size(); ++d) ev.add_inplace(sum, e[d]);
    {
        const double c = 0.01 / sh_.rowsum_shrink;
        Plaintext delta;
        ev.encode(c, sum.limbs(), sum.scale(), delta);
        if (fold) {
            // each half adds the other half of its own block (masked in the
            // constant product the sum takes anyway)
            CT up, down;
            ev.rotate_vector(sum, sh_.T / 2, up);
            ev.rotate_vector(sum, sh_.S - sh_.T / 2, down);
            ev.multiply_plain_inplace(up, half_plain(c, false, up.limbs(), sum.scale()));
            ev.multiply_plain_inplace(down, half_plain(c, true, down.limbs(), sum.scale()));
            ev.multiply_plain_inplace(sum, delta);
            ev.add_inplace(sum, up);
            ev.add_inplace(sum, down);
        } else {
            ev.multiply_plain_inplace(sum, delta);
        }
        ev.rescale_to_next_inplace(sum);
        sum.scale() /= sh_.rowsum_shrink;
    }
    std::vector<CT> one{std::move(sum)};
    bootstrap_all(one);
    CT inv = ck_.inverse(one[0]);
    {
        Plaintext delta;
        ev.encode(0.01, inv.limbs(), inv.scale(), delta);
        ev.multiply_plain_inplace(inv, delta);
        ev.rescale_to_next_inplace(inv);
    }
    ev.mod_switch_to_inplace(inv, e[0].limbs());
    mark("attention row sums");
    // P_delta = exp(S_delta) * inverse(sum) (softmax.cpp:37-40)
    for (auto &x : e) {
        ev.multiply_inplace(x, inv);
        ev.relinearize_inplace(x);
        ev.rescale_to_next_inplace(x);
    }
    if (fold) unfold_halves(e, L);
    mark("attention probabilities");

    // O_c = sum_g rot(sum_b rot(P_{G g + b}, -G g) * rot(V_c, b), G g)
    o.assign(nh, CT());
    std::vector<std::vector<CT>> pg(n_g);
    for (int g = 0; g < n_g; ++g) {
        pg[g].resize(G);
        for (int b = 0; b < G && g * G + b < L; ++b) {
            if (g) ev.rotate_vector(e[g * G + b], S - g * G, pg[g][b]);
            else pg[g][b] = e[b];
        }
    }
    for (int c = 0; c < nh; ++c) {
        CT acc, t, u;
        bool have = false;
        for (int g = 0; g < n_g; ++g) {
            CT part;
            bool hp = false;
            for (int b = 0; b < G && g * G + b < L; ++b) {
                ev.multiply(pg[g][b], vb[c][b], t);
                if (!hp) {
                    part = std::move(t);
                    hp = true;
                } else {
                    ev.add_inplace(part, t);
                }
            }
            ev.relinearize_inplace(part);
            ev.rescale_to_next_inplace(part);
            if (g) {
                ev.rotate_vector(part, g * G, u);
                part = std::move(u);
            }
            if (!have) {
                acc = std::move(part);
                have = true;
            } else {
                ev.add_inplace(acc, part);
            }
        }
        o[c] = std::move(acc);
    }
}

// LayerNorm of NEXUS (layer_norm.cpp:6-33): the sum of squares over the
// features is a sum over ciphertexts and a fold over the NB blocks
template <class EV, class CT>
void BertLayerT<EV, CT>::layer_norm(std::vector<CT> &x, bool folded)
{
    EV &ev = *ev_;
    CT sum, t;
    for (size_t c = 0; c < x.size(); ++c) {
        ev.square(x[c], t);
        ev.relinearize_inplace(t);
        ev.rescale_to_next_inplace(t);
        if (c == 0) sum = std::move(t);
        else ev.add_inplace(sum, t);
    }
    for (int m = 1; m < sh_.NB; m <<= 1) {
        ev.rotate_vector(sum, sh_.T * m, t);
        ev.add_inplace(sum, t);
    }
    if (folded) {
        // every block now holds the same sums; the two halves hold two
        // feature sets of the same tokens
        ev.rotate_vector(sum, sh_.T / 2, t);
        ev.add_inplace(sum, t);
    }
    Plaintext delta;
    ev.encode(1.0 / sh_.hidden, sum.limbs(), sum.scale(), delta);
    ev.multiply_plain_inplace(sum, delta);
    ev.rescale_to_next_inplace(sum);
    CT r = ck_.invert_sqrt(sum, 4, 2);
    for (auto &c : x) {
        ev.mod_switch_to_inplace(c, r.limbs());
        ev.multiply_inplace(c, r);
        ev.relinearize_inplace(c);
        ev.rescale_to_next_inplace(c);
    }
}

template <class EV, class CT>
void BertLayerT<EV, CT>::shrink_for_bootstrap(std::vector<CT> &cts, bool lower_half)
{
    for (auto &c : cts) {
        exact_scale_const(c, 1.0 / sh_.boot_shrink, delta_, lower_half);
        c.scale() = delta_ / sh_.boot_shrink;
    }
}

template <class EV, class CT>
void BertLayerT<EV, CT>::forward(const std::vector<CT> &x_in, std::vector<CT> &out)
{
    EV &ev = *ev_;
    if ((int)x_in.size() != sh_.n_hid) throw std::invalid_argument("forward: wrong number of input ciphertexts");
    for (auto &c : x_in)
        if (batch_of(c) != (int)lanes_.size()) throw std::invalid_argument("forward: batch does not match the lanes");
    if (x_in[0].limbs() < kVInLimbs) throw std::invalid_argument("forward: the input needs at least 4 limbs");
    begin_marks();
    const bool fold = sh_.folding();
    // the residual branch: x / boot_shrink at one limb (on the lower half of
    // each token block when folding)
    std::vector<CT> x_res = x_in;
    shrink_for_bootstrap(x_res, fold);
    for (auto &c : x_res) ev.mod_switch_to_inplace(c, 1);
    // Q and K at one limb, refreshed; V from the input at 4 limbs lands at
    // the 3 limbs the attention reads it at, so it needs no bootstrap
    std::vector<CT> x2 = x_in, x4 = x_in;
    for (auto &c : x2) ev.mod_switch_to_inplace(c, 2);
    for (auto &c : x4) ev.mod_switch_to_inplace(c, kVInLimbs);
    std::vector<CT> q, k, v;
    project(x2, LT_Q, q, fold);
    project(x2, LT_K, k, fold);
    project(x4, LT_V, v);
    mark("qkv projections");
    {
        // Q and K folded two per ciphertext through the bootstrap (bert.h),
        // unfolded at the attention's level (K with its token copies rebuilt,
        // one level above it)
        if (fold) {
            fold_halves(q);
            fold_halves(k);
        }
        const size_t nq = q.size();
        std::vector<CT> all;
        for (auto *t : {&q, &k})
            for (auto &c : *t) all.push_back(std::move(c));
        bootstrap_all(all);
        for (size_t i = 0; i < nq; ++i) q[i] = std::move(all[i]);
        for (size_t i = 0; i < k.size(); ++i) k[i] = std::move(all[nq + i]);
        if (fold) {
            for (auto &c : q) ev.mod_switch_to_inplace(c, kQKLimbs);
            unfold_halves(q, sh_.n_head);
            for (auto &c : k) ev.mod_switch_to_inplace(c, kQKLimbs + 1);
            unfold_copies(k, sh_.n_head);
        }
    }
    mark("qk bootstraps");
    std::vector<CT> o, a;
    attention(q, k, v, o);
    mark("attention values");
    project(o, LT_O, a, fold);
    // residual + LayerNorm (two hidden ciphertexts folded in one from here
    // to the layer's output when folding)
    for (int c = 0; c < sh_.n_hid; ++c) {
        a[c].scale() = x_res[c].scale();
        ev.add_inplace(a[c], x_res[c]);
    }
    if (fold) fold_halves(a);
    mark("output projection + residual");
    bootstrap_all(a);
    mark("residual bootstraps 1");
    layer_norm(a, fold);
    mark("layer norm 1");
    // FFN
    std::vector<CT> y_res = a;
    shrink_for_bootstrap(y_res);
    for (auto &c : y_res) ev.mod_switch_to_inplace(c, 1);
    for (auto &c : a) ev.mod_switch_to_inplace(c, 2);
    if (fold) unfold_halves(a, sh_.n_hid);
    std::vector<CT> h, f;
    project(a, LT_1, h, fold);
    if (fold) fold_halves(h);
    mark("ffn1 projection");
    bootstrap_all(h);
    mark("ffn hidden bootstraps");
    {
        GeLUEvaluatorT<EV, CT> gelu(ck_);
        std::vector<CT *> p;
        for (auto &c : h) p.push_back(&c);
        each(ev, p, 64, [&](CT &c) {
            CT r;
            gelu.gelu(c, r);
            c = std::move(r);
        });
    }
    mark("gelu");
    if (fold) unfold_halves(h, sh_.n_ffn);
    project(h, LT_2, f, fold);
    if (fold) fold_halves(f);
    for (size_t c = 0; c < f.size(); ++c) {
        f[c].scale() = y_res[c].scale();
        ev.add_inplace(f[c], y_res[c]);
    }
    mark("ffn2 projection + residual");
    bootstrap_all(f);
    mark("residual bootstraps 2");
    layer_norm(f, fold);
    if (fold) unfold_halves(f, sh_.n_hid);
    mark("layer norm 2");
    out = std::move(f);
}

template <class EV, class CT>
void BertLayerT<EV, CT>::begin_marks()
{
    for (auto &m : marks_) cudaEventDestroy(m.second);
    marks_.clear();
    if (timing) mark("start");
}

template <class EV, class CT>
void BertLayerT<EV, CT>::mark(const char *name)
{
    if (!timing) return;
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) throw std::runtime_error("cudaEventCreate failed");
    cudaEventRecord(e, ev_->stream());
    marks_.emplace_back(name, e);
}

template <class EV, class CT>
std::vector<std::pair<std::string, double>> BertLayerT<EV, CT>::stage_times()
{
    std::vector<std::pair<std::string, double>> r;
    for (size_t i = 1; i < marks_.size(); ++i) {
        float ms = 0.f;
        if (cudaEventSynchronize(marks_[i].second) != cudaSuccess ||
            cudaEventElapsedTime(&ms, marks_[i - 1].second, marks_[i].second) != cudaSuccess)
            throw std::runtime_error("event timing failed");
        r.emplace_back(marks_[i].first, ms);
    }
    return r;
}

template <class EV, class CT>
BertLayerT<EV, CT>::~BertLayerT()
{
    for (auto &m : marks_) cudaEventDestroy(m.second);
}

template class BertLayerT<Evaluator, Ciphertext>;
template class BertLayerT<BatchEvaluator, CtBatch>;

}  // namespace nexus
