// seal_shim.cpp -- TEST INFRASTRUCTURE.  A C ABI over the public API of the
// SEAL-4.1-bs fork bundled with NEXUS, so the tests can run the real library
// on the same inputs as the CPU restatement and the CUDA engine.  Built only
// where the NEXUS sources are present (oracle/build_ref.py); the engine never
// links it.
//
// Every array uses SEAL's own layout ([size][limbs][N], NTT form).
#include <algorithm>
#include <array>
#include <complex>
#include <cstring>
#include <sstream>
#include <memory>
#include <string>
#include <vector>

#include "seal/seal.h"

// NEXUS's own operators (src/*.h in the NEXUS tree), compiled from source
#include "ckks_evaluator.h"
#include "gelu.h"
#include "layer_norm.h"
#include "softmax.h"
// MMEvaluator keeps its expansion steps private; the shim calls them directly
#define private public
#include "matrix_mul.h"
#undef private
#include "seal/util/ntt.h"
#include "seal/util/rlwe.h"

using namespace seal;

namespace {

std::string g_err;

struct Shim {
    std::unique_ptr<SEALContext> ctx;
    std::unique_ptr<CKKSEncoder> enc;
    std::unique_ptr<Evaluator> ev;
    std::unique_ptr<KeyGenerator> kg;
    std::unique_ptr<SecretKey> sk;
    std::unique_ptr<PublicKey> pk;
    std::unique_ptr<RelinKeys> rk;
    std::unique_ptr<GaloisKeys> gk;
    std::unique_ptr<Encryptor> encryptor;
    std::unique_ptr<Decryptor> decryptor;
    size_t n = 0;
    int k = 0;
};

parms_id_type pid_for_limbs(const Shim &s, int limbs)
{
    auto cd = s.ctx->key_context_data();
    while (cd) {
        if ((int)cd->parms().coeff_modulus().size() == limbs) return cd->parms_id();
        cd = cd->next_context_data();
    }
    throw std::invalid_argument("no level with that many primes");
}

void load_ct(const Shim &s, Ciphertext &ct, const uint64_t *in, int size, int limbs, double scale)
{
    ct.resize(*s.ctx, pid_for_limbs(s, limbs), size);
    std::memcpy(ct.data(), in, sizeof(uint64_t) * size * limbs * s.n);
    ct.is_ntt_form() = true;
    ct.scale() = scale;
}

void store_ct(const Shim &s, const Ciphertext &ct, uint64_t *out)
{
    std::memcpy(out, ct.data(), sizeof(uint64_t) * ct.size() * ct.coeff_modulus_size() * s.n);
}

void copy_kswitch(const Shim &s, const std::vector<PublicKey> &kv, uint64_t *out)
{
    size_t per = 2 * (size_t)s.k * s.n;
    for (size_t j = 0; j < kv.size(); ++j) std::memcpy(out + j * per, kv[j].data().data(), sizeof(uint64_t) * per);
}

}  // namespace

#define GUARD(...)                          \
    try {                                   \
        __VA_ARGS__;                        \
    } catch (const std::exception &e) {     \
        g_err = e.what();                   \
        return -1;                          \
    }                                       \
    return 0;

extern "C" {

const char *sr_last_error() { return g_err.c_str(); }

// CKKS context over explicit primes (data primes, then the special prime),
// no security check, optional sparse secret (hamming_weight > 0), seeded
// Blake2xb PRNG so keys and encryptions are reproducible.
void *sr_create(int logn, const uint64_t *moduli, int k, uint64_t seed, int hamming_weight)
{
    try {
        auto *s = new Shim();
        EncryptionParameters parms(scheme_type::ckks);
        s->n = size_t(1) << logn;
        s->k = k;
        parms.set_poly_modulus_degree(s->n);
        std::vector<Modulus> mods;
        for (int i = 0; i < k; ++i) mods.emplace_back(moduli[i]);
        parms.set_coeff_modulus(mods);
        if (hamming_weight > 0) parms.set_secret_key_hamming_weight(hamming_weight);
        prng_seed_type sd{};
        sd[0] = seed;
        parms.set_random_generator(std::make_shared<Blake2xbPRNGFactory>(sd));
        s->ctx.reset(new SEALContext(parms, true, sec_level_type::none));
        if (!s->ctx->parameters_set()) throw std::invalid_argument(s->ctx->parameter_error_message());
        s->enc.reset(new CKKSEncoder(*s->ctx));
        s->ev.reset(new Evaluator(*s->ctx, *s->enc));
        return s;
    } catch (const std::exception &e) {
        g_err = e.what();
        return nullptr;
    }
}

void sr_destroy(void *h) { delete static_cast<Shim *>(h); }

// Secret key, public key, relinearization key and Galois keys for `steps`.
int sr_keygen(void *h, const int *steps, int nsteps)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        s.kg.reset(new KeyGenerator(*s.ctx));
        s.sk.reset(new SecretKey(s.kg->secret_key()));
        s.pk.reset(new PublicKey());
        s.kg->create_public_key(*s.pk);
        s.rk.reset(new RelinKeys());
        s.kg->create_relin_keys(*s.rk);
        s.gk.reset(new GaloisKeys());
        if (nsteps > 0) s.kg->create_galois_keys(std::vector<int>(steps, steps + nsteps), *s.gk);
        s.encryptor.reset(new Encryptor(*s.ctx, *s.pk));
        s.decryptor.reset(new Decryptor(*s.ctx, *s.sk));
    })
}

int sr_export_secret(void *h, uint64_t *out)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD(std::memcpy(out, s.sk->data().data(), sizeof(uint64_t) * s.k * s.n))
}

// relinearization key: [K-1][2][K][N]
int sr_export_relin(void *h, uint64_t *out)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD(copy_kswitch(s, s.rk->key(2), out))
}

int sr_export_galois(void *h, uint32_t elt, uint64_t *out)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD(copy_kswitch(s, s.gk->key(elt), out))
}

int sr_galois_elt(void *h, int step, uint32_t *out)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD(*out = s.ctx->key_context_data()->galois_tool()->get_elt_from_step(step))
}

// ntt_negacyclic_harvey / inverse on `count` limbs of one prime
int sr_ntt(int logn, uint64_t q, uint64_t *data, size_t count, int inverse)
{
    GUARD({
        util::NTTTables t(logn, Modulus(q));
        size_t n = size_t(1) << logn;
        for (size_t i = 0; i < count; ++i) {
            if (inverse) util::inverse_ntt_negacyclic_harvey(data + i * n, t);
            else util::ntt_negacyclic_harvey(data + i * n, t);
        }
    })
}

int sr_rescale(void *h, const uint64_t *in, int size, int limbs, double scale, uint64_t *out, double *out_scale)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        Ciphertext ct;
        load_ct(s, ct, in, size, limbs, scale);
        s.ev->rescale_to_next_inplace(ct);
        store_ct(s, ct, out);
        *out_scale = ct.scale();
    })
}

int sr_multiply(void *h, const uint64_t *a, const uint64_t *b, int limbs, uint64_t *out3)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        Ciphertext x, y;
        load_ct(s, x, a, 2, limbs, 1.0);
        load_ct(s, y, b, 2, limbs, 1.0);
        s.ev->multiply_inplace(x, y);
        store_ct(s, x, out3);
    })
}

int sr_relinearize(void *h, const uint64_t *in3, int limbs, uint64_t *out2)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        Ciphertext x;
        load_ct(s, x, in3, 3, limbs, 1.0);
        s.ev->relinearize_inplace(x, *s.rk);
        store_ct(s, x, out2);
    })
}

int sr_rotate(void *h, const uint64_t *in, int limbs, int step, uint64_t *out)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        Ciphertext x;
        load_ct(s, x, in, 2, limbs, 1.0);
        s.ev->rotate_vector_inplace(x, step, *s.gk);
        store_ct(s, x, out);
    })
}

int sr_conjugate(void *h, const uint64_t *in, int limbs, uint64_t *out)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        Ciphertext x;
        load_ct(s, x, in, 2, limbs, 1.0);
        s.ev->complex_conjugate_inplace(x, *s.gk);
        store_ct(s, x, out);
    })
}

int sr_multiply_plain(void *h, const uint64_t *ct, int size, int limbs, const uint64_t *pt, uint64_t *out)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        Ciphertext x;
        load_ct(s, x, ct, size, limbs, 1.0);
        Plaintext p;
        p.parms_id() = parms_id_zero;
        p.resize(s.n * limbs);
        std::memcpy(p.data(), pt, sizeof(uint64_t) * s.n * limbs);
        p.parms_id() = pid_for_limbs(s, limbs);
        p.scale() = 1.0;
        s.ev->multiply_plain_inplace(x, p);
        store_ct(s, x, out);
    })
}

// CKKSEncoder::encode of n complex values (re, im) at `scale` for a level
// with `limbs` primes; writes [limbs][N].
int sr_encode(void *h, const double *re, const double *im, size_t nvals, double scale, int limbs, uint64_t *out)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        std::vector<std::complex<double>> v(nvals);
        for (size_t i = 0; i < nvals; ++i) v[i] = {re[i], im ? im[i] : 0.0};
        Plaintext p;
        s.enc->encode(v, pid_for_limbs(s, limbs), scale, p);
        std::memcpy(out, p.data(), sizeof(uint64_t) * s.n * limbs);
    })
}

// CKKSEncoder::encode(double) -- the scalar path
int sr_encode_scalar(void *h, double value, double scale, int limbs, uint64_t *out)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        Plaintext p;
        s.enc->encode(value, pid_for_limbs(s, limbs), scale, p);
        std::memcpy(out, p.data(), sizeof(uint64_t) * s.n * limbs);
    })
}

// decode of a plaintext [limbs][N] into nvals complex values
int sr_decode(void *h, const uint64_t *pt, int limbs, double scale, double *re, double *im, size_t nvals)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        Plaintext p;
        p.resize(s.n * limbs);
        std::memcpy(p.data(), pt, sizeof(uint64_t) * s.n * limbs);
        p.parms_id() = pid_for_limbs(s, limbs);
        p.scale() = scale;
        std::vector<std::complex<double>> v;
        s.enc->decode(p, v);
        for (size_t i = 0; i < nvals && i < v.size(); ++i) {
            re[i] = v[i].real();
            if (im) im[i] = v[i].imag();
        }
    })
}

int sr_encrypt(void *h, const double *vals, size_t nvals, double scale, uint64_t *out)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        std::vector<double> v(vals, vals + nvals);
        Plaintext p;
        s.enc->encode(v, scale, p);
        Ciphertext c;
        s.encryptor->encrypt(p, c);
        store_ct(s, c, out);
    })
}

int sr_decrypt(void *h, const uint64_t *ct, int limbs, double scale, double *out, size_t nvals)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        Ciphertext c;
        load_ct(s, c, ct, 2, limbs, scale);
        Plaintext p;
        s.decryptor->decrypt(c, p);
        std::vector<double> v;
        s.enc->decode(p, v);
        for (size_t i = 0; i < nvals && i < v.size(); ++i) out[i] = v[i];
    })
}

// Run one NEXUS operator on a ciphertext [2][limbs][N] at in_scale with the
// shim's keys: op 0 GeLUEvaluator::gelu, 1 SoftmaxEvaluator::softmax(len=a1),
// 2 LNEvaluator::layer_norm(len=a1), 3 CKKSEvaluator::sgn_eval(a1, a2, f),
// 4 exp, 5 inverse(iter=a1), 6 invert_sqrt(a1, a2).  `base_scale` is the
// CKKSEvaluator's scale.  Writes the output and its limbs/scale.
int sr_nexus_op(void *h, int op, const uint64_t *in, int limbs, double in_scale, double base_scale, int a1, int a2,
                double f, uint64_t *out, int *out_limbs, double *out_scale)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        Ciphertext x, res;
        load_ct(s, x, in, 2, limbs, in_scale);
        CKKSEvaluator ck(*s.ctx, *s.encryptor, *s.decryptor, *s.enc, *s.ev, base_scale, *s.rk, *s.gk);
        switch (op) {
        case 0: { GeLUEvaluator g(ck); g.gelu(x, res); break; }
        case 1: { SoftmaxEvaluator sm(ck); sm.softmax(x, res, a1); break; }
        case 2: { LNEvaluator ln(ck); ln.layer_norm(x, res, a1); break; }
        case 3: res = ck.sgn_eval(x, a1, a2, f); break;
        case 4: res = ck.exp(x); break;
        case 5: res = ck.inverse(x, a1); break;
        case 6: res = ck.invert_sqrt(x, a1, a2); break;
        default: throw std::invalid_argument("unknown op");
        }
        store_ct(s, res, out);
        *out_limbs = (int)res.coeff_modulus_size();
        *out_scale = res.scale();
    })
}

// Fork ops of the bootstrapping SEAL (evaluator.cpp:395-590 / evaluator.h:1296-1386):
// op 0 add_const(a, v), 1 multiply_const(a, v), 2 add_reduced_error(a, b),
// 3 sub_reduced_error(a, b), 4 multiply_reduced_error(a, b),
// 5 multiply_vector_reduced_error(a, complex values re/im of length nv)
int sr_fork_op(void *h, int op, const uint64_t *a, int la, double sa, const uint64_t *b, int lb, double sb,
               double v, const double *re, const double *im, size_t nv, uint64_t *out, int *out_size, int *out_limbs,
               double *out_scale)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        Ciphertext x, y, r;
        load_ct(s, x, a, 2, la, sa);
        if (b) load_ct(s, y, b, 2, lb, sb);
        switch (op) {
        case 0: s.ev->add_const(x, v, r); break;
        case 1: s.ev->multiply_const(x, v, r); break;
        case 2: s.ev->add_reduced_error(x, y, r); break;
        case 3: s.ev->sub_reduced_error(x, y, r); break;
        case 4: s.ev->multiply_reduced_error(x, y, *s.rk, r); break;
        case 5: {
            std::vector<std::complex<double>> vec(nv);
            for (size_t i = 0; i < nv; ++i) vec[i] = {re[i], im[i]};
            s.ev->multiply_vector_reduced_error(x, vec, r);
            break;
        }
        default: throw std::invalid_argument("unknown op");
        }
        store_ct(s, r, out);
        *out_size = (int)r.size();
        *out_limbs = (int)r.coeff_modulus_size();
        *out_scale = r.scale();
    })
}

// Galois keys for explicit elements (the MatMul expansion uses elements, not steps)
int sr_galois_keys_from_elts(void *h, const uint32_t *elts, int n)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        s.gk.reset(new GaloisKeys());
        s.kg->create_galois_keys(std::vector<uint32_t>(elts, elts + n), *s.gk);
    })
}

// MMEvaluator::enc_compress_ciphertext (src/matrix_mul.cpp:58-99): N values -> ct at the top level
int sr_mm_compress(void *h, const double *vals, double scale, uint64_t *out, double *out_scale)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        CKKSEvaluator ck(*s.ctx, *s.encryptor, *s.decryptor, *s.enc, *s.ev, scale, *s.rk, *s.gk);
        MMEvaluator mm(ck);
        std::vector<double> v(vals, vals + s.n);
        Ciphertext ct;
        mm.enc_compress_ciphertext(v, ct);
        store_ct(s, ct, out);
        *out_scale = ct.scale();
    })
}

// MMEvaluator::multiply_power_of_x (src/matrix_mul.cpp:131-172)
int sr_mm_power_of_x(void *h, const uint64_t *in, int limbs, int index, uint64_t *out)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        CKKSEvaluator ck(*s.ctx, *s.encryptor, *s.decryptor, *s.enc, *s.ev, 1.0, *s.rk, *s.gk);
        MMEvaluator mm(ck);
        Ciphertext x, d;
        load_ct(s, x, in, 2, limbs, 1.0);
        mm.multiply_power_of_x(x, d, index);
        store_ct(s, d, out);
    })
}

// MMEvaluator::expand_ciphertext (src/matrix_mul.cpp:101-129) with m leaves,
// galois elements ckks->rots; out [m][2][limbs][N]
int sr_mm_expand(void *h, const uint64_t *in, int limbs, double scale, uint32_t m, uint64_t *out)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        CKKSEvaluator ck(*s.ctx, *s.encryptor, *s.decryptor, *s.enc, *s.ev, 1.0, *s.rk, *s.gk);
        MMEvaluator mm(ck);
        Ciphertext x;
        load_ct(s, x, in, 2, limbs, scale);
        auto leaves = mm.expand_ciphertext(x, m, *s.gk, ck.rots);
        size_t per = 2 * (size_t)limbs * s.n;
        for (size_t i = 0; i < leaves.size(); ++i) std::memcpy(out + i * per, leaves[i].data(), per * 8);
    })
}

// Ciphertext::save / load with compr_mode_type::none, and a level's parms_id
int sr_parms_id(void *h, int limbs, uint64_t *out)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        auto pid = pid_for_limbs(s, limbs);
        for (int i = 0; i < 4; ++i) out[i] = pid[i];
    })
}

int sr_ct_save(void *h, const uint64_t *in, int size, int limbs, double scale, uint8_t *out, size_t cap,
               size_t *written)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        Ciphertext ct;
        load_ct(s, ct, in, size, limbs, scale);
        std::stringstream ss;
        ct.save(ss, compr_mode_type::none);
        const std::string b = ss.str();
        *written = b.size();
        if (out) {
            if (cap < b.size()) throw std::invalid_argument("buffer too small");
            std::memcpy(out, b.data(), b.size());
        }
    })
}

int sr_ct_load(void *h, const uint8_t *in, size_t len, uint64_t *out, int *size, int *limbs, double *scale)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        Ciphertext ct;
        std::stringstream ss(std::string(reinterpret_cast<const char *>(in), len));
        ct.load(*s.ctx, ss);
        *size = (int)ct.size();
        *limbs = (int)ct.coeff_modulus_size();
        *scale = ct.scale();
        if (out) store_ct(s, ct, out);
    })
}

// ---- seeded randomness (key generation and encryption) ----------------

namespace {
// A factory that hands create() calls the seeds of a list in order, so every
// Blake2xbPRNG SEAL makes (one per sampled key, digit and encryption) gets
// its own known seed.  Test infrastructure only.
class SeedListFactory : public UniformRandomGeneratorFactory {
public:
    explicit SeedListFactory(std::vector<prng_seed_type> seeds)
        : UniformRandomGeneratorFactory(prng_seed_type{}), seeds_(std::move(seeds))
    {}

protected:
    auto create_impl(prng_seed_type) -> std::shared_ptr<UniformRandomGenerator> override
    {
        if (next_ >= seeds_.size()) throw std::logic_error("seed list exhausted");
        return std::make_shared<Blake2xbPRNG>(seeds_[next_++]);
    }

private:
    std::vector<prng_seed_type> seeds_;
    size_t next_ = 0;
};
}  // namespace

// sr_create whose PRNG factory gives create() call i the seed seeds[i] (8 words each)
void *sr_create_seed_list(int logn, const uint64_t *moduli, int k, const uint64_t *seeds, int nseeds,
                          int hamming_weight)
{
    auto *s = static_cast<Shim *>(sr_create(logn, moduli, k, 0, hamming_weight));
    if (!s) return nullptr;
    try {
        EncryptionParameters parms = s->ctx->key_context_data()->parms();
        std::vector<prng_seed_type> list((size_t)nseeds);
        for (int i = 0; i < nseeds; ++i)
            for (size_t w = 0; w < list[i].size(); ++w) list[i][w] = seeds[(size_t)i * 8 + w];
        parms.set_random_generator(std::make_shared<SeedListFactory>(std::move(list)));
        s->ctx.reset(new SEALContext(parms, true, sec_level_type::none));
        s->enc.reset(new CKKSEncoder(*s->ctx));
        s->ev.reset(new Evaluator(*s->ctx, *s->enc));
        return s;
    } catch (const std::exception &e) {
        g_err = e.what();
        delete s;
        return nullptr;
    }
}

// sr_create with the full 8-word seed of the Blake2xbPRNGFactory
void *sr_create_seeded(int logn, const uint64_t *moduli, int k, const uint64_t *seed, int hamming_weight)
{
    auto *s = static_cast<Shim *>(sr_create(logn, moduli, k, 0, hamming_weight));
    if (!s) return nullptr;
    try {
        EncryptionParameters parms = s->ctx->key_context_data()->parms();
        prng_seed_type sd{};
        for (size_t i = 0; i < sd.size(); ++i) sd[i] = seed[i];
        parms.set_random_generator(std::make_shared<Blake2xbPRNGFactory>(sd));
        s->ctx.reset(new SEALContext(parms, true, sec_level_type::none));
        s->enc.reset(new CKKSEncoder(*s->ctx));
        s->ev.reset(new Evaluator(*s->ctx, *s->enc));
        return s;
    } catch (const std::exception &e) {
        g_err = e.what();
        delete s;
        return nullptr;
    }
}

// public key [2][K][N]
int sr_export_public(void *h, uint64_t *out)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD(std::memcpy(out, s.pk->data().data(), sizeof(uint64_t) * 2 * s.k * s.n))
}

// Encryptor::encrypt (symmetric = 0, public key) or encrypt_symmetric of the
// NTT-form plaintext pt [limbs][N] at `scale` into out [2][limbs][N]
int sr_encrypt_ntt(void *h, const uint64_t *pt, int limbs, double scale, int symmetric, uint64_t *out)
{
    auto &s = *static_cast<Shim *>(h);
    GUARD({
        Plaintext p;
        p.parms_id() = parms_id_zero;
        p.resize(limbs * s.n);
        std::memcpy(p.data(), pt, sizeof(uint64_t) * limbs * s.n);
        p.parms_id() = pid_for_limbs(s, limbs);
        p.scale() = scale;
        Ciphertext c;
        if (symmetric) {
            Encryptor e(*s.ctx, *s.sk);
            e.encrypt_symmetric(p, c);
        } else {
            Encryptor e(*s.ctx, *s.pk);
            e.encrypt(p, c);
        }
        store_ct(s, c, out);
    })
}

// bytes [offset, offset + n) of the Blake2xbPRNG stream of an 8-word seed
int sr_prng_bytes(const uint64_t *seed, uint64_t offset, size_t n, uint8_t *out)
{
    GUARD({
        prng_seed_type sd{};
        for (size_t i = 0; i < sd.size(); ++i) sd[i] = seed[i];
        Blake2xbPRNG g(sd);
        std::vector<seal_byte> skip(4096);
        while (offset) {
            size_t t = (size_t)std::min<uint64_t>(offset, skip.size());
            g.generate(t, skip.data());
            offset -= t;
        }
        g.generate(n, reinterpret_cast<seal_byte *>(out));
    })
}

}  // extern "C"
