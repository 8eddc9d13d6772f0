/*
 * nexus_oracle.c -- CPU restatement of the SEAL-4.1-bs CKKS arithmetic that the
 * NEXUS encrypted-inference path runs on.
 *
 * THIS FILE IS TEST INFRASTRUCTURE.  It is the parity checker for the CUDA
 * engine in nexus_gb300/: only the tests, the smoke check and the CPU-baseline
 * leg of bench.py load it.  The engine never links or calls it.
 *
 * Every function restates one SEAL routine (paths are relative to
 * thirdparty/SEAL-4.1-bs/native/src/seal in the NEXUS tree) and keeps that
 * routine's loop structure, lazy ranges and rounding, so that every output
 * word equals SEAL's.  Plain C99 + unsigned __int128, no intrinsics, so it
 * builds and gives identical results on x86-64 and aarch64.
 *
 * Layout conventions (identical to SEAL's, so import/export is a memcpy):
 *   a polynomial in RNS form is uint64[limbs][N] (limb-major);
 *   a ciphertext is uint64[size][limbs][N];
 *   a key-switching key is uint64[digits][2][K][N] where K counts every prime
 *   of the key level (data primes then the special prime).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

typedef unsigned __int128 u128;

/* ------------------------------------------------------------------ */
/* scalar modular arithmetic                                            */
/* ------------------------------------------------------------------ */

static uint64_t mulmod(uint64_t a, uint64_t b, uint64_t q) { return (uint64_t)(((u128)a * b) % q); }

static uint64_t powmod(uint64_t b, uint64_t e, uint64_t q)
{
    uint64_t r = 1 % q;
    b %= q;
    while (e) {
        if (e & 1) r = mulmod(r, b, q);
        b = mulmod(b, b, q);
        e >>= 1;
    }
    return r;
}

/* modular inverse by extended Euclid; returns 0 when not invertible */
static uint64_t invmod(uint64_t a, uint64_t q)
{
    __int128 t = 0, nt = 1, r = q, nr = a % q;
    while (nr) {
        __int128 qt = r / nr, tmp;
        tmp = t - qt * nt; t = nt; nt = tmp;
        tmp = r - qt * nr; r = nr; nr = tmp;
    }
    if (r != 1) return 0;
    if (t < 0) t += q;
    return (uint64_t)t;
}

/* floor(w * 2^64 / q): the quotient of SEAL's MultiplyUIntModOperand
 * (util/uintarithsmallmod.h:255-285). */
static uint64_t shoup(uint64_t w, uint64_t q) { return (uint64_t)((((u128)w) << 64) / q); }

/* multiply_uint_mod_lazy (util/uintarithsmallmod.h): result in [0, 2q) */
static inline uint64_t mul_lazy(uint64_t x, uint64_t w, uint64_t wq, uint64_t q)
{
    uint64_t hi = (uint64_t)(((u128)x * wq) >> 64);
    return x * w - hi * q;
}

/* Deterministic Miller-Rabin for 64-bit inputs.  SEAL's is_prime
 * (util/numth.cpp) draws random bases; for 64-bit inputs the fixed base set
 * below answers identically. */
static int is_prime_u64(uint64_t n)
{
    static const uint64_t bases[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    if (n < 2) return 0;
    for (int i = 0; i < 12; i++) {
        if (n == bases[i]) return 1;
        if (n % bases[i] == 0) return 0;
    }
    uint64_t d = n - 1;
    int s = 0;
    while (!(d & 1)) { d >>= 1; s++; }
    for (int i = 0; i < 12; i++) {
        uint64_t x = powmod(bases[i], d, n);
        if (x == 1 || x == n - 1) continue;
        int comp = 1;
        for (int r = 1; r < s; r++) {
            x = mulmod(x, x, n);
            if (x == n - 1) { comp = 0; break; }
        }
        if (comp) return 0;
    }
    return 1;
}

/* ------------------------------------------------------------------ */
/* parameter generation                                                 */
/* ------------------------------------------------------------------ */

/* CoeffModulus::Create (modulus.cpp:143-184) over get_primes
 * (util/numth.cpp:278-311): primes p = 1 mod 2N scanned downward from
 * 2^bits; a bit size that appears several times takes its primes from the
 * SMALLEST upward (prime_table[size].back() then pop_back()).
 * Returns 0 on success. */
int or_create_coeff_modulus(uint64_t n, const int *bit_sizes, int count, uint64_t *out)
{
    uint64_t factor = 2 * n;
    for (int i = 0; i < count; i++) {
        int size = bit_sizes[i];
        int total = 0, rank = 0;
        for (int j = 0; j < count; j++) {
            if (bit_sizes[j] == size) {
                if (j < i) rank++;
                total++;
            }
        }
        /* descending list has `total` entries; position i takes entry total-1-rank */
        int want = total - 1 - rank;
        uint64_t value = ((((uint64_t)1) << size) - 1) / factor * factor + 1;
        uint64_t lower = ((uint64_t)1) << (size - 1);
        int found = -1;
        while (value > lower) {
            if (is_prime_u64(value)) {
                found++;
                if (found == want) break;
            }
            value -= factor;
        }
        if (found != want) return -1;
        out[i] = value;
    }
    return 0;
}

/* try_minimal_primitive_root (util/numth.cpp:386-412): the smallest primitive
 * degree-th root of unity.  SEAL seeds the search with a random element; the
 * minimum over all primitive roots does not depend on that seed, so this
 * restatement starts from the first generator it finds. */
uint64_t or_minimal_primitive_root(uint64_t degree, uint64_t q)
{
    uint64_t group = q - 1;
    if (group % degree) return 0;
    uint64_t quo = group / degree, root = 0;
    for (uint64_t g = 2; g < q; g++) {
        uint64_t c = powmod(g, quo, q);
        if (c && powmod(c, degree >> 1, q) == q - 1) { root = c; break; }
    }
    if (!root) return 0;
    uint64_t gsq = mulmod(root, root, q), cur = root, best = root;
    for (uint64_t i = 0; i < degree; i += 2) {
        if (cur < best) best = cur;
        cur = mulmod(cur, gsq, q);
    }
    return best;
}

static uint32_t reverse_bits(uint32_t x, int bits)
{
    uint32_t r = 0;
    for (int i = 0; i < bits; i++) { r = (r << 1) | (x & 1); x >>= 1; }
    return r;
}

/* ------------------------------------------------------------------ */
/* context: per-prime NTT tables                                        */
/* ------------------------------------------------------------------ */

typedef struct {
    int logn;
    uint64_t n;
    int k;                 /* number of primes (data primes + special prime) */
    uint64_t *q;           /* [k] */
    uint64_t *root;        /* [k] minimal primitive 2N-th root */
    uint64_t *rp, *rpq;    /* [k][n] root powers (bit-reversed) + Shoup quotients */
    uint64_t *irp, *irpq;  /* [k][n] inverse root powers (scrambled order) */
    uint64_t *inv_n, *inv_n_q; /* [k] */
} or_ctx;

/* NTTTables::initialize (util/ntt.cpp:241-300) */
static void build_tables(or_ctx *c, int j)
{
    uint64_t q = c->q[j], n = c->n;
    uint64_t root = or_minimal_primitive_root(2 * n, q);
    uint64_t inv_root = invmod(root, q);
    c->root[j] = root;
    uint64_t *rp = c->rp + j * n, *rpq = c->rpq + j * n;
    uint64_t *irp = c->irp + j * n, *irpq = c->irpq + j * n;
    uint64_t power = root;
    for (uint64_t i = 1; i < n; i++) {
        uint32_t idx = reverse_bits((uint32_t)i, c->logn);
        rp[idx] = power;
        power = mulmod(power, root, q);
    }
    rp[0] = 1;
    power = inv_root;
    for (uint64_t i = 1; i < n; i++) {
        uint32_t idx = reverse_bits((uint32_t)(i - 1), c->logn) + 1;
        irp[idx] = power;
        power = mulmod(power, inv_root, q);
    }
    irp[0] = 1;
    for (uint64_t i = 0; i < n; i++) {
        rpq[i] = shoup(rp[i], q);
        irpq[i] = shoup(irp[i], q);
    }
    c->inv_n[j] = invmod(n % q, q);
    c->inv_n_q[j] = shoup(c->inv_n[j], q);
}

or_ctx *or_ctx_create(int logn, const uint64_t *moduli, int k)
{
    or_ctx *c = (or_ctx *)calloc(1, sizeof(or_ctx));
    if (!c) return NULL;
    c->logn = logn;
    c->n = (uint64_t)1 << logn;
    c->k = k;
    c->q = (uint64_t *)malloc(sizeof(uint64_t) * k);
    c->root = (uint64_t *)malloc(sizeof(uint64_t) * k);
    c->inv_n = (uint64_t *)malloc(sizeof(uint64_t) * k);
    c->inv_n_q = (uint64_t *)malloc(sizeof(uint64_t) * k);
    size_t tb = sizeof(uint64_t) * (size_t)k * c->n;
    c->rp = (uint64_t *)malloc(tb);
    c->rpq = (uint64_t *)malloc(tb);
    c->irp = (uint64_t *)malloc(tb);
    c->irpq = (uint64_t *)malloc(tb);
    memcpy(c->q, moduli, sizeof(uint64_t) * k);
    for (int j = 0; j < k; j++) build_tables(c, j);
    return c;
}

void or_ctx_destroy(or_ctx *c)
{
    if (!c) return;
    free(c->q); free(c->root); free(c->inv_n); free(c->inv_n_q);
    free(c->rp); free(c->rpq); free(c->irp); free(c->irpq);
    free(c);
}

uint64_t or_ctx_root(const or_ctx *c, int j) { return c->root[j]; }

void or_ctx_root_powers(const or_ctx *c, int j, uint64_t *out, uint64_t *inv_out)
{
    memcpy(out, c->rp + (size_t)j * c->n, sizeof(uint64_t) * c->n);
    memcpy(inv_out, c->irp + (size_t)j * c->n, sizeof(uint64_t) * c->n);
}

/* ------------------------------------------------------------------ */
/* negacyclic NTT                                                       */
/* ------------------------------------------------------------------ */

/* DWTHandler::transform_to_rev (util/dwthandler.h:94-190) with the modular
 * Arithmetic of util/ntt.h:21-67: inputs in [0,4q), outputs in [0,4q). */
static void ntt_lazy(uint64_t *a, const or_ctx *c, int j)
{
    uint64_t q = c->q[j], two_q = 2 * q;
    const uint64_t *rp = c->rp + (size_t)j * c->n, *rq = c->rpq + (size_t)j * c->n;
    size_t n = c->n, gap = n >> 1, m = 1, ridx = 0;
    for (; m < (n >> 1); m <<= 1) {
        size_t off = 0;
        for (size_t i = 0; i < m; i++) {
            ++ridx;
            uint64_t w = rp[ridx], wq = rq[ridx];
            uint64_t *x = a + off, *y = x + gap;
            for (size_t t = 0; t < gap; t++) {
                uint64_t u = x[t] >= two_q ? x[t] - two_q : x[t];
                uint64_t v = mul_lazy(y[t], w, wq, q);
                x[t] = u + v;
                y[t] = u + two_q - v;
            }
            off += gap << 1;
        }
        gap >>= 1;
    }
    for (size_t i = 0; i < m; i++) {
        ++ridx;
        uint64_t w = rp[ridx], wq = rq[ridx];
        uint64_t u = a[0] >= two_q ? a[0] - two_q : a[0];
        uint64_t v = mul_lazy(a[1], w, wq, q);
        a[0] = u + v;
        a[1] = u + two_q - v;
        a += 2;
    }
}

/* DWTHandler::transform_from_rev (util/dwthandler.h:200-280) with the n^{-1}
 * scalar merged into the last stage: inputs in [0,2q), outputs in [0,2q). */
static void intt_lazy(uint64_t *a, const or_ctx *c, int j)
{
    uint64_t q = c->q[j], two_q = 2 * q;
    const uint64_t *rp = c->irp + (size_t)j * c->n, *rq = c->irpq + (size_t)j * c->n;
    size_t n = c->n, gap = 1, m = n >> 1, ridx = 0;
    for (; m > 1; m >>= 1) {
        size_t off = 0;
        for (size_t i = 0; i < m; i++) {
            ++ridx;
            uint64_t w = rp[ridx], wq = rq[ridx];
            uint64_t *x = a + off, *y = x + gap;
            for (size_t t = 0; t < gap; t++) {
                uint64_t u = x[t], v = y[t];
                uint64_t s = u + v;
                x[t] = s >= two_q ? s - two_q : s;
                y[t] = mul_lazy(u + two_q - v, w, wq, q);
            }
            off += gap << 1;
        }
        gap <<= 1;
    }
    /* last stage with the scalar n^{-1} merged (dwthandler.h:273-290) */
    ++ridx;
    uint64_t s = c->inv_n[j], sq = c->inv_n_q[j];
    uint64_t r = rp[ridx];
    uint64_t sr = mulmod(r, s, q), srq = shoup(sr, q);
    for (size_t t = 0; t < gap; t++) {
        uint64_t u = a[t] >= two_q ? a[t] - two_q : a[t];
        uint64_t v = a[t + gap];
        uint64_t sum = u + v;
        if (sum >= two_q) sum -= two_q;
        a[t] = mul_lazy(sum, s, sq, q);
        a[t + gap] = mul_lazy(u + two_q - v, sr, srq, q);
    }
}

/* ntt_negacyclic_harvey (util/ntt.cpp:408-430): lazy transform then reduce
 * [0,4q) -> [0,q). */
static void ntt_full(uint64_t *a, const or_ctx *c, int j)
{
    uint64_t q = c->q[j], two_q = 2 * q;
    ntt_lazy(a, c, j);
    for (size_t i = 0; i < c->n; i++) {
        uint64_t x = a[i];
        if (x >= two_q) x -= two_q;
        if (x >= q) x -= q;
        a[i] = x;
    }
}

/* inverse_ntt_negacyclic_harvey (util/ntt.cpp:445-470) */
static void intt_full(uint64_t *a, const or_ctx *c, int j)
{
    uint64_t q = c->q[j];
    intt_lazy(a, c, j);
    for (size_t i = 0; i < c->n; i++) {
        uint64_t x = a[i];
        if (x >= q) x -= q;
        a[i] = x;
    }
}

/* ---- worker threads ----
 * or_set_threads(t) makes the key switch and the rescale below spread their
 * independent per-prime loops over t threads (1: the calling thread only).
 * Every output word is computed by the same arithmetic whatever the count. */

static int g_threads = 1;

void or_set_threads(int t) { g_threads = t < 1 ? 1 : (t > 256 ? 256 : t); }
int or_get_threads(void) { return g_threads; }

typedef void (*pf_fn)(void *arg, int idx, int tid);

typedef struct {
    pf_fn fn;
    void *arg;
    int count, next;
    pthread_mutex_t mu;
} pf_job;

typedef struct {
    pf_job *job;
    int tid;
} pf_worker_arg;

static void *pf_worker(void *p)
{
    pf_worker_arg *w = (pf_worker_arg *)p;
    pf_job *j = w->job;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        int i = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (i >= j->count) break;
        j->fn(j->arg, i, w->tid);
    }
    return NULL;
}

/* fn(arg, i, tid) for i in [0, count); tid < parallel_width(count) */
static int parallel_width(int count) { return count < g_threads ? (count < 1 ? 1 : count) : g_threads; }

static void parallel_for(int count, pf_fn fn, void *arg)
{
    int nt = parallel_width(count);
    if (nt <= 1) {
        for (int i = 0; i < count; i++) fn(arg, i, 0);
        return;
    }
    pf_job job;
    job.fn = fn; job.arg = arg; job.count = count; job.next = 0;
    pthread_mutex_init(&job.mu, NULL);
    pthread_t th[256];
    pf_worker_arg wa[256];
    for (int t = 0; t < nt; t++) {
        wa[t].job = &job;
        wa[t].tid = t;
        pthread_create(&th[t], NULL, pf_worker, &wa[t]);
    }
    for (int t = 0; t < nt; t++) pthread_join(th[t], NULL);
    pthread_mutex_destroy(&job.mu);
}

/* ---- threaded batch driver over [poly][limb][N] ---- */

typedef struct {
    const or_ctx *c;
    uint64_t *data;
    size_t n_polys, limb_begin, limb_count, next, total;
    int inverse;
    pthread_mutex_t mu;
} batch_job;

static void *batch_worker(void *arg)
{
    batch_job *b = (batch_job *)arg;
    for (;;) {
        pthread_mutex_lock(&b->mu);
        size_t t = b->next++;
        pthread_mutex_unlock(&b->mu);
        if (t >= b->total) break;
        size_t limb = t % b->limb_count;
        uint64_t *p = b->data + t * b->c->n;
        int j = (int)(b->limb_begin + limb);
        if (b->inverse) intt_full(p, b->c, j); else ntt_full(p, b->c, j);
    }
    return NULL;
}

/* Forward/inverse NTT of n_polys polynomials whose limbs use primes
 * [limb_begin, limb_end) of the context; data is [n_polys][limbs][N].
 * nthreads <= 1 runs on the calling thread. */
void or_ntt_batch(const or_ctx *c, uint64_t *data, size_t n_polys, size_t limb_begin, size_t limb_end,
                  int inverse, int nthreads)
{
    batch_job b;
    b.c = c; b.data = data; b.n_polys = n_polys; b.limb_begin = limb_begin;
    b.limb_count = limb_end - limb_begin; b.next = 0; b.total = n_polys * b.limb_count;
    b.inverse = inverse;
    pthread_mutex_init(&b.mu, NULL);
    if (nthreads <= 1) {
        batch_worker(&b);
    } else {
        pthread_t th[256];
        if (nthreads > 256) nthreads = 256;
        for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, batch_worker, &b);
        for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
    }
    pthread_mutex_destroy(&b.mu);
}

/* single limb, lazy output (ntt_negacyclic_harvey_lazy, util/ntt.cpp:394) */
void or_ntt_lazy_limb(const or_ctx *c, uint64_t *a, int j) { ntt_lazy(a, c, j); }

/* ------------------------------------------------------------------ */
/* rescale                                                              */
/* ------------------------------------------------------------------ */

typedef struct {
    const or_ctx *c;
    uint64_t *polys;   /* [size][limbs][N] working copy */
    int limbs;
    uint64_t *tmp;     /* [threads][N] */
} rs_job;

/* the dropped limb of every polynomial: INTT and +q_last/2 (add_poly_scalar_coeffmod) */
static void rs_last_task(void *arg, int s, int tid)
{
    (void)tid;
    rs_job *j = (rs_job *)arg;
    const or_ctx *c = j->c;
    size_t n = c->n;
    int last = j->limbs - 1;
    uint64_t *li = j->polys + ((size_t)s * j->limbs + last) * n;
    uint64_t ql = c->q[last];
    intt_full(li, c, last);
    uint64_t half = ql >> 1;
    for (size_t t = 0; t < n; t++) li[t] = (li[t] + half) % ql;
}

/* limb i of polynomial s: (c_i - NTT(last mod q_i - half)) * q_last^-1 */
static void rs_limb_task(void *arg, int idx, int tid)
{
    rs_job *j = (rs_job *)arg;
    const or_ctx *c = j->c;
    size_t n = c->n;
    int last = j->limbs - 1;
    int s = idx / last, i = idx % last;
    uint64_t *poly = j->polys + (size_t)s * j->limbs * n;
    const uint64_t *li = poly + (size_t)last * n;
    uint64_t ql = c->q[last], half = ql >> 1;
    uint64_t *tmp = j->tmp + (size_t)tid * n;
    uint64_t qi = c->q[i];
    for (size_t t = 0; t < n; t++) tmp[t] = (qi < ql) ? li[t] % qi : li[t];
    uint64_t neg_half_mod = qi - (half % qi);
    for (size_t t = 0; t < n; t++) tmp[t] += neg_half_mod;
    uint64_t qi_lazy = qi << 2;
    ntt_lazy(tmp, c, i);
    uint64_t *ci = poly + (size_t)i * n;
    uint64_t inv = invmod(ql % qi, qi);
    for (size_t t = 0; t < n; t++) {
        uint64_t x = ci[t] + qi_lazy - tmp[t];
        ci[t] = mulmod(x, inv, qi);
    }
}

/* Evaluator::rescale_to_next (evaluator.cpp:1402-1480, 1682) on a ciphertext
 * [size][limbs][N]; writes [size][limbs-1][N] into out (may alias in).  Each
 * polynomial follows RNSTool::divide_and_round_q_last_ntt_inplace
 * (util/rns.cpp:830-905): INTT of the last limb, +q_last/2, then for every
 * other limb reduce, subtract the rounding offset, NTT-lazy, subtract and
 * multiply by q_last^-1 mod q_i. */
void or_rescale_ntt(const or_ctx *c, const uint64_t *in, int size, int limbs, uint64_t *out)
{
    size_t n = c->n;
    rs_job j;
    j.c = c;
    j.limbs = limbs;
    j.polys = (uint64_t *)malloc(sizeof(uint64_t) * n * limbs * size);
    memcpy(j.polys, in, sizeof(uint64_t) * n * limbs * size);
    int tasks = size * (limbs - 1);
    j.tmp = (uint64_t *)malloc(sizeof(uint64_t) * n * parallel_width(tasks));
    parallel_for(size, rs_last_task, &j);
    parallel_for(tasks, rs_limb_task, &j);
    for (int s = 0; s < size; s++)
        memmove(out + (size_t)s * (limbs - 1) * n, j.polys + (size_t)s * limbs * n, sizeof(uint64_t) * n * (limbs - 1));
    free(j.polys);
    free(j.tmp);
}

/* mod_switch_drop_to_next (evaluator.cpp:1483-1546): drop the last limb */
void or_drop_last_limb(const or_ctx *c, const uint64_t *in, int size, int limbs, uint64_t *out)
{
    size_t n = c->n;
    for (int s = 0; s < size; s++)
        memmove(out + (size_t)s * (limbs - 1) * n, in + (size_t)s * limbs * n, sizeof(uint64_t) * n * (limbs - 1));
}

/* ------------------------------------------------------------------ */
/* key switching                                                        */
/* ------------------------------------------------------------------ */

typedef struct {
    const or_ctx *c;
    uint64_t *ct;
    int ell, K, sp, rns;
    const uint64_t *target, *key;
    uint64_t *tt;     /* [ell][N] target in coefficient form */
    uint64_t *prod;   /* [2][rns][N] inner products */
    uint64_t *tntt;   /* [threads][N] */
    u128 *acc;        /* [threads][2][N] */
} ks_job;

static void ks_intt_task(void *arg, int j, int tid)
{
    (void)tid;
    ks_job *k = (ks_job *)arg;
    intt_full(k->tt + (size_t)j * k->c->n, k->c, j);
}

/* output prime I (the special prime when I == ell): every digit J reduced
 * into q_I and transformed (the target's own limb when I == J), times the
 * key's J-th digit, accumulated in 128 bits, one Barrett reduction */
static void ks_modup_task(void *arg, int I, int tid)
{
    ks_job *k = (ks_job *)arg;
    const or_ctx *c = k->c;
    size_t n = c->n;
    int ell = k->ell, K = k->K;
    int ki = (I == ell) ? k->sp : I;
    uint64_t qk = c->q[ki];
    uint64_t *tntt = k->tntt + (size_t)tid * n;
    u128 *acc = k->acc + (size_t)tid * 2 * n;
    memset(acc, 0, sizeof(u128) * 2 * n);
    for (int J = 0; J < ell; J++) {
        const uint64_t *op;
        if (I == J) {
            op = k->target + (size_t)J * n;
        } else {
            const uint64_t *src = k->tt + (size_t)J * n;
            if (c->q[J] <= qk) memcpy(tntt, src, sizeof(uint64_t) * n);
            else for (size_t t = 0; t < n; t++) tntt[t] = src[t] % qk;
            ntt_lazy(tntt, c, ki);
            op = tntt;
        }
        for (int comp = 0; comp < 2; comp++) {
            const uint64_t *kp = k->key + (((size_t)J * 2 + comp) * K + ki) * n;
            u128 *a = acc + (size_t)comp * n;
            for (size_t t = 0; t < n; t++) a[t] += (u128)op[t] * kp[t];
        }
    }
    /* ell < 256 always, so the final Barrett reduction applies
     * (the lazy counter never wraps) */
    for (int comp = 0; comp < 2; comp++) {
        uint64_t *dst = k->prod + ((size_t)comp * k->rns + I) * n;
        u128 *a2 = acc + (size_t)comp * n;
        for (size_t t = 0; t < n; t++) dst[t] = (uint64_t)(a2[t] % qk);
    }
}

/* special-prime limb of component comp: INTT and +q_k/2 */
static void ks_special_task(void *arg, int comp, int tid)
{
    (void)tid;
    ks_job *k = (ks_job *)arg;
    const or_ctx *c = k->c;
    size_t n = c->n;
    uint64_t qk = c->q[k->sp], qk_half = qk >> 1;
    uint64_t *tl = k->prod + ((size_t)comp * k->rns + k->ell) * n;
    intt_lazy(tl, c, k->sp);
    for (size_t t = 0; t < n; t++) tl[t] = (tl[t] + qk_half) % qk;
}

/* ModDown of component comp into data prime i, added into the ciphertext */
static void ks_moddown_task(void *arg, int idx, int tid)
{
    ks_job *k = (ks_job *)arg;
    const or_ctx *c = k->c;
    size_t n = c->n;
    int ell = k->ell;
    int comp = idx / ell, i = idx % ell;
    uint64_t qk = c->q[k->sp], qk_half = qk >> 1;
    const uint64_t *tl = k->prod + ((size_t)comp * k->rns + ell) * n;
    uint64_t *tntt = k->tntt + (size_t)tid * n;
    uint64_t qi = c->q[i];
    for (size_t t = 0; t < n; t++) tntt[t] = (qk > qi) ? tl[t] % qi : tl[t];
    uint64_t fix = qi - (qk_half % qi);
    for (size_t t = 0; t < n; t++) tntt[t] += fix;
    ntt_lazy(tntt, c, i);
    uint64_t qi_lazy = qi << 2;
    uint64_t *pi = k->prod + ((size_t)comp * k->rns + i) * n;
    uint64_t inv = invmod(qk % qi, qi);
    uint64_t *ci = k->ct + ((size_t)comp * ell + i) * n;
    for (size_t t = 0; t < n; t++) {
        uint64_t x = pi[t] + qi_lazy - tntt[t];
        x = mulmod(x, inv, qi);
        uint64_t y = ci[t] + x;
        ci[t] = y >= qi ? y - qi : y;
    }
}

/* Evaluator::switch_key_inplace (evaluator.cpp:2724-3022), CKKS branch.
 *   ct     : [2][ell][N] ciphertext in NTT form, updated in place
 *   target : [ell][N] polynomial (NTT form) to switch
 *   key    : [ell_key][2][K][N] key-switching key at the key level, where
 *            K = c->k (data primes 0..K-2, special prime K-1) and ell <= K-1
 */
void or_switch_key(const or_ctx *c, uint64_t *ct, int ell, const uint64_t *target, const uint64_t *key)
{
    size_t n = c->n;
    ks_job k;
    k.c = c; k.ct = ct; k.ell = ell; k.K = c->k; k.sp = c->k - 1; k.rns = ell + 1;
    k.target = target; k.key = key;
    int width = parallel_width(2 * ell > k.rns ? 2 * ell : k.rns);
    k.tt = (uint64_t *)malloc(sizeof(uint64_t) * n * ell);
    memcpy(k.tt, target, sizeof(uint64_t) * n * ell);
    k.prod = (uint64_t *)calloc((size_t)2 * k.rns * n, sizeof(uint64_t));
    k.tntt = (uint64_t *)malloc(sizeof(uint64_t) * n * width);
    k.acc = (u128 *)malloc(sizeof(u128) * 2 * n * width);
    parallel_for(ell, ks_intt_task, &k);
    parallel_for(k.rns, ks_modup_task, &k);
    /* modulus switching with scaling (ModDown), CKKS branch */
    parallel_for(2, ks_special_task, &k);
    parallel_for(2 * ell, ks_moddown_task, &k);
    free(k.tt); free(k.prod); free(k.tntt); free(k.acc);
}

/* relinearize_internal (evaluator.cpp:1345-1400) for a size-3 ciphertext:
 * ct [3][ell][N] -> out [2][ell][N] */
void or_relinearize(const or_ctx *c, const uint64_t *ct3, int ell, const uint64_t *relin_key, uint64_t *out)
{
    size_t n = c->n;
    memmove(out, ct3, sizeof(uint64_t) * 2 * ell * n);
    uint64_t *c2 = (uint64_t *)malloc(sizeof(uint64_t) * ell * n);
    memcpy(c2, ct3 + (size_t)2 * ell * n, sizeof(uint64_t) * ell * n);
    or_switch_key(c, out, ell, c2, relin_key);
    free(c2);
}

/* ------------------------------------------------------------------ */
/* Galois automorphisms                                                 */
/* ------------------------------------------------------------------ */

/* GaloisTool::generate_table_ntt (util/galois.cpp:18-52) */
void or_galois_table_ntt(int logn, uint32_t elt, uint32_t *out)
{
    uint32_t n = 1u << logn, mask = n - 1;
    for (uint32_t i = n; i < 2 * n; i++) {
        uint32_t rev = reverse_bits(i, logn + 1);
        uint64_t raw = ((uint64_t)elt * rev) >> 1;
        raw &= mask;
        *out++ = reverse_bits((uint32_t)raw, logn);
    }
}

/* GaloisTool::get_elt_from_step (util/galois.cpp:53-90); the generator is 5 (util/galois.h:169) */
uint32_t or_galois_elt_from_step(int logn, int step)
{
    uint32_t n = 1u << logn;
    uint64_t m = 2ull * n;
    if (step == 0) return (uint32_t)(m - 1);
    int neg = step < 0;
    uint32_t pos = (uint32_t)(neg ? -step : step);
    pos &= (uint32_t)(m - 1);
    int s = neg ? (int)(n >> 1) - (int)pos : (int)pos;
    uint64_t elt = 1;
    while (s--) { elt *= 5; elt &= m - 1; }
    return (uint32_t)elt;
}

/* apply_galois_inplace (evaluator.cpp:2563-2665), CKKS branch:
 * ct [2][ell][N] NTT form -> out [2][ell][N] */
void or_apply_galois(const or_ctx *c, const uint64_t *ct, int ell, uint32_t elt, const uint64_t *gkey, uint64_t *out)
{
    size_t n = c->n;
    uint32_t *tab = (uint32_t *)malloc(sizeof(uint32_t) * n);
    or_galois_table_ntt(c->logn, elt, tab);
    uint64_t *tmp = (uint64_t *)malloc(sizeof(uint64_t) * ell * n);
    uint64_t *res = (uint64_t *)malloc(sizeof(uint64_t) * 2 * ell * n);
    for (int j = 0; j < ell; j++)
        for (size_t t = 0; t < n; t++) res[(size_t)j * n + t] = ct[(size_t)j * n + tab[t]];
    for (int j = 0; j < ell; j++)
        for (size_t t = 0; t < n; t++) tmp[(size_t)j * n + t] = ct[((size_t)ell + j) * n + tab[t]];
    memset(res + (size_t)ell * n, 0, sizeof(uint64_t) * ell * n);
    or_switch_key(c, res, ell, tmp, gkey);
    memcpy(out, res, sizeof(uint64_t) * 2 * ell * n);
    free(tab); free(tmp); free(res);
}

/* ------------------------------------------------------------------ */
/* element-wise ciphertext arithmetic                                   */
/* ------------------------------------------------------------------ */

/* ckks_multiply (evaluator.cpp:770-850): (a0 b0, a0 b1 + a1 b0, a1 b1) */
void or_ckks_multiply(const or_ctx *c, const uint64_t *a, const uint64_t *b, int ell, uint64_t *out3)
{
    size_t n = c->n;
    for (int j = 0; j < ell; j++) {
        uint64_t q = c->q[j];
        const uint64_t *a0 = a + (size_t)j * n, *a1 = a + ((size_t)ell + j) * n;
        const uint64_t *b0 = b + (size_t)j * n, *b1 = b + ((size_t)ell + j) * n;
        uint64_t *o0 = out3 + (size_t)j * n, *o1 = out3 + ((size_t)ell + j) * n, *o2 = out3 + ((size_t)2 * ell + j) * n;
        for (size_t t = 0; t < n; t++) {
            uint64_t x0 = a0[t], x1 = a1[t], y0 = b0[t], y1 = b1[t];
            uint64_t p2 = mulmod(x1, y1, q);
            uint64_t p1 = (mulmod(x0, y1, q) + mulmod(x1, y0, q)) % q;
            uint64_t p0 = mulmod(x0, y0, q);
            o0[t] = p0; o1[t] = p1; o2[t] = p2;
        }
    }
}

/* multiply_plain_ntt (evaluator.cpp:2336-2373): dyadic product per poly */
void or_multiply_plain(const or_ctx *c, const uint64_t *ct, int size, int ell, const uint64_t *pt, uint64_t *out)
{
    size_t n = c->n;
    for (int s = 0; s < size; s++)
        for (int j = 0; j < ell; j++) {
            uint64_t q = c->q[j];
            const uint64_t *x = ct + ((size_t)s * ell + j) * n, *y = pt + (size_t)j * n;
            uint64_t *o = out + ((size_t)s * ell + j) * n;
            for (size_t t = 0; t < n; t++) o[t] = mulmod(x[t], y[t], q);
        }
}

/* add_inplace / sub_inplace (evaluator.cpp:155, 263) over [size][ell][N]; op 0 add, 1 sub */
void or_add_sub(const or_ctx *c, const uint64_t *a, const uint64_t *b, int size, int ell, int op, uint64_t *out)
{
    size_t n = c->n;
    for (int s = 0; s < size; s++)
        for (int j = 0; j < ell; j++) {
            uint64_t q = c->q[j];
            size_t o = ((size_t)s * ell + j) * n;
            for (size_t t = 0; t < n; t++) {
                uint64_t x = a[o + t], y = b[o + t];
                uint64_t r = op ? (x >= y ? x - y : x + q - y) : (x + y >= q ? x + y - q : x + y);
                out[o + t] = r;
            }
        }
}

/* ------------------------------------------------------------------ */
/* small helpers exposed for tests                                      */
/* ------------------------------------------------------------------ */
uint64_t or_mulmod(uint64_t a, uint64_t b, uint64_t q) { return mulmod(a, b, q); }
uint64_t or_invmod(uint64_t a, uint64_t q) { return invmod(a, q); }
int or_is_prime(uint64_t n) { return is_prime_u64(n); }

/* ------------------------------------------------------------------ */
/* CKKS encoder                                                         */
/* ------------------------------------------------------------------ */
/* The complex FFT below restates CKKSEncoder (ckks.cpp:13-70), the root
 * table of ComplexRoots (util/croots.cpp) and DWTHandler over complex<double>
 * (util/dwthandler.h).  Products are written as (ac - bd, ad + bc), the
 * rounding of std::complex<double> multiplication without contraction; the
 * file is compiled with -ffp-contract=off. */
#include <math.h>

typedef struct { double re, im; } cplx;

static cplx cmul(cplx a, cplx b) { cplx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static cplx cadd(cplx a, cplx b) { cplx r = {a.re + b.re, a.im + b.im}; return r; }
static cplx csubc(cplx a, cplx b) { cplx r = {a.re - b.re, a.im - b.im}; return r; }
static cplx cscale(cplx a, double s) { cplx r = {a.re * s, a.im * s}; return r; }

typedef struct {
    int logn;
    size_t n, slots;
    uint32_t *index_map;
    cplx *root_powers, *inv_root_powers;
} or_encoder;

static cplx root_get(const cplx *tab, size_t m, size_t index)
{
    index &= m - 1;
    if (index <= m / 8) return tab[index];
    if (index <= m / 4) { cplx a = tab[m / 4 - index]; cplx r = {a.im, a.re}; return r; }
    if (index <= m / 2) { cplx a = root_get(tab, m, m / 2 - index); cplx r = {-a.re, a.im}; return r; }
    if (index <= 3 * m / 4) { cplx a = root_get(tab, m, index - m / 2); cplx r = {-a.re, -a.im}; return r; }
    { cplx a = root_get(tab, m, m - index); cplx r = {a.re, -a.im}; return r; }
}

or_encoder *or_encoder_create(int logn)
{
    or_encoder *e = (or_encoder *)calloc(1, sizeof(or_encoder));
    size_t n = (size_t)1 << logn, m = n << 1;
    e->logn = logn; e->n = n; e->slots = n / 2;
    e->index_map = (uint32_t *)malloc(sizeof(uint32_t) * n);
    uint64_t pos = 1;
    for (size_t i = 0; i < e->slots; i++) {
        uint64_t i1 = (pos - 1) >> 1, i2 = (m - pos - 1) >> 1;
        e->index_map[i] = reverse_bits((uint32_t)i1, logn);
        e->index_map[e->slots | i] = reverse_bits((uint32_t)i2, logn);
        pos = (pos * 5) & (m - 1);
    }
    const double PI_ = 3.1415926535897932384626433832795028842;
    cplx *tab = (cplx *)malloc(sizeof(cplx) * (m / 8 + 1));
    for (size_t i = 0; i <= m / 8; i++) {
        double th = 2 * PI_ * (double)i / (double)m;
        tab[i].re = cos(th);
        tab[i].im = sin(th);
    }
    e->root_powers = (cplx *)calloc(n, sizeof(cplx));
    e->inv_root_powers = (cplx *)calloc(n, sizeof(cplx));
    for (size_t i = 1; i < n; i++) {
        e->root_powers[i] = root_get(tab, m, reverse_bits((uint32_t)i, logn));
        cplx a = root_get(tab, m, reverse_bits((uint32_t)(i - 1), logn) + 1);
        a.im = -a.im;
        e->inv_root_powers[i] = a;
    }
    free(tab);
    return e;
}

void or_encoder_destroy(or_encoder *e)
{
    if (!e) return;
    free(e->index_map); free(e->root_powers); free(e->inv_root_powers); free(e);
}

/* total_coeff_modulus_bit_count of the first `limbs` primes */
static int prod_bits(const or_ctx *c, int limbs)
{
    uint64_t p[70] = {0};
    p[0] = 1;
    for (int i = 0; i < limbs; i++) {
        u128 carry = 0;
        for (int w = 0; w <= limbs; w++) {
            u128 t = (u128)p[w] * c->q[i] + carry;
            p[w] = (uint64_t)t;
            carry = t >> 64;
        }
    }
    for (int w = limbs; w >= 0; w--)
        if (p[w]) return w * 64 + (64 - __builtin_clzll(p[w]));
    return 0;
}

static uint64_t words_mod(const uint64_t *w, int count, uint64_t q)
{
    u128 r = 0;
    for (int i = count - 1; i >= 0; i--) r = ((r << 64) | w[i]) % q;
    return (uint64_t)r;
}

/* CKKSEncoder::encode_internal for complex values (ckks.h:457-640); output
 * in NTT form [limbs][N].  Returns 0, -1 "scale out of bounds", -2 "encoded
 * values are too large", -3 "values_size is too large". */
int or_encode(const or_ctx *c, const or_encoder *e, const double *re, const double *im, size_t nvals, double scale,
              int limbs, uint64_t *out)
{
    size_t n = e->n;
    if (nvals > e->slots) return -3;
    int tb = prod_bits(c, limbs);
    if (scale <= 0 || ((int)log2(scale) + 1 >= tb)) return -1;
    cplx *v = (cplx *)calloc(n, sizeof(cplx));
    for (size_t i = 0; i < nvals; i++) {
        cplx a = {re[i], im ? im[i] : 0.0};
        v[e->index_map[i]] = a;
        a.im = -a.im;
        v[e->index_map[i + e->slots]] = a;
    }
    double fix = scale / (double)n;
    /* transform_from_rev with the scalar in the last stage */
    size_t gap = 1, m = n >> 1;
    const cplx *rt = e->inv_root_powers;
    for (; m > 1; m >>= 1) {
        size_t off = 0;
        for (size_t i = 0; i < m; i++) {
            cplx r = *++rt;
            cplx *x = v + off, *y = x + gap;
            for (size_t j = 0; j < gap; j++) {
                cplx u = x[j], w = y[j];
                x[j] = cadd(u, w);
                y[j] = cmul(csubc(u, w), r);
            }
            off += gap << 1;
        }
        gap <<= 1;
    }
    {
        cplx r = *++rt;
        cplx sr = cscale(r, fix);
        for (size_t j = 0; j < gap; j++) {
            cplx u = v[j], w = v[j + gap];
            v[j] = cscale(cadd(u, w), fix);
            v[j + gap] = cmul(csubc(u, w), sr);
        }
    }
    double max_coeff = 0;
    for (size_t i = 0; i < n; i++) if (fabs(v[i].re) > max_coeff) max_coeff = fabs(v[i].re);
    int max_bits = (int)ceil(log2(max_coeff > 1.0 ? max_coeff : 1.0)) + 1;
    if (max_bits >= tb) { free(v); return -2; }
    double two64 = pow(2.0, 64);
    for (size_t i = 0; i < n; i++) {
        double cd = round(v[i].re);
        int neg = signbit(cd) != 0;
        cd = fabs(cd);
        uint64_t w[40];
        int cnt = 0;
        if (max_bits <= 64) { w[0] = (uint64_t)cd; cnt = 1; }
        else if (max_bits <= 128) { w[0] = (uint64_t)fmod(cd, two64); w[1] = (uint64_t)(cd / two64); cnt = 2; }
        else { while (cd >= 1 && cnt < 40) { w[cnt++] = (uint64_t)fmod(cd, two64); cd /= two64; } }
        for (int j = 0; j < limbs; j++) {
            uint64_t q = c->q[j];
            uint64_t r = cnt ? words_mod(w, cnt, q) : 0;
            if (neg && r) r = q - r;
            out[(size_t)j * n + i] = r;
        }
    }
    free(v);
    for (int j = 0; j < limbs; j++) ntt_full(out + (size_t)j * n, c, j);
    return 0;
}

/* CKKSEncoder::encode_internal(double) (ckks.cpp:75-205): per-limb residue of
 * round(value * scale).  Returns 0, -1 scale out of bounds, -2 too large. */
int or_encode_scalar(const or_ctx *c, double value, double scale, int limbs, uint64_t *per_limb)
{
    int tb = prod_bits(c, limbs);
    if (scale <= 0 || ((int)log2(scale) >= tb)) return -1;
    value *= scale;
    int cb = (int)log2(fabs(value)) + 2;
    if (cb >= tb) return -2;
    double two64 = pow(2.0, 64);
    double cd = round(value);
    int neg = signbit(cd) != 0;
    cd = fabs(cd);
    uint64_t w[40];
    int cnt = 0;
    if (cb <= 64) { w[0] = (uint64_t)fabs(cd); cnt = 1; }
    else if (cb <= 128) { w[0] = (uint64_t)fmod(cd, two64); w[1] = (uint64_t)(cd / two64); cnt = 2; }
    else { while (cd >= 1 && cnt < 40) { w[cnt++] = (uint64_t)fmod(cd, two64); cd /= two64; } }
    for (int j = 0; j < limbs; j++) {
        uint64_t q = c->q[j];
        uint64_t r = cnt ? words_mod(w, cnt, q) : 0;
        if (neg && r) r = q - r;
        per_limb[j] = r;
    }
    return 0;
}

/* out[p][l] = in[p][l] * s[l] mod q_l */
void or_multiply_scalar(const or_ctx *c, const uint64_t *in, int polys, int limbs, const uint64_t *s, uint64_t *out)
{
    size_t n = c->n;
    for (int p = 0; p < polys; p++)
        for (int l = 0; l < limbs; l++) {
            size_t o = ((size_t)p * limbs + l) * n;
            for (size_t t = 0; t < n; t++) out[o + t] = mulmod(in[o + t], s[l], c->q[l]);
        }
}

/* out[l] = in[l] (+|-) s[l] on one polynomial (add_plain of a scalar plaintext) */
void or_add_scalar(const or_ctx *c, const uint64_t *in, int limbs, const uint64_t *s, int sub, uint64_t *out)
{
    size_t n = c->n;
    for (int l = 0; l < limbs; l++) {
        uint64_t q = c->q[l];
        for (size_t t = 0; t < n; t++) {
            uint64_t x = in[(size_t)l * n + t];
            out[(size_t)l * n + t] = sub ? (x >= s[l] ? x - s[l] : x + q - s[l]) : (x + s[l] >= q ? x + s[l] - q : x + s[l]);
        }
    }
}
