// Context construction: prime checks, minimal primitive roots and the device
// twiddle tables.  The tables reproduce the root choice of SEAL's NTTTables
// (util/ntt.cpp:241-300 in SEAL-4.1-bs): psi is the smallest primitive 2N-th
// root of unity (util/numth.cpp:386-412), stored in bit-reversed order, so the
// engine's NTT output equals SEAL's word for word.
#include <cstring>
#include <stdexcept>

#include "context.h"
#include "encoder.h"

#define CK(call)                                                                      \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e_));      \
    } while (0)

namespace nexus {

typedef unsigned __int128 u128;

uint64_t host_mulmod(uint64_t a, uint64_t b, uint64_t q) { return (uint64_t)(((u128)a * b) % q); }

uint64_t host_powmod(uint64_t a, uint64_t e, uint64_t q)
{
    uint64_t r = 1 % q;
    a %= q;
    while (e) {
        if (e & 1) r = host_mulmod(r, a, q);
        a = host_mulmod(a, a, q);
        e >>= 1;
    }
    return r;
}

uint64_t host_invmod(uint64_t a, uint64_t q)
{
    // q is prime in every use: Fermat inversion
    return host_powmod(a, q - 2, q);
}

uint64_t host_shoup(uint64_t w, uint64_t q) { return (uint64_t)((((u128)w) << 64) / q); }

static bool host_is_prime(uint64_t n)
{
    static const uint64_t bases[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    if (n < 2) return false;
    for (uint64_t b : bases) {
        if (n == b) return true;
        if (n % b == 0) return false;
    }
    uint64_t d = n - 1;
    int s = 0;
    while (!(d & 1)) {
        d >>= 1;
        ++s;
    }
    for (uint64_t b : bases) {
        uint64_t x = host_powmod(b, d, n);
        if (x == 1 || x == n - 1) continue;
        bool composite = true;
        for (int r = 1; r < s && composite; ++r) {
            x = host_mulmod(x, x, n);
            if (x == n - 1) composite = false;
        }
        if (composite) return false;
    }
    return true;
}

// Smallest primitive `degree`-th root of unity mod q (degree a power of two).
static uint64_t minimal_primitive_root(uint64_t degree, uint64_t q)
{
    uint64_t quo = (q - 1) / degree, root = 0;
    for (uint64_t g = 2; g < q && !root; ++g) {
        uint64_t c = host_powmod(g, quo, q);
        if (c && host_powmod(c, degree / 2, q) == q - 1) root = c;
    }
    if (!root) throw std::invalid_argument("no primitive root");
    // the primitive roots are the odd powers of any one of them
    uint64_t sq = host_mulmod(root, root, q), cur = root, best = root;
    for (uint64_t i = 0; i < degree; i += 2) {
        if (cur < best) best = cur;
        cur = host_mulmod(cur, sq, q);
    }
    return best;
}

static uint32_t bitrev(uint32_t x, int bits)
{
    uint32_t r = 0;
    for (int i = 0; i < bits; ++i) {
        r = (r << 1) | (x & 1);
        x >>= 1;
    }
    return r;
}

uint64_t *Context::get_scratch(size_t words)
{
    if (words > scratch_words) {
        // growing frees the old arena, which synchronises with pending work
        if (scratch) CK(cudaFree(scratch));
        scratch = nullptr;
        scratch_words = 0;
        CK(cudaMalloc(&scratch, words * sizeof(uint64_t)));
        scratch_words = words;
    }
    return scratch;
}

// GaloisTool::generate_table_ntt (util/galois.cpp:18-52): slot i of the
// permuted polynomial reads slot table[i] of the input.
const uint32_t *Context::galois_table(uint32_t elt)
{
    auto it = galois_tables.find(elt);
    if (it != galois_tables.end()) return it->second;
    if (!(elt & 1) || elt >= 2 * n) throw std::invalid_argument("Galois element is not valid");
    std::vector<uint32_t> t(n);
    const uint32_t mask = (uint32_t)n - 1;
    for (uint64_t i = n; i < 2 * n; ++i) {
        uint32_t rev = bitrev((uint32_t)i, logn + 1);
        uint64_t raw = ((uint64_t)elt * rev) >> 1;
        t[i - n] = bitrev((uint32_t)(raw & mask), logn);
    }
    uint32_t *d = nullptr;
    CK(cudaMalloc(&d, sizeof(uint32_t) * n));
    CK(cudaMemcpy(d, t.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
    galois_tables[elt] = d;
    return d;
}

std::atomic<uint64_t> g_kernel_launches{0};

static thread_local std::string g_last_error;
void set_error(const std::string &msg) { g_last_error = msg; }

}  // namespace nexus

using namespace nexus;

extern "C" const char *nexus_last_error(void) { return nexus::g_last_error.c_str(); }

extern "C" uint64_t nexus_kernel_launches(void) { return nexus::g_kernel_launches.load(); }

extern "C" int nexus_memory_info(uint64_t *pool_used, uint64_t *pool_used_high, uint64_t *pool_reserved,
                                 uint64_t *graph_reserved)
{
    int dev = 0;
    cudaMemPool_t pool = nullptr;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetDefaultMemPool(&pool, dev);
    const cudaMemPoolAttr attr[3] = {cudaMemPoolAttrUsedMemCurrent, cudaMemPoolAttrUsedMemHigh,
                                     cudaMemPoolAttrReservedMemCurrent};
    uint64_t *dst[3] = {pool_used, pool_used_high, pool_reserved};
    for (int i = 0; i < 3 && e == cudaSuccess; ++i) {
        uint64_t v = 0;  // the byte-count attributes are 64-bit
        e = cudaMemPoolGetAttribute(pool, attr[i], &v);
        if (e == cudaSuccess && dst[i]) *dst[i] = v;
    }
    if (e == cudaSuccess) {
        uint64_t v = 0;
        e = cudaDeviceGetGraphMemAttribute(dev, cudaGraphMemAttrReservedMemCurrent, &v);
        if (e == cudaSuccess && graph_reserved) *graph_reserved = v;
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error(std::string("nexus_memory_info: ") + cudaGetErrorString(e));
        return -1;
    }
    return 0;
}

extern "C" int nexus_memory_trim(void)
{
    int dev = 0;
    cudaMemPool_t pool = nullptr;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetDefaultMemPool(&pool, dev);
    if (e == cudaSuccess) e = cudaMemPoolTrimTo(pool, 0);
    if (e == cudaSuccess) e = cudaDeviceGraphMemTrim(dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error(std::string("nexus_memory_trim: ") + cudaGetErrorString(e));
        return -1;
    }
    return 0;
}

extern "C" int nexus_context_create(int log_n, const uint64_t *moduli, int n_moduli, nexus_context **out)
{
    if (!out || !moduli) {
        set_error("nexus_context_create: null argument");
        return -1;
    }
    *out = nullptr;
    if (log_n < 12 || log_n > 16) {
        set_error("nexus_context_create: log_n must be in [12, 16]");
        return -1;
    }
    if (n_moduli < 2 || n_moduli > 64) {
        set_error("nexus_context_create: need 2..64 primes (data primes + special prime)");
        return -1;
    }
    nexus_context *h = new nexus_context();
    Context &c = h->c;
    try {
        c.logn = log_n;
        c.n = 1ull << log_n;
        c.k = n_moduli;
        CK(cudaGetDevice(&c.device));
        CK(cudaDeviceGetAttribute(&c.sm_count, cudaDevAttrMultiProcessorCount, c.device));
        // keep memory freed by stream-ordered deallocation in the pool: the
        // evaluator allocates and frees ciphertexts on every operation
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, c.device) == cudaSuccess) {
            uint64_t threshold = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
        }
        c.q.assign(moduli, moduli + n_moduli);
        c.log_n1 = log_n / 2;
        c.log_n2 = log_n - c.log_n1;
        const uint64_t n = c.n;
        std::vector<ulonglong2> fwd((size_t)n_moduli * n), inv((size_t)n_moduli * n);
        for (int j = 0; j < n_moduli; ++j) {
            uint64_t q = c.q[j];
            if (q >= (1ull << 61) || q < 3 || !host_is_prime(q) || (q - 1) % (2 * n) != 0) {
                throw std::invalid_argument("modulus " + std::to_string(j) +
                                            " is not a prime below 2^61 congruent to 1 mod 2N");
            }
            uint64_t psi = minimal_primitive_root(2 * n, q);
            uint64_t psi_inv = host_invmod(psi, q);
            c.psi.push_back(psi);
            // powers psi^i and psi^{-i} scattered to bit-reversed positions
            uint64_t p = 1, pi = 1;
            for (uint64_t i = 0; i < n; ++i) {
                uint32_t r = bitrev((uint32_t)i, log_n);
                fwd[(size_t)j * n + r] = make_ulonglong2(p, host_shoup(p, q));
                inv[(size_t)j * n + r] = make_ulonglong2(pi, host_shoup(pi, q));
                p = host_mulmod(p, psi, q);
                pi = host_mulmod(pi, psi_inv, q);
            }
            PrimeConst pc;
            pc.q = q;
            u128 ratio_hi = (((u128)1) << 64) / q;           // floor(2^64/q)
            u128 rem = (((u128)1) << 64) % q;
            u128 ratio_lo = (rem << 64) / q;                 // next 64 bits of 2^128/q
            pc.r1 = (uint64_t)ratio_hi;
            pc.r0 = (uint64_t)ratio_lo;
            pc.inv_n = host_invmod(n % q, q);
            pc.inv_n_q = host_shoup(pc.inv_n, q);
            c.pc.push_back(pc);
        }
        c.inv_q.assign((size_t)n_moduli * n_moduli, make_ulonglong2(0, 0));
        for (int a = 0; a < n_moduli; ++a)
            for (int b = 0; b < n_moduli; ++b)
                if (a != b) {
                    uint64_t v = host_invmod(c.q[a] % c.q[b], c.q[b]);
                    c.inv_q[(size_t)a * n_moduli + b] = make_ulonglong2(v, host_shoup(v, c.q[b]));
                }
        CK(cudaMalloc(&c.d_inv_q, sizeof(ulonglong2) * c.inv_q.size()));
        CK(cudaMemcpy(c.d_inv_q, c.inv_q.data(), sizeof(ulonglong2) * c.inv_q.size(), cudaMemcpyHostToDevice));
        c.small_primes = true;
        for (uint64_t qq : c.q) c.small_primes = c.small_primes && qq < (1ull << 52);
        CK(cudaMalloc(&c.d_pc, sizeof(PrimeConst) * n_moduli));
        CK(cudaMemcpy(c.d_pc, c.pc.data(), sizeof(PrimeConst) * n_moduli, cudaMemcpyHostToDevice));
        CK(cudaMalloc(&c.d_tw_fwd, sizeof(ulonglong2) * fwd.size()));
        CK(cudaMalloc(&c.d_tw_inv, sizeof(ulonglong2) * inv.size()));
        CK(cudaMemcpy(c.d_tw_fwd, fwd.data(), sizeof(ulonglong2) * fwd.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c.d_tw_inv, inv.data(), sizeof(ulonglong2) * inv.size(), cudaMemcpyHostToDevice));
    } catch (const std::exception &e) {
        set_error(std::string("nexus_context_create: ") + e.what());
        cudaFree(c.d_pc);
        cudaFree(c.d_tw_fwd);
        cudaFree(c.d_tw_inv);
        cudaFree(c.d_inv_q);
        delete h;
        return -1;
    }
    *out = h;
    return 0;
}

extern "C" int nexus_context_destroy(nexus_context *h)
{
    if (!h) return 0;
    cudaFree(h->c.d_pc);
    cudaFree(h->c.d_tw_fwd);
    cudaFree(h->c.d_tw_inv);
    cudaFree(h->c.d_inv_q);
    cudaFree(h->c.scratch);
    for (auto &kv : h->c.galois_tables) cudaFree(kv.second);
    delete h->enc;
    delete h;
    return 0;
}

// CoeffModulus::Create (modulus.cpp:143-184 over util/numth.cpp:278-311 in
// SEAL-4.1-bs): for each requested bit size, primes p = 1 mod 2N scanned
// downward from 2^bits; repeated sizes take their primes smallest-first.
extern "C" int nexus_create_coeff_modulus(uint64_t poly_degree, const int *bit_sizes, int count, uint64_t *out)
{
    if (!bit_sizes || !out || count <= 0) {
        set_error("nexus_create_coeff_modulus: bad arguments");
        return -1;
    }
    if (poly_degree < 2 || (poly_degree & (poly_degree - 1)) || poly_degree > (1u << 17)) {
        set_error("nexus_create_coeff_modulus: poly_degree must be a power of two <= 2^17");
        return -1;
    }
    const uint64_t factor = 2 * poly_degree;
    for (int i = 0; i < count; ++i) {
        const int size = bit_sizes[i];
        if (size < 2 || size > 60) {
            set_error("nexus_create_coeff_modulus: bit sizes must be in [2, 60]");
            return -1;
        }
        int total = 0, rank = 0;
        for (int j = 0; j < count; ++j) {
            if (bit_sizes[j] == size) {
                rank += (j < i);
                ++total;
            }
        }
        const int want = total - 1 - rank;  // index into the descending list
        uint64_t value = ((1ull << size) - 1) / factor * factor + 1;
        const uint64_t lower = 1ull << (size - 1);
        int found = -1;
        while (value > lower) {
            if (host_is_prime(value) && ++found == want) break;
            value -= factor;
        }
        if (found != want) {
            set_error("nexus_create_coeff_modulus: failed to find enough qualifying primes");
            return -1;
        }
        out[i] = value;
    }
    return 0;
}

extern "C" int nexus_context_get_psi(const nexus_context *h, uint64_t *psi_out)
{
    if (!h || !psi_out) {
        set_error("nexus_context_get_psi: null argument");
        return -1;
    }
    std::memcpy(psi_out, h->c.psi.data(), sizeof(uint64_t) * h->c.k);
    return 0;
}
