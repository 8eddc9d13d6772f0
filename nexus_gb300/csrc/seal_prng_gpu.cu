// The bulk of sample_poly_uniform (util/rlwe.cpp:137-165) on the GPU: the
// Blake2xbPRNG refills of a fresh stream by a CUDA BLAKE2Xb (blake2b.h; one
// thread per refill root, one per 64-byte output block), then the words at or
// above their prime's bound, which SEAL redraws in order from the stream past
// the bulk, found on the device and redrawn on the host (about 2^-13 of them
// for 51-bit primes).
#include <algorithm>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "blake2b.h"
#include "context.h"
#include "seal_prng.h"

namespace nexus {
namespace sealrng {

namespace {

constexpr int kThreads = 256;
constexpr unsigned kRedrawCap = 1u << 16;

struct SeedArg {
    uint64_t w[kSeedWords];
};

struct Bounds {
    uint64_t b[64];
};

inline unsigned blocks_for(size_t n, size_t cap = 1u << 20)
{
    return (unsigned)std::min<size_t>((n + kThreads - 1) / kThreads, cap);
}

__global__ void k_xof_roots(SeedArg sd, size_t count, uint64_t *__restrict__ roots)
{
    const size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= count) return;
    uint64_t h[8];
    blake2b::xof_root(sd.w, (uint64_t)r, (uint32_t)kRefillBytes, h);
#pragma unroll
    for (int i = 0; i < 8; ++i) roots[r * 8 + i] = h[i];
}

// output block x = refill r, block i of 64: bytes [64x, 64x + 64) of the stream
__global__ void k_xof_blocks(const uint64_t *__restrict__ roots, size_t blocks, uint64_t *__restrict__ out)
{
    const size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= blocks) return;
    const size_t r = x / (kRefillBytes / 64);
    const uint32_t i = (uint32_t)(x % (kRefillBytes / 64));
    uint64_t root[8], h[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) root[k] = roots[r * 8 + k];
    blake2b::xof_block(root, i, (uint32_t)kRefillBytes, h);
#pragma unroll
    for (int k = 0; k < 8; ++k) out[x * 8 + k] = h[k];
}

// positions whose word must be redrawn (unordered; at most `cap` recorded)
__global__ void k_find_redraws(const uint64_t *__restrict__ raw, Bounds bd, int logn, size_t total,
                               unsigned *count, uint64_t *__restrict__ list, unsigned cap)
{
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        if (raw[x] >= bd.b[x >> logn]) {
            const unsigned i = atomicAdd(count, 1u);
            if (i < cap) list[i] = x;
        }
    }
}

__global__ void k_patch(uint64_t *__restrict__ raw, const uint64_t *__restrict__ pos,
                        const uint64_t *__restrict__ val, unsigned count)
{
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) raw[pos[i]] = val[i];
}

struct Temp {
    void *p = nullptr;
    cudaStream_t s;
    Temp(size_t bytes, cudaStream_t st) : s(st)
    {
        if (cudaMallocAsync(&p, bytes, s) != cudaSuccess) throw std::runtime_error("cudaMallocAsync failed");
    }
    ~Temp() { cudaFreeAsync(p, s); }
};

void check(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

void sample_uniform_raw_device(const uint64_t seed[kSeedWords], int logn, const uint64_t *q, int k, uint64_t *d_raw,
                               cudaStream_t s)
{
    if (k < 1 || k > 64) throw std::invalid_argument("sample_uniform_raw_device: 1 to 64 primes");
    const size_t n = (size_t)1 << logn, words = (size_t)k * n, bytes = words * sizeof(uint64_t);
    if (bytes % kRefillBytes) throw std::invalid_argument("sample_uniform_raw_device: not whole refills");
    const size_t refills = bytes / kRefillBytes, blocks = bytes / 64;
    // roots [refills][8] | count (padded to 16 bytes) | positions [cap] | positions, values [cap] each
    Temp t(refills * 64 + 16 + 3 * (size_t)kRedrawCap * 8, s);
    uint64_t *roots = static_cast<uint64_t *>(t.p);
    unsigned *d_count = reinterpret_cast<unsigned *>(roots + refills * 8);
    uint64_t *d_list = roots + refills * 8 + 2, *d_pos = d_list + kRedrawCap, *d_val = d_pos + kRedrawCap;
    SeedArg sd;
    std::memcpy(sd.w, seed, sizeof(sd.w));
    k_xof_roots<<<blocks_for(refills), kThreads, 0, s>>>(sd, refills, roots); NEXUS_LAUNCHED();
    k_xof_blocks<<<blocks_for(blocks, ~0u), kThreads, 0, s>>>(roots, blocks, d_raw); NEXUS_LAUNCHED();
    Bounds bd{};
    for (int j = 0; j < k; ++j) bd.b[j] = uniform_bound(q[j]);
    check(cudaMemsetAsync(d_count, 0, sizeof(unsigned), s), "cudaMemsetAsync");
    k_find_redraws<<<blocks_for(words), kThreads, 0, s>>>(d_raw, bd, logn, words, d_count, d_list, kRedrawCap);
    NEXUS_LAUNCHED();
    unsigned count = 0;
    check(cudaMemcpyAsync(&count, d_count, sizeof(count), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
    check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    if (count == 0) return;
    if (count > kRedrawCap) {   // never expected: redo the whole sample on the host
        std::vector<uint64_t> raw(words);
        Stream st(seed);
        sample_uniform_raw(st, n, q, k, raw.data());
        check(cudaMemcpyAsync(d_raw, raw.data(), bytes, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
        check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        return;
    }
    // SEAL redraws row by row, coefficient by coefficient, from the stream
    // right after the bulk: positions in increasing order
    std::vector<uint64_t> pos(count), val(count);
    check(cudaMemcpyAsync(pos.data(), d_list, count * sizeof(uint64_t), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
    check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    std::sort(pos.begin(), pos.end());
    Stream st(seed);
    st.seek(bytes);
    for (unsigned i = 0; i < count; ++i) {
        const uint64_t bound = bd.b[pos[i] >> logn];
        uint64_t v;
        do v = st.u64();
        while (v >= bound);
        val[i] = v;
    }
    check(cudaMemcpyAsync(d_pos, pos.data(), count * sizeof(uint64_t), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
    check(cudaMemcpyAsync(d_val, val.data(), count * sizeof(uint64_t), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
    k_patch<<<(count + kThreads - 1) / kThreads, kThreads, 0, s>>>(d_raw, d_pos, d_val, count); NEXUS_LAUNCHED();
    check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
}

}  // namespace sealrng
}  // namespace nexus
