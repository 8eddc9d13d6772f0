// Rate of the fifth-generation tensor cores (tcgen05) of this GPU, measured
// with hand-written MMAs, for the question whether any part of the NTT or of
// the key switch's basis conversion belongs on them.
//
// Each CTA (one per SM, 128 threads) stages an A tile of 128 rows and a B
// tile of 256 rows, 128 bytes of K per row, in shared memory in the
// no-swizzle K-major core-matrix layout (8 rows x 16 bytes per core matrix),
// allocates a 128 x 256 f32 accumulator in tensor memory, and one thread
// issues `rounds` passes of four tcgen05.mma instructions (32 bytes of K
// each: K = 16 for bf16 through kind::f16, K = 32 for e4m3 through
// kind::f8f6f4), then commits them to an mbarrier.  Every wait is bounded by
// the global timer: a wait that runs out sets a status word, waits once more
// with the same bound, frees the tensor memory and returns.  With an output
// pointer the accumulator is read back through tcgen05.ld, so the same kernel
// checks its own layout against a host product (nexus_tensor_tile).
//
// Nothing in the engine's CKKS path calls these; they are measurement aids
// with no counterpart in the reference.
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/nexus_gb300.h"
#include "context.h"

namespace nexus {
void set_error(const std::string &msg);
}

namespace {

constexpr int kM = 128, kN = 256;         // one MMA: a 128 x 256 f32 accumulator
constexpr int kRowBytes = 128;            // K bytes per operand row in shared memory
constexpr int kSteps = kRowBytes / 32;    // MMAs per pass over the tiles (32 bytes of K each)
constexpr uint32_t kTmemCols = 256;       // one f32 column per accumulator column
constexpr int kSmemA = kM * kRowBytes;    // 16 KB
constexpr int kSmemB = kN * kRowBytes;    // 32 KB
// more than half of the SM's shared memory, so that exactly one CTA (and one
// tensor-memory allocation) sits on each SM
constexpr int kSmemDyn = 160 * 1024;
constexpr int kThreadsTc = 128;

// kind::f16: D f32 (bits 4-5 = 1), A and B bf16 (bits 7-9 and 10-12 = 1),
// both K-major (bits 15, 16 = 0), N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t kIdescBf16 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kN >> 3) << 17) |
                                ((uint32_t)(kM >> 4) << 24);
// kind::f8f6f4: D f32, A and B e4m3 (format 0), same shape fields.
constexpr uint32_t kIdescE4m3 = (1u << 4) | ((uint32_t)(kN >> 3) << 17) | ((uint32_t)(kM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Shared-memory matrix descriptor, no swizzle, K-major: start address >> 4
// (bits 0-13), leading byte offset >> 4 (bits 16-29: the step between the two
// K-adjacent core matrices of one MMA, 128 B here), stride byte offset >> 4
// (bits 32-45: the step between 8-row groups, 8 core matrices x 128 B), the
// descriptor version 1 at bit 46, base offset 0, layout type 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46);
}

template <int KIND>
__device__ __forceinline__ void mma(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t accumulate)
{
    if (KIND == 0)
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate)
            : "memory");
    else
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate)
            : "memory");
}

// true once the mbarrier's phase `parity` has completed; false when
// `limit_ns` of global time (or 2^26 polls) pass first
__device__ __forceinline__ bool wait_parity(uint32_t bar, uint32_t parity, uint64_t limit_ns)
{
    const uint64_t t0 = global_ns();
    for (uint32_t i = 0; i < (1u << 26); ++i) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
    return false;
}

// a: kM rows, b: kN rows, kRowBytes each (row-major); d: kM x kN f32 per CTA
// or null; status: set to 1 if a wait ran out
template <int KIND>
__global__ void __launch_bounds__(kThreadsTc, 1)
    k_tc_rate(const uint4 *__restrict__ a, const uint4 *__restrict__ b, float *__restrict__ d, int rounds,
              uint64_t limit_ns, int *status)
{
    extern __shared__ __align__(1024) uint8_t tiles[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // 16-byte chunk kc of row r goes to core matrix (r / 8, kc), row r % 8
    constexpr int kChunks = kRowBytes / 16;
    for (int i = tid; i < kM * kChunks; i += kThreadsTc) {
        const int r = i / kChunks, kc = i % kChunks;
        *reinterpret_cast<uint4 *>(tiles + (((r >> 3) * kChunks + kc) << 7) + ((r & 7) << 4)) = a[i];
    }
    for (int i = tid; i < kN * kChunks; i += kThreadsTc) {
        const int r = i / kChunks, kc = i % kChunks;
        *reinterpret_cast<uint4 *>(tiles + kSmemA + (((r >> 3) * kChunks + kc) << 7) + ((r & 7) << 4)) = b[i];
    }
    // the tensor core reads shared memory through the async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const uint32_t bar = smem_u32(&mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;

    if (tid == 0) {
        const uint32_t a0 = smem_u32(tiles), b0 = a0 + kSmemA;
        const uint32_t idesc = KIND == 0 ? kIdescBf16 : kIdescE4m3;
        for (int r = 0; r < rounds; ++r) {
#pragma unroll
            for (int s = 0; s < kSteps; ++s)
                mma<KIND>(tmem, smem_desc(a0 + s * 256), smem_desc(b0 + s * 256), idesc, (uint32_t)(r | s));
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                     : "memory");
    }
    bool done = wait_parity(bar, 0, limit_ns);
    if (!done) {
        atomicExch(status, 1);
        done = wait_parity(bar, 0, limit_ns);
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // tcgen05.ld is warp-collective: a warp reads only if all its lanes saw the commit
    if (d && __all_sync(0xffffffffu, done)) {
        // warp w owns tensor-memory lanes 32w .. 32w + 31: accumulator row 32w + lane
        float *out = d + (size_t)blockIdx.x * kM * kN + (size_t)(warp * 32 + lane) * kN;
        for (int c = 0; c < kN; c += 8) {
            uint32_t v[8];
            const uint32_t addr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c;
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                         : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                           "=r"(v[7])
                         : "r"(addr)
                         : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int k = 0; k < 8; ++k) out[c + k] = __uint_as_float(v[k]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

struct DevBufs {
    void *a = nullptr, *b = nullptr, *d = nullptr;
    int *status = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ~DevBufs()
    {
        cudaFree(a);
        cudaFree(b);
        cudaFree(d);
        cudaFree(status);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    }
};

void ck(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

void check_device()
{
    int dev = 0, major = 0;
    ck(cudaGetDevice(&dev), "cudaGetDevice");
    ck(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev), "device query");
    if (major != 10) throw std::runtime_error("the tcgen05 kernels are built for sm_103a only");
}

// wait bound handed to the kernel: 2 s plus 1 us per MMA a CTA issues
uint64_t limit_for(int rounds) { return 2000000000ull + (uint64_t)rounds * kSteps * 1000ull; }

void launch(int kind, unsigned grid, const DevBufs &m, float *d, int rounds, cudaStream_t s)
{
    const uint64_t lim = limit_for(rounds);
    if (kind == 0)
        k_tc_rate<0><<<grid, kThreadsTc, kSmemDyn, s>>>((const uint4 *)m.a, (const uint4 *)m.b, d, rounds, lim,
                                                        m.status);
    else
        k_tc_rate<1><<<grid, kThreadsTc, kSmemDyn, s>>>((const uint4 *)m.a, (const uint4 *)m.b, d, rounds, lim,
                                                        m.status);
    NEXUS_LAUNCHED();
    ck(cudaGetLastError(), "tensor-core kernel launch");
}

void prepare(int kind, DevBufs &m, const void *a_host, const void *b_host)
{
    ck(cudaFuncSetAttribute(k_tc_rate<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemDyn), "smem attribute");
    ck(cudaFuncSetAttribute(k_tc_rate<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemDyn), "smem attribute");
    (void)kind;
    ck(cudaMalloc(&m.a, kSmemA), "cudaMalloc");
    ck(cudaMalloc(&m.b, kSmemB), "cudaMalloc");
    ck(cudaMalloc(&m.status, sizeof(int)), "cudaMalloc");
    ck(cudaMemset(m.status, 0, sizeof(int)), "cudaMemset");
    ck(cudaMemcpy(m.a, a_host, kSmemA, cudaMemcpyHostToDevice), "cudaMemcpy");
    ck(cudaMemcpy(m.b, b_host, kSmemB, cudaMemcpyHostToDevice), "cudaMemcpy");
}

void check_status(const DevBufs &m)
{
    int st = 0;
    ck(cudaMemcpy(&st, m.status, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy");
    if (st) throw std::runtime_error("a tensor-core wait ran out of time");
}

// operand bytes for the rate runs: small integers (|v| <= 2) in the operand
// format, from a fixed xorshift stream
void rate_operands(int kind, std::vector<uint8_t> &a, std::vector<uint8_t> &b)
{
    static const uint16_t bf16[5] = {0xC000, 0xBF80, 0x0000, 0x3F80, 0x4000};
    static const uint8_t e4m3[5] = {0xC0, 0xB8, 0x00, 0x38, 0x40};
    uint64_t st = 0x2545F4914F6CDD1Dull;
    auto fill = [&](std::vector<uint8_t> &v, size_t bytes) {
        v.resize(bytes);
        if (kind == 0) {
            for (size_t i = 0; i < bytes / 2; ++i) {
                st ^= st << 13, st ^= st >> 7, st ^= st << 17;
                const uint16_t w = bf16[st % 5];
                v[2 * i] = (uint8_t)w, v[2 * i + 1] = (uint8_t)(w >> 8);
            }
        } else {
            for (size_t i = 0; i < bytes; ++i) {
                st ^= st << 13, st ^= st >> 7, st ^= st << 17;
                v[i] = e4m3[st % 5];
            }
        }
    };
    fill(a, kSmemA);
    fill(b, kSmemB);
}

}  // namespace

namespace nexus {

double tensor_rate(int kind, int rounds, double *ms_out)
{
    if (kind < 0 || kind > 1) throw std::invalid_argument("kind must be 0 (bf16, kind::f16) or 1 (e4m3, kind::f8f6f4)");
    if (rounds < 1 || rounds > (1 << 22)) throw std::invalid_argument("rounds must lie in [1, 2^22]");
    check_device();
    int dev = 0, sms = 0;
    ck(cudaGetDevice(&dev), "cudaGetDevice");
    ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device query");
    std::vector<uint8_t> ha, hb;
    rate_operands(kind, ha, hb);
    DevBufs m;
    prepare(kind, m, ha.data(), hb.data());
    ck(cudaEventCreate(&m.e0), "cudaEventCreate");
    ck(cudaEventCreate(&m.e1), "cudaEventCreate");
    launch(kind, (unsigned)sms, m, nullptr, rounds, 0);  // warm-up
    const int reps = 5;
    ck(cudaEventRecord(m.e0, 0), "cudaEventRecord");
    for (int i = 0; i < reps; ++i) launch(kind, (unsigned)sms, m, nullptr, rounds, 0);
    ck(cudaEventRecord(m.e1, 0), "cudaEventRecord");
    ck(cudaEventSynchronize(m.e1), "tensor-core kernel");
    float ms = 0.f;
    ck(cudaEventElapsedTime(&ms, m.e0, m.e1), "cudaEventElapsedTime");
    check_status(m);
    const double per_launch = ms / reps;
    if (ms_out) *ms_out = per_launch;
    const double k_per_mma = kind == 0 ? 16.0 : 32.0;
    const double flop = 2.0 * kM * kN * k_per_mma * kSteps * (double)rounds * sms;
    return flop / (per_launch * 1e-3);
}

void tensor_tile(int kind, int rounds, const void *a_host, const void *b_host, float *d_host)
{
    if (kind < 0 || kind > 1) throw std::invalid_argument("kind must be 0 (bf16, kind::f16) or 1 (e4m3, kind::f8f6f4)");
    if (rounds < 1 || rounds > 64) throw std::invalid_argument("rounds must lie in [1, 64]");
    check_device();
    DevBufs m;
    prepare(kind, m, a_host, b_host);
    ck(cudaMalloc(&m.d, sizeof(float) * kM * kN), "cudaMalloc");
    ck(cudaMemset(m.d, 0, sizeof(float) * kM * kN), "cudaMemset");
    launch(kind, 1, m, (float *)m.d, rounds, 0);
    ck(cudaDeviceSynchronize(), "tensor-core kernel");
    check_status(m);
    ck(cudaMemcpy(d_host, m.d, sizeof(float) * kM * kN, cudaMemcpyDeviceToHost), "cudaMemcpy");
}

}  // namespace nexus

extern "C" int nexus_tensor_rate(int kind, int rounds, double *flops_per_s, double *ms)
{
    if (!flops_per_s) {
        nexus::set_error("nexus_tensor_rate: null argument");
        return -1;
    }
    try {
        *flops_per_s = nexus::tensor_rate(kind, rounds, ms);
    } catch (const std::exception &e) {
        nexus::set_error(std::string("nexus_tensor_rate: ") + e.what());
        return -1;
    }
    return 0;
}

extern "C" int nexus_tensor_tile(int kind, int rounds, const void *a, const void *b, float *d)
{
    if (!a || !b || !d) {
        nexus::set_error("nexus_tensor_tile: null argument");
        return -1;
    }
    try {
        nexus::tensor_tile(kind, rounds, a, b, d);
    } catch (const std::exception &e) {
        nexus::set_error(std::string("nexus_tensor_tile: ") + e.what());
        return -1;
    }
    return 0;
}
