// C ABI entry points (declared in include/nexus_gb300.h).  Each validates
// its arguments, converts C++ exceptions to a status code and records the
// message for nexus_last_error().
#include <stdexcept>
#include <string>

#include "../../include/nexus_gb300.h"
#include "context.h"
#include "ntt.h"

using namespace nexus;

namespace {

int fail(const char *fn, const std::string &msg)
{
    set_error(std::string(fn) + ": " + msg);
    return -1;
}

int check_launch(const char *fn)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(fn, cudaGetErrorString(e));
    return 0;
}

int check_limbs(const char *fn, const nexus_context *ctx, const void *d, int lb, int le)
{
    if (!ctx || !d) return fail(fn, "null argument");
    if (lb < 0 || le > ctx->c.k || lb >= le) return fail(fn, "limb range must satisfy 0 <= begin < end <= n_moduli");
    return 0;
}

}  // namespace

extern "C" int nexus_ntt_forward(nexus_context *ctx, uint64_t *d_data, size_t n_polys, int limb_begin, int limb_end,
                                 void *stream)
{
    static const char *fn = "nexus_ntt_forward";
    if (check_limbs(fn, ctx, d_data, limb_begin, limb_end)) return -1;
    try {
        ntt_forward(ctx->c, d_data, n_polys, limb_begin, limb_end, (cudaStream_t)stream);
    } catch (const std::exception &e) {
        return fail(fn, e.what());
    }
    return check_launch(fn);
}

extern "C" int nexus_ntt_inverse(nexus_context *ctx, uint64_t *d_data, size_t n_polys, int limb_begin, int limb_end,
                                 void *stream)
{
    static const char *fn = "nexus_ntt_inverse";
    if (check_limbs(fn, ctx, d_data, limb_begin, limb_end)) return -1;
    try {
        ntt_inverse(ctx->c, d_data, n_polys, limb_begin, limb_end, (cudaStream_t)stream);
    } catch (const std::exception &e) {
        return fail(fn, e.what());
    }
    return check_launch(fn);
}
