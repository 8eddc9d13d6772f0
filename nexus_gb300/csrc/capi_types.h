// Definitions of the C ABI's opaque handles shared by the capi_*.cu units.
#pragma once
#include "../../include/nexus_gb300.h"
#include <stdexcept>

#include "batch.h"
#include "ckks.h"
#include "context.h"
#include "nexus_ops.h"

struct nexus_evaluator {
    nexus_context *ctx;
    nexus::Evaluator ev;
    nexus::CKKSEvaluator ck;
    nexus_evaluator(nexus_context *c, double scale) : ctx(c), ev(c->c), ck(ev, scale) {}
};

struct nexus_ciphertext {
    nexus_context *ctx;
    nexus::Ciphertext ct;
};

// an input ciphertext must hold data and belong to the evaluator's context
inline const char *input_problem(const nexus_context *ctx, const nexus_ciphertext *c)
{
    if (c->ctx != ctx) return "ciphertext belongs to another context";
    if (c->ct.empty()) return "ciphertext is empty";
    return nullptr;
}

// gather `count` ciphertexts of one size, level and scale into a batch
inline nexus::CtBatch gather_batch(nexus_evaluator *ev, const nexus_ciphertext *const *cts, int count)
{
    const nexus::Ciphertext &first = cts[0]->ct;
    if (first.empty()) throw std::invalid_argument("empty ciphertext");
    for (int b = 1; b < count; ++b) {
        const nexus::Ciphertext &c = cts[b]->ct;
        if (c.size() != first.size() || c.limbs() != first.limbs())
            throw std::invalid_argument("the ciphertexts of a batch must share one size and level");
        if (c.scale() != first.scale()) throw std::invalid_argument("the ciphertexts of a batch must share one scale");
    }
    nexus::Context &ctx = ev->ctx->c;
    cudaStream_t s = ev->ev.stream();
    nexus::CtBatch in;
    in.resize(ctx, count, first.size(), first.limbs(), s);
    in.scale() = first.scale();
    for (int b = 0; b < count; ++b)
        if (cudaMemcpyAsync(in.ct(b), cts[b]->ct.data(), in.words_per_ct() * 8, cudaMemcpyDeviceToDevice, s) !=
            cudaSuccess)
            throw std::runtime_error("copy failed");
    return in;
}

// copy ciphertext b of a batch into res[b]
inline void scatter_batch(nexus_evaluator *ev, const nexus::CtBatch &out, nexus_ciphertext *const *res)
{
    nexus::Context &ctx = ev->ctx->c;
    cudaStream_t s = ev->ev.stream();
    for (int b = 0; b < out.batch(); ++b) {
        nexus::Ciphertext &r = res[b]->ct;
        r.resize(ctx, out.size(), out.limbs(), s);
        r.scale() = out.scale();
        if (cudaMemcpyAsync(r.data(), out.ct(b), out.words_per_ct() * 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            throw std::runtime_error("copy failed");
    }
}
