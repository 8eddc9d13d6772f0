// Definitions of the C ABI's opaque handles shared by the capi_*.cu units.
#pragma once
#include "../../include/nexus_gb300.h"
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
