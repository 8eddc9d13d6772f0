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
