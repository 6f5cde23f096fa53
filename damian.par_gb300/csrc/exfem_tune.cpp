// exfem_tune.cpp — the autotuner of the FP32 step (exfem_gpu_autotune).
//
// It times every candidate shape of the FP32 form on the caller's own model
// and keeps the fastest: kernel variant (0 direct gather, 4 the same as a
// persistent grid, 5 the direct gather in its list form from 50,000 nodes,
// where 0 reads fixed-size node records, 1 shared-memory tiles, 2 bulk-copy
// pipeline when nrhs is a multiple of 4, 3 tensor-core step when nrhs is a
// multiple of 16), block size (128, 256, 512) and right-hand sides per
// thread (1, 2, 4 dividing nrhs).
// Each candidate gets its own context (exfem_gpu_create with that shape), a
// few warm-up steps, and a burst timed with CUDA events on the context's
// stream (exfem_gpu_run_timed).  Results are cached in the process per
// (elements, nodes, right-hand sides, device), so a host that creates many
// contexts on one mesh tunes once.  No counterpart in the reference, whose
// element loop has one shape (explicit.f90:129-142).
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "exfem_ctx.h"
#include "exfem_gpu.h"
#include "exfem_plan.h"

namespace {

struct TuneKey {
    int ne, nn, nrhs, device, max_variant;
    bool operator<(const TuneKey &o) const {
        return std::tie(ne, nn, nrhs, device, max_variant) < std::tie(o.ne, o.nn, o.nrhs, o.device, o.max_variant);
    }
};
struct TuneVal {
    int variant, block_threads, rhs_per_thread;
    double ms_per_step;
};

std::mutex g_tune_mu;
std::map<TuneKey, TuneVal> g_tune_cache;

// Steps per captured graph (exfem_gpu_run's rule).
int graph_len(const exfem_opts &o) {
    int g = o.graph_steps > 0 ? o.graph_steps : 16;
    return g + (g & 1);
}

// Steps a candidate runs before its timed steps: `warmup` and one graph's
// worth, rounded up to an even count, so that the graph is captured and
// instantiated before the clock starts and the timed steps begin at the
// parity it was captured from.
int pre_steps(const exfem_opts &o, int warmup) {
    const int n = warmup + (o.use_graph ? graph_len(o) : 0);
    return n + (n & 1);
}

// The timed steps: `steps` rounded up to whole graph replays, so the timing
// is of replays only (as a long run is), not of single-step launches.
int timed_steps(const exfem_opts &o, int steps) {
    if (!o.use_graph) return steps;
    const int g = graph_len(o);
    return std::max(g, (steps + g - 1) / g * g);
}

// Times `steps` steps after pre_steps(o, warmup) of one candidate; < 0 when
// the candidate cannot run (unsupported shape, out of memory, failed step).
double time_candidate(const exfem_mesh *mesh, const exfem_problem *prob, const exfem_opts &o, int warmup,
                      int steps) {
    exfem_ctx *ctx = nullptr;
    if (exfem_gpu_create(mesh, prob, &o, &ctx) != EXFEM_OK) return -1.0;
    double ms = -1.0;
    if (exfem_gpu_init_explicit(ctx, nullptr) == EXFEM_OK && exfem_gpu_run(ctx, pre_steps(o, warmup)) == EXFEM_OK &&
        exfem_gpu_sync(ctx) == EXFEM_OK) {
        double t = 0.0;
        if (exfem_gpu_run_timed(ctx, steps, &t) == EXFEM_OK && exfem_gpu_sync(ctx) == EXFEM_OK) ms = t / steps;
    }
    exfem_gpu_destroy(ctx);
    return ms;
}

}  // namespace

namespace exfem {

// The tuner behind exfem_gpu_autotune, over variants 0..max_variant (the
// server tunes the direct gather only: its admission reserved that
// variant's footprint).
int autotune_shapes(const exfem_mesh *mesh, const exfem_problem *prob, exfem_opts *opts, int steps, int max_variant,
                    double *ms_per_step) {
    if (!mesh || !prob || !opts || steps < 1 || steps > 1000) return EXFEM_E_ARG;
    if (opts->precision != EXFEM_FP32_KAHAN) return EXFEM_E_ARG;
    // the right-hand sides the context will carry (an odd count is padded)
    const int R = std::max(opts->pad_rhs == 0 ? padded_rhs(prob->nrhs) : prob->nrhs, 1);
    const TuneKey key{mesh->nelems, mesh->nnodes, R, opts->device, max_variant};
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            opts->variant = it->second.variant;
            opts->block_threads = it->second.block_threads;
            opts->rhs_per_thread = it->second.rhs_per_thread;
            if (ms_per_step) *ms_per_step = it->second.ms_per_step;
            return EXFEM_OK;
        }
    }
    const int warmup = 3;
    exfem_problem p = *prob;   // enough steps for the timing, whatever the problem's length
    const int tsteps = timed_steps(*opts, steps);
    p.nsteps = pre_steps(*opts, warmup) + tsteps;
    if (p.io_interval < 1) p.io_interval = 1;
    std::vector<int> variants = {0, 4};
    if (mesh->nnodes >= kSlotMinNodes) variants.push_back(5);
    if (max_variant >= 1) variants.push_back(1);
    if (max_variant >= 2 && R % 4 == 0) variants.push_back(2);
    if (max_variant >= 3 && R % 16 == 0) variants.push_back(3);
    TuneVal best{-1, 0, 0, 0.0};
    for (int v : variants)
        for (int rpt : {1, 2, 4}) {
            if (R % rpt || (v == 3 && rpt != 2)) continue;   // the tensor-core step has one shape
            for (int bt : {128, 256, 512}) {
                if (v == 3 && bt != 256) continue;
                exfem_opts o = *opts;
                o.variant = v;
                o.block_threads = bt;
                o.rhs_per_thread = rpt;
                const double ms = time_candidate(mesh, &p, o, warmup, tsteps);
                if (ms > 0.0 && (best.variant < 0 || ms < best.ms_per_step)) best = TuneVal{v, bt, rpt, ms};
            }
        }
    if (best.variant < 0) return EXFEM_E_CUDA;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_cache[key] = best;
    }
    opts->variant = best.variant;
    opts->block_threads = best.block_threads;
    opts->rhs_per_thread = best.rhs_per_thread;
    if (ms_per_step) *ms_per_step = best.ms_per_step;
    return EXFEM_OK;
}

}  // namespace exfem

extern "C" int exfem_gpu_autotune(const exfem_mesh *mesh, const exfem_problem *prob, exfem_opts *opts, int steps,
                                  double *ms_per_step) {
    return exfem::autotune_shapes(mesh, prob, opts, steps, 3, ms_per_step);
}
