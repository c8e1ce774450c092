// flow_f32_api.cu -- host side of the FP32-deviation flow path (same C ABI as FP64).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "ctx.h"
#include "flow.h"
#include "lbgpu.h"

namespace lbg {

static void fill_args32(lbgpu_ctx *ctx, FlowArgs32 &a)
{
    std::memset(&a, 0, sizeof(a));
    const LbConst64 &K = ctx->K64;
    a.mask = ctx->d_mask;
    a.g0 = ctx->d_g[0];
    a.g1 = ctx->d_g[1];
    a.jx = ctx->d_j[0];
    a.jy = ctx->d_j[1];
    a.jz = ctx->d_j[2];
    a.rho = ctx->d_rho;
    a.N = ctx->N;
    a.lx = ctx->p.lx;
    a.ly = ctx->p.ly;
    a.lz = ctx->p.lz;
    for (int w = 0; w < 3; ++w) {
        a.w[w] = (float)K.a0[w];
        a.a1[w] = (float)K.a1[w];
        a.a2[w] = (float)K.a2[w];
        a.two_a2[w] = (float)K.two_a2[w];
        a.w64[w] = K.a0[w];
    }
    a.c1 = (float)K.c1;
    a.c2 = (float)K.c2;
    a.c3 = (float)K.c3;
    a.rho0 = (float)ctx->p.rho0;
    a.rho0d = ctx->p.rho0;
    for (int d = 0; d < 3; ++d) a.F[d] = (float)ctx->p.f_ext[d];
    a.minb_even = ctx->aa_minb[0];
    a.minb_odd = ctx->aa_minb[1];
    a.Nf = ctx->Nf;
    a.wide = ctx->aa_wide;
    a.nw = ctx->nw;
    a.cpos = ctx->d_cpos;
    a.cmask = ctx->d_cmask;
    a.rowtab = ctx->d_rowtab;
    a.xbits = ctx->xbits;
    a.ybits = ctx->ybits;
    const double c2 = K.c2, c3 = K.c3, cs2 = 1.0 / 3.0;
    for (int w = 0; w < 3; ++w) {
        a.c2w[w] = (float)(c2 * K.a0[w]);
        a.c2a1[w] = (float)(c2 * K.a1[w]);
        a.c2a2[w] = (float)(c2 * K.a2[w]);
        a.c2a2cs2[w] = (float)(c2 * K.a2[w] * cs2);
        a.c3a1[w] = (float)(c3 * K.a1[w]);
    }
    for (int p = 0; p < 9; ++p) {
        const int l = pair_l(p);
        const Vel c = vel(l);
        const double cF = c.x * ctx->p.f_ext[0] + c.y * ctx->p.f_ext[1] + c.z * ctx->p.f_ext[2];
        a.kF[p] = (float)(c3 * K.a1[wclass(l)] * cF);
        a.kT[p] = (float)(c3 * K.two_a2[wclass(l)] * cF);
    }
}

int f32_flow_init(lbgpu_ctx *ctx)
{
    FlowArgs32 a;
    fill_args32(ctx, a);
    LBG_CK(ctx, launch_init_f32(a, ctx->stream));
    ctx->aa_phase = 0;  // AA: the zero deviations are the natural-order state n_0
    ctx->cur = 0;
    ctx->prev_kind = PREV_RAW;
    ctx->prev_force_moment = 0;
    ctx->force_last_collide = 0;
    LBG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return LBGPU_OK;
}

int f32_flow_set(lbgpu_ctx *ctx, const double *n, const double *density, const double *jx,
                 const double *jy, const double *jz)
{
    const long long N = ctx->N;
    cudaStream_t s = ctx->stream;
    FlowArgs32 a;
    fill_args32(ctx, a);
    // populations page-locked by lbgpu_host_register are read in place by the conversion kernel
    // (no device copy of the FP64 array); others are staged through device memory
    double *tmp = nullptr;
    const double *src = static_cast<const double *>(pinned_device_view(n, sizeof(double) * Q * N));
    if (!src) {
        LBG_CK(ctx, cudaMallocAsync(&tmp, sizeof(double) * Q * N, s));
        LBG_CK(ctx, cudaMemcpyAsync(tmp, n, sizeof(double) * Q * N, cudaMemcpyHostToDevice, s));
        src = tmp;
    }
    if (ctx->aa) LBG_CK(ctx, launch_to_dev_compact32(a, src, ctx->d_g[0], s));
    else LBG_CK(ctx, launch_to_dev32(a, src, ctx->d_g[1], s));
    if (tmp) LBG_CK(ctx, cudaFreeAsync(tmp, s));
    if (ctx->aa) {
        // AA: the populations are the natural-order state; the next launch collides them with
        // the current phase's force.  density and j are implied by n.
        ctx->aa_phase = 0;
        ctx->prev_kind = PREV_RAW;
        ctx->prev_force_moment = ctx->force_last_collide;
        LBG_CK(ctx, cudaStreamSynchronize(s));
        return LBGPU_OK;
    }
    LBG_CK(ctx, cudaMemcpyAsync(ctx->d_rho, density, sizeof(double) * N, cudaMemcpyHostToDevice, s));
    const double *j[3] = {jx, jy, jz};
    for (int q = 0; q < 3; ++q)
        LBG_CK(ctx, cudaMemcpyAsync(ctx->d_j[q], j[q], sizeof(double) * N, cudaMemcpyHostToDevice, s));
    a.parity = 1;
    a.force_collide = ctx->force_last_collide;
    LBG_CK(ctx, launch_collide_f32(a, s));
    ctx->cur = 0;
    ctx->prev_kind = PREV_RAW;
    ctx->prev_force_moment = ctx->force_last_collide;
    LBG_CK(ctx, cudaStreamSynchronize(s));
    return LBGPU_OK;
}

int f32_flow_get(lbgpu_ctx *ctx, double *n, double *density, double *jx, double *jy, double *jz)
{
    if (ctx->prev_kind == PREV_NONE)
        return ctx_fail(ctx, LBGPU_ERR_INVALID, "lbgpu_flow_get: no flow state (call lbgpu_flow_init)");
    const long long N = ctx->N;
    cudaStream_t s = ctx->stream;
    FlowArgs32 a;
    fill_args32(ctx, a);
    a.parity = 1 - ctx->cur;
    a.force_moment = ctx->prev_force_moment;
    double *tmp = nullptr;
    if (n) {
        LBG_CK(ctx, cudaMallocAsync(&tmp, sizeof(double) * Q * N, s));
        a.nout = tmp;
    }
    if (ctx->aa) {
        // the AA kernels touch fluid nodes only: solid nodes report the reference's zeros
        LBG_CK(ctx, cudaMemsetAsync(ctx->d_rho, 0, sizeof(double) * N, s));
        for (int q = 0; q < 3; ++q) LBG_CK(ctx, cudaMemsetAsync(ctx->d_j[q], 0, sizeof(double) * N, s));
        if (tmp) LBG_CK(ctx, cudaMemsetAsync(tmp, 0, sizeof(double) * Q * N, s));
        LBG_CK(ctx, launch_aa_finalize_f32(a, ctx->aa_phase == 1, s));
    }
    else LBG_CK(ctx, launch_finalize_f32(a, ctx->prev_kind == PREV_POST, s));
    if (n) LBG_CK(ctx, cudaMemcpyAsync(n, tmp, sizeof(double) * Q * N, cudaMemcpyDeviceToHost, s));
    if (density) LBG_CK(ctx, cudaMemcpyAsync(density, ctx->d_rho, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
    double *j[3] = {jx, jy, jz};
    for (int q = 0; q < 3; ++q)
        if (j[q]) LBG_CK(ctx, cudaMemcpyAsync(j[q], ctx->d_j[q], sizeof(double) * N, cudaMemcpyDeviceToHost, s));
    if (tmp) LBG_CK(ctx, cudaFreeAsync(tmp, s));
    LBG_CK(ctx, cudaStreamSynchronize(s));
    return LBGPU_OK;
}

// Launch-bound tuner of the AA kernels: each variant (3..6 resident blocks per SM) of the even
// and of the odd launch is timed on a scratch copy of the box's populations (the state is not
// advanced), and the fastest is kept.  Small boxes (under 2^20 fluid nodes) keep the default;
// LBGPU_AA_MINB=<even>,<odd> fixes the variants and skips the tuner.
static int aa_tune(lbgpu_ctx *ctx)
{
    if (ctx->aa_tuned) return LBGPU_OK;
    ctx->aa_tuned = true;
    if (ctx->aa_minb_fixed || ctx->Nf < (1u << 20)) return LBGPU_OK;
    cudaStream_t s = ctx->stream;
    float *scratch = nullptr;
    const size_t bytes = sizeof(float) * Q * (size_t)ctx->Nf;
    if (cudaMallocAsync(&scratch, bytes, s) != cudaSuccess) {
        cudaGetLastError();   // no room for the scratch copy: keep the default variants
        return LBGPU_OK;
    }
    LBG_CK(ctx, cudaMemcpyAsync(scratch, ctx->d_g[0], bytes, cudaMemcpyDeviceToDevice, s));
    FlowArgs32 a;
    fill_args32(ctx, a);
    a.g0 = scratch;
    a.force_moment = a.force_collide = 1;
    for (int odd = 0; odd < 2; ++odd) {
        float best = 1e30f;
        for (int minb = 3; minb <= 6; ++minb) {
            a.minb_even = a.minb_odd = minb;
            for (int k = 0; k < 2; ++k) LBG_CK(ctx, launch_aa_step_f32(a, odd, s));
            LBG_CK(ctx, cudaEventRecord(ctx->ev0, s));
            for (int k = 0; k < 6; ++k) LBG_CK(ctx, launch_aa_step_f32(a, odd, s));
            LBG_CK(ctx, cudaEventRecord(ctx->ev1, s));
            LBG_CK(ctx, cudaEventSynchronize(ctx->ev1));
            float ms = 0.0f;
            LBG_CK(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
            if (ms < best) {
                best = ms;
                ctx->aa_minb[odd] = minb;
            }
        }
    }
    LBG_CK(ctx, cudaFreeAsync(scratch, s));
    LBG_CK(ctx, cudaStreamSynchronize(s));
    return LBGPU_OK;
}

// AA launches.  A launch computes the moments of the state it reads (force of the collision
// that produced it: prev_force_moment) and performs the next collision (force_last_collide);
// then the force of the following collision becomes force_on.  This reproduces the A/B
// bookkeeping step for step, so both layouts give identical results.
static int aa_steps(lbgpu_ctx *ctx, int nsteps, int force_on, float *ms)
{
    cudaStream_t s = ctx->stream;
    int rc0 = aa_tune(ctx);
    if (rc0) return rc0;
    FlowArgs32 a;
    fill_args32(ctx, a);
    auto one = [&]() -> int {
        a.force_moment = ctx->prev_force_moment;
        a.force_collide = ctx->force_last_collide;
        LBG_CK(ctx, launch_aa_step_f32(a, ctx->aa_phase == 1, s));
        ctx->aa_phase ^= 1;
        ctx->prev_force_moment = ctx->force_last_collide;
        ctx->force_last_collide = force_on;
        ctx->prev_kind = PREV_POST;
        return LBGPU_OK;
    };
    int rc;
    if (!ms) {
        for (int t = 0; t < nsteps; ++t)
            if ((rc = one())) return rc;
        return LBGPU_OK;
    }
    // settle the force bookkeeping and the parity outside the timed region
    int guard = 0;
    while ((ctx->prev_force_moment != force_on || ctx->force_last_collide != force_on ||
            ctx->aa_phase != 0) && guard++ < 4)
        if ((rc = one())) return rc;
    if (!ctx->graph_fixed[force_on] || ctx->graph_fixed_parity[force_on] != 0) {
        if (ctx->graph_fixed[force_on]) cudaGraphExecDestroy(ctx->graph_fixed[force_on]);
        cudaGraph_t g;
        LBG_CK(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        a.force_moment = force_on;
        a.force_collide = force_on;
        for (int k = 0; k < 2; ++k) {
            cudaError_t e = launch_aa_step_f32(a, k == 1, s);
            if (e != cudaSuccess) {
                cudaStreamEndCapture(s, &g);
                return ctx_cuda(ctx, e, "capture");
            }
        }
        LBG_CK(ctx, cudaStreamEndCapture(s, &g));
        LBG_CK(ctx, cudaGraphInstantiate(&ctx->graph_fixed[force_on], g, 0));
        cudaGraphDestroy(g);
        ctx->graph_fixed_parity[force_on] = 0;
    }
    LBG_CK(ctx, cudaEventRecord(ctx->ev0, s));
    for (int k = 0; k < nsteps / 2; ++k) LBG_CK(ctx, cudaGraphLaunch(ctx->graph_fixed[force_on], s));
    if (nsteps & 1)
        if ((rc = one())) return rc;
    LBG_CK(ctx, cudaEventRecord(ctx->ev1, s));
    LBG_CK(ctx, cudaEventSynchronize(ctx->ev1));
    LBG_CK(ctx, cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1));
    return LBGPU_OK;
}

// The reference loop of equilibration.f90:143-491 on an FP32 in-place context: graphs of
// (AA launch of step t, check launch of S_t) pairs; each check decides the forces of the next AA
// launch on the device, launches after the exit return at once, and the host only reads the
// control block between graphs.
int f32_equilibration(lbgpu_ctx *ctx, int max_steps, double *l2err_hist, int hist_cap, int *steps_out)
{
    if (!ctx->aa)
        return ctx_fail(ctx, LBGPU_ERR_UNSUPPORTED,
                        "lbgpu_equilibration: the FP32 reference loop runs in the in-place layout");
    int rc = aa_tune(ctx);
    if (rc) return rc;
    // j_old of the first check: the moments of the current state
    if ((rc = f32_flow_get(ctx, nullptr, nullptr, nullptr, nullptr, nullptr))) return rc;
    cudaStream_t s = ctx->stream;
    double *d_hist = nullptr;
    if (hist_cap > 0) {
        LBG_CK(ctx, cudaMallocAsync(&d_hist, sizeof(double) * hist_cap, s));
        LBG_CK(ctx, cudaMemsetAsync(d_hist, 0, sizeof(double) * hist_cap, s));
    }
    FlowCtl c;
    std::memset(&c, 0, sizeof(c));
    c.t = 1;
    c.max_steps = max_steps;
    c.target_error = ctx->p.target_error;
    c.hist_cap = hist_cap;
    c.aa_fm = ctx->prev_force_moment;   // moments of the current state
    c.aa_fc = 0;                        // phase A: no force (equilibration.f90:143-190)
    c.check_fm = 0;
    c.exit_phase = ctx->aa_phase;
    LBG_CK(ctx, cudaMemcpyAsync(ctx->d_ctl, &c, sizeof(c), cudaMemcpyHostToDevice, s));
    FlowArgs32 a;
    fill_args32(ctx, a);
    a.ctl = ctx->d_ctl;
    a.hist = d_hist;
    // an even number of (AA, check) pairs per graph, so every replay starts at the same phase
    const int G = 2 * (int)std::min<long long>(128, std::max<long long>(4, (1LL << 23) / std::max<unsigned>(ctx->Nf, 1u)));
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    LBG_CK(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < G; ++k) {
        const bool odd = ((ctx->aa_phase + k) & 1) != 0;   // an even launch leaves the state swapped
        cudaError_t e = launch_aa_step_f32(a, odd, s);
        if (e == cudaSuccess) e = launch_aa_check_f32(a, !odd, s);
        if (e != cudaSuccess) {
            cudaStreamEndCapture(s, &graph);
            return ctx_cuda(ctx, e, "capture FP32 reference loop");
        }
    }
    LBG_CK(ctx, cudaStreamEndCapture(s, &graph));
    LBG_CK(ctx, cudaGraphInstantiate(&exec, graph, 0));
    cudaGraphDestroy(graph);
    FlowCtl h;
    rc = LBGPU_OK;
    for (;;) {
        cudaError_t e = cudaGraphLaunch(exec, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&h, ctx->d_ctl, sizeof(h), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            rc = ctx_cuda(ctx, e, "lbgpu_equilibration (FP32)");
            break;
        }
        if (h.done) break;
    }
    cudaGraphExecDestroy(exec);
    if (rc) return rc;
    ctx->aa_phase = h.exit_phase;
    ctx->prev_force_moment = h.exit_force_moment;
    ctx->force_last_collide = h.aa_fc;
    ctx->prev_kind = PREV_POST;
    if (steps_out) *steps_out = h.exit_step;
    if (d_hist) {
        LBG_CK(ctx, cudaMemcpyAsync(l2err_hist, d_hist, sizeof(double) * hist_cap, cudaMemcpyDeviceToHost, s));
        LBG_CK(ctx, cudaFreeAsync(d_hist, s));
    }
    LBG_CK(ctx, cudaStreamSynchronize(s));
    if (h.status & LBGPU_ERR_NEGATIVE_POPULATION)
        return ctx_fail(ctx, LBGPU_ERR_NEGATIVE_POPULATION, "In equilibration, the population n(x,y,z,vel) < 0");
    if (h.status & LBGPU_ERR_NONFINITE)
        return ctx_fail(ctx, LBGPU_ERR_NONFINITE, "equilibration: non-finite population");
    if (h.status & LBGPU_ERR_STEP_CAP)
        return ctx_fail(ctx, LBGPU_ERR_STEP_CAP, "equilibration: step cap reached before the second convergence");
    return LBGPU_OK;
}

int f32_flow_steps(lbgpu_ctx *ctx, int nsteps, int force_on, float *ms)
{
    force_on = force_on ? 1 : 0;
    if (ctx->aa) return aa_steps(ctx, nsteps, force_on, ms);
    cudaStream_t s = ctx->stream;
    FlowArgs32 a;
    fill_args32(ctx, a);
    auto one = [&]() -> int {
        a.parity = ctx->cur;
        a.force_moment = ctx->force_last_collide;
        a.force_collide = force_on;
        LBG_CK(ctx, launch_flow_step_f32(a, 0, s));
        ctx->prev_force_moment = ctx->force_last_collide;
        ctx->force_last_collide = force_on;
        ctx->cur ^= 1;
        ctx->prev_kind = PREV_POST;
        return LBGPU_OK;
    };
    int rc;
    if (!ms) {
        for (int t = 0; t < nsteps; ++t)
            if ((rc = one())) return rc;
        return LBGPU_OK;
    }
    if (ctx->force_last_collide != force_on)
        if ((rc = one())) return rc;
    if (!ctx->graph_fixed[force_on] || ctx->graph_fixed_parity[force_on] != ctx->cur) {
        if (ctx->graph_fixed[force_on]) cudaGraphExecDestroy(ctx->graph_fixed[force_on]);
        cudaGraph_t g;
        LBG_CK(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < 2; ++k) {
            a.parity = ctx->cur ^ k;
            a.force_moment = force_on;
            a.force_collide = force_on;
            cudaError_t e = launch_flow_step_f32(a, 0, s);
            if (e != cudaSuccess) {
                cudaStreamEndCapture(s, &g);
                return ctx_cuda(ctx, e, "capture");
            }
        }
        LBG_CK(ctx, cudaStreamEndCapture(s, &g));
        LBG_CK(ctx, cudaGraphInstantiate(&ctx->graph_fixed[force_on], g, 0));
        cudaGraphDestroy(g);
        ctx->graph_fixed_parity[force_on] = ctx->cur;
    }
    LBG_CK(ctx, cudaEventRecord(ctx->ev0, s));
    for (int k = 0; k < nsteps / 2; ++k) LBG_CK(ctx, cudaGraphLaunch(ctx->graph_fixed[force_on], s));
    if (nsteps & 1) {
        if ((rc = one())) return rc;
    } else if (nsteps > 0) {
        ctx->prev_force_moment = force_on;
        ctx->prev_kind = PREV_POST;
    }
    LBG_CK(ctx, cudaEventRecord(ctx->ev1, s));
    LBG_CK(ctx, cudaEventSynchronize(ctx->ev1));
    LBG_CK(ctx, cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1));
    return LBGPU_OK;
}

}  // namespace lbg
