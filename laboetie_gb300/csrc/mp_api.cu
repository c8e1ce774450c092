// mp_api.cu -- C ABI of the tracer moment propagation (drop_tracers.f90:8-55,
// module_moment_propagation.f90:30-289,350-366).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"
#include "flow.h"
#include "lbgpu.h"
#include "trace.h"
#include "mp.h"

namespace lbg {

struct MpState {
    // FP32 slab step: tensor maps of V, P[0], P[1] for its bulk tensor copies (tma_ok)
    CUtensorMap tm[3];
    bool tma_ok = false;
    int prec = LBGPU_FP64;
    lbgpu_tracer tr{};
    int ads = 0;
    double K = 0, lambda = 0, bw = 0;
    MpArgs64 a64{};
    MpArgs32 a32{};
    std::vector<void *> allocs;
    unsigned nblocks = 0;
    int it_next = 1;
    int converged = 0;
    unsigned pending = 0;  // error raised at init, reported by the first propagate
    double vacf0[3] = {0, 0, 0};
};

void mp_release(lbgpu_ctx *ctx)
{
    if (!ctx->mp) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (void *p : ctx->mp->allocs) cudaFree(p);
    delete ctx->mp;
    ctx->mp = nullptr;
}

namespace {

template <typename T>
int alloc_zero(lbgpu_ctx *ctx, MpState *s, T **p, size_t count)
{
    LBG_CK(ctx, cudaMalloc((void **)p, count * sizeof(T)));
    s->allocs.push_back(*p);
    LBG_CK(ctx, cudaMemsetAsync(*p, 0, count * sizeof(T), ctx->stream));
    return LBGPU_OK;
}

constexpr double EPS = 2.220446049250313e-16;  // epsilon(1._dp)

// refresh ctx->d_rho / d_j with the moments of the current flow state
int flow_moments_on_device(lbgpu_ctx *ctx)
{
    return lbgpu_flow_get(ctx, nullptr, nullptr, nullptr, nullptr, nullptr);
}

}  // namespace
}  // namespace lbg

using namespace lbg;

extern "C" {

namespace lbg {
namespace {
int mp_init_impl(lbgpu_ctx *ctx, const lbgpu_tracer *tr, const double *density, const double *jx,
                 const double *jy, const double *jz, double vacf0[3], bool allow_charged);
}
}  // namespace lbg

int lbgpu_mp_init(lbgpu_ctx *ctx, const lbgpu_tracer *tr, const double *density, const double *jx,
                  const double *jy, const double *jz, double vacf0[3])
{
    TraceRange trace_("lbgpu_mp_init");
    return mp_init_impl(ctx, tr, density, jx, jy, jz, vacf0, false);
}

int lbgpu_mp_init_charged(lbgpu_ctx *ctx, const lbgpu_tracer *tr, const double *density,
                          const double *jx, const double *jy, const double *jz, double vacf0[3])
{
    TraceRange trace_("lbgpu_mp_init_charged");
    return mp_init_impl(ctx, tr, density, jx, jy, jz, vacf0, true);
}

}  // extern "C"

namespace lbg {
namespace {
int mp_init_impl(lbgpu_ctx *ctx, const lbgpu_tracer *tr, const double *density, const double *jx,
                 const double *jy, const double *jz, double vacf0[3], bool allow_charged)
{
    if (!ctx || !tr) return LBGPU_ERR_INVALID;
    if ((density == nullptr) != (jx == nullptr) || (jx == nullptr) != (jy == nullptr) ||
        (jy == nullptr) != (jz == nullptr))
        return ctx_fail(ctx, LBGPU_ERR_INVALID, "lbgpu_mp_init: give all of density, jx, jy, jz or none");
    // drop_tracers.f90:88-89 and module_moment_propagation.f90:41-79
    if (!(tr->Db > EPS))
        return ctx_fail(ctx, LBGPU_ERR_INVALID,
                        "The diffusion coefficient (tracer_Db in input file) is invalid");
    if (tr->ka < -EPS) return ctx_fail(ctx, LBGPU_ERR_INVALID, "I detected tracer%ka to be <0");
    if (tr->kd < -EPS) return ctx_fail(ctx, LBGPU_ERR_INVALID, "I detected tracer%kd to be <0");
    if (std::fabs(tr->Ds) > EPS)
        return ctx_fail(ctx, LBGPU_ERR_UNSUPPORTED,
                        "Tracers you defined have non-zero surface diffusion coefficient");
    const bool charged = std::fabs(tr->z) > EPS;
    if (charged && !allow_charged)
        return ctx_fail(ctx, LBGPU_ERR_UNSUPPORTED, "charged tracers are not implemented");
    const double *d_phi = charged ? pnp_potential(ctx) : nullptr;
    if (charged && !d_phi)
        return ctx_fail(ctx, LBGPU_ERR_INVALID,
                        "lbgpu_mp_init_charged: no potential (run lbgpu_pnp_init and the "
                        "Poisson-Nernst-Planck loop, or lbgpu_pnp_set, first)");
    const long long N = ctx->N;
    cudaStream_t st = ctx->stream;
    double K = std::fabs(tr->kd) <= EPS ? 0.0 : tr->ka / tr->kd;
    double Pstat = (double)ctx->counts[0] + K * (double)ctx->counts[2];  // :97
    if (charged) {
        // module_moment_propagation.f90:99-100 in the Fortran SUM order (storage order), on the
        // host: SUM(exp(-z phi)) over fluid nodes + SUM(exp(-z phi) K) over interfacial fluid
        std::vector<double> phi((size_t)N);
        std::vector<uint32_t> msk((size_t)N);
        LBG_CK(ctx, cudaMemcpyAsync(phi.data(), d_phi, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
        LBG_CK(ctx, cudaMemcpyAsync(msk.data(), ctx->d_mask, sizeof(uint32_t) * N, cudaMemcpyDeviceToHost, st));
        LBG_CK(ctx, cudaStreamSynchronize(st));
        double s1 = 0.0, s2 = 0.0;
        for (long long r = 0; r < N; ++r)
            if (msk[r] & FLUID_BIT) s1 = s1 + std::exp(-(tr->z * phi[r]));
        for (long long r = 0; r < N; ++r)
            if ((msk[r] & FLUID_BIT) && (msk[r] & INTERFACIAL_BIT)) s2 = s2 + std::exp(-(tr->z * phi[r])) * K;
        Pstat = s1 + s2;
    }
    mp_release(ctx);
    MpState *s = new MpState();
    ctx->mp = s;
    // the fused FP64 mode runs the FP64 tracer with fused gathers (a64.fused)
    s->prec = ctx->p.precision == LBGPU_FP32_DEV ? LBGPU_FP32_DEV : LBGPU_FP64;
    s->tr = *tr;
    s->K = K;
    s->ads = std::fabs(s->K) > EPS;
    const volatile double kBT = 1.0 / 3.0;
    s->lambda = 4.0 * tr->Db / kBT;                         // module_moment_propagation.f90:331-337
    s->bw = 1.0 / Pstat;
    int rc;

    // moments the tracer populations are built from (node%solventDensity / solventFlux)
    double *rho = ctx->d_rho, *J[3] = {ctx->d_j[0], ctx->d_j[1], ctx->d_j[2]};
    double *tmp = nullptr;
    if (density) {
        LBG_CK(ctx, cudaMallocAsync(&tmp, sizeof(double) * 4 * N, st));
        const double *h[4] = {density, jx, jy, jz};
        for (int q = 0; q < 4; ++q)
            LBG_CK(ctx, cudaMemcpyAsync(tmp + q * N, h[q], sizeof(double) * N, cudaMemcpyHostToDevice, st));
        rho = tmp;
        for (int d = 0; d < 3; ++d) J[d] = tmp + (d + 1) * N;
    } else {
        if (ctx->prev_kind == PREV_NONE)
            return ctx_fail(ctx, LBGPU_ERR_INVALID, "lbgpu_mp_init: no flow state and no moments given");
        if ((rc = flow_moments_on_device(ctx))) return rc;
    }

    MpArgs64 &a = s->a64;
    std::memset(&a, 0, sizeof(a));
    a.mask = ctx->d_mask;
    a.rho = rho;
    a.jx = J[0];
    a.jy = J[1];
    a.jz = J[2];
    a.N = N;
    a.lx = ctx->p.lx;
    a.ly = ctx->p.ly;
    a.lz = ctx->p.lz;
    a.ads = s->ads;
    a.lambda = s->lambda;
    a.ka = tr->ka;
    a.kd = tr->kd;
    a.one_minus_kd = 1.0 - tr->kd;
    a.bw = s->bw;
    for (int w = 0; w < 3; ++w) {
        a.a0[w] = ctx->K64.a0[w];
        a.a1[w] = ctx->K64.a1[w];
        const volatile double lw = s->lambda * ctx->K64.a0[w];
        a.lw[w] = lw;
        a.lwh[w] = lw * 0.5;
    }
    for (int d = 0; d < 3; ++d) {
        a.fext[d] = tr->f_ext[d];
        a.E[d] = tr->elec_slope[d];
    }
    a.q = tr->z;
    a.D = tr->Db;
    a.phi = d_phi;      // charged: exp(-z phi)/Pstat per node, fermi factors per link
    a.z = tr->z;
    a.pstat = Pstat;
    a.fused = ctx->p.precision == LBGPU_FP64_FUSED;
    a.fidx = ctx->d_fidx;
    a.Nf = ctx->d_fidx ? (long long)ctx->counts[0] : 0;
    s->nblocks = (unsigned)((N + MP_BLOCK - 1) / MP_BLOCK);
    int zc = 0;
    const unsigned resident = s->prec == LBGPU_FP64 ? 0u : mp32_slab_resident();
    const unsigned slab = s->prec == LBGPU_FP64 ? 0u : mp32_slab_grid(a.lx, a.ly, a.lz, resident, &zc);
    if ((rc = alloc_zero(ctx, s, &a.partial, 3 * (size_t)std::max(s->nblocks, slab)))) return rc;
    if ((rc = alloc_zero(ctx, s, &a.ctl, 1))) return rc;

    if (s->prec == LBGPU_FP64) {
        if ((rc = alloc_zero(ctx, s, &a.coef, (size_t)18 * N))) return rc;
        if ((rc = alloc_zero(ctx, s, &a.frac, (size_t)N))) return rc;
        for (int d = 0; d < 3; ++d)
            if ((rc = alloc_zero(ctx, s, &a.us[d], (size_t)N))) return rc;
        for (int b = 0; b < 2; ++b)
            for (int d = 0; d < 3; ++d) {
                if ((rc = alloc_zero(ctx, s, &a.P[b][d], (size_t)N))) return rc;
                if (s->ads && (rc = alloc_zero(ctx, s, &a.A[b][d], (size_t)N))) return rc;
            }
        LBG_CK(ctx, launch_mp_init_f64(a, s->nblocks, st));
    } else {
        MpArgs32 &b = s->a32;
        std::memset(&b, 0, sizeof(b));
        b.mask = ctx->d_mask;
        float4 *V;
        if ((rc = alloc_zero(ctx, s, &V, (size_t)N))) return rc;
        b.V = V;
        for (int q = 0; q < 2; ++q) {
            if ((rc = alloc_zero(ctx, s, &b.P[q], (size_t)N))) return rc;
            if (s->ads && (rc = alloc_zero(ctx, s, &b.A[q], (size_t)N))) return rc;
        }
        if ((rc = alloc_zero(ctx, s, &b.aux, (size_t)N))) return rc;
        b.partial = a.partial;
        b.ctl = a.ctl;
        b.N = N;
        b.lx = a.lx;
        b.ly = a.ly;
        b.lz = a.lz;
        b.ads = s->ads;
        // LBGPU_MP_TEST_SKIP_COPIES=1 (tests only): the slab step arms its barriers without
        // issuing the bulk copies, and its bounded waits (50 ms then) run out
        const char *skip_env = std::getenv("LBGPU_MP_TEST_SKIP_COPIES");
        b.skip_copies = skip_env && std::string(skip_env) == "1";
        b.wait_ns = b.skip_copies ? 50000000ull : 2000000000ull;
        // LBGPU_MP_SLAB=0: the grid-stride step everywhere (same per-node arithmetic)
        const char *slab_env = std::getenv("LBGPU_MP_SLAB");
        b.slab = !(slab_env && std::string(slab_env) == "0");
        if (ctx->aa && ctx->d_cpos) {   // in-place context: walk its fluid nodes
            b.cpos = ctx->d_cpos;
            b.Nf = ctx->Nf;
            b.xbits = ctx->xbits;
            b.ybits = ctx->ybits;
        }
        b.slab_resident = resident;
        b.ka = (float)tr->ka;
        b.kd = (float)tr->kd;
        b.one_minus_kd = (float)(1.0 - tr->kd);
        for (int w = 0; w < 3; ++w) {
            b.a1[w] = (float)a.a1[w];
            b.lwh[w] = (float)a.lwh[w];
            b.lw[w] = (float)a.lw[w];
        }
        b.charged = charged ? 1 : 0;
        b.z = (float)tr->z;
        b.inv_pstat = (float)(1.0 / Pstat);
        for (int d = 0; d < 3; ++d) b.E[d] = (float)tr->elec_slope[d];
        LBG_CK(ctx, launch_mp_v32(a, V, st));
        LBG_CK(ctx, launch_mp_init_f32(b, (float)s->bw, s->nblocks, st));
        // bulk tensor copies for the slab step's interior tiles (LBGPU_MP_TMA=0: per-thread copies)
        const char *tma_env = std::getenv("LBGPU_MP_TMA");
        s->tma_ok = !(tma_env && std::string(tma_env) == "0") && mp32_tensor_map(&s->tm[0], b.V, a.lx, a.ly, a.lz) &&
                    mp32_tensor_map(&s->tm[1], b.P[0], a.lx, a.ly, a.lz) &&
                    mp32_tensor_map(&s->tm[2], b.P[1], a.lx, a.ly, a.lz);
    }
    LBG_CK(ctx, launch_mp_reduce_init(a.partial, s->nblocks, a.ctl, st));
    if (tmp) LBG_CK(ctx, cudaFreeAsync(tmp, st));
    // the ρ/j pointers of the init are not used by the steps
    a.rho = a.jx = a.jy = a.jz = nullptr;
    MpCtl h;
    LBG_CK(ctx, cudaMemcpyAsync(&h, a.ctl, sizeof(h), cudaMemcpyDeviceToHost, st));
    LBG_CK(ctx, cudaStreamSynchronize(st));
    for (int d = 0; d < 3; ++d) s->vacf0[d] = h.vacf[d];
    if (vacf0)
        for (int d = 0; d < 3; ++d) vacf0[d] = h.vacf[d];
    s->pending = h.status & LBGPU_ERR_FRACTION;
    s->it_next = 1;
    return LBGPU_OK;
}
}  // namespace
}  // namespace lbg

extern "C" {

static int mp_run(lbgpu_ctx *ctx, int nsteps, double *vacf_out, int *steps_done, int *is_converged,
                  bool timing, float *ms)
{
    TraceRange trace_("moment propagation");
    MpState *s = ctx->mp;
    if (!s) return ctx_fail(ctx, LBGPU_ERR_INVALID, "moment propagation: call lbgpu_mp_init first");
    if (s->pending)
        return ctx_fail(ctx, LBGPU_ERR_FRACTION, "somewhere restpart is negative");
    if (steps_done) *steps_done = 0;
    if (is_converged) *is_converged = s->converged;
    if (nsteps <= 0) return LBGPU_OK;
    cudaStream_t st = ctx->stream;
    MpCtl c;
    LBG_CK(ctx, cudaMemcpyAsync(&c, s->a64.ctl, sizeof(c), cudaMemcpyDeviceToHost, st));
    LBG_CK(ctx, cudaStreamSynchronize(st));
    c.it = s->it_next;
    c.it_base = s->it_next;
    c.max_it = s->it_next + nsteps - 1;
    c.done = 0;
    c.converged = 0;
    c.blocks_done = 0;
    // module_moment_propagation.f90:284: |vacf| < 1/(2 lx ly lz / Db) and < 1.e-12 (a default real)
    if (timing) {
        c.thr1 = c.thr2 = -1.0;  // never converges: every step runs
    } else {
        const volatile double den = 2.0 * ctx->p.lx * ctx->p.ly * ctx->p.lz / s->tr.Db;
        c.thr1 = 1.0 / den;
        c.thr2 = (double)1.e-12f;
    }
    LBG_CK(ctx, cudaMemcpyAsync(s->a64.ctl, &c, sizeof(c), cudaMemcpyHostToDevice, st));
    double *hist = nullptr;
    if (!timing) LBG_CK(ctx, cudaMallocAsync(&hist, sizeof(double) * 3 * (size_t)nsteps, st));
    s->a64.hist = hist;
    s->a32.hist = hist;
    const int G = std::min(nsteps, 256);
    cudaGraph_t g;
    cudaGraphExec_t exec;
    LBG_CK(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < G; ++k) {
        // the FP64 step walks the fluid-node list: one thread per fluid node
        const unsigned grid = std::min(s->prec == LBGPU_FP64 && s->a64.fidx
                                           ? (unsigned)((s->a64.Nf + MP_BLOCK - 1) / MP_BLOCK)
                                           : s->nblocks,
                                       MP_MAX_BLOCKS);
        cudaError_t e = s->prec == LBGPU_FP64 ? launch_mp_step_f64(s->a64, grid, st)
                                              : launch_mp_step_f32(s->a32, grid, s->tma_ok ? s->tm : nullptr, st);
        if (e != cudaSuccess) {
            cudaStreamEndCapture(st, &g);
            return ctx_cuda(ctx, e, "capture moment propagation");
        }
    }
    LBG_CK(ctx, cudaStreamEndCapture(st, &g));
    LBG_CK(ctx, cudaGraphInstantiate(&exec, g, 0));
    cudaGraphDestroy(g);
    int rc = LBGPU_OK;
    if (timing) {
        LBG_CK(ctx, cudaEventRecord(ctx->ev0, st));
        for (int k = 0; k < (nsteps + G - 1) / G; ++k) LBG_CK(ctx, cudaGraphLaunch(exec, st));
        LBG_CK(ctx, cudaEventRecord(ctx->ev1, st));
        LBG_CK(ctx, cudaEventSynchronize(ctx->ev1));
        LBG_CK(ctx, cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1));
        LBG_CK(ctx, cudaMemcpyAsync(&c, s->a64.ctl, sizeof(c), cudaMemcpyDeviceToHost, st));
        LBG_CK(ctx, cudaStreamSynchronize(st));
    } else {
        for (;;) {
            cudaError_t e = cudaGraphLaunch(exec, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(&c, s->a64.ctl, sizeof(c), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) {
                rc = ctx_cuda(ctx, e, "moment propagation");
                break;
            }
            if (c.done || (c.status & LBGPU_ERR_TIMEOUT)) break;
        }
    }
    cudaGraphExecDestroy(exec);
    if (rc) return rc;
    if (c.status & LBGPU_ERR_TIMEOUT)
        return ctx_fail(ctx, LBGPU_ERR_TIMEOUT,
                        "moment propagation: a bulk copy into shared memory did not complete within its wait limit");
    const int done = c.last_it - c.it_base + 1;
    if (hist) {
        if (vacf_out && done > 0)
            LBG_CK(ctx, cudaMemcpyAsync(vacf_out, hist, sizeof(double) * 3 * (size_t)done,
                                        cudaMemcpyDeviceToHost, st));
        LBG_CK(ctx, cudaFreeAsync(hist, st));
        LBG_CK(ctx, cudaStreamSynchronize(st));
    }
    s->a64.hist = s->a32.hist = nullptr;
    s->it_next = c.last_it + 1;
    s->converged = c.converged;
    if (steps_done) *steps_done = done;
    if (is_converged) *is_converged = c.converged;
    return LBGPU_OK;
}

int lbgpu_mp_propagate(lbgpu_ctx *ctx, int nsteps, double *vacf, int *steps_done, int *is_converged)
{
    if (!ctx) return LBGPU_ERR_INVALID;
    return mp_run(ctx, nsteps, vacf, steps_done, is_converged, false, nullptr);
}

int lbgpu_time_mp_steps(lbgpu_ctx *ctx, int nsteps, float *ms)
{
    if (!ctx || !ms) return LBGPU_ERR_INVALID;
    return mp_run(ctx, nsteps, nullptr, nullptr, nullptr, true, ms);
}

int lbgpu_mp_get(lbgpu_ctx *ctx, double *P, double *P_ads)
{
    if (!ctx) return LBGPU_ERR_INVALID;
    MpState *s = ctx->mp;
    if (!s) return ctx_fail(ctx, LBGPU_ERR_INVALID, "lbgpu_mp_get: no moment propagation state");
    const long long N = ctx->N;
    cudaStream_t st = ctx->stream;
    MpCtl c;
    LBG_CK(ctx, cudaMemcpyAsync(&c, s->a64.ctl, sizeof(c), cudaMemcpyDeviceToHost, st));
    LBG_CK(ctx, cudaStreamSynchronize(st));
    const int par = c.parity;
    double *outs[2] = {P, P_ads};
    for (int q = 0; q < 2; ++q) {
        if (!outs[q]) continue;
        if (q == 1 && !s->ads) {
            std::memset(outs[q], 0, sizeof(double) * 3 * N);
            continue;
        }
        std::vector<double> comp((size_t)3 * N);
        for (int d = 0; d < 3; ++d) {
            if (s->prec == LBGPU_FP64) {
                const double *src = q == 0 ? s->a64.P[par][d] : s->a64.A[par][d];
                LBG_CK(ctx, cudaMemcpyAsync(comp.data() + d * N, src, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
            } else if (d == 0) {
                std::vector<float4> f(N);
                const float4 *src = q == 0 ? s->a32.P[par] : s->a32.A[par];
                LBG_CK(ctx, cudaMemcpyAsync(f.data(), src, sizeof(float4) * N, cudaMemcpyDeviceToHost, st));
                LBG_CK(ctx, cudaStreamSynchronize(st));
                for (long long i = 0; i < N; ++i) {
                    comp[i] = f[i].x;
                    comp[N + i] = f[i].y;
                    comp[2 * N + i] = f[i].z;
                }
            }
        }
        LBG_CK(ctx, cudaStreamSynchronize(st));
        for (long long i = 0; i < N; ++i)
            for (int d = 0; d < 3; ++d) outs[q][3 * i + d] = comp[d * N + i];
    }
    return LBGPU_OK;
}

int lbgpu_mp_set(lbgpu_ctx *ctx, const double *P, const double *P_ads, int it_next)
{
    if (!ctx) return LBGPU_ERR_INVALID;
    MpState *s = ctx->mp;
    if (!s) return ctx_fail(ctx, LBGPU_ERR_INVALID, "lbgpu_mp_set: call lbgpu_mp_init first");
    if (!P || it_next < 1 || (s->ads && !P_ads))
        return ctx_fail(ctx, LBGPU_ERR_INVALID, "lbgpu_mp_set: P (and P_ads with adsorption) and it_next >= 1");
    const long long N = ctx->N;
    cudaStream_t st = ctx->stream;
    MpCtl c;
    LBG_CK(ctx, cudaMemcpyAsync(&c, s->a64.ctl, sizeof(c), cudaMemcpyDeviceToHost, st));
    LBG_CK(ctx, cudaStreamSynchronize(st));
    const int par = c.parity;   // the buffers the next step reads
    const double *ins[2] = {P, s->ads ? P_ads : nullptr};
    for (int q = 0; q < 2; ++q) {
        if (!ins[q]) continue;
        if (s->prec == LBGPU_FP64) {
            std::vector<double> comp((size_t)3 * N);
            for (long long i = 0; i < N; ++i)
                for (int d = 0; d < 3; ++d) comp[d * N + i] = ins[q][3 * i + d];
            for (int d = 0; d < 3; ++d) {
                double *dst = q == 0 ? s->a64.P[par][d] : s->a64.A[par][d];
                LBG_CK(ctx, cudaMemcpyAsync(dst, comp.data() + d * N, sizeof(double) * N, cudaMemcpyHostToDevice, st));
            }
            LBG_CK(ctx, cudaStreamSynchronize(st));   // comp goes out of scope
        } else {
            std::vector<float4> f(N);
            for (long long i = 0; i < N; ++i)
                f[i] = make_float4((float)ins[q][3 * i], (float)ins[q][3 * i + 1], (float)ins[q][3 * i + 2], 0.0f);
            float4 *dst = q == 0 ? s->a32.P[par] : s->a32.A[par];
            LBG_CK(ctx, cudaMemcpyAsync(dst, f.data(), sizeof(float4) * N, cudaMemcpyHostToDevice, st));
            LBG_CK(ctx, cudaStreamSynchronize(st));
        }
    }
    s->it_next = it_next;
    s->converged = 0;
    return LBGPU_OK;
}

int lbgpu_mp_release(lbgpu_ctx *ctx)
{
    if (!ctx) return LBGPU_ERR_INVALID;
    mp_release(ctx);
    return LBGPU_OK;
}

}  // extern "C"
