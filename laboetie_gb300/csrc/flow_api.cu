// flow_api.cu -- C ABI of the flow phase: device set-up, state transfers, the reference
// operators on host arrays, and the device-resident step loop (equilibration.f90:143-491).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "compact.cuh"
#include "ctx.h"
#include "flow.h"
#include "lbgpu.h"
#include "trace.h"

using namespace lbg;

namespace lbg {

namespace {

template <typename T>
cudaError_t dalloc(T **p, size_t count)
{
    return cudaMalloc((void **)p, count * sizeof(T));
}

void free_op(lbgpu_ctx *ctx)
{
    if (!ctx->op) return;
    for (auto *p : ctx->op->n) cudaFree(p);
    for (auto *p : ctx->op->m) cudaFree(p);
    for (auto *p : ctx->op->F) cudaFree(p);
    delete ctx->op;
    ctx->op = nullptr;
}

// AA layout over the fluid nodes (ctx.h): compact index in lattice order, packed positions and
// row bitmask table built on the host from nature; flag words gathered on the device.
int build_compact_layout(lbgpu_ctx *ctx, const int8_t *nature)
{
    const int lx = ctx->p.lx, ly = ctx->p.ly, lz = ctx->p.lz;
    std::vector<uint2> tab;
    std::vector<uint32_t> pos;
    int nw = 0, xbits = 0, ybits = 0;
    if (!build_compact_tables(lx, ly, lz, nature, tab, pos, nw, xbits, ybits))
        return ctx_fail(ctx, LBGPU_ERR_INVALID,
                        "FP32 in-place streaming: box shape beyond the packed-position limits "
                        "(use LBGPU_FP32_STREAMING=ab)");
    const uint32_t c = (uint32_t)pos.size();
    ctx->Nf = c;
    ctx->nw = nw;
    ctx->xbits = xbits;
    ctx->ybits = ybits;
    cudaStream_t s = ctx->stream;
    LBG_CK(ctx, dalloc(&ctx->d_rowtab, tab.size()));
    LBG_CK(ctx, dalloc(&ctx->d_cpos, pos.size()));
    LBG_CK(ctx, dalloc(&ctx->d_cmask, pos.size()));
    LBG_CK(ctx, cudaMemcpyAsync(ctx->d_rowtab, tab.data(), sizeof(uint2) * tab.size(), cudaMemcpyHostToDevice, s));
    LBG_CK(ctx, cudaMemcpyAsync(ctx->d_cpos, pos.data(), sizeof(uint32_t) * pos.size(), cudaMemcpyHostToDevice, s));
    FlowArgs32 a;
    std::memset(&a, 0, sizeof(a));
    a.mask = ctx->d_mask;
    a.Nf = c;
    a.cpos = ctx->d_cpos;
    a.lx = lx;
    a.ly = ly;
    a.xbits = xbits;
    a.ybits = ybits;
    LBG_CK(ctx, launch_compact_mask(a, ctx->d_cmask, s));
    LBG_CK(ctx, cudaStreamSynchronize(s));   // host tables go out of scope
    return LBGPU_OK;
}

// dst[i] = src[i], 16 bytes per thread: a device copy of a host array read in place through its
// page-locked mapping
__global__ void k_copy16(const double2 *__restrict__ src, double2 *__restrict__ dst, size_t n2)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

// Host -> device copy of `count` doubles: read in place by a kernel when the host range lies in
// one range registered by lbgpu_host_register (the copy runs at the link's read bandwidth and
// with the kernel's many loads in flight), else by cudaMemcpyAsync.
cudaError_t upload_f64(double *dst, const double *src, size_t count, cudaStream_t s)
{
    const void *view = pinned_device_view(src, sizeof(double) * count);
    if (view && count % 2 == 0 && ((uintptr_t)view & 15u) == 0 && ((uintptr_t)dst & 15u) == 0) {
        const size_t n2 = count / 2;
        const unsigned grid = (unsigned)std::min<size_t>((n2 + 255) / 256, 152u * 16u);
        k_copy16<<<grid, 256, 0, s>>>(static_cast<const double2 *>(view), reinterpret_cast<double2 *>(dst), n2);
        return cudaGetLastError();
    }
    return cudaMemcpyAsync(dst, src, sizeof(double) * count, cudaMemcpyHostToDevice, s);
}

// LBGPU_ERR_OOM unless `need` bytes are free on the device
int check_room(lbgpu_ctx *ctx, size_t need)
{
    size_t fr = 0, tot = 0;
    LBG_CK(ctx, cudaMemGetInfo(&fr, &tot));
    if (need > fr)
        return ctx_fail(ctx, LBGPU_ERR_OOM,
                        "lbgpu_create: box needs " + std::to_string(need >> 20) + " MiB, " +
                            std::to_string(fr >> 20) + " MiB free on the device");
    return LBGPU_OK;
}

}  // namespace

int ctx_init_device(lbgpu_ctx *ctx, const int8_t *nature)
{
    const lbgpu_params &p = ctx->p;
    const long long N = ctx->N;
    LBG_CK(ctx, cudaSetDevice(p.device));
    LBG_CK(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    LBG_CK(ctx, cudaEventCreate(&ctx->ev0));
    LBG_CK(ctx, cudaEventCreate(&ctx->ev1));
    // per lattice node: nature, flag word, rho and j (FP64), and for FP64 two population sets;
    // FP32 populations are checked once the layout (A/B or fluid nodes only) is known
    const size_t pop = p.precision != LBGPU_FP32_DEV ? 2 * Q * sizeof(double) : 0;
    if (int rc = check_room(ctx, (size_t)N * (1 + 4 + pop + 4 * sizeof(double)) + (1 << 20))) return rc;
    LBG_CK(ctx, dalloc(&ctx->d_nature, N));
    LBG_CK(ctx, dalloc(&ctx->d_mask, N));
    LBG_CK(ctx, cudaMemcpyAsync(ctx->d_nature, nature, N, cudaMemcpyHostToDevice, ctx->stream));
    LBG_CK(ctx, launch_node_flags(ctx->d_nature, ctx->d_mask, p.lx, p.ly, p.lz, ctx->stream));
    LBG_CK(ctx, dalloc(&ctx->d_scratch, 1));
    LBG_CK(ctx, cudaMemsetAsync(ctx->d_scratch, 0, sizeof(Scratch), ctx->stream));
    LBG_CK(ctx, launch_count_nodes(ctx->d_mask, N, ctx->d_scratch->counts, ctx->stream));
    LBG_CK(ctx, cudaMemcpyAsync(ctx->counts, ctx->d_scratch->counts, sizeof(ctx->counts),
                                cudaMemcpyDeviceToHost, ctx->stream));
    LBG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->counts[0] == 0)  // supercell_definition.f90:189-191
        return ctx_fail(ctx, LBGPU_ERR_INVALID, "All nodes are solid: no fluid, no fluid dynamics!");
    if (p.precision != LBGPU_FP32_DEV) {
        for (int b = 0; b < 2; ++b) LBG_CK(ctx, dalloc(&ctx->d_f[b], (size_t)Q * N));
        std::vector<uint32_t> fidx;
        fidx.reserve(ctx->counts[0]);
        for (long long i = 0; i < N; ++i)
            if (nature[i] == 0) fidx.push_back((uint32_t)i);
        if (fidx.size() != ctx->counts[0])
            return ctx_fail(ctx, LBGPU_ERR_CUDA, "fluid node count differs between host and device");
        LBG_CK(ctx, dalloc(&ctx->d_fidx, fidx.size()));
        LBG_CK(ctx, cudaMemcpyAsync(ctx->d_fidx, fidx.data(), sizeof(uint32_t) * fidx.size(),
                                    cudaMemcpyHostToDevice, ctx->stream));
        LBG_CK(ctx, cudaStreamSynchronize(ctx->stream));   // the host list goes out of scope
    } else {
        const char *mode = std::getenv("LBGPU_FP32_STREAMING");
        ctx->aa = !(mode && std::string(mode) == "ab");
        // AA: one set of Q*Nf populations + packed position and flag word per fluid node; A/B: two
        // sets per lattice node
        const unsigned long long nf = ctx->counts[0];
        if (int rc = check_room(ctx, ctx->aa ? nf * (Q * sizeof(float) + 8) : 2ull * Q * sizeof(float) * N))
            return rc;
        // beyond 2^32 slots the odd launches form 64-bit offsets (LBGPU_AA_WIDE=1 forces them)
        const char *wide = std::getenv("LBGPU_AA_WIDE");
        ctx->aa_wide = (unsigned long long)Q * nf >= (1ULL << 32) || (wide && std::string(wide) == "1");
        if (const char *e = std::getenv("LBGPU_AA_MINB")) {  // "<even>,<odd>", e.g. "4,3"
            int ev = 0, od = 0;
            if (std::sscanf(e, "%d,%d", &ev, &od) == 2) {
                ctx->aa_minb[0] = ev;
                ctx->aa_minb[1] = od;
                ctx->aa_minb_fixed = true;
            }
        }
        if (ctx->aa) {
            int rc = build_compact_layout(ctx, nature);
            if (rc) return rc;
            LBG_CK(ctx, dalloc(&ctx->d_g[0], (size_t)Q * ctx->Nf));
        } else {
            for (int b = 0; b < 2; ++b) LBG_CK(ctx, dalloc(&ctx->d_g[b], (size_t)Q * N));
        }
    }
    for (int d = 0; d < 3; ++d) LBG_CK(ctx, dalloc(&ctx->d_j[d], N));
    LBG_CK(ctx, dalloc(&ctx->d_rho, N));
    LBG_CK(ctx, dalloc(&ctx->d_ctl, 1));
    LBG_CK(ctx, cudaMemsetAsync(ctx->d_ctl, 0, sizeof(FlowCtl), ctx->stream));
    return LBGPU_OK;
}


void ctx_release_device(lbgpu_ctx *ctx)
{
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    mp_release(ctx);
    pnp_release(ctx);
    free_op(ctx);
    if (ctx->graph_ref) cudaGraphExecDestroy(ctx->graph_ref);
    for (int f = 0; f < 2; ++f)
        if (ctx->graph_fixed[f]) cudaGraphExecDestroy(ctx->graph_fixed[f]);
    cudaFree(ctx->d_nature);
    cudaFree(ctx->d_mask);
    cudaFree(ctx->d_fidx);
    cudaFree(ctx->d_cpos);
    cudaFree(ctx->d_cmask);
    cudaFree(ctx->d_rowtab);
    for (int b = 0; b < 2; ++b) {
        cudaFree(ctx->d_f[b]);
        cudaFree(ctx->d_g[b]);
    }
    for (int d = 0; d < 3; ++d) {
        cudaFree(ctx->d_j[d]);
        cudaFree(ctx->d_F[d]);
    }
    cudaFree(ctx->d_rho);
    cudaFree(ctx->d_ctl);
    cudaFree(ctx->d_scratch);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
}

}  // namespace lbg

namespace {

OpBuffers *op_buffers(lbgpu_ctx *ctx, int &rc)
{
    rc = LBGPU_OK;
    if (ctx->op) return ctx->op;
    OpBuffers *o = new OpBuffers();
    const long long N = ctx->N;
    cudaError_t err = cudaSuccess;
    for (int b = 0; b < 2 && err == cudaSuccess; ++b) err = cudaMalloc(&o->n[b], sizeof(double) * Q * N);
    for (int q = 0; q < 4 && err == cudaSuccess; ++q) err = cudaMalloc(&o->m[q], sizeof(double) * N);
    for (int d = 0; d < 3 && err == cudaSuccess; ++d) err = cudaMalloc(&o->F[d], sizeof(double) * N);
    ctx->op = o;
    if (err != cudaSuccess) {
        rc = ctx_cuda(ctx, err, "operator buffers");
        free_op(ctx);
        return nullptr;
    }
    return o;
}

}  // namespace

namespace {

int need_fp64(lbgpu_ctx *ctx, const char *fn)
{
    if (ctx->p.precision == LBGPU_FP32_DEV)
        return ctx_fail(ctx, LBGPU_ERR_INVALID, std::string(fn) + ": needs an FP64 context");
    return LBGPU_OK;
}

int read_scratch(lbgpu_ctx *ctx, Scratch &s)
{
    LBG_CK(ctx, cudaMemcpyAsync(&s, ctx->d_scratch, sizeof(Scratch), cudaMemcpyDeviceToHost, ctx->stream));
    LBG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return LBGPU_OK;
}

int reset_scratch(lbgpu_ctx *ctx)
{
    LBG_CK(ctx, cudaMemsetAsync(ctx->d_scratch, 0, 16, ctx->stream));
    return LBGPU_OK;
}

}  // namespace

// FP32-deviation entry points live in flow_f32_api.cu
namespace lbg {
int f32_flow_init(lbgpu_ctx *ctx);
int f32_flow_set(lbgpu_ctx *ctx, const double *n, const double *density, const double *jx,
                 const double *jy, const double *jz);
int f32_flow_get(lbgpu_ctx *ctx, double *n, double *density, double *jx, double *jy, double *jz);
int f32_equilibration(lbgpu_ctx *ctx, int max_steps, double *l2err_hist, int hist_cap, int *steps_out);
int f32_flow_steps(lbgpu_ctx *ctx, int nsteps, int force_on, float *ms);
}  // namespace lbg

extern "C" {

int lbgpu_flow_init(lbgpu_ctx *ctx)
{
    if (!ctx) return LBGPU_ERR_INVALID;
    if (ctx->p.precision == LBGPU_FP32_DEV) return f32_flow_init(ctx);
    FlowArgs64 a;
    fill_args64(ctx, a);
    a.parity = 1;  // raw n = w*rho into buffer 1
    LBG_CK(ctx, launch_init_f64(a, ctx->p.rho0, ctx->stream));
    a.force_collide = 0;  // collision of step 1 is without force (equilibration.f90:94-96)
    LBG_CK(ctx, launch_collide_f64(a, 0, false, ctx->stream));
    ctx->cur = 0;
    ctx->prev_kind = PREV_RAW;
    ctx->prev_force_moment = 0;
    ctx->force_last_collide = 0;
    ctx->moments_valid = true;
    return lbgpu_sync(ctx);
}

int lbgpu_flow_set(lbgpu_ctx *ctx, const double *n, const double *density, const double *jx,
                   const double *jy, const double *jz)
{
    if (!ctx || !n || !density || !jx || !jy || !jz) return LBGPU_ERR_INVALID;
    if (ctx->p.precision == LBGPU_FP32_DEV) return f32_flow_set(ctx, n, density, jx, jy, jz);
    const long long N = ctx->N;
    cudaStream_t s = ctx->stream;
    LBG_CK(ctx, upload_f64(ctx->d_f[1], n, (size_t)Q * N, s));
    LBG_CK(ctx, upload_f64(ctx->d_rho, density, (size_t)N, s));
    const double *j[3] = {jx, jy, jz};
    for (int d = 0; d < 3; ++d) LBG_CK(ctx, upload_f64(ctx->d_j[d], j[d], (size_t)N, s));
    FlowArgs64 a;
    fill_args64(ctx, a);
    a.parity = 1;
    a.force_collide = ctx->force_last_collide;
    LBG_CK(ctx, launch_collide_f64(a, force_mask(ctx->p.f_ext), false, s));
    ctx->cur = 0;
    ctx->prev_kind = PREV_RAW;
    ctx->prev_force_moment = ctx->force_last_collide;
    ctx->moments_valid = true;
    return lbgpu_sync(ctx);
}

int lbgpu_flow_get(lbgpu_ctx *ctx, double *n, double *density, double *jx, double *jy, double *jz)
{
    if (!ctx) return LBGPU_ERR_INVALID;
    if (ctx->p.precision == LBGPU_FP32_DEV) return f32_flow_get(ctx, n, density, jx, jy, jz);
    if (ctx->prev_kind == PREV_NONE)
        return ctx_fail(ctx, LBGPU_ERR_INVALID, "lbgpu_flow_get: no flow state (call lbgpu_flow_init)");
    const long long N = ctx->N;
    cudaStream_t s = ctx->stream;
    const int prev = 1 - ctx->cur;
    double *nsrc = ctx->d_f[prev];
    double *tmp = nullptr;
    if (ctx->prev_kind == PREV_POST) {
        // populations after streaming = pull of the post-collision buffer; moments with it
        FlowArgs64 a;
        fill_args64(ctx, a);
        a.parity = prev;
        a.force_moment = ctx->prev_force_moment;
        if (n) {
            LBG_CK(ctx, cudaMallocAsync(&tmp, sizeof(double) * Q * N, s));
            a.nout = tmp;
            nsrc = tmp;
        }
        a.err_bits = nullptr;
        a.status = nullptr;
        // with a per-node force field (compensate_f_ext) the moments take the field once the
        // force is on, as every moment evaluation of the equilibration loop does
        const bool field = ctx->d_F[0] != nullptr && ctx->prev_force_moment;
        a.Fx = ctx->d_F[0];
        a.Fy = ctx->d_F[1];
        a.Fz = ctx->d_F[2];
        LBG_CK(ctx, launch_finalize_f64(a, field, s));
    }
    if (n) LBG_CK(ctx, cudaMemcpyAsync(n, nsrc, sizeof(double) * Q * N, cudaMemcpyDeviceToHost, s));
    if (density) LBG_CK(ctx, cudaMemcpyAsync(density, ctx->d_rho, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
    double *j[3] = {jx, jy, jz};
    for (int d = 0; d < 3; ++d)
        if (j[d]) LBG_CK(ctx, cudaMemcpyAsync(j[d], ctx->d_j[d], sizeof(double) * N, cudaMemcpyDeviceToHost, s));
    if (tmp) LBG_CK(ctx, cudaFreeAsync(tmp, s));
    return lbgpu_sync(ctx);
}

int lbgpu_collide(lbgpu_ctx *ctx, double *n, const double *density, const double *jx,
                  const double *jy, const double *jz, const double *f_ext_x,
                  const double *f_ext_y, const double *f_ext_z)
{
    if (!ctx || !n || !density || !jx || !jy || !jz || !f_ext_x || !f_ext_y || !f_ext_z)
        return LBGPU_ERR_INVALID;
    int rc = need_fp64(ctx, "lbgpu_collide");
    if (rc) return rc;
    OpBuffers *ob = op_buffers(ctx, rc);
    if (!ob) return rc;
    const long long N = ctx->N;
    cudaStream_t s = ctx->stream;
    LBG_CK(ctx, cudaMemcpyAsync(ob->n[0], n, sizeof(double) * Q * N, cudaMemcpyHostToDevice, s));
    const double *in[7] = {density, jx, jy, jz, f_ext_x, f_ext_y, f_ext_z};
    double *dv[7] = {ob->m[0], ob->m[1], ob->m[2], ob->m[3], ob->F[0], ob->F[1], ob->F[2]};
    for (int q = 0; q < 7; ++q)
        LBG_CK(ctx, cudaMemcpyAsync(dv[q], in[q], sizeof(double) * N, cudaMemcpyHostToDevice, s));
    FlowArgs64 a;
    fill_args64(ctx, a);
    a.f0 = ob->n[0];
    a.f1 = ob->n[1];
    a.rho = ob->m[0];
    a.jx = ob->m[1];
    a.jy = ob->m[2];
    a.jz = ob->m[3];
    a.Fx = ob->F[0];
    a.Fy = ob->F[1];
    a.Fz = ob->F[2];
    a.parity = 0;
    a.force_collide = 1;
    LBG_CK(ctx, launch_collide_f64(a, 7, true, s));
    LBG_CK(ctx, cudaMemcpyAsync(n, ob->n[1], sizeof(double) * Q * N, cudaMemcpyDeviceToHost, s));
    return lbgpu_sync(ctx);
}

int lbgpu_bounce_back_stream(lbgpu_ctx *ctx, double *n)
{
    if (!ctx || !n) return LBGPU_ERR_INVALID;
    int rc = need_fp64(ctx, "lbgpu_bounce_back_stream");
    if (rc) return rc;
    OpBuffers *ob = op_buffers(ctx, rc);
    if (!ob) return rc;
    const long long N = ctx->N;
    cudaStream_t s = ctx->stream;
    LBG_CK(ctx, cudaMemcpyAsync(ob->n[0], n, sizeof(double) * Q * N, cudaMemcpyHostToDevice, s));
    FlowArgs64 a;
    fill_args64(ctx, a);
    a.f0 = ob->n[0];
    a.f1 = ob->n[1];
    a.parity = 0;
    a.nout = ob->n[1];
    LBG_CK(ctx, launch_stream_f64(a, s));
    LBG_CK(ctx, cudaMemcpyAsync(n, ob->n[1], sizeof(double) * Q * N, cudaMemcpyDeviceToHost, s));
    return lbgpu_sync(ctx);
}

int lbgpu_moments(lbgpu_ctx *ctx, const double *n, const double *f_ext_x, const double *f_ext_y,
                  const double *f_ext_z, double *density, double *jx, double *jy, double *jz,
                  double *l2err)
{
    if (!ctx || !n || !f_ext_x || !f_ext_y || !f_ext_z || !density || !jx || !jy || !jz)
        return LBGPU_ERR_INVALID;
    int rc = need_fp64(ctx, "lbgpu_moments");
    if (rc) return rc;
    OpBuffers *ob = op_buffers(ctx, rc);
    if (!ob) return rc;
    const long long N = ctx->N;
    cudaStream_t s = ctx->stream;
    LBG_CK(ctx, cudaMemcpyAsync(ob->n[0], n, sizeof(double) * Q * N, cudaMemcpyHostToDevice, s));
    const double *in[6] = {jx, jy, jz, f_ext_x, f_ext_y, f_ext_z};
    double *dv[6] = {ob->m[1], ob->m[2], ob->m[3], ob->F[0], ob->F[1], ob->F[2]};
    for (int q = 0; q < 6; ++q)
        LBG_CK(ctx, cudaMemcpyAsync(dv[q], in[q], sizeof(double) * N, cudaMemcpyHostToDevice, s));
    if ((rc = reset_scratch(ctx))) return rc;
    FlowArgs64 a;
    fill_args64(ctx, a);
    a.f0 = ob->n[0];
    a.f1 = ob->n[1];
    a.parity = 0;
    a.rho = ob->m[0];
    a.jx = ob->m[1];
    a.jy = ob->m[2];
    a.jz = ob->m[3];
    a.Fx = ob->F[0];
    a.Fy = ob->F[1];
    a.Fz = ob->F[2];
    LBG_CK(ctx, launch_moments_f64(a, true, s));
    double *out[4] = {density, jx, jy, jz};
    for (int q = 0; q < 4; ++q)
        LBG_CK(ctx, cudaMemcpyAsync(out[q], ob->m[q], sizeof(double) * N, cudaMemcpyDeviceToHost, s));
    Scratch sc;
    if ((rc = read_scratch(ctx, sc))) return rc;
    if (l2err) std::memcpy(l2err, &sc.err_bits, sizeof(double));
    return moments_status(ctx, sc.status);
}

int lbgpu_equilibration(lbgpu_ctx *ctx, int max_steps, double *l2err_hist, int hist_cap,
                        int *steps_out)
{
    TraceRange trace_("lbgpu_equilibration");
    if (!ctx) return LBGPU_ERR_INVALID;
    if (ctx->prev_kind == PREV_NONE)
        return ctx_fail(ctx, LBGPU_ERR_INVALID, "lbgpu_equilibration: call lbgpu_flow_init first");
    if (hist_cap < 0 || (hist_cap > 0 && !l2err_hist)) return LBGPU_ERR_INVALID;
    if (ctx->p.precision == LBGPU_FP32_DEV) {
        if (ctx->d_F[0])
            return ctx_fail(ctx, LBGPU_ERR_UNSUPPORTED,
                            "lbgpu_equilibration: a per-node force field needs an FP64 context");
        return f32_equilibration(ctx, max_steps, l2err_hist, hist_cap, steps_out);
    }
    cudaStream_t s = ctx->stream;
    double *d_hist = nullptr;
    if (hist_cap > 0) {
        LBG_CK(ctx, cudaMallocAsync(&d_hist, sizeof(double) * hist_cap, s));
        LBG_CK(ctx, cudaMemsetAsync(d_hist, 0, sizeof(double) * hist_cap, s));
    }
    FlowCtl c;
    std::memset(&c, 0, sizeof(c));
    c.t = 1;
    c.parity = ctx->cur;
    c.force_moment = ctx->force_last_collide;
    c.force_collide = 0;
    c.max_steps = max_steps;
    c.target_error = ctx->p.target_error;
    c.hist_cap = hist_cap;
    LBG_CK(ctx, cudaMemcpyAsync(ctx->d_ctl, &c, sizeof(c), cudaMemcpyHostToDevice, s));
    FlowArgs64 a;
    fill_args64(ctx, a);
    a.ctl = ctx->d_ctl;
    a.hist = d_hist;
    const int fmask = force_mask(ctx->p.f_ext);
    const bool field = ctx->d_F[0] != nullptr;  // compensate_f_ext: a per-node force field
    a.Fx = ctx->d_F[0];
    a.Fy = ctx->d_F[1];
    a.Fz = ctx->d_F[2];
    // one CUDA graph of G launches; the control block makes launches after the exit no-ops
    const long long N = ctx->N;
    int G = (int)std::min<long long>(512, std::max<long long>(8, (1LL << 24) / std::max<long long>(N, 1)));
    if (max_steps > 0) G = std::min(G, max_steps + 8);
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    LBG_CK(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int g = 0; g < G; ++g) {
        cudaError_t e = launch_flow_step_f64(a, fmask, field, true, true, 0, s);
        if (e != cudaSuccess) {
            cudaStreamEndCapture(s, &graph);
            return ctx_cuda(ctx, e, "capture flow step");
        }
    }
    LBG_CK(ctx, cudaStreamEndCapture(s, &graph));
    LBG_CK(ctx, cudaGraphInstantiate(&exec, graph, 0));
    cudaGraphDestroy(graph);
    FlowCtl h;
    int rc = LBGPU_OK;
    for (;;) {
        cudaError_t e = cudaGraphLaunch(exec, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&h, ctx->d_ctl, sizeof(h), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            rc = ctx_cuda(ctx, e, "lbgpu_equilibration");
            break;
        }
        if (h.done) break;
    }
    cudaGraphExecDestroy(exec);
    if (rc) return rc;
    ctx->cur = h.parity;
    ctx->prev_kind = PREV_POST;
    ctx->prev_force_moment = h.exit_force_moment;
    ctx->force_last_collide = h.force_collide;
    ctx->moments_valid = false;
    if (steps_out) *steps_out = h.exit_step;
    if (d_hist) {
        LBG_CK(ctx, cudaMemcpyAsync(l2err_hist, d_hist, sizeof(double) * hist_cap, cudaMemcpyDeviceToHost, s));
        LBG_CK(ctx, cudaFreeAsync(d_hist, s));
    }
    LBG_CK(ctx, cudaStreamSynchronize(s));
    if (h.status & LBGPU_ERR_NEGATIVE_POPULATION)
        return ctx_fail(ctx, LBGPU_ERR_NEGATIVE_POPULATION,
                        "In equilibration, the population n(x,y,z,vel) < 0");
    if (h.status & LBGPU_ERR_NONFINITE)
        return ctx_fail(ctx, LBGPU_ERR_NONFINITE, "equilibration: non-finite population");
    if (h.status & LBGPU_ERR_STEP_CAP)
        return ctx_fail(ctx, LBGPU_ERR_STEP_CAP,
                        "equilibration: step cap reached before the second convergence");
    return LBGPU_OK;
}

int lbgpu_flow_steps(lbgpu_ctx *ctx, int nsteps, int force_on)
{
    TraceRange trace_("lbgpu_flow_steps");
    if (!ctx || nsteps < 0) return LBGPU_ERR_INVALID;
    if (ctx->prev_kind == PREV_NONE)
        return ctx_fail(ctx, LBGPU_ERR_INVALID, "lbgpu_flow_steps: call lbgpu_flow_init first");
    if (ctx->p.precision == LBGPU_FP32_DEV) return f32_flow_steps(ctx, nsteps, force_on, nullptr);
    FlowArgs64 a;
    fill_args64(ctx, a);
    const int fmask = force_mask(ctx->p.f_ext);
    for (int t = 0; t < nsteps; ++t) {
        a.parity = ctx->cur;
        a.force_moment = ctx->force_last_collide;
        a.force_collide = force_on ? 1 : 0;
        LBG_CK(ctx, launch_flow_step_f64(a, fmask, false, false, false, 0, ctx->stream));
        ctx->prev_force_moment = ctx->force_last_collide;
        ctx->force_last_collide = a.force_collide;
        ctx->cur ^= 1;
        ctx->prev_kind = PREV_POST;
        ctx->moments_valid = false;
    }
    return LBGPU_OK;
}

int lbgpu_time_flow_steps(lbgpu_ctx *ctx, int nsteps, int force_on, float *ms)
{
    if (!ctx || nsteps < 0 || !ms) return LBGPU_ERR_INVALID;
    if (ctx->prev_kind == PREV_NONE)
        return ctx_fail(ctx, LBGPU_ERR_INVALID, "lbgpu_time_flow_steps: call lbgpu_flow_init first");
    if (ctx->p.precision == LBGPU_FP32_DEV) return f32_flow_steps(ctx, nsteps, force_on, ms);
    int rc;
    force_on = force_on ? 1 : 0;
    if (ctx->force_last_collide != force_on) {  // settle the phase outside the timed region
        if ((rc = lbgpu_flow_steps(ctx, 1, force_on))) return rc;
    }
    cudaStream_t s = ctx->stream;
    // a graph of two steps (buffer cur -> other -> cur) replayed nsteps/2 times
    if (!ctx->graph_fixed[force_on] || ctx->graph_fixed_parity[force_on] != ctx->cur) {
        if (ctx->graph_fixed[force_on]) cudaGraphExecDestroy(ctx->graph_fixed[force_on]);
        FlowArgs64 a;
        fill_args64(ctx, a);
        const int fmask = force_mask(ctx->p.f_ext);
        cudaGraph_t g;
        LBG_CK(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < 2; ++k) {
            a.parity = ctx->cur ^ k;
            a.force_moment = force_on;
            a.force_collide = force_on;
            cudaError_t e = launch_flow_step_f64(a, fmask, false, false, false, 0, s);
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
        if ((rc = lbgpu_flow_steps(ctx, 1, force_on))) return rc;
    } else if (nsteps > 0) {
        ctx->prev_force_moment = force_on;
        ctx->prev_kind = PREV_POST;
        ctx->moments_valid = false;
    }
    LBG_CK(ctx, cudaEventRecord(ctx->ev1, s));
    LBG_CK(ctx, cudaEventSynchronize(ctx->ev1));
    LBG_CK(ctx, cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1));
    return LBGPU_OK;
}

}  // extern "C"
