// api.cu -- C ABI of liblbgpu: contexts, host<->device transfers, the reference loop driver.
//
// Host arrays are Fortran column-major (x fastest); the device uses the same node order and
// velocity-major structure-of-arrays for populations, so FP64 transfers are plain copies.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "ctx.h"
#include "flow.h"
#include "lbgpu.h"

using namespace lbg;

namespace {
thread_local std::string g_last_error;  // failures before a context exists

int fail_global(int code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}
}  // namespace

namespace lbg {

int ctx_fail(lbgpu_ctx *ctx, int code, const std::string &msg)
{
    if (ctx) ctx->last_error = msg;
    else g_last_error = msg;
    return code;
}

int ctx_cuda(lbgpu_ctx *ctx, cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return LBGPU_OK;
    return ctx_fail(ctx, LBGPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int moments_status(lbgpu_ctx *ctx, unsigned raised)
{
    const int bad = (int)(raised & (LBGPU_ERR_NEGATIVE_POPULATION | LBGPU_ERR_NONFINITE));
    if (!bad) return LBGPU_OK;
    if (bad & LBGPU_ERR_NEGATIVE_POPULATION)
        return ctx_fail(ctx, bad, "In equilibration, the population n(x,y,z,vel) < 0");
    return ctx_fail(ctx, bad, "moments: a population is not finite (NaN or Inf)");
}

// module_lbmodel.f90:127-147 and module_collision.f90:28,99-103, evaluated as the reference
// does (every operation separately rounded).
LbConst64 make_const64(double tau)
{
    LbConst64 K{};
    volatile double csq = 1.0 / 3.0;  // volatile: keep each operation separately rounded
    const double a00 = 1.0 / 3.0, a01 = 1.0 / 18.0, a02 = 1.0 / 36.0;
    const double csq2 = csq * csq;
    const double two_csq2 = 2 * csq2;
    K.a0[0] = a00;
    K.a0[1] = a01;
    K.a0[2] = a02;
    K.a1[0] = a00 / csq;
    K.a1[1] = a01 / csq;
    K.a1[2] = a02 / csq;
    K.a2[0] = a00 / two_csq2;
    K.a2[1] = a01 / two_csq2;
    K.a2[2] = a02 / two_csq2;
    for (int w = 0; w < 3; ++w) K.two_a2[w] = 2.0 * K.a2[w];
    const double one = 1.0, zero = 0.0;
    K.k1 = one * one - csq;
    K.k0 = zero * zero - csq;
    const volatile double t = tau;
    K.c1 = 1.0 - 1.0 / t;
    K.c2 = 1.0 / t;
    K.c3 = 1.0 - 1.0 / (2.0 * t);
    for (int w = 0; w < 3; ++w) {
        K.c2a0[w] = K.c2 * K.a0[w];
        K.c2a1[w] = K.c2 * K.a1[w];
        K.c2a2[w] = K.c2 * K.a2[w];
        K.c2a2cs2[w] = K.c2a2[w] * csq;
        K.c3a1[w] = K.c3 * K.a1[w];
    }
    return K;
}

void fill_args64(lbgpu_ctx *ctx, FlowArgs64 &a)
{
    std::memset(&a, 0, sizeof(a));
    a.mask = ctx->d_mask;
    a.f0 = ctx->d_f[0];
    a.f1 = ctx->d_f[1];
    a.jx = ctx->d_j[0];
    a.jy = ctx->d_j[1];
    a.jz = ctx->d_j[2];
    a.rho = ctx->d_rho;
    a.N = ctx->N;
    a.fidx = ctx->d_fidx;
    a.Nf = ctx->d_fidx ? (long long)ctx->counts[0] : 0;
    a.lx = ctx->p.lx;
    a.ly = ctx->p.ly;
    a.lz = ctx->p.lz;
    a.K = ctx->K64;
    for (int d = 0; d < 3; ++d) a.F[d] = ctx->p.f_ext[d];
    // c_l . f_ext in the order of module_collision.f90:103 (cx*fx + cy*fy) + cz*fz
    for (int l = 0; l < Q; ++l) {
        const Vel c = vel(l);
        volatile double s = (double)c.x * a.F[0];
        s = s + (double)c.y * a.F[1];
        s = s + (double)c.z * a.F[2];
        a.cf[l] = s;
    }
    // LBGPU_FP64_FUSED: per pair of opposite velocities, c3 a1 (c.F) and c3 2 a2 (c.F)
    a.fused = ctx->p.precision == LBGPU_FP64_FUSED;
    for (int p = 0; p < 9; ++p) {
        const int l = pair_l(p), w = wclass(l);
        a.kF[p] = ctx->K64.c3a1[w] * a.cf[l];
        a.kT[p] = ctx->K64.c3 * ctx->K64.two_a2[w] * a.cf[l];
    }
    a.err_bits = &ctx->d_scratch->err_bits;
    a.status = &ctx->d_scratch->status;
}

int force_mask(const double f[3])
{
    int m = (f[0] != 0.0 ? 1 : 0) | (f[1] != 0.0 ? 2 : 0) | (f[2] != 0.0 ? 4 : 0);
    if (m == 3 || m == 5 || m == 6) m = 7;
    return m;
}

}  // namespace lbg

namespace lbg {
int geometry_build(int label, int lx, int ly, int lz, const double *params, int8_t *d_nature,
                   long long *nfluid, cudaStream_t s, std::string &err);
int geometry_check(int label, int lx, int ly, int lz, const double *params, std::string &err);
}  // namespace lbg

namespace lbg {
// Host ranges page-locked through lbgpu_host_register: [begin, end).
std::mutex g_pinned_mutex;
std::vector<std::pair<uintptr_t, uintptr_t>> g_pinned;

const void *pinned_device_view(const void *p, size_t bytes)
{
    const uintptr_t b = reinterpret_cast<uintptr_t>(p), e = b + bytes;
    bool inside = false;
    {
        std::lock_guard<std::mutex> lock(g_pinned_mutex);
        for (const auto &r : g_pinned)
            if (r.first <= b && e <= r.second) {
                inside = true;
                break;
            }
    }
    void *d = nullptr;
    if (!inside || cudaHostGetDevicePointer(&d, const_cast<void *>(p), 0) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return d;
}
}  // namespace lbg

extern "C" {

void lbgpu_default_params(lbgpu_params *p, int lx, int ly, int lz)
{
    std::memset(p, 0, sizeof(*p));
    p->lx = lx;
    p->ly = ly;
    p->lz = lz;
    p->precision = LBGPU_FP64;
    p->relaxation_time = 1.0;
    p->target_error = 1e-10;
    p->rho0 = 1.0;
    p->device = 0;
}

int lbgpu_last_error(const lbgpu_ctx *ctx, char *buf, size_t len)
{
    if (!buf || !len) return LBGPU_ERR_INVALID;
    const std::string &m = ctx ? ctx->last_error : g_last_error;
    std::snprintf(buf, len, "%s", m.c_str());
    return LBGPU_OK;
}

int lbgpu_create(const lbgpu_params *p, const int8_t *nature, lbgpu_ctx **out)
{
    if (!p || !nature || !out) return fail_global(LBGPU_ERR_INVALID, "lbgpu_create: null argument");
    *out = nullptr;
    if (p->lx <= 0 || p->ly <= 0 || p->lz <= 0)
        return fail_global(LBGPU_ERR_INVALID, "lbgpu_create: lx, ly, lz must be > 0");
    if (!(p->relaxation_time >= 0.5))
        return fail_global(LBGPU_ERR_INVALID, "relaxation_time must be > 0.5");
    if (p->precision != LBGPU_FP64 && p->precision != LBGPU_FP32_DEV && p->precision != LBGPU_FP64_FUSED)
        return fail_global(LBGPU_ERR_INVALID, "lbgpu_create: unknown precision");
    const long long N = (long long)p->lx * p->ly * p->lz;
    if (N >= (1LL << 31)) return fail_global(LBGPU_ERR_INVALID, "lbgpu_create: more than 2^31 nodes");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail_global(LBGPU_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (p->device < 0 || p->device >= ndev) return fail_global(LBGPU_ERR_INVALID, "bad device ordinal");
    for (long long i = 0; i < N; ++i)
        if (nature[i] != 0 && nature[i] != 1)
            return fail_global(LBGPU_ERR_INVALID, "nature must be 0 (fluid) or 1 (solid)");

    lbgpu_ctx *ctx = new lbgpu_ctx();
    ctx->p = *p;
    ctx->N = N;
    ctx->K64 = make_const64(p->relaxation_time);
    int rc = ctx_init_device(ctx, nature);
    if (rc) {
        g_last_error = ctx->last_error;
        lbgpu_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return LBGPU_OK;
}

int lbgpu_geometry(int device, int label, int lx, int ly, int lz, const double *params, int8_t *nature)
{
    if (!nature) return fail_global(LBGPU_ERR_INVALID, "lbgpu_geometry: null nature");
    if (lx <= 0 || ly <= 0 || lz <= 0)
        return fail_global(LBGPU_ERR_INVALID, "lbgpu_geometry: lx, ly, lz must be > 0");
    const long long N = (long long)lx * ly * lz;
    if (N >= (1LL << 31)) return fail_global(LBGPU_ERR_INVALID, "lbgpu_geometry: more than 2^31 nodes");
    std::string err;
    if (geometry_check(label, lx, ly, lz, params, err)) return fail_global(LBGPU_ERR_INVALID, err);
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail_global(LBGPU_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (device < 0 || device >= ndev) return fail_global(LBGPU_ERR_INVALID, "bad device ordinal");
    if ((e = cudaSetDevice(device)) != cudaSuccess)
        return fail_global(LBGPU_ERR_CUDA, std::string("lbgpu_geometry: ") + cudaGetErrorString(e));
    cudaStream_t s = nullptr;
    int8_t *d = nullptr;
    if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaMallocAsync(&d, (size_t)N, s)) != cudaSuccess) {
        if (s) cudaStreamDestroy(s);
        return fail_global(LBGPU_ERR_CUDA, std::string("lbgpu_geometry: ") + cudaGetErrorString(e));
    }
    long long nfluid = 0;
    int rc = geometry_build(label, lx, ly, lz, params, d, &nfluid, s, err);
    if (rc == LBGPU_OK) {
        e = cudaMemcpyAsync(nature, d, (size_t)N, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            rc = LBGPU_ERR_CUDA;
            err = std::string("lbgpu_geometry: ") + cudaGetErrorString(e);
        }
    }
    cudaFreeAsync(d, s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return rc ? fail_global(rc, err) : LBGPU_OK;
}

int lbgpu_create_label(const lbgpu_params *p, int label, const double *params, lbgpu_ctx **out)
{
    if (!p || !out) return fail_global(LBGPU_ERR_INVALID, "lbgpu_create_label: null argument");
    *out = nullptr;
    if (p->lx <= 0 || p->ly <= 0 || p->lz <= 0)
        return fail_global(LBGPU_ERR_INVALID, "lbgpu_create_label: lx, ly, lz must be > 0");
    const long long N = (long long)p->lx * p->ly * p->lz;
    if (N >= (1LL << 31)) return fail_global(LBGPU_ERR_INVALID, "lbgpu_create_label: more than 2^31 nodes");
    // the compact layout of FP32 boxes is planned on the host, so the box comes back once
    std::vector<int8_t> nature((size_t)N);
    const int rc = lbgpu_geometry(p->device, label, p->lx, p->ly, p->lz, params, nature.data());
    if (rc) return rc;
    return lbgpu_create(p, nature.data(), out);
}

void lbgpu_destroy(lbgpu_ctx *ctx)
{
    if (!ctx) return;
    ctx_release_device(ctx);
    delete ctx;
}

int lbgpu_interfacial(lbgpu_ctx *ctx, uint8_t *out)
{
    if (!ctx || !out) return LBGPU_ERR_INVALID;
    std::vector<uint32_t> m(ctx->N);
    int rc = ctx_cuda(ctx, cudaMemcpy(m.data(), ctx->d_mask, ctx->N * sizeof(uint32_t),
                                      cudaMemcpyDeviceToHost), "lbgpu_interfacial");
    if (rc) return rc;
    for (long long i = 0; i < ctx->N; ++i) out[i] = (m[i] & INTERFACIAL_BIT) ? 1 : 0;
    return LBGPU_OK;
}

int lbgpu_node_counts(lbgpu_ctx *ctx, long long counts[4])
{
    if (!ctx || !counts) return LBGPU_ERR_INVALID;
    for (int q = 0; q < 4; ++q) counts[q] = (long long)ctx->counts[q];
    return LBGPU_OK;
}

int lbgpu_host_register(void *ptr, size_t bytes)
{
    if (!ptr || !bytes) return fail_global(LBGPU_ERR_INVALID, "lbgpu_host_register: empty range");
    cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
    if (e != cudaSuccess) return fail_global(LBGPU_ERR_CUDA, std::string("cudaHostRegister: ") + cudaGetErrorString(e));
    std::lock_guard<std::mutex> lock(lbg::g_pinned_mutex);
    lbg::g_pinned.emplace_back(reinterpret_cast<uintptr_t>(ptr), reinterpret_cast<uintptr_t>(ptr) + bytes);
    return LBGPU_OK;
}

int lbgpu_host_unregister(void *ptr)
{
    if (!ptr) return LBGPU_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lock(lbg::g_pinned_mutex);
        auto &v = lbg::g_pinned;
        for (size_t k = 0; k < v.size(); ++k)
            if (v[k].first == reinterpret_cast<uintptr_t>(ptr)) {
                v.erase(v.begin() + (long)k);
                break;
            }
    }
    cudaError_t e = cudaHostUnregister(ptr);
    if (e != cudaSuccess) return fail_global(LBGPU_ERR_CUDA, std::string("cudaHostUnregister: ") + cudaGetErrorString(e));
    return LBGPU_OK;
}

int lbgpu_sync(lbgpu_ctx *ctx)
{
    if (!ctx) return LBGPU_ERR_INVALID;
    return ctx_cuda(ctx, cudaStreamSynchronize(ctx->stream), "lbgpu_sync");
}

}  // extern "C"
