// profiles.cu -- the reference's 1D observables reduced on the device (equilibration.f90:154-176,
// 499-516): per plane normal to an axis, the mass flux SUM(jx), SUM(jy), SUM(jz) and the mean
// density SUM(density) / MAX(COUNT(density > epsilon(1._dp)), 1).  Each plane is summed by one
// thread with a single accumulator in array element order (first remaining index fastest), the
// order of the Fortran SUM intrinsic, so the profiles are bit-identical to the reference's on the
// same state; only O(lx + ly + lz) numbers leave the device.
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "ctx.h"
#include "lbgpu.h"

namespace lbg {
namespace {

__global__ void k_profiles(const double *__restrict__ rho, const double *__restrict__ jx,
                           const double *__restrict__ jy, const double *__restrict__ jz, int lx,
                           int ly, int lz, int axis, double *flux, double *dens)
{
    const int n[3] = {lx, ly, lz};
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n[axis]) return;
    const int a = axis == 0 ? 1 : 0, b = axis == 2 ? 1 : 2;  // remaining axes, a fastest
    const long long stride[3] = {1, lx, (long long)lx * ly};
    const double eps = 2.220446049250313e-16;                 // EPSILON(1._dp)
    double sx = 0.0, sy = 0.0, sz = 0.0, sd = 0.0;
    long long cnt = 0;
    for (int q = 0; q < n[b]; ++q)
        for (int p = 0; p < n[a]; ++p) {
            const long long r = k * stride[axis] + p * stride[a] + q * stride[b];
            sx = sx + jx[r];
            sy = sy + jy[r];
            sz = sz + jz[r];
            const double d = rho[r];
            sd = sd + d;
            cnt += d > eps;
        }
    flux[3 * k] = sx;
    flux[3 * k + 1] = sy;
    flux[3 * k + 2] = sz;
    dens[k] = sd / (double)(cnt > 0 ? cnt : 1);
}

}  // namespace
}  // namespace lbg

using namespace lbg;

extern "C" int lbgpu_profiles(lbgpu_ctx *ctx, int axis, double *flux, double *mean_density)
{
    if (!ctx || axis < 0 || axis > 2 || !flux || !mean_density)
        return ctx_fail(ctx, LBGPU_ERR_INVALID, "lbgpu_profiles: axis must be 0, 1 or 2 and outputs non-null");
    int rc = lbgpu_flow_get(ctx, nullptr, nullptr, nullptr, nullptr, nullptr);  // moments on the device
    if (rc) return rc;
    const int L = axis == 0 ? ctx->p.lx : axis == 1 ? ctx->p.ly : ctx->p.lz;
    cudaStream_t s = ctx->stream;
    double *d = nullptr;
    LBG_CK(ctx, cudaMallocAsync(&d, sizeof(double) * 4 * (size_t)L, s));
    k_profiles<<<(L + 63) / 64, 64, 0, s>>>(ctx->d_rho, ctx->d_j[0], ctx->d_j[1], ctx->d_j[2], ctx->p.lx,
                                             ctx->p.ly, ctx->p.lz, axis, d, d + 3 * (size_t)L);
    LBG_CK(ctx, cudaGetLastError());
    LBG_CK(ctx, cudaMemcpyAsync(flux, d, sizeof(double) * 3 * (size_t)L, cudaMemcpyDeviceToHost, s));
    LBG_CK(ctx, cudaMemcpyAsync(mean_density, d + 3 * (size_t)L, sizeof(double) * L, cudaMemcpyDeviceToHost, s));
    LBG_CK(ctx, cudaFreeAsync(d, s));
    LBG_CK(ctx, cudaStreamSynchronize(s));
    return LBGPU_OK;
}
