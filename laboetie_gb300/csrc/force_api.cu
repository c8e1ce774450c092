// force_api.cu -- the per-node force field of compensate_f_ext (equilibration.f90:388-487).
//
// With compensate_f_ext the reference applies, from the first convergence on, the force f_ext
// spread over a spherical "particle" of odd diameter around a node, compensated by a uniform
// background force in a solid-free box (geometryLabel -1) so that the net force vanishes.  The
// field depends only on the geometry and lb.in, so it is built once on the host (here, for hosts
// that do not build it themselves) and kept on the device; the step kernels then read it per
// node instead of the uniform f_ext.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "ctx.h"
#include "lbgpu.h"

namespace {

// gfortran's NORM2 (scaled sum of squares, scale starting at 1)
double norm2_f(const double *v, int m)
{
    double result = 0.0, scale = 1.0;
    for (int i = 0; i < m; ++i) {
        if (v[i] != 0.0) {
            const double ax = std::fabs(v[i]);
            if (scale < ax) {
                const double val = scale / ax;
                result = 1.0 + result * val * val;
                scale = ax;
            } else {
                const double val = ax / scale;
                result += val * val;
            }
        }
    }
    return scale * std::sqrt(result);
}

}  // namespace

using namespace lbg;

extern "C" {

int lbgpu_compensated_force_field(lbgpu_ctx *ctx, int particle_diameter, const int particle_coords[3],
                                  int geometry_label, double *fx, double *fy, double *fz)
{
    if (!ctx || !fx || !fy || !fz) return LBGPU_ERR_INVALID;
    const int lx = ctx->p.lx, ly = ctx->p.ly, lz = ctx->p.lz;
    const long long N = ctx->N;
    const double *fl = ctx->p.f_ext;
    const int pd = particle_diameter;
    if (pd % 2 == 0) return ctx_fail(ctx, LBGPU_ERR_INVALID, "ERROR: l. 285 particle diameter must be odd");
    if (lx % 2 == 0 || ly % 2 == 0 || lz % 2 == 0)
        return ctx_fail(ctx, LBGPU_ERR_INVALID,
                        "when compensate_f_ext, there should be odd number of nodes in all directions");
    std::vector<int8_t> nat(N);
    LBG_CK(ctx, cudaMemcpy(nat.data(), ctx->d_nature, N, cudaMemcpyDeviceToHost));
    const int pdr = pd / 2;
    for (long long r = 0; r < N; ++r) fx[r] = fy[r] = fz[r] = 0.0;
    const int px = particle_coords && particle_coords[0] > 0 ? particle_coords[0] : lx / 2 + 1;
    const int py = particle_coords && particle_coords[1] > 0 ? particle_coords[1] : ly / 2 + 1;
    const int pz = particle_coords && particle_coords[2] > 0 ? particle_coords[2] : lz / 2 + 1;
    long long cnt = 0;
    bool err = false;
    for (int i = px - pdr; i <= px + pdr; ++i)
        for (int j = py - pdr; j <= py + pdr; ++j)
            for (int k = pz - pdr; k <= pz + pdr; ++k) {
                const double v[3] = {(double)(i - px), (double)(j - py), (double)(k - pz)};
                if (norm2_f(v, 3) > (double)pd / 2.0) continue;
                if (i < 1 || i > lx || j < 1 || j > ly || k < 1 || k > lz)
                    return ctx_fail(ctx, LBGPU_ERR_INVALID, "particle crosses the box boundary");
                const long long r = (i - 1) + (long long)lx * ((j - 1) + (long long)ly * (k - 1));
                if (nat[r] != 0) err = true;
                fx[r] = fl[0];
                fy[r] = fl[1];
                fz[r] = fl[2];
                cnt = cnt + 1;
            }
    if (err) return ctx_fail(ctx, LBGPU_ERR_INVALID, "ERROR: l306 of equilibration.f90. Dominika's particle at a solid node");
    const long long nf = (long long)ctx->counts[0];
    if (geometry_label == -1) {
        for (long long r = 0; r < N; ++r) {
            if (fx[r] == fl[0] && fy[r] == fl[1] && fz[r] == fl[2]) {
                fx[r] = -fl[0] / nf + fx[r] / cnt;
                fy[r] = -fl[1] / nf + fy[r] / cnt;
                fz[r] = -fl[2] / nf + fz[r] / cnt;
            } else {
                fx[r] = -fl[0] / nf;
                fy[r] = -fl[1] / nf;
                fz[r] = -fl[2] / nf;
            }
        }
        double sx = 0, sy = 0, sz = 0;
        for (long long r = 0; r < N; ++r) {
            sx += fx[r];
            sy += fy[r];
            sz += fz[r];
        }
        const double eps = 2.220446049250313e-16;
        if (std::fabs(sx / nf) > eps || std::fabs(sy / nf) > eps || std::fabs(sz / nf) > eps)
            return ctx_fail(ctx, LBGPU_ERR_INVALID, "The compensation is not well-implemented.");
    } else {
        for (long long r = 0; r < N; ++r) {
            if (fx[r] == fl[0] && fy[r] == fl[1] && fz[r] == fl[2]) {
                fx[r] = fx[r] / cnt;
                fy[r] = fy[r] / cnt;
                fz[r] = fz[r] / cnt;
            } else {
                fx[r] = 0.0;
                fy[r] = 0.0;
                fz[r] = 0.0;
            }
        }
    }
    for (long long r = 0; r < N; ++r)
        if (nat[r] != 0) fx[r] = fy[r] = fz[r] = 0.0;
    return LBGPU_OK;
}

int lbgpu_set_force_field(lbgpu_ctx *ctx, const double *fx, const double *fy, const double *fz)
{
    if (!ctx) return LBGPU_ERR_INVALID;
    if ((fx == nullptr) != (fy == nullptr) || (fy == nullptr) != (fz == nullptr))
        return ctx_fail(ctx, LBGPU_ERR_INVALID, "lbgpu_set_force_field: give all three components or none");
    if (ctx->p.precision == LBGPU_FP32_DEV)
        return ctx_fail(ctx, LBGPU_ERR_INVALID, "lbgpu_set_force_field: needs an FP64 context");
    if (!fx) {
        for (int d = 0; d < 3; ++d) {
            cudaFree(ctx->d_F[d]);
            ctx->d_F[d] = nullptr;
        }
        return LBGPU_OK;
    }
    const double *h[3] = {fx, fy, fz};
    for (int d = 0; d < 3; ++d) {
        if (!ctx->d_F[d]) LBG_CK(ctx, cudaMalloc((void **)&ctx->d_F[d], sizeof(double) * ctx->N));
        LBG_CK(ctx, cudaMemcpyAsync(ctx->d_F[d], h[d], sizeof(double) * ctx->N, cudaMemcpyHostToDevice, ctx->stream));
    }
    return lbgpu_sync(ctx);
}

}  // extern "C"
