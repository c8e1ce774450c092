// ek.cu -- the operators of the reference's coupled electrokinetic loop, one C-ABI call each
// (compiled with -fmad=false): electrostatic_pot.f90, comp_j.f90, smolu.f90, advect.f90.
//
// In the reference these subroutines are called only from src/trash/equilibration_*.f90, a time
// loop that no longer builds; each is still a self-contained update of module variables (phi,
// phi_tot, c_plus, c_minus, node%solventFlux, solute_force, the currents), which the library
// keeps in the context's charged-solute state (pnp.h) or takes as host arrays.
//
// Every node's result is formed in the reference's operation order, so the operators without an
// exponential (electrostatic_pot, comp_j, advect) are bit-identical to it; smolu's link factors
// use the device exp(), and its currents are sums over all links formed in a fixed order of their
// own (within 1e-12 of the reference's sequential sums).
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "ctx.h"
#include "lbgpu.h"
#include "pnp.h"
#include "reduce.cuh"
#include "trace.h"

namespace lbg {
namespace {

constexpr int EB = MP_BLOCK;

__device__ __forceinline__ void ek_coords(long long r, int lx, int ly, int &x, int &y, int &z)
{
    const unsigned nd = (unsigned)r;
    x = (int)(nd % (unsigned)lx);
    const unsigned yz = nd / (unsigned)lx;
    y = (int)(yz % (unsigned)ly);
    z = (int)(yz / (unsigned)ly);
}

// module_system.f90:99-112 (pbc) for a step of -1, 0 or +1
__device__ __forceinline__ int ek_wrap(int x, int d, int L)
{
    return d > 0 ? wrap_plus(x, L) : (d < 0 ? wrap_minus(x, L) : x);
}

// electrostatic_pot.f90:7-21: phi_tot = phi + sum(elec_slope * [i,j,k]) (1-based), one
// accumulator from 0 over x, y, z; or phi itself when elec_slope is all zero.
__global__ void __launch_bounds__(EB) k_ek_pot(const double *phi, double *phi_tot, long long N, int lx, int ly,
                                               double e0, double e1, double e2, int zero)
{
    const long long r = (long long)blockIdx.x * EB + threadIdx.x;
    if (r >= N) return;
    if (zero) {
        phi_tot[r] = phi[r];
        return;
    }
    int x, y, z;
    ek_coords(r, lx, ly, x, y, z);
    double s = 0.0;
    s = s + e0 * (double)(x + 1);
    s = s + e1 * (double)(y + 1);
    s = s + e2 * (double)(z + 1);
    phi_tot[r] = phi[r] + s;
}

// comp_j.f90:14-27: j = 0.5*(j + sum(n(i,j,k,:)*coo(d))), the sum from 0 over l = 1..19 with
// every product formed (n*0 included).
__global__ void __launch_bounds__(EB) k_comp_j(const double *n, double *jx, double *jy, double *jz, long long N)
{
    const long long r = (long long)blockIdx.x * EB + threadIdx.x;
    if (r >= N) return;
    double s[3] = {0.0, 0.0, 0.0};
    static_for<0, Q>([&](auto L) {
        constexpr int l = decltype(L)::value;
        constexpr Vel c = vel(l);
        const double f = n[(long long)l * N + r];
        s[0] = s[0] + f * (double)c.x;
        s[1] = s[1] + f * (double)c.y;
        s[2] = s[2] + f * (double)c.z;
    });
    jx[r] = 0.5 * (jx[r] + s[0]);
    jy[r] = 0.5 * (jy[r] + s[1]);
    jz[r] = 0.5 * (jz[r] + s[2]);
}

struct SmoluArgs {
    const uint32_t *mask;
    const double *phi_tot, *cp, *cm;
    double *fp, *fm, *sf;
    double *partial;     // 6 per block: el_curr x,y,z, ion_curr x,y,z
    long long N;
    int lx, ly, lz;
    double Dp, Dm, dit, kbt;
    double es[3], ls[3];
    double a1[3], delta[3];
};

// smolu.f90:27-115 at fluid node r: the site fluxes (sum over the fluid-fluid links in l order),
// the node's solute_force (accumulated onto its value), and this node's share of the currents.
__global__ void __launch_bounds__(EB) k_smolu(const SmoluArgs a)
{
    double t[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (long long r = (long long)blockIdx.x * EB + threadIdx.x; r < a.N; r += (long long)gridDim.x * EB) {
        const uint32_t m = a.mask[r];
        if (!(m & FLUID_BIT)) continue;
        int x, y, z;
        ek_coords(r, a.lx, a.ly, x, y, z);
        const double pr = a.phi_tot[r], cpr = a.cp[r], cmr = a.cm[r];
        double fp = 0.0, fm = 0.0;
        double f0 = a.sf[r], f1 = a.sf[r + a.N], f2 = a.sf[r + 2 * a.N];
        static_for<1, Q>([&](auto L) {
            constexpr int l = decltype(L)::value;
            constexpr Vel c = vel(l);
            constexpr int w = wclass(l);
            const int xp = ek_wrap(x, c.x, a.lx), yp = ek_wrap(y, c.y, a.ly), zp = ek_wrap(z, c.z, a.lz);
            const long long rp = xp + (long long)a.lx * (yp + (long long)a.ly * zp);
            const double cx = (double)c.x, cy = (double)c.y, cz = (double)c.z;
            const double a1 = a.a1[w];
            if (a.mask[rp] & FLUID_BIT) {
                double e = exp(a.phi_tot[rp] - pr);
                // smolu.f90:46-51: every matching case applies, in this order
                if (x == a.lx - 1 && xp == 0) e = e * exp(a.es[0] * (double)a.lx);
                if (y == a.ly - 1 && yp == 0) e = e * exp(a.es[1] * (double)a.ly);
                if (z == a.lz - 1 && zp == 0) e = e * exp(a.es[2] * (double)a.lz);
                if (x == 0 && xp == a.lx - 1) e = e * exp(-(a.es[0] * (double)a.lx));
                if (y == 0 && yp == a.ly - 1) e = e * exp(-(a.es[1] * (double)a.ly));
                if (z == 0 && zp == a.lz - 1) e = e * exp(-(a.es[2] * (double)a.lz));
                const double em = 1.0 / e;
                double sl = 0.0;
                sl = sl + a.ls[0] * cx;
                sl = sl + a.ls[1] * cy;
                sl = sl + a.ls[2] * cz;
                const double edl = exp(sl);
                const double emdl = 1.0 / edl;
                const double cpp = a.cp[rp], cmp = a.cm[rp];
                double flp = 0.5 * (1.0 + em * emdl) * (cpp * e * edl - cpr);
                double flm = 0.5 * (1.0 + e * emdl) * (cmp * em * edl - cmr);
                const double elc = flp * a.Dp - flm * a.Dm;
                const double ionc = flp * a.Dp + flm * a.Dm;
                const double fpl = 0.5 * (1.0 + em) * (cpp * e - cpr);
                const double fmi = 0.5 * (1.0 + e) * (cmp * em - cmr);
                double fmic = a.kbt * (fpl + fmi);
                fmic = fmic - a.kbt * (cpp - cpr + cmp - cmr);
                flp = flp * (a.Dp / a.delta[w]);
                flm = flm * (a.Dm / a.delta[w]);
                fp = fp + flp;
                fm = fm + flm;
                t[0] = t[0] + a1 * cx * elc / a.dit;
                t[1] = t[1] + a1 * cy * elc / a.dit;
                t[2] = t[2] + a1 * cz * elc / a.dit;
                t[3] = t[3] + a1 * cx * ionc / a.dit;
                t[4] = t[4] + a1 * cy * ionc / a.dit;
                t[5] = t[5] + a1 * cz * ionc / a.dit;
                f0 = f0 + a1 * cx * fmic / a.dit;
                f1 = f1 + a1 * cy * fmic / a.dit;
                f2 = f2 + a1 * cz * fmic / a.dit;
            } else {
                // smolu.f90:94-112: the force on the solid; no lncb_slope, no elec_slope term
                const double e = exp(a.phi_tot[rp] - pr);
                const double em = 1.0 / e;
                const double fpl = cpr * (1.0 - em);
                const double fmi = cmr * (1.0 - e);
                const double fmic = a.kbt * (fpl + fmi);
                f0 = f0 + a1 * cx * fmic / a.dit;
                f1 = f1 + a1 * cy * fmic / a.dit;
                f2 = f2 + a1 * cz * fmic / a.dit;
            }
        });
        a.fp[r] = fp;
        a.fm[r] = fm;
        a.sf[r] = f0;
        a.sf[r + a.N] = f1;
        a.sf[r + 2 * a.N] = f2;
    }
    // fixed-order block sums of the six currents (the last kernel adds the blocks in order)
    __shared__ double sh[6][EB / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int q = 0; q < 6; ++q) t[q] = warp_sum_fixed(t[q]);
    if (lane == 0)
        for (int q = 0; q < 6; ++q) sh[q][wid] = t[q];
    __syncthreads();
    if (wid == 0)
        for (int q = 0; q < 6; ++q) {
            double v = lane < EB / 32 ? sh[q][lane] : 0.0;
            v = warp_sum_fixed(v);
            if (lane == 0) a.partial[6 * blockIdx.x + q] = v;
        }
}

// smolu.f90:118-121 (c += flux on fluid nodes) and the sums of the site fluxes over the fluid
// nodes for the check of :137-141 (block partials 6*b + {0, 1}).
__global__ void __launch_bounds__(EB) k_smolu_update(const SmoluArgs a)
{
    double t[2] = {0.0, 0.0};
    for (long long r = (long long)blockIdx.x * EB + threadIdx.x; r < a.N; r += (long long)gridDim.x * EB) {
        if (!(a.mask[r] & FLUID_BIT)) continue;
        const double fp = a.fp[r], fm = a.fm[r];
        const_cast<double *>(a.cp)[r] = a.cp[r] + fp;
        const_cast<double *>(a.cm)[r] = a.cm[r] + fm;
        t[0] = t[0] + fp;
        t[1] = t[1] + fm;
    }
    __shared__ double sh[2][EB / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int q = 0; q < 2; ++q) t[q] = warp_sum_fixed(t[q]);
    if (lane == 0)
        for (int q = 0; q < 2; ++q) sh[q][wid] = t[q];
    __syncthreads();
    if (wid == 0)
        for (int q = 0; q < 2; ++q) {
            double v = lane < EB / 32 ? sh[q][lane] : 0.0;
            v = warp_sum_fixed(v);
            if (lane == 0) a.partial[6 * blockIdx.x + q] = v;
        }
}

// Sum of the first nq of 6 values per block over nb blocks, in block order, by one thread.
__global__ void k_sum6(const double *partial, unsigned nb, int nq, double *out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double t[6] = {0, 0, 0, 0, 0, 0};
    for (unsigned b = 0; b < nb; ++b)
        for (int q = 0; q < nq; ++q) t[q] = t[q] + partial[6 * b + q];
    for (int q = 0; q < nq; ++q) out[q] = t[q];
}

struct AdvectArgs {
    const int8_t *nature;
    const double *jx, *jy, *jz, *cp, *cm;
    double *fp, *fm;
    long long N;
    int lx, ly, lz;
};

// The distinct coordinates x - 1, x, x + 1 (periodic) in ascending order: the sources along one
// axis whose links can reach x.
__device__ __forceinline__ int ek_sources(int x, int L, int (&c)[3])
{
    int v[3] = {wrap_minus(x, L), x, wrap_plus(x, L)};
    // sort three values, then drop repeats
    if (v[0] > v[1]) { int t = v[0]; v[0] = v[1]; v[1] = t; }
    if (v[1] > v[2]) { int t = v[1]; v[1] = v[2]; v[2] = t; }
    if (v[0] > v[1]) { int t = v[0]; v[0] = v[1]; v[1] = t; }
    int n = 0;
    for (int i = 0; i < 3; ++i)
        if (n == 0 || v[i] != c[n - 1]) c[n++] = v[i];
    return n;
}

// advect.f90:52-96 gathered at the target r: the reference walks the sources s in loop order
// (i, then j, then k) and, for each of its 27 links d in (ix, iy, iz) order, subtracts the link's
// flux at s and adds it at s + d.  Node r's flux_site therefore receives, in that order, the
// subtractions of its own links (when s = r) and the additions of every link that ends at r;
// replaying exactly those events onto the value it held gives the reference's bits.
__global__ void __launch_bounds__(EB) k_advect(const AdvectArgs a)
{
    const long long r = (long long)blockIdx.x * EB + threadIdx.x;
    if (r >= a.N) return;
    const double eps = DBL_EPSILON;
    int x, y, z;
    ek_coords(r, a.lx, a.ly, x, y, z);
    int sx[3], sy[3], sz[3];
    const int nx = ek_sources(x, a.lx, sx), ny = ek_sources(y, a.ly, sy), nz = ek_sources(z, a.lz, sz);
    double fp = a.fp[r], fm = a.fm[r];
    const int8_t nat_r = a.nature[r];
    for (int ia = 0; ia < nx; ++ia)
        for (int ja = 0; ja < ny; ++ja)
            for (int ka = 0; ka < nz; ++ka) {
                const int i = sx[ia], j = sy[ja], k = sz[ka];
                const long long s = i + (long long)a.lx * (j + (long long)a.ly * k);
                const double cps = a.cp[s], cms = a.cm[s];
                if (fabs(cps) <= eps && fabs(cms) <= eps) continue;   // advect.f90:60
                const bool self = s == r;
                const double vx = a.jx[s], vy = a.jy[s], vz = a.jz[s];
                const int8_t nat_s = a.nature[s];
                for (int ix = -1; ix <= 1; ++ix)
                    for (int iy = -1; iy <= 1; ++iy)
                        for (int iz = -1; iz <= 1; ++iz) {
                            const int ti = ek_wrap(i, ix, a.lx), tj = ek_wrap(j, iy, a.ly),
                                      tk = ek_wrap(k, iz, a.lz);
                            const bool to_r = ti == x && tj == y && tk == z;
                            if (!self && !to_r) continue;
                            const long long t = ti + (long long)a.lx * (tj + (long long)a.ly * tk);
                            const double ax = vx * (double)ix, ay = vy * (double)iy, az = vz * (double)iz;
                            double flp = 0.0, flm = 0.0;
                            if (ax >= 0.0 && ay >= 0.0 && az >= 0.0 && nat_s == (to_r ? nat_r : a.nature[t])) {
                                const double fx = ix == 0 ? 1.0 - fabs(vx) : ax;
                                const double fy = iy == 0 ? 1.0 - fabs(vy) : ay;
                                const double fz = iz == 0 ? 1.0 - fabs(vz) : az;
                                flp = fx * fy * fz * cps;
                                flm = fx * fy * fz * cms;
                            }
                            if (self) {
                                fm = fm - flm;
                                fp = fp - flp;
                            }
                            if (to_r) {
                                fm = fm + flm;
                                fp = fp + flp;
                            }
                        }
            }
    a.fp[r] = fp;
    a.fm[r] = fm;
}

// advect.f90:99-103: c += flux_site on fluid nodes
__global__ void __launch_bounds__(EB) k_advect_update(const int8_t *nature, const double *fp, const double *fm,
                                                      double *cp, double *cm, long long N)
{
    const long long r = (long long)blockIdx.x * EB + threadIdx.x;
    if (r >= N || nature[r] != 0) return;
    cm[r] = cm[r] + fm[r];
    cp[r] = cp[r] + fp[r];
}

unsigned blocks(long long N) { return (unsigned)((N + EB - 1) / EB); }

int need_charges(lbgpu_ctx *ctx, const char *fn)
{
    if (!ctx->pnp)
        return ctx_fail(ctx, LBGPU_ERR_INVALID, std::string(fn) + ": call lbgpu_pnp_init (or lbgpu_pnp_set) first");
    return LBGPU_OK;
}

int alloc_zero(lbgpu_ctx *ctx, double **p, size_t n)
{
    if (*p) return LBGPU_OK;
    LBG_CK(ctx, cudaMalloc((void **)p, n * sizeof(double)));
    ctx->pnp->allocs.push_back(*p);
    LBG_CK(ctx, cudaMemsetAsync(*p, 0, n * sizeof(double), ctx->stream));
    return LBGPU_OK;
}

int download(lbgpu_ctx *ctx, std::vector<double> &h, const double *d)
{
    h.resize((size_t)ctx->N);
    LBG_CK(ctx, cudaMemcpyAsync(h.data(), d, sizeof(double) * ctx->N, cudaMemcpyDeviceToHost, ctx->stream));
    LBG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return LBGPU_OK;
}

}  // namespace
}  // namespace lbg

using namespace lbg;

extern "C" {

int lbgpu_electrostatic_pot(lbgpu_ctx *ctx, const double elec_slope[3])
{
    if (!ctx || !elec_slope) return LBGPU_ERR_INVALID;
    int rc = need_charges(ctx, "lbgpu_electrostatic_pot");
    if (rc) return rc;
    PnpState *s = ctx->pnp;
    if ((rc = alloc_zero(ctx, &s->phi_tot, (size_t)ctx->N))) return rc;
    const int zero = elec_slope[0] == 0.0 && elec_slope[1] == 0.0 && elec_slope[2] == 0.0;
    k_ek_pot<<<blocks(ctx->N), EB, 0, ctx->stream>>>(s->phi[s->par], s->phi_tot, ctx->N, ctx->p.lx, ctx->p.ly,
                                                     elec_slope[0], elec_slope[1], elec_slope[2], zero);
    LBG_CK(ctx, cudaGetLastError());
    return lbgpu_sync(ctx);
}

int lbgpu_comp_j(lbgpu_ctx *ctx, const double *n, double *jx, double *jy, double *jz)
{
    if (!ctx || !n || !jx || !jy || !jz) return LBGPU_ERR_INVALID;
    TraceRange trace_("lbgpu_comp_j");
    const long long N = ctx->N;
    cudaStream_t st = ctx->stream;
    double *d = nullptr;
    LBG_CK(ctx, cudaMallocAsync((void **)&d, sizeof(double) * 22 * (size_t)N, st));
    double *dj[3] = {d + 19 * N, d + 20 * N, d + 21 * N};
    double *hj[3] = {jx, jy, jz};
    cudaError_t e = cudaMemcpyAsync(d, n, sizeof(double) * 19 * N, cudaMemcpyHostToDevice, st);
    for (int q = 0; q < 3 && e == cudaSuccess; ++q)
        e = cudaMemcpyAsync(dj[q], hj[q], sizeof(double) * N, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        k_comp_j<<<blocks(N), EB, 0, st>>>(d, dj[0], dj[1], dj[2], N);
        e = cudaGetLastError();
    }
    for (int q = 0; q < 3 && e == cudaSuccess; ++q)
        e = cudaMemcpyAsync(hj[q], dj[q], sizeof(double) * N, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return ctx_cuda(ctx, e, "lbgpu_comp_j");
}

int lbgpu_smolu(lbgpu_ctx *ctx, int time, int D_iter, const double elec_slope[3],
                const double lncb_slope[3], double el_curr[3], double ion_curr[3])
{
    if (!ctx || !elec_slope || !lncb_slope || !el_curr || !ion_curr) return LBGPU_ERR_INVALID;
    TraceRange trace_("lbgpu_smolu");
    int rc = need_charges(ctx, "lbgpu_smolu");
    if (rc) return rc;
    PnpState *s = ctx->pnp;
    if (!s->phi_tot)
        return ctx_fail(ctx, LBGPU_ERR_INVALID, "lbgpu_smolu: call lbgpu_electrostatic_pot first (phi_tot)");
    const long long N = ctx->N;
    if ((rc = alloc_zero(ctx, &s->solute_force, 3 * (size_t)N))) return rc;
    SmoluArgs a;
    a.mask = ctx->d_mask;
    a.phi_tot = s->phi_tot;
    a.cp = s->cp;
    a.cm = s->cm;
    a.fp = s->fp;      // just_eq_smolu's scratch: smolu's site fluxes are local arrays too
    a.fm = s->fm;
    a.sf = s->solute_force;
    a.partial = nullptr;
    a.N = N;
    a.lx = ctx->p.lx;
    a.ly = ctx->p.ly;
    a.lz = ctx->p.lz;
    a.Dp = s->p.D_plus;
    a.Dm = s->p.D_minus;
    a.dit = (double)D_iter;
    a.kbt = 1.0 / 3.0;                                // module_system.f90:94
    for (int d = 0; d < 3; ++d) {
        a.es[d] = elec_slope[d];
        a.ls[d] = lncb_slope[d];
    }
    const double csq = 1.0 / 3.0;                     // module_lbmodel.f90:127-136
    a.a1[0] = (1.0 / 3.0) / csq;
    a.a1[1] = (1.0 / 18.0) / csq;
    a.a1[2] = (1.0 / 36.0) / csq;
    a.delta[0] = 0.0;
    a.delta[1] = 1.0;
    a.delta[2] = std::sqrt(2.0);                      // module_lbmodel.f90:137
    const unsigned grid = std::min(blocks(N), (unsigned)MP_MAX_BLOCKS);
    double *part = nullptr, *res = nullptr;
    LBG_CK(ctx, cudaMallocAsync((void **)&part, sizeof(double) * (6 * (size_t)grid + 6), ctx->stream));
    res = part + 6 * (size_t)grid;
    a.partial = part;
    double cur[6], fs[2];
    cudaError_t e;
    k_smolu<<<grid, EB, 0, ctx->stream>>>(a);
    k_sum6<<<1, 32, 0, ctx->stream>>>(part, grid, 6, res);
    e = cudaMemcpyAsync(cur, res, sizeof(cur), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) {
        k_smolu_update<<<grid, EB, 0, ctx->stream>>>(a);
        k_sum6<<<1, 32, 0, ctx->stream>>>(part, grid, 2, res);
        e = cudaMemcpyAsync(fs, res, sizeof(fs), cudaMemcpyDeviceToHost, ctx->stream);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaFreeAsync(part, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx_cuda(ctx, e, "lbgpu_smolu");
    for (int d = 0; d < 3; ++d) {
        el_curr[d] = el_curr[d] + cur[d];
        ion_curr[d] = ion_curr[d] + cur[3 + d];
    }
    if (time > 0) {
        // n_fluidsites = sum(node%nature, mask=node%nature==fluid) (smolu.f90:125): the natures
        // of fluid nodes are 0, so the reference divides the currents by zero
        volatile double n_fluidsites = 0.0;
        for (int d = 0; d < 3; ++d) {
            el_curr[d] = el_curr[d] / n_fluidsites;
            ion_curr[d] = ion_curr[d] / n_fluidsites;
        }
    }
    if (std::fabs(fs[0]) > (double)1.0e-12f || std::fabs(fs[1]) > (double)1.0e-12f)
        return ctx_fail(ctx, LBGPU_ERR_FLUX_SUM, "in smolu.f90 the sum of all fluxes does not add up to zero! stop.");
    return LBGPU_OK;
}

int lbgpu_advect(lbgpu_ctx *ctx, const double *jx, const double *jy, const double *jz,
                 double el_curr[3], double ion_curr[3])
{
    if (!ctx || !jx || !jy || !jz || !el_curr || !ion_curr) return LBGPU_ERR_INVALID;
    TraceRange trace_("lbgpu_advect");
    int rc = need_charges(ctx, "lbgpu_advect");
    if (rc) return rc;
    PnpState *s = ctx->pnp;
    const long long N = ctx->N;
    const double eps = DBL_EPSILON;
    std::vector<double> cp, cm;
    std::vector<int8_t> nat((size_t)N);
    if ((rc = download(ctx, cp, s->cp)) || (rc = download(ctx, cm, s->cm))) return rc;
    LBG_CK(ctx, cudaMemcpyAsync(nat.data(), ctx->d_nature, (size_t)N, cudaMemcpyDeviceToHost, ctx->stream));
    LBG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    // advect.f90:32-50 on the host, in the reference's element order
    bool all_zero = true, all_diff0 = true, all_sum0 = true;
    for (long long r = 0; r < N; ++r) {
        if (!(std::fabs(cp[r]) <= eps && std::fabs(cm[r]) <= eps)) all_zero = false;
        if (!(std::fabs(cp[r] - cm[r]) <= eps)) all_diff0 = false;
        if (!(std::fabs(cp[r] + cm[r]) <= eps)) all_sum0 = false;
    }
    if (all_zero) return LBGPU_OK;
    const double *J[3] = {jx, jy, jz};
    if (all_diff0) {
        el_curr[0] = el_curr[1] = el_curr[2] = 0.0;
    } else {
        for (int d = 0; d < 3; ++d) {
            double acc = 0.0;
            for (long long r = 0; r < N; ++r)
                if (nat[r] == 0) acc = acc + J[d][r] * (cp[r] - cm[r]);
            el_curr[d] = -acc;
        }
    }
    if (all_sum0) {   // advect.f90:46-49 zeroes el_curr in this branch, not ion_curr
        el_curr[0] = el_curr[1] = el_curr[2] = 0.0;
    } else {
        for (int d = 0; d < 3; ++d) {
            double acc = 0.0;
            for (long long r = 0; r < N; ++r)
                if (nat[r] == 0) acc = acc + J[d][r] * (cp[r] + cm[r]);
            ion_curr[d] = -acc;
        }
    }
    double cp_old = 0.0, cm_old = 0.0;
    for (long long r = 0; r < N; ++r) cp_old = cp_old + cp[r];
    for (long long r = 0; r < N; ++r) cm_old = cm_old + cm[r];
    if ((rc = alloc_zero(ctx, &s->adv_fp, (size_t)N)) || (rc = alloc_zero(ctx, &s->adv_fm, (size_t)N))) return rc;
    double *dj = nullptr;
    cudaStream_t st = ctx->stream;
    LBG_CK(ctx, cudaMallocAsync((void **)&dj, sizeof(double) * 3 * (size_t)N, st));
    cudaError_t e = cudaSuccess;
    for (int d = 0; d < 3 && e == cudaSuccess; ++d)
        e = cudaMemcpyAsync(dj + d * N, J[d], sizeof(double) * N, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        AdvectArgs a{ctx->d_nature, dj, dj + N, dj + 2 * N, s->cp, s->cm, s->adv_fp, s->adv_fm, N,
                     ctx->p.lx, ctx->p.ly, ctx->p.lz};
        k_advect<<<blocks(N), EB, 0, st>>>(a);
        k_advect_update<<<blocks(N), EB, 0, st>>>(ctx->d_nature, s->adv_fp, s->adv_fm, s->cp, s->cm, N);
        e = cudaGetLastError();
    }
    cudaFreeAsync(dj, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return ctx_cuda(ctx, e, "lbgpu_advect");
    if ((rc = download(ctx, cp, s->cp)) || (rc = download(ctx, cm, s->cm))) return rc;
    double cm_new = 0.0, cp_new = 0.0;
    for (long long r = 0; r < N; ++r) cm_new = cm_new + cm[r];
    for (long long r = 0; r < N; ++r) cp_new = cp_new + cp[r];
    if (std::fabs(cm_new - cm_old) > (double)1.e-8f || std::fabs(cp_new - cp_old) > (double)1.e-8f)
        return ctx_fail(ctx, LBGPU_ERR_CHARGE,
                        "Total concentration has changed in advect.f90. STOP but unsure STOP is needed");
    return LBGPU_OK;
}

int lbgpu_ek_get(lbgpu_ctx *ctx, double *phi_tot, double *solute_force)
{
    if (!ctx) return LBGPU_ERR_INVALID;
    int rc = need_charges(ctx, "lbgpu_ek_get");
    if (rc) return rc;
    PnpState *s = ctx->pnp;
    const long long N = ctx->N;
    if (phi_tot) {
        if (!s->phi_tot) return ctx_fail(ctx, LBGPU_ERR_INVALID, "lbgpu_ek_get: no phi_tot yet");
        LBG_CK(ctx, cudaMemcpyAsync(phi_tot, s->phi_tot, sizeof(double) * N, cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (solute_force) {
        if (s->solute_force)
            LBG_CK(ctx, cudaMemcpyAsync(solute_force, s->solute_force, sizeof(double) * 3 * N,
                                        cudaMemcpyDeviceToHost, ctx->stream));
        else
            std::memset(solute_force, 0, sizeof(double) * 3 * N);
    }
    return lbgpu_sync(ctx);
}

}  // extern "C"
