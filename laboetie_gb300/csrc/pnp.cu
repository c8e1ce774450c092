// pnp.cu -- Poisson + Nernst-Planck equilibration of the ion densities (compiled with
// -fmad=false): charges_init.f90, sor.f90, just_eq_smolu.f90, poisson_nernst_planck.f90,
// check_charge_distribution_equilibrium.f90, charge_test.f90.
//
// The potential and the ion densities stay in FP64.  The reference solver ("SOR", sor.f90) is an
// over-relaxed Jacobi sweep with the D3Q19 weights including the self weight 1/3; each sweep is
// reproduced operation for operation, so the iterates are bit-identical to the reference's.  The
// fast solver is a 4-colour successive over-relaxation of the same discrete equation
// (2/3) phi - sum_{l>0} w_l phi(x - c_l) = 4 pi bjl kBT/2 (c+ - c-): no two D3Q19 neighbours share
// a colour ((x+z) mod 2, (y+z) mod 2) when lx, ly, lz are even.
//
// Sums that decide a stopping rule are formed in a fixed order (block partials added in block
// order), so runs are reproducible; the normalisations that the reference forms once per call
// (anormf0 = sum|phi|, charges_init.f90:126) are summed on the host in the reference's order.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "ctx.h"
#include "lbgpu.h"
#include "trace.h"
#include "pnp.h"
#include "reduce.cuh"

namespace lbg {

namespace {
constexpr int PB = MP_BLOCK;
constexpr double PI_D = 3.141592653589793;   // acos(-1.0_dp), module_constants.f90:19
}

const double *pnp_potential(const lbgpu_ctx *ctx)
{
    return ctx->pnp ? ctx->pnp->phi[ctx->pnp->par] : nullptr;
}

void pnp_release(lbgpu_ctx *ctx)
{
    if (!ctx->pnp) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    PnpState *ps = ctx->pnp;
    if (ps->anorm_thread.joinable()) {
        {
            std::lock_guard<std::mutex> lk(ps->anorm_m);
            ps->anorm_quit = true;
        }
        ps->anorm_cv.notify_all();
        ps->anorm_thread.join();
    }
    if (ps->anorm_ev) cudaEventDestroy(ps->anorm_ev);
    for (cudaGraphExec_t g : ctx->pnp->sor_exec)
        if (g) cudaGraphExecDestroy(g);
    for (void *p : ctx->pnp->allocs) cudaFree(p);
    if (ctx->pnp->phi_host) cudaFreeHost(ctx->pnp->phi_host);
    delete ctx->pnp;
    ctx->pnp = nullptr;
}

namespace {

struct PnpArgs {
    const uint32_t *mask;
    const double *phi;
    double *phi_out;
    const double *cp, *cm;
    double *fp, *fm;
    double *partial;
    PnpCtl *ctl;
    long long N;
    int lx, ly, lz;
    double a0[3];
    double factor, omega, one_minus_omega;
    double eDp, eDm;
    double delta_axis, delta_diag;
    int color;        // multicolour SOR: the colour of this launch
    int ncolor;       // colours per sweep (the last colour's launch decides the stopping test)
    int gen;          // general colouring (some side odd): colour from k_sor_color_gen's rule
    int kx, ky, kz;   // colours per axis of the general colouring (1, 2 or 3)
    int loop_bug;     // just_eq_smolu.f90:68-70
};

__device__ __forceinline__ void coords(long long r, int lx, int ly, int &x, int &y, int &z)
{
    const unsigned nd = (unsigned)r;
    x = (int)(nd % (unsigned)lx);
    const unsigned yz = nd / (unsigned)lx;
    y = (int)(yz % (unsigned)ly);
    z = (int)(yz / (unsigned)ly);
}

// offset of (x + dx, y + dy, z + dz), periodic, dx.. in {-1,0,1}
__device__ __forceinline__ long long nb(int x, int y, int z, int dx, int dy, int dz, int lx, int ly, int lz)
{
    const int xx = dx > 0 ? wrap_plus(x, lx) : (dx < 0 ? wrap_minus(x, lx) : x);
    const int yy = dy > 0 ? wrap_plus(y, ly) : (dy < 0 ? wrap_minus(y, ly) : y);
    const int zz = dz > 0 ? wrap_plus(z, lz) : (dz < 0 ? wrap_minus(z, lz) : z);
    return xx + (long long)lx * (yy + (long long)ly * zz);
}

// Final sum of the 4-value block partials of the last kernel, in block order.
// The control block of a solve, set on the device (a kernel parameter, no staged host copy).
__global__ void k_ctl_set(PnpCtl *ctl, const PnpCtl c) { *ctl = c; }

__global__ void __launch_bounds__(PB) k_sum4(const double *partial, unsigned nb, double *out)
{
    __shared__ double sh[4][PB / 32];
    double t[4] = {0, 0, 0, 0};
    for (unsigned i = threadIdx.x; i < nb; i += PB)
        for (int q = 0; q < 4; ++q) t[q] += partial[4 * i + q];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int q = 0; q < 4; ++q) t[q] = warp_sum_fixed(t[q]);
    if (lane == 0)
        for (int q = 0; q < 4; ++q) sh[q][wid] = t[q];
    __syncthreads();
    if (wid == 0) {
        for (int q = 0; q < 4; ++q) {
            double v = lane < PB / 32 ? sh[q][lane] : 0.0;
            v = warp_sum_fixed(v);
            if (lane == 0) out[q] = v;
        }
    }
}

__device__ __forceinline__ void block_partial4(double (&t)[4], double *partial)
{
    __shared__ double sh[4][PB / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int q = 0; q < 4; ++q) t[q] = warp_sum_fixed(t[q]);
    if (lane == 0)
        for (int q = 0; q < 4; ++q) sh[q][wid] = t[q];
    __syncthreads();
    if (wid == 0) {
        for (int q = 0; q < 4; ++q) {
            double v = lane < PB / 32 ? sh[q][lane] : 0.0;
            v = warp_sum_fixed(v);
            if (lane == 0) partial[4 * blockIdx.x + q] = v;
        }
    }
}

// sor.f90:48-70 one Jacobi sweep over every node (solid included), then the stopping test of
// sor.f90:78 by the last block.
__global__ void __launch_bounds__(PB) k_sor_jacobi(const PnpArgs a, double *phi0, double *phi1)
{
    const volatile PnpCtl *vc = a.ctl;
    if (vc->done) return;
    const int par = vc->parity;
    const double *__restrict__ src = par ? phi1 : phi0;
    double *__restrict__ dst = par ? phi0 : phi1;
    double t[3] = {0.0, 0.0, 0.0};
    for (long long r = (long long)blockIdx.x * PB + threadIdx.x; r < a.N; r += (long long)gridDim.x * PB) {
        int x, y, z;
        coords(r, a.lx, a.ly, x, y, z);
        double phistar = 0.0;
        static_for<0, Q>([&](auto L) {
            constexpr int l = decltype(L)::value;
            constexpr Vel c = vel(l);
            // phi(pbc(i - c_l)) (sor.f90:54-57)
            phistar = phistar + a.a0[wclass(l)] * src[nb(x, y, z, -c.x, -c.y, -c.z, a.lx, a.ly, a.lz)];
        });
        phistar = phistar + a.factor * (a.cp[r] - a.cm[r]);
        const double phiold = src[r];
        dst[r] = a.omega * phistar + a.one_minus_omega * phiold;
        t[0] = t[0] + fabs(phistar - phiold);
    }
    grid_sum3(t, a.partial, &a.ctl->blocks_done, [&](const double (&tot)[3]) {
        PnpCtl *c = a.ctl;
        c->anorm = tot[0];
        c->parity ^= 1;  // phi = phitmp (sor.f90:70)
        c->iter += 1;
        if (tot[0] <= c->limit) {
            c->converged = 1;
            c->done = 1;
        } else if (c->iter >= c->max_iter) {
            c->done = 1;
        }
    });
}

// Colour of a coordinate along one axis for the multicolour SOR: a proper colouring of the
// periodic ring of L nodes (adjacent nodes, the wrap included, get different colours): 0 for a
// one-wide axis (a step along it returns to the node itself), x mod 2 for even L, and x mod 2
// with the last node coloured 2 for odd L.
__device__ __forceinline__ int ring_colour(int x, int L)
{
    if (L == 1) return 0;
    if ((L & 1) == 0) return x & 1;
    return x == L - 1 ? 2 : (x & 1);
}

// Update of one node of the multicolour SOR: phi <- (1-omega) phi + omega * 1.5 (sum_{l>0} w_l
// phi(x-c_l) + b); returns the node's part of the stopping measure, |phi* - phi| with phi* the
// reference's Jacobi target sum_{l>=0} w_l phi(x-c_l) + b at the current state (the quantity the
// reference's test sums, sor.f90:67,78), so both solvers stop on the same residual.
__device__ __forceinline__ double sor_node(const PnpArgs &a, double *phi, int x, int y, int z, long long r)
{
    // this solver is not the reference's, so it may fuse: explicit multiply-adds (the file is
    // built without contraction for the reference sweeps) halve its FP64 instructions
    double s = 0.0;
    static_for<1, Q>([&](auto L) {
        constexpr int l = decltype(L)::value;
        constexpr Vel c = vel(l);
        s = __fma_rn(a.a0[wclass(l)], phi[nb(x, y, z, -c.x, -c.y, -c.z, a.lx, a.ly, a.lz)], s);
    });
    const double rhs = __fma_rn(a.factor, a.cp[r] - a.cm[r], s);
    const double old = phi[r];
    phi[r] = __fma_rn(a.one_minus_omega, old, a.omega * (1.5 * rhs));
    return fabs(__fma_rn(-a.a0[0] * 2.0, old, rhs));   // |phi* - phi| = |rhs - (2/3) phi|
}

// The colour's last launch of a sweep decides the stopping test of the multicolour SOR.
__device__ __forceinline__ void sor_colour_done(const PnpArgs &a, const double (&tot)[3])
{
    PnpCtl *c = a.ctl;
    c->anorm += tot[0];
    if (a.color == a.ncolor - 1) {
        c->iter += 1;
        if (c->anorm <= c->limit) {
            c->converged = 1;
            c->done = 1;
        } else if (c->iter >= c->max_iter) {
            c->done = 1;
        }
        if (!c->done) c->anorm = 0.0;
    }
}

// One colour of the 4-colour SOR of boxes with even sides ((x+z)&1 | ((y+z)&1)<<1): the threads
// walk only the colour's N/4 nodes: in plane z the colour holds the rows y = 2j + (c1 ^ z&1) and
// in them the nodes x = 2i + (c0 ^ z&1), c0 and c1 the colour's bits.
__global__ void __launch_bounds__(PB) k_sor_color(const PnpArgs a, double *phi)
{
    const volatile PnpCtl *vc = a.ctl;
    if (vc->done) return;
    double t[3] = {0.0, 0.0, 0.0};
    const int hx = a.lx >> 1, hy = a.ly >> 1;
    const long long Nc = (long long)hx * hy * a.lz;
    for (long long k = (long long)blockIdx.x * PB + threadIdx.x; k < Nc; k += (long long)gridDim.x * PB) {
        const long long q = k / hx;
        const int z = (int)(q / hy), zp = z & 1;
        const int x = 2 * (int)(k - q * hx) + ((a.color & 1) ^ zp);
        const int y = 2 * (int)(q - (long long)z * hy) + (((a.color >> 1) & 1) ^ zp);
        const long long r = x + (long long)a.lx * (y + (long long)a.ly * z);
        t[0] = t[0] + sor_node(a, phi, x, y, z, r);
    }
    grid_sum3(t, a.partial, &a.ctl->blocks_done, [&](const double (&tot)[3]) { sor_colour_done(a, tot); });
}

// One colour of the multicolour SOR of any box (some side odd or one wide).  With gx, gy, gz the
// ring colours of the node's coordinates (kx, ky, kz colours each), the node's colour is
// A + ka B, A = (gx + gz) mod ka, B = (gy + gz) mod kb, ka = max(kx, kz), kb = max(ky, kz).  For
// fixed gz, A is one-to-one in gx, and for fixed gx in gz (likewise B), so every D3Q19 link
// changes A or B: a step along x or xy changes A (gz fixed), along y B, along z, xz or yz the
// sum with the unchanged coordinate; nodes of one colour never neighbour each other, and a
// colour's launch can update them in place.  Up to 9 colours (all sides odd); a 1 x 1 x N
// column needs 2 (N even) or 3.  Grid-stride over every node, updating those of the colour.
__global__ void __launch_bounds__(PB) k_sor_color_gen(const PnpArgs a, double *phi)
{
    const volatile PnpCtl *vc = a.ctl;
    if (vc->done) return;
    double t[3] = {0.0, 0.0, 0.0};
    const int ka = max(a.kx, a.kz), kb = max(a.ky, a.kz);
    for (long long r = (long long)blockIdx.x * PB + threadIdx.x; r < a.N; r += (long long)gridDim.x * PB) {
        int x, y, z;
        coords(r, a.lx, a.ly, x, y, z);
        const int gx = ring_colour(x, a.lx), gy = ring_colour(y, a.ly), gz = ring_colour(z, a.lz);
        const int colour = (gx + gz) % ka + ka * ((gy + gz) % kb);
        if (colour != a.color) continue;
        t[0] = t[0] + sor_node(a, phi, x, y, z, r);
    }
    grid_sum3(t, a.partial, &a.ctl->blocks_done, [&](const double (&tot)[3]) { sor_colour_done(a, tot); });
}

// Sum of the reference's stopping measure |phi* - phi| over every node at the current phi (no
// update): the residual both solvers are compared on.
__global__ void __launch_bounds__(PB) k_residual(const PnpArgs a, const double *phi)
{
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long r = (long long)blockIdx.x * PB + threadIdx.x; r < a.N; r += (long long)gridDim.x * PB) {
        int x, y, z;
        coords(r, a.lx, a.ly, x, y, z);
        double phistar = 0.0;
        static_for<0, Q>([&](auto L) {
            constexpr int l = decltype(L)::value;
            constexpr Vel c = vel(l);
            phistar = phistar + a.a0[wclass(l)] * phi[nb(x, y, z, -c.x, -c.y, -c.z, a.lx, a.ly, a.lz)];
        });
        phistar = phistar + a.factor * (a.cp[r] - a.cm[r]);
        t[0] = t[0] + fabs(phistar - phi[r]);
    }
    block_partial4(t, a.partial);
}

// Sum of phi over every node (block partials), and phi -= shift: the multicolour SOR's solution is
// pinned to the sum of phi it started from, which the reference's Jacobi sweep keeps (its weights
// sum to 1 and a neutral system's charge terms sum to 0), so that both solvers return the same
// member of the family of solutions of the periodic problem (they differ by a constant).
__global__ void __launch_bounds__(PB) k_sum_phi(const double *phi, long long N, double *partial)
{
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long r = (long long)blockIdx.x * PB + threadIdx.x; r < N; r += (long long)gridDim.x * PB)
        t[0] = t[0] + phi[r];
    block_partial4(t, partial);
}

__global__ void __launch_bounds__(PB) k_shift_phi(double *phi, long long N, double shift)
{
    for (long long r = (long long)blockIdx.x * PB + threadIdx.x; r < N; r += (long long)gridDim.x * PB)
        phi[r] = phi[r] - shift;
}

// Link flux of just_eq_smolu.f90:86-99 from site a (origin) to site b along direction l.
__device__ __forceinline__ void link_flux(const PnpArgs &k, long long ra, long long rb, double delta,
                                          double &Jp, double &Jm)
{
    const double e = exp(k.phi[rb] - k.phi[ra]);
    const double em = 1.0 / e;
    Jp = 0.5 * (1.0 + em) * (k.cp[rb] * e - k.cp[ra]);
    Jp = Jp * k.eDp / delta;
    Jm = 0.5 * (1.0 + e) * (k.cm[rb] * em - k.cm[ra]);
    Jm = Jm * k.eDm / delta;
}

// flux_site_plus/minus of just_eq_smolu.f90:61-103 in gather form: every site adds the fluxes
// of the links it starts (l = 2,4,..,18 of the reference) and subtracts those that end on it;
// with loop_bug only sites of the line (i, ly, lz) start links.  Also the four sums of the
// conservation test (108-112) and of the norm (122-129).
__global__ void __launch_bounds__(PB) k_np_flux(const PnpArgs a)
{
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long r = (long long)blockIdx.x * PB + threadIdx.x; r < a.N; r += (long long)gridDim.x * PB) {
        int x, y, z;
        coords(r, a.lx, a.ly, x, y, z);
        const bool fl = a.mask[r] & FLUID_BIT;
        double sp = 0.0, sm = 0.0;
        if (fl) {
            const bool origin_me = !a.loop_bug || (y == a.ly - 1 && z == a.lz - 1);
            static_for<0, 9>([&](auto P) {
                // l = 2, 4, ..., 18 of the reference (just_eq_smolu.f90:66): one of each pair
                constexpr int l = 2 * decltype(P)::value + 1;
                constexpr Vel c = vel(l);
                const double delta = wclass(l) == 1 ? a.delta_axis : a.delta_diag;
                if (origin_me) {
                    const long long rb = nb(x, y, z, c.x, c.y, c.z, a.lx, a.ly, a.lz);
                    if (a.mask[rb] & FLUID_BIT) {
                        double Jp, Jm;
                        link_flux(a, r, rb, delta, Jp, Jm);
                        sp = sp + Jp;
                        sm = sm + Jm;
                    }
                }
                // link that ends here: starts at r - c_l
                const int ox = c.x > 0 ? wrap_minus(x, a.lx) : (c.x < 0 ? wrap_plus(x, a.lx) : x);
                const int oy = c.y > 0 ? wrap_minus(y, a.ly) : (c.y < 0 ? wrap_plus(y, a.ly) : y);
                const int oz = c.z > 0 ? wrap_minus(z, a.lz) : (c.z < 0 ? wrap_plus(z, a.lz) : z);
                const bool origin_o = !a.loop_bug || (oy == a.ly - 1 && oz == a.lz - 1);
                const long long ro = ox + (long long)a.lx * (oy + (long long)a.ly * oz);
                if (origin_o && (a.mask[ro] & FLUID_BIT)) {
                    double Jp, Jm;
                    link_flux(a, ro, r, delta, Jp, Jm);
                    sp = sp - Jp;
                    sm = sm - Jm;
                }
            });
        }
        a.fp[r] = sp;
        a.fm[r] = sm;
        t[0] = t[0] + sp;
        t[1] = t[1] + sm;
        if (fl) {
            t[2] = t[2] + sp * sp;
            t[3] = t[3] + sm * sm;
        }
    }
    block_partial4(t, a.partial);
}

// c+- += flux on fluid nodes (just_eq_smolu.f90:115-118)
__global__ void __launch_bounds__(PB) k_np_update(const PnpArgs a, double *cp, double *cm)
{
    for (long long r = (long long)blockIdx.x * PB + threadIdx.x; r < a.N; r += (long long)gridDim.x * PB) {
        if (a.mask[r] & FLUID_BIT) {
            cp[r] = cp[r] + a.fp[r];
            cm[r] = cm[r] + a.fm[r];
        }
    }
}

// check_charge_distribution_equilibrium.f90:30-37: sums of |(v - v_old)/v_old| over |v_old| > 1e-12
// and the counts, for phi (q = 0), c+ (1), c- (2).  Two launches: (phi, c+) and (c-).
__global__ void __launch_bounds__(PB) k_rel_change(const double *v0, const double *o0, const double *v1,
                                                   const double *o1, long long N, double *partial)
{
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long r = (long long)blockIdx.x * PB + threadIdx.x; r < N; r += (long long)gridDim.x * PB) {
        const double eps = 1.0e-12;
        if (fabs(o0[r]) > eps) {
            t[0] = t[0] + fabs((v0[r] - o0[r]) / o0[r]);
            t[1] = t[1] + 1.0;
        }
        if (v1 && fabs(o1[r]) > eps) {
            t[2] = t[2] + fabs((v1[r] - o1[r]) / o1[r]);
            t[3] = t[3] + 1.0;
        }
    }
    block_partial4(t, partial);
}

// charge_test.f90:15-19: charge on solid and on fluid nodes.
__global__ void __launch_bounds__(PB) k_charges(const uint32_t *mask, const double *cp, const double *cm,
                                                long long N, double *partial)
{
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long r = (long long)blockIdx.x * PB + threadIdx.x; r < N; r += (long long)gridDim.x * PB) {
        const double q = cp[r] - cm[r];
        if (mask[r] & FLUID_BIT) t[1] = t[1] + q;
        else t[0] = t[0] + q;
    }
    block_partial4(t, partial);
}

unsigned grid_for(long long N)
{
    const long long g = (N + PB - 1) / PB;
    return (unsigned)std::min<long long>(g, MP_MAX_BLOCKS);
}

void fill_pnp_args(lbgpu_ctx *ctx, PnpArgs &a)
{
    PnpState *s = ctx->pnp;
    std::memset(&a, 0, sizeof(a));
    a.mask = ctx->d_mask;
    a.phi = s->phi[s->par];
    a.cp = s->cp;
    a.cm = s->cm;
    a.fp = s->fp;
    a.fm = s->fm;
    a.partial = s->partial;
    a.ctl = s->ctl;
    a.N = ctx->N;
    a.lx = ctx->p.lx;
    a.ly = ctx->p.ly;
    a.lz = ctx->p.lz;
    for (int w = 0; w < 3; ++w) a.a0[w] = ctx->K64.a0[w];
    const volatile double kBT = 1.0 / 3.0;
    a.factor = 4.0 * PI_D * s->p.bjl * kBT / 2.0;   // sor.f90:36
    a.eDp = 0.1 * s->p.D_plus;                      // just_eq_smolu.f90:35-38
    a.eDm = 0.1 * s->p.D_minus;
    a.delta_axis = 1.0;
    a.delta_diag = std::sqrt(2.0);
    a.loop_bug = s->p.np_loop_bug;
}

int read4(lbgpu_ctx *ctx, unsigned nb, double out[4])
{
    PnpState *s = ctx->pnp;
    LBG_CK(ctx, cudaGetLastError());
    k_sum4<<<1, PB, 0, ctx->stream>>>(s->partial, nb, s->result);
    LBG_CK(ctx, cudaGetLastError());
    LBG_CK(ctx, cudaMemcpyAsync(out, s->result, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    LBG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return LBGPU_OK;
}

// Two block-partial reductions (partials at s->partial and at s->partial + 4 nb) read back with
// one synchronisation; each is summed exactly as read4 sums it.
int read4x2(lbgpu_ctx *ctx, unsigned nb, double out0[4], double out1[4])
{
    PnpState *s = ctx->pnp;
    LBG_CK(ctx, cudaGetLastError());
    k_sum4<<<1, PB, 0, ctx->stream>>>(s->partial, nb, s->result);
    k_sum4<<<1, PB, 0, ctx->stream>>>(s->partial + 4 * (size_t)nb, nb, s->result + 4);
    LBG_CK(ctx, cudaGetLastError());
    double h[8];
    LBG_CK(ctx, cudaMemcpyAsync(h, s->result, 8 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    LBG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    for (int q = 0; q < 4; ++q) {
        out0[q] = h[q];
        out1[q] = h[4 + q];
    }
    return LBGPU_OK;
}

// anormf0 = sum(abs(phi)) in the reference's order (sor.f90:90), on the host, from a page-locked
// copy of phi.  anorm_begin enqueues the copy and hands the sum to the state's worker thread,
// which waits for the copy (an event) and adds the values up in element order; anorm_end waits
// for it and stores anormf0.  Between the two the caller may go on (the outer loop runs its
// Nernst-Planck update and convergence test, which do not read anormf0).
void anorm_worker(PnpState *s, long long N, int device)
{
    cudaSetDevice(device);   // the context's device, current on this thread too
    for (;;) {
        std::unique_lock<std::mutex> lk(s->anorm_m);
        s->anorm_cv.wait(lk, [s] { return s->anorm_job || s->anorm_quit; });
        if (s->anorm_quit) return;
        s->anorm_job = false;
        lk.unlock();
        const bool ok = cudaEventSynchronize(s->anorm_ev) == cudaSuccess;
        double a = 0.0;
        if (ok)
            for (long long i = 0; i < N; ++i) a = a + std::fabs(s->phi_host[i]);
        lk.lock();
        s->anorm_sum = a;
        s->anorm_failed = !ok;
        s->anorm_ready = true;
        lk.unlock();
        s->anorm_cv.notify_all();
    }
}

int anorm_begin(lbgpu_ctx *ctx)
{
    PnpState *s = ctx->pnp;
    if (!s->phi_host) LBG_CK(ctx, cudaMallocHost((void **)&s->phi_host, sizeof(double) * ctx->N));
    if (!s->anorm_ev) LBG_CK(ctx, cudaEventCreateWithFlags(&s->anorm_ev, cudaEventDisableTiming));
    if (!s->anorm_thread.joinable()) s->anorm_thread = std::thread(anorm_worker, s, ctx->N, ctx->p.device);
    LBG_CK(ctx, cudaMemcpyAsync(s->phi_host, s->phi[s->par], sizeof(double) * ctx->N, cudaMemcpyDeviceToHost,
                                ctx->stream));
    LBG_CK(ctx, cudaEventRecord(s->anorm_ev, ctx->stream));
    {
        std::lock_guard<std::mutex> lk(s->anorm_m);
        s->anorm_job = true;
        s->anorm_pending = true;
        s->anorm_ready = false;
    }
    s->anorm_cv.notify_all();
    return LBGPU_OK;
}

int anorm_end(lbgpu_ctx *ctx)
{
    PnpState *s = ctx->pnp;
    std::unique_lock<std::mutex> lk(s->anorm_m);
    if (!s->anorm_pending) return LBGPU_OK;
    s->anorm_cv.wait(lk, [s] { return s->anorm_ready; });
    s->anorm_pending = false;
    s->anorm_ready = false;
    if (s->anorm_failed) return ctx_fail(ctx, LBGPU_ERR_CUDA, "anormf0: copy of phi failed");
    s->anormf0 = s->anorm_sum;
    return LBGPU_OK;
}

int need_pnp(lbgpu_ctx *ctx, const char *fn)
{
    if (!ctx->pnp)
        return ctx_fail(ctx, LBGPU_ERR_INVALID, std::string(fn) + ": call lbgpu_pnp_init first");
    return LBGPU_OK;
}

}  // namespace
}  // namespace lbg

using namespace lbg;

extern "C" {

int lbgpu_pnp_init(lbgpu_ctx *ctx, const lbgpu_pnp_params *p, double *anormf0)
{
    if (!ctx || !p) return LBGPU_ERR_INVALID;
    const double eps = 2.220446049250313e-16;
    if (p->D_plus < 0.0) return ctx_fail(ctx, LBGPU_ERR_INVALID, "D_plus <0. critical.");
    if (p->D_minus < 0.0) return ctx_fail(ctx, LBGPU_ERR_INVALID, "D_minus <0. critical.");
    if (p->solver != LBGPU_POISSON_REFERENCE && p->solver != LBGPU_POISSON_SOR4 &&
        p->solver != LBGPU_POISSON_JACOBI)
        return ctx_fail(ctx, LBGPU_ERR_INVALID, "lbgpu_pnp_init: unknown solver");
    pnp_release(ctx);
    PnpState *s = new PnpState();
    ctx->pnp = s;
    s->p = *p;
    const long long N = ctx->N;
    cudaStream_t st = ctx->stream;
    auto alloc = [&](double **q, size_t n) -> int {
        LBG_CK(ctx, cudaMalloc((void **)q, n * sizeof(double)));
        s->allocs.push_back(*q);
        LBG_CK(ctx, cudaMemsetAsync(*q, 0, n * sizeof(double), st));
        return LBGPU_OK;
    };
    int rc;
    for (int b = 0; b < 2; ++b)
        if ((rc = alloc(&s->phi[b], N))) return rc;
    if ((rc = alloc(&s->cp, N)) || (rc = alloc(&s->cm, N)) || (rc = alloc(&s->fp, N)) ||
        (rc = alloc(&s->fm, N)))
        return rc;
    for (int q = 0; q < 3; ++q)
        if ((rc = alloc(&s->bak[q], N))) return rc;
    // partials: 4 per block, twice (two reductions read back together); results: 4, twice
    if ((rc = alloc(&s->partial, 8 * (size_t)MP_MAX_BLOCKS)) || (rc = alloc(&s->result, 8))) return rc;
    LBG_CK(ctx, cudaMalloc((void **)&s->ctl, sizeof(PnpCtl)));
    s->allocs.push_back(s->ctl);
    LBG_CK(ctx, cudaMemsetAsync(s->ctl, 0, sizeof(PnpCtl), st));

    // charges_init.f90:23-135 on the host, node by node in the reference's order
    if (p->bjl <= eps) {                       // :25 no charge at all
        if (anormf0) *anormf0 = 0.0;
        return lbgpu_sync(ctx);
    }
    const double pi = PI_D, kBT = 1.0 / 3.0;
    double rho_0 = std::fabs(p->lambda_D) <= eps ? 0.0 : 1.0 / (4.0 * pi * p->bjl * (p->lambda_D * p->lambda_D));
    s->rho_ch = 1.0 / (4.0 * pi * p->bjl * (p->lambda_D * p->lambda_D));
    if (!(std::fabs(p->sigma) > eps)) {
        if (anormf0) *anormf0 = 0.0;
        return lbgpu_sync(ctx);
    }
    if (p->charge_distrib != 0)                // 'sol' stops the reference (charges_init.f90:96-100)
        return ctx_fail(ctx, LBGPU_ERR_UNSUPPORTED, "only surface charge is implemented for now in charge_init.f90");
    s->charged = true;
    std::vector<uint32_t> m(N);
    LBG_CK(ctx, cudaMemcpyAsync(m.data(), ctx->d_mask, sizeof(uint32_t) * N, cudaMemcpyDeviceToHost, st));
    LBG_CK(ctx, cudaStreamSynchronize(st));
    const long long count_fluid = (long long)ctx->counts[0], count_solid_int = (long long)ctx->counts[3];
    const double sigma_solid = count_solid_int != 0 ? p->sigma / count_solid_int : 0.0;
    const double sigma_fluid = count_fluid != 0 ? -1.0 * p->sigma / count_fluid : 0.0;
    const double cps = +0.5 * sigma_solid, cms = -0.5 * sigma_solid;
    double cpf, cmf;
    if (sigma_fluid > 0.0) {
        cpf = 0.5 * rho_0 + sigma_fluid;
        cmf = 0.5 * rho_0;
    } else {
        cpf = 0.5 * rho_0;
        cmf = 0.5 * rho_0 - sigma_fluid;
    }
    std::vector<double> hp(N), hm(N);
    double sum = 0.0;
    for (long long i = 0; i < N; ++i) {
        const bool fluid = m[i] & FLUID_BIT, inter = m[i] & INTERFACIAL_BIT;
        if (!fluid && inter) { hp[i] = cps; hm[i] = cms; }
        else if (!fluid) { hp[i] = 0.0; hm[i] = 0.0; }
        else { hp[i] = cpf; hm[i] = cmf; }
        sum = sum + (hp[i] + hm[i]);
    }
    s->anormf0 = 4.0 * pi * p->bjl * kBT / 2.0 * sum;   // charges_init.f90:126
    LBG_CK(ctx, cudaMemcpyAsync(s->cp, hp.data(), sizeof(double) * N, cudaMemcpyHostToDevice, st));
    LBG_CK(ctx, cudaMemcpyAsync(s->cm, hm.data(), sizeof(double) * N, cudaMemcpyHostToDevice, st));
    LBG_CK(ctx, cudaStreamSynchronize(st));
    if (anormf0) *anormf0 = s->anormf0;
    return LBGPU_OK;
}

int lbgpu_pnp_set(lbgpu_ctx *ctx, const double *c_plus, const double *c_minus, const double *phi,
                  double anormf0)
{
    if (!ctx || !c_plus || !c_minus || !phi) return LBGPU_ERR_INVALID;
    int rc = need_pnp(ctx, "lbgpu_pnp_set");
    if (rc) return rc;
    PnpState *s = ctx->pnp;
    const size_t b = sizeof(double) * ctx->N;
    LBG_CK(ctx, cudaMemcpyAsync(s->cp, c_plus, b, cudaMemcpyHostToDevice, ctx->stream));
    LBG_CK(ctx, cudaMemcpyAsync(s->cm, c_minus, b, cudaMemcpyHostToDevice, ctx->stream));
    LBG_CK(ctx, cudaMemcpyAsync(s->phi[s->par], phi, b, cudaMemcpyHostToDevice, ctx->stream));
    s->anormf0 = anormf0;
    s->charged = true;
    return lbgpu_sync(ctx);
}

int lbgpu_pnp_get(lbgpu_ctx *ctx, double *c_plus, double *c_minus, double *phi, double *anormf0)
{
    if (!ctx) return LBGPU_ERR_INVALID;
    int rc = need_pnp(ctx, "lbgpu_pnp_get");
    if (rc) return rc;
    PnpState *s = ctx->pnp;
    const size_t b = sizeof(double) * ctx->N;
    if (c_plus) LBG_CK(ctx, cudaMemcpyAsync(c_plus, s->cp, b, cudaMemcpyDeviceToHost, ctx->stream));
    if (c_minus) LBG_CK(ctx, cudaMemcpyAsync(c_minus, s->cm, b, cudaMemcpyDeviceToHost, ctx->stream));
    if (phi) LBG_CK(ctx, cudaMemcpyAsync(phi, s->phi[s->par], b, cudaMemcpyDeviceToHost, ctx->stream));
    if (anormf0) *anormf0 = s->anormf0;
    return lbgpu_sync(ctx);
}

static int sor_solve(lbgpu_ctx *ctx, int *iters, bool defer_anorm);

int lbgpu_sor(lbgpu_ctx *ctx, int *iters)
{
    TraceRange trace_("lbgpu_sor");
    if (!ctx) return LBGPU_ERR_INVALID;
    int rc = need_pnp(ctx, "lbgpu_sor");
    if (rc) return rc;
    return sor_solve(ctx, iters, false);
}

// The solve of lbgpu_sor; with defer_anorm the new anormf0 is still being summed on return
// (anorm_end, which the next solve calls first, completes it).
static int sor_solve(lbgpu_ctx *ctx, int *iters, bool defer_anorm)
{
    int rc = anorm_end(ctx);   // the limit below uses the previous solve's anormf0
    if (rc) return rc;
    PnpState *s = ctx->pnp;
    cudaStream_t st = ctx->stream;
    if (iters) *iters = 0;
    if (s->p.sigma == 0.0) {   // sor.f90:29-33
        LBG_CK(ctx, cudaMemsetAsync(s->phi[s->par], 0, sizeof(double) * ctx->N, st));
        return lbgpu_sync(ctx);
    }
    PnpArgs a;
    fill_pnp_args(ctx, a);
    const bool multi = s->p.solver == LBGPU_POISSON_SOR4;
    const bool four = multi && ctx->p.lx % 2 == 0 && ctx->p.ly % 2 == 0 && ctx->p.lz % 2 == 0;
    auto ring = [](int L) { return L == 1 ? 1 : (L % 2 == 0 ? 2 : 3); };
    a.kx = ring(ctx->p.lx);
    a.ky = ring(ctx->p.ly);
    a.kz = ring(ctx->p.lz);
    a.gen = multi && !four;
    a.ncolor = four ? 4 : std::max(a.kx, a.kz) * std::max(a.ky, a.kz);
    PnpCtl c;
    std::memset(&c, 0, sizeof(c));
    c.parity = s->par;
    if (s->p.solver == LBGPU_POISSON_REFERENCE) {
        a.omega = 1.4;                                  // sor.f90:19
        c.limit = (double)1.0e-5f * s->anormf0;         // sor.f90:18,78
        c.max_iter = s->p.max_iter > 0 ? s->p.max_iter : 500000;
    } else {
        a.omega = s->p.omega;
        c.limit = s->p.tol * s->anormf0;
        c.max_iter = s->p.max_iter > 0 ? s->p.max_iter : 500000;
    }
    a.one_minus_omega = 1.0 - a.omega;
    k_ctl_set<<<1, 1, 0, st>>>(s->ctl, c);
    LBG_CK(ctx, cudaGetLastError());
    const unsigned grid = grid_for(ctx->N);
    // sweeps after the exit are no-ops (the control block is done): a graph of one sweep first
    // (in the outer loop of the Poisson-Nernst-Planck solve most solves end at their first
    // sweep), then graphs of 64 until the solve converges or reaches its cap
    for (int k = 0; k < 2; ++k) {
        if (s->sor_exec[k]) continue;
        const int G = k == 0 ? 1 : 64;
        cudaGraph_t g;
        LBG_CK(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        for (int q = 0; q < G; ++q) {
            if (multi) {
                for (int col = 0; col < a.ncolor; ++col) {
                    PnpArgs b = a;
                    b.color = col;
                    if (four) k_sor_color<<<grid, PB, 0, st>>>(b, s->phi[s->par]);
                    else k_sor_color_gen<<<grid, PB, 0, st>>>(b, s->phi[s->par]);
                }
            } else {
                k_sor_jacobi<<<grid, PB, 0, st>>>(a, s->phi[0], s->phi[1]);
            }
        }
        cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (ce != cudaSuccess) return ctx_cuda(ctx, ce, "capture sor");
        ce = cudaGraphInstantiate(&s->sor_exec[k], g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            s->sor_exec[k] = nullptr;
            return ctx_cuda(ctx, ce, "instantiate sor");
        }
    }
    double sum0 = 0.0;
    if (multi) {
        double r4[4];
        k_sum_phi<<<grid, PB, 0, st>>>(s->phi[s->par], ctx->N, s->partial);
        if ((rc = read4(ctx, grid, r4))) return rc;
        sum0 = r4[0];
    }
    cudaError_t e = cudaSuccess;
    for (int round = 0;; ++round) {
        e = cudaGraphLaunch(s->sor_exec[round == 0 ? 0 : 1], st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&c, s->ctl, sizeof(c), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess || c.done) break;
    }
    if (e != cudaSuccess) return ctx_cuda(ctx, e, "lbgpu_sor");
    if (multi) {
        double r4[4];
        k_sum_phi<<<grid, PB, 0, st>>>(s->phi[s->par], ctx->N, s->partial);
        if ((rc = read4(ctx, grid, r4))) return rc;
        k_shift_phi<<<grid, PB, 0, st>>>(s->phi[s->par], ctx->N, (r4[0] - sum0) / (double)ctx->N);
        LBG_CK(ctx, cudaGetLastError());
    }
    if (!multi) s->par = c.parity;
    if (iters) *iters = s->p.solver == LBGPU_POISSON_SOR4 ? c.iter : c.iter - 1;  // sor.f90:87
    if ((rc = anorm_begin(ctx))) return rc;                       // sor.f90:90
    if (!defer_anorm && (rc = anorm_end(ctx))) return rc;
    if (!c.converged)
        return ctx_fail(ctx, LBGPU_ERR_STEP_CAP, "maximum iterations 500 000 reached without convergence in sor");
    return LBGPU_OK;
}

int lbgpu_just_eq_smolu(lbgpu_ctx *ctx, int *iters)
{
    TraceRange trace_("lbgpu_just_eq_smolu");
    if (!ctx) return LBGPU_ERR_INVALID;
    int rc = need_pnp(ctx, "lbgpu_just_eq_smolu");
    if (rc) return rc;
    PnpState *s = ctx->pnp;
    cudaStream_t st = ctx->stream;
    PnpArgs a;
    fill_pnp_args(ctx, a);
    const unsigned grid = grid_for(ctx->N);
    const double crit = (double)5.e-6f;           // just_eq_smolu.f90:20
    const double big = 1.7976931348623157e308;
    double tot_p = big, tot_m = big;
    const int max_iter = 10;                      // just_eq_smolu.f90:35-38
    const double cf = (double)ctx->counts[0];
    int iter = 0;
    while (tot_m + tot_p > crit && iter < max_iter) {
        k_np_flux<<<grid, PB, 0, st>>>(a);
        double r4[4];
        if ((rc = read4(ctx, grid, r4))) return rc;
        if (std::fabs(r4[0]) > (double)1.e-12f || std::fabs(r4[1]) > (double)1.e-12f)
            return ctx_fail(ctx, LBGPU_ERR_FLUX_SUM,
                            "the sum of all flux does not add up. problem in just_eq_smolu.f90");
        k_np_update<<<grid, PB, 0, st>>>(a, s->cp, s->cm);
        LBG_CK(ctx, cudaGetLastError());
        if (s->p.sigma != 0 && a.eDp != 0.0 && a.eDm != 0.0) {
            tot_p = std::sqrt(r4[2]) / cf / (0.5 * s->rho_ch * a.eDp) / s->p.sigma;
            tot_m = std::sqrt(r4[3]) / cf / (0.5 * s->rho_ch * a.eDm) / s->p.sigma;
        }
        iter = iter + 1;
    }
    if (iters) *iters = iter;
    return lbgpu_sync(ctx);
}

int lbgpu_poisson_residual(lbgpu_ctx *ctx, double *residual, double *anormf0)
{
    if (!ctx || !residual) return LBGPU_ERR_INVALID;
    int rc = need_pnp(ctx, "lbgpu_poisson_residual");
    if (rc) return rc;
    PnpState *s = ctx->pnp;
    PnpArgs a;
    fill_pnp_args(ctx, a);
    const unsigned grid = grid_for(ctx->N);
    k_residual<<<grid, PB, 0, ctx->stream>>>(a, s->phi[s->par]);
    double r4[4];
    if ((rc = read4(ctx, grid, r4))) return rc;
    *residual = r4[0];
    if (anormf0) *anormf0 = s->anormf0;
    return LBGPU_OK;
}

int lbgpu_charge_test(lbgpu_ctx *ctx, double *solid_charge, double *fluid_charge)
{
    if (!ctx) return LBGPU_ERR_INVALID;
    int rc = need_pnp(ctx, "lbgpu_charge_test");
    if (rc) return rc;
    PnpState *s = ctx->pnp;
    const unsigned grid = grid_for(ctx->N);
    k_charges<<<grid, PB, 0, ctx->stream>>>(ctx->d_mask, s->cp, s->cm, ctx->N, s->partial);
    double r4[4];
    if ((rc = read4(ctx, grid, r4))) return rc;
    if (solid_charge) *solid_charge = r4[0];
    if (fluid_charge) *fluid_charge = r4[1];
    const double tol = (double)1.0e-10f;         // charge_test.f90:10
    if (std::fabs(r4[0] - s->p.sigma) > tol || std::fabs(r4[1] + s->p.sigma) > tol)
        return ctx_fail(ctx, LBGPU_ERR_CHARGE, "charge is not conserved. check charge_test.f90. stop");
    return LBGPU_OK;
}

int lbgpu_poisson_nernst_planck(lbgpu_ctx *ctx, int max_outer, int *outer, int *sor_iters_total)
{
    TraceRange trace_("lbgpu_poisson_nernst_planck");
    if (!ctx) return LBGPU_ERR_INVALID;
    int rc = need_pnp(ctx, "lbgpu_poisson_nernst_planck");
    if (rc) return rc;
    PnpState *s = ctx->pnp;
    cudaStream_t st = ctx->stream;
    if (outer) *outer = 0;
    if (sor_iters_total) *sor_iters_total = 0;
    if (!(std::fabs(s->p.sigma) > 2.220446049250313e-16)) return LBGPU_OK;   // poisson_nernst_planck.f90:20-21
    const size_t b = sizeof(double) * ctx->N;
    const unsigned grid = grid_for(ctx->N);
    int n = 0, total = 0;
    bool converged = false;
    // every exit leaves anormf0 complete (no sum still running on the worker thread)
    struct AnormDone {
        lbgpu_ctx *ctx;
        ~AnormDone() { anorm_end(ctx); }
    } anorm_done_{ctx};
    while (!converged) {
        if (max_outer > 0 && n >= max_outer) {
            if (outer) *outer = n;
            if (sor_iters_total) *sor_iters_total = total;
            return ctx_fail(ctx, LBGPU_ERR_STEP_CAP, "Equilibrium distribution of salts not found");
        }
        // backup_phi_c_plus_c_minus.f90
        LBG_CK(ctx, cudaMemcpyAsync(s->bak[0], s->phi[s->par], b, cudaMemcpyDeviceToDevice, st));
        LBG_CK(ctx, cudaMemcpyAsync(s->bak[1], s->cp, b, cudaMemcpyDeviceToDevice, st));
        LBG_CK(ctx, cudaMemcpyAsync(s->bak[2], s->cm, b, cudaMemcpyDeviceToDevice, st));
        int it = 0;
        if ((rc = sor_solve(ctx, &it, true))) return rc;   // anormf0 summed meanwhile
        total += it;
        if ((rc = lbgpu_just_eq_smolu(ctx, nullptr))) return rc;
        // check_charge_distribution_equilibrium.f90:24-44
        double r4[4], q4[4];
        k_rel_change<<<grid, PB, 0, st>>>(s->phi[s->par], s->bak[0], s->cp, s->bak[1], ctx->N, s->partial);
        k_rel_change<<<grid, PB, 0, st>>>(s->cm, s->bak[2], nullptr, nullptr, ctx->N, s->partial + 4 * (size_t)grid);
        if ((rc = read4x2(ctx, grid, r4, q4))) return rc;
        const double eps = 1.0e-12;
        const double dphi = r4[1] != 0 ? r4[0] / r4[1] : 0.0;
        const double dcp = r4[3] != 0 ? r4[2] / r4[3] : 0.0;
        const double dcm = q4[1] != 0 ? q4[0] / q4[1] : 0.0;
        converged = dphi < eps && dcp < eps && dcm < eps;
        n++;
    }
    if (outer) *outer = n;
    if (sor_iters_total) *sor_iters_total = total;
    if ((rc = anorm_end(ctx))) return rc;
    double sc, fc;
    return lbgpu_charge_test(ctx, &sc, &fc);   // poisson_nernst_planck.f90:50
}

}  // extern "C"
