// mp_f64.cu -- FP64 strict tracer moment propagation (compiled with -fmad=false).
//
// The scattering probabilities (module_moment_propagation.f90:341-346; fermi = 1/2 for a neutral
// tracer, per link from the potential for a charged one) depend only on the converged flow (and
// the potential), so they are computed once, in the reference's
// operation order, into a table coef[(l-1)*N + r] = scattprop of node r+c_l towards r.  A step
// then gathers P_now from the fluid neighbours through that table, in l order, exactly as the
// reference's sweep does (module_moment_propagation.f90:207-253): the propagated quantities are
// bit-identical to the reference; only the VACF node sum runs in a different (fixed) order.
// Storing the table instead of recomputing it matters on GB300, whose FP64 rate is low.
#include "common.cuh"
#include "lbgpu.h"
#include "mp.h"
#include "reduce.cuh"

namespace lbg {
namespace {

__device__ __forceinline__ void nb_offsets(long long node, int lx, int ly, int lz, long long (&X)[3],
                                           long long (&Y)[3], long long (&Z)[3])
{
    const unsigned nd = (unsigned)node;
    const int x = (int)(nd % (unsigned)lx);
    const unsigned yz = nd / (unsigned)lx;
    const int y = (int)(yz % (unsigned)ly), z = (int)(yz / (unsigned)ly);
    const long long sy = lx, sz = (long long)lx * ly;
    // [c+1] = coordinate of (x + c), periodic
    X[0] = wrap_minus(x, lx);       X[1] = x;       X[2] = wrap_plus(x, lx);
    Y[0] = wrap_minus(y, ly) * sy;  Y[1] = y * sy;  Y[2] = wrap_plus(y, ly) * sy;
    Z[0] = wrap_minus(z, lz) * sz;  Z[1] = z * sz;  Z[2] = wrap_plus(z, lz) * sz;
}

// tracer population n_l (drop_tracers.f90:97-100, fluid node):
// a0*rho + a1*sum(c(:)*(J(:) + f_ext(:) - rho*q*D*E(:)))
template <int L>
__device__ __forceinline__ double n_tracer(double rho, double Jx, double Jy, double Jz,
                                           const MpArgs64 &a)
{
    constexpr Vel c = vel(L);
    constexpr int w = wclass(L);
    double s = 0.0;
    if constexpr (c.x != 0) {
        const double t = Jx + a.fext[0] - rho * a.q * a.D * a.E[0];
        s = c.x > 0 ? s + t : s - t;
    }
    if constexpr (c.y != 0) {
        const double t = Jy + a.fext[1] - rho * a.q * a.D * a.E[1];
        s = c.y > 0 ? s + t : s - t;
    }
    if constexpr (c.z != 0) {
        const double t = Jz + a.fext[2] - rho * a.q * a.D * a.E[2];
        s = c.z > 0 ? s + t : s - t;
    }
    if constexpr (L == 0) return a.a0[w] * rho;
    else return a.a0[w] * rho + a.a1[w] * s;
}

template <int L>
__device__ __forceinline__ double scattprop(double n, double rho, const MpArgs64 &a)
{
    // n/rho - w + lambda*w*fermi with fermi = 1/2   (module_moment_propagation.f90:345)
    return n / rho - a.a0[wclass(L)] + a.lwh[wclass(L)];
}

// module_moment_propagation.f90:303-322: phi(r') - phi(r) of the link from (x, y, z) to
// (xp, yp, zp) (0-based), with the elec_slope correction of a link across the periodic boundary;
// only the first matching case of the reference's chain applies.
__device__ __forceinline__ double dphi64(const MpArgs64 &a, long long r, long long rp, int x, int y,
                                         int z, int xp, int yp, int zp)
{
    double d = a.phi[rp] - a.phi[r];
    if (x == a.lx - 1 && xp == 0) d = d + a.E[0] * (double)(a.lx + 1);
    else if (x == 0 && xp == a.lx - 1) d = d - a.E[0] * (double)(a.lx + 1);
    else if (y == a.ly - 1 && yp == 0) d = d + a.E[1] * (double)(a.ly + 1);
    else if (y == 0 && yp == a.ly - 1) d = d - a.E[1] * (double)(a.ly + 1);
    else if (z == a.lz - 1 && zp == 0) d = d + a.E[2] * (double)(a.lz + 1);
    else if (z == 0 && zp == a.lz - 1) d = d - a.E[2] * (double)(a.lz + 1);
    return d;
}

// n/rho - w + (lambda*w)*fermi (module_moment_propagation.f90:345) for a link's fermi factor
template <int L>
__device__ __forceinline__ double scattprop_f(double n, double rho, double fermi, const MpArgs64 &a)
{
    return n / rho - a.a0[wclass(L)] + a.lw[wclass(L)] * fermi;
}

// module_moment_propagation.f90:30-160 (init) for every fluid node: scattering table, remaining
// fraction, u*, P(t=1) and this block's share of VACF(0).  CHARGED: Boltzmann weight
// exp(-z phi)/Pstat per node and fermi = 1/(1 + exp(z dphi)) per link (:97-135, 295-327); the
// table then holds the charged scatterings and the step kernel is the same.
template <bool CHARGED>
__global__ void __launch_bounds__(MP_BLOCK) k_mp_init(const MpArgs64 a)
{
    __shared__ double sh[MP_BLOCK / 32];
    const long long N = a.N;
    const long long r = (long long)blockIdx.x * MP_BLOCK + threadIdx.x;
    double v[3] = {0.0, 0.0, 0.0};
    unsigned bad = 0;
    if (r < N) {
        const uint32_t m = a.mask[r];
        if (m & FLUID_BIT) {
            long long X[3], Y[3], Z[3];
            nb_offsets(r, a.lx, a.ly, a.lz, X, Y, Z);
            const double rho = a.rho[r], Jx = a.jx[r], Jy = a.jy[r], Jz = a.jz[r];
            double frac = 1.0, ux = 0.0, uy = 0.0, uz = 0.0;
            double P[3] = {0.0, 0.0, 0.0};
            // boltz_weight (module_moment_propagation.f90:105-111)
            const double bw = CHARGED ? exp(-(a.z * a.phi[r])) / a.pstat : a.bw;
            const int sx = a.lx, sxy = a.lx * a.ly;
            const int x = (int)(r % sx), y = (int)((r / sx) % a.ly), z = (int)(r / sxy);
            static_for<1, Q>([&](auto L) {
                constexpr int l = decltype(L)::value;
                constexpr int li = inv(l);
                constexpr Vel c = vel(l);
                constexpr Vel ci = vel(li);
                if ((m >> li) & 1u) {   // neighbour r + c_l is solid
                    a.coef[(long long)(l - 1) * N + r] = 0.0;
                    return;
                }
                const long long rp = X[c.x + 1] + Y[c.y + 1] + Z[c.z + 1];
                double sp, spp, emd = 1.0;
                const double rhop = a.rho[rp];
                if constexpr (CHARGED) {
                    const int xp = (int)(X[c.x + 1]), yp = (int)(Y[c.y + 1] / sx), zp = (int)(Z[c.z + 1] / sxy);
                    const double e = exp(a.z * dphi64(a, r, rp, x, y, z, xp, yp, zp));
                    emd = 1.0 / e;
                    const double fermi = 1.0 / (1.0 + e);
                    sp = scattprop_f<l>(n_tracer<l>(rho, Jx, Jy, Jz, a), rho, fermi, a);
                    spp = scattprop_f<li>(n_tracer<li>(rhop, a.jx[rp], a.jy[rp], a.jz[rp], a), rhop,
                                          1.0 - fermi, a);
                } else {
                    sp = scattprop<l>(n_tracer<l>(rho, Jx, Jy, Jz, a), rho, a);
                    spp = scattprop<li>(n_tracer<li>(rhop, a.jx[rp], a.jy[rp], a.jz[rp], a), rhop, a);
                }
                frac = frac - sp;
                if constexpr (c.x != 0) ux = c.x > 0 ? ux + sp : ux - sp;
                if constexpr (c.y != 0) uy = c.y > 0 ? uy + sp : uy - sp;
                if constexpr (c.z != 0) uz = c.z > 0 ? uz + sp : uz - sp;
                const double bs = bw * sp;
                if constexpr (c.x != 0) v[0] = v[0] + bs;
                if constexpr (c.y != 0) v[1] = v[1] + bs;
                if constexpr (c.z != 0) v[2] = v[2] + bs;
                a.coef[(long long)(l - 1) * N + r] = spp;
                // P(r,1) += exp_min_dphi * scattprop_p * c_inv * boltz_weight
                // (exp_min_dphi = 1 for a neutral tracer: the product is dropped, exactly)
                const double t = CHARGED ? emd * spp : spp;
                if constexpr (ci.x != 0) P[0] = P[0] + (ci.x > 0 ? t : -t) * bw;
                if constexpr (ci.y != 0) P[1] = P[1] + (ci.y > 0 ? t : -t) * bw;
                if constexpr (ci.z != 0) P[2] = P[2] + (ci.z > 0 ? t : -t) * bw;
            });
            a.frac[r] = frac;
            a.us[0][r] = ux;
            a.us[1][r] = uy;
            a.us[2][r] = uz;
            for (int d = 0; d < 3; ++d) a.P[0][d][r] = P[d];
            const double fr = (a.ads && (m & INTERFACIAL_BIT)) ? frac - a.ka : frac;
            if (fr < 2.220446049250313e-16) bad = LBGPU_ERR_FRACTION;
        }
    }
    for (int d = 0; d < 3; ++d) {
        const double b = block_sum_fixed(v[d], sh);
        if (threadIdx.x == 0) a.partial[3 * blockIdx.x + d] = b;
    }
    if (bad) atomicOr(&a.ctl->status, bad);
}

// module_moment_propagation.f90:164-289, one step.  Grid-stride over the nodes.  The gathers
// are branch-free: a link to a solid neighbour has coefficient 0 and the neighbour's P is 0, so
// it adds an exact zero where the reference skips it (only the sign of an exact zero can differ).
// FUSED (LBGPU_FP64_FUSED): each link's gather and the remaining-fraction terms as fused
// multiply-adds, in the same order (within 1e-12 relative of the separately rounded form).
template <bool FUSED>
__global__ void __launch_bounds__(MP_BLOCK) k_mp_step(const MpArgs64 a)
{
    const volatile MpCtl *vc = a.ctl;
    if (vc->done) return;
    const int par = vc->parity;
    const long long N = a.N;
    const double *__restrict__ Px = a.P[par][0];
    const double *__restrict__ Py = a.P[par][1];
    const double *__restrict__ Pz = a.P[par][2];
    double v[3] = {0.0, 0.0, 0.0};
    // the fluid nodes through their list (every lane of a warp does work), else every lattice node
    const long long n_it = a.fidx ? a.Nf : N;
    for (long long i = (long long)blockIdx.x * MP_BLOCK + threadIdx.x; i < n_it;
         i += (long long)gridDim.x * MP_BLOCK) {
        const long long r = a.fidx ? (long long)a.fidx[i] : i;
        const uint32_t m = a.mask[r];
        if (!(m & FLUID_BIT)) continue;
        long long X[3], Y[3], Z[3];
        nb_offsets(r, a.lx, a.ly, a.lz, X, Y, Z);
        double n0 = 0.0, n1 = 0.0, n2 = 0.0;
        static_for<1, Q>([&](auto L) {
            constexpr int l = decltype(L)::value;
            constexpr Vel c = vel(l);
            const long long rp = X[c.x + 1] + Y[c.y + 1] + Z[c.z + 1];
            const double cf = a.coef[(long long)(l - 1) * N + r];
            if constexpr (FUSED) {
                n0 = __fma_rn(Px[rp], cf, n0);
                n1 = __fma_rn(Py[rp], cf, n1);
                n2 = __fma_rn(Pz[rp], cf, n2);
            } else {
                n0 = n0 + Px[rp] * cf;
                n1 = n1 + Py[rp] * cf;
                n2 = n2 + Pz[rp] * cf;
            }
        });
        const double p0 = Px[r], p1 = Py[r], p2 = Pz[r];
        v[0] = v[0] + p0 * a.us[0][r];
        v[1] = v[1] + p1 * a.us[1][r];
        v[2] = v[2] + p2 * a.us[2][r];
        const double frac = a.frac[r];
        if (FUSED && (!a.ads || !(m & INTERFACIAL_BIT))) {
            n0 = __fma_rn(frac, p0, n0);
            n1 = __fma_rn(frac, p1, n1);
            n2 = __fma_rn(frac, p2, n2);
        } else if (!a.ads || !(m & INTERFACIAL_BIT)) {
            n0 = n0 + frac * p0;
            n1 = n1 + frac * p1;
            n2 = n2 + frac * p2;
        } else {
            const double f2 = frac - a.ka;
            const double q0 = a.A[par][0][r], q1 = a.A[par][1][r], q2 = a.A[par][2][r];
            n0 = n0 + f2 * p0 + q0 * a.kd;
            n1 = n1 + f2 * p1 + q1 * a.kd;
            n2 = n2 + f2 * p2 + q2 * a.kd;
            a.A[par ^ 1][0][r] = q0 * a.one_minus_kd + p0 * a.ka;
            a.A[par ^ 1][1][r] = q1 * a.one_minus_kd + p1 * a.ka;
            a.A[par ^ 1][2][r] = q2 * a.one_minus_kd + p2 * a.ka;
        }
        a.P[par ^ 1][0][r] = n0;
        a.P[par ^ 1][1][r] = n1;
        a.P[par ^ 1][2][r] = n2;
    }
    grid_sum3(v, a.partial, &a.ctl->blocks_done,
              [&](const double (&tot)[3]) { mp_control(a.ctl, a.hist, tot); });
}

// Sum of the init partials in block order -> ctl->vacf (VACF at t = 0).
__global__ void __launch_bounds__(MP_BLOCK) k_mp_reduce(const double *partial, unsigned nb, MpCtl *ctl)
{
    __shared__ double sh[MP_BLOCK / 32];
    double t[3] = {0.0, 0.0, 0.0};
    for (unsigned i = threadIdx.x; i < nb; i += MP_BLOCK)
        for (int d = 0; d < 3; ++d) t[d] += partial[3 * i + d];
    for (int d = 0; d < 3; ++d) {
        const double s = block_sum_fixed(t[d], sh);
        if (threadIdx.x == 0) ctl->vacf[d] = s;
    }
}

}  // namespace

cudaError_t launch_mp_init_f64(const MpArgs64 &a, unsigned grid, cudaStream_t s)
{
    if (a.phi) k_mp_init<true><<<grid, MP_BLOCK, 0, s>>>(a);
    else k_mp_init<false><<<grid, MP_BLOCK, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_mp_step_f64(const MpArgs64 &a, unsigned grid, cudaStream_t s)
{
    if (a.fused) k_mp_step<true><<<grid, MP_BLOCK, 0, s>>>(a);
    else k_mp_step<false><<<grid, MP_BLOCK, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_mp_reduce_init(double *partial, unsigned nblocks, MpCtl *ctl, cudaStream_t s)
{
    k_mp_reduce<<<1, MP_BLOCK, 0, s>>>(partial, nblocks, ctl);
    return cudaGetLastError();
}

}  // namespace lbg
