// flow_f64.cu -- FP64 D3Q19 kernels (compiled with -fmad=false): the strict form, and the fused
// step of LBGPU_FP64_FUSED (explicit fused multiply-adds, collide_node_fused).
//
// Bit-exactness with the reference.  Every product and sum is evaluated in the operand order
// of the Fortran source with separate roundings (no fused multiply-add in this translation
// unit).  Terms that the reference multiplies by a velocity component of 0 are exactly +-0 and
// are left out; terms multiplied by +-1 are exact and become additions or subtractions.  Both
// transformations keep every intermediate value identical (at most the sign of an exact zero
// can differ), so the populations, densities and fluxes equal the reference's operation for
// operation.  This matters on GB300 beyond parity: FP64 issues at a small fraction of FP32,
// so every FP64 operation skipped is time saved.
//
// Streaming.  The reference swaps populations across fluid/solid links and then pushes
// (equilibration.f90:204-243).  Each population takes part in at most one swap, so the pair is
// exactly the pull rule  n_new(x,l) = n*(x - c_l, l)  if nature(x - c_l) == nature(x),
// else n*(x, inv l).  The kernels pull; bit l of the node flag word says which source to use.
#include <cfloat>

#include "common.cuh"
#include "flow.h"
#include "lbgpu.h"

namespace lbg {
namespace {

constexpr int BLOCK = 256;

// (cx*x + cy*y) + cz*z with the zero-velocity terms left out (c = +-1 terms are exact).
template <int CX, int CY, int CZ>
__device__ __forceinline__ double dotc(double x, double y, double z)
{
    const double tx = CX > 0 ? x : -x, ty = CY > 0 ? y : -y, tz = CZ > 0 ? z : -z;
    if constexpr (CX != 0 && CY != 0 && CZ != 0) return (tx + ty) + tz;
    else if constexpr (CX != 0 && CY != 0) return tx + ty;
    else if constexpr (CX != 0 && CZ != 0) return tx + tz;
    else if constexpr (CY != 0 && CZ != 0) return ty + tz;
    else if constexpr (CX != 0) return tx;
    else if constexpr (CY != 0) return ty;
    else if constexpr (CZ != 0) return tz;
    else return 0.0;
}

template <int SIGN>
__device__ __forceinline__ double addsgn(double s, double t)
{
    if constexpr (SIGN > 0) return s + t;
    else if constexpr (SIGN < 0) return s - t;
    else return s;
}

// module_collision.f90:77-108 for one fluid node, all 19 velocities.
// FMASK: which components of the force are non-zero (bit 0 x, 1 y, 2 z); 0 = no force.
// UCF: the force is the launch-uniform f_ext and c_l.F is taken from a.cf.
template <int FMASK, bool UCF>
__device__ __forceinline__ void collide_node(double (&n)[Q], const double rho, const double jx,
                                             const double jy, const double jz, const double fx,
                                             const double fy, const double fz,
                                             const FlowArgs64 &a)
{
    const LbConst64 &K = a.K;
    const double ux = jx / rho, uy = jy / rho, uz = jz / rho;
    const double Pxx = jx * ux, Pxy = jx * uy, Pxz = jx * uz;
    const double Pyx = jy * ux, Pyy = jy * uy, Pyz = jy * uz;
    const double Pzx = jz * ux, Pzy = jz * uy, Pzz = jz * uz;
    const double Dx1 = Pxx * K.k1, Dx0 = Pxx * K.k0;
    const double Dy1 = Pyy * K.k1, Dy0 = Pyy * K.k0;
    const double Dz1 = Pzz * K.k1, Dz0 = Pzz * K.k0;
    const double ar[3] = {K.a0[0] * rho, K.a0[1] * rho, K.a0[2] * rho};
    // (c_a - u_a) * f_a for c_a = 0, +1, -1
    double gx0 = 0, gxp = 0, gxm = 0, gy0 = 0, gyp = 0, gym = 0, gz0 = 0, gzp = 0, gzm = 0;
    if constexpr (FMASK & 1) { gx0 = (-ux) * fx; gxp = (1.0 - ux) * fx; gxm = (-1.0 - ux) * fx; }
    if constexpr (FMASK & 2) { gy0 = (-uy) * fy; gyp = (1.0 - uy) * fy; gym = (-1.0 - uy) * fy; }
    if constexpr (FMASK & 4) { gz0 = (-uz) * fz; gzp = (1.0 - uz) * fz; gzm = (-1.0 - uz) * fz; }

    static_for<0, Q>([&](auto L) {
        constexpr int l = decltype(L)::value;
        constexpr Vel c = vel(l);
        constexpr int w = wclass(l);
        // a2 term: jx*ux*(cx^2-cs^2) + jx*uy*cx*cy + ... + jz*uz*(cz^2-cs^2)
        double S = c.x != 0 ? Dx1 : Dx0;
        S = addsgn<c.x * c.y>(S, Pxy);
        S = addsgn<c.x * c.z>(S, Pxz);
        S = addsgn<c.y * c.x>(S, Pyx);
        S = S + (c.y != 0 ? Dy1 : Dy0);
        S = addsgn<c.y * c.z>(S, Pyz);
        S = addsgn<c.z * c.x>(S, Pzx);
        S = addsgn<c.z * c.y>(S, Pzy);
        S = S + (c.z != 0 ? Dz1 : Dz0);
        double neq;
        if constexpr (l == 0) {
            neq = ar[0] + K.a2[0] * S;
        } else {
            const double cj = dotc<c.x, c.y, c.z>(jx, jy, jz);
            neq = (ar[w] + K.a1[w] * cj) + K.a2[w] * S;
        }
        double r = K.c1 * n[l] + K.c2 * neq;
        if constexpr (FMASK != 0) {
            // a1*((cx-ux)*fx + (cy-uy)*fy + (cz-uz)*fz) + 2*a2*(c.u)*(c.f)
            double t1 = 0.0;
            if constexpr (FMASK & 1) t1 = c.x > 0 ? gxp : (c.x < 0 ? gxm : gx0);
            if constexpr (FMASK & 2) {
                const double g = c.y > 0 ? gyp : (c.y < 0 ? gym : gy0);
                if constexpr (FMASK & 1) t1 = t1 + g;
                else t1 = g;
            }
            if constexpr (FMASK & 4) {
                const double g = c.z > 0 ? gzp : (c.z < 0 ? gzm : gz0);
                if constexpr (FMASK & 3) t1 = t1 + g;
                else t1 = g;
            }
            double T = K.a1[w] * t1;
            constexpr bool hasT2 = ((FMASK & 1) && c.x != 0) || ((FMASK & 2) && c.y != 0) ||
                                   ((FMASK & 4) && c.z != 0);
            if constexpr (hasT2) {
                const double cu = dotc<c.x, c.y, c.z>(ux, uy, uz);
                double cfl;
                if constexpr (UCF) cfl = a.cf[l];
                else cfl = dotc<(FMASK & 1) ? c.x : 0, (FMASK & 2) ? c.y : 0, (FMASK & 4) ? c.z : 0>(fx, fy, fz);
                T = T + K.two_a2[w] * cu * cfl;
            }
            r = r + K.c3 * T;
        }
        n[l] = r;
    });
}

// LBGPU_FP64_FUSED: density and flux from the pair sums and differences of opposite velocities
// (n_l + n_inv l, n_l - n_inv l): fewer FP64 additions than the term-by-term sums of moments19.
__device__ __forceinline__ void moments19_pairs(const double (&n)[Q], double fhx, double fhy, double fhz,
                                                double &rho, double &jx, double &jy, double &jz)
{
    double r = n[0], X = fhx, Y = fhy, Z = fhz;
    static_for<0, 9>([&](auto P) {
        constexpr int l = pair_l(decltype(P)::value);
        constexpr int li = inv(l);
        constexpr Vel c = vel(l);
        r = r + (n[l] + n[li]);
        const double d = n[l] - n[li];
        X = addsgn<c.x>(X, d);
        Y = addsgn<c.y>(Y, d);
        Z = addsgn<c.z>(Z, d);
    });
    rho = r;
    jx = X;
    jy = Y;
    jz = Z;
}

// LBGPU_FP64_FUSED: the same BGK + Guo collision regrouped per pair of opposite velocities
// (l, inv l), where c.j, c.u and c.F change sign and nothing else does:
//   n_l   <- c1 n_l   + (E + O),   n_inv <- c1 n_inv + (E - O)
//   E = c2 [a0 rho + a2 ((c.j)(c.u) - cs^2 j.u)] + c3 [2 a2 (c.u)(c.F) - a1 u.F]
//   O = c2 a1 (c.j) + c3 a1 (c.F)
// evaluated with fused multiply-adds and one reciprocal of rho: about half the FP64 operations
// of the operation-for-operation form, which bounds this kernel on GB300's FP64 pipe.  UCF: the
// uniform f_ext, with c3 a1 (c.F) and c3 2 a2 (c.F) taken per pair from a.kF / a.kT.
template <int FMASK, bool UCF>
__device__ __forceinline__ void collide_node_fused(double (&n)[Q], const double rho, const double jx,
                                                   const double jy, const double jz, const double fx,
                                                   const double fy, const double fz,
                                                   const FlowArgs64 &a)
{
    const LbConst64 &K = a.K;
    const double ir = 1.0 / rho;
    const double ux = jx * ir, uy = jy * ir, uz = jz * ir;
    const double ju = __fma_rn(jx, ux, __fma_rn(jy, uy, jz * uz));
    double base[3];
#pragma unroll
    for (int w = 0; w < 3; ++w) base[w] = __fma_rn(K.c2a0[w], rho, -(K.c2a2cs2[w] * ju));
    if constexpr (FMASK != 0) {
        const double uF = __fma_rn(ux, fx, __fma_rn(uy, fy, uz * fz));
#pragma unroll
        for (int w = 0; w < 3; ++w) base[w] = __fma_rn(-K.c3a1[w], uF, base[w]);
    }
    n[0] = __fma_rn(K.c1, n[0], base[0]);
    static_for<0, 9>([&](auto P) {
        constexpr int p = decltype(P)::value;
        constexpr int l = pair_l(p);
        constexpr int li = inv(l);
        constexpr Vel c = vel(l);
        constexpr int w = wclass(l);
        const double cj = dotc<c.x, c.y, c.z>(jx, jy, jz);
        const double cu = dotc<c.x, c.y, c.z>(ux, uy, uz);
        double A = __fma_rn(K.c2a2[w], cj * cu, base[w]);
        double B = K.c2a1[w] * cj;
        if constexpr (FMASK != 0) {
            double kT, kF;
            if constexpr (UCF) {
                kT = a.kT[p];
                kF = a.kF[p];
            } else {
                const double cF = dotc<c.x, c.y, c.z>(fx, fy, fz);
                kT = (K.c3 * K.two_a2[w]) * cF;
                kF = K.c3a1[w] * cF;
            }
            A = __fma_rn(kT, cu, A);
            B = B + kF;
        }
        n[l] = __fma_rn(K.c1, n[l], A + B);
        n[li] = __fma_rn(K.c1, n[li], A - B);
    });
}

struct Coords {
    int x, y, z;
    long long X[3], Y[3], Z[3];  // [c+1]: offset of coordinate (x - c) along each axis
};

__device__ __forceinline__ Coords coords_of(long long node, int lx, int ly, int lz)
{
    Coords k;
    const unsigned nd = (unsigned)node;
    k.x = (int)(nd % (unsigned)lx);
    const unsigned yz = nd / (unsigned)lx;
    k.y = (int)(yz % (unsigned)ly);
    k.z = (int)(yz / (unsigned)ly);
    const long long sx = 1, sy = lx, sz = (long long)lx * ly;
    // index [c+1] holds the coordinate of (x - c): c = -1 -> x+1, c = 0 -> x, c = 1 -> x-1
    k.X[0] = wrap_plus(k.x, lx) * sx;  k.X[1] = k.x * sx;  k.X[2] = wrap_minus(k.x, lx) * sx;
    k.Y[0] = wrap_plus(k.y, ly) * sy;  k.Y[1] = k.y * sy;  k.Y[2] = wrap_minus(k.y, ly) * sy;
    k.Z[0] = wrap_plus(k.z, lz) * sz;  k.Z[1] = k.z * sz;  k.Z[2] = wrap_minus(k.z, lz) * sz;
    return k;
}

// Pull the 19 populations of `node` from src with halfway bounce-back (equilibration.f90:204-243).
__device__ __forceinline__ void pull19(double (&n)[Q], const double *__restrict__ src,
                                       long long node, uint32_t m, const Coords &k, long long N)
{
    static_for<0, Q>([&](auto L) {
        constexpr int l = decltype(L)::value;
        constexpr Vel c = vel(l);
        if constexpr (l == 0) {
            n[0] = src[node];
        } else {
            const long long s = k.X[c.x + 1] + k.Y[c.y + 1] + k.Z[c.z + 1];
            n[l] = ((m >> l) & 1u) ? src[(long long)inv(l) * N + node] : src[(long long)l * N + s];
        }
    });
}

// density = SUM(n,4); j = F/2 + sum_l n_l c_l   (equilibration.f90:254,293-300)
__device__ __forceinline__ void moments19(const double (&n)[Q], double fhx, double fhy,
                                          double fhz, double &rho, double &jx, double &jy,
                                          double &jz)
{
    double r = n[0], X = fhx, Y = fhy, Z = fhz;
#pragma unroll
    for (int l = 1; l < Q; ++l) r = r + n[l];
    static_for<0, Q>([&](auto L) {
        constexpr int l = decltype(L)::value;
        constexpr Vel c = vel(l);
        X = addsgn<c.x>(X, n[l]);
        Y = addsgn<c.y>(Y, n[l]);
        Z = addsgn<c.z>(Z, n[l]);
    });
    rho = r;
    jx = X;
    jy = Y;
    jz = Z;
}

__device__ __forceinline__ unsigned check19(const double (&n)[Q])
{
    unsigned bad = 0;
#pragma unroll
    for (int l = 0; l < Q; ++l) {
        if (n[l] < 0.0) bad |= LBGPU_ERR_NEGATIVE_POPULATION;
        if (!(fabs(n[l]) <= DBL_MAX)) bad |= LBGPU_ERR_NONFINITE;
    }
    return bad;
}

__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max_nonneg(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ unsigned warp_or(unsigned v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v |= __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide max/or; result valid in thread 0.
__device__ __forceinline__ void block_max_or(double &err, unsigned &bad)
{
    __shared__ double se[BLOCK / 32];
    __shared__ unsigned sb[BLOCK / 32];
    err = warp_max(err);
    bad = warp_or(bad);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { se[wid] = err; sb[wid] = bad; }
    __syncthreads();
    if (wid == 0) {
        err = lane < BLOCK / 32 ? se[lane] : 0.0;
        bad = lane < BLOCK / 32 ? sb[lane] : 0u;
        err = warp_max(err);
        bad = warp_or(bad);
    }
}

// Reference phase machine, equilibration.f90:346-489 (non-compensated force), executed by the
// last block of a step once every block has contributed its |j - j_old| maximum.  Every exit
// leaves the block "advanced": parity names the buffer that the next step would read, and the
// buffer parity^1 holds the input of the exit step (exit_force_moment its moment force).
__device__ void control_step(FlowCtl *c, double *hist)
{
    const unsigned long long eb = atomicExch(&c->err_bits, 0ull);
    const double l2 = __longlong_as_double((long long)eb);
    c->blocks_done = 0;
    const unsigned st = atomicOr(&c->status, 0u);
    const int t = c->t;
    bool finish = false;
    if (st & (LBGPU_ERR_NEGATIVE_POPULATION | LBGPU_ERR_NONFINITE)) {
        finish = true;
    } else if (c->redo) {
        c->redo = 0;  // repeat of step t with the force switched on; its l2err is not used
    } else {
        if (hist && t - 1 < c->hist_cap) hist[t - 1] = l2;
        c->last_l2err = l2;
        const bool converged = (l2 <= c->target_error) && t > 2;
        if (converged) {
            if (!c->conv_without) c->conv_without = 1;
            else c->conv_with = 1;
            if (c->conv_without && c->conv_with) {
                finish = true;
            } else {
                // first convergence: f_ext acts from the collision of step t+1 on; that
                // collision already ran in this launch with the force off, so step t repeats.
                c->force_collide = 1;
                c->redo = 1;
                return;
            }
        }
    }
    c->exit_force_moment = c->force_moment;
    c->exit_step = t;
    c->parity ^= 1;
    c->force_moment = c->force_collide;
    c->t = t + 1;
    if (!finish && c->max_steps > 0 && c->t > c->max_steps) {
        finish = true;
        atomicOr(&c->status, (unsigned)LBGPU_ERR_STEP_CAP);
    }
    if (finish) c->done = 1;
}

template <int FMASK, bool FIELD, bool CHECK, bool REF, bool FUSED>
__global__ void __launch_bounds__(BLOCK) k_flow_step(const FlowArgs64 a)
{
    int parity = a.parity, fm = a.force_moment, fc = a.force_collide;
    if constexpr (REF) {
        const volatile FlowCtl *c = a.ctl;
        if (c->done) return;
        parity = c->parity;
        fm = c->force_moment;
        fc = c->force_collide;
    }
    const double *__restrict__ src = parity ? a.f1 : a.f0;
    double *__restrict__ dst = parity ? a.f0 : a.f1;
    const long long N = a.N;
    // one thread per fluid node through the list (every lane of a warp does work), else one per
    // lattice node
    const long long i = (long long)blockIdx.x * BLOCK + threadIdx.x;
    const long long node = a.fidx ? (i < a.Nf ? (long long)a.fidx[i] : N) : i;
    double err = 0.0;
    unsigned bad = 0;
    if (node < N) {
        const uint32_t m = a.mask[node];
        if (m & FLUID_BIT) {
            const Coords k = coords_of(node, a.lx, a.ly, a.lz);
            double n[Q];
            pull19(n, src, node, m, k, N);
            if constexpr (CHECK) bad = check19(n);
            double fx = 0.0, fy = 0.0, fz = 0.0;
            if constexpr (FIELD) {
                fx = a.Fx[node];
                fy = a.Fy[node];
                fz = a.Fz[node];
            } else {
                fx = a.F[0];
                fy = a.F[1];
                fz = a.F[2];
            }
            double rho, jx, jy, jz;
            if constexpr (FUSED) {
                if (fm) moments19_pairs(n, fx / 2.0, fy / 2.0, fz / 2.0, rho, jx, jy, jz);
                else moments19_pairs(n, 0.0, 0.0, 0.0, rho, jx, jy, jz);
            } else {
                if (fm) moments19(n, fx / 2.0, fy / 2.0, fz / 2.0, rho, jx, jy, jz);
                else moments19(n, 0.0, 0.0, 0.0, rho, jx, jy, jz);
            }
            if constexpr (CHECK) {
                const double ox = a.jx[node], oy = a.jy[node], oz = a.jz[node];
                err = max_nonneg(max_nonneg(fabs(jx - ox), fabs(jy - oy)), fabs(jz - oz));
                a.jx[node] = jx;
                a.jy[node] = jy;
                a.jz[node] = jz;
            }
            if constexpr (FUSED) {
                if (fc) collide_node_fused<FMASK, !FIELD>(n, rho, jx, jy, jz, fx, fy, fz, a);
                else collide_node_fused<0, true>(n, rho, jx, jy, jz, 0.0, 0.0, 0.0, a);
            } else {
                if (fc) collide_node<FMASK, !FIELD>(n, rho, jx, jy, jz, fx, fy, fz, a);
                else collide_node<0, true>(n, rho, jx, jy, jz, 0.0, 0.0, 0.0, a);
            }
#pragma unroll
            for (int l = 0; l < Q; ++l) dst[(long long)l * N + node] = n[l];
        }
    }
    if constexpr (CHECK) {
        block_max_or(err, bad);
        if (threadIdx.x == 0) {
            unsigned long long *eb = REF ? &a.ctl->err_bits : a.err_bits;
            unsigned *st = REF ? &a.ctl->status : a.status;
            atomic_max_nonneg(eb, err);
            if (bad) atomicOr(st, bad);
            if constexpr (REF) {
                __threadfence();
                const unsigned prev = atomicAdd(&a.ctl->blocks_done, 1u);
                if (prev == gridDim.x - 1) {
                    __threadfence();
                    control_step(a.ctl, a.hist);
                }
            }
        }
    }
}

// Collision only: pre-collision n in buffer `parity` (all fluid nodes), density and j from
// a.rho/a.j*, post-collision populations written to the other buffer; solid nodes copied.
template <int FMASK, bool FIELD>
__global__ void __launch_bounds__(BLOCK) k_collide(const FlowArgs64 a)
{
    const double *__restrict__ src = a.parity ? a.f1 : a.f0;
    double *__restrict__ dst = a.parity ? a.f0 : a.f1;
    const long long N = a.N;
    const long long node = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (node >= N) return;
    double n[Q];
#pragma unroll
    for (int l = 0; l < Q; ++l) n[l] = src[(long long)l * N + node];
    const uint32_t m = a.mask[node];
    if (m & FLUID_BIT) {
        double fx, fy, fz;
        if constexpr (FIELD) {
            fx = a.Fx[node];
            fy = a.Fy[node];
            fz = a.Fz[node];
        } else {
            fx = a.F[0];
            fy = a.F[1];
            fz = a.F[2];
        }
        if (a.force_collide)
            collide_node<FMASK, !FIELD>(n, a.rho[node], a.jx[node], a.jy[node], a.jz[node], fx, fy, fz, a);
        else
            collide_node<0, true>(n, a.rho[node], a.jx[node], a.jy[node], a.jz[node], 0.0, 0.0, 0.0, a);
    }
#pragma unroll
    for (int l = 0; l < Q; ++l) dst[(long long)l * N + node] = n[l];
}

// Bounce-back + streaming for every node (solid included): buffer `parity` -> nout.
__global__ void __launch_bounds__(BLOCK) k_stream(const FlowArgs64 a)
{
    const double *__restrict__ src = a.parity ? a.f1 : a.f0;
    const long long N = a.N;
    const long long node = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (node >= N) return;
    const uint32_t m = a.mask[node];
    const Coords k = coords_of(node, a.lx, a.ly, a.lz);
    double n[Q];
    pull19(n, src, node, m, k, N);
#pragma unroll
    for (int l = 0; l < Q; ++l) a.nout[(long long)l * N + node] = n[l];
}

// Moments of the populations in buffer `parity` at every node (equilibration.f90:248-343).
template <bool FIELD, bool PULL>
__global__ void __launch_bounds__(BLOCK) k_moments(const FlowArgs64 a)
{
    const double *__restrict__ src = a.parity ? a.f1 : a.f0;
    const long long N = a.N;
    const long long node = (long long)blockIdx.x * BLOCK + threadIdx.x;
    double err = 0.0;
    unsigned bad = 0;
    if (node < N) {
        const uint32_t m = a.mask[node];
        double n[Q];
        if constexpr (PULL) {
            const Coords k = coords_of(node, a.lx, a.ly, a.lz);
            pull19(n, src, node, m, k, N);
        } else {
#pragma unroll
            for (int l = 0; l < Q; ++l) n[l] = src[(long long)l * N + node];
        }
        bad = check19(n);
        double fx = 0.0, fy = 0.0, fz = 0.0;
        if constexpr (FIELD) {
            fx = a.Fx[node];
            fy = a.Fy[node];
            fz = a.Fz[node];
        } else if (a.force_moment && (m & FLUID_BIT)) {
            fx = a.F[0];
            fy = a.F[1];
            fz = a.F[2];
        }
        double rho, jx, jy, jz;
        moments19(n, fx / 2.0, fy / 2.0, fz / 2.0, rho, jx, jy, jz);
        const double ox = a.jx[node], oy = a.jy[node], oz = a.jz[node];
        err = max_nonneg(max_nonneg(fabs(jx - ox), fabs(jy - oy)), fabs(jz - oz));
        a.rho[node] = rho;
        a.jx[node] = jx;
        a.jy[node] = jy;
        a.jz[node] = jz;
        if (PULL && a.nout) {
#pragma unroll
            for (int l = 0; l < Q; ++l) a.nout[(long long)l * N + node] = n[l];
        }
    }
    block_max_or(err, bad);
    if (threadIdx.x == 0) {
        if (a.err_bits) atomic_max_nonneg(a.err_bits, err);
        if (bad && a.status) atomicOr(a.status, bad);
    }
}

// init_simu.f90:31-39 and equilibration.f90:75-80: raw n = w_l*rho into buffer `parity`.
__global__ void __launch_bounds__(BLOCK) k_init(const FlowArgs64 a, const double rho0)
{
    double *__restrict__ dst = a.parity ? a.f1 : a.f0;
    const long long N = a.N;
    const long long node = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (node >= N) return;
    const uint32_t m = a.mask[node];
    const double rho = (m & FLUID_BIT) ? rho0 : 0.0;
    a.rho[node] = rho;
    a.jx[node] = 0.0;
    a.jy[node] = 0.0;
    a.jz[node] = 0.0;
    static_for<0, Q>([&](auto L) {
        constexpr int l = decltype(L)::value;
        dst[(long long)l * N + node] = rho * a.K.a0[wclass(l)];
    });
}

unsigned grid_of(long long N) { return (unsigned)((N + BLOCK - 1) / BLOCK); }

template <bool FIELD, bool CHECK, bool REF, bool FUSED>
cudaError_t step_dispatch(const FlowArgs64 &a, int fmask, unsigned grid, cudaStream_t s)
{
    switch (fmask) {
    case 0: k_flow_step<0, FIELD, CHECK, REF, FUSED><<<grid, BLOCK, 0, s>>>(a); break;
    case 1: k_flow_step<1, FIELD, CHECK, REF, FUSED><<<grid, BLOCK, 0, s>>>(a); break;
    case 2: k_flow_step<2, FIELD, CHECK, REF, FUSED><<<grid, BLOCK, 0, s>>>(a); break;
    case 4: k_flow_step<4, FIELD, CHECK, REF, FUSED><<<grid, BLOCK, 0, s>>>(a); break;
    default: k_flow_step<7, FIELD, CHECK, REF, FUSED><<<grid, BLOCK, 0, s>>>(a); break;
    }
    return cudaGetLastError();
}

template <bool FUSED>
cudaError_t launch_step(const FlowArgs64 &a, int fmask, bool field, bool check, bool ref,
                        unsigned grid, cudaStream_t s)
{
    if (field) {
        // a per-node force field: every component may be non-zero
        if (ref) k_flow_step<7, true, true, true, FUSED><<<grid, BLOCK, 0, s>>>(a);
        else if (check) k_flow_step<7, true, true, false, FUSED><<<grid, BLOCK, 0, s>>>(a);
        else k_flow_step<7, true, false, false, FUSED><<<grid, BLOCK, 0, s>>>(a);
        return cudaGetLastError();
    }
    if (ref) return step_dispatch<false, true, true, FUSED>(a, fmask, grid, s);
    return check ? step_dispatch<false, true, false, FUSED>(a, fmask, grid, s)
                 : step_dispatch<false, false, false, FUSED>(a, fmask, grid, s);
}

}  // namespace

cudaError_t launch_flow_step_f64(const FlowArgs64 &a, int fmask, bool field, bool check,
                                 bool ref, unsigned grid, cudaStream_t s)
{
    if (!grid) grid = grid_of(a.fidx ? a.Nf : a.N);
    return a.fused ? launch_step<true>(a, fmask, field, check, ref, grid, s)
                   : launch_step<false>(a, fmask, field, check, ref, grid, s);
}

cudaError_t launch_collide_f64(const FlowArgs64 &a, int fmask, bool field, cudaStream_t s)
{
    const unsigned g = grid_of(a.N);
    if (field) {
        k_collide<7, true><<<g, BLOCK, 0, s>>>(a);
    } else {
        switch (fmask) {
        case 0: k_collide<0, false><<<g, BLOCK, 0, s>>>(a); break;
        case 1: k_collide<1, false><<<g, BLOCK, 0, s>>>(a); break;
        case 2: k_collide<2, false><<<g, BLOCK, 0, s>>>(a); break;
        case 4: k_collide<4, false><<<g, BLOCK, 0, s>>>(a); break;
        default: k_collide<7, false><<<g, BLOCK, 0, s>>>(a); break;
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_stream_f64(const FlowArgs64 &a, cudaStream_t s)
{
    k_stream<<<grid_of(a.N), BLOCK, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_moments_f64(const FlowArgs64 &a, bool field, cudaStream_t s)
{
    if (field) k_moments<true, false><<<grid_of(a.N), BLOCK, 0, s>>>(a);
    else k_moments<false, false><<<grid_of(a.N), BLOCK, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_finalize_f64(const FlowArgs64 &a, bool field, cudaStream_t s)
{
    if (field) k_moments<true, true><<<grid_of(a.N), BLOCK, 0, s>>>(a);
    else k_moments<false, true><<<grid_of(a.N), BLOCK, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_init_f64(const FlowArgs64 &a, double rho0, cudaStream_t s)
{
    k_init<<<grid_of(a.N), BLOCK, 0, s>>>(a, rho0);
    return cudaGetLastError();
}

}  // namespace lbg
