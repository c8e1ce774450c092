// flow_f32.cu -- FP32-deviation D3Q19 kernels.
//
// Populations are stored as single-precision deviations d_l = f_l - w_l*rho0 from the rest
// state of density rho0 (lb.in initialSolventDensity).  Since sum_l w_l c_l = 0 and
// w_l = w_inv(l), the deviations stream and bounce back exactly like f, the momentum is
// j = F/2 + sum_l d_l c_l, and BGK relaxes d the same way it relaxes f:
//   d*_l = (1-1/tau) d_l + (1/tau) dneq_l + (1-1/(2 tau)) T_l
//   dneq_l = w_l (rho - rho0) + a1_l (c.j) + a2_l ((c.j)(c.u) - cs^2 (j.u))
//   T_l    = a1_l (c.F - u.F) + 2 a2_l (c.u)(c.F)
// which is module_collision.f90:87-104 with the a2 double sum written as a contraction.
// Storing deviations keeps the ~7 significant digits of FP32 for the flow signal rather than
// for the rest density.  Moments handed back to the host are accumulated in FP64.
#include <algorithm>
#include <cfloat>
#include <type_traits>

#include "collide32.cuh"
#include "common.cuh"
#include "compact.cuh"
#include "flow.h"
#include "lbgpu.h"

namespace lbg {
namespace {

constexpr int BLOCK = 256;

struct Coords32 {
    int X[3], Y[3], Z[3];
};

__device__ __forceinline__ Coords32 coords32(unsigned node, int lx, int ly, int lz)
{
    Coords32 k;
    const int x = (int)(node % (unsigned)lx);
    const unsigned yz = node / (unsigned)lx;
    const int y = (int)(yz % (unsigned)ly), z = (int)(yz / (unsigned)ly);
    const int sy = lx, sz = lx * ly;
    k.X[0] = wrap_plus(x, lx);       k.X[1] = x;       k.X[2] = wrap_minus(x, lx);
    k.Y[0] = wrap_plus(y, ly) * sy;  k.Y[1] = y * sy;  k.Y[2] = wrap_minus(y, ly) * sy;
    k.Z[0] = wrap_plus(z, lz) * sz;  k.Z[1] = z * sz;  k.Z[2] = wrap_minus(z, lz) * sz;
    return k;
}

__device__ __forceinline__ void pull19f(float (&g)[Q], const float *__restrict__ src,
                                        unsigned node, uint32_t m, const Coords32 &k, size_t N)
{
    static_for<0, Q>([&](auto L) {
        constexpr int l = decltype(L)::value;
        constexpr Vel c = vel(l);
        if constexpr (l == 0) {
            g[0] = __ldg(src + node);
        } else {
            const unsigned s = (unsigned)(k.X[c.x + 1] + k.Y[c.y + 1] + k.Z[c.z + 1]);
            g[l] = ((m >> l) & 1u) ? __ldg(src + (size_t)inv(l) * N + node)
                                   : __ldg(src + (size_t)l * N + s);
        }
    });
}

// BGK + Guo forcing on deviations, split into the parts even and odd in c for each pair of
// opposite velocities (c.j, c.u and c.F change sign, everything else does not):
//   dneq = E +- O,  E = w drho + a2 ((c.j)(c.u) - cs^2 j.u),  O = a1 c.j
//   T    = TE +- TO, TE = 2 a2 (c.u)(c.F) - a1 u.F,           TO = a1 c.F
//   d*_l = c1 d_l + (c2 E + c3 TE) +- (c2 O + c3 TO)
// which halves the arithmetic of a direction-by-direction evaluation.  The per-pair force
// constants kF = c3 a1 c.F and kT = c3 2 a2 c.F are precomputed on the host.
// Fused pull-stream + moments + collision, FP32 deviations.
template <int FMASK>
__global__ void __launch_bounds__(BLOCK) k_step32(const FlowArgs32 a)
{
    const unsigned node = blockIdx.x * BLOCK + threadIdx.x;
    if (node >= (unsigned)a.N) return;
    const uint32_t m = __ldg(a.mask + node);
    if (!(m & FLUID_BIT)) return;
    const float *__restrict__ src = a.parity ? a.g1 : a.g0;
    float *__restrict__ dst = a.parity ? a.g0 : a.g1;
    const size_t N = (size_t)a.N;
    const Coords32 k = coords32(node, a.lx, a.ly, a.lz);
    float g[Q];
    pull19f(g, src, node, m, k, N);
    float drho = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
    static_for<0, Q>([&](auto L) {
        constexpr int l = decltype(L)::value;
        constexpr Vel c = vel(l);
        drho += g[l];
        if constexpr (c.x > 0) jx += g[l];
        if constexpr (c.x < 0) jx -= g[l];
        if constexpr (c.y > 0) jy += g[l];
        if constexpr (c.y < 0) jy -= g[l];
        if constexpr (c.z > 0) jz += g[l];
        if constexpr (c.z < 0) jz -= g[l];
    });
    if (FMASK && a.force_moment) {
        jx = __fadd_rn(jx, __fmul_rn(0.5f, a.F[0]));
        jy = __fadd_rn(jy, __fmul_rn(0.5f, a.F[1]));
        jz = __fadd_rn(jz, __fmul_rn(0.5f, a.F[2]));
    }
    collide_dev<FMASK>(g, drho, jx, jy, jz, a, a.force_collide != 0);
#pragma unroll
    for (int l = 0; l < Q; ++l) __stcs(dst + (size_t)l * N + node, g[l]);
}

// In-place AA-pattern step (one population buffer).  Even launches read the node's own 19
// slots and write the post-collision populations back into the opposite slots; odd launches
// read the 19 slots that stream into the node and write the post-collision populations into
// the slots they stream to.  In both cases a thread writes exactly the slots it read (so the
// update is race-free and every store lands on a sector that is already in L2), and after an
// odd launch the buffer holds the streamed populations in natural order again.
// Halfway bounce-back (equilibration.f90:204-243): a population whose source (or destination)
// across link l is of the other nature is read from (written to) the node itself.
// Only fluid nodes are stored (compact index i in lattice order), so the even launch reads and
// writes 19 dense arrays with no solid node in any sector, and the odd launch finds a fluid
// neighbour's slot through the row bitmask table.
// One AA update of the compact node i; odd launches take its flag word m and lattice index p.
// Off: type of the slot offsets of an odd launch (64-bit once Q*Nf reaches 2^32).
template <bool ODD, int FMASK, typename Off>
__device__ __forceinline__ void aa_update(const FlowArgs32 &a, unsigned i, uint32_t m, unsigned p,
                                          Off (*soff)[BLOCK], int fm, int fc)
{
    // Each thread writes only the slots it has read, and every value it writes depends on all
    // of them: no store can overtake a load, so the two views of the buffer may be restricted.
    const float *__restrict__ gin = a.g0;
    float *__restrict__ gout = a.g0;
    const unsigned Nf = a.Nf;  // even launches step pointers by Nf: 64-bit addresses throughout
    float f[Q];
    if constexpr (ODD) {
        aa_gather_offsets<Off>(a, i, p, m, [&](int l, Off o) {
            soff[l][threadIdx.x] = o;
            f[l] = __ldg(gin + o);
        });
    } else {
        const float *q = gin + i;
#pragma unroll
        for (int l = 0; l < Q; ++l, q += Nf) f[l] = __ldg(q);
    }
    float drho = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
    static_for<0, Q>([&](auto L) {
        constexpr int l = decltype(L)::value;
        constexpr Vel c = vel(l);
        drho += f[l];
        if constexpr (c.x > 0) jx += f[l];
        if constexpr (c.x < 0) jx -= f[l];
        if constexpr (c.y > 0) jy += f[l];
        if constexpr (c.y < 0) jy -= f[l];
        if constexpr (c.z > 0) jz += f[l];
        if constexpr (c.z < 0) jz -= f[l];
    });
    if (FMASK && fm) {
        jx = __fadd_rn(jx, __fmul_rn(0.5f, a.F[0]));
        jy = __fadd_rn(jy, __fmul_rn(0.5f, a.F[1]));
        jz = __fadd_rn(jz, __fmul_rn(0.5f, a.F[2]));
    }
    collide_dev<FMASK>(f, drho, jx, jy, jz, a, fc != 0);
    if constexpr (ODD) {
        // the population leaving along l goes to the slot the opposite direction was read from
#pragma unroll
        for (int l = 0; l < Q; ++l) gout[soff[inv(l)][threadIdx.x]] = f[l];
    } else {
        float *q = gout + i;
#pragma unroll
        for (int l = 0; l < Q; ++l, q += Nf) *q = f[inv(l)];
    }
}

// One compact node per thread (the odd launches' gather chain position -> neighbour index ->
// gather is covered by occupancy: the tuner in flow_f32_api.cu picks the launch bounds).  Odd
// launches walk the nodes in reverse block order, so each launch starts on the nodes the
// previous one wrote last, which are still in L2 (about 55 MB of the 323 MB of populations of the
// 192^3 benchmark box).  WIDE: 64-bit slot offsets, for boxes with Q*Nf >= 2^32.
template <bool ODD, int FMASK, int MINB, bool LOOP, bool WIDE = false>
__global__ void __launch_bounds__(BLOCK, MINB) k_aa32(const FlowArgs32 a)
{
    using Off = std::conditional_t<WIDE, unsigned long long, unsigned>;
    // odd launches: element index of the slot read for direction l, parked in shared memory
    // ([l][thread], conflict-free) so that it does not occupy registers across the collision
    __shared__ Off soff[ODD ? Q : 1][BLOCK];
    int fm = a.force_moment, fc = a.force_collide;
    if constexpr (LOOP) {   // reference loop: forces decided on the device; no-op after the exit
        const volatile FlowCtl *c = a.ctl;
        if (c->done) return;
        fm = c->aa_fm;
        fc = c->aa_fc;
    }
    const unsigned blk = ODD ? gridDim.x - 1 - blockIdx.x : blockIdx.x;
    const unsigned i = blk * BLOCK + threadIdx.x;   // compact (fluid) node
    if (i >= a.Nf) return;
    if constexpr (!ODD) aa_update<false, FMASK>(a, i, 0u, 0u, soff, fm, fc);
    else aa_update<true, FMASK>(a, i, __ldg(a.cmask + i), __ldg(a.cpos + i), soff, fm, fc);
}

// Control step of the FP32 reference loop, run by the last block of a check launch: the
// equilibration.f90:339-489 decisions (l2err history, convergence at l2err <= target_error and
// t > 2, f_ext from the next collision on at the first convergence, exit at the second) for the
// state S_t of step t.  Unlike the FP64 fused step no step is repeated: the decision is taken
// before the AA launch of step t+1 collides S_t.
__device__ void control_step32(FlowCtl *c, double *hist, int phase)
{
    const unsigned long long eb = atomicExch(&c->err_bits, 0ull);
    const double l2 = __longlong_as_double((long long)eb);
    c->blocks_done = 0;
    const unsigned st = atomicOr(&c->status, 0u);
    const int t = c->t;
    const int fm = c->check_fm;   // moment force of S_t
    bool finish = false;
    if (st & (LBGPU_ERR_NEGATIVE_POPULATION | LBGPU_ERR_NONFINITE)) {
        finish = true;
    } else {
        if (hist && t - 1 < c->hist_cap) hist[t - 1] = l2;
        c->last_l2err = l2;
        if (l2 <= c->target_error && t > 2) {
            if (!c->conv_without) {
                c->conv_without = 1;
                c->aa_fc = 1;          // f_ext acts from the collision of step t+1 on
            } else {
                c->conv_with = 1;
                finish = true;
            }
        }
    }
    c->exit_force_moment = fm;
    c->exit_step = t;
    c->exit_phase = phase;
    c->aa_fm = fm;
    c->check_fm = c->aa_fc;        // S_{t+1} = collide(S_t) with aa_fc: its moments carry it
    c->t = t + 1;
    if (!finish && c->max_steps > 0 && t >= c->max_steps) {
        finish = true;
        atomicOr(&c->status, (unsigned)LBGPU_ERR_STEP_CAP);
    }
    if (finish) c->done = 1;
}

// Check launch of the FP32 reference loop: FP64 moments of the AA state (natural order after
// an odd launch, SWAPPED after an even one) with the state's moment force, max |j - j_old| over
// the fluid nodes, n = d + w rho0 < 0 and non-finite tests, j stored for the next check; the
// last block runs the control step.  A no-op once the loop has exited.
template <bool SWAPPED, typename Off = unsigned>
__global__ void __launch_bounds__(BLOCK) k_aa_check32(const FlowArgs32 a)
{
    const volatile FlowCtl *vc = a.ctl;
    if (vc->done) return;
    const int fm = vc->check_fm;
    const unsigned i = blockIdx.x * BLOCK + threadIdx.x;
    double err = 0.0;
    unsigned bad = 0;
    if (i < a.Nf) {
        const unsigned c = a.cpos[i];
        const unsigned p = lattice_of(a, c);
        const float *g = a.g0;
        float f[Q];
        if constexpr (SWAPPED) {
            aa_gather_offsets<Off>(a, i, c, a.cmask[i], [&](int l, Off o) { f[l] = g[o]; });
        } else {
#pragma unroll
            for (int l = 0; l < Q; ++l) f[l] = g[(size_t)l * a.Nf + i];
        }
        double drho = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;
        static_for<0, Q>([&](auto L) {
            constexpr int l = decltype(L)::value;
            constexpr Vel v = vel(l);
            const double d = (double)f[l];
            drho += d;
            jx += v.x * d;
            jy += v.y * d;
            jz += v.z * d;
            const double n = d + a.w64[wclass(l)] * a.rho0d;
            if (n < 0.0) bad |= LBGPU_ERR_NEGATIVE_POPULATION;
            if (!(fabs(n) <= DBL_MAX)) bad |= LBGPU_ERR_NONFINITE;
        });
        if (fm) {
            jx += 0.5 * (double)a.F[0];
            jy += 0.5 * (double)a.F[1];
            jz += 0.5 * (double)a.F[2];
        }
        err = fmax(fmax(fabs(jx - a.jx[p]), fabs(jy - a.jy[p])), fabs(jz - a.jz[p]));
        a.jx[p] = jx;
        a.jy[p] = jy;
        a.jz[p] = jz;
        a.rho[p] = a.rho0d + drho;
    }
    // block max of err (IEEE order of non-negative doubles = order of their bits) and OR of bad
    __shared__ unsigned long long smax;
    __shared__ unsigned sbad;
    if (threadIdx.x == 0) {
        smax = 0ull;
        sbad = 0u;
    }
    __syncthreads();
    if (err > 0.0 || !(err == err)) atomicMax(&smax, (unsigned long long)__double_as_longlong(err == err ? err : INFINITY));
    if (bad) atomicOr(&sbad, bad);
    __syncthreads();
    if (threadIdx.x == 0) {
        FlowCtl *c = a.ctl;
        if (smax) atomicMax(&c->err_bits, smax);
        if (sbad) atomicOr(&c->status, sbad);
        __threadfence();
        if (atomicAdd(&c->blocks_done, 1u) == gridDim.x - 1) {
            __threadfence();
            control_step32(c, a.hist, SWAPPED ? 1 : 0);
        }
    }
}

// Moments (FP64) of an AA buffer: natural order after an odd launch (SWAPPED = false), or
// post-collision values in opposite slots after an even launch (SWAPPED = true, gathered as
// the next odd launch would).
template <bool SWAPPED, typename Off = unsigned>
__global__ void __launch_bounds__(BLOCK) k_aa_finalize32(const FlowArgs32 a)
{
    // solid nodes: the outputs were zeroed by the host (the reference's zeros)
    const unsigned i = blockIdx.x * BLOCK + threadIdx.x;
    if (i >= a.Nf) return;
    const unsigned c = a.cpos[i];
    const unsigned p = lattice_of(a, c);
    const size_t N = (size_t)a.N;
    const float *g = a.g0;
    float f[Q];
    if constexpr (SWAPPED) {
        aa_gather_offsets<Off>(a, i, c, a.cmask[i], [&](int l, Off o) { f[l] = g[o]; });
    } else {
#pragma unroll
        for (int l = 0; l < Q; ++l) f[l] = g[(size_t)l * a.Nf + i];
    }
    double drho = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;
    static_for<0, Q>([&](auto L) {
        constexpr int l = decltype(L)::value;
        constexpr Vel c = vel(l);
        const double v = (double)f[l];
        drho += v;
        jx += c.x * v;
        jy += c.y * v;
        jz += c.z * v;
        if (a.nout) a.nout[(size_t)l * N + p] = v + a.w64[wclass(l)] * a.rho0d;
    });
    if (a.force_moment) {
        jx += 0.5 * (double)a.F[0];
        jy += 0.5 * (double)a.F[1];
        jz += 0.5 * (double)a.F[2];
    }
    a.rho[p] = a.rho0d + drho;
    a.jx[p] = jx;
    a.jy[p] = jy;
    a.jz[p] = jz;
}

// cmask[i] = flag word of the compact node i
__global__ void __launch_bounds__(BLOCK) k_compact_mask(const FlowArgs32 a, uint32_t *cmask)
{
    const unsigned i = blockIdx.x * BLOCK + threadIdx.x;
    if (i < a.Nf) cmask[i] = a.mask[lattice_of(a, a.cpos[i])];
}

// d_l = n_l - w_l rho0 at the fluid nodes, into the AA layout
__global__ void __launch_bounds__(BLOCK) k_to_dev_compact32(const FlowArgs32 a, const double *__restrict__ n,
                                                            float *__restrict__ out)
{
    const size_t t = (size_t)blockIdx.x * BLOCK + threadIdx.x;
    const size_t Nf = a.Nf;
    if (t >= (size_t)Q * Nf) return;
    const int l = (int)(t / Nf);
    const unsigned i = (unsigned)(t - (size_t)l * Nf);
    out[t] = (float)(n[(size_t)l * (size_t)a.N + lattice_of(a, a.cpos[i])] - a.w64[wclass(l)] * a.rho0d);
}

// Zero deviations: the rest state rho = rho0, j = 0 (init_simu.f90:31-39 on fluid nodes).
__global__ void __launch_bounds__(BLOCK) k_init32(const FlowArgs32 a)
{
    const size_t i = (size_t)blockIdx.x * BLOCK + threadIdx.x;
    const size_t total = (size_t)Q * (a.g1 ? (size_t)a.N : (size_t)a.Nf);  // A/B or AA layout
    if (i < total) {
        a.g0[i] = 0.0f;
        if (a.g1) a.g1[i] = 0.0f;
    }
}

// Moments in FP64 (and optionally f = d + w rho0) of the populations in buffer `parity`
// (after streaming when PULL, else as stored); solid nodes report the reference's zeros.
template <bool PULL>
__global__ void __launch_bounds__(BLOCK) k_finalize32(const FlowArgs32 a)
{
    const unsigned node = blockIdx.x * BLOCK + threadIdx.x;
    if (node >= (unsigned)a.N) return;
    const uint32_t m = a.mask[node];
    const size_t N = (size_t)a.N;
    if (!(m & FLUID_BIT)) {
        a.rho[node] = 0.0;
        a.jx[node] = 0.0;
        a.jy[node] = 0.0;
        a.jz[node] = 0.0;
        if (a.nout)
            for (int l = 0; l < Q; ++l) a.nout[(size_t)l * N + node] = 0.0;
        return;
    }
    const float *__restrict__ src = a.parity ? a.g1 : a.g0;
    float g[Q];
    if constexpr (PULL) {
        const Coords32 k = coords32(node, a.lx, a.ly, a.lz);
        pull19f(g, src, node, m, k, N);
    } else {
#pragma unroll
        for (int l = 0; l < Q; ++l) g[l] = src[(size_t)l * N + node];
    }
    double drho = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;
    static_for<0, Q>([&](auto L) {
        constexpr int l = decltype(L)::value;
        constexpr Vel c = vel(l);
        const double v = (double)g[l];
        drho += v;
        jx += c.x * v;
        jy += c.y * v;
        jz += c.z * v;
        if (a.nout) a.nout[(size_t)l * N + node] = v + a.w64[wclass(l)] * a.rho0d;
    });
    if (a.force_moment) {
        jx += 0.5 * (double)a.F[0];
        jy += 0.5 * (double)a.F[1];
        jz += 0.5 * (double)a.F[2];
    }
    a.rho[node] = a.rho0d + drho;
    a.jx[node] = jx;
    a.jy[node] = jy;
    a.jz[node] = jz;
}

// Collision of raw deviations in buffer `parity` with the given FP64 density and flux
// (a.rho, a.j*), written to the other buffer (the start of a step, module_collision.f90:15).
template <int FMASK>
__global__ void __launch_bounds__(BLOCK) k_collide32(const FlowArgs32 a)
{
    const unsigned node = blockIdx.x * BLOCK + threadIdx.x;
    if (node >= (unsigned)a.N) return;
    const size_t N = (size_t)a.N;
    const float *__restrict__ src = a.parity ? a.g1 : a.g0;
    float *__restrict__ dst = a.parity ? a.g0 : a.g1;
    float g[Q];
#pragma unroll
    for (int l = 0; l < Q; ++l) g[l] = src[(size_t)l * N + node];
    if (a.mask[node] & FLUID_BIT) {
        const float drho = (float)(a.rho[node] - a.rho0d);
        collide_dev<FMASK>(g, drho, (float)a.jx[node], (float)a.jy[node], (float)a.jz[node], a,
                           a.force_collide != 0);
    }
#pragma unroll
    for (int l = 0; l < Q; ++l) dst[(size_t)l * N + node] = g[l];
}

// d_l = n_l - w_l rho0 for every node: FP64 host populations into FP32 deviations.
__global__ void __launch_bounds__(BLOCK) k_to_dev32(const FlowArgs32 a, const double *__restrict__ n,
                                                    float *__restrict__ out)
{
    const size_t i = (size_t)blockIdx.x * BLOCK + threadIdx.x;
    const size_t N = (size_t)a.N;
    if (i >= (size_t)Q * N) return;
    const int l = (int)(i / N);
    out[i] = (float)(n[i] - a.w64[wclass(l)] * a.rho0d);
}

}  // namespace

cudaError_t launch_to_dev32(const FlowArgs32 &a, const double *n, float *out, cudaStream_t s)
{
    const size_t total = (size_t)Q * (size_t)a.N;
    k_to_dev32<<<(unsigned)((total + BLOCK - 1) / BLOCK), BLOCK, 0, s>>>(a, n, out);
    return cudaGetLastError();
}

cudaError_t launch_collide_f32(const FlowArgs32 &a, cudaStream_t s)
{
    const unsigned grid = (unsigned)((a.N + BLOCK - 1) / BLOCK);
    int fm = (a.F[0] != 0.0f ? 1 : 0) | (a.F[1] != 0.0f ? 2 : 0) | (a.F[2] != 0.0f ? 4 : 0);
    if (fm) k_collide32<7><<<grid, BLOCK, 0, s>>>(a);
    else k_collide32<0><<<grid, BLOCK, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_flow_step_f32(const FlowArgs32 &a, unsigned grid, cudaStream_t s)
{
    if (!grid) grid = (unsigned)((a.N + BLOCK - 1) / BLOCK);
    const bool fm = a.F[0] != 0.0f || a.F[1] != 0.0f || a.F[2] != 0.0f;
    if (fm) k_step32<7><<<grid, BLOCK, 0, s>>>(a);
    else k_step32<0><<<grid, BLOCK, 0, s>>>(a);
    return cudaGetLastError();
}

// minb: resident blocks per SM the kernel is compiled for (3, 4, 5 or 6 -> at most 85, 64, 51
// or 42 registers per thread); picked per box by the tuner in flow_f32_api.cu.
template <int FM, int MINB>
static void aa_launch(const FlowArgs32 &a, bool odd, unsigned grid, cudaStream_t s)
{
    // the loop variant is a separate instantiation: the control-block read costs the hot
    // fixed-step kernel ~2 % when it is only a run-time branch
    if (odd && a.wide) {   // one variant: the tuner's choice applies to 32-bit offsets
        if (a.ctl) k_aa32<true, FM, 4, true, true><<<grid, BLOCK, 0, s>>>(a);
        else k_aa32<true, FM, 4, false, true><<<grid, BLOCK, 0, s>>>(a);
    } else if (a.ctl) {
        if (odd) k_aa32<true, FM, MINB, true><<<grid, BLOCK, 0, s>>>(a);
        else k_aa32<false, FM, MINB, true><<<grid, BLOCK, 0, s>>>(a);
    } else {
        if (odd) k_aa32<true, FM, MINB, false><<<grid, BLOCK, 0, s>>>(a);
        else k_aa32<false, FM, MINB, false><<<grid, BLOCK, 0, s>>>(a);
    }
}

template <int FM>
static void aa_launch_minb(const FlowArgs32 &a, bool odd, int minb, unsigned grid, cudaStream_t s)
{
    if (minb <= 3) aa_launch<FM, 3>(a, odd, grid, s);
    else if (minb == 4) aa_launch<FM, 4>(a, odd, grid, s);
    else if (minb == 5) aa_launch<FM, 5>(a, odd, grid, s);
    else aa_launch<FM, 6>(a, odd, grid, s);
}

cudaError_t launch_aa_step_f32(const FlowArgs32 &a, bool odd, cudaStream_t s)
{
    const unsigned grid = (a.Nf + BLOCK - 1) / BLOCK;
    // one instantiation: with the force switched off (force_collide = 0) the force terms are
    // skipped at run time
    aa_launch_minb<7>(a, odd, odd ? a.minb_odd : a.minb_even, grid, s);
    return cudaGetLastError();
}

cudaError_t launch_aa_check_f32(const FlowArgs32 &a, bool swapped, cudaStream_t s)
{
    const unsigned grid = (a.Nf + BLOCK - 1) / BLOCK;
    if (swapped && a.wide) k_aa_check32<true, unsigned long long><<<grid, BLOCK, 0, s>>>(a);
    else if (swapped) k_aa_check32<true><<<grid, BLOCK, 0, s>>>(a);
    else k_aa_check32<false><<<grid, BLOCK, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_compact_mask(const FlowArgs32 &a, uint32_t *cmask, cudaStream_t s)
{
    k_compact_mask<<<(a.Nf + BLOCK - 1) / BLOCK, BLOCK, 0, s>>>(a, cmask);
    return cudaGetLastError();
}

cudaError_t launch_to_dev_compact32(const FlowArgs32 &a, const double *n, float *out, cudaStream_t s)
{
    const size_t total = (size_t)Q * a.Nf;
    k_to_dev_compact32<<<(unsigned)((total + BLOCK - 1) / BLOCK), BLOCK, 0, s>>>(a, n, out);
    return cudaGetLastError();
}

cudaError_t launch_aa_finalize_f32(const FlowArgs32 &a, bool swapped, cudaStream_t s)
{
    const unsigned grid = (a.Nf + BLOCK - 1) / BLOCK;
    if (swapped && a.wide) k_aa_finalize32<true, unsigned long long><<<grid, BLOCK, 0, s>>>(a);
    else if (swapped) k_aa_finalize32<true><<<grid, BLOCK, 0, s>>>(a);
    else k_aa_finalize32<false><<<grid, BLOCK, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_init_f32(const FlowArgs32 &a, cudaStream_t s)
{
    const size_t total = (size_t)Q * (a.g1 ? (size_t)a.N : (size_t)a.Nf);
    k_init32<<<(unsigned)((total + BLOCK - 1) / BLOCK), BLOCK, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_finalize_f32(const FlowArgs32 &a, bool pull, cudaStream_t s)
{
    const unsigned grid = (unsigned)((a.N + BLOCK - 1) / BLOCK);
    if (pull) k_finalize32<true><<<grid, BLOCK, 0, s>>>(a);
    else k_finalize32<false><<<grid, BLOCK, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace lbg
