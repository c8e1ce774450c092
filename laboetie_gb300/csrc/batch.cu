// batch.cu -- kernels stepping many independent boxes together (FP32 deviations, in-place AA;
// FP32 tracer moment propagation).
//
// Large boxes are stored in the fluid-only layout of compact.cuh and cut into tiles of
// BATCH_BLOCK consecutive fluid nodes; one launch steps every tile of every large box in a phase
// (a tile never straddles two boxes, so a block reads one descriptor).  In the tracer phase,
// large boxes at least 32 x 8 wide run shared-memory slab tiles (mp_slab.cuh).  Small boxes are
// stepped by a persistent block each that loads the whole box (lattice layout) into shared
// memory, runs all the steps of a call there with a block barrier between steps, and writes it
// back: HBM is touched twice per call instead of twice per step.  Every box is updated by its
// own threads only and its arithmetic does not depend on which other boxes share the launch,
// so a box gives the same result alone and in any mix, and in either path.  The tracer is the
// single box's FP32 difference form (mp_f32.cu) with the same helpers and link order in every
// path, so a batched box's P is bit-identical to a single box's on the same flow moments.
#include <algorithm>
#include <cfloat>

#include "batch.h"
#include "collide32.cuh"
#include "common.cuh"
#include "compact.cuh"
#include "lbgpu.h"
#include "mp_slab.cuh"

namespace lbg {
namespace {

// Moments and collision of one node's 19 deviations (the same operations in every layout).
__device__ __forceinline__ void aa_collide(float (&f)[Q], const BatchInst &I)
{
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
    if (I.force) {
        jx = __fadd_rn(jx, __fmul_rn(0.5f, I.F[0]));
        jy = __fadd_rn(jy, __fmul_rn(0.5f, I.F[1]));
        jz = __fadd_rn(jz, __fmul_rn(0.5f, I.F[2]));
    }
    collide_dev<7>(f, drho, jx, jy, jz, I, I.force != 0);
}

// One AA update of one fluid node (x, y, z) of a box in the lattice layout whose populations
// start at g (global or shared).
template <bool ODD>
__device__ __forceinline__ void aa_node(float *g, unsigned N, unsigned node, uint32_t m, int x, int y,
                                        int z, const BatchInst &I)
{
    float f[Q];
    unsigned off[Q];
    if constexpr (ODD) {
        const int lx = I.lx, ly = I.ly, lz = I.lz;
        const int sy = lx, sz = lx * ly;
        // [c+1] = coordinate of (x - c)
        const int X[3] = {wrap_plus(x, lx), x, wrap_minus(x, lx)};
        const int Y[3] = {wrap_plus(y, ly) * sy, y * sy, wrap_minus(y, ly) * sy};
        const int Z[3] = {wrap_plus(z, lz) * sz, z * sz, wrap_minus(z, lz) * sz};
        static_for<0, Q>([&](auto L) {
            constexpr int l = decltype(L)::value;
            constexpr Vel c = vel(l);
            if constexpr (l == 0) {
                off[0] = node;
            } else {
                const unsigned s = (unsigned)(X[c.x + 1] + Y[c.y + 1] + Z[c.z + 1]);
                off[l] = ((m >> l) & 1u) ? (unsigned)l * N + node : (unsigned)inv(l) * N + s;
            }
        });
#pragma unroll
        for (int l = 0; l < Q; ++l) f[l] = g[off[l]];
    } else {
#pragma unroll
        for (int l = 0; l < Q; ++l) f[l] = g[(unsigned)l * N + node];
    }
    aa_collide(f, I);
    if constexpr (ODD) {
#pragma unroll
        for (int l = 0; l < Q; ++l) g[off[inv(l)]] = f[l];
    } else {
#pragma unroll
        for (int l = 0; l < Q; ++l) g[(unsigned)inv(l) * N + node] = f[l];
    }
}

// One AA update of the compact node i of a box in the fluid-only layout (compact.cuh).  A thread
// writes exactly the slots it read, so the read-only cache path is safe for the loads.  Odd
// launches park the slot of each direction in shared memory ([l][thread], conflict-free) so that
// it does not occupy registers across the collision.
template <bool ODD>
__device__ __forceinline__ void aa_node_compact(const BatchInst &I, unsigned i, unsigned (*soff)[BATCH_BLOCK])
{
    float *g = I.g;
    const unsigned Nf = I.Nf;
    float f[Q];
    if constexpr (ODD) {
        aa_gather_offsets(I, i, __ldg(I.cpos + i), __ldg(I.cmask + i), [&](int l, unsigned o) {
            soff[l][threadIdx.x] = o;
            f[l] = __ldg(g + o);
        });
    } else {
#pragma unroll
        for (int l = 0; l < Q; ++l) f[l] = __ldg(g + (unsigned)l * Nf + i);
    }
    aa_collide(f, I);
    if constexpr (ODD) {
#pragma unroll
        for (int l = 0; l < Q; ++l) g[soff[inv(l)][threadIdx.x]] = f[l];
    } else {
#pragma unroll
        for (int l = 0; l < Q; ++l) g[(unsigned)inv(l) * Nf + i] = f[l];
    }
}

// One tracer step at fluid node r in the difference form of mp_f32.cu:k_mp32, with the same
// operations in the same order (mp_slab.cuh helpers, mp_link_order), so a batched box's P is
// bit-identical to a single box's; with INIT, P(t=1), the node's fixed (u*, D) in aux and its
// VACF(0) term (before the 1/Pstat factor) instead (module_moment_propagation.f90:112-136).
// vt receives the node's VACF term in FP32 (a thread's few nodes; FP64 across threads, as the
// single box sums them).
template <bool INIT>
__device__ __forceinline__ void mp_node(const float4 *V, const float4 *Pn, float4 *Pnext,
                                        const float4 *An, float4 *Anext, float4 *aux, unsigned r, int x,
                                        int y, int z, uint32_t m, const BatchInst &I, float (&vt)[3],
                                        unsigned &bad)
{
    const int lx = I.lx, ly = I.ly, lz = I.lz;
    const int sy = lx, sz = lx * ly;
    // [c+1] = coordinate of (x + c), periodic
    const int X[3] = {wrap_minus(x, lx), x, wrap_plus(x, lx)};
    const int Y[3] = {wrap_minus(y, ly) * sy, y * sy, wrap_plus(y, ly) * sy};
    const int Z[3] = {wrap_minus(z, lz) * sz, z * sz, wrap_plus(z, lz) * sz};
    float4 vr = make_float4(0.f, 0.f, 0.f, 0.f), p = vr, ax = vr;
    if constexpr (INIT) {
        vr = V[r];
    } else {
        p = Pn[r];
        ax = __ldg(aux + r);   // issued before the links, so that its latency overlaps them
    }
    float frac = 1.0f, ux = 0.0f, uy = 0.0f, uz = 0.0f;
    float n0 = 0.0f, n1 = 0.0f, n2 = 0.0f;
    float v0 = 0.0f, v1 = 0.0f, v2 = 0.0f;
    double dnet = 0.0;
    static_for<1, Q>([&](auto L) {
        constexpr int l = INIT ? decltype(L)::value : mp_link_order(decltype(L)::value);
        constexpr Vel c = vel(l);
        constexpr int w = wclass(l);
        const unsigned rp = (unsigned)(X[c.x + 1] + Y[c.y + 1] + Z[c.z + 1]);
        const bool blocked = INIT && ((m >> inv(l)) & 1u);  // r + c_l is solid
        // a step takes the neighbour's fluid flag from V.w (V = 0 on a solid node): the bits of
        // mp32_scatter with no test of the link's bit
        const float4 vn = V[rp];
        const float spp = INIT ? mp32_scatter(blocked, I.a1[w], mp32_cdot<-c.x, -c.y, -c.z>(vn), I.lwh[w])
                               : mp32_scatter_flag(I.a1[w], mp32_cdot<-c.x, -c.y, -c.z>(vn), __fmul_rn(I.lwh[w], vn.w));
        if constexpr (INIT) {
            const float sp = mp32_scatter(blocked, I.a1[w], mp32_cdot<c.x, c.y, c.z>(vr), I.lwh[w]);
            frac -= sp;
            ux += c.x * sp;
            uy += c.y * sp;
            uz += c.z * sp;
            dnet += (double)spp - (double)sp;
            v0 += c.x * c.x * sp;
            v1 += c.y * c.y * sp;
            v2 += c.z * c.z * sp;
            n0 -= c.x * spp;
            n1 -= c.y * spp;
            n2 -= c.z * spp;
        } else {
            mp32_link(spp, Pn[rp], p, n0, n1, n2);
        }
    });
    if constexpr (INIT) {
        Pnext[r] = make_float4(n0 * I.bw, n1 * I.bw, n2 * I.bw, 0.0f);
        aux[r] = make_float4(ux, uy, uz, (float)dnet);
        vt[0] += v0;
        vt[1] += v1;
        vt[2] += v2;
        const float fr = (I.ads && (m & INTERFACIAL_BIT)) ? frac - I.ka : frac;
        if (fr < 1.1920929e-07f) bad = 1u;
    } else {
        vt[0] += p.x * ax.x;
        vt[1] += p.y * ax.y;
        vt[2] += p.z * ax.z;
        mp32_finish(p, ax.w, n0, n1, n2);
        if (I.ads && (m & INTERFACIAL_BIT)) Anext[r] = mp32_adsorb(p, An[r], I.ka, I.kd, I.one_minus_kd, n0, n1, n2);
        Pnext[r] = make_float4(n0, n1, n2, 0.0f);
    }
}

__device__ __forceinline__ void lattice_xyz(const BatchInst &I, unsigned r, int &x, int &y, int &z)
{
    x = (int)(r % (unsigned)I.lx);
    const unsigned yz = r / (unsigned)I.lx;
    y = (int)(yz % (unsigned)I.ly);
    z = (int)(yz / (unsigned)I.ly);
}

__device__ __forceinline__ unsigned compact_xyz(const BatchInst &I, unsigned c, int &x, int &y, int &z)
{
    x = (int)(c & ((1u << I.xbits) - 1u));
    y = (int)((c >> I.xbits) & ((1u << I.ybits) - 1u));
    z = (int)(c >> (I.xbits + I.ybits));
    return (unsigned)x + (unsigned)I.lx * ((unsigned)y + (unsigned)I.ly * (unsigned)z);
}

// Coordinates of the nodes threadIdx.x, threadIdx.x + T, threadIdx.x + 2T, ... of a box, advanced
// by additions (one division per walk instead of two per node).
struct NodeWalk {
    int x, y, z, dx, dy, dz, lx, ly;
    __device__ __forceinline__ NodeWalk(const BatchInst &I, unsigned T) : lx(I.lx), ly(I.ly)
    {
        lattice_xyz(I, threadIdx.x, x, y, z);
        dx = (int)(T % (unsigned)lx);
        const unsigned q = T / (unsigned)lx;
        dy = (int)(q % (unsigned)ly);
        dz = (int)(q / (unsigned)ly);
    }
    __device__ __forceinline__ void next()
    {
        x += dx;
        y += dy;
        z += dz;
        if (x >= lx) {
            x -= lx;
            ++y;
        }
        if (y >= ly) {
            y -= ly;
            ++z;
        }
    }
};

// Sum of 3 doubles over the block in a fixed order (lanes by shuffle tree, then warps in index
// order); valid in thread 0.  Any block size that is a multiple of 32, up to 1024.
__device__ __forceinline__ void block_sum3(double (&v)[3])
{
    __shared__ double sh[3][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[d] += __shfl_down_sync(0xffffffffu, v[d], o);
    __syncthreads();  // sh may still be read by a previous call
    if (lane == 0)
        for (int d = 0; d < 3; ++d) sh[d][wid] = v[d];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int d = 0; d < 3; ++d) {
            double s = 0.0;
            for (int k = 0; k < nw; ++k) s += sh[d][k];
            v[d] = s;
        }
}

__device__ __forceinline__ unsigned *status_word(const BatchInst &I)
{
    return reinterpret_cast<unsigned *>(I.tacc + (size_t)I.ntacc * BATCH_TACC);
}

// Velocity u = j/rho of a node in natural order (after an even number of AA launches); g holds
// the populations with stride N (lattice) or Nf (compact), node is the index in that layout.
__device__ __forceinline__ float3 node_velocity(const float *g, unsigned N, unsigned node,
                                                const BatchInst &I)
{
    float drho = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
    static_for<0, Q>([&](auto L) {
        constexpr int l = decltype(L)::value;
        constexpr Vel c = vel(l);
        const float v = g[(unsigned)l * N + node];
        drho += v;
        if constexpr (c.x > 0) jx += v;
        if constexpr (c.x < 0) jx -= v;
        if constexpr (c.y > 0) jy += v;
        if constexpr (c.y < 0) jy -= v;
        if constexpr (c.z > 0) jz += v;
        if constexpr (c.z < 0) jz -= v;
    });
    if (I.force) {
        jx += 0.5f * I.F[0];
        jy += 0.5f * I.F[1];
        jz += 0.5f * I.F[2];
    }
    const float ir = 1.0f / (I.rho0 + drho);
    return make_float3(jx * ir, jy * ir, jz * ir);
}

// max |u - u_prev| of a node as the bits of a non-negative float (a non-finite velocity gives
// the bits of a NaN, 0x7fffffff, which exceed those of every finite value and of infinity), so
// that maxima of the bits, unlike fmaxf, keep a NaN; u_prev := u.
__device__ __forceinline__ unsigned du_and_store(float4 *uprev, unsigned node, const float3 u)
{
    const float4 p = uprev[node];
    uprev[node] = make_float4(u.x, u.y, u.z, 0.0f);
    const float d = fmaxf(fmaxf(fabsf(u.x - p.x), fabsf(u.y - p.y)), fabsf(u.z - p.z));
    const bool finite = fabsf(u.x) <= FLT_MAX && fabsf(u.y) <= FLT_MAX && fabsf(u.z) <= FLT_MAX;
    return finite ? __float_as_uint(d) : 0x7fffffffu;
}

// FP64 density and flux of a fluid node in natural order (index in the box's layout).
__device__ __forceinline__ void node_moments64(const BatchInst &I, unsigned node, double &rho,
                                               double &X, double &Y, double &Z)
{
    const unsigned N = I.compact ? I.Nf : (unsigned)I.N;
    double d = 0.0;
    X = Y = Z = 0.0;
    static_for<0, Q>([&](auto L) {
        constexpr int l = decltype(L)::value;
        constexpr Vel c = vel(l);
        const double v = (double)I.g[(unsigned)l * N + node];
        d += v;
        X += c.x * v;
        Y += c.y * v;
        Z += c.z * v;
    });
    if (I.force) {
        X += 0.5 * (double)I.F[0];
        Y += 0.5 * (double)I.F[1];
        Z += 0.5 * (double)I.F[2];
    }
    rho = (double)I.rho0 + d;
}

// One AA launch over the tiles of the tiled boxes (always in the compact layout); MINB resident
// blocks per SM (3..6, picked by the tuner in batch_api.cu).  Odd launches take the tiles in
// reverse order, starting on the tiles the even launch wrote last (still in L2).
template <bool ODD, int MINB>
__global__ void __launch_bounds__(BATCH_BLOCK, MINB) k_batch_aa(const BatchInst *__restrict__ insts,
                                                                const BatchTile *__restrict__ tiles)
{
    __shared__ unsigned soff[ODD ? Q : 1][BATCH_BLOCK];
    const BatchTile t = tiles[ODD ? gridDim.x - 1 - blockIdx.x : blockIdx.x];
    const BatchInst &I = insts[t.inst];
    const unsigned i = (unsigned)t.start + threadIdx.x;
    if (i < I.Nf) aa_node_compact<ODD>(I, i, soff);
}

// Persistent work-list forms of the tiled launches: a fixed grid of blocks (a few per SM) claims
// `tpc` consecutive tiles at a time from an atomic ticket until the list is used up, so blocks
// that draw cheap tiles (few fluid lanes) take more of them.  The last block to leave resets the
// ticket for the next launch of the stream; no block ever waits on another.  Per tile the work
// is the one-block-per-tile launch's, so the results are bit-identical to it.
__device__ __forceinline__ bool claim_tiles(BatchTicket *tk, int ntiles, int tpc, unsigned &b0, unsigned &b1)
{
    __shared__ unsigned base;
    __syncthreads();   // every thread has read the previous claim
    if (threadIdx.x == 0) base = atomicAdd(&tk->next, (unsigned)tpc);
    __syncthreads();
    b0 = base;
    if (b0 >= (unsigned)ntiles) return false;
    b1 = min(b0 + (unsigned)tpc, (unsigned)ntiles);
    return true;
}

__device__ __forceinline__ void release_ticket(BatchTicket *tk)
{
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&tk->done, 1u) == gridDim.x - 1) {   // every block has made its last claim
            tk->next = 0u;
            tk->done = 0u;
            __threadfence();
        }
    }
}

template <bool ODD, int MINB>
__global__ void __launch_bounds__(BATCH_BLOCK, MINB) k_batch_aa_list(const BatchInst *__restrict__ insts,
                                                                     const BatchTile *__restrict__ tiles,
                                                                     int ntiles, int tpc, BatchTicket *tk)
{
    __shared__ unsigned soff[ODD ? Q : 1][BATCH_BLOCK];
    unsigned b0, b1;
    while (claim_tiles(tk, ntiles, tpc, b0, b1)) {
        for (unsigned k = b0; k < b1; ++k) {
            // odd launches walk the list from its end, as the one-block-per-tile form does
            const BatchTile t = tiles[ODD ? (unsigned)ntiles - 1u - k : k];
            const BatchInst &I = insts[t.inst];
            const unsigned i = (unsigned)t.start + threadIdx.x;
            if (i < I.Nf) aa_node_compact<ODD>(I, i, soff);
        }
    }
    release_ticket(tk);
}

// One tracer step of every tiled box in the tracer phase; with INIT (one box, the tiles of
// `inst` in order), the start of its tracer phase.  Each tile keeps its own running sums.
template <bool INIT>
__global__ void __launch_bounds__(BATCH_BLOCK) k_batch_mp(const BatchInst *__restrict__ insts,
                                                          const BatchTile *__restrict__ tiles,
                                                          int inst, int par)
{
    BatchTile t;
    if constexpr (INIT) t = BatchTile{inst, (int)blockIdx.x * BATCH_BLOCK};
    else t = tiles[blockIdx.x];
    const BatchInst &I = insts[t.inst];
    const unsigned k = (unsigned)t.start + threadIdx.x;   // node in the box's layout
    float vt32[3] = {0.0f, 0.0f, 0.0f};
    unsigned bad = 0;
    if (k < batch_units(I)) {
        uint32_t m;
        unsigned r;
        int x, y, z;
        if (I.compact) {
            m = __ldg(I.cmask + k);
            r = compact_xyz(I, __ldg(I.cpos + k), x, y, z);
        } else {
            m = __ldg(I.mask + k);
            r = k;
            lattice_xyz(I, r, x, y, z);
        }
        if (m & FLUID_BIT) {
            if constexpr (INIT) mp_node<true>(I.V, nullptr, I.P[0], nullptr, nullptr, I.aux, r, x, y, z, m, I, vt32, bad);
            else mp_node<false>(I.V, I.P[par], I.P[par ^ 1], I.A[par], I.A[par ^ 1], I.aux, r, x, y, z, m, I, vt32, bad);
        }
    }
    double vt[3] = {(double)vt32[0], (double)vt32[1], (double)vt32[2]};
    block_sum3(vt);
    if (threadIdx.x == 0) {
        double *acc = I.tacc + (size_t)(t.start / BATCH_BLOCK) * BATCH_TACC;
        if constexpr (INIT) {
            for (int d = 0; d < 3; ++d) {
                acc[d] = vt[d] * (double)I.bw;
                acc[3 + d] = 0.0;
                acc[6 + d] = 0.0;
            }
        } else {
            for (int d = 0; d < 3; ++d) {
                acc[3 + d] += vt[d];
                acc[6 + d] = vt[d];
            }
        }
    }
    if constexpr (INIT) {
        if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(status_word(I), (unsigned)LBGPU_ERR_FRACTION);
    }
}

// The work-list form of the tiled tracer step (see k_batch_aa_list).
__global__ void __launch_bounds__(BATCH_BLOCK) k_batch_mp_list(const BatchInst *__restrict__ insts,
                                                               const BatchTile *__restrict__ tiles,
                                                               int ntiles, int tpc, int par, BatchTicket *tk)
{
    unsigned b0, b1;
    while (claim_tiles(tk, ntiles, tpc, b0, b1)) {
        for (unsigned kt = b0; kt < b1; ++kt) {
            const BatchTile t = tiles[kt];
            const BatchInst &I = insts[t.inst];
            const unsigned k = (unsigned)t.start + threadIdx.x;
            float vt32[3] = {0.0f, 0.0f, 0.0f};
            unsigned bad = 0;
            if (k < batch_units(I)) {
                uint32_t m;
                unsigned r;
                int x, y, z;
                if (I.compact) {
                    m = __ldg(I.cmask + k);
                    r = compact_xyz(I, __ldg(I.cpos + k), x, y, z);
                } else {
                    m = __ldg(I.mask + k);
                    r = k;
                    lattice_xyz(I, r, x, y, z);
                }
                if (m & FLUID_BIT)
                    mp_node<false>(I.V, I.P[par], I.P[par ^ 1], I.A[par], I.A[par ^ 1], I.aux, r, x, y, z, m, I,
                                   vt32, bad);
            }
            double vt[3] = {(double)vt32[0], (double)vt32[1], (double)vt32[2]};
            block_sum3(vt);
            if (threadIdx.x == 0) {
                double *acc = I.tacc + (size_t)(t.start / BATCH_BLOCK) * BATCH_TACC;
                for (int d = 0; d < 3; ++d) {
                    acc[3 + d] += vt[d];
                    acc[6 + d] = vt[d];
                }
            }
        }
    }
    release_ticket(tk);
}

// One tracer step of the slab tiles of boxes in the tracer phase (mp_slab.cuh); each tile keeps
// its own running sums.
__global__ void __launch_bounds__(BATCH_BLOCK, 4) k_batch_mp_slab(const BatchInst *__restrict__ insts,
                                                               const BatchTile *__restrict__ tiles, int par)
{
    extern __shared__ float4 sm4[];
    const BatchTile t = tiles[blockIdx.x];
    const BatchInst &I = insts[t.inst];
    const int tiles_x = (I.lx + MPS_TX - 1) / MPS_TX, tiles_y = (I.ly + MPS_TY - 1) / MPS_TY;
    const int nxy = tiles_x * tiles_y;
    const int tile = t.start % nxy, chunk = t.start / nxy;
    const int z0 = chunk * I.zc;
    float vt[3] = {0.0f, 0.0f, 0.0f};
    mp_slab_planes(I, par, (tile % tiles_x) * MPS_TX, (tile / tiles_x) * MPS_TY, z0, min(z0 + I.zc, I.lz), sm4,
                   vt, nullptr, nullptr, nullptr);
    double v[3] = {(double)vt[0], (double)vt[1], (double)vt[2]};
    block_sum3(v);
    if (threadIdx.x == 0) {
        double *acc = I.tacc + (size_t)t.start * BATCH_TACC;
        for (int d = 0; d < 3; ++d) {
            acc[3 + d] += v[d];
            acc[6 + d] = v[d];
        }
    }
}

// V = (j + f_ext)/rho of one box from its flow state (FP64 moments rounded once to FP32).
__global__ void __launch_bounds__(BATCH_BLOCK) k_batch_mp_v(const BatchInst *__restrict__ insts, int inst)
{
    // compact boxes: V stays zero on solid nodes (the allocation is zeroed when the box is added)
    const BatchInst &I = insts[inst];
    const unsigned k = blockIdx.x * BATCH_BLOCK + threadIdx.x;
    if (k >= batch_units(I)) return;
    const unsigned r = I.compact ? lattice_of(I, I.cpos[k]) : k;
    if (!I.compact && !(I.mask[k] & FLUID_BIT)) {
        I.V[r] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    double rho, J[3];
    node_moments64(I, k, rho, J[0], J[1], J[2]);
    float o[3];
    for (int d = 0; d < 3; ++d) o[d] = (float)((J[d] + I.tfext[d]) / rho);
    I.V[r] = make_float4(o[0], o[1], o[2], 1.0f);   // w: fluid flag (the slab step's link mask)
}

// One block per small box in the flow phase, for all the steps of a call: load, nsteps steps in
// shared memory, optional convergence check, store.  nsteps is even, so a box ends in natural
// order.  (The tracer phase is a kernel of its own, so that neither phase's register allocation
// is set by the other's code.  A box's shared memory keeps one block per SM, so both kernels are
// bounded for one resident block: the compiler may then use up to 128 registers for 512 threads,
// which lets it issue more of a node's shared-memory reads ahead.)
template <int MAXT>
__global__ void __launch_bounds__(MAXT, 1) k_batch_smem_flow(const BatchInst *__restrict__ insts,
                                                          const int *__restrict__ list, int nsteps,
                                                          int check, unsigned *du_out)
{
    extern __shared__ float4 sm4[];
    const int id = list[blockIdx.x];
    const BatchInst &I = insts[id];
    const unsigned N = (unsigned)I.N;
    const unsigned T = blockDim.x;
    {
        float *g = reinterpret_cast<float *>(sm4);
        uint32_t *msk = reinterpret_cast<uint32_t *>(g + (size_t)Q * N);
        for (unsigned i = threadIdx.x; i < (unsigned)Q * N; i += T) g[i] = I.g[i];
        for (unsigned i = threadIdx.x; i < N; i += T) msk[i] = I.mask[i];
        __syncthreads();
        for (int s = 0; s < nsteps; ++s) {
            NodeWalk w(I, T);
            for (unsigned node = threadIdx.x; node < N; node += T, w.next()) {
                const uint32_t m = msk[node];
                if (!(m & FLUID_BIT)) continue;
                if (s & 1) aa_node<true>(g, N, node, m, w.x, w.y, w.z, I);
                else aa_node<false>(g, N, node, m, w.x, w.y, w.z, I);
            }
            __syncthreads();
        }
        if (check) {
            unsigned du = 0u;
            for (unsigned node = threadIdx.x; node < N; node += T)
                if (msk[node] & FLUID_BIT) du = max(du, du_and_store(I.uprev, node, node_velocity(g, N, node, I)));
            for (int o = 16; o > 0; o >>= 1) du = max(du, __shfl_xor_sync(0xffffffffu, du, o));
            if ((threadIdx.x & 31) == 0) atomicMax(du_out + id, du);
        }
        for (unsigned i = threadIdx.x; i < (unsigned)Q * N; i += T) I.g[i] = g[i];
    }
}

// One block per small box in the tracer phase, for all the steps of a call: load V, P (and A)
// into shared memory, nsteps steps, store; nsteps is even, so P(now) ends in P[0].  The fixed
// (u*, D) of the nodes stay in global memory (read once per node and step, from L2), which keeps
// a 1 x 50 x 50 cell with adsorption within shared memory.
template <int MAXT>
__global__ void __launch_bounds__(MAXT, 1) k_batch_smem_mp(const BatchInst *__restrict__ insts,
                                                        const int *__restrict__ list, int nsteps)
{
    extern __shared__ float4 sm4[];
    const int id = list[blockIdx.x];
    const BatchInst &I = insts[id];
    const unsigned N = (unsigned)I.N;
    const unsigned T = blockDim.x;
    const int ads = I.ads;
    float4 *V = sm4, *P0 = sm4 + N, *P1 = sm4 + 2 * (size_t)N;
    float4 *A0 = ads ? sm4 + 3 * (size_t)N : nullptr, *A1 = ads ? sm4 + 4 * (size_t)N : nullptr;
    uint32_t *msk = reinterpret_cast<uint32_t *>(sm4 + (size_t)(ads ? 5 : 3) * N);
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    for (unsigned i = threadIdx.x; i < N; i += T) {
        V[i] = I.V[i];
        P0[i] = I.P[0][i];
        P1[i] = zero;
        if (ads) {
            A0[i] = I.A[0][i];
            A1[i] = zero;
        }
        msk[i] = I.mask[i];
    }
    __syncthreads();
    // this thread's VACF terms: summed over the call's steps in FP64, and the last step's; the
    // block adds them up once, after the last step
    double sum[3] = {0.0, 0.0, 0.0};
    float last32[3] = {0.0f, 0.0f, 0.0f};
    unsigned bad = 0;
    for (int s = 0; s < nsteps; ++s) {
        const bool odd = s & 1;
        const float4 *Pn = odd ? P1 : P0, *An = odd ? A1 : A0;
        float4 *Px = odd ? P0 : P1, *Ax = odd ? A0 : A1;
        float vt32[3] = {0.0f, 0.0f, 0.0f};
        NodeWalk w(I, T);
        for (unsigned node = threadIdx.x; node < N; node += T, w.next()) {
            const uint32_t m = msk[node];
            if (m & FLUID_BIT) mp_node<false>(V, Pn, Px, An, Ax, I.aux, node, w.x, w.y, w.z, m, I, vt32, bad);
        }
        for (int d = 0; d < 3; ++d) {
            sum[d] += (double)vt32[d];
            last32[d] = vt32[d];
        }
        __syncthreads();   // this step's P before the next step reads it
    }
    double last[3] = {(double)last32[0], (double)last32[1], (double)last32[2]};
    block_sum3(sum);
    block_sum3(last);
    __syncthreads();
    for (unsigned i = threadIdx.x; i < N; i += T) {
        I.P[0][i] = P0[i];
        if (ads) I.A[0][i] = A0[i];
    }
    if (threadIdx.x == 0 && nsteps > 0)
        for (int d = 0; d < 3; ++d) {
            I.tacc[3 + d] += sum[d];
            I.tacc[6 + d] = last[d];
        }
}

// Convergence check of the tiled boxes (natural order): du_out[box] = max |u - u_prev|.
__global__ void __launch_bounds__(BATCH_BLOCK) k_batch_check(const BatchInst *__restrict__ insts,
                                                             const BatchTile *__restrict__ tiles,
                                                             unsigned *du_out)
{
    const BatchTile t = tiles[blockIdx.x];
    const BatchInst &I = insts[t.inst];
    const unsigned node = (unsigned)t.start + threadIdx.x;
    unsigned du = 0u;   // tiled boxes are in the compact layout: every node is fluid
    if (node < I.Nf) du = du_and_store(I.uprev, node, node_velocity(I.g, I.Nf, node, I));
    for (int o = 16; o > 0; o >>= 1) du = max(du, __shfl_xor_sync(0xffffffffu, du, o));
    if ((threadIdx.x & 31) == 0) atomicMax(du_out + t.inst, du);
}

// Density and flux (FP64) of one box in natural order; solid nodes report zeros.
__global__ void __launch_bounds__(BATCH_BLOCK) k_batch_moments(const BatchInst *__restrict__ insts, int inst,
                                                               double *rho, double *jx, double *jy,
                                                               double *jz)
{
    const BatchInst &I = insts[inst];
    const unsigned k = blockIdx.x * BATCH_BLOCK + threadIdx.x;
    if (k >= batch_units(I)) return;
    if (I.compact) {
        const unsigned r = lattice_of(I, I.cpos[k]);
        node_moments64(I, k, rho[r], jx[r], jy[r], jz[r]);
        return;
    }
    if (!(I.mask[k] & FLUID_BIT)) {
        rho[k] = jx[k] = jy[k] = jz[k] = 0.0;
        return;
    }
    node_moments64(I, k, rho[k], jx[k], jy[k], jz[k]);
}

}  // namespace

cudaError_t batch_configure(int max_smem_bytes)
{
    const void *k[4] = {(const void *)k_batch_smem_flow<512>, (const void *)k_batch_smem_flow<1024>,
                        (const void *)k_batch_smem_mp<512>, (const void *)k_batch_smem_mp<1024>};
    for (const void *f : k) {
        const cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem_bytes);
        if (e != cudaSuccess) return e;
    }
    return cudaFuncSetAttribute(k_batch_mp_slab, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)MPS_SMEM);
}

template <int MINB>
static void batch_aa(const BatchInst *insts, const BatchTile *tiles, int ntiles, bool odd, cudaStream_t s)
{
    if (odd) k_batch_aa<true, MINB><<<ntiles, BATCH_BLOCK, 0, s>>>(insts, tiles);
    else k_batch_aa<false, MINB><<<ntiles, BATCH_BLOCK, 0, s>>>(insts, tiles);
}

cudaError_t launch_batch_aa(const BatchInst *insts, const BatchTile *tiles, int ntiles, bool odd, int minb,
                            cudaStream_t s)
{
    if (ntiles <= 0) return cudaSuccess;
    if (minb <= 3) batch_aa<3>(insts, tiles, ntiles, odd, s);
    else if (minb == 4) batch_aa<4>(insts, tiles, ntiles, odd, s);
    else if (minb == 5) batch_aa<5>(insts, tiles, ntiles, odd, s);
    else batch_aa<6>(insts, tiles, ntiles, odd, s);
    return cudaGetLastError();
}

cudaError_t launch_batch_mp(const BatchInst *insts, const BatchTile *tiles, int ntiles, int par,
                            cudaStream_t s)
{
    if (ntiles <= 0) return cudaSuccess;
    k_batch_mp<false><<<ntiles, BATCH_BLOCK, 0, s>>>(insts, tiles, 0, par);
    return cudaGetLastError();
}

template <int MINB>
static void batch_aa_list(const BatchInst *insts, const BatchTile *tiles, int ntiles, bool odd, int grid,
                          int tpc, BatchTicket *tk, cudaStream_t s)
{
    if (odd) k_batch_aa_list<true, MINB><<<grid, BATCH_BLOCK, 0, s>>>(insts, tiles, ntiles, tpc, tk);
    else k_batch_aa_list<false, MINB><<<grid, BATCH_BLOCK, 0, s>>>(insts, tiles, ntiles, tpc, tk);
}

cudaError_t launch_batch_aa_list(const BatchInst *insts, const BatchTile *tiles, int ntiles, bool odd, int minb,
                                 int grid, int tpc, BatchTicket *tk, cudaStream_t s)
{
    if (ntiles <= 0) return cudaSuccess;
    grid = std::max(1, std::min(grid, (ntiles + tpc - 1) / tpc));
    if (minb <= 3) batch_aa_list<3>(insts, tiles, ntiles, odd, grid, tpc, tk, s);
    else if (minb == 4) batch_aa_list<4>(insts, tiles, ntiles, odd, grid, tpc, tk, s);
    else if (minb == 5) batch_aa_list<5>(insts, tiles, ntiles, odd, grid, tpc, tk, s);
    else batch_aa_list<6>(insts, tiles, ntiles, odd, grid, tpc, tk, s);
    return cudaGetLastError();
}

cudaError_t launch_batch_mp_list(const BatchInst *insts, const BatchTile *tiles, int ntiles, int par, int grid,
                                 int tpc, BatchTicket *tk, cudaStream_t s)
{
    if (ntiles <= 0) return cudaSuccess;
    grid = std::max(1, std::min(grid, (ntiles + tpc - 1) / tpc));
    k_batch_mp_list<<<grid, BATCH_BLOCK, 0, s>>>(insts, tiles, ntiles, tpc, par, tk);
    return cudaGetLastError();
}

cudaError_t launch_batch_mp_slab(const BatchInst *insts, const BatchTile *tiles, int ntiles, int par,
                                 cudaStream_t s)
{
    if (ntiles <= 0) return cudaSuccess;
    k_batch_mp_slab<<<ntiles, BATCH_BLOCK, MPS_SMEM, s>>>(insts, tiles, par);
    return cudaGetLastError();
}

cudaError_t launch_batch_mp_start(const BatchInst *insts, int inst, unsigned units, cudaStream_t s)
{
    const unsigned grid = (units + BATCH_BLOCK - 1) / BATCH_BLOCK;
    k_batch_mp_v<<<grid, BATCH_BLOCK, 0, s>>>(insts, inst);
    k_batch_mp<true><<<grid, BATCH_BLOCK, 0, s>>>(insts, nullptr, inst, 0);
    return cudaGetLastError();
}

cudaError_t launch_batch_smem(const BatchInst *insts, const int *list, int nflow, int nmp, int nsteps,
                              bool check, unsigned *du, int bytes_flow, int bytes_mp, int threads,
                              cudaStream_t s)
{
    // up to 512 threads: the variants with up to 128 registers per thread; 1024: at most 64
    const int c = check ? 1 : 0;
    if (nflow > 0) {
        if (threads <= 512) k_batch_smem_flow<512><<<nflow, threads, bytes_flow, s>>>(insts, list, nsteps, c, du);
        else k_batch_smem_flow<1024><<<nflow, 1024, bytes_flow, s>>>(insts, list, nsteps, c, du);
    }
    if (nmp > 0) {
        if (threads <= 512) k_batch_smem_mp<512><<<nmp, threads, bytes_mp, s>>>(insts, list + nflow, nsteps);
        else k_batch_smem_mp<1024><<<nmp, 1024, bytes_mp, s>>>(insts, list + nflow, nsteps);
    }
    return cudaGetLastError();
}

cudaError_t launch_batch_check(const BatchInst *insts, const BatchTile *tiles, int ntiles,
                               unsigned *du, cudaStream_t s)
{
    if (ntiles <= 0) return cudaSuccess;
    k_batch_check<<<ntiles, BATCH_BLOCK, 0, s>>>(insts, tiles, du);
    return cudaGetLastError();
}

cudaError_t launch_batch_moments(const BatchInst *insts, int inst, unsigned units, double *rho, double *jx,
                                 double *jy, double *jz, cudaStream_t s)
{
    k_batch_moments<<<(units + BATCH_BLOCK - 1) / BATCH_BLOCK, BATCH_BLOCK, 0, s>>>(insts, inst, rho, jx, jy, jz);
    return cudaGetLastError();
}

}  // namespace lbg
