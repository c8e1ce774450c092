// mp_slab.cuh -- FP32 tracer step of a column tile with V and P staged in shared memory.
//
// A block steps the nodes (x0..x0+31, y0..y0+7, z0..z1-1) of a box with lx >= 32, ly >= 8,
// lz >= 3.  A ring of 4 planes of V and P with a one-node halo is filled by asynchronous copies
// (or bulk tensor copies) ahead of use, so the neighbour reads are shared-memory reads and every
// V and P value is fetched from L2/HBM about 1.3 times (halo) per step; the column's flag words
// (and the node's fixed (u*, D)) are loaded into registers ahead of use, and an interfacial
// node's adsorbed part is copied into a slot of the thread's own two steps before it finishes.
// One block barrier per plane.  mp_slab_planes is the difference form of mp_f32.cu:k_mp32 (same operations in the same
// order, so P is bit-identical) visiting each plane once, for single boxes and batched ones alike.
// The argument struct provides V (its w component: the node's fluid flag, 1 or 0), P[2], A[2],
// aux, mask, lx, ly, lz, ads, ka, kd, one_minus_kd, a1[3], lwh[3], wait_ns, skip_copies.
#pragma once

#include <type_traits>

#include "common.cuh"
#include "cpasync.cuh"
#include "lbgpu.h"
#include "mp.h"
#include "tma.cuh"

namespace lbg {

constexpr int SHX = MPS_TX + 2, SHY = MPS_TY + 2, SPL = SHX * SHY;  // a plane with its halo
// plane stride in float4: 344 = SPL rounded up to 128 bytes (a bulk tensor copy lands on a
// 128-byte boundary)
constexpr int SPLP = (SPL * 16 + 127) / 128 * 8;
constexpr unsigned MPS_TMA_BYTES = SPL * 16;                        // one plane of V or of P
// 4 planes of V and of P, 4 mbarriers, two adsorbed-part slots per thread, and slack to align the
// ring to 128 bytes
constexpr size_t MPS_SMEM = 128 + sizeof(float4) * 8 * SPLP + 4 * sizeof(uint64_t) + 2 * MP_BLOCK * sizeof(float4);

// Scattering probability of a link, a1 (c.V) + lambda w / 2 rounded once, or 0 across a
// bounce-back link (blocked).  The reference multiplies by a 0/1 factor instead; the sums it
// enters are the same, as a product with -0 and with +0 adds nothing to a sum that is never -0.
__device__ __forceinline__ float mp32_scatter(bool blocked, float a1, float cv, float lwh)
{
    return blocked ? 0.0f : __fmaf_rn(a1, cv, lwh);
}

// The same from the neighbour's staged record: lwhf = (lambda w / 2) * (its fluid flag, 1 or 0)
// and V = 0 on a solid neighbour, so a blocked link gives fma(a1, 0, 0) = 0 and an open one
// fma(a1, c.V, lambda w / 2): the bits of mp32_scatter with no test of the link's bit.
__device__ __forceinline__ float mp32_scatter_flag(float a1, float cv, float lwhf)
{
    return __fmaf_rn(a1, cv, lwhf);
}

// One incoming link of an FP32 step: n += sp_in (P(r + c_l) - P(r)).
__device__ __forceinline__ void mp32_link(float spp, const float4 &pn, const float4 &p, float &n0,
                                          float &n1, float &n2)
{
    n0 = __fmaf_rn(spp, __fsub_rn(pn.x, p.x), n0);
    n1 = __fmaf_rn(spp, __fsub_rn(pn.y, p.y), n1);
    n2 = __fmaf_rn(spp, __fsub_rn(pn.z, p.z), n2);
}

// End of an FP32 step: n = P(r) + (n + D P(r)), D = sum sp_in - sum sp_out of the node.
__device__ __forceinline__ void mp32_finish(const float4 &p, float D, float &n0, float &n1, float &n2)
{
    n0 = __fadd_rn(p.x, __fmaf_rn(D, p.x, n0));
    n1 = __fadd_rn(p.y, __fmaf_rn(D, p.y, n1));
    n2 = __fadd_rn(p.z, __fmaf_rn(D, p.z, n2));
}

// Adsorption exchange at an interfacial fluid node (module_moment_propagation.f90:239-246), after
// mp32_finish: n += kd A - ka P; returns A_next = (1 - kd) A + ka P.  Fused operations in a fixed
// order, so every kernel that calls it rounds alike.
__device__ __forceinline__ float4 mp32_adsorb(const float4 &p, const float4 &qa, float ka, float kd,
                                              float one_minus_kd, float &n0, float &n1, float &n2)
{
    n0 = __fmaf_rn(qa.x, kd, __fmaf_rn(-ka, p.x, n0));
    n1 = __fmaf_rn(qa.y, kd, __fmaf_rn(-ka, p.y, n1));
    n2 = __fmaf_rn(qa.z, kd, __fmaf_rn(-ka, p.z, n2));
    return make_float4(__fmaf_rn(p.x, ka, __fmul_rn(qa.x, one_minus_kd)),
                       __fmaf_rn(p.y, ka, __fmul_rn(qa.y, one_minus_kd)),
                       __fmaf_rn(p.z, ka, __fmul_rn(qa.z, one_minus_kd)), 0.0f);
}

// c.V of a link (x, y, z summed in that order, signs folded): the one definition every FP32 tracer
// kernel uses, so that their scattering probabilities round alike.  The first term is taken as it
// is (not added to 0), which differs from 0 + term only in the sign of a zero; c.V enters only
// fma(a1, c.V, lwh) with lwh >= +0, where a zero of either sign gives the same result, so the
// scattering probabilities keep their bits and an axis link costs no addition.
template <int CX, int CY, int CZ>
__device__ __forceinline__ float mp32_cdot(const float4 &v)
{
    static_assert(CX != 0 || CY != 0 || CZ != 0, "rest link");
    constexpr int first = CX != 0 ? 0 : (CY != 0 ? 1 : 2);
    float s = first == 0 ? (CX > 0 ? v.x : -v.x) : (first == 1 ? (CY > 0 ? v.y : -v.y) : (CZ > 0 ? v.z : -v.z));
    if constexpr (first < 1 && CY > 0) s += v.y;
    if constexpr (first < 1 && CY < 0) s -= v.y;
    if constexpr (first < 2 && CZ > 0) s += v.z;
    if constexpr (first < 2 && CZ < 0) s -= v.z;
    return s;
}

// Link of velocity (dx, dy, dz).
__host__ __device__ constexpr int link_of(int dx, int dy, int dz)
{
    for (int l = 0; l < Q; ++l)
        if (vel(l).x == dx && vel(l).y == dy && vel(l).z == dz) return l;
    return -1;
}

// The nine points (dx, dy) of a column's neighbourhood in one plane, in the order the plane-wise
// step visits them.  Restricted to the links of one z offset this is ascending link order.
__host__ __device__ constexpr int pt_dx(int k) { return k == 1 || k == 5 || k == 7 ? 1 : (k == 2 || k == 6 || k == 8 ? -1 : 0); }
__host__ __device__ constexpr int pt_dy(int k) { return k == 3 || k == 5 || k == 6 ? 1 : (k == 4 || k == 7 || k == 8 ? -1 : 0); }

// The order in which a difference-form step sums a node's 18 incoming links (k = 1..18): the
// links from the plane below (c.z = -1), from its own plane, then from the plane above, each
// group in ascending link order.  Both FP32 tracer steps (mp_f32.cu) use it, so their P is
// bit-identical.
__host__ __device__ constexpr int mp_link_order(int k)
{
    int n = 0;
    for (int dz = -1; dz <= 1; ++dz)
        for (int l = 1; l < Q; ++l)
            if (vel(l).z == dz && ++n == k) return l;
    return -1;
}

// visiting the nine points in order adds each node's links of one z offset in ascending order,
// the offsets in the order -1, 0, +1: the sum order of mp_link_order
__host__ __device__ constexpr bool plane_order_is_link_order()
{
    int k = 0;
    for (int dz = -1; dz <= 1; ++dz)
        for (int p = 0; p < 9; ++p) {
            const int l = link_of(pt_dx(p), pt_dy(p), dz);
            if (l > 0 && l != mp_link_order(++k)) return false;
        }
    return k == Q - 1;
}
static_assert(plane_order_is_link_order(), "plane-wise visit order differs from mp_link_order");

// Difference-form sweep of one tile (a box's FP32 step, mp_f32.cu:k_mp32's arithmetic in
// mp_link_order): P(par) -> P(par^1) (and A) for its fluid nodes, P(r) + [sum_l sp_in(l)
// (P(r+c_l) - P(r)) + D P(r)] with the node's fixed (u*, D) from a.aux; vt += the VACF terms.
//
// Plane-wise: each plane zz = z0-1 .. z1 is read once.  A thread reads the nine points
// (x+dx, y+dy, zz) of its column's neighbourhood (V and P: 18 shared-memory reads instead of the
// 37 a node-wise step makes) and adds each point's incoming links to the nodes of its column that
// they reach: (dx, dy, -1) to node zz+1, (dx, dy, 0) to node zz, (dx, dy, +1) to node zz-1.  The
// three nodes in flight keep their sums, P and flag words in registers; node zz-1 is complete
// after plane zz and is written.  Ring of 4 plane slots: at step zz plane zz+1 has arrived (its
// centre P enters the registers), and after the step's barrier the fetch of plane zz+3 reuses the
// slot of plane zz-1, which no thread reads any more.
// tmV / tmP (nullptr: per-thread copies everywhere): tensor maps of V and of P(par); a tile whose
// plane with its halo lies inside the box (no periodic wrap in x or y) stages each plane with two
// bulk tensor copies issued by one thread and completed on the ring slot's mbarrier; a wait that
// runs out of its bound sets LBGPU_ERR_TIMEOUT in *status and the tile's nodes are left alone.
template <typename Args>
__device__ __forceinline__ void mp_slab_planes(const Args &a, int par, int x0, int y0, int z0, int z1,
                                               float4 *sm_raw, float (&vt)[3], const CUtensorMap *tmV,
                                               const CUtensorMap *tmP, unsigned *status)
{
    // align the ring to 128 bytes by offsetting the shared-memory pointer itself (rounding its
    // generic address would hide from the compiler that it points to shared memory, and every
    // ring read would become a generic load)
    float4 *sm = sm_raw + ((128u - (smem_addr(sm_raw) & 127u)) & 127u) / 16u;
    float4 *sV = sm, *sP = sm + 4 * SPLP;
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + 8 * SPLP);   // one per ring slot
    // this thread's adsorbed-part slots (node z in slot z & 1), filled by its own cp.async
    float4 *sA = sm + 8 * SPLP + 2 + threadIdx.x;
    const int lx = a.lx, ly = a.ly, lz = a.lz;
    const float4 *__restrict__ Vg = a.V;
    const float4 *__restrict__ Pg = a.P[par];
    const bool tma = tmV != nullptr && x0 >= 1 && x0 + MPS_TX + 1 <= lx && y0 >= 1 && y0 + MPS_TY + 1 <= ly;
    if (tma) {
        if (threadIdx.x == 0) {
            for (int q = 0; q < 4; ++q) mbar_init(&bars[q], 1);
            mbar_fence_init();
        }
        __syncthreads();
    }
    auto slot = [&](int zz) { return (zz - z0 + 1) & 3; };
    const unsigned long long wait_ns = a.wait_ns ? a.wait_ns : 2000000000ull;
    const bool skip_copies = a.skip_copies != 0;
    int last_issued = z0 - 2, last_waited = z0 - 2;   // bulk-copied planes issued / arrived
    // plane zz (<= z1) into its slot; per-thread copies commit one group per call (an empty one
    // past z1), so that "plane zz+1 arrived" is always "all but the latest group complete"
    auto load_plane = [&](int zz) {
        if (zz <= z1) {
            const int gz = zz < 0 ? zz + lz : (zz >= lz ? zz - lz : zz);
            float4 *dv = sV + slot(zz) * SPLP, *dp = sP + slot(zz) * SPLP;
            if (tma) {
                if (threadIdx.x == 0) {
                    mbar_arrive_expect_tx(&bars[slot(zz)], 2 * MPS_TMA_BYTES);
                    if (!skip_copies) {
                        tma_load_4d(dv, tmV, 0, x0 - 1, y0 - 1, gz, &bars[slot(zz)]);
                        tma_load_4d(dp, tmP, 0, x0 - 1, y0 - 1, gz, &bars[slot(zz)]);
                    }
                }
                last_issued = zz;
            } else {
                for (int k = threadIdx.x; k < SPL; k += MP_BLOCK) {
                    const int hx = k % SHX, hy = k / SHX;
                    int gx = x0 + hx - 1, gy = y0 + hy - 1;
                    gx = gx < 0 ? gx + lx : (gx >= lx ? gx - lx : gx);   // lx >= 32: one wrap at most
                    gy = gy < 0 ? gy + ly : (gy >= ly ? gy - ly : gy);   // ly >= 8
                    const size_t idx = (size_t)gx + (size_t)lx * ((size_t)gy + (size_t)ly * gz);
                    cp_async16(dv + k, Vg + idx);
                    cp_async16(dp + k, Pg + idx);
                }
            }
        }
        if (!tma) cp_async_commit();
    };
    // plane zz has arrived (this thread's view; the barrier that follows makes it everyone's); the
    // fill of plane zz is its slot's ((zz - z0 + 1) / 4)-th: the phase parity to wait for
    auto wait_plane = [&](int zz) {
        if (!tma) {
            cp_async_wait1();
            return true;
        }
        const bool done = mbar_wait(&bars[slot(zz)], (unsigned)(((zz - z0 + 1) >> 2) & 1), wait_ns);
        if (done) last_waited = zz;
        return done;
    };
    const int tx = threadIdx.x % MPS_TX, ty = threadIdx.x / MPS_TX;
    const int x = x0 + tx, y = y0 + ty;
    const bool col = x < lx && y < ly;
    const int c0 = (ty + 1) * SHX + (tx + 1);
    // node offsets in 32 bits (a box holds fewer than 2^31 nodes); the column's arrays are
    // addressed from its first node
    const unsigned col0 = (unsigned)x + (unsigned)lx * (unsigned)y, plane = (unsigned)lx * (unsigned)ly;
    const uint32_t *__restrict__ mcol = a.mask + col0;
    const float4 *__restrict__ auxcol = a.aux + col0;
    float4 *__restrict__ Pout = a.P[par ^ 1] + col0;
    // flag word of the column's node z; 0 (no fluid bit, no work) outside the tile's nodes
    auto mask_at = [&](int z) { return (col && z < z1) ? __ldg(mcol + plane * (unsigned)z) : 0u; };
    const float4 zero = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    bool ok = true;   // false once a wait for a bulk copy ran out
    // a node of the column in flight: P (also the centre point of its plane for the links of
    // the nodes above and below), running sums (x and y as one packed pair), flag word
    struct Node {
        float4 p;
        float2 nxy;
        float nz;
        uint32_t m;
    };
    Node S0, S1, S2;
    S0.m = S1.m = S2.m = 0u;
    S0.p = S1.p = S2.p = zero;
    S0.nxy = S1.nxy = S2.nxy = make_float2(0.0f, 0.0f);
    S0.nz = S1.nz = S2.nz = 0.0f;
    uint32_t m_next = mask_at(z0);   // flag word of node zz+1 at the start of step zz
    // Step zz with A = node zz-1, B = node zz, C = node zz+1 (DA, DB, DC: which of them can be
    // nodes of the tile: the first step zz = z0-1 has only C, the last zz = z1 only A, and each
    // computes only their links).
    auto step = [&](auto DA, auto DB, auto DC, Node &A, Node &B, Node &C, int zz) {
        constexpr bool da = decltype(DA)::value, db = decltype(DB)::value, dc = decltype(DC)::value;
        // node zz-1's fixed (u*, D), needed at the end of this step: loaded before the links, so
        // that they hide its latency
        float4 axA = zero;
        if constexpr (da)
            if (A.m & FLUID_BIT) axA = __ldg(auxcol + plane * (unsigned)(zz - 1));
        if (dc && ok) ok = wait_plane(zz + 1);
        // one verdict for the block: once a wait has run out, no thread uses the ring and no new
        // copy is issued (the per-thread path never fails)
        ok = __syncthreads_and(ok);
        if (ok) load_plane(zz + 3);
        if constexpr (dc) {   // node zz+1 enters; its centre P is the next step's centre point
            C.m = m_next;
            m_next = mask_at(zz + 2);
            C.p = (ok && col) ? sP[slot(zz + 1) * SPLP + c0] : zero;
            C.nxy = make_float2(0.0f, 0.0f);
            C.nz = 0.0f;
        }
        // every lane runs the links (no branch: a warp runs them whenever one of its lanes has a
        // fluid node in flight); a lane without one adds onto a running sum it never stores
        if (ok) {
            const int s0 = slot(zz) * SPLP + c0;
            static_for<0, 9>([&](auto K) {
                constexpr int k = decltype(K)::value;
                constexpr int dx = pt_dx(k), dy = pt_dy(k);
                constexpr bool axis = dx * dx + dy * dy <= 1;   // links (dx, dy, -1) and (dx, dy, +1)
                if constexpr ((dc && axis) || (db && (dx != 0 || dy != 0)) || (da && axis)) {
                    const float4 vn = sV[s0 + dy * SHX + dx];
                    float4 pn;
                    if constexpr (dx == 0 && dy == 0) pn = B.p;
                    else pn = sP[s0 + dy * SHX + dx];
                    // lambda w / 2 of the point's two weight classes times its fluid flag: axis
                    // links (dx, dy) = (0, 0) in z and the in-plane axis links, diagonal the rest
                    constexpr bool need_ax = (dx == 0 && dy == 0) || (db && dx * dx + dy * dy == 1);
                    constexpr bool need_dg = (dx * dx + dy * dy == 2 && db) || (dx * dx + dy * dy == 1 && (dc || da));
                    float lw_ax = 0.0f, lw_dg = 0.0f;
                    if constexpr (need_ax) lw_ax = __fmul_rn(a.lwh[1], vn.w);
                    if constexpr (need_dg) lw_dg = __fmul_rn(a.lwh[2], vn.w);
                    if constexpr (dc && axis) {   // link (dx, dy, -1) of node zz+1
                        constexpr int l = link_of(dx, dy, -1);
                        constexpr int w = wclass(l);
                        mp32_link(mp32_scatter_flag(a.a1[w], mp32_cdot<-dx, -dy, 1>(vn), w == 1 ? lw_ax : lw_dg),
                                   pn, C.p, C.nxy.x, C.nxy.y, C.nz);
                    }
                    if constexpr (db && (dx != 0 || dy != 0)) {   // link (dx, dy, 0) of node zz
                        constexpr int l = link_of(dx, dy, 0);
                        constexpr int w = wclass(l);
                        mp32_link(mp32_scatter_flag(a.a1[w], mp32_cdot<-dx, -dy, 0>(vn), w == 1 ? lw_ax : lw_dg),
                                   pn, B.p, B.nxy.x, B.nxy.y, B.nz);
                    }
                    if constexpr (da && axis) {   // link (dx, dy, +1) of node zz-1
                        constexpr int l = link_of(dx, dy, 1);
                        constexpr int w = wclass(l);
                        mp32_link(mp32_scatter_flag(a.a1[w], mp32_cdot<-dx, -dy, -1>(vn), w == 1 ? lw_ax : lw_dg),
                                   pn, A.p, A.nxy.x, A.nxy.y, A.nz);
                    }
                }
            });
        }
        if constexpr (da) {
            if (ok && (A.m & FLUID_BIT)) {   // node zz-1 has all its links
                const unsigned r = plane * (unsigned)(zz - 1);
                float n0 = A.nxy.x, n1 = A.nxy.y, n2 = A.nz;
                const float4 p = A.p;
                vt[0] += p.x * axA.x;
                vt[1] += p.y * axA.y;
                vt[2] += p.z * axA.z;
                mp32_finish(p, axA.w, n0, n1, n2);
                if (a.ads && (A.m & INTERFACIAL_BIT)) {
                    cp_async_wait1();   // node zz-1's copy was committed a step ago
                    a.A[par ^ 1][col0 + r] =
                        mp32_adsorb(p, sA[((zz - 1) & 1) * MP_BLOCK], a.ka, a.kd, a.one_minus_kd, n0, n1, n2);
                }
                __stcs(Pout + r, make_float4(n0, n1, n2, 0.0f));
            }
        }
        // node zz+1's adsorbed part into the slot node zz-1 has just read: committed with the next
        // plane's copies (or on its own where the planes are bulk-copied), it has landed by the
        // time node zz+1 finishes, two steps on
        if constexpr (dc) {
            if (ok && a.ads && (C.m & INTERFACIAL_BIT))
                cp_async16(sA + ((zz + 1) & 1) * MP_BLOCK, a.A[par] + col0 + plane * (unsigned)(zz + 1));
            if (tma) cp_async_commit();
        }
    };
    using T = std::true_type;
    using F = std::false_type;
    load_plane(z0 - 1);
    load_plane(z0);
    ok = wait_plane(z0 - 1);
    ok = __syncthreads_and(ok);
    if (ok) load_plane(z0 + 1);
    __syncthreads();
    S0.p = (ok && col) ? sP[slot(z0 - 1) * SPLP + c0] : zero;   // centre P of plane z0-1
    // S0, S1, S2 = nodes zz-1, zz, zz+1 at step zz (a loop unrolled by three to rotate the slots
    // instead costs more in instruction fetch than the register moves it saves)
    step(F{}, F{}, T{}, S2, S0, S1, z0 - 1);
    for (int zz = z0; zz < z1; ++zz) {
        step(T{}, T{}, T{}, S0, S1, S2, zz);
        S0 = S1;
        S1 = S2;
    }
    step(T{}, F{}, F{}, S0, S1, S2, z1);   // the last node's links from plane z1
    cp_async_wait0();   // no copy of this thread still lands when the block leaves
    if (!ok) {
        // a wait ran out: let the copies already issued into this block's shared memory land
        // (each wait bounded again) before the block leaves, then report
        if (tma)
            for (int zz = last_waited + 1; zz <= last_issued; ++zz)
                if (zz >= z0 - 1) mbar_wait(&bars[slot(zz)], (unsigned)(((zz - z0 + 1) >> 2) & 1), wait_ns);
        if (status && threadIdx.x == 0) atomicOr(status, (unsigned)LBGPU_ERR_TIMEOUT);
    }
}

}  // namespace lbg
