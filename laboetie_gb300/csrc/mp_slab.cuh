// mp_slab.cuh -- FP32 tracer step of a column tile with V and P staged in shared memory.
//
// The step of mp_f32.cu:k_mp32 (same operations in the same order, so P is bit-identical), for
// the nodes (x0..x0+31, y0..y0+7, z0..z1-1) of a box with lx >= 32, ly >= 8, lz >= 3.  A ring
// of 4 planes (z-1, z, z+1 and the one being fetched) of V and P with a one-node halo is filled
// by asynchronous copies one plane ahead, so the neighbour reads are shared-memory reads and
// every V and P value is fetched from L2/HBM about 1.3 times (halo) per step; the column's flag
// word (and the node's fixed (u*, D)) is loaded into registers a plane ahead.  One block barrier
// per plane: after it, plane z+1 is in shared memory and every thread is done with plane z-1, so
// the fetch of plane z+2 may overwrite the slot of plane z-2.  The argument struct provides V,
// P[2], A[2], mask, lx, ly, lz, ads, ka, kd, one_minus_kd, a1[3], lwh[3] (and aux for the
// difference form).
#pragma once

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
// 4 planes of V and of P, 4 mbarriers, and slack to align the ring to 128 bytes
constexpr size_t MPS_SMEM = 128 + sizeof(float4) * 8 * SPLP + 4 * sizeof(uint64_t);

// Scattering probability of a link, on * (a1 (c.V) + lambda w / 2) (on = 0 across a
// bounce-back link), rounded as written.
__device__ __forceinline__ float mp32_scatter(float on, float a1, float cv, float lwh)
{
    return __fmul_rn(on, __fmaf_rn(a1, cv, lwh));
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

template <int CX, int CY, int CZ>
__device__ __forceinline__ float slab_cdot(const float4 &v)
{
    float s = 0.0f;
    if constexpr (CX > 0) s += v.x;
    if constexpr (CX < 0) s -= v.x;
    if constexpr (CY > 0) s += v.y;
    if constexpr (CY < 0) s -= v.y;
    if constexpr (CZ > 0) s += v.z;
    if constexpr (CZ < 0) s -= v.z;
    return s;
}

// Sweep of one tile: P(par) -> P(par^1) (and A) for its fluid nodes; vt += the nodes' VACF
// terms (FP32, per thread).  sm: MPS_SMEM bytes of shared memory.  Every thread of the block
// (MP_BLOCK = 256 = 32 x 8) must call it.  AUX: the difference form of mp_f32.cu:k_mp32 with the
// node's fixed (u*, D) from a.aux (18 scatterings per node and step); otherwise the flux form
// P(r) + sum_l [P(r+c_l) sp_in(l) - P(r) sp_out(l)] (36 scatterings).
// TMA, with tmV / tmP the tensor maps of V and of P(par) (mp32_tensor_map; nullptr turns it off
// at run time): a tile whose plane with its halo lies inside the box (no periodic wrap in x or y)
// stages each plane with two bulk tensor copies issued by one thread and completed on the ring
// slot's mbarrier, instead of 2 x 340 per-thread copies with wrap arithmetic; a wait that runs
// out of its bound sets LBGPU_ERR_TIMEOUT in *status and the tile's nodes are left alone.
// Without TMA none of that is compiled (the barriers, the 128-byte pad and the predicate cost a
// caller 11 registers).
template <bool AUX, bool TMA, typename Args>
__device__ __forceinline__ void mp_slab_sweep(const Args &a, int par, int x0, int y0, int z0, int z1,
                                              float4 *sm_raw, float (&vt)[3],
                                              const CUtensorMap *tmV = nullptr,
                                              const CUtensorMap *tmP = nullptr,
                                              unsigned *status = nullptr)
{
    // align the ring to 128 bytes by offsetting the shared-memory pointer itself (rounding its
    // generic address would hide from the compiler that it points to shared memory, and every
    // ring read would become a generic load)
    float4 *sm = TMA ? sm_raw + ((128u - (smem_addr(sm_raw) & 127u)) & 127u) / 16u : sm_raw;
    float4 *sV = sm, *sP = sm + 4 * SPLP;
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + 8 * SPLP);   // one per ring slot
    const int lx = a.lx, ly = a.ly, lz = a.lz;
    const float4 *__restrict__ Vg = a.V;
    const float4 *__restrict__ Pg = a.P[par];
    const bool tma = TMA && tmV != nullptr && x0 >= 1 && x0 + MPS_TX + 1 <= lx && y0 >= 1 && y0 + MPS_TY + 1 <= ly;
    if (tma) {
        if (threadIdx.x == 0) {
            for (int q = 0; q < 4; ++q) mbar_init(&bars[q], 1);
            mbar_fence_init();
        }
        __syncthreads();
    }
    auto load_plane = [&](int zz) {
        const int gz = zz < 0 ? zz + lz : (zz >= lz ? zz - lz : zz);
        const int slot = (zz - z0 + 1) & 3;
        float4 *dv = sV + slot * SPLP, *dp = sP + slot * SPLP;
        if (tma) {
            if (threadIdx.x == 0) {
                mbar_arrive_expect_tx(&bars[slot], 2 * MPS_TMA_BYTES);
                tma_load_4d(dv, tmV, 0, x0 - 1, y0 - 1, gz, &bars[slot]);
                tma_load_4d(dp, tmP, 0, x0 - 1, y0 - 1, gz, &bars[slot]);
            }
            return;
        }
        for (int k = threadIdx.x; k < SPL; k += MP_BLOCK) {
            const int hx = k % SHX, hy = k / SHX;
            int gx = x0 + hx - 1, gy = y0 + hy - 1;
            gx = gx < 0 ? gx + lx : (gx >= lx ? gx - lx : gx);   // lx >= 32: one wrap at most
            gy = gy < 0 ? gy + ly : (gy >= ly ? gy - ly : gy);   // ly >= 8
            const size_t idx = (size_t)gx + (size_t)lx * ((size_t)gy + (size_t)ly * gz);
            cp_async16(dv + k, Vg + idx);
            cp_async16(dp + k, Pg + idx);
        }
        cp_async_commit();
    };
    const int tx = threadIdx.x % MPS_TX, ty = threadIdx.x / MPS_TX;
    const int x = x0 + tx, y = y0 + ty;
    const bool col = x < lx && y < ly;
    // the fill of plane zz is its slot's ((zz - z0 + 1) / 4)-th: the phase parity to wait for
    auto wait_plane = [&](int zz) {
        return mbar_wait(&bars[(zz - z0 + 1) & 3], (unsigned)(((zz - z0 + 1) >> 2) & 1));
    };
    load_plane(z0 - 1);
    load_plane(z0);
    load_plane(z0 + 1);
    bool ok = true;
    if (tma) ok = wait_plane(z0 - 1) && wait_plane(z0);
    // the column's flag word (and, AUX, fixed node data) of the next plane, loaded a plane ahead
    // so that no plane starts on a global-memory round trip
    const size_t col0 = (size_t)x + (size_t)lx * (size_t)y, plane = (size_t)lx * (size_t)ly;
    uint32_t m_next = col ? __ldg(a.mask + col0 + plane * z0) : 0u;
    float4 ax_next = make_float4(0.f, 0.f, 0.f, 0.f);
    if constexpr (AUX)
        if (col) ax_next = __ldg(a.aux + col0 + plane * z0);
    for (int z = z0; z < z1; ++z) {
        if (!tma) cp_async_wait0();
        else if (TMA && ok) ok = wait_plane(z + 1);
        __syncthreads();
        if (z + 2 <= z1) load_plane(z + 2);
        const size_t r = col0 + plane * z;
        const uint32_t m = m_next;
        const float4 ax = ax_next;
        if (col && z + 1 < z1) {
            m_next = __ldg(a.mask + r + plane);
            if constexpr (AUX) ax_next = __ldg(a.aux + r + plane);
        }
        if ((!TMA || ok) && (m & FLUID_BIT)) {
            const int c0 = (ty + 1) * SHX + (tx + 1);
            const int s0 = (z - z0 + 1) & 3;
            const float4 vr = sV[s0 * SPLP + c0];
            const float4 p = sP[s0 * SPLP + c0];
            float ux = 0.0f, uy = 0.0f, uz = 0.0f;
            float n0 = 0.0f, n1 = 0.0f, n2 = 0.0f;
            static_for<1, Q>([&](auto L) {
                constexpr int l = decltype(L)::value;
                constexpr Vel c = vel(l);
                constexpr int w = wclass(l);
                const float on = ((m >> inv(l)) & 1u) ? 0.0f : 1.0f;  // r + c_l is fluid
                const int q = ((z + c.z - z0 + 1) & 3) * SPLP + c0 + c.y * SHX + c.x;
                const float4 vn = sV[q];
                const float4 pn = sP[q];
                if constexpr (AUX) {
                    mp32_link(mp32_scatter(on, a.a1[w], slab_cdot<-c.x, -c.y, -c.z>(vn), a.lwh[w]), pn, p,
                              n0, n1, n2);
                } else {
                    const float sp = on * (a.a1[w] * slab_cdot<c.x, c.y, c.z>(vr) + a.lwh[w]);
                    const float spp = on * (a.a1[w] * slab_cdot<-c.x, -c.y, -c.z>(vn) + a.lwh[w]);
                    ux += c.x * sp;
                    uy += c.y * sp;
                    uz += c.z * sp;
                    n0 += pn.x * spp - p.x * sp;
                    n1 += pn.y * spp - p.y * sp;
                    n2 += pn.z * spp - p.z * sp;
                }
            });
            if constexpr (AUX) {
                vt[0] += p.x * ax.x;
                vt[1] += p.y * ax.y;
                vt[2] += p.z * ax.z;
                mp32_finish(p, ax.w, n0, n1, n2);
            } else {
                vt[0] += p.x * ux;
                vt[1] += p.y * uy;
                vt[2] += p.z * uz;
                n0 += p.x;
                n1 += p.y;
                n2 += p.z;
            }
            if (a.ads && (m & INTERFACIAL_BIT)) {
                const float4 qa = a.A[par][r];
                n0 += qa.x * a.kd - a.ka * p.x;
                n1 += qa.y * a.kd - a.ka * p.y;
                n2 += qa.z * a.kd - a.ka * p.z;
                a.A[par ^ 1][r] = make_float4(qa.x * a.one_minus_kd + p.x * a.ka,
                                              qa.y * a.one_minus_kd + p.y * a.ka,
                                              qa.z * a.one_minus_kd + p.z * a.ka, 0.0f);
            }
            __stcs(a.P[par ^ 1] + r, make_float4(n0, n1, n2, 0.0f));
        }
    }
    if (TMA && !ok && status) atomicOr(status, (unsigned)LBGPU_ERR_TIMEOUT);
}

}  // namespace lbg
