// mp_slab.cuh -- FP32 tracer step of a column tile with V and P staged in shared memory.
//
// The flux form of mp_f32.cu:k_mp32 (same operations in the same order, so P is bit-identical),
// for the nodes (x0..x0+31, y0..y0+7, z0..z1-1) of a box with lx >= 32, ly >= 8, lz >= 3.  A ring
// of 4 planes (z-1, z, z+1 and the one being fetched) of V and P with a one-node halo is filled
// by asynchronous copies one plane ahead, so the 36 neighbour reads per node are shared-memory
// reads and every V and P value is fetched from L2/HBM about 1.3 times (halo) per step.  One
// block barrier per plane: after it, plane z+1 is in shared memory and every thread is done with
// plane z-1, so the fetch of plane z+2 may overwrite the slot of plane z-2.  The argument struct
// provides V, P[2], A[2], mask, lx, ly, lz, ads, ka, kd, one_minus_kd, a1[3], lwh[3].
#pragma once

#include "common.cuh"
#include "cpasync.cuh"
#include "mp.h"

namespace lbg {

constexpr int SHX = MPS_TX + 2, SHY = MPS_TY + 2, SPL = SHX * SHY;  // a plane with its halo
constexpr size_t MPS_SMEM = sizeof(float4) * 8 * SPL;                // 4 planes of V and of P

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
// (MP_BLOCK = 256 = 32 x 8) must call it.
template <typename Args>
__device__ __forceinline__ void mp_slab_sweep(const Args &a, int par, int x0, int y0, int z0, int z1,
                                              float4 *sm, float (&vt)[3])
{
    float4 *sV = sm, *sP = sm + 4 * SPL;
    const int lx = a.lx, ly = a.ly, lz = a.lz;
    const float4 *__restrict__ Vg = a.V;
    const float4 *__restrict__ Pg = a.P[par];
    auto load_plane = [&](int zz) {
        const int gz = zz < 0 ? zz + lz : (zz >= lz ? zz - lz : zz);
        float4 *dv = sV + ((zz - z0 + 1) & 3) * SPL, *dp = sP + ((zz - z0 + 1) & 3) * SPL;
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
    load_plane(z0 - 1);
    load_plane(z0);
    load_plane(z0 + 1);
    for (int z = z0; z < z1; ++z) {
        cp_async_wait0();
        __syncthreads();
        if (z + 2 <= z1) load_plane(z + 2);
        const size_t r = (size_t)x + (size_t)lx * ((size_t)y + (size_t)ly * z);
        const uint32_t m = col ? __ldg(a.mask + r) : 0u;
        if (m & FLUID_BIT) {
            const int c0 = (ty + 1) * SHX + (tx + 1);
            const int s0 = (z - z0 + 1) & 3;
            const float4 vr = sV[s0 * SPL + c0];
            const float4 p = sP[s0 * SPL + c0];
            float ux = 0.0f, uy = 0.0f, uz = 0.0f;
            float n0 = 0.0f, n1 = 0.0f, n2 = 0.0f;
            static_for<1, Q>([&](auto L) {
                constexpr int l = decltype(L)::value;
                constexpr Vel c = vel(l);
                constexpr int w = wclass(l);
                const float on = ((m >> inv(l)) & 1u) ? 0.0f : 1.0f;  // r + c_l is fluid
                const int q = ((z + c.z - z0 + 1) & 3) * SPL + c0 + c.y * SHX + c.x;
                const float4 vn = sV[q];
                const float sp = on * (a.a1[w] * slab_cdot<c.x, c.y, c.z>(vr) + a.lwh[w]);
                const float spp = on * (a.a1[w] * slab_cdot<-c.x, -c.y, -c.z>(vn) + a.lwh[w]);
                ux += c.x * sp;
                uy += c.y * sp;
                uz += c.z * sp;
                const float4 pn = sP[q];
                n0 += pn.x * spp - p.x * sp;
                n1 += pn.y * spp - p.y * sp;
                n2 += pn.z * spp - p.z * sp;
            });
            vt[0] += p.x * ux;
            vt[1] += p.y * uy;
            vt[2] += p.z * uz;
            n0 += p.x;
            n1 += p.y;
            n2 += p.z;
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
}

}  // namespace lbg
