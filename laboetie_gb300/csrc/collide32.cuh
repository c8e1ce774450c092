// collide32.cuh -- the FP32-deviation BGK + Guo collision shared by the single-box and the
// batched kernels.  Args provides c1, c2w, c2a1, c2a2, c2a2cs2, c3a1 (per weight class), the
// per-pair force constants kF, kT, the force F and the rest density rho0 (all float).
//
// Populations are single-precision deviations d_l = f_l - w_l*rho0 from the rest state.  The
// collision is module_collision.f90:87-104 written for deviations and split into the parts even
// and odd in c for each pair of opposite velocities (c.j, c.u and c.F change sign, everything
// else does not):
//   dneq = E +- O,  E = w drho + a2 ((c.j)(c.u) - cs^2 j.u),  O = a1 c.j
//   T    = TE +- TO, TE = 2 a2 (c.u)(c.F) - a1 u.F,           TO = a1 c.F
//   d*_l = c1 d_l + (c2 E + c3 TE) +- (c2 O + c3 TO)
// with kF = c3 a1 c.F and kT = c3 2 a2 c.F precomputed per pair.
#pragma once

#include "common.cuh"

namespace lbg {

template <int CX, int CY, int CZ>
__device__ __forceinline__ float dotf(float x, float y, float z)
{
    float s = 0.0f;
    if constexpr (CX > 0) s += x;
    if constexpr (CX < 0) s -= x;
    if constexpr (CY > 0) s += y;
    if constexpr (CY < 0) s -= y;
    if constexpr (CZ > 0) s += z;
    if constexpr (CZ < 0) s -= z;
    return s;
}


// Every product and sum below is an explicit fused or separately rounded intrinsic, so the
// same inputs give the same bits in every kernel that inlines this function (the compiler may
// not re-contract it differently in different kernels).
template <int FMASK, typename Args>
__device__ __forceinline__ void collide_dev(float (&g)[Q], const float drho, const float jx,
                                            const float jy, const float jz, const Args &a,
                                            const bool force)
{
    const float rho = __fadd_rn(a.rho0, drho);
    const float ir = __fdiv_rn(1.0f, rho);
    const float ux = __fmul_rn(jx, ir), uy = __fmul_rn(jy, ir), uz = __fmul_rn(jz, ir);
    const float ju = __fmaf_rn(jx, ux, __fmaf_rn(jy, uy, __fmul_rn(jz, uz)));
    float base[3];
#pragma unroll
    for (int w = 0; w < 3; ++w) base[w] = __fmaf_rn(a.c2w[w], drho, -__fmul_rn(a.c2a2cs2[w], ju));
    if constexpr (FMASK != 0) {
        if (force) {
            const float uF = __fmaf_rn(ux, a.F[0], __fmaf_rn(uy, a.F[1], __fmul_rn(uz, a.F[2])));
#pragma unroll
            for (int w = 0; w < 3; ++w) base[w] = __fmaf_rn(-a.c3a1[w], uF, base[w]);
        }
    }
    g[0] = __fmaf_rn(a.c1, g[0], base[0]);
    static_for<0, 9>([&](auto P) {
        constexpr int p = decltype(P)::value;
        constexpr int l = pair_l(p);
        constexpr int li = inv(l);
        constexpr Vel c = vel(l);
        constexpr int w = wclass(l);
        const float cj = dotf<c.x, c.y, c.z>(jx, jy, jz);
        const float cu = dotf<c.x, c.y, c.z>(ux, uy, uz);
        float A = __fmaf_rn(a.c2a2[w], __fmul_rn(cj, cu), base[w]);
        float B = __fmul_rn(a.c2a1[w], cj);
        if constexpr (FMASK != 0) {
            if (force) {
                A = __fmaf_rn(a.kT[p], cu, A);
                B = __fadd_rn(B, a.kF[p]);
            }
        }
        g[l] = __fmaf_rn(a.c1, g[l], __fadd_rn(A, B));
        g[li] = __fmaf_rn(a.c1, g[li], __fsub_rn(A, B));
    });
}

}  // namespace lbg
