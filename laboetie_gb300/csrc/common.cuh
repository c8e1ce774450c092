// common.cuh -- D3Q19 tables, compile-time loops and device helpers shared by all kernels.
//
// Node index: node = x + lx*(y + ly*z) (0-based), the reference's column-major order.
// Flow populations are structure-of-arrays f[l*N + node]; velocity order and weights follow
// module_lbmodel.f90:68-86,143-147.
#pragma once

#include <cstdint>
#include <type_traits>
#include <utility>

namespace lbg {

constexpr int Q = 19;

struct Vel {
    int x, y, z;
};

// module_lbmodel.f90:68-86 (0-based l = reference l - 1)
__host__ __device__ constexpr Vel vel(int l)
{
    return l == 0    ? Vel{0, 0, 0}
           : l == 1  ? Vel{1, 0, 0}
           : l == 2  ? Vel{-1, 0, 0}
           : l == 3  ? Vel{0, 1, 0}
           : l == 4  ? Vel{0, -1, 0}
           : l == 5  ? Vel{0, 0, 1}
           : l == 6  ? Vel{0, 0, -1}
           : l == 7  ? Vel{1, 1, 0}
           : l == 8  ? Vel{-1, 1, 0}
           : l == 9  ? Vel{1, -1, 0}
           : l == 10 ? Vel{-1, -1, 0}
           : l == 11 ? Vel{1, 0, 1}
           : l == 12 ? Vel{-1, 0, 1}
           : l == 13 ? Vel{1, 0, -1}
           : l == 14 ? Vel{-1, 0, -1}
           : l == 15 ? Vel{0, 1, 1}
           : l == 16 ? Vel{0, -1, 1}
           : l == 17 ? Vel{0, 1, -1}
                     : Vel{0, -1, -1};
}

// module_lbmodel.f90:156-162
__host__ __device__ constexpr int inv(int l)
{
    return l == 0 ? 0 : (l <= 6 ? ((l & 1) ? l + 1 : l - 1)
                                : (l == 7 ? 10 : l == 10 ? 7 : l == 8 ? 9 : l == 9 ? 8
                                  : l == 11 ? 14 : l == 14 ? 11 : l == 12 ? 13 : l == 13 ? 12
                                  : l == 15 ? 18 : l == 18 ? 15 : l == 16 ? 17 : 16));
}

// The 9 pairs (l, inv l) of opposite velocities; l is the first of pair p.
__host__ __device__ constexpr int pair_l(int p)
{
    return p == 0 ? 1 : p == 1 ? 3 : p == 2 ? 5 : p == 3 ? 7 : p == 4 ? 8 : p == 5 ? 11 : p == 6 ? 12
           : p == 7 ? 15 : 16;
}

// weight class: 0 rest (1/3), 1 axis (1/18), 2 face diagonal (1/36)
__host__ __device__ constexpr int wclass(int l) { return l == 0 ? 0 : (l < 7 ? 1 : 2); }

// Node flag word: bit l (1..18) = the pull source node - c_l has a different nature
// (halfway bounce-back on that link); FLUID and INTERFACIAL as below.
constexpr uint32_t BB_BITS = 0x7FFFEu;
constexpr uint32_t FLUID_BIT = 1u << 20;
constexpr uint32_t INTERFACIAL_BIT = 1u << 21;

template <int I, int N, typename F>
__host__ __device__ __forceinline__ void static_for(F &&f)
{
    if constexpr (I < N) {
        f(std::integral_constant<int, I>{});
        static_for<I + 1, N>(f);
    }
}

// Reference constants in FP64, computed once on the host (module_lbmodel.f90:127-147,
// module_collision.f90:28,99-103) and passed by value to the kernels.
struct LbConst64 {
    double a0[3], a1[3], a2[3], two_a2[3];  // per weight class
    double k1, k0;                          // (1 - cs^2) and (0 - cs^2)
    double c1, c2, c3;                      // 1-1/tau, 1/tau, 1-1/(2 tau)
    // the pair-symmetric collision of LBGPU_FP64_FUSED, per weight class: c2 a0, c2 a1, c2 a2,
    // c2 a2 cs^2, c3 a1
    double c2a0[3], c2a1[3], c2a2[3], c2a2cs2[3], c3a1[3];
};

// Device-resident control block of the reference flow loop (equilibration.f90:143-491).
struct FlowCtl {
    int t;              // reference step computed by the next launch (1-based)
    int parity;         // buffer holding the post-collision populations feeding step t
    int force_moment;   // 1 if f_ext enters the moments of step t (j = F/2 + ...)
    int force_collide;  // 1 if f_ext enters the collision that ends step t
    int redo;           // 1: the next launch repeats step t (force switched on)
    int done;           // 1: loop left; launches return at once
    int conv_without, conv_with;
    int max_steps;
    int exit_step;
    unsigned status;               // lbgpu_status bits raised on the device
    unsigned blocks_done;          // last-block-done counter
    unsigned long long err_bits;   // running max of |j - j_old| as IEEE bits (non-negative)
    double target_error;
    double last_l2err;
    int hist_cap;
    int exit_force_moment;  // force_moment of the exit step (its moments include F/2)
    // FP32 in-place loop (a check launch after every AA launch): the moment force of the state
    // the next check reads, and the moment / collision forces of the next AA launch
    int check_fm, aa_fm, aa_fc;
    int exit_phase;         // AA phase of the state the loop exited on
};

// Maximum of two values that are each non-negative or a NaN with the sign bit clear (what fabs
// returns), taken on their IEEE bit patterns: the order of non-negative doubles is the order of
// their bits, and a NaN's bits lie above +Inf's, so a NaN is never dropped as fmax drops it.
__device__ __forceinline__ double max_nonneg(double a, double b)
{
    const unsigned long long ia = (unsigned long long)__double_as_longlong(a);
    const unsigned long long ib = (unsigned long long)__double_as_longlong(b);
    return __longlong_as_double((long long)(ia > ib ? ia : ib));
}

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long *addr, double v)
{
    // IEEE-754 ordering of non-negative doubles equals the ordering of their bit patterns.
    atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// Periodic neighbour coordinate (module_system.f90:99-112): one step across the boundary.
__device__ __forceinline__ int wrap_minus(int x, int n) { return x == 0 ? n - 1 : x - 1; }
__device__ __forceinline__ int wrap_plus(int x, int n) { return x == n - 1 ? 0 : x + 1; }

template <int C>
__device__ __forceinline__ int pick(int xm, int x, int xp)
{
    // coordinate of (x - C) with periodic wrap, C in {-1,0,1}
    if constexpr (C == 1) return xm;
    else if constexpr (C == -1) return xp;
    else return x;
}

}  // namespace lbg
