// reduce.cuh -- deterministic block and grid sums and the propagation loop control.
//
// Sums are formed in a fixed order (shuffle tree within a warp, then the warps in index order,
// then the block partials in index order by the last block to finish), so a result never
// depends on which block ran first: repeated runs are bit-identical.
#pragma once

#include "common.cuh"
#include "lbgpu.h"
#include "mp.h"

namespace lbg {

__device__ __forceinline__ double warp_sum_fixed(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Sum of v over a block of MP_BLOCK threads; valid in thread 0.  sh: MP_BLOCK/32 doubles.
__device__ __forceinline__ double block_sum_fixed(double v, double *sh)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_sum_fixed(v);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = lane < MP_BLOCK / 32 ? sh[lane] : 0.0;
        v = warp_sum_fixed(v);
    }
    return v;
}

// Sum of 3 values over a block of MP_BLOCK threads in one pass (fixed order); valid in thread 0.
__device__ __forceinline__ void block_sum3_fixed(double (&v)[3])
{
    __shared__ double sh[3][MP_BLOCK / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int d = 0; d < 3; ++d) v[d] = warp_sum_fixed(v[d]);
    __syncthreads();  // sh may still be read by a previous call
    if (lane == 0)
        for (int d = 0; d < 3; ++d) sh[d][wid] = v[d];
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            v[d] = lane < MP_BLOCK / 32 ? sh[d][lane] : 0.0;
            v[d] = warp_sum_fixed(v[d]);
        }
    }
}

// Every block stores its 3 partial sums; the last block to finish adds the partials in block
// order and runs `finish(total)` in thread 0.
template <typename Fin>
__device__ __forceinline__ void grid_sum3(const double (&v)[3], double *partial, unsigned *counter,
                                          Fin &&finish)
{
    __shared__ bool last;
    double b[3] = {v[0], v[1], v[2]};
    block_sum3_fixed(b);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) partial[3 * blockIdx.x + d] = b[d];
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double t[3] = {0.0, 0.0, 0.0};
    for (unsigned i = threadIdx.x; i < gridDim.x; i += MP_BLOCK) {
        const volatile double *p = partial + 3 * i;
#pragma unroll
        for (int d = 0; d < 3; ++d) t[d] += p[d];
    }
    block_sum3_fixed(t);
    if (threadIdx.x == 0) {
        *counter = 0;
        finish(t);
    }
}

// module_moment_propagation.f90:262-288 after the sweep of step ctl->it: record VACF, rotate
// now/next, test convergence (it > 2 and |VACF| below both thresholds).
__device__ __forceinline__ void mp_control(MpCtl *c, double *hist, const double (&v)[3])
{
    const int it = c->it;
    if (hist) {
        const int k = it - c->it_base;
        for (int d = 0; d < 3; ++d) hist[3 * k + d] = v[d];
    }
    for (int d = 0; d < 3; ++d) c->vacf[d] = v[d];
    bool conv = it > 2;
    for (int d = 0; d < 3; ++d)
        if (!(fabs(v[d]) < c->thr1) || !(fabs(v[d]) < c->thr2)) conv = false;
    c->parity ^= 1;
    c->last_it = it;
    c->it = it + 1;
    if (conv) {
        c->converged = 1;
        c->done = 1;
    }
    if (it >= c->max_it) c->done = 1;
    // a block's bounded wait ran out (its tile was left alone): no further step is meaningful
    if (atomicOr(&c->status, 0u) & LBGPU_ERR_TIMEOUT) c->done = 1;
}

}  // namespace lbg
