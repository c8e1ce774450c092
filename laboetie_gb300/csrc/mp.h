// mp.h -- tracer moment propagation (drop_tracers.f90, module_moment_propagation.f90).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

namespace lbg {

constexpr int MP_BLOCK = 256;
// Blocks of the propagation kernels: grid-stride over the nodes with at most 8 blocks per SM
// of a 152-SM GB300, so the last block adds at most 1216 partials.
constexpr unsigned MP_MAX_BLOCKS = 152 * 8;

// Device control block of the propagation loop (module_moment_propagation.f90:164-289).
struct MpCtl {
    int it;              // next step (1-based)
    int parity;          // buffer holding P(now)
    int done;            // converged or step budget used: launches return at once
    int converged;
    int last_it;         // last step completed
    int max_it;          // last step this call may run
    int it_base;         // first step of this call (history index 0)
    unsigned status;
    unsigned blocks_done;
    double thr1, thr2;   // convergence thresholds (module_moment_propagation.f90:284)
    double vacf[3];      // VACF of the last step
};

struct MpArgs64 {
    const uint32_t *mask;
    const double *rho, *jx, *jy, *jz;  // node%solventDensity / solventFlux after the flow phase
    double *coef;                      // 18*N: coef[(l-1)*N + r] = scattprop of r+c_l towards r
    double *frac;                      // remaining fraction at r (before the adsorption term)
    double *us[3];                     // u*(r)
    double *P[2][3];                   // propagated quantity, now/next by parity
    double *A[2][3];                   // adsorbed part (adsorption only)
    double *partial;                   // 3 per block
    MpCtl *ctl;
    double *hist;                      // 3 per step
    long long N;
    const uint32_t *fidx;              // lattice indices of the Nf fluid nodes (step kernel), or null
    long long Nf;
    int lx, ly, lz;
    int ads;
    double lambda, ka, kd, one_minus_kd, bw;
    double a0[3], a1[3], lwh[3];       // lwh = (lambda*a0)*0.5 (fermi = 1/2 for a neutral tracer)
    double fext[3], q, D, E[3];        // drop_tracers.f90:88-100
    // charged tracer (lbgpu_mp_init_charged): lambda*a0, the potential, tracer_z and
    // 1/Pstat's denominator Pstat = SUM(exp(-z phi)) over fluid (+ K over interfacial fluid)
    double lw[3];
    const double *phi;
    double z, pstat;
    int fused;                         // LBGPU_FP64_FUSED: the step's gathers as fused multiply-adds
};

struct MpArgs32 {
    const uint32_t *mask;
    const float4 *V;                   // (j + f_ext)/rho at every fluid node (w unused)
    float4 *P[2];                      // propagated quantity (x, y, z, 0), now/next by parity
    float4 *A[2];                      // adsorbed part
    // per fluid node, fixed for the run (set by the init pass): u* = sum_l c_l sp_out(l) and
    // D = sum_l sp_in(l) - sum_l sp_out(l), with sp_in / sp_out the link's scattering into the
    // node from r + c_l / out of it towards r + c_l (0 across a bounce-back link)
    float4 *aux;                       // (u*x, u*y, u*z, D)
    double *partial;
    MpCtl *ctl;
    double *hist;
    long long N;
    int lx, ly, lz;
    int ads;
    float ka, kd, one_minus_kd;
    float a1[3], lwh[3];
    int slab;                          // shared-memory slab step where the box allows it
    unsigned slab_resident;            // slab blocks resident on the device at once
    // charged tracer: V.w holds the potential phi at every node; lambda*a0, tracer_z, 1/Pstat
    // and elec_slope for the per-link fermi factors (the grid-stride step is used)
    int charged;
    float lw[3], z, inv_pstat, E[3];
    // the fluid nodes of an in-place (AA) FP32 context: their packed positions (compact.cuh), which
    // the grid-stride step walks (one thread per fluid node), or null (every lattice node)
    const uint32_t *cpos;
    unsigned Nf;
    int xbits, ybits;
    // bounded waits of the slab step's bulk copies: the limit (ns); skip_copies (set only by a
    // test, LBGPU_MP_TEST_SKIP_COPIES=1) arms each plane's barrier without issuing its copies, so
    // the wait runs out and the step reports LBGPU_ERR_TIMEOUT without any fault
    unsigned long long wait_ns;
    int skip_copies;
};

// Shared-memory slab variant of the FP32 step (mp_f32.cu): 32 x 8 column tiles sweeping a chunk
// of z planes.  Used when lx >= 32, ly >= 8 and lz >= 3.  Returns the grid (0: not eligible) and
// the planes per block in *zc.  A chunk reads two planes beyond its own, so the chunks are as long
// as filling the device once allows (resident: blocks resident at once), and at least 8 planes.
// resident 0 (the step's shared memory could not be granted): not eligible.
constexpr int MPS_TX = 32, MPS_TY = 8;
inline unsigned mp32_slab_grid(int lx, int ly, int lz, unsigned resident, int *zc)
{
    if (lx < MPS_TX || ly < MPS_TY || lz < 3 || resident == 0) return 0;
    const int nxy = ((lx + MPS_TX - 1) / MPS_TX) * ((ly + MPS_TY - 1) / MPS_TY);
    int nz = (int)(resident / (unsigned)nxy);
    if (nz > lz / 8) nz = lz / 8;
    if (nz < 1) nz = 1;
    const int c = (lz + nz - 1) / nz;
    *zc = c;
    return (unsigned)(nxy * ((lz + c - 1) / c));
}

cudaError_t launch_mp_init_f64(const MpArgs64 &a, unsigned grid, cudaStream_t s);
cudaError_t launch_mp_step_f64(const MpArgs64 &a, unsigned grid, cudaStream_t s);
cudaError_t launch_mp_reduce_init(double *partial, unsigned nblocks, MpCtl *ctl, cudaStream_t s);
cudaError_t launch_mp_v32(const MpArgs64 &a64, float4 *V, cudaStream_t s);
// tm: the tensor maps of V, P[0], P[1] for the slab step's bulk tensor copies, or null (the slab
// step then stages every tile with per-thread asynchronous copies)
cudaError_t launch_mp_step_f32(const MpArgs32 &a, unsigned grid, const CUtensorMap *tm, cudaStream_t s);
// tensor maps of a box's float4 field (V or P) for the slab step: dims (4 components, lx, ly, lz),
// box (4, 34, 10, 1); false if the driver refuses them
bool mp32_tensor_map(CUtensorMap *tm, const float4 *field, int lx, int ly, int lz);
// blocks of the slab step resident on the current device at once (SMs x blocks per SM)
unsigned mp32_slab_resident();
cudaError_t launch_mp_init_f32(const MpArgs32 &a, float bw, unsigned grid, cudaStream_t s);

}  // namespace lbg
