// flow.h -- host-side launch interface of the flow kernels (FP64 strict and FP32 deviation).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

namespace lbg {

// Arguments of every FP64 flow kernel.  Passed by value (kernel parameter space).
struct FlowArgs64 {
    const uint32_t *mask;        // node flags (bounce-back bits, fluid, interfacial)
    double *f0, *f1;             // A/B population buffers, f[l*N + node]
    double *jx, *jy, *jz;        // moments of the last step (j_old for l2err)
    double *rho;                 // density output (finalize / moments)
    double *nout;                // optional populations output (finalize / stream)
    const double *Fx, *Fy, *Fz;  // per-node force field (field mode), else unused
    FlowCtl *ctl;                // reference-mode control block, else nullptr
    double *hist;                // l2err history (reference mode)
    unsigned long long *err_bits;// operator-mode max reduction target
    unsigned *status;            // operator-mode status bits
    long long N;
    const uint32_t *fidx;        // lattice indices of the Nf fluid nodes (step kernel), or null
    long long Nf;
    int lx, ly, lz;
    int parity;                  // fixed mode: buffer read this step
    int force_moment;            // fixed mode: f_ext in the moments of this step
    int force_collide;           // fixed mode: f_ext in the collision
    LbConst64 K;
    double F[3];                 // uniform force f_ext (fluid nodes)
    double cf[Q];                // c_l . f_ext in the reference's evaluation order
    int fused;                   // LBGPU_FP64_FUSED: the pair-symmetric collision with FMAs
    double kF[9], kT[9];         // per pair: c3 a1 (c.F), c3 2 a2 (c.F) (fused, uniform force)
};

// FP32-deviation arguments: populations stored as d = f - w*rho0 (float).
struct FlowArgs32 {
    const uint32_t *mask;
    float *g0, *g1;
    double *jx, *jy, *jz;        // moments output (finalize)
    double *rho;
    double *nout;
    long long N;
    int lx, ly, lz;
    int parity;
    int force_moment, force_collide;
    float w[3], a1[3], a2[3], two_a2[3];
    float c1, c2, c3, rho0;
    float F[3];
    // collision constants of the pair-symmetric form (flow_f32.cu)
    float c2w[3], c2a1[3], c2a2[3], c2a2cs2[3], c3a1[3];
    float kF[9], kT[9];
    double rho0d;
    double w64[3];
    int minb_even, minb_odd;     // AA kernel variants (resident blocks per SM)
    // AA layout over the fluid nodes only (ctx.h): g0 holds Q*Nf deviations
    unsigned Nf;
    int wide;                    // Q*Nf >= 2^32: gathers form 64-bit slot offsets
    int nw;
    const uint32_t *cpos, *cmask;
    const uint2 *rowtab;
    int xbits, ybits;            // cpos = x | y << xbits | z << (xbits + ybits)
    // reference loop (lbgpu_equilibration): control block read by the AA launches, l2err history
    FlowCtl *ctl;
    double *hist;
};

// FP64 strict ---------------------------------------------------------------------------
// fused step: pull-stream (halfway bounce-back) + moments + [l2err, j store] + collision
cudaError_t launch_flow_step_f64(const FlowArgs64 &a, int fmask, bool field, bool check,
                                 bool ref, unsigned grid, cudaStream_t s);
// collision only, reading pre-collision n from src buffer (parity) and density/j arrays,
// writing post-collision populations to the other buffer
cudaError_t launch_collide_f64(const FlowArgs64 &a, int fmask, bool field, cudaStream_t s);
// bounce-back + stream only (all nodes), src buffer (parity) -> nout
cudaError_t launch_stream_f64(const FlowArgs64 &a, cudaStream_t s);
// moments of populations in buffer (parity) for all nodes: rho, j (F/2 + ...), l2err, n<0
cudaError_t launch_moments_f64(const FlowArgs64 &a, bool field, cudaStream_t s);
// pull from buffer (parity) + moments, writing n_t (if nout), rho and j for all nodes
cudaError_t launch_finalize_f64(const FlowArgs64 &a, bool field, cudaStream_t s);
// init_simu.f90:31-39: raw n = w*rho0 into buffer (parity), rho, j = 0
cudaError_t launch_init_f64(const FlowArgs64 &a, double rho0, cudaStream_t s);

// FP32 deviation ------------------------------------------------------------------------
cudaError_t launch_flow_step_f32(const FlowArgs32 &a, unsigned grid, cudaStream_t s);
cudaError_t launch_init_f32(const FlowArgs32 &a, cudaStream_t s);
// AA layout: flag word of every compact node
cudaError_t launch_compact_mask(const FlowArgs32 &a, uint32_t *cmask, cudaStream_t s);
// AA layout: d[l*Nf + i] = n[l*N + lattice index of i] - w_l rho0
cudaError_t launch_to_dev_compact32(const FlowArgs32 &a, const double *n, float *out, cudaStream_t s);
cudaError_t launch_finalize_f32(const FlowArgs32 &a, bool pull, cudaStream_t s);
cudaError_t launch_collide_f32(const FlowArgs32 &a, cudaStream_t s);
cudaError_t launch_aa_step_f32(const FlowArgs32 &a, bool odd, cudaStream_t s);
// reference loop: FP64 moments, l2err, n<0 / non-finite checks of the AA state (swapped after an
// even launch) and the phase decision in the control block a.ctl
cudaError_t launch_aa_check_f32(const FlowArgs32 &a, bool swapped, cudaStream_t s);
cudaError_t launch_aa_finalize_f32(const FlowArgs32 &a, bool swapped, cudaStream_t s);
cudaError_t launch_to_dev32(const FlowArgs32 &a, const double *n, float *out, cudaStream_t s);

// geometry ------------------------------------------------------------------------------
cudaError_t launch_node_flags(const int8_t *nature, uint32_t *mask, int lx, int ly, int lz,
                              cudaStream_t s);
cudaError_t launch_count_nodes(const uint32_t *mask, long long N, unsigned long long *counts,
                               cudaStream_t s);

}  // namespace lbg
