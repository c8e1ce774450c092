// batch.h -- many independent boxes of uneven size stepped together (FP32 deviations).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"
#include "mp.h"

namespace lbg {

constexpr int BATCH_BLOCK = 256;        // threads per tile of the HBM kernels
constexpr int BATCH_SMEM_THREADS = 512; // default threads of a shared-memory-resident box (256, 512
                                        // or 1024, picked by the tuner in batch_api.cu)
constexpr int BATCH_SMEM_BYTES_MAX = 227 * 1024;
constexpr int BATCH_TACC = 9;           // doubles per tile: VACF(0) part, sum over steps, last step

// Shared memory a box needs while its phase runs with the whole box resident:
// flow: 19 FP32 populations + the flag word; tracer: V, P now/next (+ A now/next) as float4
// records + the flag word.
__host__ __device__ constexpr int batch_smem_flow(int N) { return N * (Q * 4 + 4); }
__host__ __device__ constexpr int batch_smem_mp(int N, int ads) { return N * (16 * (ads ? 5 : 3) + 4); }

enum BatchPhase { BATCH_FLOW = 0, BATCH_MP = 1 };

// Device descriptor of one box.  The collision constants follow collide32.cuh; the tracer
// constants follow mp_f32.cu.
struct BatchInst {
    float *g;               // Q*N deviations, structure-of-arrays within the box
    const uint32_t *mask;   // N node flag words
    float4 *uprev;          // velocity at the previous convergence check
    float4 *V;              // tracer phase: (j + f_ext)/rho per node (0 on solid nodes)
    float4 *P[2], *A[2];    // propagated quantity / adsorbed part, by step parity
    float4 *aux;            // per fluid node, fixed for the tracer phase: (u*, D) of mp_f32.cu
    double *tacc;           // BATCH_TACC doubles per tile of BATCH_BLOCK nodes, then a status word
    int lx, ly, lz, N;
    int phase, ads;
    float c1, c2w[3], c2a1[3], c2a2[3], c2a2cs2[3], c3a1[3];
    float kF[9], kT[9];
    float F[3];
    float rho0;
    int force;              // f_ext in moments and collisions
    float a1[3], lwh[3], ka, kd, one_minus_kd;
    float bw;               // 1 / (fluid + K * interfacial fluid) nodes, rounded to FP32
    double tfext[3];        // tracer f_ext added to j in V
    // Tiled boxes use the fluid-only AA layout of compact.cuh: g[l*Nf + i], uprev[i], tiles of
    // compact indices.  Shared-memory boxes keep the lattice layout g[l*N + node].
    int compact;
    unsigned Nf;
    int nw, xbits, ybits;
    const uint32_t *cpos, *cmask;
    const uint2 *rowtab;
    // tracer phase of a tiled box with lx >= 32, ly >= 8, lz >= 3: shared-memory slab tiles of
    // 32 x 8 columns and zc planes (mp_slab.cuh); 0 otherwise
    int zc;
    int ntacc;              // tiles with VACF accumulators in tacc (the status word follows)
    // the slab step's bounded waits (batch tiles stage with per-thread copies: unused, zero)
    unsigned long long wait_ns;
    int skip_copies;
};

// Nodes a box's kernels iterate (compact fluid nodes or lattice nodes) and its 256-node tiles.
__host__ __device__ inline unsigned batch_units(const BatchInst &I) { return I.compact ? I.Nf : (unsigned)I.N; }
__host__ __device__ inline unsigned batch_ntile(const BatchInst &I) { return (batch_units(I) + BATCH_BLOCK - 1) / BATCH_BLOCK; }

struct BatchTile {
    int inst;   // index into the descriptor array
    int start;  // first node of the tile
};

// Work-list ticket of the persistent tiled launches: next tile to claim, blocks that left.
struct BatchTicket {
    unsigned next, done;
};

// one AA launch over the tiles of the tiled boxes (compact layout); minb: 3..6 resident blocks
cudaError_t launch_batch_aa(const BatchInst *insts, const BatchTile *tiles, int ntiles, bool odd, int minb,
                            cudaStream_t s);
// the same as a persistent work list: `grid` blocks claim `tpc` tiles at a time from the ticket tk
// (zero before the first launch; the last block of each launch zeroes it again)
cudaError_t launch_batch_aa_list(const BatchInst *insts, const BatchTile *tiles, int ntiles, bool odd, int minb,
                                 int grid, int tpc, BatchTicket *tk, cudaStream_t s);
// one tracer step of the tiled boxes: P[par] -> P[par^1]
cudaError_t launch_batch_mp(const BatchInst *insts, const BatchTile *tiles, int ntiles, int par,
                            cudaStream_t s);
cudaError_t launch_batch_mp_list(const BatchInst *insts, const BatchTile *tiles, int ntiles, int par, int grid,
                                 int tpc, BatchTicket *tk, cudaStream_t s);
// the same for boxes with slab tiles (tile start = slab tile index within the box)
cudaError_t launch_batch_mp_slab(const BatchInst *insts, const BatchTile *tiles, int ntiles, int par,
                                 cudaStream_t s);
constexpr int BATCH_SLAB_ZC = 16;   // planes per slab tile
// slab tiles of a box (0: not eligible)
__host__ __device__ inline int batch_slab_tiles(int lx, int ly, int lz)
{
    if (lx < MPS_TX || ly < MPS_TY || lz < 3) return 0;
    return ((lx + MPS_TX - 1) / MPS_TX) * ((ly + MPS_TY - 1) / MPS_TY) * ((lz + BATCH_SLAB_ZC - 1) / BATCH_SLAB_ZC);
}
// Shared-memory boxes: list holds nflow boxes in the flow phase, then nmp in the tracer phase,
// each group with its own dynamic shared memory size.  du: one word per descriptor, max
// |u - u_prev| of the flow check as IEEE bits (non-negative).
cudaError_t launch_batch_smem(const BatchInst *insts, const int *list, int nflow, int nmp, int nsteps,
                              bool check, unsigned *du, int bytes_flow, int bytes_mp, int threads,
                              cudaStream_t s);
cudaError_t launch_batch_check(const BatchInst *insts, const BatchTile *tiles, int ntiles,
                               unsigned *du, cudaStream_t s);
// density and flux of one box at every lattice node (compact boxes: the caller zeroes the
// outputs first, solid nodes stay zero)
cudaError_t launch_batch_moments(const BatchInst *insts, int inst, unsigned units, double *rho, double *jx,
                                 double *jy, double *jz, cudaStream_t s);
// start of the tracer phase of one box (units = batch_units): V from the flow state, P(t=1) and
// VACF(0) per tile
cudaError_t launch_batch_mp_start(const BatchInst *insts, int inst, unsigned units, cudaStream_t s);
cudaError_t batch_configure(int max_smem_bytes);

}  // namespace lbg
