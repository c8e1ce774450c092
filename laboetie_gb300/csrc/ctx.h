// ctx.h -- the library context: device allocations and host-side bookkeeping of one box.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "common.cuh"
#include "lbgpu.h"

namespace lbg {

// Small device-resident results of the operator kernels.
struct Scratch {
    unsigned long long err_bits;
    unsigned status;
    unsigned pad;
    unsigned long long counts[4];
};

// How the populations in the "previous" buffer relate to the state the host asks for.
enum PrevKind { PREV_NONE = 0, PREV_RAW = 1, PREV_POST = 2 };

// Operator-mode scratch (lbgpu_collide & co.): populations in/out, moments, force field.
struct OpBuffers {
    double *n[2] = {nullptr, nullptr};
    double *m[4] = {nullptr, nullptr, nullptr, nullptr};  // rho, jx, jy, jz
    double *F[3] = {nullptr, nullptr, nullptr};
};

struct MpState;   // tracer moment propagation (mp.cu)
struct PnpState;  // Poisson-Nernst-Planck (pnp.cu)

}  // namespace lbg

struct lbgpu_ctx {
    lbgpu_params p{};
    long long N = 0;
    unsigned long long counts[4] = {0, 0, 0, 0};
    std::string last_error;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    // geometry
    int8_t *d_nature = nullptr;
    uint32_t *d_mask = nullptr;

    // FP64 contexts: the lattice indices of the fluid nodes in lattice order (counts[0] of them);
    // the FP64 step kernels run one thread per entry, so no lane of a warp idles on a solid node
    uint32_t *d_fidx = nullptr;

    // flow state.  FP64: d_f[2] doubles; FP32 deviation: d_g[2] floats.
    double *d_f[2] = {nullptr, nullptr};
    float *d_g[2] = {nullptr, nullptr};
    double *d_j[3] = {nullptr, nullptr, nullptr};
    double *d_rho = nullptr;
    // per-node force field applied from the first convergence on (compensate_f_ext), or null
    double *d_F[3] = {nullptr, nullptr, nullptr};
    lbg::FlowCtl *d_ctl = nullptr;
    lbg::Scratch *d_scratch = nullptr;
    lbg::LbConst64 K64{};

    int cur = 0;                 // buffer read by the next step
    int prev_kind = lbg::PREV_NONE;
    int prev_force_moment = 0;   // f_ext in the moments of the state held in buffer 1-cur
    int force_last_collide = 0;  // f_ext in the collision that produced buffer cur
    bool moments_valid = false;  // d_rho / d_j hold the moments of the state
    // FP32 deviations: in-place AA streaming (one buffer) unless LBGPU_FP32_STREAMING=ab
    bool aa = true;
    int aa_phase = 0;            // parity of the next AA launch (1: buffer holds swapped f*)
    int aa_minb[2] = {4, 4};     // AA kernel variants for even / odd launches
    bool aa_minb_fixed = false;  // set by LBGPU_AA_MINB
    bool aa_tuned = false;
    // AA layout: only the Nf fluid nodes are stored, in lattice order (compact index i);
    // cpos[i] = x | y << xbits | z << (xbits + ybits), cmask[i] = flag word,
    // rowtab[row*nw + w] = {fluid bits of word w of lattice row y + ly*z, compact index of the
    // first fluid node of that word}
    unsigned Nf = 0;
    bool aa_wide = false;        // Q*Nf >= 2^32 (or LBGPU_AA_WIDE=1): 64-bit gather offsets
    int nw = 0, xbits = 0, ybits = 0;
    uint32_t *d_cpos = nullptr, *d_cmask = nullptr;
    uint2 *d_rowtab = nullptr;

    // cached CUDA graphs of the step loop
    cudaGraphExec_t graph_ref = nullptr;
    int graph_ref_len = 0;
    cudaGraphExec_t graph_fixed[2] = {nullptr, nullptr};  // [force_on], two steps each
    int graph_fixed_parity[2] = {-1, -1};

    lbg::OpBuffers *op = nullptr;
    lbg::MpState *mp = nullptr;
    lbg::PnpState *pnp = nullptr;
};

namespace lbg {

int ctx_fail(lbgpu_ctx *ctx, int code, const std::string &msg);
int ctx_cuda(lbgpu_ctx *ctx, cudaError_t e, const char *what);
// The status of a moments operator from the bits its kernel raised: LBGPU_ERR_NEGATIVE_POPULATION
// (the reference's stop, equilibration.f90:248) and/or LBGPU_ERR_NONFINITE, with their message.
int moments_status(lbgpu_ctx *ctx, unsigned raised);
int ctx_init_device(lbgpu_ctx *ctx, const int8_t *nature);
void ctx_release_device(lbgpu_ctx *ctx);
LbConst64 make_const64(double tau);
struct FlowArgs64;
void fill_args64(lbgpu_ctx *ctx, FlowArgs64 &a);
int force_mask(const double f[3]);
void mp_release(lbgpu_ctx *ctx);
void pnp_release(lbgpu_ctx *ctx);
// device potential phi of the Poisson-Nernst-Planck state (N doubles), or null without one
const double *pnp_potential(const lbgpu_ctx *ctx);
// The device address of the host range [p, p + bytes) if it lies inside one range page-locked by
// lbgpu_host_register (kernels may then read it in place), else null.
const void *pinned_device_view(const void *p, size_t bytes);

#define LBG_CK(ctx, call)                                                   \
    do {                                                                    \
        cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess) return ::lbg::ctx_cuda((ctx), e_, #call);   \
    } while (0)

}  // namespace lbg
