// pnp.h -- device state of the charged-solute operators of a context: the Poisson-Nernst-Planck
// equilibration (pnp.cu) and the coupled electrokinetic operators (ek.cu) share the potential and
// the ion densities (the reference's module variables phi, c_plus, c_minus, phi_tot and their
// previous values, module_system.f90:79-84).
#pragma once

#include <cuda_runtime.h>

#include <condition_variable>
#include <mutex>
#include <thread>
#include <vector>

#include "lbgpu.h"

namespace lbg {

struct PnpCtl {
    int iter, done, converged, parity;
    int max_iter;
    unsigned blocks_done;
    double anorm, limit;  // stop when anorm <= limit
};

struct PnpState {
    lbgpu_pnp_params p{};
    double *phi[2] = {nullptr, nullptr};
    double *cp = nullptr, *cm = nullptr;
    double *fp = nullptr, *fm = nullptr;    // flux_site_plus / flux_site_minus
    double *bak[3] = {nullptr, nullptr, nullptr};  // phi_old, c_plus_old, c_minus_old
    double *partial = nullptr;              // 4 per block
    double *result = nullptr;               // 4 reduced sums
    PnpCtl *ctl = nullptr;
    int par = 0;                            // buffer holding phi
    double anormf0 = 0.0, rho_ch = 0.0;
    bool charged = false;
    std::vector<void *> allocs;
    // CUDA graphs of 8 and of 64 sweeps, captured at the first solve and replayed by every later
    // one (their arguments are fixed until the state is released)
    cudaGraphExec_t sor_exec[2] = {nullptr, nullptr};
    // electrokinetic operators (ek.cu), allocated at their first use: the total potential
    // phi_tot, the force of the solutes on the fluid solute_force(lx,ly,lz,3) (accumulated over
    // smolu calls, as the reference's module variable), and advect's flux_site_plus / minus,
    // module variables of the reference that advect allocates once and never resets
    double *phi_tot = nullptr;
    double *solute_force = nullptr;
    double *adv_fp = nullptr, *adv_fm = nullptr;
    // page-locked host copy of phi for anormf0 = SUM(ABS(phi)), summed on the host in the
    // reference's order after every solve (allocated at its first use), by a worker thread of the
    // state (pnp.cu: anorm_begin / anorm_end), so that the outer loop's Nernst-Planck update and
    // convergence test run meanwhile
    double *phi_host = nullptr;
    std::thread anorm_thread;
    std::mutex anorm_m;
    std::condition_variable anorm_cv;
    // job: a sum to start (set by anorm_begin); pending: a sum begun and not yet consumed by
    // anorm_end; ready: the worker finished it
    bool anorm_job = false, anorm_pending = false, anorm_ready = false, anorm_quit = false;
    bool anorm_failed = false;
    double anorm_sum = 0.0;
    cudaEvent_t anorm_ev = nullptr;
};

}  // namespace lbg
