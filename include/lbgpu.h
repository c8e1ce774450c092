/*
 * lbgpu.h -- C ABI of the GB300 (sm_103a) lattice-Boltzmann library for laboetie.
 *
 * The Fortran host of laboetie (maxlevesque/laboetie) keeps lb.in parsing, geometry and all
 * output; through iso_c_binding it calls these entry points in place of its hot loops:
 *
 *   collide / bounce-back / streaming / moments   src/module_collision.f90:15,
 *                                                 src/equilibration.f90:143-491
 *   tracer moment propagation + VACF              src/drop_tracers.f90:63-123,
 *                                                 src/module_moment_propagation.f90:30-289
 *   Poisson solve + Nernst-Planck update          src/sor.f90:7-91, src/just_eq_smolu.f90:6-135,
 *                                                 src/poisson_nernst_planck.f90:38-48
 *
 * Conventions
 *   - Every host array is a 1-based Fortran array passed by address: column-major, x fastest.
 *     A field f(lx,ly,lz) has element (i,j,k) at f[(i-1) + lx*((j-1) + ly*(k-1))].
 *     Flow populations are n(lx,ly,lz,19) (equilibration.f90 layout, velocity slowest).
 *     Tracer quantities P(3,lx,ly,lz) have the component fastest (module_moment_propagation.f90:138).
 *   - nature: int8, 0 = fluid, 1 = solid (module_system.f90:32).
 *   - Velocity index l is the reference's order (module_lbmodel.f90:68-86).
 *   - Every function returns an int status: 0 = LBGPU_OK, otherwise a bit mask of
 *     lbgpu_status; lbgpu_last_error() gives the message.  The reference has no error returns
 *     (it STOPs), so the Fortran shim maps a non-zero status to ERROR STOP.
 *   - A context owns all device memory and one CUDA stream; it is not thread-safe.  One context
 *     per host thread.  The library never falls back to the CPU: without a usable GPU,
 *     lbgpu_create() fails with LBGPU_ERR_CUDA.
 */
#ifndef LBGPU_H
#define LBGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBGPU_ABI_VERSION 1

typedef struct lbgpu_ctx lbgpu_ctx;

/* Status bits.  Several may be set at once. */
enum lbgpu_status {
    LBGPU_OK = 0,
    LBGPU_ERR_INVALID = 1 << 0,            /* bad argument or call order */
    LBGPU_ERR_CUDA = 1 << 1,               /* CUDA runtime error, or no GPU */
    LBGPU_ERR_NEGATIVE_POPULATION = 1 << 2,/* equilibration.f90:248 "n(x,y,z,vel) < 0" */
    LBGPU_ERR_NONFINITE = 1 << 3,          /* a population or moment became NaN/Inf */
    LBGPU_ERR_FRACTION = 1 << 4,           /* module_moment_propagation.f90:249 "restpart is negative" */
    LBGPU_ERR_STEP_CAP = 1 << 5,           /* step / iteration cap reached without convergence */
    LBGPU_ERR_OOM = 1 << 6,                /* device memory budget exceeded */
    LBGPU_ERR_FLUX_SUM = 1 << 7,           /* just_eq_smolu.f90:108-112 "sum of all flux does not add up" */
    LBGPU_ERR_CHARGE = 1 << 8,             /* charge_test.f90:20-24 "charge is not conserved" */
    LBGPU_ERR_UNSUPPORTED = 1 << 9,        /* an input the reference has no defined result for */
    LBGPU_ERR_TIMEOUT = 1 << 10            /* a device-side wait ran out of its iteration limit */
};

/* Storage / arithmetic of the flow and tracer populations. */
enum lbgpu_precision {
    LBGPU_FP64 = 0,      /* plain FP64, the reference's arithmetic operation by operation */
    LBGPU_FP32_DEV = 1,  /* FP32 deviations f - w*rho0 with FP32 collision; FP64 sums */
    LBGPU_FP64_FUSED = 2 /* FP64 storage and arithmetic, the collision regrouped per pair of
                            opposite velocities and evaluated with fused multiply-adds, and the
                            tracer gathers fused: within 1e-12 relative of LBGPU_FP64, not
                            bit-identical (the operator calls lbgpu_collide, lbgpu_moments and
                            lbgpu_bounce_back_stream stay operation for operation) */
};

typedef struct {
    int lx, ly, lz;              /* lb.in lx, ly, lz (equilibration.f90:40-42) */
    int precision;               /* enum lbgpu_precision */
    double relaxation_time;      /* lb.in relaxation_time (module_collision.f90:38), > 0.5 */
    double target_error;         /* lb.in target_error (equilibration.f90:57), default 1e-10 */
    double f_ext[3];             /* lb.in f_ext (equilibration.f90:379, drop_tracers.f90:92) */
    double rho0;                 /* lb.in initialSolventDensity (init_simu.f90:31) */
    int device;                  /* CUDA device ordinal */
} lbgpu_params;

/* Fill *p with the reference defaults for a lx*ly*lz box (tau 1, target 1e-10, rho0 1). */
void lbgpu_default_params(lbgpu_params *p, int lx, int ly, int lz);

/* Create a context for one box: copies the geometry to the device, classifies every node
 * (fluid/solid, interfacial as supercell_definition.f90:115-147) and allocates the flow state.
 * Replaces the allocations of equilibration.f90:59-119. */
int lbgpu_create(const lbgpu_params *p, const int8_t *nature, lbgpu_ctx **out);
void lbgpu_destroy(lbgpu_ctx *ctx);

/* Copy the message of the last failed call into buf (always NUL-terminated). */
int lbgpu_last_error(const lbgpu_ctx *ctx, char *buf, size_t len);

/* ---------------------------------------------------------------- geometry */

/* detectInterfacialNodes (supercell_definition.f90:115-147): out[node] = 1 if any of the 18
 * periodic neighbours has a different nature, else 0. */
int lbgpu_interfacial(lbgpu_ctx *ctx, uint8_t *out);

/* counts[0..3] = fluid, solid, fluid&interfacial, solid&interfacial node counts. */
int lbgpu_node_counts(lbgpu_ctx *ctx, long long counts[4]);

/* ---------------------------------------------------------------- geometry on the device
 * The builders of module_geometry.f90 selected by geometryLabel (supercell_definition.f90:52-80)
 * evaluated on the GPU: -1 no solid, 1 slit, 2 cylinder, 3 cc, 4 disc, 5 sinusoidal walls,
 * 6 planes with two radii, 7 tube with varying diameter (params = {lw_o_lx, a_o_R}, the two
 * numbers of tube.in), 8 spherical cavity, 9 sphere, 10 cylinders between walls; the others take
 * params = NULL.  Distances are gfortran's NORM2 with separately rounded operations, so every
 * node falls on the reference's side of each threshold.  Labels 0 (geom.in) and 11 (geom.pbm)
 * read files: the host parses them and passes nature to lbgpu_create.
 * The reference's STOP conditions (e.g. label 2 with lx /= ly) and a box without fluid node
 * ("All nodes are solid: no fluid, no fluid dynamics!", supercell_definition.f90:92-94) return
 * LBGPU_ERR_INVALID with the reference's message in lbgpu_last_error(NULL, ...); they are
 * checked before any device work, so they are reported without a GPU too.
 * lbgpu_geometry writes nature(lx,ly,lz) (0 fluid, 1 solid, x fastest) to the host array
 * nature; lbgpu_create_label is lbgpu_create on the box built on the device (p->lx, ly, lz). */
int lbgpu_geometry(int device, int label, int lx, int ly, int lz, const double *params,
                   int8_t *nature);
int lbgpu_create_label(const lbgpu_params *p, int label, const double *params, lbgpu_ctx **out);

/* ---------------------------------------------------------------- flow: state transfer */

/* init_simu.f90:31-39 on the device: density = rho0 on fluid, 0 on solid; n_l = w_l*density;
 * j = 0 and the force field = 0 (equilibration.f90:75-80,94-96). */
int lbgpu_flow_init(lbgpu_ctx *ctx);

/* n(lx,ly,lz,19), density, jx, jy, jz: host <-> device copies of the device-resident state.
 * After lbgpu_flow_steps / lbgpu_equilibration, get returns the populations n after the last
 * streaming and the moments of that step (the reference's state at loop exit). */
int lbgpu_flow_set(lbgpu_ctx *ctx, const double *n, const double *density, const double *jx,
                   const double *jy, const double *jz);
int lbgpu_flow_get(lbgpu_ctx *ctx, double *n, double *density, double *jx, double *jy,
                   double *jz);

/* ---------------------------------------------------------------- flow: reference operators
 * One call = one reference operator on host arrays (copied in and out on every call).  These
 * let the Fortran loop of equilibration.f90 stay as it is, statement for statement. */

/* collide(n, density, jx, jy, jz, f_ext_x, f_ext_y, f_ext_z), module_collision.f90:15-108:
 * n (lx,ly,lz,19) is updated in place on fluid nodes. */
int lbgpu_collide(lbgpu_ctx *ctx, double *n, const double *density, const double *jx,
                  const double *jy, const double *jz, const double *f_ext_x,
                  const double *f_ext_y, const double *f_ext_z);

/* Halfway bounce-back swap + periodic streaming, equilibration.f90:204-243: n in place. */
int lbgpu_bounce_back_stream(lbgpu_ctx *ctx, double *n);

/* equilibration.f90:248,254,266-268,293-300,339-343: density = SUM(n,4);
 * j = f_ext/2 + sum_l n_l c_l; *l2err = max|j - j_old| with j_old read from jx/jy/jz on entry
 * (a NaN difference makes l2err NaN).  Returns LBGPU_ERR_NEGATIVE_POPULATION if any n < 0 and
 * LBGPU_ERR_NONFINITE if any n is NaN or infinite (results are still written). */
int lbgpu_moments(lbgpu_ctx *ctx, const double *n, const double *f_ext_x,
                  const double *f_ext_y, const double *f_ext_z, double *density, double *jx,
                  double *jy, double *jz, double *l2err);

/* ---------------------------------------------------------------- flow: device-resident loop */

enum lbgpu_flow_mode {
    LBGPU_FLOW_FIXED = 0,     /* nsteps steps with the current force, no convergence test */
    LBGPU_FLOW_REFERENCE = 1  /* equilibration.f90:143-491 semantics, see lbgpu_equilibration */
};

/* Run the flow phase of equilibration.f90:143-491 on the device: fused collide + bounce-back +
 * stream + moments + l2err each step, the two-phase f_ext state machine (force switched on at
 * the first convergence, exit at the second) evaluated on the device between steps.
 * Stops at convergence or after max_steps (LBGPU_ERR_STEP_CAP).  l2err_hist (optional,
 * capacity hist_cap) receives l2err(t) for t = 1..steps (the output/l2err.dat series).
 * *steps_out = the exit step t.  FP64 contexts: bit-identical to the reference.  FP32-deviation
 * contexts: the same loop in FP32 (a check after each in-place step, l2err from FP64 moments);
 * l2err cannot fall below the FP32 resolution of j (about 1e-7 of |j|), so a target_error under
 * that is never met and the loop ends at max_steps. */
int lbgpu_equilibration(lbgpu_ctx *ctx, int max_steps, double *l2err_hist, int hist_cap,
                        int *steps_out);

/* compensate_f_ext (equilibration.f90:388-487): the per-node field of f_ext spread over a
 * spherical particle of odd diameter centred at particle_coords (1-based; NULL or zeros: the
 * box centre), compensated by a uniform background force when geometry_label is -1.  Computed
 * on the host from the context's geometry into fx/fy/fz (lx*ly*lz each); the reference's
 * errors (even diameter, even box side, particle on a solid node) are returned as
 * LBGPU_ERR_INVALID with its message. */
int lbgpu_compensated_force_field(lbgpu_ctx *ctx, int particle_diameter,
                                  const int particle_coords[3], int geometry_label, double *fx,
                                  double *fy, double *fz);

/* Force field applied by lbgpu_equilibration from the first convergence on, instead of the
 * uniform f_ext on fluid nodes (FP64 contexts).  All three NULL: back to the uniform f_ext. */
int lbgpu_set_force_field(lbgpu_ctx *ctx, const double *fx, const double *fy, const double *fz);

/* The reference's profile output (equilibration.f90:154-176 every print_files_frequency steps,
 * 499-516 at exit), reduced on the device from the current flow state: for each plane normal to
 * axis (0 = x, 1 = y, 2 = z; L = lx, ly or lz planes), flux[3k..3k+2] = SUM of jx, jy, jz over
 * the plane and mean_density[k] = SUM(density)/MAX(COUNT(density > epsilon), 1), summed in the
 * Fortran SUM order (bit-identical to the reference on the same state). */
int lbgpu_profiles(lbgpu_ctx *ctx, int axis, double *flux, double *mean_density);

/* Fixed-step flow: nsteps fused steps with the force of the given phase (0 = no force,
 * 1 = f_ext on fluid nodes), no convergence test (the timing mode). */
int lbgpu_flow_steps(lbgpu_ctx *ctx, int nsteps, int force_on);

/* Time nsteps fixed steps with CUDA events on the context's stream (one launch per step,
 * replayed from a CUDA graph).  *ms = elapsed device time. */
int lbgpu_time_flow_steps(lbgpu_ctx *ctx, int nsteps, int force_on, float *ms);

/* Wait for all work of the context. */
int lbgpu_sync(lbgpu_ctx *ctx);

/* Page-lock (pin) an existing host array so that the copies of the calls above run at full
 * host<->device bandwidth, e.g. the Fortran host's n(:,:,:,:).  Unregister before freeing it.
 * An FP32 context's lbgpu_flow_set reads populations that lie inside one registered range in
 * place (the device converts them straight from host memory, no device copy of the FP64 array). */
int lbgpu_host_register(void *ptr, size_t bytes);
int lbgpu_host_unregister(void *ptr);

/* ---------------------------------------------------------------- no-allocation variant
 * No counterpart in the reference.  For callers that cannot let the library allocate device
 * memory (their populations already live on the GPU under their own allocator, or their loop
 * runs under a fixed device-memory budget): the moments of lbgpu_moments on caller-owned
 * device arrays, with no context and no cudaMalloc.  d_n is n(lx,ly,lz,19); d_jx/d_jy/d_jz hold
 * j_old on entry and j on exit; *l2err (host, optional) = max|j - j_old|.  Outputs and status
 * bits are those of lbgpu_moments, non-finite input included.  Boxes of more than
 * 16,777,216 nodes (256^3) are rejected (LBGPU_ERR_INVALID): the reduction scratch is a fixed
 * ~1 MiB device array per GPU, shared by all calls, so calls that overlap on the GPU race.
 * stream: a cudaStream_t, or NULL for the default stream.  Every call waits for its stream
 * before it returns, so it cannot be captured into a CUDA graph. */
int lbgpu_moments_noalloc(int lx, int ly, int lz, const double *d_n, const double *d_fx,
                          const double *d_fy, const double *d_fz, double *d_density,
                          double *d_jx, double *d_jy, double *d_jz, double *l2err, void *stream);

/* ---------------------------------------------------------------- tracer moment propagation */

/* The lb.in tracer tags (drop_tracers.f90:88-92, module_moment_propagation.f90:41-71). */
typedef struct {
    double Db;             /* tracer_Db, bulk diffusion coefficient (> epsilon) */
    double ka, kd;         /* tracer_ka, tracer_kd adsorption / desorption rates (>= 0) */
    double Ds;             /* tracer_Ds, must be 0 as in the reference */
    double z;              /* tracer_z; lbgpu_mp_init refuses z != 0 as the reference does */
    double f_ext[3];       /* lb.in f_ext, added to the flux of the tracer populations */
    double elec_slope[3];  /* system elec_slope (0 unless the PNP stage read it) */
} lbgpu_tracer;

/* update_tracer_population + moment_propagation::init (drop_tracers.f90:63-123,
 * module_moment_propagation.f90:30-160): builds the tracer populations from the flow moments,
 * the scattering probabilities (fermi = 1/2), P(t=1) and VACF(t=0) (written to vacf0).
 * density/jx/jy/jz are node%solventDensity/solventFlux as host arrays, or all NULL to use the
 * moments of the context's own flow state (after lbgpu_equilibration).  Propagation runs in the
 * context's precision.  A remaining fraction below epsilon is reported by the first
 * lbgpu_mp_propagate (module_moment_propagation.f90:249,257), as the reference stops there. */
int lbgpu_mp_init(lbgpu_ctx *ctx, const lbgpu_tracer *tracer, const double *density,
                  const double *jx, const double *jy, const double *jz, double vacf0[3]);

/* lbgpu_mp_init for a charged tracer (tracer->z != 0), which the reference refuses
 * (module_moment_propagation.f90:71-79) although it holds the formulas; no counterpart call.
 * The potential is the context's Poisson-Nernst-Planck phi (after lbgpu_pnp_init and
 * lbgpu_poisson_nernst_planck, or lbgpu_pnp_set; LBGPU_ERR_INVALID without one), with
 * tracer->elec_slope.  Pstat = SUM(exp(-z phi)) over fluid nodes + SUM(exp(-z phi) K) over
 * interfacial fluid nodes, in Fortran SUM order (:97-101); each node's Boltzmann weight
 * exp(-z phi)/Pstat (:110); each link's fermi = 1/(1 + exp(z dphi)), dphi = phi(r') - phi(r)
 * plus the elec_slope term of a link across the periodic boundary (:295-322); P(t=1) with the
 * factor exp(-z dphi) (:123-135).  The steps are lbgpu_mp_propagate's.  z = 0 is lbgpu_mp_init. */
int lbgpu_mp_init_charged(lbgpu_ctx *ctx, const lbgpu_tracer *tracer, const double *density,
                          const double *jx, const double *jy, const double *jz, double vacf0[3]);

/* moment_propagation::propagate (module_moment_propagation.f90:164-289) for steps it = k+1 ...
 * k+nsteps, stopping early once converged (it > 2 and |VACF| < min(Db/(2 lx ly lz), 1e-12)).
 * vacf (optional, capacity 3*nsteps) receives VACF(it) for each step run (vacf.dat rows);
 * *steps_done the number of steps run, *is_converged the convergence flag. */
int lbgpu_mp_propagate(lbgpu_ctx *ctx, int nsteps, double *vacf, int *steps_done,
                       int *is_converged);

/* Current P(3,lx,ly,lz) and adsorbed part (zeros when no adsorption); either may be NULL.
 * Together with lbgpu_mp_set: a checkpoint of the tracer phase. */
int lbgpu_mp_get(lbgpu_ctx *ctx, double *P, double *P_ads);

/* Resume a tracer phase from a checkpoint (no counterpart in the reference, which has none):
 * after lbgpu_mp_init with the same tracer on the same flow moments, P and (with adsorption, else
 * ignored and may be NULL) P_ads become the propagated quantity, as lbgpu_mp_get returned them,
 * and it_next (>= 1) the reference's step counter it of the next lbgpu_mp_propagate (its
 * convergence test starts at it > 2).  K steps, lbgpu_mp_get, then lbgpu_mp_init + lbgpu_mp_set
 * in another context and K more steps give the bits of 2K steps in one run (FP32 values make the
 * round trip through FP64 exactly). */
int lbgpu_mp_set(lbgpu_ctx *ctx, const double *P, const double *P_ads, int it_next);

/* deallocate_propagated_quantity (module_moment_propagation.f90:350-353). */
int lbgpu_mp_release(lbgpu_ctx *ctx);

/* Time nsteps propagation steps (convergence test disabled) with CUDA events. */
int lbgpu_time_mp_steps(lbgpu_ctx *ctx, int nsteps, float *ms);

/* ---------------------------------------------------------------- batches of boxes, serving
 * No counterpart in the reference, which runs one lb.in per process.
 * Many independent boxes (cells) of any size stepped together in FP32 deviations with in-place
 * streaming, each in one of two phases: flow, then (optionally) the moment propagation of a
 * neutral tracer in the box's final flow field (the single box's FP32 tracer arithmetic: given
 * the same flow moments, P is bit-identical to lbgpu_mp_get's).  Large boxes are stepped by one tiled launch
 * per step and phase, boxes of up to ~2,700 nodes by one block each that keeps the box in
 * shared memory for all the steps of a call; one call's launches run as a CUDA graph.  The
 * force acts from the first step on (a steady-state solve, no two-phase loop); the convergence
 * test is max|u - u_prev| between two checks.  A box's results do not depend on the other
 * boxes in the batch.  Errors of these calls are read with lbgpu_last_error(NULL, ...). */
typedef struct lbgpu_batch lbgpu_batch;

typedef struct {
    int lx, ly, lz;
    double relaxation_time;
    double f_ext[3];
    double rho0;
    lbgpu_tracer tracer;   /* Db = 0: no tracer phase; else a neutral tracer (z = 0, Ds = 0) */
} lbgpu_cell;

/* memory_budget: bytes of device memory the batch may hold (0 = 90 % of the free memory). */
int lbgpu_batch_create(int device, size_t memory_budget, lbgpu_batch **out);
void lbgpu_batch_destroy(lbgpu_batch *b);
/* Device bytes a box of this cell takes (its share of the memory budget). */
size_t lbgpu_batch_footprint(const lbgpu_cell *cell);
/* Add a box at rest (rho = rho0, j = 0) in the flow phase; *id is its slot.  LBGPU_ERR_OOM
 * beyond the budget. */
int lbgpu_batch_add(lbgpu_batch *b, const lbgpu_cell *cell, const int8_t *nature, int *id);
/* lbgpu_batch_add of the box of geometryLabel `label` (cell->lx, ly, lz; params as for
 * lbgpu_geometry), built on the batch's device: no host geometry. */
int lbgpu_batch_add_label(lbgpu_batch *b, const lbgpu_cell *cell, int label, const double *params,
                          int *id);
int lbgpu_batch_remove(lbgpu_batch *b, int id);
/* nsteps (even) steps of every box in its phase; with check, du[id] = max|u - u_prev| per slot
 * of the flow-phase boxes (u_prev: the velocity at the previous check, 0 at the first). */
int lbgpu_batch_steps(lbgpu_batch *b, int nsteps, int check, float *du);
int lbgpu_batch_time_steps(lbgpu_batch *b, int nsteps, float *ms);
/* density and flux (FP64) of box id from its flow populations */
int lbgpu_batch_moments(lbgpu_batch *b, int id, double *density, double *jx, double *jy,
                        double *jz);
/* Tracer phase of box id (drop_tracers.f90, module_moment_propagation.f90:30-160 in FP32):
 * V = (j + f_ext)/rho from the flow state, P(t=1) and VACF(0); LBGPU_ERR_FRACTION if a
 * remaining fraction is below epsilon.  The box's later steps propagate the tracer. */
int lbgpu_batch_mp_start(lbgpu_batch *b, int id);
/* VACF(0), sum of VACF(t) over the tracer steps so far, VACF of the last step (FP64 sums of
 * per-tile FP64 partials); D_eff = vacf0/2 + vacf_sum (Green-Kubo, unit time step). */
int lbgpu_batch_mp_get(lbgpu_batch *b, int id, double vacf0[3], double vacf_sum[3],
                       double vacf_last[3], int *steps);
/* Current P(3,lx,ly,lz) and adsorbed part (zeros when no adsorption) of a box in its tracer
 * phase, as lbgpu_mp_get; either may be NULL. */
int lbgpu_batch_mp_fields(lbgpu_batch *b, int id, double *P, double *P_ads);
int lbgpu_batch_info(lbgpu_batch *b, int *active, long long *fluid_nodes, int *smem_boxes,
                     size_t *bytes_used);

/* The batch tuner's choices.  The first call that holds at least 1024 flow-phase tiles times, on
 * scratch copies of the tiled boxes (their state does not advance), every variant of the even
 * and of the odd in-place step launch: one block per 256-node tile at 3..6 resident blocks per
 * SM, or a persistent work list (4..6 blocks per SM claiming 1, 2 or 4 tiles at a time from an
 * atomic ticket), and keeps the fastest; then the steps per CUDA graph of the tiled boxes' launches
 * (8, 32 or 128: the smallest within 1 % of the fastest; the shared-memory boxes step a whole call
 * in one launch); the first call with at least 64 shared-memory boxes picks their block size. */
typedef struct {
    int tuned;                    /* 1 once the tiled launches were tuned */
    int aa_work_list[2];          /* even, odd launch: 1 persistent work list, 0 block per tile */
    int aa_min_blocks[2];         /* resident blocks per SM of the chosen variant */
    int aa_tiles_per_claim[2];    /* tiles a work-list block claims at a time */
    int smem_threads;             /* threads per shared-memory-resident box */
    int steps_per_graph;          /* steps of one CUDA graph (0: one graph per call) */
    float aa_ms[2];               /* time of one launch of the chosen variant when tuned */
    long long tiled_fluid_nodes;  /* fluid nodes of the flow-phase tiled boxes it was timed on */
} lbgpu_batch_tuning;
int lbgpu_batch_get_tuning(lbgpu_batch *b, lbgpu_batch_tuning *out);

typedef struct {
    lbgpu_cell cell;
    const int8_t *nature;   /* the caller keeps it alive until lbgpu_serve returns */
    double arrival;         /* seconds after the start of lbgpu_serve */
    int max_steps;          /* flow step cap (0: none) */
    int mp_steps;           /* tracer steps after the flow (0: none; needs cell.tracer.Db > 0),
                               rounded up to whole rounds of check_every */
    double *out_density, *out_jx, *out_jy, *out_jz;   /* optional: final flow moments */
} lbgpu_request;

typedef struct {
    double admitted, finished;   /* seconds after the start; -1 if never */
    int steps, converged, status, mp_steps;
    long long fluid_nodes;
    double vacf0[3], vacf_sum[3];
} lbgpu_request_result;

/* result status: 0, or LBGPU_ERR_STEP_CAP (flow capped before converging; its tracer steps still
 * ran), LBGPU_ERR_NONFINITE (its flow produced a non-finite velocity; it left at once),
 * LBGPU_ERR_FRACTION (tracer start refused), LBGPU_ERR_OOM (can never fit the budget),
 * LBGPU_ERR_INVALID / LBGPU_ERR_UNSUPPORTED (refused cell).  Other requests are unaffected. */
/* Request server (continuous batching) on an empty batch: a request is admitted once it has
 * arrived and its buffers fit the batch's memory budget (in arrival order), is stepped with all
 * resident boxes in rounds of check_every steps, ends its flow when du < du_tol at a check
 * after the first or at its step cap, then runs its tracer steps, and leaves.  Admission,
 * phase changes and departures happen between rounds, so requests that arrive while others
 * run join the next round. */
int lbgpu_serve(lbgpu_batch *b, const lbgpu_request *requests, int n, double du_tol,
                int check_every, lbgpu_request_result *results);

/* ---------------------------------------------------------------- Poisson + Nernst-Planck */

enum lbgpu_poisson_solver {
    LBGPU_POISSON_REFERENCE = 0,  /* sor.f90: over-relaxed Jacobi, omega 1.4, stop when
                                     sum|phi* - phi| <= 1e-5 * anormf0 (bit-identical sweeps) */
    LBGPU_POISSON_SOR4 = 1,       /* multicolour successive over-relaxation of the same discrete
                                     equation with the given omega and tol: 4 colours when lx, ly,
                                     lz are even, up to 9 otherwise (2 for a 1 x 1 x even column),
                                     so any box shape is coloured; stops on the reference's
                                     measure, sum|phi* - phi| <= tol * anormf0, with phi* the
                                     Jacobi target at each node as it is updated */
    LBGPU_POISSON_JACOBI = 2      /* the reference's Jacobi sweep with the given omega and tol
                                     (stop when sum|phi* - phi| <= tol * anormf0) */
};

/* The lb.in tags of the charged system (charges_init.f90:23-134, poisson_nernst_planck.f90). */
typedef struct {
    double bjl, sigma, lambda_D, D_plus, D_minus;
    int charge_distrib;   /* 0 = 'int' (charge on interfacial solid nodes); 1 = 'sol' (refused,
                             as the reference stops on it) */
    int solver;           /* enum lbgpu_poisson_solver */
    double omega, tol;    /* LBGPU_POISSON_SOR4 and LBGPU_POISSON_JACOBI */
    int max_iter;         /* sweeps per solve; 0 = the reference's 500 000 */
    int np_loop_bug;      /* 1: Nernst-Planck links start only on the line (i, ly, lz), as the
                             loop bounds of just_eq_smolu.f90:68-70 do; 0: every site */
} lbgpu_pnp_params;

/* charges_init.f90:23-135: c+, c- on the device, phi = 0; *anormf0 as the reference. */
int lbgpu_pnp_init(lbgpu_ctx *ctx, const lbgpu_pnp_params *p, double *anormf0);
int lbgpu_pnp_set(lbgpu_ctx *ctx, const double *c_plus, const double *c_minus, const double *phi,
                  double anormf0);
int lbgpu_pnp_get(lbgpu_ctx *ctx, double *c_plus, double *c_minus, double *phi, double *anormf0);

/* sor.f90:7-91 (then anormf0 = sum|phi|).  *iters = the count the reference prints (iter-1). */
int lbgpu_sor(lbgpu_ctx *ctx, int *iters);

/* just_eq_smolu.f90:6-135 (eD = 0.1 D, at most 10 iterations, since time = 0 there). */
int lbgpu_just_eq_smolu(lbgpu_ctx *ctx, int *iters);

/* poisson_nernst_planck.f90:38-48 (until the relative changes of phi, c+ and c- are all below
 * 1e-12, or max_outer iterations: LBGPU_ERR_STEP_CAP), then charge_test.f90. */
int lbgpu_poisson_nernst_planck(lbgpu_ctx *ctx, int max_outer, int *outer, int *sor_iters_total);

/* The residual of the discrete Poisson equation at the current phi, without changing it:
 * *residual = sum over every node of |phi* - phi| (phi* the Jacobi target of sor.f90:54-62), the
 * quantity the reference's stopping test compares with 1e-5 * anormf0; *anormf0 (optional) is
 * the state's normalisation.  Solvers are compared on it at equal tolerance. */
int lbgpu_poisson_residual(lbgpu_ctx *ctx, double *residual, double *anormf0);

/* charge_test.f90:15-24: charges on solid and fluid nodes; LBGPU_ERR_CHARGE if they differ from
 * sigma and -sigma by more than 1e-10. */
int lbgpu_charge_test(lbgpu_ctx *ctx, double *solid_charge, double *fluid_charge);

/* ---------------------------------------------------------------- coupled electrokinetics
 * The operators of the reference's coupled electrokinetic time loop (its only driver,
 * src/trash/equilibration_without_constraint.f90:26-34, no longer builds), one call per
 * subroutine, on the context's charged-solute state (after lbgpu_pnp_init or lbgpu_pnp_set):
 * the potential phi, the ion densities c+ and c-, and the reference's module variables phi_tot,
 * solute_force(lx,ly,lz,3) (accumulated over lbgpu_smolu calls, zero at the first) and advect's
 * flux_site arrays (accumulated over lbgpu_advect calls: the reference allocates them once and
 * never resets them).  Host arrays jx/jy/jz are node%solventFlux(x:z). */

/* electrostatic_pot.f90:7-21: phi_tot = phi + sum(elec_slope*[i,j,k]) (1-based node indices),
 * or phi when elec_slope is all zero. */
int lbgpu_electrostatic_pot(lbgpu_ctx *ctx, const double elec_slope[3]);

/* comp_j.f90:14-27: j = 0.5*(j + sum_l n(:,:,:,l)*c_l) at every node (n(lx,ly,lz,19) host
 * array; jx, jy, jz updated in place). */
int lbgpu_comp_j(lbgpu_ctx *ctx, const double *n, double *jx, double *jy, double *jz);

/* smolu.f90:1-144 with phi_tot (lbgpu_electrostatic_pot first): the fluid-fluid link fluxes of
 * c+ and c- (with the elec_slope correction of links across the periodic boundary and the
 * lncb_slope salt gradient), c+- += the site fluxes on fluid nodes, solute_force += the force of
 * the solutes on the fluid, el_curr / ion_curr (in/out) += the currents divided by D_iter, then,
 * when time > 0, divided by n_fluidsites = sum(node%nature, mask=fluid), which is 0 in the
 * reference (so the currents become +-Inf or NaN there and here).  LBGPU_ERR_FLUX_SUM with the
 * reference's message if a site-flux sum exceeds 1.0e-12 (the densities are updated first). */
int lbgpu_smolu(lbgpu_ctx *ctx, int time, int D_iter, const double elec_slope[3],
                const double lncb_slope[3], double el_curr[3], double ion_curr[3]);

/* advect.f90:2-116: volumetric advection of c+ and c- by the solvent flux j; el_curr / ion_curr
 * (in/out) as the reference sets them (its branch for c+ + c- = 0 zeroes el_curr).  The
 * reference reads ip_all(ix) of an array declared ip_all(3) with ix = -1, 0, 1 (advect.f90:57-66),
 * which has no defined result for -1 and 0; the library takes the neighbour pbc(i + ix) that
 * the code around it intends.  LBGPU_ERR_CHARGE with the reference's message if a total
 * concentration changes by more than 1.e-8 (the densities are updated first). */
int lbgpu_advect(lbgpu_ctx *ctx, const double *jx, const double *jy, const double *jz,
                 double el_curr[3], double ion_curr[3]);

/* phi_tot(lx,ly,lz) and solute_force(lx,ly,lz,3) (zeros before the first lbgpu_smolu); either
 * may be NULL. */
int lbgpu_ek_get(lbgpu_ctx *ctx, double *phi_tot, double *solute_force);

#ifdef __cplusplus
}
#endif
#endif
