/*
 * lb_oracle.h -- CPU restatement of laboetie's lattice-Boltzmann hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU library is checked against: only the
 * test suite, the smoke check and the CPU-baseline leg of bench.py load it.  The product
 * library (liblbgpu) never links or calls it.
 *
 * Conventions
 *   - Node (i,j,k), 0-based, is stored at  node = i + lx*(j + ly*k)  (Fortran column-major).
 *   - Flow populations n(x,y,z,l) at  n[node + N*l]  (N = lx*ly*lz, l = 0..18).
 *   - Tracer populations n(l,x,y,z) at  n[l + 19*node].
 *   - Tracer propagated quantity P(c,x,y,z) at  P[c + 3*node]  (c = x,y,z).
 *   - l is 0-based here: l = Fortran l - 1.  Velocity order as module_lbmodel.f90:68-86.
 *   - nature: 0 = fluid, 1 = solid (module_system.f90:32).
 *
 * Every function cites the reference source it restates.
 */
#ifndef LB_ORACLE_H
#define LB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ORC_OK = 0,
    ORC_ERR_NEGATIVE_POPULATION = 1,   /* equilibration.f90:248 */
    ORC_ERR_MAX_STEPS = 2,             /* safety cap reached (the reference would loop on) */
    ORC_ERR_BAD_INPUT = 3,             /* an ERROR STOP / STOP on input in the reference */
    ORC_ERR_FRACTION = 4,              /* module_moment_propagation.f90:249,257 */
    ORC_ERR_NOT_CONVERGED = 5,         /* sor.f90:83 */
    ORC_ERR_FLUX_SUM = 6,              /* just_eq_smolu.f90:108-112 */
    ORC_ERR_CHARGE = 7                 /* charge_test.f90:20-24 */
};

/* module_lbmodel.f90:66-86,122-162 */
void orc_lbm_tables(int c[19][3], int inv[19], double a0[19], double a1[19], double a2[19],
                    double delta[19]);

/* supercell_definition.f90:115-147 (detectInterfacialNodes) */
void orc_detect_interfacial(int lx, int ly, int lz, const int8_t *nature, uint8_t *interfacial);

/* init_simu.f90:31-39: density = svden on non-solid, 0 on solid; n(:,:,:,l) = density*a0(l) */
void orc_init_populations(int lx, int ly, int lz, const int8_t *nature, double svden,
                          double *n, double *density);

/* module_collision.f90:15-108 (second-order branch; first_order_only is refused, see .c) */
int orc_collide(int lx, int ly, int lz, const int8_t *nature, double relaxation_time,
                double *n, const double *density, const double *jx, const double *jy,
                const double *jz, const double *fx, const double *fy, const double *fz);

/* equilibration.f90:204-243: halfway bounce-back swap followed by periodic push streaming */
void orc_bounce_back_stream(int lx, int ly, int lz, const int8_t *nature, double *n,
                            int nthreads);

/* equilibration.f90:248,254,266-268,293-300,339-343: n<0 check, density, j, l2err.
 * j_old is read from jx/jy/jz on entry; returns ORC_ERR_NEGATIVE_POPULATION on n<0. */
int orc_moments(int lx, int ly, int lz, const double *n, const double *fx, const double *fy,
                const double *fz, double *density, double *jx, double *jy, double *jz,
                double *l2err);

typedef struct {
    int lx, ly, lz;
    double relaxation_time;   /* module_collision.f90:38 */
    double target_error;      /* equilibration.f90:57 */
    double f_ext[3];          /* equilibration.f90:379 */
    int compensate_f_ext;     /* equilibration.f90:123 */
    int particle_diameter;    /* equilibration.f90:389 (dominika_particle_diameter) */
    int particle_coords[3];   /* equilibration.f90:414 (1-based; 0 = default centre) */
    int geometry_label;       /* equilibration.f90:442 */
    int max_steps;            /* safety cap on t; 0 = no cap */
    int fixed_steps;          /* >0: run exactly this many steps, no phase machine (timing) */
    int nthreads;             /* OpenMP threads for the streaming loop (equilibration.f90:227) */
} orc_flow_params;

/* equilibration.f90:143-491 and 551-555.  On entry n holds the initial populations and
 * density the initial solvent density; on exit n, density, j and the force field hold the
 * state at the exit step.  l2err_hist (optional, capacity hist_cap) receives l2err(t). */
int orc_equilibration(const orc_flow_params *p, const int8_t *nature, double *n,
                      double *density, double *jx, double *jy, double *jz, double *fx,
                      double *fy, double *fz, double *l2err_hist, int hist_cap,
                      int *steps_out);

/* drop_tracers.f90:63-105: n(l,x,y,z) from the converged flow */
void orc_update_tracer_population(int lx, int ly, int lz, const int8_t *nature,
                                  const double *density, const double *jx, const double *jy,
                                  const double *jz, const double f_ext[3], double tracer_z,
                                  double tracer_D, const double elec_slope[3], double *n_mp);

typedef struct {
    int lx, ly, lz;
    double ka, kd, K, Db, Ds, z, lambda;
    int consider_adsorption;
    double vacf[3];           /* VACF of the last step (vacf(:,past) after rotation) */
    double *P_now, *P_next;   /* 3*N each */
    double *A_now, *A_next;   /* 3*N each when adsorption is considered, else NULL */
    int nthreads;
    /* charged tracer (orc_mp_init_charged): the potential phi (N, a copy) and elec_slope */
    double *phi;
    double E[3];
} orc_mp_state;

/* module_moment_propagation.f90:30-160 (init) for a neutral tracer.  Allocates the state's
 * arrays; vacf0 receives VACF(t=0). */
int orc_mp_init(orc_mp_state *s, int lx, int ly, int lz, const int8_t *nature,
                const uint8_t *interfacial, const double *density, const double *n_mp,
                double ka, double kd, double Db, double Ds, double z, double vacf0[3]);

/* The same for a charged tracer (z != 0) in the potential phi(lx,ly,lz) with elec_slope E, by
 * the formulas the reference holds but stops before (module_moment_propagation.f90:71-79):
 * Pstat = SUM(exp(-z phi), fluid) + SUM(exp(-z phi) K, fluid .and. interfacial) (:97-101),
 * boltz_weight = exp(-z phi)/Pstat (:110), fermi = 1/(1 + exp(z dphi)) per link and
 * P(r,1) += exp(-z dphi) scattprop_p c_inv boltz_weight (:123-135), dphi with the elec_slope
 * correction of a link across the periodic boundary (:303-322).  z = 0 is orc_mp_init. */
int orc_mp_init_charged(orc_mp_state *s, int lx, int ly, int lz, const int8_t *nature,
                        const uint8_t *interfacial, const double *density, const double *n_mp,
                        double ka, double kd, double Db, double z, const double *phi,
                        const double elec_slope[3], double vacf0[3]);

/* module_moment_propagation.f90:164-289 (propagate), one step `it` (1-based). */
int orc_mp_propagate(orc_mp_state *s, int it, const int8_t *nature, const uint8_t *interfacial,
                     const double *density, const double *n_mp, double vacf_out[3],
                     int *is_converged);

void orc_mp_free(orc_mp_state *s);

/* charges_init.f90:23-135.  Returns rho_ch (system rho_ch) and anormf0. */
int orc_charges_init(int lx, int ly, int lz, const int8_t *nature, const uint8_t *interfacial,
                     double bjl, double sigma, double lambda_D, int charge_distrib_int,
                     double *c_plus, double *c_minus, double *phi, double *anormf0,
                     double *rho_ch);

/* sor.f90:7-91.  Over-relaxed Jacobi, omega = 1.4, tolerance 1e-5 (single-precision literal)
 * relative to anormf0; updates anormf0 = sum(|phi|) on exit.  iters_out = iter-1 as printed. */
int orc_sor(int lx, int ly, int lz, double sigma, double bjl, const double *c_plus,
            const double *c_minus, double *phi, double *anormf0, int *iters_out);

/* Jacobi sweeps with a caller-given omega and a caller-given tolerance, as orc_sor otherwise.
 * Used as the tightly converged reference for the fast solvers. */
int orc_sor_custom(int lx, int ly, int lz, double sigma, double bjl, const double *c_plus,
                   const double *c_minus, double *phi, double *anormf0, double omega,
                   double tol, int maxiter, int *iters_out);

/* just_eq_smolu.f90:6-135.  loop_bug != 0 reproduces the j/k loop bounds of
 * just_eq_smolu.f90:68-70 (only the line (i, ly, lz) is visited). */
int orc_just_eq_smolu(int lx, int ly, int lz, const int8_t *nature, const double *phi,
                      double *c_plus, double *c_minus, double D_plus, double D_minus,
                      double rho_ch, double sigma, int loop_bug, int *iters_out);

/* check_charge_distribution_equilibrium.f90:24-44 */
int orc_check_charge_equilibrium(int N, const double *phi, const double *phi_old,
                                 const double *c_plus, const double *c_plus_old,
                                 const double *c_minus, const double *c_minus_old,
                                 double diffs[3]);

/* charge_test.f90:15-24 */
int orc_charge_test(int N, const int8_t *nature, const double *c_plus, const double *c_minus,
                    double sigma, double *solid_charge, double *fluid_charge);

/* poisson_nernst_planck.f90:38-48 (outer loop; capped at max_outer iterations). */
int orc_pnp(int lx, int ly, int lz, const int8_t *nature, double bjl, double sigma,
            double D_plus, double D_minus, double rho_ch, int loop_bug, double *c_plus,
            double *c_minus, double *phi, double *anormf0, int max_outer, int *outer_out,
            int *sor_iters_total);

/* ----------------------------------------------------------- coupled electrokinetics
 * The operators of the reference's coupled loop (src/trash/equilibration_without_constraint.f90:
 * 26-34, a driver that no longer builds), each restated as the subroutine it is. */

/* electrostatic_pot.f90:7-21: phi_tot = phi, or phi + sum(elec_slope*[i,j,k]) (1-based i,j,k)
 * when elec_slope is not all zero. */
void orc_electrostatic_pot(int lx, int ly, int lz, const double *phi, const double elec_slope[3],
                           double *phi_tot);

/* comp_j.f90:14-27: solventFlux = 0.5*(solventFlux + sum_l n(:,:,:,l)*c_l) at every node. */
void orc_comp_j(int lx, int ly, int lz, const double *n, double *jx, double *jy, double *jz);

/* smolu.f90:1-144: link fluxes from phi_tot, c+ and c- (fluid-fluid links, with the elec_slope
 * and lncb_slope corrections), c+- += the site fluxes on fluid nodes, the currents el_curr and
 * ion_curr (in/out, accumulated, divided by n_fluidsites when time > 0) and solute_force
 * (lx,ly,lz,3, in/out, accumulated).  ORC_ERR_FLUX_SUM if a flux sum exceeds 1.0e-12. */
int orc_smolu(int lx, int ly, int lz, const int8_t *nature, const double *phi_tot,
              double *c_plus, double *c_minus, double D_plus, double D_minus, int time,
              int D_iter, const double elec_slope[3], const double lncb_slope[3],
              double el_curr[3], double ion_curr[3], double *solute_force);

/* advect.f90:2-116 with the solvent flux j: the volumetric advection of c+ and c- (flux_site
 * arrays fp, fm are the reference's module variables, kept by the caller across calls), the
 * currents (in/out).  The reference indexes ip_all(3) with ix = -1, 0, 1 (advect.f90:57-66), an
 * undefined result for -1 and 0; this restatement takes the neighbour pbc(i + ix) that the code
 * around it intends.  ORC_ERR_CHARGE if a total concentration changes by more than 1.e-8. */
int orc_advect(int lx, int ly, int lz, const int8_t *nature, const double *jx, const double *jy,
               const double *jz, double *c_plus, double *c_minus, double *fp, double *fm,
               double el_curr[3], double ion_curr[3]);

/* equilibration.f90:159-175, 504-516: mass-flux and mean-density profiles along an axis. */
void orc_profiles(int lx, int ly, int lz, const double *density, const double *jx,
                  const double *jy, const double *jz, int axis, double *flux, double *mean_density);

/* module_geometry.f90 builders selected by geometryLabel (supercell_definition.f90:52-80):
 * -1 no solid, 1 slit, 2 cylinder, 3 cc, 4 disc (Benichou), 5 sinusoidal walls, 6 planes with
 * two radii, 7 tube with varying diameter (params = {lw_o_lx, a_o_R} of tube.in), 8 spherical
 * cavity, 9 sphere (Benichou), 10 cylinders between walls.  nature(lx,ly,lz) x fastest, 0 fluid,
 * 1 solid.  Returns 0, or the number of the reference's STOP condition that the box meets
 * (1: shape, 2: parameters, 3: label outside -1..10 or file-based (0, 11), 4: no fluid node). */
int orc_geometry(int label, int lx, int ly, int lz, const double *params, int8_t *nature);

#ifdef __cplusplus
}
#endif
#endif
