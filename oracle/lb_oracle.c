/*
 * lb_oracle.c -- CPU restatement of laboetie's lattice-Boltzmann hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, the smoke check and bench.py's CPU-baseline leg
 * load this code, and only as the checker.  The product library never links or calls it.
 *
 * Parity status.  The reference (maxlevesque/laboetie) is Fortran 2008 and ships no golden
 * vectors; no Fortran compiler exists where this was written.  This restatement is therefore
 * pinned by analytic known answers (slit Poiseuille profile, mass conservation, bulk and
 * adsorbing-slit diffusion, closed-form VACF(0)) in tests/, not by outputs of the reference:
 * "parity unpinned" against the reference's own outputs.
 *
 * Arithmetic.  IEEE binary64 with no fused multiply-add (built with -ffp-contract=off), which
 * is what the reference Makefile build (-O3 -fopenmp -funroll-loops, no -march) does on
 * x86-64.  Every expression keeps the operand order and association of the Fortran source.
 * Fortran default-real literals (1.e-12, 1.0e-5, 5.e-6, 1.0e-10) are single precision in the
 * reference and are reproduced as (double)(float) values.
 *
 * Loop orders.  Array statements and DO CONCURRENT nests run in storage order (first index
 * fastest), as gfortran generates them.  The OpenMP reduction of propagate() is restated as
 * per-z-slice partial sums added in slice order, which is deterministic for any thread count.
 */
#include "lb_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define Q 19

/* module_lbmodel.f90:68-86 (D3Q19 velocity set, lmin = 1 is the rest velocity) */
static const int VC[Q][3] = {
    {0, 0, 0},  {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0}, {0, 0, 1},  {0, 0, -1},
    {1, 1, 0},  {-1, 1, 0}, {1, -1, 0}, {-1, -1, 0}, {1, 0, 1},  {-1, 0, 1}, {1, 0, -1},
    {-1, 0, -1}, {0, 1, 1},  {0, -1, 1}, {0, 1, -1}, {0, -1, -1}};

/* module_lbmodel.f90:127-136: weights and their cs^-2 / cs^-4 scalings */
static const double CSQ = 1.0 / 3.0;
#define A00 (1.0 / 3.0)
#define A01 (1.0 / 18.0)
#define A02 (1.0 / 36.0)

static double W0[Q], W1[Q], W2[Q], DELTA[Q];
static int INV[Q];
static int tables_ready = 0;

static void init_tables(void)
{
    if (tables_ready) return;
    const double a_10 = A00 / CSQ, a_11 = A01 / CSQ, a_12 = A02 / CSQ;
    const double a_20 = A00 / (2 * (CSQ * CSQ)), a_21 = A01 / (2 * (CSQ * CSQ)),
                 a_22 = A02 / (2 * (CSQ * CSQ));
    const double nnn = sqrt(2.0);
    for (int l = 0; l < Q; ++l) {
        int cls = (l == 0) ? 0 : (l < 7 ? 1 : 2);   /* module_lbmodel.f90:143-147 */
        W0[l] = cls == 0 ? A00 : (cls == 1 ? A01 : A02);
        W1[l] = cls == 0 ? a_10 : (cls == 1 ? a_11 : a_12);
        W2[l] = cls == 0 ? a_20 : (cls == 1 ? a_21 : a_22);
        DELTA[l] = cls == 0 ? 0.0 : (cls == 1 ? 1.0 : nnn);
    }
    /* module_lbmodel.f90:156-162 */
    for (int l = 0; l < Q; ++l)
        for (int li = 0; li < Q; ++li)
            if (VC[l][0] == -VC[li][0] && VC[l][1] == -VC[li][1] && VC[l][2] == -VC[li][2])
                INV[l] = li;
    tables_ready = 1;
}

void orc_lbm_tables(int c[19][3], int inv[19], double a0[19], double a1[19], double a2[19],
                    double delta[19])
{
    init_tables();
    for (int l = 0; l < Q; ++l) {
        for (int d = 0; d < 3; ++d) c[l][d] = VC[l][d];
        inv[l] = INV[l];
        a0[l] = W0[l];
        a1[l] = W1[l];
        a2[l] = W2[l];
        delta[l] = DELTA[l];
    }
}

/* module_system.f90:99-112 (pbc), 0-based: one step across the periodic boundary */
static inline int pbc0(int i, int imax)
{
    if (i < 0) return imax - 1;
    if (i >= imax) return 0;
    return i;
}

static inline long nid(int i, int j, int k, int lx, int ly) { return i + (long)lx * (j + (long)ly * k); }

/* supercell_definition.f90:115-147 */
void orc_detect_interfacial(int lx, int ly, int lz, const int8_t *nature, uint8_t *interfacial)
{
    init_tables();
    for (int i = 0; i < lx; ++i)
        for (int j = 0; j < ly; ++j)
            for (int k = 0; k < lz; ++k) {
                long r = nid(i, j, k, lx, ly);
                interfacial[r] = 0;
                for (int l = 1; l < Q; ++l) {
                    long rn = nid(pbc0(i + VC[l][0], lx), pbc0(j + VC[l][1], ly),
                                  pbc0(k + VC[l][2], lz), lx, ly);
                    if (nature[r] != nature[rn]) {
                        interfacial[r] = 1;
                        break;
                    }
                }
            }
}

/* init_simu.f90:31-39 */
void orc_init_populations(int lx, int ly, int lz, const int8_t *nature, double svden,
                          double *n, double *density)
{
    init_tables();
    long N = (long)lx * ly * lz;
    for (long r = 0; r < N; ++r) density[r] = nature[r] != 1 ? svden : 0.0;
    for (int l = 0; l < Q; ++l)
        for (long r = 0; r < N; ++r) n[r + N * l] = density[r] * W0[l];
}

/* module_collision.f90:15-108.  first_order_only (module_collision.f90:110-126) reads the
 * velocity arrays that are only allocated in the other branch (73-75), so the reference has no
 * defined result for it; it is not restated. */
int orc_collide(int lx, int ly, int lz, const int8_t *nature, double relaxation_time,
                double *n, const double *density, const double *jx, const double *jy,
                const double *jz, const double *fx, const double *fy, const double *fz)
{
    init_tables();
    if (relaxation_time < 0.5) return ORC_ERR_BAD_INPUT;   /* module_collision.f90:39 */
    long N = (long)lx * ly * lz;
    double *ux = (double *)calloc(N, sizeof(double));
    double *uy = (double *)calloc(N, sizeof(double));
    double *uz = (double *)calloc(N, sizeof(double));
    double *neq = (double *)calloc(N, sizeof(double));
    /* module_collision.f90:77-85 */
    for (long r = 0; r < N; ++r) {
        if (nature[r] == 0) {
            ux[r] = jx[r] / density[r];
            uy[r] = jy[r] / density[r];
            uz[r] = jz[r] / density[r];
        } else {
            ux[r] = 0;
            uy[r] = 0;
            uz[r] = 0;
        }
    }
    const double c1 = 1.0 - 1.0 / relaxation_time;
    const double c2 = 1.0 / relaxation_time;
    const double c3 = 1.0 - 1.0 / (2.0 * relaxation_time);
    /* module_collision.f90:87-108: one masked pass per velocity */
    for (int l = 0; l < Q; ++l) {
        const double cx = VC[l][0], cy = VC[l][1], cz = VC[l][2];
        const double a0 = W0[l], a1 = W1[l], a2 = W2[l];
        double *nl = n + N * l;
        for (long r = 0; r < N; ++r) {
            if (nature[r] != 0) continue;
            const double JX = jx[r], JY = jy[r], JZ = jz[r];
            const double UX = ux[r], UY = uy[r], UZ = uz[r];
            neq[r] = a0 * density[r] + a1 * (cx * JX + cy * JY + cz * JZ) +
                     a2 * (JX * UX * (cx * cx - CSQ) + JX * UY * cx * cy + JX * UZ * cx * cz +
                           JY * UX * cy * cx + JY * UY * (cy * cy - CSQ) + JY * UZ * cy * cz +
                           JZ * UX * cz * cx + JZ * UY * cz * cy + JZ * UZ * (cz * cz - CSQ));
            nl[r] = c1 * nl[r] + c2 * neq[r] +
                    c3 * (a1 * ((cx - UX) * fx[r] + (cy - UY) * fy[r] + (cz - UZ) * fz[r]) +
                          2.0 * a2 * (cx * UX + cy * UY + cz * UZ) *
                              (cx * fx[r] + cy * fy[r] + cz * fz[r]));
        }
    }
    free(ux);
    free(uy);
    free(uz);
    free(neq);
    return ORC_OK;
}

/* equilibration.f90:204-243 */
void orc_bounce_back_stream(int lx, int ly, int lz, const int8_t *nature, double *n,
                            int nthreads)
{
    init_tables();
    long N = (long)lx * ly * lz;
    /* equilibration.f90:204-222: swap across links whose end points differ in nature */
    for (int l = 0; l < Q; l += 2) {
        int li = INV[l];
        for (int k = 0; k < lz; ++k) {
            int kp = pbc0(k + VC[l][2], lz);
            for (int j = 0; j < ly; ++j) {
                int jp = pbc0(j + VC[l][1], ly);
                for (int i = 0; i < lx; ++i) {
                    int ip = pbc0(i + VC[l][0], lx);
                    long r = nid(i, j, k, lx, ly), rp = nid(ip, jp, kp, lx, ly);
                    if (nature[r] != nature[rp]) {
                        double t = n[r + N * l];
                        n[r + N * l] = n[rp + N * li];
                        n[rp + N * li] = t;
                    }
                }
            }
        }
    }
    /* equilibration.f90:227-243: push streaming, parallel over the velocity */
    (void)nthreads;
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) schedule(static)
    for (int l = 0; l < Q; ++l) {
        double *old = (double *)malloc(sizeof(double) * N);
        memcpy(old, n + N * l, sizeof(double) * N);
        for (int k = 0; k < lz; ++k) {
            int kp = pbc0(k + VC[l][2], lz);
            for (int j = 0; j < ly; ++j) {
                int jp = pbc0(j + VC[l][1], ly);
                for (int i = 0; i < lx; ++i) {
                    int ip = pbc0(i + VC[l][0], lx);
                    n[nid(ip, jp, kp, lx, ly) + N * l] = old[nid(i, j, k, lx, ly)];
                }
            }
        }
        free(old);
    }
}

/* equilibration.f90:248,254,266-268,293-300,339-343 */
int orc_moments(int lx, int ly, int lz, const double *n, const double *fx, const double *fy,
                const double *fz, double *density, double *jx, double *jy, double *jz,
                double *l2err)
{
    init_tables();
    long N = (long)lx * ly * lz;
    int negative = 0;
    for (long q = 0; q < N * Q; ++q)
        if (n[q] < 0) negative = 1;
    double err = 0.0;
    for (long r = 0; r < N; ++r) {
        double s = 0.0;
        for (int l = 0; l < Q; ++l) s = s + n[r + N * l];
        density[r] = s;
        double ox = jx[r], oy = jy[r], oz = jz[r];
        double X = fx[r] / 2.0, Y = fy[r] / 2.0, Z = fz[r] / 2.0;
        for (int l = 0; l < Q; ++l) {
            double nl = n[r + N * l];
            X = X + nl * (double)VC[l][0];
            Y = Y + nl * (double)VC[l][1];
            Z = Z + nl * (double)VC[l][2];
        }
        jx[r] = X;
        jy[r] = Y;
        jz[r] = Z;
        double d;
        d = fabs(X - ox); if (d > err) err = d;
        d = fabs(Y - oy); if (d > err) err = d;
        d = fabs(Z - oz); if (d > err) err = d;
    }
    if (l2err) *l2err = err;
    return negative ? ORC_ERR_NEGATIVE_POPULATION : ORC_OK;
}

/* gfortran's NORM2 (scaled sum of squares, scale starting at 1) */
static double norm2_f(const double *v, int m)
{
    double result = 0.0, scale = 1.0;
    for (int i = 0; i < m; ++i) {
        if (v[i] != 0.0) {
            double ax = fabs(v[i]);
            if (scale < ax) {
                double val = scale / ax;
                result = 1.0 + result * val * val;
                scale = ax;
            } else {
                double val = ax / scale;
                result += val * val;
            }
        }
    }
    return scale * sqrt(result);
}

/* equilibration.f90:388-487: force on a central particle, compensated or not */
static int compensate_field(const orc_flow_params *p, const int8_t *nature, double *fx,
                            double *fy, double *fz)
{
    int lx = p->lx, ly = p->ly, lz = p->lz;
    long N = (long)lx * ly * lz;
    int pd = p->particle_diameter > 0 ? p->particle_diameter : 1;
    if (pd % 2 == 0) return ORC_ERR_BAD_INPUT;
    if (lx % 2 == 0 || ly % 2 == 0 || lz % 2 == 0) return ORC_ERR_BAD_INPUT;
    int pdr = pd / 2;
    const double *fl = p->f_ext;
    for (long r = 0; r < N; ++r) fx[r] = fy[r] = fz[r] = 0.0;
    int px = p->particle_coords[0] > 0 ? p->particle_coords[0] : lx / 2 + 1;
    int py = p->particle_coords[1] > 0 ? p->particle_coords[1] : ly / 2 + 1;
    int pz = p->particle_coords[2] > 0 ? p->particle_coords[2] : lz / 2 + 1;
    int cnt = 0, err = 0;
    for (int i = px - pdr; i <= px + pdr; ++i)
        for (int j = py - pdr; j <= py + pdr; ++j)
            for (int k = pz - pdr; k <= pz + pdr; ++k) {
                double v[3] = {(double)(i - px), (double)(j - py), (double)(k - pz)};
                if (norm2_f(v, 3) > (double)pd / 2.0) continue;
                if (i < 1 || i > lx || j < 1 || j > ly || k < 1 || k > lz) return ORC_ERR_BAD_INPUT;
                long r = nid(i - 1, j - 1, k - 1, lx, ly);
                if (nature[r] != 0) err = 1;
                fx[r] = fl[0];
                fy[r] = fl[1];
                fz[r] = fl[2];
                cnt = cnt + 1;
            }
    if (err) return ORC_ERR_BAD_INPUT;
    long fluid_nodes = 0;
    for (long r = 0; r < N; ++r) fluid_nodes += nature[r] == 0;
    if (p->geometry_label == -1) {
        for (long r = 0; r < N; ++r) {
            if (fx[r] == fl[0] && fy[r] == fl[1] && fz[r] == fl[2]) {
                fx[r] = -fl[0] / fluid_nodes + fx[r] / cnt;
                fy[r] = -fl[1] / fluid_nodes + fy[r] / cnt;
                fz[r] = -fl[2] / fluid_nodes + fz[r] / cnt;
            } else {
                fx[r] = -fl[0] / fluid_nodes;
                fy[r] = -fl[1] / fluid_nodes;
                fz[r] = -fl[2] / fluid_nodes;
            }
        }
        double sx = 0, sy = 0, sz = 0;
        for (long r = 0; r < N; ++r) { sx += fx[r]; sy += fy[r]; sz += fz[r]; }
        const double eps = 2.220446049250313e-16;
        if (fabs(sx / fluid_nodes) > eps || fabs(sy / fluid_nodes) > eps ||
            fabs(sz / fluid_nodes) > eps)
            return ORC_ERR_BAD_INPUT;
    } else {
        for (long r = 0; r < N; ++r) {
            if (fx[r] == fl[0] && fy[r] == fl[1] && fz[r] == fl[2]) {
                fx[r] = fx[r] / cnt;
                fy[r] = fy[r] / cnt;
                fz[r] = fz[r] / cnt;
            } else {
                fx[r] = 0.0;
                fy[r] = 0.0;
                fz[r] = 0.0;
            }
        }
    }
    for (long r = 0; r < N; ++r)
        if (nature[r] != 0) fx[r] = fy[r] = fz[r] = 0.0;
    return ORC_OK;
}

/* equilibration.f90:143-491 */
int orc_equilibration(const orc_flow_params *p, const int8_t *nature, double *n,
                      double *density, double *jx, double *jy, double *jz, double *fx,
                      double *fy, double *fz, double *l2err_hist, int hist_cap,
                      int *steps_out)
{
    init_tables();
    int lx = p->lx, ly = p->ly, lz = p->lz;
    long N = (long)lx * ly * lz;
    if (p->relaxation_time < 0.5) return ORC_ERR_BAD_INPUT;
    /* equilibration.f90:75-80,94-96 */
    for (long r = 0; r < N; ++r) {
        jx[r] = jy[r] = jz[r] = 0.0;
        fx[r] = fy[r] = fz[r] = 0.0;
    }
    int conv_without = 0, conv_with = 0;
    int rc = ORC_OK;
    int t;
    for (t = 1;; ++t) {
        if (p->max_steps > 0 && t > p->max_steps) { rc = ORC_ERR_MAX_STEPS; t = p->max_steps; break; }
        rc = orc_collide(lx, ly, lz, nature, p->relaxation_time, n, density, jx, jy, jz, fx,
                         fy, fz);
        if (rc) break;
        orc_bounce_back_stream(lx, ly, lz, nature, n, p->nthreads);
        double l2err = 0.0;
        rc = orc_moments(lx, ly, lz, n, fx, fy, fz, density, jx, jy, jz, &l2err);
        if (l2err_hist && t - 1 < hist_cap) l2err_hist[t - 1] = l2err;
        if (rc) break;
        if (p->fixed_steps > 0) {
            if (t >= p->fixed_steps) break;
            continue;
        }
        int converged = (l2err <= p->target_error && t > 2);   /* equilibration.f90:346-350 */
        if (converged) {                                        /* equilibration.f90:355-365 */
            if (!conv_without) conv_without = 1;
            else conv_with = 1;
        }
        if (converged) {                                        /* equilibration.f90:370-489 */
            if (conv_without && conv_with && t > 2) break;
            if (conv_without && !conv_with) {
                if (!p->compensate_f_ext) {
                    for (long r = 0; r < N; ++r)
                        if (nature[r] == 0) {
                            fx[r] = p->f_ext[0];
                            fy[r] = p->f_ext[1];
                            fz[r] = p->f_ext[2];
                        }
                } else {
                    rc = compensate_field(p, nature, fx, fy, fz);
                    if (rc) break;
                }
            }
        }
    }
    if (steps_out) *steps_out = t;
    return rc;
}

/* drop_tracers.f90:63-105 */
void orc_update_tracer_population(int lx, int ly, int lz, const int8_t *nature,
                                  const double *density, const double *jx, const double *jy,
                                  const double *jz, const double f_ext[3], double tracer_z,
                                  double tracer_D, const double elec_slope[3], double *n_mp)
{
    init_tables();
    long N = (long)lx * ly * lz;
    for (long r = 0; r < N; ++r) {
        const double J[3] = {jx[r], jy[r], jz[r]};
        for (int l = 0; l < Q; ++l) {
            double s = 0.0;
            if (nature[r] == 0) {
                for (int d = 0; d < 3; ++d)
                    s = s + (double)VC[l][d] *
                                (J[d] + f_ext[d] - density[r] * tracer_z * tracer_D * elec_slope[d]);
            } else {
                for (int d = 0; d < 3; ++d) s = s + (double)VC[l][d] * J[d];
            }
            n_mp[l + Q * r] = W0[l] * density[r] + W1[l] * s;
        }
    }
}

/* module_moment_propagation.f90:341-346 */
static inline double scattprop(double n, double rho, double w, double lambda, double fermi)
{
    return n / rho - w + lambda * w * fermi;
}

/* module_moment_propagation.f90:30-160 */
/* module_moment_propagation.f90:303-322: phi(r') - phi(r), corrected by elec_slope for a link
 * across the periodic boundary; only the first matching case of the chain applies (0-based). */
static double orc_dphi(const orc_mp_state *s, int i, int j, int k, int ip, int jp, int kp)
{
    const int lx = s->lx, ly = s->ly, lz = s->lz;
    double d = s->phi[nid(ip, jp, kp, lx, ly)] - s->phi[nid(i, j, k, lx, ly)];
    if (i == lx - 1 && ip == 0) d = d + s->E[0] * (double)(lx + 1);
    else if (i == 0 && ip == lx - 1) d = d - s->E[0] * (double)(lx + 1);
    else if (j == ly - 1 && jp == 0) d = d + s->E[1] * (double)(ly + 1);
    else if (j == 0 && jp == ly - 1) d = d - s->E[1] * (double)(ly + 1);
    else if (k == lz - 1 && kp == 0) d = d + s->E[2] * (double)(lz + 1);
    else if (k == 0 && kp == lz - 1) d = d - s->E[2] * (double)(lz + 1);
    return d;
}

/* module_moment_propagation.f90:295-301 */
static double orc_exp_dphi(const orc_mp_state *s, int i, int j, int k, int ip, int jp, int kp)
{
    if (!s->phi) return 1.0;
    return exp(s->z * orc_dphi(s, i, j, k, ip, jp, kp));
}

static int mp_init_any(orc_mp_state *s, int lx, int ly, int lz, const int8_t *nature,
                       const uint8_t *interfacial, const double *density, const double *n_mp,
                       double ka, double kd, double Db, double Ds, double z, const double *phi,
                       const double E[3], double vacf0[3])
{
    init_tables();
    const double eps = 2.220446049250313e-16;
    const double kBT = 1.0 / 3.0;
    memset(s, 0, sizeof(*s));
    s->lx = lx; s->ly = ly; s->lz = lz;
    s->nthreads = 1;
    if (ka < -eps || kd < -eps) return ORC_ERR_BAD_INPUT;
    s->ka = ka; s->kd = kd;
    s->K = fabs(kd) <= eps ? 0.0 : ka / kd;
    s->consider_adsorption = fabs(s->K) > eps;
    s->Db = Db; s->Ds = Ds;
    if (fabs(Ds) > eps) return ORC_ERR_BAD_INPUT;          /* module_moment_propagation.f90:60-66 */
    s->lambda = 4.0 * Db / kBT;                            /* module_moment_propagation.f90:331-337 */
    s->z = z;
    const int charged = fabs(z) > eps;
    if (charged && !phi) return ORC_ERR_BAD_INPUT;          /* module_moment_propagation.f90:71-79 */
    long N = (long)lx * ly * lz;
    s->P_now = (double *)calloc(3 * N, sizeof(double));
    s->P_next = (double *)calloc(3 * N, sizeof(double));
    if (s->consider_adsorption) {
        s->A_now = (double *)calloc(3 * N, sizeof(double));
        s->A_next = (double *)calloc(3 * N, sizeof(double));
    }
    if (charged) {
        s->phi = (double *)malloc(sizeof(double) * N);
        memcpy(s->phi, phi, sizeof(double) * N);
        for (int d = 0; d < 3; ++d) s->E[d] = E[d];
    }
    double Pstat;
    if (!charged) {
        long nf = 0, nfi = 0;
        for (long r = 0; r < N; ++r) {
            nf += nature[r] == 0;
            nfi += nature[r] == 0 && interfacial[r];
        }
        Pstat = (double)nf + s->K * (double)nfi;           /* module_moment_propagation.f90:97 */
    } else {                                               /* module_moment_propagation.f90:99-100 */
        double s1 = 0.0, s2 = 0.0;
        for (long r = 0; r < N; ++r)
            if (nature[r] == 0) s1 = s1 + exp(-(z * phi[r]));
        for (long r = 0; r < N; ++r)
            if (nature[r] == 0 && interfacial[r]) s2 = s2 + exp(-(z * phi[r])) * s->K;
        Pstat = s1 + s2;
    }
    double v[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < lz; ++k)
        for (int j = 0; j < ly; ++j)
            for (int i = 0; i < lx; ++i) {
                long r = nid(i, j, k, lx, ly);
                if (nature[r] != 0) continue;
                const double bw = charged ? exp(-(z * phi[r])) / Pstat : 1.0 / Pstat;
                const double rho = density[r];
                double *P = s->P_now + 3 * r;
                for (int l = 1; l < Q; ++l) {
                    const int ip = pbc0(i + VC[l][0], lx), jp = pbc0(j + VC[l][1], ly),
                              kp = pbc0(k + VC[l][2], lz);
                    long rp = nid(ip, jp, kp, lx, ly);
                    if (nature[rp] == 1) continue;
                    const double exp_dphi = orc_exp_dphi(s, i, j, k, ip, jp, kp);
                    const double exp_min_dphi = 1.0 / exp_dphi;
                    const double fermi = 1.0 / (1.0 + exp_dphi);
                    double sp = scattprop(n_mp[l + Q * r], rho, W0[l], s->lambda, fermi);
                    for (int d = 0; d < 3; ++d) v[d] = v[d] + bw * sp * (double)(VC[l][d] * VC[l][d]);
                    int li = INV[l];
                    double spp = scattprop(n_mp[li + Q * rp], density[rp], W0[li], s->lambda,
                                           1.0 - fermi);
                    for (int d = 0; d < 3; ++d) P[d] = P[d] + exp_min_dphi * spp * (double)VC[li][d] * bw;
                }
            }
    for (int d = 0; d < 3; ++d) {
        vacf0[d] = v[d];
        s->vacf[d] = v[d];
    }
    return ORC_OK;
}

int orc_mp_init(orc_mp_state *s, int lx, int ly, int lz, const int8_t *nature,
                const uint8_t *interfacial, const double *density, const double *n_mp,
                double ka, double kd, double Db, double Ds, double z, double vacf0[3])
{
    const double eps = 2.220446049250313e-16;
    if (fabs(z) > eps) {                                    /* module_moment_propagation.f90:71-79 */
        memset(s, 0, sizeof(*s));
        return ORC_ERR_BAD_INPUT;
    }
    return mp_init_any(s, lx, ly, lz, nature, interfacial, density, n_mp, ka, kd, Db, Ds, z, NULL,
                       NULL, vacf0);
}

int orc_mp_init_charged(orc_mp_state *s, int lx, int ly, int lz, const int8_t *nature,
                        const uint8_t *interfacial, const double *density, const double *n_mp,
                        double ka, double kd, double Db, double z, const double *phi,
                        const double elec_slope[3], double vacf0[3])
{
    return mp_init_any(s, lx, ly, lz, nature, interfacial, density, n_mp, ka, kd, Db, 0.0, z, phi,
                       elec_slope, vacf0);
}

/* module_moment_propagation.f90:164-289 */
int orc_mp_propagate(orc_mp_state *s, int it, const int8_t *nature, const uint8_t *interfacial,
                     const double *density, const double *n_mp, double vacf_out[3],
                     int *is_converged)
{
    const int lx = s->lx, ly = s->ly, lz = s->lz;
    const double lambda = s->lambda, ka = s->ka, kd = s->kd;
    const int ads = s->consider_adsorption;
    const double eps = 2.220446049250313e-16;
    double *part = (double *)calloc(3 * (size_t)lz, sizeof(double));
    int error = 0;
#pragma omp parallel for num_threads(s->nthreads > 0 ? s->nthreads : 1) schedule(static) reduction(|| : error)
    for (int k = 0; k < lz; ++k) {
        double vk[3] = {0.0, 0.0, 0.0};
        for (int j = 0; j < ly; ++j)
            for (int i = 0; i < lx; ++i) {
                long r = nid(i, j, k, lx, ly);
                if (nature[r] != 0) continue;
                double us[3] = {0.0, 0.0, 0.0};
                double frac = 1.0;
                const double *nl = n_mp + Q * r;
                double Pl[3] = {s->P_next[3 * r], s->P_next[3 * r + 1], s->P_next[3 * r + 2]};
                for (int l = 1; l < Q; ++l) {
                    const int ip = pbc0(i + VC[l][0], lx), jp = pbc0(j + VC[l][1], ly),
                              kp = pbc0(k + VC[l][2], lz);
                    long rp = nid(ip, jp, kp, lx, ly);
                    if (nature[rp] != 0) continue;
                    const double fermi = 1.0 / (1.0 + orc_exp_dphi(s, i, j, k, ip, jp, kp));
                    double sp = scattprop(nl[l], density[r], W0[l], lambda, fermi);
                    frac = frac - sp;
                    for (int d = 0; d < 3; ++d) us[d] = us[d] + sp * (double)VC[l][d];
                    int li = INV[l];
                    double spp = scattprop(n_mp[li + Q * rp], density[rp], W0[li], lambda, 1.0 - fermi);
                    for (int d = 0; d < 3; ++d) Pl[d] = Pl[d] + s->P_now[3 * rp + d] * spp;
                }
                double *Pn = s->P_next + 3 * r;
                const double *Pc = s->P_now + 3 * r;
                for (int d = 0; d < 3; ++d) Pn[d] = Pl[d];
                for (int d = 0; d < 3; ++d) vk[d] = vk[d] + Pc[d] * us[d];
                if ((!interfacial[r] && ads) || !ads) {
                    for (int d = 0; d < 3; ++d) Pn[d] = Pn[d] + frac * Pc[d];
                } else {
                    frac = frac - ka;
                    double *An = s->A_next + 3 * r;
                    const double *Ac = s->A_now + 3 * r;
                    for (int d = 0; d < 3; ++d) {
                        Pn[d] = Pn[d] + frac * Pc[d] + Ac[d] * kd;
                        An[d] = Ac[d] * (1.0 - kd) + Pc[d] * ka;
                    }
                }
                if (frac < eps) error = 1;
            }
        for (int d = 0; d < 3; ++d) part[3 * k + d] = vk[d];
    }
    double v[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < lz; ++k)
        for (int d = 0; d < 3; ++d) v[d] = v[d] + part[3 * k + d];
    free(part);
    /* module_moment_propagation.f90:262-267: rotate now <- next, next <- 0 */
    long N = (long)lx * ly * lz;
    double *t = s->P_now; s->P_now = s->P_next; s->P_next = t;
    memset(s->P_next, 0, sizeof(double) * 3 * N);
    if (ads) {
        t = s->A_now; s->A_now = s->A_next; s->A_next = t;
        memset(s->A_next, 0, sizeof(double) * 3 * N);
    }
    for (int d = 0; d < 3; ++d) {
        vacf_out[d] = v[d];
        s->vacf[d] = v[d];
    }
    /* module_moment_propagation.f90:284-288 */
    const double thr1 = 1.0 / (2.0 * lx * ly * lz / s->Db);
    const double thr2 = (double)1.e-12f;
    int conv = it > 2;
    for (int d = 0; d < 3; ++d)
        if (!(fabs(v[d]) < thr1) || !(fabs(v[d]) < thr2)) conv = 0;
    if (is_converged) *is_converged = conv;
    (void)it;
    return error ? ORC_ERR_FRACTION : ORC_OK;
}

void orc_mp_free(orc_mp_state *s)
{
    free(s->P_now);
    free(s->P_next);
    free(s->A_now);
    free(s->A_next);
    free(s->phi);
    s->P_now = s->P_next = s->A_now = s->A_next = NULL;
    s->phi = NULL;
}

static const double PI_F = 3.141592653589793;   /* acos(-1.0_dp), module_constants.f90:19 */

/* charges_init.f90:23-135 */
int orc_charges_init(int lx, int ly, int lz, const int8_t *nature, const uint8_t *interfacial,
                     double bjl, double sigma, double lambda_D, int charge_distrib_int,
                     double *c_plus, double *c_minus, double *phi, double *anormf0,
                     double *rho_ch)
{
    const double eps = 2.220446049250313e-16;
    const double kBT = 1.0 / 3.0;
    long N = (long)lx * ly * lz;
    if (bjl <= eps) return ORC_OK;
    double rho_0;
    if (fabs(lambda_D) <= eps) rho_0 = 0.0;
    else rho_0 = 1.0 / (4.0 * PI_F * bjl * (lambda_D * lambda_D));
    *rho_ch = 1.0 / (4.0 * PI_F * bjl * (lambda_D * lambda_D));
    long count_solid = 0, count_solid_int = 0, count_fluid = 0;
    for (long r = 0; r < N; ++r) {
        count_solid += nature[r] == 1;
        count_solid_int += nature[r] == 1 && interfacial[r];
        count_fluid += nature[r] == 0;
    }
    if (fabs(sigma) > eps) {
        for (long r = 0; r < N; ++r) phi[r] = 0.0;
        double sigma_solid, sigma_fluid;
        if (!charge_distrib_int) {
            /* charges_init.f90:96-100: the 'sol' distribution stops the reference */
            return ORC_ERR_BAD_INPUT;
        }
        sigma_solid = count_solid_int != 0 ? sigma / count_solid_int : 0.0;
        sigma_fluid = count_fluid != 0 ? -1.0 * sigma / count_fluid : 0.0;
        double in_c_plus_solid = +0.5 * sigma_solid;
        double in_c_minus_solid = -0.5 * sigma_solid;
        double in_c_plus_fluid, in_c_minus_fluid;
        if (sigma_fluid > 0.0) {
            in_c_plus_fluid = 0.5 * rho_0 + sigma_fluid;
            in_c_minus_fluid = 0.5 * rho_0;
        } else {
            in_c_plus_fluid = 0.5 * rho_0;
            in_c_minus_fluid = 0.5 * rho_0 - sigma_fluid;
        }
        for (long r = 0; r < N; ++r) {
            if (nature[r] == 1 && interfacial[r]) {
                c_plus[r] = in_c_plus_solid;
                c_minus[r] = in_c_minus_solid;
            } else if (nature[r] == 1 && !interfacial[r]) {
                c_plus[r] = 0.0;
                c_minus[r] = 0.0;
            } else if (nature[r] == 0) {
                c_plus[r] = in_c_plus_fluid;
                c_minus[r] = in_c_minus_fluid;
            }
        }
        double s = 0.0;
        for (long r = 0; r < N; ++r) s = s + (c_plus[r] + c_minus[r]);
        *anormf0 = 4.0 * PI_F * bjl * kBT / 2.0 * s;
    }
    return ORC_OK;
}

int orc_sor_custom(int lx, int ly, int lz, double sigma, double bjl, const double *c_plus,
                   const double *c_minus, double *phi, double *anormf0, double omega,
                   double tol, int maxiter, int *iters_out)
{
    init_tables();
    const double kBT = 1.0 / 3.0;
    long N = (long)lx * ly * lz;
    if (sigma == 0.0) {
        for (long r = 0; r < N; ++r) phi[r] = 0.0;
        if (iters_out) *iters_out = 0;
        return ORC_OK;
    }
    double *tmp = (double *)malloc(sizeof(double) * N);
    const double factor = 4.0 * PI_F * bjl * kBT / 2.0;
    int iter, rc = ORC_OK;
    for (iter = 1; iter <= maxiter; ++iter) {
        double anorm = 0.0;
        for (int i = 0; i < lx; ++i)
            for (int j = 0; j < ly; ++j)
                for (int k = 0; k < lz; ++k) {
                    double phistar = 0.0;
                    for (int l = 0; l < Q; ++l) {
                        long rn = nid(pbc0(i - VC[l][0], lx), pbc0(j - VC[l][1], ly),
                                      pbc0(k - VC[l][2], lz), lx, ly);
                        phistar = phistar + W0[l] * phi[rn];
                    }
                    long r = nid(i, j, k, lx, ly);
                    phistar = phistar + factor * (c_plus[r] - c_minus[r]);
                    double phiold = phi[r];
                    tmp[r] = omega * phistar + (1.0 - omega) * phiold;
                    anorm = anorm + fabs(phistar - phiold);
                }
        memcpy(phi, tmp, sizeof(double) * N);
        if (anorm <= tol * *anormf0) break;
        if (iter == maxiter) { rc = ORC_ERR_NOT_CONVERGED; break; }
    }
    if (iters_out) *iters_out = iter - 1;
    double s = 0.0;
    for (long r = 0; r < N; ++r) s = s + fabs(phi[r]);
    *anormf0 = s;
    free(tmp);
    return rc;
}

/* sor.f90:7-91 */
int orc_sor(int lx, int ly, int lz, double sigma, double bjl, const double *c_plus,
            const double *c_minus, double *phi, double *anormf0, int *iters_out)
{
    return orc_sor_custom(lx, ly, lz, sigma, bjl, c_plus, c_minus, phi, anormf0, 1.4,
                          (double)1.0e-5f, 500000, iters_out);
}

/* just_eq_smolu.f90:6-135 (time = 0 and D_equil = 0 in the reference, hence eD = 0.1 D and
 * at most 10 iterations: just_eq_smolu.f90:33-38) */
int orc_just_eq_smolu(int lx, int ly, int lz, const int8_t *nature, const double *phi,
                      double *c_plus, double *c_minus, double D_plus, double D_minus,
                      double rho_ch, double sigma, int loop_bug, int *iters_out)
{
    init_tables();
    long N = (long)lx * ly * lz;
    double *fp = (double *)malloc(sizeof(double) * N);
    double *fm = (double *)malloc(sizeof(double) * N);
    double tot_plus = 1.7976931348623157e308, tot_minus = 1.7976931348623157e308;
    const double eD_plus = 0.1 * D_plus, eD_minus = 0.1 * D_minus;
    const int max_iter = 10;
    const double crit = (double)5.e-6f;
    int iter = 0, rc = ORC_OK;
    long count_fluid = 0;
    for (long r = 0; r < N; ++r) count_fluid += nature[r] == 0;
    while (tot_minus + tot_plus > crit && iter < max_iter) {
        for (long r = 0; r < N; ++r) fp[r] = fm[r] = 0.0;
        int j0 = loop_bug ? ly - 1 : 0, k0 = loop_bug ? lz - 1 : 0;
        for (int i = 0; i < lx; ++i)
            for (int j = j0; j < ly; ++j)
                for (int k = k0; k < lz; ++k) {
                    for (int l = 1; l < Q; l += 2) {
                        int ip = pbc0(i + VC[l][0], lx), jp = pbc0(j + VC[l][1], ly),
                            kp = pbc0(k + VC[l][2], lz);
                        long r = nid(i, j, k, lx, ly), rp = nid(ip, jp, kp, lx, ly);
                        if (nature[r] == 0 && nature[rp] == 0) {
                            double e = exp(phi[rp] - phi[r]);
                            double em = 1.0 / e;
                            double flp = 0.5 * (1.0 + em) * (c_plus[rp] * e - c_plus[r]);
                            flp = flp * eD_plus / DELTA[l];
                            double flm = 0.5 * (1.0 + e) * (c_minus[rp] * em - c_minus[r]);
                            flm = flm * eD_minus / DELTA[l];
                            fp[r] = fp[r] + flp;
                            fm[r] = fm[r] + flm;
                            fp[rp] = fp[rp] - flp;
                            fm[rp] = fm[rp] - flm;
                        }
                    }
                }
        double sp = 0.0, sm = 0.0;
        for (long r = 0; r < N; ++r) { sp = sp + fp[r]; sm = sm + fm[r]; }
        if (fabs(sp) > (double)1.e-12f || fabs(sm) > (double)1.e-12f) { rc = ORC_ERR_FLUX_SUM; break; }
        for (long r = 0; r < N; ++r)
            if (nature[r] == 0) {
                c_plus[r] = c_plus[r] + fp[r];
                c_minus[r] = c_minus[r] + fm[r];
            }
        if (sigma != 0 && eD_plus != 0.0 && eD_minus != 0.0) {
            double qp = 0.0, qm = 0.0;
            for (long r = 0; r < N; ++r)
                if (nature[r] == 0) { qp = qp + fp[r] * fp[r]; qm = qm + fm[r] * fm[r]; }
            tot_plus = sqrt(qp) / count_fluid / (0.5 * rho_ch * eD_plus) / sigma;
            tot_minus = sqrt(qm) / count_fluid / (0.5 * rho_ch * eD_minus) / sigma;
        }
        iter = iter + 1;
    }
    if (iters_out) *iters_out = iter;
    free(fp);
    free(fm);
    return rc;
}

/* check_charge_distribution_equilibrium.f90:24-44 */
int orc_check_charge_equilibrium(int N, const double *phi, const double *phi_old,
                                 const double *c_plus, const double *c_plus_old,
                                 const double *c_minus, const double *c_minus_old,
                                 double diffs[3])
{
    const double eps = 1.0e-12;
    const double *a[3] = {phi, c_plus, c_minus}, *o[3] = {phi_old, c_plus_old, c_minus_old};
    for (int q = 0; q < 3; ++q) {
        long cnt = 0;
        double s = 0.0;
        for (long r = 0; r < N; ++r)
            if (fabs(o[q][r]) > eps) {
                cnt++;
                s = s + fabs((a[q][r] - o[q][r]) / o[q][r]);
            }
        diffs[q] = cnt != 0 ? s / (double)cnt : 0.0;
    }
    return diffs[0] < eps && diffs[1] < eps && diffs[2] < eps;
}

/* charge_test.f90:15-24 */
int orc_charge_test(int N, const int8_t *nature, const double *c_plus, const double *c_minus,
                    double sigma, double *solid_charge, double *fluid_charge)
{
    double s = 0.0, f = 0.0;
    for (long r = 0; r < N; ++r) {
        if (nature[r] == 1) s = s + (c_plus[r] - c_minus[r]);
        if (nature[r] == 0) f = f + (c_plus[r] - c_minus[r]);
    }
    *solid_charge = s;
    *fluid_charge = f;
    const double tol = (double)1.0e-10f;
    if (fabs(s - sigma) > tol || fabs(f + sigma) > tol) return ORC_ERR_CHARGE;
    return ORC_OK;
}

/* poisson_nernst_planck.f90:38-48 */
int orc_pnp(int lx, int ly, int lz, const int8_t *nature, double bjl, double sigma,
            double D_plus, double D_minus, double rho_ch, int loop_bug, double *c_plus,
            double *c_minus, double *phi, double *anormf0, int max_outer, int *outer_out,
            int *sor_iters_total)
{
    long N = (long)lx * ly * lz;
    double *po = (double *)malloc(sizeof(double) * N);
    double *cpo = (double *)malloc(sizeof(double) * N);
    double *cmo = (double *)malloc(sizeof(double) * N);
    int outer = 0, rc = ORC_OK, converged = 0, total = 0;
    while (!converged) {
        if (outer >= max_outer) { rc = ORC_ERR_NOT_CONVERGED; break; }
        memcpy(cpo, c_plus, sizeof(double) * N);   /* backup_phi_c_plus_c_minus.f90 */
        memcpy(cmo, c_minus, sizeof(double) * N);
        memcpy(po, phi, sizeof(double) * N);
        int it = 0;
        rc = orc_sor(lx, ly, lz, sigma, bjl, c_plus, c_minus, phi, anormf0, &it);
        total += it;
        if (rc) break;
        rc = orc_just_eq_smolu(lx, ly, lz, nature, phi, c_plus, c_minus, D_plus, D_minus,
                               rho_ch, sigma, loop_bug, NULL);
        if (rc) break;
        double d[3];
        converged = orc_check_charge_equilibrium((int)N, phi, po, c_plus, cpo, c_minus, cmo, d);
        outer++;
    }
    if (outer_out) *outer_out = outer;
    if (sor_iters_total) *sor_iters_total = total;
    free(po);
    free(cpo);
    free(cmo);
    return rc;
}

/* equilibration.f90:159-175 (and 504-516 at exit): per plane normal to `axis` (0 = x, 1 = y,
 * 2 = z), SUM(jx), SUM(jy), SUM(jz) and SUM(density)/MAX(COUNT(density > eps), 1), each SUM a
 * single accumulator over the plane in array element order (first remaining index fastest). */
void orc_profiles(int lx, int ly, int lz, const double *density, const double *jx,
                  const double *jy, const double *jz, int axis, double *flux, double *mean_density)
{
    const double eps = 2.220446049250313e-16; /* EPSILON(1._dp) */
    const int n[3] = {lx, ly, lz};
    const int L = n[axis];
    const int a = axis == 0 ? 1 : 0, b = axis == 2 ? 1 : 2; /* remaining axes, a fastest */
    for (int k = 0; k < L; ++k) {
        double sx = 0.0, sy = 0.0, sz = 0.0, sd = 0.0;
        long cnt = 0;
        for (int q = 0; q < n[b]; ++q)
            for (int p = 0; p < n[a]; ++p) {
                int c[3];
                c[axis] = k;
                c[a] = p;
                c[b] = q;
                const long r = nid(c[0], c[1], c[2], lx, ly);
                sx = sx + jx[r];
                sy = sy + jy[r];
                sz = sz + jz[r];
                sd = sd + density[r];
                cnt += density[r] > eps;
            }
        flux[3 * k] = sx;
        flux[3 * k + 1] = sy;
        flux[3 * k + 2] = sz;
        mean_density[k] = sd / (double)(cnt > 0 ? cnt : 1);   /* MAX(COUNT(...), 1) */
    }
}

/* ------------------------------------------------------------------ geometry builders */

/* gfortran's inline NORM2 (scaled sum of squares, scale starting at 1): the reference's
 * distance in every builder of module_geometry.f90. */
static double orc_norm2(int n, const double *v)
{
    double scale = 1.0, ssq = 0.0;
    for (int q = 0; q < n; ++q) {
        if (v[q] != 0.0) {
            const double ax = fabs(v[q]);
            if (scale < ax) {
                const double t = scale / ax;
                ssq = 1.0 + ssq * t * t;
                scale = ax;
            } else {
                const double t = ax / scale;
                ssq = ssq + t * t;
            }
        }
    }
    return scale * sqrt(ssq);
}

static double n2(double a, double b)
{
    const double v[2] = {a, b};
    return orc_norm2(2, v);
}

static double n3(double a, double b, double c)
{
    const double v[3] = {a, b, c};
    return orc_norm2(3, v);
}

int orc_geometry(int label, int lx, int ly, int lz, const double *params, int8_t *nature)
{
    const long long N = (long long)lx * ly * lz;
    if (lx < 1 || ly < 1 || lz < 1) return 1;
#define NAT(i, j, k) nature[((i) - 1) + (long long)lx * (((j) - 1) + (long long)ly * ((k) - 1))]
    for (long long q = 0; q < N; ++q) nature[q] = 0;   /* supercell_definition.f90:45 */
    switch (label) {
    case -1:
        break;
    case 1:   /* module_geometry.f90:158-166 */
        for (int j = 1; j <= ly; ++j)
            for (int i = 1; i <= lx; ++i) {
                NAT(i, j, 1) = 1;
                NAT(i, j, lz) = 1;
            }
        break;
    case 2: { /* module_geometry.f90:253-277 */
        if (lx != ly || lx < 3) return 1;
        const double ox = (double)(lx + 1) / 2.0, oy = (double)(ly + 1) / 2.0;
        const double radius = (double)(lx - 1) / 2.0;
        for (int i = 1; i <= lx; ++i)
            for (int j = 1; j <= ly; ++j) {
                const int8_t v = n2((double)i - ox, (double)j - oy) >= radius;
                for (int k = 1; k <= lz; ++k) NAT(i, j, k) = v;
            }
        break;
    }
    case 3: { /* module_geometry.f90:206-245 */
        if (lx != ly || lx != lz) return 1;
        const double thr = (double)(lx - 1) * sqrt(3.0) / 4.0;
        const double cen[9][3] = {{1, 1, 1}, {lx, 1, 1}, {1, ly, 1}, {1, 1, lz}, {lx, ly, 1},
                                  {lx, 1, lz}, {1, ly, lz}, {lx, ly, lz},
                                  {(double)(float)(lx + 1) / 2.0, (double)(float)(ly + 1) / 2.0,
                                   (double)(float)(lz + 1) / 2.0}};
        for (int k = 1; k <= lz; ++k)
            for (int j = 1; j <= ly; ++j)
                for (int i = 1; i <= lx; ++i) {
                    int in = 0;
                    for (int c = 0; c < 9; ++c)
                        if (n3((double)i - cen[c][0], (double)j - cen[c][1], (double)k - cen[c][2]) <= thr) in = 1;
                    NAT(i, j, k) = (int8_t)in;
                }
        break;
    }
    case 4: { /* module_geometry.f90:336-378 */
        if (lx != ly || lx % 2 == 0) return 1;
        const double ox = (double)(lx + 1) / 2.0, oy = (double)(ly + 1) / 2.0;
        const double radius = n2(1.0 - ox, (double)((lx + 1) / 2) - oy);
        for (int i = 1; i <= lx; ++i)
            for (int j = 1; j <= ly; ++j) {
                const int8_t v = n2((double)i - ox, (double)j - oy) > radius;
                for (int k = 1; k <= lz; ++k) NAT(i, j, k) = v;
            }
        break;
    }
    case 5: { /* module_geometry.f90:122-153 */
        if (ly % 2 == 0) return 1;
        const int midly = (ly + 1) / 2;
        const double b = (double)((float)(2.0f / 3.0f) * (float)midly);   /* 2./3.*midly, REAL */
        const double a = (double)midly - b - 1.0;
        if (a <= 0.0 || b <= 0.0) return 2;
        const double pi = 3.141592653589793;   /* acos(-1.0_dp) */
        for (int i = 1; i <= lx; ++i) {
            const double xi = (double)(i - 1);
            const double yi = a * sin(2.0 * pi * xi / (double)lx) + b + (double)midly;
            const long ninty = lround(yi);   /* NINT: half away from zero */
            for (int j = midly; j <= ly; ++j) {
                const int8_t v = (long)j < ninty ? 0 : 1;
                const int mirror = 2 * midly - j;
                for (int k = 1; k <= lz; ++k) {
                    NAT(i, j, k) = v;
                    NAT(i, mirror, k) = v;
                }
            }
        }
        break;
    }
    case 6: { /* module_geometry.f90:96-119 */
        for (int k = 1; k <= lz; ++k)
            for (int i = 1; i <= lx; ++i) {
                NAT(i, 1, k) = 1;
                NAT(i, ly, k) = 1;
                if (i > lx / 2) {
                    for (int j = 2; j <= 1 + (ly - 2) / 4; ++j) NAT(i, j, k) = 1;
                    for (int j = ly - (ly - 2) / 4; j <= ly - 1; ++j) NAT(i, j, k) = 1;
                }
            }
        break;
    }
    case 7: { /* module_geometry.f90:52-89 */
        if (ly != lz) return 1;
        if (!params) return 2;
        const double lw_o_lx = params[0], a_o_R = params[1];
        const double R = (double)((float)(ly - 1) / 2.0f);   /* real(ly-1)/2.0, REAL */
        const double a = a_o_R * R;
        const double r0y = (double)((float)(ly + 1) / 2.0f), r0z = (double)((float)(lz + 1) / 2.0f);
        for (int k = 1; k <= lz; ++k)
            for (int j = 1; j <= ly; ++j) {
                const double d = n2((double)(float)j - r0y, (double)(float)k - r0z);
                for (int i = 1; i <= lx; ++i) {
                    const int fluid = (double)i > lw_o_lx * (double)lx ? d < a : d < R;
                    NAT(i, j, k) = fluid ? 0 : 1;
                }
            }
        break;
    }
    case 8: { /* module_geometry.f90:173-198 */
        if (lx != ly || lx != lz || lx < 3) return 1;
        const double o = (double)(lx + 1) / 2.0, radius = (double)(lx - 1) / 2.0;
        for (int k = 1; k <= lz; ++k)
            for (int j = 1; j <= ly; ++j)
                for (int i = 1; i <= lx; ++i)
                    NAT(i, j, k) = n3((double)i - o, (double)j - o, (double)k - o) >= radius;
        break;
    }
    case 9: { /* module_geometry.f90:287-331 */
        if (lx != ly || lx != lz || lx % 2 == 0) return 1;
        const double o = (double)(lx + 1) / 2.0;
        const double radius = n3(1.0 - o, (double)((ly + 1) / 2) - o, (double)((lz + 1) / 2) - o);
        for (int k = 1; k <= lz; ++k)
            for (int j = 1; j <= ly; ++j)
                for (int i = 1; i <= lx; ++i)
                    NAT(i, j, k) = n3((double)i - o, (double)j - o, (double)k - o) > radius;
        break;
    }
    case 10: { /* module_geometry.f90:11-49 */
        const float s3 = sqrtf(3.0f);
        if (fabsf((float)ly / (float)lx - s3) / s3 >= 0.05f) return 1;
        if (lz < 3) return 1;
        const double midx = (double)(lx + 1) / 2.0, midy = (double)(ly + 1) / 2.0;
        const double cx[4] = {1.0, (double)lx, midx, midx}, cy[4] = {midy, midy, 1.0, (double)ly};
        const double radius = 0.2 * (double)lx;
        for (int i = 1; i <= lx; ++i)
            for (int j = 1; j <= ly; ++j) {
                int in = 0;
                for (int c = 0; c < 4 && !in; ++c)
                    if (n2((double)i - cx[c], (double)j - cy[c]) <= radius) in = 1;
                if (in)
                    for (int k = 1; k <= lz; ++k) NAT(i, j, k) = 1;
            }
        for (int j = 1; j <= ly; ++j)
            for (int i = 1; i <= lx; ++i) {
                NAT(i, j, 1) = 1;
                NAT(i, j, lz) = 1;
            }
        break;
    }
    default:
        return 3;
    }
#undef NAT
    for (long long q = 0; q < N; ++q)   /* supercell_definition.f90:92-94 */
        if (nature[q] == 0) return 0;
    return 4;
}

/* ------------------------------------------------------------ coupled electrokinetics */

/* electrostatic_pot.f90:7-21 */
void orc_electrostatic_pot(int lx, int ly, int lz, const double *phi, const double es[3],
                           double *phi_tot)
{
    const long N = (long)lx * ly * lz;
    if (es[0] == 0.0 && es[1] == 0.0 && es[2] == 0.0) {
        for (long r = 0; r < N; ++r) phi_tot[r] = phi[r];
        return;
    }
    for (int k = 0; k < lz; ++k)
        for (int j = 0; j < ly; ++j)
            for (int i = 0; i < lx; ++i) {
                /* sum(elec_slope * real([i,j,k],dp)): one accumulator from 0, x then y then z */
                double s = 0.0;
                s = s + es[0] * (double)(i + 1);
                s = s + es[1] * (double)(j + 1);
                s = s + es[2] * (double)(k + 1);
                const long r = nid(i, j, k, lx, ly);
                phi_tot[r] = phi[r] + s;
            }
}

/* comp_j.f90:14-27 */
void orc_comp_j(int lx, int ly, int lz, const double *n, double *jx, double *jy, double *jz)
{
    init_tables();
    const long N = (long)lx * ly * lz;
    double *j[3] = {jx, jy, jz};
    for (long r = 0; r < N; ++r)
        for (int d = 0; d < 3; ++d) {
            double s = 0.0;   /* sum(n(i,j,k,:)*coo(d)) over l = 1..19 */
            for (int l = 0; l < Q; ++l) s = s + n[(long)l * N + r] * (double)VC[l][d];
            j[d][r] = 0.5 * (j[d][r] + s);
        }
}

/* smolu.f90:1-144 */
int orc_smolu(int lx, int ly, int lz, const int8_t *nature, const double *phi_tot,
              double *c_plus, double *c_minus, double D_plus, double D_minus, int time,
              int D_iter, const double es[3], const double ls[3], double el_curr[3],
              double ion_curr[3], double *sf)
{
    init_tables();
    const long N = (long)lx * ly * lz;
    const double kBT = 1.0 / 3.0;
    const double dit = (double)D_iter;
    double *fp = (double *)calloc((size_t)N, sizeof(double));
    double *fm = (double *)calloc((size_t)N, sizeof(double));
    for (int i = 0; i < lx; ++i)
        for (int j = 0; j < ly; ++j)
            for (int k = 0; k < lz; ++k) {
                const long r = nid(i, j, k, lx, ly);
                for (int l = 1; l < Q; ++l) {
                    const int ip = pbc0(i + VC[l][0], lx), jp = pbc0(j + VC[l][1], ly),
                              kp = pbc0(k + VC[l][2], lz);
                    const long rp = nid(ip, jp, kp, lx, ly);
                    const double cx = (double)VC[l][0], cy = (double)VC[l][1], cz = (double)VC[l][2];
                    if (nature[r] == 0 && nature[rp] == 0) {
                        double e = exp(phi_tot[rp] - phi_tot[r]);
                        /* smolu.f90:46-51: every matching case applies, in this order */
                        if (i == lx - 1 && ip == 0) e = e * exp(es[0] * (double)lx);
                        if (j == ly - 1 && jp == 0) e = e * exp(es[1] * (double)ly);
                        if (k == lz - 1 && kp == 0) e = e * exp(es[2] * (double)lz);
                        if (i == 0 && ip == lx - 1) e = e * exp(-(es[0] * (double)lx));
                        if (j == 0 && jp == ly - 1) e = e * exp(-(es[1] * (double)ly));
                        if (k == 0 && kp == lz - 1) e = e * exp(-(es[2] * (double)lz));
                        const double em = 1.0 / e;
                        double sl = 0.0;
                        sl = sl + ls[0] * cx;
                        sl = sl + ls[1] * cy;
                        sl = sl + ls[2] * cz;
                        const double edl = exp(sl);
                        const double emdl = 1.0 / edl;
                        double flp = 0.5 * (1.0 + em * emdl) * (c_plus[rp] * e * edl - c_plus[r]);
                        double flm = 0.5 * (1.0 + e * emdl) * (c_minus[rp] * em * edl - c_minus[r]);
                        const double elc = flp * D_plus - flm * D_minus;
                        const double ionc = flp * D_plus + flm * D_minus;
                        const double f_plus = 0.5 * (1.0 + em) * (c_plus[rp] * e - c_plus[r]);
                        const double f_minus = 0.5 * (1.0 + e) * (c_minus[rp] * em - c_minus[r]);
                        double fmi = kBT * (f_plus + f_minus);
                        fmi = fmi - kBT * (c_plus[rp] - c_plus[r] + c_minus[rp] - c_minus[r]);
                        flp = flp * (D_plus / DELTA[l]);
                        flm = flm * (D_minus / DELTA[l]);
                        fp[r] = fp[r] + flp;
                        fm[r] = fm[r] + flm;
                        el_curr[0] = el_curr[0] + W1[l] * cx * elc / dit;
                        el_curr[1] = el_curr[1] + W1[l] * cy * elc / dit;
                        el_curr[2] = el_curr[2] + W1[l] * cz * elc / dit;
                        ion_curr[0] = ion_curr[0] + W1[l] * cx * ionc / dit;
                        ion_curr[1] = ion_curr[1] + W1[l] * cy * ionc / dit;
                        ion_curr[2] = ion_curr[2] + W1[l] * cz * ionc / dit;
                        sf[r] = sf[r] + W1[l] * cx * fmi / dit;
                        sf[r + N] = sf[r + N] + W1[l] * cy * fmi / dit;
                        sf[r + 2 * N] = sf[r + 2 * N] + W1[l] * cz * fmi / dit;
                    } else if (nature[r] == 0 && nature[rp] == 1) {
                        const double e = exp(phi_tot[rp] - phi_tot[r]);
                        const double em = 1.0 / e;
                        const double f_plus = c_plus[r] * (1.0 - em);
                        const double f_minus = c_minus[r] * (1.0 - e);
                        const double fmi = kBT * (f_plus + f_minus);
                        sf[r] = sf[r] + W1[l] * cx * fmi / dit;
                        sf[r + N] = sf[r + N] + W1[l] * cy * fmi / dit;
                        sf[r + 2 * N] = sf[r + 2 * N] + W1[l] * cz * fmi / dit;
                    }
                }
            }
    for (long r = 0; r < N; ++r)
        if (nature[r] == 0) {
            c_plus[r] = c_plus[r] + fp[r];
            c_minus[r] = c_minus[r] + fm[r];
        }
    if (time > 0) {
        /* n_fluidsites = sum(node%nature, mask=node%nature==fluid): fluid is 0, so the sum is 0
         * and the currents are divided by zero (smolu.f90:126-134) */
        long nfs = 0;
        for (long r = 0; r < N; ++r)
            if (nature[r] == 0) nfs += nature[r];
        const double d = (double)nfs;
        for (int q = 0; q < 3; ++q) {
            el_curr[q] = el_curr[q] / d;
            ion_curr[q] = ion_curr[q] / d;
        }
    }
    double sp = 0.0, sm = 0.0;
    for (long r = 0; r < N; ++r)
        if (nature[r] == 0) {
            sp = sp + fp[r];
            sm = sm + fm[r];
        }
    free(fp);
    free(fm);
    if (fabs(sp) > (double)1.0e-12f || fabs(sm) > (double)1.0e-12f) return ORC_ERR_FLUX_SUM;
    return ORC_OK;
}

/* advect.f90:2-116 */
int orc_advect(int lx, int ly, int lz, const int8_t *nature, const double *jx, const double *jy,
               const double *jz, double *c_plus, double *c_minus, double *fp, double *fm,
               double el_curr[3], double ion_curr[3])
{
    const long N = (long)lx * ly * lz;
    const double eps = 2.220446049250313e-16;   /* epsilon(1._dp) */
    const double *J[3] = {jx, jy, jz};
    int all_zero = 1, all_diff0 = 1, all_sum0 = 1;
    for (long r = 0; r < N; ++r) {
        if (!(fabs(c_plus[r]) <= eps && fabs(c_minus[r]) <= eps)) all_zero = 0;
        if (!(fabs(c_plus[r] - c_minus[r]) <= eps)) all_diff0 = 0;
        if (!(fabs(c_plus[r] + c_minus[r]) <= eps)) all_sum0 = 0;
    }
    if (all_zero) return ORC_OK;   /* advect.f90:32-34: no charge, nothing to advect */
    if (all_diff0) {
        el_curr[0] = el_curr[1] = el_curr[2] = 0.0;
    } else {
        for (int d = 0; d < 3; ++d) {
            double s = 0.0;
            for (long r = 0; r < N; ++r)
                if (nature[r] == 0) s = s + J[d][r] * (c_plus[r] - c_minus[r]);
            el_curr[d] = -s;
        }
    }
    if (all_sum0) {   /* advect.f90:46-49 sets el_curr here, not ion_curr */
        el_curr[0] = el_curr[1] = el_curr[2] = 0.0;
    } else {
        for (int d = 0; d < 3; ++d) {
            double s = 0.0;
            for (long r = 0; r < N; ++r)
                if (nature[r] == 0) s = s + J[d][r] * (c_plus[r] + c_minus[r]);
            ion_curr[d] = -s;
        }
    }
    double cp_old = 0.0, cm_old = 0.0;
    for (long r = 0; r < N; ++r) cp_old = cp_old + c_plus[r];
    for (long r = 0; r < N; ++r) cm_old = cm_old + c_minus[r];
    for (int i = 0; i < lx; ++i)
        for (int j = 0; j < ly; ++j)
            for (int k = 0; k < lz; ++k) {
                const long r = nid(i, j, k, lx, ly);
                if (fabs(c_plus[r]) <= eps && fabs(c_minus[r]) <= eps) continue;
                const double vx = jx[r], vy = jy[r], vz = jz[r];
                for (int ix = -1; ix <= 1; ++ix) {
                    double ax = vx * (double)ix;
                    for (int iy = -1; iy <= 1; ++iy) {
                        double ay = vy * (double)iy;
                        for (int iz = -1; iz <= 1; ++iz) {
                            const long rp = nid(pbc0(i + ix, lx), pbc0(j + iy, ly), pbc0(k + iz, lz), lx, ly);
                            double az = vz * (double)iz;
                            double flp, flm;
                            if (ax >= 0.0 && ay >= 0.0 && az >= 0.0 && nature[r] == nature[rp]) {
                                if (ix == 0) ax = 1.0 - fabs(vx);
                                if (iy == 0) ay = 1.0 - fabs(vy);
                                if (iz == 0) az = 1.0 - fabs(vz);
                                flp = ax * ay * az * c_plus[r];
                                flm = ax * ay * az * c_minus[r];
                            } else {
                                flp = 0.0;
                                flm = 0.0;
                            }
                            fm[r] = fm[r] - flm;
                            fm[rp] = fm[rp] + flm;
                            fp[r] = fp[r] - flp;
                            fp[rp] = fp[rp] + flp;
                        }
                    }
                }
            }
    for (long r = 0; r < N; ++r)
        if (nature[r] == 0) {
            c_minus[r] = c_minus[r] + fm[r];
            c_plus[r] = c_plus[r] + fp[r];
        }
    double cm_new = 0.0, cp_new = 0.0;
    for (long r = 0; r < N; ++r) cm_new = cm_new + c_minus[r];
    for (long r = 0; r < N; ++r) cp_new = cp_new + c_plus[r];
    if (fabs(cm_new - cm_old) > (double)1.e-8f || fabs(cp_new - cp_old) > (double)1.e-8f)
        return ORC_ERR_CHARGE;
    return ORC_OK;
}
