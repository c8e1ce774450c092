/*
 * conformance.c -- a plain C client of include/lbgpu.h, compiled by gcc in the tests.
 *
 * "layout": prints, for every struct of the C ABI, its size and each field's offset and size
 *   ("<struct> <field> <offset> <size>" lines, then "<struct> sizeof <n>"); the test compares
 *   them with the bind(C) derived types the Fortran host declares.
 * "c1 [max_steps]": the reference's C1 flow phase through the C ABI from C: a 4 x 4 x 34 slit
 *   (geometryLabel 1: solid planes z = 1 and z = 34, module_geometry.f90), tau 1, rho0 1,
 *   f_ext (1e-5, 0, 0), target 1e-10, lbgpu_create -> lbgpu_flow_init -> lbgpu_equilibration
 *   -> lbgpu_flow_get.  Prints "steps <t>", then "l2err <t> <hex float>" per step and
 *   "jx <node> <hex float>" per node.  A failing call prints "status <rc> <message>" on
 *   stderr and exits with 3 (no GPU: LBGPU_ERR_CUDA from lbgpu_create, never a CPU result).
 */
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "lbgpu.h"

#define F(S, m) printf(#S " " #m " %zu %zu\n", offsetof(S, m), sizeof(((S *)0)->m))
#define Z(S) printf(#S " sizeof %zu\n", sizeof(S))

static int layout(void)
{
    F(lbgpu_params, lx); F(lbgpu_params, ly); F(lbgpu_params, lz); F(lbgpu_params, precision);
    F(lbgpu_params, relaxation_time); F(lbgpu_params, target_error); F(lbgpu_params, f_ext);
    F(lbgpu_params, rho0); F(lbgpu_params, device); Z(lbgpu_params);

    F(lbgpu_tracer, Db); F(lbgpu_tracer, ka); F(lbgpu_tracer, kd); F(lbgpu_tracer, Ds);
    F(lbgpu_tracer, z); F(lbgpu_tracer, f_ext); F(lbgpu_tracer, elec_slope); Z(lbgpu_tracer);

    F(lbgpu_pnp_params, bjl); F(lbgpu_pnp_params, sigma); F(lbgpu_pnp_params, lambda_D);
    F(lbgpu_pnp_params, D_plus); F(lbgpu_pnp_params, D_minus);
    F(lbgpu_pnp_params, charge_distrib); F(lbgpu_pnp_params, solver);
    F(lbgpu_pnp_params, omega); F(lbgpu_pnp_params, tol); F(lbgpu_pnp_params, max_iter);
    F(lbgpu_pnp_params, np_loop_bug); Z(lbgpu_pnp_params);

    F(lbgpu_cell, lx); F(lbgpu_cell, ly); F(lbgpu_cell, lz); F(lbgpu_cell, relaxation_time);
    F(lbgpu_cell, f_ext); F(lbgpu_cell, rho0); F(lbgpu_cell, tracer); Z(lbgpu_cell);

    F(lbgpu_request, cell); F(lbgpu_request, nature); F(lbgpu_request, arrival);
    F(lbgpu_request, max_steps); F(lbgpu_request, mp_steps); F(lbgpu_request, out_density);
    F(lbgpu_request, out_jx); F(lbgpu_request, out_jy); F(lbgpu_request, out_jz);
    Z(lbgpu_request);

    F(lbgpu_request_result, admitted); F(lbgpu_request_result, finished);
    F(lbgpu_request_result, steps); F(lbgpu_request_result, converged);
    F(lbgpu_request_result, status); F(lbgpu_request_result, mp_steps);
    F(lbgpu_request_result, fluid_nodes); F(lbgpu_request_result, vacf0);
    F(lbgpu_request_result, vacf_sum); Z(lbgpu_request_result);

    F(lbgpu_batch_tuning, tuned); F(lbgpu_batch_tuning, aa_work_list);
    F(lbgpu_batch_tuning, aa_min_blocks); F(lbgpu_batch_tuning, aa_tiles_per_claim);
    F(lbgpu_batch_tuning, smem_threads); F(lbgpu_batch_tuning, steps_per_graph);
    F(lbgpu_batch_tuning, aa_ms); F(lbgpu_batch_tuning, tiled_fluid_nodes);
    Z(lbgpu_batch_tuning);
    return 0;
}

static int fail(lbgpu_ctx *ctx, int rc, const char *what)
{
    char buf[512];
    lbgpu_last_error(ctx, buf, sizeof buf);
    fprintf(stderr, "status %d %s: %s\n", rc, what, buf);
    return 3;
}

static int c1(int max_steps)
{
    enum { LX = 4, LY = 4, LZ = 34, N = LX * LY * LZ };
    static int8_t nature[N];
    for (int k = 0; k < LZ; ++k)
        for (int j = 0; j < LY; ++j)
            for (int i = 0; i < LX; ++i)
                nature[i + LX * (j + LY * k)] = (k == 0 || k == LZ - 1) ? 1 : 0;
    lbgpu_params p;
    lbgpu_default_params(&p, LX, LY, LZ);
    p.f_ext[0] = 1e-5;
    p.precision = LBGPU_FP64;
    lbgpu_ctx *ctx = NULL;
    int rc = lbgpu_create(&p, nature, &ctx);
    if (rc) return fail(ctx, rc, "lbgpu_create");
    if ((rc = lbgpu_flow_init(ctx))) return fail(ctx, rc, "lbgpu_flow_init");
    const int cap = 1 << 16;
    double *hist = calloc(cap, sizeof(double));
    double *n = malloc(sizeof(double) * 19 * N), *m = malloc(sizeof(double) * 4 * N);
    int steps = 0;
    if ((rc = lbgpu_equilibration(ctx, max_steps, hist, cap, &steps)))
        return fail(ctx, rc, "lbgpu_equilibration");
    if ((rc = lbgpu_flow_get(ctx, n, m, m + N, m + 2 * N, m + 3 * N)))
        return fail(ctx, rc, "lbgpu_flow_get");
    printf("steps %d\n", steps);
    for (int t = 0; t < steps && t < cap; ++t) printf("l2err %d %a\n", t + 1, hist[t]);
    for (int q = 0; q < N; ++q) printf("jx %d %a\n", q, m[N + q]);
    lbgpu_destroy(ctx);
    free(hist);
    free(n);
    free(m);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc > 1 && !strcmp(argv[1], "layout")) return layout();
    if (argc > 1 && !strcmp(argv[1], "c1")) return c1(argc > 2 ? atoi(argv[2]) : 0);
    fprintf(stderr, "usage: %s layout | c1 [max_steps]\n", argv[0]);
    return 2;
}
