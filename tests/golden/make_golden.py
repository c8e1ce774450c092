"""Generates the fixtures of tests/golden/ from the CPU oracle.

The reference (Fortran) ships no golden vectors and no Fortran compiler is available where this
project is built, so these fixtures record the oracle's outputs on the Poiseuille slit of the
reference's small case (4x4x34, tau 1, f_ext (1e-5,0,0), target 1e-10; tracer Db 0.01 with and without adsorption,
K = e with kd 0.01).  They pin the oracle against regressions and give the GPU tests fixed
expected values; they are not outputs of the reference itself.

pnp_cc48.npz records the oracle's Poisson-Nernst-Planck equilibration of the charged-solutes
case on touching spheres 48^3 (bjl 0.4, lambda_D 4, D+ = D- = 0.05, surface charge -0.01 e per
interfacial solid node, the reference's Jacobi solver and loop bounds) run to the reference's own
convergence test (poisson_nernst_planck.f90:38-48: mean relative changes of phi, c+ and c- all
below 1e-12): the outer and sweep counts and the converged fields (a few minutes of CPU).

Run from the repository root:  python tests/golden/make_golden.py [c1] [pnp]
"""
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from laboetie_gb300 import geometry as geo  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def save_pnp_cc48(r):
    """Counts, every field on the sub-lattice of every 4th node along each axis, and each field's
    sum and sum of squares over all nodes (the full fields would take about 1 MB)."""
    out = dict(outer=r["outer"], sor_iters=r["sor_iters"], anormf0=r["anormf0"])
    for k in ("phi", "c_plus", "c_minus"):
        f = np.asarray(r[k])
        out[k + "_sub4"] = f[::4, ::4, ::4]
        out[k + "_sum"] = f.sum()
        out[k + "_sumsq"] = (f * f).sum()
    np.savez_compressed(os.path.join(HERE, "pnp_cc48.npz"), **out)


def pnp_cc48():
    nat = geo.cc(48, 48, 48)
    inter = oracle.detect_interfacial(nat)
    sigma = -0.01 * int(((nat == 1) & (inter == 1)).sum())
    cp, cm, phi, an, rho_ch = oracle.charges_init(nat, inter, 0.4, sigma, 4.0)
    r = oracle.pnp(nat, 0.4, sigma, 0.05, 0.05, rho_ch, cp, cm, phi, an, loop_bug=True,
                   max_outer=100000)
    save_pnp_cc48(r)
    print("pnp cc48: outer", r["outer"], "sweeps", r["sor_iters"])


def main(parts):
    if "pnp" in parts:
        pnp_cc48()
    if "c1" not in parts:
        return
    nat = geo.slit(4, 4, 34)
    r = oracle.equilibration(nat, tau=1.0, target_error=1e-10, f_ext=(1e-5, 0, 0), max_steps=100000)
    np.savez(os.path.join(HERE, "c1_flow.npz"), steps=r["steps"], l2err_head=r["l2err"][:50],
             l2err_tail=r["l2err"][-50:], jx_z=r["j"][0][:, 0, 0], rho_z=r["rho"][:, 0, 0])
    out = {}
    for tag, ka in (("noads", 0.0), ("ads", 0.01 * math.e)):
        kd = 0.01 if ka else 0.0
        nmp = oracle.update_tracer_population(nat, r["rho"], r["j"], (1e-5, 0, 0), 0.0, 0.01)
        mp = oracle.MomentPropagation(nat, oracle.detect_interfacial(nat), r["rho"], nmp,
                                      ka=ka, kd=kd, Db=0.01)
        vac = [mp.vacf0] + [mp.propagate(it)[0] for it in range(1, 201)]
        mp.close()
        out[f"vacf_{tag}"] = np.array(vac)
    np.savez(os.path.join(HERE, "c1_mp.npz"), **out)
    print("steps", r["steps"])


if __name__ == "__main__":
    main(sys.argv[1:] or ["c1", "pnp"])
