"""Generates the fixtures of tests/golden/ from the CPU oracle.

The reference (Fortran) ships no golden vectors and no Fortran compiler is available where this
project is built, so these fixtures record the oracle's outputs on the Poiseuille slit of the
reference's small case (4x4x34, tau 1, f_ext (1e-5,0,0), target 1e-10; tracer Db 0.01 with and without adsorption,
K = e with kd 0.01).  They pin the oracle against regressions and give the GPU tests fixed
expected values; they are not outputs of the reference itself.

Run from the repository root:  python tests/golden/make_golden.py
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


def main():
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
    main()
