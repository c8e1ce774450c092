"""Parity at the benchmark configurations' own length and size.

* Slit 4x4x34 (tau 1, rho0 1, f_ext (1e-5,0,0)): the flow run to the reference's convergence test
  on the device, then the tracer phase of drop_tracers.f90:40-49 for its full 10000 steps
  (tmom 5000 -> tmax 15000), neutral tracer Db 0.01, with and without adsorption on the
  wall-adjacent fluid nodes (K = exp(-beta dF) = e, kd 0.01).  FP64: P and P_ads bit-identical to
  the oracle after 10000 steps, VACF within 1e-12 of |VACF(0)| at every step.
* Touching spheres 48^3 with surface charge -0.01 e per interfacial solid node (bjl 0.4,
  lambda_D 4, D+ = D- = 0.05), the reference's Jacobi solver and loop bounds: charges_init and
  every sweep of the first 20 outer iterations bit-identical, the same sweep counts, ion densities
  within 1e-12; then the outer loop run on the device to the reference's own convergence test
  (poisson_nernst_planck.f90:38-48), against the oracle's converged run recorded in
  tests/golden/pnp_cc48.npz (made by tests/golden/make_golden.py).
"""
import math
import os

import numpy as np
import pytest

from laboetie_gb300 import FP64, Box
from laboetie_gb300 import geometry as geo

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
BJL, LAMBDA_D, DPM = 0.4, 4.0, 0.05


@pytest.mark.parametrize("adsorb", [False, True])
def test_slit_tracer_phase_full_10000_steps_fp64(oracle_mod, adsorb):
    nat = geo.slit(4, 4, 34)
    f_ext = (1e-5, 0.0, 0.0)
    ref = oracle_mod.equilibration(nat, tau=1.0, target_error=1e-10, f_ext=f_ext, max_steps=200000)
    tr = dict(Db=0.01, ka=0.01 * math.e, kd=0.01) if adsorb else dict(Db=0.01)
    steps = 10000
    nmp = oracle_mod.update_tracer_population(nat, ref["rho"], ref["j"], f_ext, 0.0, tr["Db"])
    mp = oracle_mod.MomentPropagation(nat, oracle_mod.detect_interfacial(nat), ref["rho"], nmp,
                                      ka=tr.get("ka", 0.0), kd=tr.get("kd", 0.0), Db=tr["Db"])
    v0 = mp.vacf0.copy()
    vac, conv = [], False
    for it in range(1, steps + 1):
        v, conv = mp.propagate(it)
        vac.append(v)
        if conv:
            break
    vac = np.array(vac)
    P = mp.P().reshape(nat.shape + (3,))
    A = mp.Pads()
    A = A.reshape(nat.shape + (3,)) if A is not None else np.zeros(nat.shape + (3,))
    mp.close()
    with Box(nat, relaxation_time=1.0, f_ext=f_ext, precision=FP64) as box:
        box.flow_init()
        gsteps, _ = box.equilibration(max_steps=200000)
        assert gsteps == ref["steps"]
        g0 = box.mp_init(f_ext=f_ext, **tr)
        gv, gconv = box.mp_propagate(steps)
        GP, GA = box.mp_get()
    scale = np.abs(v0).max()
    assert np.max(np.abs(g0 - v0)) <= 1e-12 * scale
    assert len(gv) == len(vac) == steps and gconv == conv
    assert np.max(np.abs(gv - vac)) <= 1e-12 * scale
    assert np.array_equal(GP, P)
    assert np.array_equal(GA, A)
    if adsorb:
        assert np.abs(GA).sum() > 0


def _charged_cc48(oracle):
    nat = geo.cc(48, 48, 48)
    inter = oracle.detect_interfacial(nat)
    sigma = -0.01 * int(((nat == 1) & (inter == 1)).sum())
    cp, cm, phi, an, rho_ch = oracle.charges_init(nat, inter, BJL, sigma, LAMBDA_D)
    return nat, sigma, cp, cm, phi, an, rho_ch


def _close(a, b, rel):
    return np.max(np.abs(a - b)) <= rel * max(np.abs(b).max(), 1e-300)


def test_touching_spheres_48_first_outer_iterations(oracle_mod):
    nat, sigma, cp, cm, phi, an, rho_ch = _charged_cc48(oracle_mod)
    outer = 20
    with Box(nat) as box:
        an_g = box.pnp_init(bjl=BJL, sigma=sigma, lambda_D=LAMBDA_D, D_plus=DPM, D_minus=DPM)
        gcp, gcm, gphi, _ = box.pnp_get()
        assert an_g == an and np.array_equal(gcp, cp) and np.array_equal(gcm, cm)
        it = box.sor()
        _, _, gphi1, gan1 = box.pnp_get()
        phi1, an1, it1 = oracle_mod.sor(nat, sigma, BJL, cp, cm, phi, an)
        assert it == it1 and np.array_equal(gphi1, phi1) and gan1 == an1
        box.pnp_set(cp, cm, phi, an)   # back to the initial state for the outer loop
        g_outer, g_tot, rc = box.poisson_nernst_planck(max_outer=outer, check=False)
        gcp, gcm, gphi, _ = box.pnp_get()
    r = oracle_mod.pnp(nat, BJL, sigma, DPM, DPM, rho_ch, cp, cm, phi, an, loop_bug=True,
                       max_outer=outer, check=False)
    assert g_outer == r["outer"] == outer and g_tot == r["sor_iters"]
    assert rc != 0 and r["status"] != 0   # neither has converged after 20 iterations
    assert _close(gphi, r["phi"], 1e-11)
    assert _close(gcp, r["c_plus"], 1e-12) and _close(gcm, r["c_minus"], 1e-12)
    assert not np.array_equal(gcp, cp)     # charges do move in this geometry


def test_touching_spheres_48_run_to_the_reference_convergence(oracle_mod):
    g = np.load(os.path.join(GOLDEN, "pnp_cc48.npz"))
    nat, sigma, cp, cm, phi, an, rho_ch = _charged_cc48(oracle_mod)
    with Box(nat) as box:
        box.pnp_init(bjl=BJL, sigma=sigma, lambda_D=LAMBDA_D, D_plus=DPM, D_minus=DPM)
        outer, tot = box.poisson_nernst_planck(max_outer=100000)
        gcp, gcm, gphi, _ = box.pnp_get()
        rc_q, qs, qf = box.charge_test()
    # the device's exp() and flux sums differ from the oracle's in the last bits, so the
    # iteration at which the mean relative change first falls below 1e-12 may move by a step
    assert abs(outer - int(g["outer"])) <= 2
    assert tot == int(g["sor_iters"])
    for name, f in (("phi", gphi), ("c_plus", gcp), ("c_minus", gcm)):
        assert _close(f[::4, ::4, ::4], g[name + "_sub4"], 1e-10), name
        assert abs(f.sum() - g[name + "_sum"]) <= 1e-10 * np.abs(f).sum(), name
        assert abs((f * f).sum() - g[name + "_sumsq"]) <= 1e-10 * g[name + "_sumsq"], name
    assert rc_q == 0 and abs(qs - sigma) < 1e-10 and abs(qf + sigma) < 1e-10
