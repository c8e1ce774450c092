"""LBGPU_FP64_FUSED: FP64 flow and tracer with fused multiply-adds, within 1e-12 of the oracle.

The strict FP64 context reproduces the reference operation for operation; the fused one regroups
the collision per pair of opposite velocities and fuses multiply-adds (about half the FP64
operations, which bound the FP64 kernels on GB300), and fuses the tracer gathers.  The bar is the
FP64 parity tolerance of the benchmark configurations, 1e-12 relative: for populations and
density of their largest value; for the flux of the density's scale, because j is a sum of
populations that nearly cancel (|j| ~ 1e-4 |n| here) and any regrouping of the reference's
arithmetic moves it by a few 1e-12 of its own largest value after a few hundred steps
(tests/test_oracle_np.py::test_flux_rounding_floor_under_regrouping shows two CPU restatements
that differ only in grouping doing so), so it is also held to 1e-10 of its own largest value;
VACF of |VACF(0)|.  Checked on the reference's small slit case (flow to the reference's
convergence test, then the full 10000-step tracer phase), a touching-spheres cell 12^3 and two
steps of the 192^3 porous medium.
"""
import math

import numpy as np
import pytest

from laboetie_gb300 import FP64, FP64_FUSED, Box
from laboetie_gb300 import geometry as geo

from test_flow_gpu import oracle_fixed_steps

pytestmark = pytest.mark.gpu


def _close(a, b, rel=1e-12, scale=None):
    scale = np.max(np.abs(b)) if scale is None else scale
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) <= rel * scale


def _flux_close(j, j_ref, rho_ref):
    return _close(j, j_ref, 1e-12, scale=np.max(np.abs(rho_ref))) and _close(j, j_ref, 1e-10)


def test_slit_flow_and_full_tracer_phase(oracle_mod):
    nat = geo.slit(4, 4, 34)
    f_ext = (1e-5, 0.0, 0.0)
    ref = oracle_mod.equilibration(nat, tau=1.0, target_error=1e-10, f_ext=f_ext, max_steps=200000)
    with Box(nat, relaxation_time=1.0, f_ext=f_ext, precision=FP64_FUSED) as box:
        box.flow_init()
        steps, hist = box.equilibration(max_steps=200000, hist_cap=200000)
        n, rho, j = box.flow_get()
        tr = dict(Db=0.01, ka=0.01 * math.e, kd=0.01)
        g0 = box.mp_init(f_ext=f_ext, **tr)
        gv, _ = box.mp_propagate(10000)
        GP, GA = box.mp_get()
    # the exit step is decided by l2err <= 1e-10 at the step where l2err falls below it; a
    # last-bit difference in l2err could move it by one step
    assert abs(steps - ref["steps"]) <= 1
    assert _flux_close(j[0], ref["j"][0], ref["rho"]) and _close(rho, ref["rho"])
    nmp = oracle_mod.update_tracer_population(nat, ref["rho"], ref["j"], f_ext, 0.0, tr["Db"])
    mp = oracle_mod.MomentPropagation(nat, oracle_mod.detect_interfacial(nat), ref["rho"], nmp,
                                      ka=tr["ka"], kd=tr["kd"], Db=tr["Db"])
    v0 = mp.vacf0.copy()
    vac = np.array([mp.propagate(it)[0] for it in range(1, 10001)])
    P = mp.P().reshape(nat.shape + (3,))
    A = mp.Pads().reshape(nat.shape + (3,))
    mp.close()
    scale = np.abs(v0).max()
    assert np.max(np.abs(g0 - v0)) <= 1e-12 * scale
    assert np.max(np.abs(gv - vac)) <= 1e-12 * scale
    assert _close(GP, P) and _close(GA, A)


def test_cc12_fixed_steps(oracle_mod):
    nat = geo.cc(12, 12, 12)
    f_ext = (2e-5, -1e-5, 5e-6)
    K = 300
    with Box(nat, relaxation_time=0.8, f_ext=f_ext, precision=FP64_FUSED) as box:
        box.flow_init()
        box.flow_steps(K, force_on=True)
        n, rho, j = box.flow_get()
    n_o, rho_o, j_o = oracle_fixed_steps(oracle_mod, nat, 0.8, f_ext, K)
    assert _close(n, n_o) and _close(rho, rho_o)
    for d in range(3):
        assert _flux_close(j[d], j_o[d], rho_o)


def test_porous_192_two_steps_and_speed(oracle_mod):
    medium = geo.porous_spheres(192, 8.0, 0.60, 20261203)
    FE = (1e-6, 0.0, 0.0)
    with Box(medium, relaxation_time=0.8, f_ext=FE, precision=FP64_FUSED) as box:
        box.flow_init()
        box.flow_steps(2, force_on=True)
        n, rho, j = box.flow_get()
        ms_fused = box.time_flow_steps(40)
    n_o, rho_o, j_o = oracle_fixed_steps(oracle_mod, medium, 0.8, FE, 2)
    assert _close(n, n_o) and _close(rho, rho_o) and _flux_close(j[0], j_o[0], rho_o)
    with Box(medium, relaxation_time=0.8, f_ext=FE, precision=FP64) as box:
        box.flow_init()
        ms_strict = box.time_flow_steps(40)
    # the fused step does about half the FP64 operations of the strict one
    assert ms_fused < 0.75 * ms_strict, (ms_fused, ms_strict)
