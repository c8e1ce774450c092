"""Charged tracers (lbgpu_mp_init_charged) against the oracle's restatement of the reference's
formulas (module_moment_propagation.f90:97-135, 223-229, 295-327), which the reference itself
stops before.  Parity here is with the oracle only (unpinned against the reference's outputs).

* FP64: the scattering table is built with device exp(), the oracle with the C library's, so P
  and VACF are compared within 1e-12 (relative to max |P| and to |VACF(0)|), not bit for bit.
* FP32 against FP64: VACF within 1e-5 of |VACF(0)| after 200 steps.
* A uniform potential gives the neutral tracer's results; lbgpu_mp_init still refuses z != 0,
  and the charged init refuses a context without a potential.
"""
import numpy as np
import pytest

from laboetie_gb300 import FP32_DEV, Box, LbgpuError
from laboetie_gb300 import geometry as geo

pytestmark = pytest.mark.gpu

BJL, LAMBDA_D, DPM = 0.4, 4.0, 0.05


def potential(oracle, nat):
    """charges_init + the reference SOR (oracle): the converged potential phi of the box."""
    inter = oracle.detect_interfacial(nat)
    sigma = -0.01 * int(((nat == 1) & (inter == 1)).sum())
    cp, cm, phi, an, rho_ch = oracle.charges_init(nat, inter, BJL, sigma, LAMBDA_D)
    phi, an, _ = oracle.sor(nat, sigma, BJL, cp, cm, phi, an)
    return cp, cm, phi, an, inter


def flow_moments(nat, seed):
    rng = np.random.default_rng(seed)
    fl = nat == 0
    rho = np.where(fl, 1.0 + 1e-3 * rng.standard_normal(nat.shape), 0.0)
    j = [np.where(fl, 2e-4 * rng.standard_normal(nat.shape), 0.0) for _ in range(3)]
    return rho, j


def oracle_run(oracle, nat, inter, rho, j, phi, steps, z, E=(0.0, 0.0, 0.0), **tr):
    nmp = oracle.update_tracer_population(nat, rho, j, (0, 0, 0), z, tr["Db"], elec_slope=E)
    mp = oracle.MomentPropagation(nat, inter, rho, nmp, ka=tr.get("ka", 0.0), kd=tr.get("kd", 0.0),
                                  Db=tr["Db"], z=z, phi=phi, elec_slope=E)
    v0 = mp.vacf0.copy()
    v = np.array([mp.propagate(it)[0] for it in range(1, steps + 1)])
    P = mp.P().reshape(nat.shape + (3,))
    mp.close()
    return v0, v, P


def gpu_run(nat, rho, j, pnp, steps, z, precision=None, E=(0.0, 0.0, 0.0), **tr):
    cp, cm, phi, an = pnp
    kw = {} if precision is None else dict(precision=precision)
    with Box(nat, **kw) as box:
        box.pnp_init(bjl=BJL, sigma=0.0, lambda_D=LAMBDA_D, D_plus=DPM, D_minus=DPM)
        box.pnp_set(cp, cm, phi, an)
        v0 = box.mp_init(moments=(rho, j), charged=True, z=z, elec_slope=E, **tr)
        v, _ = box.mp_propagate(steps)
        P, _ = box.mp_get()
    return v0, v, P


@pytest.mark.parametrize("name,make,z,E", [
    ("cc12", lambda: geo.cc(12, 12, 12), 1.0, (0.0, 0.0, 0.0)),
    ("slit64", lambda: geo.slit(1, 1, 64), -2.0, (0.0, 0.0, 0.0)),
    ("cc10 field", lambda: geo.cc(10, 10, 10), 1.0, (1e-3, -2e-3, 5e-4)),
])
def test_fp64_charged_tracer_matches_oracle(oracle_mod, name, make, z, E):
    nat = make()
    cp, cm, phi, an, inter = potential(oracle_mod, nat)
    rho, j = flow_moments(nat, seed=len(name))
    tr = dict(Db=0.01, ka=0.01 * np.e, kd=0.01)
    v0, v, P = oracle_run(oracle_mod, nat, inter, rho, j, phi, 60, z, E, **tr)
    g0, gv, GP = gpu_run(nat, rho, j, (cp, cm, phi, an), 60, z, E=E, **tr)
    s = np.abs(v0).max()
    assert np.max(np.abs(g0 - v0)) <= 1e-12 * s
    assert len(gv) == len(v) and np.max(np.abs(gv - v)) <= 1e-12 * s
    assert np.max(np.abs(GP - P)) <= 1e-12 * np.abs(P).max()


def test_fp32_charged_tracer_against_fp64(oracle_mod):
    nat = geo.cc(16, 16, 16)
    cp, cm, phi, an, inter = potential(oracle_mod, nat)
    rho, j = flow_moments(nat, seed=3)
    tr = dict(Db=0.01, ka=0.01 * np.e, kd=0.01)
    g0, gv, _ = gpu_run(nat, rho, j, (cp, cm, phi, an), 200, 1.0, **tr)
    f0, fv, _ = gpu_run(nat, rho, j, (cp, cm, phi, an), 200, 1.0, precision=FP32_DEV, **tr)
    s = np.abs(g0).max()
    assert np.max(np.abs(f0 - g0)) <= 1e-5 * s
    assert np.max(np.abs(fv - gv)) <= 1e-5 * s


def test_uniform_potential_gives_the_neutral_tracer(oracle_mod):
    nat = geo.cc(10, 10, 10)
    cp, cm, _, an, _ = potential(oracle_mod, nat)
    rho, j = flow_moments(nat, seed=5)
    tr = dict(Db=0.02, ka=0.02, kd=0.01)
    phi = np.full(nat.shape, 0.4)
    g0, gv, GP = gpu_run(nat, rho, j, (cp, cm, phi, an), 30, 2.0, **tr)
    with Box(nat) as box:
        n0 = box.mp_init(moments=(rho, j), **tr)
        nv, _ = box.mp_propagate(30)
        NP, _ = box.mp_get()
    s = np.abs(n0).max()
    assert np.max(np.abs(g0 - n0)) <= 1e-13 * s and np.max(np.abs(gv - nv)) <= 1e-13 * s
    assert np.max(np.abs(GP - NP)) <= 1e-13 * np.abs(NP).max()


def test_refusals():
    nat = geo.cc(8, 8, 8)
    rho, j = flow_moments(nat, seed=1)
    with Box(nat) as box:
        with pytest.raises(LbgpuError, match="charged tracers are not implemented"):
            box.mp_init(moments=(rho, j), Db=0.01, z=1.0)
        with pytest.raises(LbgpuError, match="no potential"):
            box.mp_init(moments=(rho, j), charged=True, Db=0.01, z=1.0)
