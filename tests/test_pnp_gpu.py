"""Parity of the GPU Poisson + Nernst-Planck path (C ABI) with the CPU oracle.

charges_init and every Jacobi sweep of the reference solver are bit-identical (the sweeps keep
the reference's operand order, FP64 without fused multiply-add); the Nernst-Planck link fluxes
use exp() and a different summation order, so ion densities are compared with tolerance 1e-12
relative to their largest value.  The 4-colour SOR is checked against a tightly converged
reference solve (same discrete equation).
"""
import numpy as np
import pytest

from laboetie_gb300 import Box, LbgpuError
from laboetie_gb300 import geometry as geo
from laboetie_gb300.lbgpu import POISSON_JACOBI, POISSON_SOR4

pytestmark = pytest.mark.gpu

BJL, LAMBDA_D, DPM = 0.4, 4.0, 0.05


def charged(oracle, nat):
    inter = oracle.detect_interfacial(nat)
    sigma = -0.01 * int(((nat == 1) & (inter == 1)).sum())
    cp, cm, phi, an, rho_ch = oracle.charges_init(nat, inter, BJL, sigma, LAMBDA_D)
    return sigma, cp, cm, phi, an, rho_ch


def ragged(shape, frac, seed):
    """A random box with thin and odd sides (fluid at the first node)."""
    rng = np.random.default_rng(seed)
    nat = (rng.random(shape) < frac).astype(np.int8)
    nat.flat[0] = 0
    return nat


def close(a, b, rel):
    scale = max(np.abs(b).max(), 1e-300)
    return np.max(np.abs(a - b)) <= rel * scale


@pytest.mark.parametrize("name,make", [("slit64", lambda: geo.slit(1, 1, 64)),
                                       ("cc8", lambda: geo.cc(8, 8, 8)),
                                       ("cyl", lambda: geo.cylinder(9, 9, 4)),
                                       ("random-7x5x6", lambda: ragged((6, 5, 7), 0.3, 21)),
                                       ("random-5x9x4", lambda: ragged((4, 9, 5), 0.35, 22))])
def test_charges_init_and_reference_sor_bit_exact(oracle_mod, name, make):
    nat = make()
    sigma, cp, cm, phi, an, rho_ch = charged(oracle_mod, nat)
    with Box(nat) as box:
        an_g = box.pnp_init(bjl=BJL, sigma=sigma, lambda_D=LAMBDA_D, D_plus=DPM, D_minus=DPM)
        gcp, gcm, gphi, _ = box.pnp_get()
        assert an_g == an
        assert np.array_equal(gcp, cp) and np.array_equal(gcm, cm) and np.all(gphi == 0)
        it = box.sor()
        gcp, gcm, gphi, gan = box.pnp_get()
    phi_o, an_o, it_o = oracle_mod.sor(nat, sigma, BJL, cp, cm, phi, an)
    assert it == it_o
    assert np.array_equal(gphi, phi_o)
    assert gan == an_o


@pytest.mark.parametrize("make,corner_solid", [(lambda: geo.cc(8, 8, 8), True),
                                               (lambda: ragged((6, 5, 7), 0.3, 21), False)],
                         ids=["cc8", "random-7x5x6"])
@pytest.mark.parametrize("loop_bug", [True, False])
def test_just_eq_smolu(oracle_mod, loop_bug, make, corner_solid):
    nat = make()
    sigma, cp, cm, phi, an, rho_ch = charged(oracle_mod, nat)
    phi_o, an_o, _ = oracle_mod.sor(nat, sigma, BJL, cp, cm, phi, an)
    cp_o, cm_o, it_o = oracle_mod.just_eq_smolu(nat, phi_o, cp, cm, DPM, DPM, rho_ch, sigma,
                                                loop_bug=loop_bug)
    with Box(nat) as box:
        box.pnp_init(bjl=BJL, sigma=sigma, lambda_D=LAMBDA_D, D_plus=DPM, D_minus=DPM,
                     np_loop_bug=loop_bug)
        box.sor()
        it = box.just_eq_smolu()
        gcp, gcm, _, _ = box.pnp_get()
    assert it == it_o
    assert close(gcp, cp_o, 1e-12) and close(gcm, cm_o, 1e-12)
    # with the reference's loop bounds only the line (i, ly, lz) starts links: in cc8 that line
    # lies in the solid corner spheres and no charge moves; in the random box it holds fluid
    # nodes and charge moves either way
    if corner_solid:
        assert np.array_equal(cp_o, cp) == loop_bug
    else:
        assert not np.array_equal(cp_o, cp)


@pytest.mark.parametrize("loop_bug", [True, False])
def test_pnp_outer_loop(oracle_mod, loop_bug):
    """poisson_nernst_planck.f90:38-48 for 4 outer iterations (the reference's 1e-12 relative
    change criterion is not met that early: both stop at the cap in the same state), then the
    charge conservation test."""
    nat = geo.cc(8, 8, 8)
    sigma, cp, cm, phi, an, rho_ch = charged(oracle_mod, nat)
    r = oracle_mod.pnp(nat, BJL, sigma, DPM, DPM, rho_ch, cp, cm, phi, an, loop_bug=loop_bug,
                       max_outer=4, check=False)
    with Box(nat) as box:
        box.pnp_init(bjl=BJL, sigma=sigma, lambda_D=LAMBDA_D, D_plus=DPM, D_minus=DPM,
                     np_loop_bug=loop_bug)
        outer, tot, rc = box.poisson_nernst_planck(max_outer=4, check=False)
        gcp, gcm, gphi, gan = box.pnp_get()
        rc_q, qs, qf = box.charge_test()
    assert (rc != 0) == (r["status"] != 0)
    assert outer == r["outer"] and tot == r["sor_iters"]
    assert close(gphi, r["phi"], 1e-11)
    assert close(gcp, r["c_plus"], 1e-12) and close(gcm, r["c_minus"], 1e-12)
    assert rc_q == 0 and abs(qs - sigma) < 1e-10 and abs(qf + sigma) < 1e-10


def test_pnp_slit_converges_in_one_outer_iteration(oracle_mod):
    """1x1x64 slit: the line (i, ly, lz) that just_eq_smolu visits is a wall node, so no charge
    moves and the loop stops after the first iteration, as in the reference."""
    nat = geo.slit(1, 1, 64)
    sigma, cp, cm, phi, an, rho_ch = charged(oracle_mod, nat)
    r = oracle_mod.pnp(nat, BJL, sigma, DPM, DPM, rho_ch, cp, cm, phi, an, loop_bug=True)
    with Box(nat) as box:
        box.pnp_init(bjl=BJL, sigma=sigma, lambda_D=LAMBDA_D, D_plus=DPM, D_minus=DPM)
        outer, tot = box.poisson_nernst_planck(max_outer=100)
        _, _, gphi, _ = box.pnp_get()
    assert outer == r["outer"] == 1 and tot == r["sor_iters"]
    assert np.array_equal(gphi, r["phi"])


def test_sor4_reaches_the_same_fixed_point(oracle_mod):
    nat = geo.cc(8, 8, 8)
    sigma, cp, cm, phi, an, rho_ch = charged(oracle_mod, nat)
    phi_o, _, _ = oracle_mod.sor(nat, sigma, BJL, cp, cm, phi, an, omega=1.4, tol=1e-14)
    with Box(nat) as box:
        box.pnp_init(bjl=BJL, sigma=sigma, lambda_D=LAMBDA_D, D_plus=DPM, D_minus=DPM,
                     solver=POISSON_SOR4, omega=1.8, tol=1e-13)
        it = box.sor()
        _, _, gphi, _ = box.pnp_get()
    assert it > 0
    assert close(gphi, phi_o, 1e-9)


def test_pnp_refusals():
    nat = geo.slit(1, 1, 16)
    with Box(nat) as box:
        with pytest.raises(LbgpuError):
            box.pnp_init(sigma=-0.02, charge_distrib="sol")   # charges_init.f90:96-100
        with pytest.raises(LbgpuError):
            box.pnp_init(sigma=-0.02, D_plus=-1.0)            # charges_init.f90:132


# --------------------------------------------------------------- multicolour SOR on any box

@pytest.mark.parametrize("name,make", [("slit64", lambda: geo.slit(1, 1, 64)),
                                       ("slit63", lambda: geo.slit(1, 1, 63)),
                                       ("cc9", lambda: geo.cc(9, 9, 9)),
                                       ("cyl", lambda: geo.cylinder(9, 9, 4))])
def test_multicolour_sor_on_any_box_reaches_the_fixed_point(oracle_mod, name, make):
    nat = make()
    sigma, cp, cm, phi, an, rho_ch = charged(oracle_mod, nat)
    phi_o, _, _ = oracle_mod.sor(nat, sigma, BJL, cp, cm, phi, an, omega=1.4, tol=1e-14)
    with Box(nat) as box:
        box.pnp_init(bjl=BJL, sigma=sigma, lambda_D=LAMBDA_D, D_plus=DPM, D_minus=DPM,
                     solver=POISSON_SOR4, omega=1.8, tol=1e-13)
        it = box.sor()
        _, _, gphi, _ = box.pnp_get()
    assert it > 0
    assert close(gphi, phi_o, 1e-9)


@pytest.mark.parametrize("name,make", [("slit64", lambda: geo.slit(1, 1, 64)),
                                       ("cc8", lambda: geo.cc(8, 8, 8))])
def test_jacobi_with_the_reference_tolerance_is_the_reference_solver(oracle_mod, name, make):
    """LBGPU_POISSON_JACOBI with omega 1.4 and tol = the reference's 1.0e-5 (a default real)
    sweeps exactly as the reference solver; the residual query returns the reference's stopping
    measure at the final potential."""
    from oracle import np_oracle as npo

    nat = make()
    sigma, cp, cm, phi, an, rho_ch = charged(oracle_mod, nat)
    phi_o, an_o, it_o = oracle_mod.sor(nat, sigma, BJL, cp, cm, phi, an)
    with Box(nat) as box:
        box.pnp_init(bjl=BJL, sigma=sigma, lambda_D=LAMBDA_D, D_plus=DPM, D_minus=DPM,
                     solver=POISSON_JACOBI, omega=1.4, tol=float(np.float32(1e-5)))
        it = box.sor()
        _, _, gphi, gan = box.pnp_get()
        res, _ = box.poisson_residual()
    assert it == it_o and np.array_equal(gphi, phi_o) and gan == an_o
    # the measure restated on the host: sum |phi* - phi| with phi* = sum_l w_l phi(x - c_l) + b
    factor = 4.0 * npo.PI * BJL * npo.KBT / 2.0
    star = sum(npo.A0[l] * npo._shift(phi_o, npo.C[l]) for l in range(19)) + factor * (cp - cm)
    want = np.abs(star - phi_o).sum()
    assert abs(res - want) <= 1e-12 * want
