"""The CPU oracle against known answers: the reference's own invariants, analytic solutions and
the committed fixtures in tests/golden/ (generated by tests/golden/make_golden.py).

The reference ships no golden vectors and cannot be built here (no Fortran compiler), so these
known answers are what pins the oracle.
"""
import math
import os

import numpy as np
import pytest

from laboetie_gb300 import geometry as geo

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_lattice_tables(oracle_mod):
    c, inv, a0, a1, a2, de = oracle_mod.tables()
    assert abs(a0.sum() - 1.0) <= np.finfo(np.float32).eps        # module_lbmodel.f90:151
    assert np.array_equal(c[inv], -c)                             # module_lbmodel.f90:156-162
    assert np.allclose(a1, 3 * a0, rtol=1e-15) and np.allclose(a2, 4.5 * a0, rtol=1e-15)
    # second-order isotropy of D3Q19: sum_l w c_a c_b = cs^2 delta_ab
    M = np.einsum("l,la,lb->ab", a0, c, c)
    assert np.allclose(M, np.eye(3) / 3, atol=1e-16)
    assert de[0] == 0 and np.all(de[1:7] == 1) and np.all(de[7:] == math.sqrt(2.0))


def test_interfacial_slit(oracle_mod):
    nat = geo.slit(3, 2, 9)
    inter = oracle_mod.detect_interfacial(nat)
    want = np.zeros(nat.shape, np.uint8)
    want[[0, 1, -2, -1]] = 1
    assert np.array_equal(inter, want)


def test_interfacial_matches_a_numpy_restatement(oracle_mod):
    rng = np.random.default_rng(4)
    nat = (rng.random((5, 6, 7)) < 0.3).astype(np.int8)
    c, *_ = oracle_mod.tables()
    diff = np.zeros(nat.shape, bool)
    for l in range(1, 19):
        nb = np.roll(nat, shift=(-c[l, 2], -c[l, 1], -c[l, 0]), axis=(0, 1, 2))
        diff |= nb != nat
    assert np.array_equal(oracle_mod.detect_interfacial(nat), diff.astype(np.uint8))


def test_collide_keeps_the_rest_state(oracle_mod):
    nat = geo.slit(2, 3, 6)
    n, rho = oracle_mod.init_populations(nat, 1.0)
    z = [np.zeros(nat.shape)] * 3
    out = oracle_mod.collide(nat, 0.8, n, rho, z, z)
    assert np.allclose(out, n, rtol=0, atol=1e-17)


def test_stream_conserves_populations(oracle_mod):
    rng = np.random.default_rng(5)
    nat = (rng.random((4, 5, 6)) < 0.3).astype(np.int8)
    n = rng.random((19,) + nat.shape)
    out = oracle_mod.bounce_back_stream(nat, n)
    assert np.isclose(out.sum(), n.sum(), rtol=1e-14)
    # pull form of the swap + push (the rule the GPU kernels implement)
    c, inv, *_ = oracle_mod.tables()
    want = np.empty_like(n)
    for l in range(19):
        src = np.roll(n[l], shift=(c[l, 2], c[l, 1], c[l, 0]), axis=(0, 1, 2))
        srcnat = np.roll(nat, shift=(c[l, 2], c[l, 1], c[l, 0]), axis=(0, 1, 2))
        want[l] = np.where(srcnat == nat, src, n[inv[l]])
    assert np.array_equal(out, want)


@pytest.fixture(scope="module")
def c1_flow(oracle_mod):
    nat = geo.slit(4, 4, 34)
    return nat, oracle_mod.equilibration(nat, tau=1.0, target_error=1e-10, f_ext=(1e-5, 0, 0),
                                         max_steps=100000)


def test_c1_poiseuille_and_mass(c1_flow):
    """Steady slit flow: u(z) is the parabola of curvature -F/nu between the halfway walls (up to
    a uniform slip), and the mass of the fluid is conserved."""
    nat, r = c1_flow
    F, nu = 1e-5, (1.0 - 0.5) / 3.0
    u = (r["j"][0] / np.where(r["rho"] > 0, r["rho"], 1.0))[:, 0, 0]
    d2 = u[2:-3] - 2 * u[3:-2] + u[4:-1]
    assert np.allclose(d2, -F / nu, rtol=2e-6), d2
    z = np.arange(1, 35, dtype=float)
    ua = F / (2 * nu) * (z - 1.5) * (34 - 0.5 - z)
    slip = (u - ua)[1:-1]
    assert np.ptp(slip) < 2e-5 * ua.max()
    assert abs(r["rho"].sum() - (nat == 0).sum()) < 2e-12 * (nat == 0).sum()


def test_c1_phase_machine(c1_flow):
    nat, r = c1_flow
    h = r["l2err"]
    assert h[0] == 0.0 and h[1] == 0.0 and h[2] == 0.0   # at rest until the force is switched on
    assert h[3] > 1e-6                                     # force on from the collision of step 4
    assert h[-1] <= 1e-10 and np.all(h[3:-1] > 1e-10)


def test_bulk_vacf_known_answer(oracle_mod):
    nat = geo.bulk(4, 3, 5)
    rho = np.ones(nat.shape)
    j = [np.zeros(nat.shape)] * 3
    nmp = oracle_mod.update_tracer_population(nat, rho, j, (0, 0, 0), 0.0, 0.02)
    mp = oracle_mod.MomentPropagation(nat, oracle_mod.detect_interfacial(nat), rho, nmp, Db=0.02)
    assert np.allclose(mp.vacf0, 0.04, rtol=1e-14)
    v, conv = mp.propagate(1)
    assert np.all(v == 0.0)
    mp.close()


def test_vacf0_closed_form_in_the_slit(oracle_mod):
    """Fluid at rest: VACF_a(0) = bw * sum_r sum_{l fluid link} (lambda w_l / 2) c_la^2."""
    nat = geo.slit(2, 3, 8)
    rho = np.where(nat == 0, 1.0, 0.0)
    j = [np.zeros(nat.shape)] * 3
    Db, ka, kd = 0.01, 0.02, 0.01
    inter = oracle_mod.detect_interfacial(nat)
    nmp = oracle_mod.update_tracer_population(nat, rho, j, (0, 0, 0), 0.0, Db)
    mp = oracle_mod.MomentPropagation(nat, inter, rho, nmp, ka=ka, kd=kd, Db=Db)
    c, inv, a0, *_ = oracle_mod.tables()
    lam = 4 * Db / (1 / 3)
    nf = (nat == 0).sum()
    nfi = ((nat == 0) & (inter == 1)).sum()
    bw = 1.0 / (nf + (ka / kd) * nfi)
    want = np.zeros(3)
    for l in range(1, 19):
        nbnat = np.roll(nat, shift=(-c[l, 2], -c[l, 1], -c[l, 0]), axis=(0, 1, 2))
        links = ((nat == 0) & (nbnat == 0)).sum()
        want += links * lam * a0[l] / 2 * c[l] ** 2
    assert np.allclose(mp.vacf0, bw * want, rtol=1e-13)
    mp.close()


def _charged_case(oracle_mod, seed=4):
    nat = geo.cc(7, 7, 7)
    rng = np.random.default_rng(seed)
    phi = 0.3 * rng.standard_normal(nat.shape)
    rho = np.where(nat == 0, 1.0, 0.0)
    j = [np.zeros(nat.shape)] * 3
    inter = oracle_mod.detect_interfacial(nat)
    return nat, phi, rho, j, inter


def test_charged_tracer_vacf0_closed_form(oracle_mod):
    """Fluid at rest, no field: n/rho - w = 0, so each link scatters lambda w_l fermi_l with
    fermi_l = 1/(1 + exp(z dphi)): VACF_a(0) = sum_r w_B(r) sum_{fluid links} lambda w_l fermi_l
    c_la^2, w_B(r) = exp(-z phi(r)) / (sum_fluid exp(-z phi) + K sum_interfacial exp(-z phi))."""
    nat, phi, rho, j, inter = _charged_case(oracle_mod)
    Db, ka, kd, z = 0.01, 0.01 * np.e, 0.01, 1.0
    nmp = oracle_mod.update_tracer_population(nat, rho, j, (0, 0, 0), z, Db)
    mp = oracle_mod.MomentPropagation(nat, inter, rho, nmp, ka=ka, kd=kd, Db=Db, z=z, phi=phi)
    c, inv, a0, *_ = oracle_mod.tables()
    lam = 4 * Db / (1 / 3)
    fl = nat == 0
    b = np.exp(-z * phi)
    pstat = b[fl].sum() + (ka / kd) * b[fl & (inter == 1)].sum()
    want = np.zeros(3)
    for l in range(1, 19):
        sh = lambda a: np.roll(a, shift=(-c[l, 2], -c[l, 1], -c[l, 0]), axis=(0, 1, 2))
        link = fl & (sh(nat) == 0)
        fermi = 1.0 / (1.0 + np.exp(z * (sh(phi) - phi)))
        want += (b / pstat * lam * a0[l] * fermi)[link].sum() * c[l] ** 2
    assert np.allclose(mp.vacf0, want, rtol=1e-12)
    mp.close()


def test_charged_tracer_in_a_uniform_potential_is_the_neutral_tracer(oracle_mod):
    nat, _, _, _, inter = _charged_case(oracle_mod)
    rng = np.random.default_rng(9)
    rho = np.where(nat == 0, 1.0 + 0.01 * rng.standard_normal(nat.shape), 0.0)
    j = [np.where(nat == 0, 1e-3 * rng.standard_normal(nat.shape), 0.0) for _ in range(3)]
    Db, ka, kd = 0.02, 0.02, 0.01
    out = []
    for z, phi in ((0.0, None), (1.5, np.full(nat.shape, 0.7))):
        nmp = oracle_mod.update_tracer_population(nat, rho, j, (1e-4, 0, 0), z, Db)
        mp = oracle_mod.MomentPropagation(nat, inter, rho, nmp, ka=ka, kd=kd, Db=Db, z=z, phi=phi)
        v = [mp.propagate(it)[0] for it in range(1, 6)]
        out.append((mp.vacf0.copy(), np.array(v), mp.P()))
        mp.close()
    (v0a, va, Pa), (v0b, vb, Pb) = out
    s = np.abs(v0a).max()
    assert np.max(np.abs(v0a - v0b)) <= 1e-13 * s and np.max(np.abs(va - vb)) <= 1e-13 * s
    assert np.max(np.abs(Pa - Pb)) <= 1e-13 * np.abs(Pa).max()


def test_charged_tracer_sign_symmetry(oracle_mod):
    """(z, phi) and (-z, -phi) give the same Boltzmann weights and fermi factors, bit for bit."""
    nat, phi, rho, j, inter = _charged_case(oracle_mod, seed=6)
    out = []
    for z, p in ((1.0, phi), (-1.0, -phi)):
        nmp = oracle_mod.update_tracer_population(nat, rho, j, (0, 0, 0), 0.0, 0.01)
        mp = oracle_mod.MomentPropagation(nat, inter, rho, nmp, ka=0.03, kd=0.01, Db=0.01, z=z, phi=p)
        v = [mp.propagate(it)[0] for it in range(1, 4)]
        out.append((mp.vacf0.copy(), np.array(v), mp.P()))
        mp.close()
    assert all(np.array_equal(a, b) for a, b in zip(out[0], out[1]))


def test_neutral_init_still_refuses_a_charged_tracer(oracle_mod):
    nat, phi, rho, j, inter = _charged_case(oracle_mod)
    nmp = oracle_mod.update_tracer_population(nat, rho, j, (0, 0, 0), 1.0, 0.01)
    with pytest.raises(oracle_mod.OracleError):
        oracle_mod.MomentPropagation(nat, inter, rho, nmp, Db=0.01, z=1.0)


def test_pnp_conserves_charge(oracle_mod):
    nat = geo.slit(1, 1, 16)
    inter = oracle_mod.detect_interfacial(nat)
    sigma = -0.01 * int(((nat == 1) & (inter == 1)).sum())
    cp, cm, phi, an, rho_ch = oracle_mod.charges_init(nat, inter, 0.4, sigma, 4.0)
    rc, s, f = oracle_mod.charge_test(nat, cp, cm, sigma)
    assert rc == 0 and abs(s - sigma) < 1e-14 and abs(f + sigma) < 1e-14
    r = oracle_mod.pnp(nat, 0.4, sigma, 0.05, 0.05, rho_ch, cp, cm, phi, an, max_outer=5000)
    rc, s, f = oracle_mod.charge_test(nat, r["c_plus"], r["c_minus"], sigma)
    assert rc == 0


def test_poisson_fixed_point(oracle_mod):
    """A tightly converged Jacobi solve satisfies (2/3) phi - sum_{l>0} w_l phi(x - c_l) = k rho_c."""
    nat = geo.cc(8, 8, 8)
    inter = oracle_mod.detect_interfacial(nat)
    sigma = -0.01 * int(((nat == 1) & (inter == 1)).sum())
    cp, cm, phi, an, _ = oracle_mod.charges_init(nat, inter, 0.4, sigma, 4.0)
    phi, an2, it = oracle_mod.sor(nat, sigma, 0.4, cp, cm, phi, an, omega=1.4, tol=1e-14)
    c, inv, a0, *_ = oracle_mod.tables()
    lap = (1 - a0[0]) * phi
    for l in range(1, 19):
        lap -= a0[l] * np.roll(phi, shift=(c[l, 2], c[l, 1], c[l, 0]), axis=(0, 1, 2))
    k = 4 * math.pi * 0.4 * (1 / 3) / 2
    assert np.max(np.abs(lap - k * (cp - cm))) < 1e-12 * np.max(np.abs(k * (cp - cm)))


def test_golden_fixtures(oracle_mod, c1_flow):
    g = np.load(os.path.join(GOLD, "c1_flow.npz"))
    nat, r = c1_flow
    assert r["steps"] == int(g["steps"])
    assert np.array_equal(r["l2err"][:50], g["l2err_head"])
    assert np.array_equal(r["l2err"][-50:], g["l2err_tail"])
    assert np.array_equal(r["j"][0][:, 0, 0], g["jx_z"])
    assert np.array_equal(r["rho"][:, 0, 0], g["rho_z"])
    m = np.load(os.path.join(GOLD, "c1_mp.npz"))
    rho, j = r["rho"], r["j"]
    for tag, ka in (("noads", 0.0), ("ads", 0.01 * math.e)):
        kd = 0.01 if ka else 0.0
        nmp = oracle_mod.update_tracer_population(nat, rho, j, (1e-5, 0, 0), 0.0, 0.01)
        mp = oracle_mod.MomentPropagation(nat, oracle_mod.detect_interfacial(nat), rho, nmp,
                                          ka=ka, kd=kd, Db=0.01)
        vac = [mp.vacf0] + [mp.propagate(it)[0] for it in range(1, 201)]
        mp.close()
        assert np.array_equal(np.array(vac), m[f"vacf_{tag}"])


def test_profiles_restatement_matches_plane_sums(oracle_mod):
    """equilibration.f90:159-175: per-plane sums of j and the mean density over nodes with
    density > epsilon; integer-valued fields make every sum exact, so any summation order agrees
    bit for bit."""
    rng = np.random.default_rng(4)
    lz, ly, lx = 5, 4, 7
    nat = np.zeros((lz, ly, lx), dtype=np.int8)
    rho = rng.integers(0, 3, size=(lz, ly, lx)).astype(np.float64)
    j = [rng.integers(-5, 6, size=(lz, ly, lx)).astype(np.float64) for _ in range(3)]
    for axis, red in ((0, (0, 1)), (1, (0, 2)), (2, (1, 2))):
        flux, dens = oracle_mod.profiles(nat, rho, j, axis)
        for d in range(3):
            assert np.array_equal(flux[:, d], j[d].sum(axis=red))
        cnt = np.maximum((rho > np.finfo(float).eps).sum(axis=red), 1)
        assert np.array_equal(dens, rho.sum(axis=red) / cnt)
