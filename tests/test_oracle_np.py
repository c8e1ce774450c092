"""Two independent restatements of the reference agree bit for bit.

oracle/lb_oracle.c (C) and oracle/np_oracle.py (numpy) were each written from the Fortran
sources of the reference.  The reference cannot be compiled here (no Fortran compiler), so its
own outputs are not available; two restatements that agree to the last bit on the collision,
the bounce-back + streaming, the moments, the whole flow loop (with the uniform and with the
compensated force), the tracer init and propagation,
charges_init, the Poisson sweeps, the Nernst-Planck update, the outer Poisson-Nernst-Planck
loop with its convergence and charge tests and the per-plane profiles make a misreading of the
Fortran by either one visible.  Sums that the
reference itself forms in an unspecified order (OpenMP reductions of the VACF) are compared to
1e-12 of |VACF(0)|.
"""
import math

import numpy as np
import pytest

from oracle import np_oracle as npo
from laboetie_gb300 import geometry as geo


def _random_nature(shape, frac, seed):
    rng = np.random.default_rng(seed)
    nat = (rng.random(shape) < frac).astype(np.int8)
    nat.flat[0] = 0
    return nat


def _random_state(nature, seed, amp=0.02):
    rng = np.random.default_rng(seed)
    n = npo.A0[:, None, None, None] * (1.0 + amp * rng.standard_normal((19,) + nature.shape))
    rho = n.sum(axis=0)
    j = [(n * npo.C[:, d][:, None, None, None]).sum(axis=0) + amp * rng.standard_normal(nature.shape)
         for d in range(3)]
    f = [1e-4 * rng.standard_normal(nature.shape) for _ in range(3)]
    return n, rho, j, f


BOXES = [
    ("slit-c1", lambda: geo.slit(4, 4, 34)),
    ("cc8", lambda: geo.cc(8, 8, 8)),
    ("random-6x5x7", lambda: _random_nature((7, 5, 6), 0.3, 1)),
    ("thin-x", lambda: _random_nature((9, 8, 1), 0.25, 2)),
    ("thin-2", lambda: _random_nature((2, 3, 2), 0.3, 3)),
    ("line-z", lambda: _random_nature((11, 1, 1), 0.3, 4)),
    ("cylinder", lambda: geo.cylinder(9, 9, 5)),
]


def test_tables_agree(oracle_mod):
    c, inv, a0, a1, a2, _ = oracle_mod.tables()
    assert np.array_equal(c, npo.C) and np.array_equal(inv, npo.INV)
    assert np.array_equal(a0, npo.A0) and np.array_equal(a1, npo.A1) and np.array_equal(a2, npo.A2)


@pytest.mark.parametrize("name,make", BOXES)
def test_interfacial_agrees(oracle_mod, name, make):
    nat = make()
    assert np.array_equal(oracle_mod.detect_interfacial(nat).astype(bool), npo.detect_interfacial(nat))


@pytest.mark.parametrize("tau", [0.6, 0.8, 1.0, 1.7])
@pytest.mark.parametrize("name,make", BOXES)
def test_collide_bit_exact(oracle_mod, name, make, tau):
    nat = make()
    n, rho, j, f = _random_state(nat, 11)
    want = oracle_mod.collide(nat, tau, n, rho, j, f)
    got = npo.collide(nat, tau, n, rho, *j, *f)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("name,make", BOXES)
def test_bounce_back_stream_bit_exact(oracle_mod, name, make):
    nat = make()
    n, _, _, _ = _random_state(nat, 12)
    assert np.array_equal(npo.bounce_back_stream(nat, n), oracle_mod.bounce_back_stream(nat, n))


@pytest.mark.parametrize("name,make", BOXES)
def test_moments_bit_exact(oracle_mod, name, make):
    nat = make()
    n, _, j, f = _random_state(nat, 13)
    rc, rho, jj, err = oracle_mod.moments(nat, n, f, j)
    neg, rho2, jj2, err2 = npo.moments(n, *f, *j)
    assert (rc != 0) == neg
    assert np.array_equal(rho2, rho) and all(np.array_equal(a, b) for a, b in zip(jj2, jj))
    assert err2 == err


@pytest.mark.parametrize("name,make,tau,f_ext,target", [
    ("slit-c1", lambda: geo.slit(4, 4, 34), 1.0, (1e-5, 0.0, 0.0), 1e-10),
    ("cc8", lambda: geo.cc(8, 8, 8), 0.8, (2e-5, 0.0, 0.0), 1e-9),
    ("random", lambda: _random_nature((5, 6, 7), 0.25, 5), 1.3, (0.0, 1e-5, 3e-6), 1e-9),
])
def test_flow_loop_bit_exact(oracle_mod, name, make, tau, f_ext, target):
    nat = make()
    ref = oracle_mod.equilibration(nat, tau=tau, target_error=target, f_ext=f_ext,
                                   max_steps=20000, check=False)
    got = npo.equilibration(nat, tau=tau, target_error=target, f_ext=f_ext, max_steps=20000)
    assert got["steps"] == ref["steps"]
    assert np.array_equal(got["l2err"], ref["l2err"])
    assert np.array_equal(got["n"], ref["n"]) and np.array_equal(got["rho"], ref["rho"])
    assert all(np.array_equal(a, b) for a, b in zip(got["j"], ref["j"]))


@pytest.mark.parametrize("label,make", [(-1, lambda: geo.bulk(9, 9, 9)),
                                        (1, lambda: geo.slit(9, 7, 11))])
def test_flow_loop_with_compensated_force_bit_exact(oracle_mod, label, make):
    """compensate_f_ext (equilibration.f90:388-487): the force on a particle of diameter 3 at the
    box centre, with the compensating background in the solid-free box (label -1) and without it
    between walls: the force field and the whole flow loop bit for bit."""
    nat = make()
    fe = (1e-4, 2e-5, 0.0)
    ref = oracle_mod.equilibration(nat, tau=1.0, target_error=1e-10, f_ext=fe, max_steps=20000,
                                   compensate_f_ext=True, particle_diameter=3, geometry_label=label)
    f = npo.compensated_force_field(nat, fe, 3, (0, 0, 0), label)
    assert all(np.array_equal(f[d], ref["f"][d]) for d in range(3))
    got = npo.equilibration(nat, tau=1.0, target_error=1e-10, f_ext=fe, max_steps=20000,
                            compensate_f_ext=True, particle_diameter=3, geometry_label=label)
    assert got["steps"] == ref["steps"]
    assert np.array_equal(got["l2err"], ref["l2err"])
    assert np.array_equal(got["n"], ref["n"]) and np.array_equal(got["rho"], ref["rho"])
    assert all(np.array_equal(a, b) for a, b in zip(got["j"], ref["j"]))
    assert all(np.array_equal(a, b) for a, b in zip(got["f"], ref["f"]))


@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("name,make", BOXES)
def test_profiles_bit_exact(oracle_mod, name, make, axis):
    """The per-plane flux and mean-density profiles the reference writes, from a random state:
    each plane's sums in the reference's element order, bit for bit."""
    nat = make()
    n, rho, j, f = _random_state(nat, 7)
    rho = np.where(nat == 0, rho, 0.0)
    ref = oracle_mod.profiles(nat, rho, j, axis)
    got = npo.profiles(rho, j, axis)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])


@pytest.mark.parametrize("adsorb", [False, True])
@pytest.mark.parametrize("name,make,tau,f_ext", [
    ("slit-c1", lambda: geo.slit(4, 4, 34), 1.0, (1e-5, 0.0, 0.0)),
    ("cc8", lambda: geo.cc(8, 8, 8), 0.8, (2e-5, 0.0, 0.0)),
])
def test_tracer_bit_exact(oracle_mod, name, make, tau, f_ext, adsorb):
    nat = make()
    ref = oracle_mod.equilibration(nat, tau=tau, target_error=1e-9, f_ext=f_ext, max_steps=50000)
    rho, j = ref["rho"], ref["j"]
    ka, kd = (0.01 * math.e, 0.01) if adsorb else (0.0, 0.0)
    nmp = oracle_mod.update_tracer_population(nat, rho, j, f_ext, 0.0, 0.01)
    nmp2 = npo.update_tracer_population(nat, rho, j, f_ext)
    assert np.array_equal(nmp2, nmp.reshape(nmp2.shape))
    mp = oracle_mod.MomentPropagation(nat, oracle_mod.detect_interfacial(nat), rho, nmp,
                                      ka=ka, kd=kd, Db=0.01)
    mp2 = npo.MomentPropagation(nat, rho, nmp2, ka=ka, kd=kd, Db=0.01)
    scale = np.abs(mp.vacf0).max()
    assert np.max(np.abs(mp2.vacf0 - mp.vacf0)) <= 1e-12 * scale
    assert np.array_equal(mp2.P, mp.P().reshape(mp2.P.shape))
    for it in range(1, 301):
        v, conv = mp.propagate(it)
        v2, conv2 = mp2.propagate(it)
        assert conv2 == conv
        assert np.max(np.abs(v2 - v)) <= 1e-12 * scale
        if conv:
            break
    assert np.array_equal(mp2.P, mp.P().reshape(mp2.P.shape))
    if adsorb:
        assert np.array_equal(mp2.A, mp.Pads().reshape(mp2.A.shape))
    mp.close()


@pytest.mark.parametrize("adsorb", [False, True])
@pytest.mark.parametrize("name,shape,frac,seed", [("random-7x5x6", (7, 5, 6), 0.3, 11),
                                                  ("random-9x8x3", (9, 8, 3), 0.2, 12),
                                                  ("random-2x3x5", (2, 3, 5), 0.25, 13)])
def test_tracer_bit_exact_on_ragged_boxes(oracle_mod, name, shape, frac, seed, adsorb):
    """The tracer restatements agree on ragged random boxes (thin axes, bounce-back links in
    every direction) from synthetic moments: any flow state is a valid input to both."""
    nat = _random_nature(shape, frac, seed)
    rng = np.random.default_rng(seed + 100)
    fl = nat == 0
    rho = np.where(fl, 1.0 + 0.01 * rng.standard_normal(nat.shape), 0.0)
    j = [np.where(fl, 2e-4 * rng.standard_normal(nat.shape), 0.0) for _ in range(3)]
    f_ext = (1e-5, -2e-6, 3e-6)
    ka, kd = (0.01 * math.e, 0.01) if adsorb else (0.0, 0.0)
    nmp = oracle_mod.update_tracer_population(nat, rho, j, f_ext, 0.0, 0.01)
    nmp2 = npo.update_tracer_population(nat, rho, j, f_ext)
    assert np.array_equal(nmp2, nmp.reshape(nmp2.shape))
    mp = oracle_mod.MomentPropagation(nat, oracle_mod.detect_interfacial(nat), rho, nmp,
                                      ka=ka, kd=kd, Db=0.01)
    mp2 = npo.MomentPropagation(nat, rho, nmp2, ka=ka, kd=kd, Db=0.01)
    scale = np.abs(mp.vacf0).max()
    assert np.max(np.abs(mp2.vacf0 - mp.vacf0)) <= 1e-12 * scale
    for it in range(1, 121):
        v, conv = mp.propagate(it)
        v2, conv2 = mp2.propagate(it)
        assert conv2 == conv
        assert np.max(np.abs(v2 - v)) <= 1e-12 * scale
        if conv:
            break
    assert np.array_equal(mp2.P, mp.P().reshape(mp2.P.shape)) and np.abs(mp2.P).max() > 0
    if adsorb:
        assert np.array_equal(mp2.A, mp.Pads().reshape(mp2.A.shape))
    mp.close()


@pytest.mark.parametrize("name,make", [("slit64", lambda: geo.slit(1, 1, 64)),
                                       ("random-7x5x6", lambda: _random_nature((7, 5, 6), 0.3, 21)),
                                       ("random-5x9x4", lambda: _random_nature((5, 9, 4), 0.35, 22)),
                                       ("cc8", lambda: geo.cc(8, 8, 8)),
                                       ("cyl", lambda: geo.cylinder(9, 9, 4))])
def test_poisson_sweeps_bit_exact(oracle_mod, name, make):
    nat = make()
    inter = oracle_mod.detect_interfacial(nat)
    sigma = -0.01 * int(((nat == 1) & (inter == 1)).sum())
    cp, cm, phi, an, _ = oracle_mod.charges_init(nat, inter, 0.4, sigma, 4.0)
    phi_o, an_o, it_o = oracle_mod.sor(nat, sigma, 0.4, cp, cm, phi, an)
    phi_n, an_n, it_n = npo.sor(nat, sigma, 0.4, cp, cm, phi, an)
    assert it_n == it_o
    assert np.array_equal(phi_n, phi_o)
    assert an_n == an_o


PNP_BOXES = [("slit64", lambda: geo.slit(1, 1, 64)),
             ("cc8", lambda: geo.cc(8, 8, 8)),
             ("cyl", lambda: geo.cylinder(9, 9, 4)),
             ("random-7x5x6", lambda: _random_nature((6, 5, 7), 0.3, 21))]


def _charged(oracle_mod, nat):
    inter = oracle_mod.detect_interfacial(nat)
    return inter, -0.01 * int(((nat == 1) & (inter == 1)).sum())


@pytest.mark.parametrize("name,make", PNP_BOXES)
def test_charges_init_bit_exact(oracle_mod, name, make):
    nat = make()
    inter, sigma = _charged(oracle_mod, nat)
    ref = oracle_mod.charges_init(nat, inter, 0.4, sigma, 4.0)
    got = npo.charges_init(nat, inter, 0.4, sigma, 4.0)
    for a, b in zip(got[:3], ref[:3]):
        assert np.array_equal(a, b)
    assert got[3] == ref[3] and got[4] == ref[4] and got[3] > 0


@pytest.mark.parametrize("loop_bug", [True, False])
@pytest.mark.parametrize("name,make", PNP_BOXES)
def test_just_eq_smolu_bit_exact(oracle_mod, name, make, loop_bug):
    """The Nernst-Planck update of the two restatements, from the charged state after the
    reference Poisson solve, with the reference's loop bounds (only the line (i, ly, lz) starts
    links) and with full ones: densities and iteration counts bit for bit."""
    nat = make()
    inter, sigma = _charged(oracle_mod, nat)
    cp, cm, phi, an, rho_ch = oracle_mod.charges_init(nat, inter, 0.4, sigma, 4.0)
    phi_o, _, _ = oracle_mod.sor(nat, sigma, 0.4, cp, cm, phi, an)
    ref = oracle_mod.just_eq_smolu(nat, phi_o, cp, cm, 0.05, 0.05, rho_ch, sigma, loop_bug=loop_bug)
    got = npo.just_eq_smolu(nat, phi_o, cp, cm, 0.05, 0.05, rho_ch, sigma, loop_bug=loop_bug)
    assert got[2] == ref[2] >= 1
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    if not loop_bug:
        assert not np.array_equal(got[0], cp)   # charge moved


@pytest.mark.parametrize("loop_bug", [True, False])
@pytest.mark.parametrize("name,make", PNP_BOXES)
def test_pnp_outer_loop_bit_exact(oracle_mod, name, make, loop_bug):
    """Three outer iterations of the Poisson-Nernst-Planck loop (backup, Poisson solve, one
    Nernst-Planck update, convergence test) in both restatements: fields, anormf0, the sweep
    total bit for bit, and the charge-conservation test alike."""
    nat = make()
    inter, sigma = _charged(oracle_mod, nat)
    cp, cm, phi, an, rho_ch = oracle_mod.charges_init(nat, inter, 0.4, sigma, 4.0)
    ref = oracle_mod.pnp(nat, 0.4, sigma, 0.05, 0.05, rho_ch, cp, cm, phi, an, loop_bug=loop_bug,
                         max_outer=3, check=False)
    got = npo.pnp(nat, 0.4, sigma, 0.05, 0.05, rho_ch, cp, cm, phi, an, loop_bug=loop_bug,
                  max_outer=3)
    assert got["outer"] == ref["outer"] and got["sor_iters"] == ref["sor_iters"]
    for k in ("c_plus", "c_minus", "phi"):
        assert np.array_equal(got[k], ref[k])
    assert got["anormf0"] == ref["anormf0"]
    assert got["converged"] == (ref["status"] == 0)
    rc, s_ref, f_ref = oracle_mod.charge_test(nat, ref["c_plus"], ref["c_minus"], sigma)
    ok, s_got, f_got = npo.charge_test(nat, got["c_plus"], got["c_minus"], sigma)
    assert (s_got, f_got) == (s_ref, f_ref) and ok == (rc == 0)


def _collide_regrouped(nature, tau, n, rho, jx, jy, jz, fx, fy, fz):
    """The reference's collision (module_collision.f90:77-104) with its terms regrouped as
    E +- O per velocity pair: mathematically equal, rounded differently."""
    fl = nature == 0
    with np.errstate(divide="ignore", invalid="ignore"):
        ir = np.where(fl, 1.0 / rho, 0.0)
    ux, uy, uz = jx * ir, jy * ir, jz * ir
    ju = jx * ux + jy * uy + jz * uz
    uF = ux * fx + uy * fy + uz * fz
    c1, c2, c3 = 1 - 1 / tau, 1 / tau, 1 - 1 / (2 * tau)
    out = n.copy()
    for l in range(19):
        c = npo.C[l].astype(float)
        cj, cu, cF = (c[0] * a + c[1] * b + c[2] * d for a, b, d in ((jx, jy, jz), (ux, uy, uz), (fx, fy, fz)))
        E = c2 * (npo.A0[l] * rho + npo.A2[l] * (cj * cu - npo.CSQ * ju)) + c3 * (2 * npo.A2[l] * cu * cF - npo.A1[l] * uF)
        O = c2 * npo.A1[l] * cj + c3 * npo.A1[l] * cF
        out[l] = np.where(fl, c1 * n[l] + (E + O), n[l])
    return out


def test_flux_rounding_floor_under_regrouping():
    """The rounding floor that any FP64 implementation other than an operation-for-operation one
    meets: the reference's loop with its collision regrouped (above) against the operation-for-
    operation restatement, 300 forced steps on a touching-spheres cell 12^3.  Populations and
    density stay within ~1e-15 of their scale, while the flux, a sum of populations that nearly
    cancel, moves by more than 1e-13 of its own largest value (a few 1e-12 here) and stays far
    below 1e-12 of the density's scale: the scale the FP64 fused context's flux is held to."""
    nat = geo.cc(12, 12, 12)
    f_ext, tau, K = (2e-5, -1e-5, 5e-6), 0.8, 300

    def run(coll):
        n, rho = npo.init_populations(nat)
        z = np.zeros(nat.shape)
        j = [z.copy(), z.copy(), z.copy()]
        fon = [np.where(nat == 0, f_ext[d], 0.0) for d in range(3)]
        for t in range(1, K + 1):
            f = [z, z, z] if t == 1 else fon
            n = coll(nat, tau, n, rho, *j, *f)
            n = npo.bounce_back_stream(nat, n)
            _, rho, j, _ = npo.moments(n, *f, *j)
        return n, rho, j

    a, b = run(npo.collide), run(_collide_regrouped)
    assert np.max(np.abs(a[0] - b[0])) <= 1e-14 * np.max(np.abs(a[0]))
    assert np.max(np.abs(a[1] - b[1])) <= 1e-14 * np.max(np.abs(a[1]))
    worst = max(np.max(np.abs(a[2][d] - b[2][d])) / np.max(np.abs(a[2][d])) for d in range(3))
    assert worst > 1e-13                 # the flux's own scale: a floor near 1e-12
    for d in range(3):
        assert np.max(np.abs(a[2][d] - b[2][d])) <= 1e-14 * np.max(np.abs(a[1]))
