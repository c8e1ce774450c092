"""The coupled electrokinetic operators: electrostatic_pot, comp_j, smolu, advect.

The reference calls them only from its coupled time loop in src/trash/ (which no longer builds),
so each is checked as the operator it is: the two CPU restatements (oracle/lb_oracle.c and
oracle/np_oracle.py) agree bit for bit (the numpy one calls the C library's exp, as the C one
does), and the library (-m gpu) agrees with the oracle bit for bit where no exponential is
involved (electrostatic_pot, comp_j, advect) and within 1e-12 of each value's scale in smolu
(device exp and a different order of the global current sums).  States come from the
charged-solute setup of the benchmark (charges_init, then the reference Poisson solve) on boxes
of every shape class: one-wide, two-wide, ragged, and a touching-spheres cell.
"""
import numpy as np
import pytest

from laboetie_gb300 import geometry as geo
from oracle import np_oracle as npo

BJL, LAMBDA_D, DPM = 0.4, 4.0, 0.05
ES = (2e-3, -1e-3, 5e-4)


def _random_nature(shape, frac, seed):
    rng = np.random.default_rng(seed)
    nat = (rng.random(shape) < frac).astype(np.int8)
    nat.flat[0] = 0
    return nat


BOXES = [
    ("cc8", lambda: geo.cc(8, 8, 8)),
    ("slit-1x1x16", lambda: geo.slit(1, 1, 16)),
    ("random-2x3x5", lambda: _random_nature((5, 3, 2), 0.3, 7)),
    ("cylinder", lambda: geo.cylinder(9, 9, 4)),
]


def charged_state(oracle, nat):
    inter = oracle.detect_interfacial(nat)
    sigma = -0.01 * max(int(((nat == 1) & (inter == 1)).sum()), 1)
    cp, cm, phi, an, _ = oracle.charges_init(nat, inter, BJL, sigma, LAMBDA_D)
    phi, an, _ = oracle.sor(nat, sigma, BJL, cp, cm, phi, an)
    return sigma, cp, cm, phi, an


def flow_state(nat, seed, amp=0.05):
    rng = np.random.default_rng(seed)
    n = npo.A0[:, None, None, None] * (1.0 + amp * rng.standard_normal((19,) + nat.shape))
    j = [amp * rng.standard_normal(nat.shape) for _ in range(3)]
    return n, j


# ------------------------------------------------------------------------------------ CPU

@pytest.mark.parametrize("name,make", BOXES)
def test_electrostatic_pot_and_comp_j_two_restatements(oracle_mod, name, make):
    nat = make()
    _, _, _, phi, _ = charged_state(oracle_mod, nat)
    for es in ((0.0, 0.0, 0.0), ES):
        assert np.array_equal(oracle_mod.electrostatic_pot(phi, es), npo.electrostatic_pot(phi, es))
    n, j = flow_state(nat, 3)
    a, b = oracle_mod.comp_j(n, j), npo.comp_j(n, j)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("time", [0, 4])
@pytest.mark.parametrize("name,make", BOXES)
def test_smolu_two_restatements(oracle_mod, name, make, time):
    nat = make()
    _, cp, cm, phi, _ = charged_state(oracle_mod, nat)
    pt = oracle_mod.electrostatic_pot(phi, ES)
    sf0 = np.zeros((3,) + nat.shape)
    args = (nat, pt, cp, cm, DPM, 0.7 * DPM, time, 3, ES, (1e-3, 0.0, -2e-3), (0.1, 0.0, 0.0),
            (0.0, 0.2, 0.0), sf0)
    rc, cp1, cm1, el1, io1, sf1 = oracle_mod.smolu(*args)
    ok, cp2, cm2, el2, io2, sf2 = npo.smolu(*args)
    assert (rc == 0) == ok
    assert np.array_equal(cp1, cp2) and np.array_equal(cm1, cm2)
    assert np.array_equal(sf1, sf2)
    assert np.array_equal(el1, el2, equal_nan=True) and np.array_equal(io1, io2, equal_nan=True)


@pytest.mark.parametrize("name,make", BOXES)
def test_advect_two_restatements_over_two_calls(oracle_mod, name, make):
    nat = make()
    _, cp, cm, _, _ = charged_state(oracle_mod, nat)
    fp1, fm1 = np.zeros(nat.shape), np.zeros(nat.shape)
    fp2, fm2 = np.zeros(nat.shape), np.zeros(nat.shape)
    el1 = io1 = el2 = io2 = (0.0, 0.0, 0.0)
    c1 = c2 = (cp, cm)
    for seed in (5, 6):   # the flux_site arrays carry over from one call to the next
        _, j = flow_state(nat, seed, amp=0.2)
        rc, a, b, el1, io1 = oracle_mod.advect(nat, j, *c1, fp1, fm1, el1, io1)
        ok, x, y, el2, io2 = npo.advect(nat, j, *c2, fp2, fm2, el2, io2)
        assert (rc == 0) == ok
        assert np.array_equal(a, x) and np.array_equal(b, y)
        assert np.array_equal(fp1, fp2) and np.array_equal(fm1, fm2)
        assert np.array_equal(el1, el2) and np.array_equal(io1, io2)
        c1, c2 = (a, b), (x, y)
    assert not np.array_equal(c1[0], cp)


# ------------------------------------------------------------------------------------ GPU

def _close(a, b, rel):
    scale = max(np.nanmax(np.abs(b)), 1e-300)
    return np.nanmax(np.abs(a - b)) <= rel * scale


@pytest.mark.gpu
@pytest.mark.parametrize("name,make", BOXES)
def test_electrostatic_pot_and_comp_j_bit_exact(oracle_mod, name, make):
    from laboetie_gb300 import Box

    nat = make()
    sigma, cp, cm, phi, an = charged_state(oracle_mod, nat)
    n, j = flow_state(nat, 3)
    with Box(nat) as box:
        box.pnp_init(bjl=BJL, sigma=sigma, lambda_D=LAMBDA_D, D_plus=DPM, D_minus=DPM)
        box.pnp_set(cp, cm, phi, an)
        for es in ((0.0, 0.0, 0.0), ES):
            box.electrostatic_pot(es)
            pt, _ = box.ek_get()
            assert np.array_equal(pt, oracle_mod.electrostatic_pot(phi, es))
        gj = box.comp_j(n, j)
    assert all(np.array_equal(x, y) for x, y in zip(gj, oracle_mod.comp_j(n, j)))


@pytest.mark.gpu
@pytest.mark.parametrize("name,make", BOXES)
def test_smolu_within_1e12(oracle_mod, name, make):
    """Two smolu calls in a row (solute_force accumulates), time 0 then time 4 (currents divided
    by n_fluidsites = 0 as in the reference)."""
    from laboetie_gb300 import Box

    nat = make()
    sigma, cp, cm, phi, an = charged_state(oracle_mod, nat)
    ls = (1e-3, 0.0, -2e-3)
    pt = oracle_mod.electrostatic_pot(phi, ES)
    sf = np.zeros((3,) + nat.shape)
    el = io = (0.1, 0.0, 0.0)
    with Box(nat) as box:
        box.pnp_init(bjl=BJL, sigma=sigma, lambda_D=LAMBDA_D, D_plus=DPM, D_minus=0.7 * DPM)
        box.pnp_set(cp, cm, phi, an)
        box.electrostatic_pot(ES)
        gel = gio = el
        ocp, ocm = cp, cm
        for time in (0, 4):
            gel, gio, grc = box.smolu(time=time, D_iter=3, elec_slope=ES, lncb_slope=ls,
                                      el_curr=gel, ion_curr=gio, check=False)
            rc, ocp, ocm, el, io, sf = oracle_mod.smolu(nat, pt, ocp, ocm, DPM, 0.7 * DPM, time, 3,
                                                        ES, ls, el, io, sf)
            gcp, gcm, _, _ = box.pnp_get()
            _, gsf = box.ek_get()
            assert (grc == 0) == (rc == 0)
            assert _close(gcp, ocp, 1e-12) and _close(gcm, ocm, 1e-12)
            assert _close(gsf, sf, 1e-12)
            if time == 0:
                assert _close(gel, el, 1e-12) and _close(gio, io, 1e-12)
            else:   # divided by zero: the same infinities (or NaN where a current is 0)
                assert np.array_equal(np.isnan(gel), np.isnan(el))
                fin = ~np.isnan(el)
                assert np.array_equal(gel[fin], el[fin]) and np.array_equal(gio[fin], io[fin])


@pytest.mark.gpu
@pytest.mark.parametrize("name,make", BOXES)
def test_advect_bit_exact_over_two_calls(oracle_mod, name, make):
    from laboetie_gb300 import Box

    nat = make()
    sigma, cp, cm, phi, an = charged_state(oracle_mod, nat)
    fp, fm = np.zeros(nat.shape), np.zeros(nat.shape)
    el = io = (0.0, 0.0, 0.0)
    with Box(nat) as box:
        box.pnp_init(bjl=BJL, sigma=sigma, lambda_D=LAMBDA_D, D_plus=DPM, D_minus=DPM)
        box.pnp_set(cp, cm, phi, an)
        gel = gio = el
        for seed in (5, 6):
            _, j = flow_state(nat, seed, amp=0.2)
            gel, gio, grc = box.advect(j, gel, gio, check=False)
            rc, cp, cm, el, io = oracle_mod.advect(nat, j, cp, cm, fp, fm, el, io)
            gcp, gcm, _, _ = box.pnp_get()
            assert (grc == 0) == (rc == 0)
            assert np.array_equal(gcp, cp) and np.array_equal(gcm, cm)
            assert np.array_equal(gel, el) and np.array_equal(gio, io)
