"""Checks at the benchmark's full size: the 192^3 porous medium (spheres r = 8, porosity 0.60,
seed 20261203; 4,245,990 fluid of 7,077,888 nodes), tau 0.8, f_ext (1e-6, 0, 0).

* FP64 strict flow: two steps bit-identical to the oracle (which takes a few seconds per step on
  the host cores at this size).
* FP64 strict tracer: initialisation and two propagation steps from a seeded flow field, P
  bit-identical to the oracle, VACF within 1e-12 of |VACF(0)|.
* FP32 in place (fluid-only AA) against FP32 two-buffer (lattice A/B): bit-identical after an odd
  number of steps (the in-place state is then in its swapped form).
* FP32 mass conservation over 2000 steps: total mass within 1e-9 relative (the collision and the
  streaming conserve it exactly in exact arithmetic; the deviations keep the rounding small).

And beyond 2^32 population slots: a cylinder (geometryLabel 2) in an 800 x 800 x 480 box,
241 M fluid of 307 M nodes, 19 Nf = 4.6e9, where the in-place layout forms 64-bit slot offsets:
its per-plane flux and density profiles along x, y and z equal the two-buffer layout's after an
odd and an even number of steps (about 32 GB and 58 GB of device memory, one after the other).
"""
import numpy as np
import pytest

from laboetie_gb300 import FP32_DEV, Box
from laboetie_gb300 import geometry as geo

from test_flow_gpu import oracle_fixed_steps

pytestmark = pytest.mark.gpu

TAU = 0.8
FE = (1e-6, 0.0, 0.0)


@pytest.fixture(scope="module")
def medium():
    return geo.porous_spheres(192, 8.0, 0.60, 20261203)


def test_fp64_steps_bit_identical_to_oracle_at_full_size(oracle_mod, medium):
    K = 2
    with Box(medium, relaxation_time=TAU, f_ext=FE) as box:
        box.flow_init()
        box.flow_steps(K, force_on=True)
        n, rho, j = box.flow_get()
    n_o, rho_o, j_o = oracle_fixed_steps(oracle_mod, medium, TAU, FE, K)
    assert np.array_equal(rho, rho_o)
    for d in range(3):
        assert np.array_equal(j[d], j_o[d])
    assert np.array_equal(n, n_o)


def test_fp64_tracer_bit_identical_to_oracle_at_full_size(oracle_mod, medium):
    rng = np.random.default_rng(192)
    fluid = medium == 0
    rho = np.where(fluid, 1.0 + 1e-3 * rng.standard_normal(medium.shape), 0.0)
    j = [np.where(fluid, 1e-4 * rng.standard_normal(medium.shape), 0.0) for _ in range(3)]
    tr = dict(Db=0.01, ka=0.01 * np.exp(2.0), kd=0.01)
    inter = oracle_mod.detect_interfacial(medium)
    nmp = oracle_mod.update_tracer_population(medium, rho, j, FE, 0.0, tr["Db"])
    mp = oracle_mod.MomentPropagation(medium, inter, rho, nmp, ka=tr["ka"], kd=tr["kd"], Db=tr["Db"])
    v0 = mp.vacf0.copy()
    vac = [mp.propagate(it)[0] for it in (1, 2)]
    P = mp.P().reshape(medium.shape + (3,))
    A = mp.Pads().reshape(medium.shape + (3,))
    mp.close()
    with Box(medium, relaxation_time=TAU, f_ext=FE) as box:
        g0 = box.mp_init(moments=(rho, j), f_ext=FE, **tr)
        gv, _ = box.mp_propagate(2)
        GP, GA = box.mp_get()
    scale = np.abs(v0).max()
    assert np.max(np.abs(g0 - v0)) <= 1e-12 * scale
    assert np.max(np.abs(gv - np.array(vac))) <= 1e-12 * scale
    assert np.array_equal(GP, P) and np.array_equal(GA, A)


def test_fp32_in_place_equals_two_buffer_at_full_size(monkeypatch, medium):
    out = {}
    for mode in ("ab", "aa"):
        monkeypatch.setenv("LBGPU_FP32_STREAMING", mode)
        with Box(medium, relaxation_time=TAU, f_ext=FE, precision=FP32_DEV) as box:
            box.flow_init()
            box.flow_steps(21, force_on=True)
            out[mode] = box.flow_get()
    (na, ra, ja), (nb, rb, jb) = out["ab"], out["aa"]
    assert np.array_equal(ra, rb) and np.array_equal(na, nb)
    for d in range(3):
        assert np.array_equal(ja[d], jb[d])


def test_fp32_mass_conservation_at_full_size(medium):
    nf = int((medium == 0).sum())
    with Box(medium, relaxation_time=TAU, f_ext=FE, precision=FP32_DEV) as box:
        box.flow_init()
        box.flow_steps(2000, force_on=True)
        _, rho, j = box.flow_get(populations=False)
    assert abs(rho.sum() - nf) <= 1e-9 * nf
    assert j[0].sum() > 0.0 and np.all(rho[medium == 1] == 0.0)


def test_fp32_in_place_beyond_2_32_slots_equals_two_buffer(monkeypatch):
    shape = (800, 800, 480)
    out = {}
    for mode in ("ab", "aa"):
        monkeypatch.setenv("LBGPU_FP32_STREAMING", mode)
        res = []
        with Box.from_label(2, *shape, relaxation_time=TAU, f_ext=(0.0, 0.0, 1e-6),
                            precision=FP32_DEV) as box:
            nf = box.node_counts()["fluid"]
            box.flow_init()
            for k in (7, 5):   # 7 steps: swapped state; 12: natural order
                box.flow_steps(k, force_on=True)
                res.append([box.profiles(axis) for axis in range(3)])
        out[mode] = (nf, res)
    assert out["aa"][0] == out["ab"][0] and 19 * out["aa"][0] >= 2**32
    for pa, pb in zip(out["ab"][1], out["aa"][1]):
        for (fa, da), (fb, db) in zip(pa, pb):
            assert np.array_equal(fa, fb) and np.array_equal(da, db)
    flux_z = out["aa"][1][-1][2][0][:, 2]
    assert np.all(flux_z > 0.0)
