"""Parity of the GPU tracer moment propagation (C ABI) with the CPU oracle.

FP64: the propagated quantity P (and its adsorbed part) is bit-identical to the oracle at every
node, since each node's sum runs in the reference's l order with separate roundings.  VACF is a
sum over all nodes that the GPU forms in a different (fixed) order, so it is compared relative
to |VACF(0)| with tolerance 1e-12.  FP32 is compared with the tolerances stated in each test.
"""
import math

import numpy as np
import pytest

from laboetie_gb300 import FP32_DEV, FP64, Box, LbgpuError
from laboetie_gb300 import geometry as geo

pytestmark = pytest.mark.gpu


def converged_flow(oracle, nat, tau, f_ext, target=1e-10, max_steps=200000):
    r = oracle.equilibration(nat, tau=tau, target_error=target, f_ext=f_ext, max_steps=max_steps)
    return r["rho"], r["j"]


def oracle_mp(oracle, nat, rho, j, f_ext, steps, **tr):
    inter = oracle.detect_interfacial(nat)
    nmp = oracle.update_tracer_population(nat, rho, j, f_ext, 0.0, tr["Db"])
    mp = oracle.MomentPropagation(nat, inter, rho, nmp, ka=tr.get("ka", 0.0), kd=tr.get("kd", 0.0),
                                  Db=tr["Db"])
    v0 = mp.vacf0.copy()
    P1 = mp.P().reshape(nat.shape + (3,))
    vac = []
    conv = False
    for it in range(1, steps + 1):
        v, conv = mp.propagate(it)
        vac.append(v)
        if conv:
            break
    P = mp.P().reshape(nat.shape + (3,))
    A = mp.Pads()
    A = A.reshape(nat.shape + (3,)) if A is not None else np.zeros(nat.shape + (3,))
    mp.close()
    return v0, P1, np.array(vac), conv, P, A


@pytest.mark.parametrize("adsorb", [False, True])
def test_mp_c1_fp64(oracle_mod, adsorb):
    """The small slit case: slit 4x4x34, tau 1, f_ext (1e-5,0,0), Db 0.01, K = e with kd 0.01."""
    nat = geo.slit(4, 4, 34)
    f_ext = (1e-5, 0.0, 0.0)
    rho, j = converged_flow(oracle_mod, nat, 1.0, f_ext)
    tr = dict(Db=0.01, ka=0.01 * math.e, kd=0.01) if adsorb else dict(Db=0.01)
    steps = 600
    v0, P1, vac, conv, P, A = oracle_mp(oracle_mod, nat, rho, j, f_ext, steps, **tr)
    with Box(nat, relaxation_time=1.0, f_ext=f_ext) as box:
        g0 = box.mp_init(moments=(rho, j), f_ext=f_ext, **tr)
        G1, _ = box.mp_get()
        gv, gconv = box.mp_propagate(steps)
        GP, GA = box.mp_get()
    scale = np.abs(v0).max()
    assert np.max(np.abs(g0 - v0)) <= 1e-12 * scale
    assert np.array_equal(G1, P1)
    assert len(gv) == len(vac) and gconv == conv
    assert np.max(np.abs(gv - vac)) <= 1e-12 * scale
    assert np.array_equal(GP, P)
    assert np.array_equal(GA, A)


@pytest.mark.parametrize("adsorb", [False, True])
@pytest.mark.parametrize("shape,frac,seed", [((7, 5, 6), 0.3, 31), ((9, 8, 3), 0.2, 32), ((2, 3, 5), 0.25, 33)])
def test_mp_fp64_on_ragged_random_boxes(oracle_mod, shape, frac, seed, adsorb):
    """FP64 tracer on ragged random boxes (thin and odd axes, bounce-back links in every
    direction) from synthetic moments: P and P_ads bit-identical to the oracle after 120 steps,
    VACF within 1e-12 of |VACF(0)|."""
    rng = np.random.default_rng(seed)
    nat = (rng.random(shape) < frac).astype(np.int8)
    nat.flat[0] = 0
    fl = nat == 0
    rho = np.where(fl, 1.0 + 0.01 * rng.standard_normal(nat.shape), 0.0)
    j = [np.where(fl, 2e-4 * rng.standard_normal(nat.shape), 0.0) for _ in range(3)]
    f_ext = (1e-5, -2e-6, 3e-6)
    tr = dict(Db=0.01, ka=0.01 * math.e, kd=0.01) if adsorb else dict(Db=0.01)
    steps = 120
    v0, P1, vac, conv, P, A = oracle_mp(oracle_mod, nat, rho, j, f_ext, steps, **tr)
    with Box(nat, relaxation_time=1.0, f_ext=f_ext) as box:
        g0 = box.mp_init(moments=(rho, j), f_ext=f_ext, **tr)
        gv, gconv = box.mp_propagate(steps)
        GP, GA = box.mp_get()
    scale = np.abs(v0).max()
    assert np.max(np.abs(g0 - v0)) <= 1e-12 * scale
    assert len(gv) == len(vac) and gconv == conv
    assert np.max(np.abs(gv - vac)) <= 1e-12 * scale
    assert np.array_equal(GP, P) and np.abs(P).max() > 0
    assert np.array_equal(GA, A)


def test_mp_from_device_flow_state(oracle_mod):
    """drop_tracers after equilibration with no host round trip: moments taken on the device."""
    nat = geo.cc(12, 12, 12)
    f_ext = (2e-5, 0.0, 0.0)
    ref = oracle_mod.equilibration(nat, tau=0.8, target_error=1e-9, f_ext=f_ext, max_steps=50000)
    v0, P1, vac, conv, P, A = oracle_mp(oracle_mod, nat, ref["rho"], ref["j"], f_ext, 100,
                                        Db=0.02, ka=0.02, kd=0.01)
    with Box(nat, relaxation_time=0.8, f_ext=f_ext, target_error=1e-9) as box:
        box.flow_init()
        box.equilibration(max_steps=50000)
        g0 = box.mp_init(f_ext=f_ext, Db=0.02, ka=0.02, kd=0.01)
        gv, _ = box.mp_propagate(100)
        GP, GA = box.mp_get()
    scale = np.abs(v0).max()
    assert np.max(np.abs(g0 - v0)) <= 1e-12 * scale
    assert np.max(np.abs(gv - vac)) <= 1e-12 * scale
    assert np.array_equal(GP, P) and np.array_equal(GA, A)


def test_mp_bulk_known_answer(oracle_mod):
    """Bulk fluid at rest: VACF(0) = 2 Db per component (kBT = 1/3, lambda = 12 Db), VACF(t>=1) = 0,
    converged at it = 3, hence D_eff = VACF(0)/2 = Db."""
    nat = geo.bulk(5, 4, 6)
    rho = np.ones(nat.shape)
    j = [np.zeros(nat.shape) for _ in range(3)]
    Db = 0.03
    with Box(nat) as box:
        v0 = box.mp_init(moments=(rho, j), Db=Db)
        vac, conv = box.mp_propagate(50)
    assert np.allclose(v0, 2 * Db, rtol=1e-14, atol=0)
    assert conv and len(vac) == 3
    assert np.all(np.abs(vac) < 1e-18)


def test_mp_refusals():
    nat = geo.slit(2, 2, 6)
    rho = np.where(nat == 0, 1.0, 0.0)
    j = [np.zeros(nat.shape) for _ in range(3)]
    with Box(nat) as box:
        with pytest.raises(LbgpuError):
            box.mp_init(moments=(rho, j), Db=0.0)          # drop_tracers.f90:89
        with pytest.raises(LbgpuError):
            box.mp_init(moments=(rho, j), Db=0.01, Ds=0.1)  # module_moment_propagation.f90:60-66
        with pytest.raises(LbgpuError):
            box.mp_init(moments=(rho, j), Db=0.01, z=1.0)   # module_moment_propagation.f90:71-79
        # a remaining fraction below epsilon stops the first propagate (:249,257)
        box.mp_init(moments=(rho, j), Db=0.2, ka=0.9, kd=0.1)
        with pytest.raises(LbgpuError) as e:
            box.mp_propagate(1)
        assert e.value.status & (1 << 4)


def test_mp_fp32_tracks_fp64(oracle_mod):
    """FP32 propagation (on-the-fly scattering, FP64 VACF sums) vs FP64 on the C1 slit with
    adsorption: VACF within 1e-5 of |VACF(0)| and the Green-Kubo D_eff within 1e-5 relative."""
    nat = geo.slit(4, 4, 34)
    f_ext = (1e-5, 0.0, 0.0)
    rho, j = converged_flow(oracle_mod, nat, 1.0, f_ext)
    tr = dict(Db=0.01, ka=0.01 * math.e, kd=0.01, f_ext=f_ext)
    out = {}
    for prec in (FP64, FP32_DEV):
        with Box(nat, relaxation_time=1.0, f_ext=f_ext, precision=prec) as box:
            v0 = box.mp_init(moments=(rho, j), **tr)
            vac, _ = box.mp_propagate(2000)
        out[prec] = (v0, vac)
    v64, v32 = out[FP64], out[FP32_DEV]
    scale = np.abs(v64[0]).max()
    assert np.max(np.abs(v32[0] - v64[0])) <= 1e-6 * scale
    assert np.max(np.abs(v32[1] - v64[1])) <= 1e-5 * scale
    d64 = v64[0] / 2 + v64[1].sum(axis=0)
    d32 = v32[0] / 2 + v32[1].sum(axis=0)
    assert abs(d32[0] - d64[0]) <= 1e-5 * abs(d64[0])


def test_mp_fp32_slab_and_grid_stride_steps_agree(monkeypatch):
    """The shared-memory slab step (boxes with lx >= 32, ly >= 8) and the grid-stride step do
    the same per-node arithmetic: P and P_ads are bit-identical after any number of steps.  The
    VACF terms are summed per thread in FP32 before the FP64 sums, over the nodes of a column's
    z-chunk (slab) or a grid-stride walk, so the per-step VACF differs by that grouping: 1e-9 of
    |VACF(0)| (observed ~1e-12)."""
    nat = geo.porous_spheres(L=40, radius=5.0, porosity=0.6, seed=3)
    rng = np.random.default_rng(5)
    rho = np.where(nat == 0, 1.0 + 1e-3 * rng.standard_normal(nat.shape), 0.0)
    j = [np.where(nat == 0, 1e-3 * rng.standard_normal(nat.shape), 0.0) for _ in range(3)]
    out = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("LBGPU_MP_SLAB", mode)
        with Box(nat, precision=FP32_DEV) as box:
            v0 = box.mp_init(moments=(rho, j), Db=0.01, ka=0.02, kd=0.01)
            vac, _ = box.mp_propagate(37)
            P, A = box.mp_get()
        out[mode] = (v0, vac, P, A)
    a, b = out["1"], out["0"]
    assert np.array_equal(a[2], b[2]) and np.array_equal(a[3], b[3])
    assert len(a[1]) == len(b[1]) == 37
    assert np.max(np.abs(a[1] - b[1])) <= 1e-9 * np.abs(a[0]).max()


@pytest.mark.parametrize("shape", [(20, 13, 40), (11, 21, 70)])
def test_mp_fp32_slab_partial_tiles_in_x_and_y(monkeypatch, shape):
    """Boxes whose sides are not multiples of the slab tile (32 x 8): the last tile of a row and
    of a column holds lanes outside the box, and its halo wraps across the periodic boundary.  With
    adsorption (the adsorbed part staged per thread): P and P_ads bit-identical to the grid-stride
    step."""
    rng = np.random.default_rng(17)
    nat = (rng.random(shape) < 0.3).astype(np.int8)
    rho = np.where(nat == 0, 1.0 + 1e-3 * rng.standard_normal(nat.shape), 0.0)
    j = [np.where(nat == 0, 1e-3 * rng.standard_normal(nat.shape), 0.0) for _ in range(3)]
    out = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("LBGPU_MP_SLAB", mode)
        with Box(nat, precision=FP32_DEV) as box:
            box.mp_init(moments=(rho, j), Db=0.01, ka=0.02, kd=0.01)
            box.mp_propagate(29)
            out[mode] = box.mp_get()
    assert np.array_equal(out["1"][0], out["0"][0]) and np.array_equal(out["1"][1], out["0"][1])
    assert np.abs(out["1"][1]).max() > 0


def test_fp32_slab_bulk_tensor_copies_equal_per_thread_copies(monkeypatch):
    """The slab step stages interior tiles by bulk tensor copies (TMA) and edge tiles (periodic
    wrap) by per-thread copies; with LBGPU_MP_TMA=0 every tile uses per-thread copies and with
    LBGPU_MP_SLAB=0 the grid-stride kernel runs: P and P_ads bit-identical in all three.  100 x 40
    x 43 has interior tiles in x (x0 = 32) and y (y0 = 8 .. 24) beside edge tiles, and z chunks of
    9, 9, 9, 9 and 7 planes (the first and the last reading across the periodic z boundary)."""
    rng = np.random.default_rng(11)
    nat = (rng.random((43, 40, 100)) < 0.3).astype(np.int8)
    rho = np.where(nat == 0, 1.0 + 1e-3 * rng.standard_normal(nat.shape), 0.0)
    j = [np.where(nat == 0, 1e-3 * rng.standard_normal(nat.shape), 0.0) for _ in range(3)]
    out = {}
    for name, env in (("tma", {}), ("copies", {"LBGPU_MP_TMA": "0"}), ("grid", {"LBGPU_MP_SLAB": "0"})):
        for k in ("LBGPU_MP_TMA", "LBGPU_MP_SLAB"):
            monkeypatch.delenv(k, raising=False)
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        with Box(nat, precision=FP32_DEV) as box:
            box.mp_init(moments=(rho, j), Db=0.01, ka=0.02, kd=0.01)
            box.mp_propagate(23)
            out[name] = box.mp_get()
    for name in ("copies", "grid"):
        assert np.array_equal(out["tma"][0], out[name][0]) and np.array_equal(out["tma"][1], out[name][1])
