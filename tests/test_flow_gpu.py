"""Parity of the GPU flow path (C ABI) with the CPU oracle.

FP64 results must be bit-identical (numpy array_equal; +0 and -0 compare equal): the kernels
evaluate every operation of the Fortran source in the same order with separate roundings.
The FP32-deviation path is checked against FP64 with the tolerance stated in each test.
"""
import numpy as np
import pytest

from laboetie_gb300 import FP32_DEV, FP64, FP64_FUSED, Box, LbgpuError
from laboetie_gb300 import geometry as geo

pytestmark = pytest.mark.gpu


def random_nature(shape, solid_frac, seed):
    rng = np.random.default_rng(seed)
    nat = (rng.random(shape) < solid_frac).astype(np.int8)
    nat.flat[0] = 0
    return nat


def random_state(nature, seed, amp=0.02):
    """A positive population field with its own density and a random flux."""
    import oracle

    rng = np.random.default_rng(seed)

    c, inv, a0, a1, a2, de = oracle.tables()
    n = a0[:, None, None, None] * (1.0 + amp * rng.standard_normal((19,) + nature.shape))
    n[:, nature == 1] = rng.random((19, int((nature == 1).sum()))) * 0.05
    rho = n.sum(axis=0)
    j = [(n * c[:, d][:, None, None, None]).sum(axis=0) + amp * rng.standard_normal(nature.shape)
         for d in range(3)]
    return n, rho, j


GEOMS = [
    ("slit", lambda: geo.slit(4, 4, 12)),
    ("cylinder", lambda: geo.cylinder(9, 9, 5)),
    ("cc", lambda: geo.cc(8, 8, 8)),
    ("cavity", lambda: geo.spherical_cavity(7, 7, 7)),
    ("tube", lambda: geo.tube_varying_diameter(10, 9, 9)),
    ("random", lambda: random_nature((6, 5, 7), 0.3, 1)),
    ("thin-x", lambda: random_nature((9, 8, 1), 0.25, 2)),
    ("thin-2", lambda: random_nature((2, 3, 2), 0.3, 3)),
]


@pytest.mark.parametrize("name,make", GEOMS)
def test_interfacial_and_counts_bit_exact(oracle_mod, name, make):
    nat = make()
    with Box(nat) as box:
        got = box.interfacial()
        want = oracle_mod.detect_interfacial(nat)
        assert np.array_equal(got, want)
        cnt = box.node_counts()
        assert cnt["fluid"] == int((nat == 0).sum())
        assert cnt["solid"] == int((nat == 1).sum())
        assert cnt["fluid_interfacial"] == int(((nat == 0) & (want == 1)).sum())
        assert cnt["solid_interfacial"] == int(((nat == 1) & (want == 1)).sum())


@pytest.mark.parametrize("fkind", ["field", "x-only", "zero"])
@pytest.mark.parametrize("tau", [1.0, 0.8, 1.7])
def test_collide_operator_bit_exact(oracle_mod, fkind, tau):
    nat = random_nature((6, 7, 5), 0.3, 11)
    n, rho, j = random_state(nat, 5)
    rng = np.random.default_rng(7)
    if fkind == "field":
        f = [1e-3 * rng.standard_normal(nat.shape) * (nat == 0) for _ in range(3)]
    elif fkind == "x-only":
        f = [np.where(nat == 0, 1e-5, 0.0), np.zeros(nat.shape), np.zeros(nat.shape)]
    else:
        f = [np.zeros(nat.shape) for _ in range(3)]
    with Box(nat, relaxation_time=tau) as box:
        got = box.collide(n, rho, j, f)
    want = oracle_mod.collide(nat, tau, n, rho, j, f)
    assert np.array_equal(got, want)


def test_bounce_back_stream_operator_bit_exact(oracle_mod):
    for seed, shape in ((1, (5, 6, 7)), (2, (3, 4, 1)), (3, (1, 1, 8)), (4, (2, 2, 2))):
        nat = random_nature(shape, 0.35, seed)
        n, _, _ = random_state(nat, seed)
        with Box(nat) as box:
            got = box.bounce_back_stream(n)
        want = oracle_mod.bounce_back_stream(nat, n)
        assert np.array_equal(got, want), shape


def test_moments_operator_bit_exact(oracle_mod):
    nat = random_nature((6, 5, 4), 0.3, 21)
    n, _, jold = random_state(nat, 22)
    rng = np.random.default_rng(23)
    f = [1e-4 * rng.standard_normal(nat.shape) for _ in range(3)]
    with Box(nat) as box:
        st, rho, j, err = box.moments(n, f, jold)
    st_o, rho_o, j_o, err_o = oracle_mod.moments(nat, n, f, jold)
    assert st == 0 and st_o == 0
    assert np.array_equal(rho, rho_o)
    for d in range(3):
        assert np.array_equal(j[d], j_o[d])
    assert err == err_o
    # a negative population is reported (equilibration.f90:248)
    n2 = n.copy()
    n2[3, 1, 2, 1] = -1e-9
    with Box(nat) as box:
        st, *_ = box.moments(n2, f, jold)
    assert st & 4


def oracle_fixed_steps(oracle, nat, tau, f_ext, K, svden=1.0):
    """Reference loop of equilibration.f90 with the force switched on after step 1."""
    n, rho = oracle.init_populations(nat, svden)
    j = [np.zeros(nat.shape) for _ in range(3)]
    zero = [np.zeros(nat.shape) for _ in range(3)]
    fon = [np.where(nat == 0, f_ext[d], 0.0) for d in range(3)]
    for t in range(1, K + 1):
        f = zero if t == 1 else fon
        n = oracle.collide(nat, tau, n, rho, j, f)
        n = oracle.bounce_back_stream(nat, n)
        st, rho, j, _ = oracle.moments(nat, n, f, j)
        assert st == 0
    return n, rho, j


@pytest.mark.parametrize("f_ext", [(1e-5, 0.0, 0.0), (0.0, 2e-5, 0.0), (1e-5, -3e-6, 2e-6)])
def test_fused_fixed_steps_bit_exact(oracle_mod, f_ext):
    nat = geo.porous_spheres(L=10, radius=2.0, porosity=0.7, seed=5)
    K = 25
    with Box(nat, relaxation_time=0.8, f_ext=f_ext) as box:
        box.flow_init()
        box.flow_steps(K, force_on=True)
        n, rho, j = box.flow_get()
    n_o, rho_o, j_o = oracle_fixed_steps(oracle_mod, nat, 0.8, f_ext, K)
    assert np.array_equal(n, n_o)
    assert np.array_equal(rho, rho_o)
    for d in range(3):
        assert np.array_equal(j[d], j_o[d])


def test_equilibration_c1_bit_exact(oracle_mod):
    """Flow phase of the small slit case: slit 4x4x34, tau 1, f_ext (1e-5,0,0), target 1e-10."""
    nat = geo.slit(4, 4, 34)
    ref = oracle_mod.equilibration(nat, tau=1.0, target_error=1e-10, f_ext=(1e-5, 0, 0),
                                   max_steps=100000)
    with Box(nat, relaxation_time=1.0, f_ext=(1e-5, 0, 0), target_error=1e-10) as box:
        box.flow_init()
        steps, hist = box.equilibration(max_steps=100000, hist_cap=100000)
        n, rho, j = box.flow_get()
    assert steps == ref["steps"]
    assert np.array_equal(hist, ref["l2err"])
    assert np.array_equal(n, ref["n"])
    assert np.array_equal(rho, ref["rho"])
    for d in range(3):
        assert np.array_equal(j[d], ref["j"][d])


def test_equilibration_cc_bit_exact(oracle_mod):
    """Touching spheres (geometryLabel 3) 12^3, tau 0.8, oblique force, target 1e-9."""
    nat = geo.cc(12, 12, 12)
    kw = dict(tau=0.8, target_error=1e-9, f_ext=(2e-5, 1e-5, 0.0))
    ref = oracle_mod.equilibration(nat, max_steps=50000, **kw)
    with Box(nat, relaxation_time=0.8, f_ext=kw["f_ext"], target_error=1e-9) as box:
        box.flow_init()
        steps, hist = box.equilibration(max_steps=50000, hist_cap=50000)
        n, rho, j = box.flow_get()
    assert steps == ref["steps"]
    assert np.array_equal(hist, ref["l2err"])
    assert np.array_equal(n, ref["n"])
    for d in range(3):
        assert np.array_equal(j[d], ref["j"][d])


def test_equilibration_step_cap_state_bit_exact(oracle_mod):
    """A random porous medium with isolated fluid pockets never meets the target (the reference
    would loop for ever); at a step cap both stop at the same step in the same state."""
    nat = geo.porous_spheres(L=12, radius=2.5, porosity=0.65, seed=9)
    kw = dict(tau=0.8, target_error=1e-9, f_ext=(2e-5, 1e-5, 0.0))
    ref = oracle_mod.equilibration(nat, max_steps=1500, check=False, **kw)
    assert ref["status"] == 2 and ref["steps"] == 1500
    with Box(nat, relaxation_time=0.8, f_ext=kw["f_ext"], target_error=1e-9) as box:
        box.flow_init()
        steps, hist, rc = box.equilibration(max_steps=1500, hist_cap=1500, check=False)
        n, rho, j = box.flow_get()
    assert rc & (1 << 5) and steps == 1500
    assert np.array_equal(hist, ref["l2err"])
    assert np.array_equal(n, ref["n"])
    assert np.array_equal(rho, ref["rho"])
    for d in range(3):
        assert np.array_equal(j[d], ref["j"][d])


def test_equilibration_without_force_exits_at_step_4(oracle_mod):
    nat = geo.slit(1, 1, 12)
    ref = oracle_mod.equilibration(nat, max_steps=100)
    with Box(nat) as box:
        box.flow_init()
        steps, _ = box.equilibration(max_steps=100)
    assert steps == ref["steps"] == 4


def test_equilibration_step_cap_and_negative_population():
    nat = geo.slit(4, 4, 20)
    with Box(nat, relaxation_time=1.0, f_ext=(1e-5, 0, 0)) as box:
        box.flow_init()
        with pytest.raises(LbgpuError) as e:
            box.equilibration(max_steps=50)
        assert e.value.status & (1 << 5)
    with Box(nat, relaxation_time=3.0, f_ext=(0.5, 0, 0), target_error=1e-300) as box:
        box.flow_init()
        with pytest.raises(LbgpuError) as e:
            box.equilibration(max_steps=5000)
        assert e.value.status & 4


def test_fp32_deviation_tracks_fp64_on_the_slit():
    """FP32-deviation storage vs FP64 on the C1 slit after 4000 forced steps:
    the velocity profile agrees to 1e-4 relative to its maximum."""
    nat = geo.slit(4, 4, 34)
    out = {}
    for prec in (FP64, FP32_DEV):
        with Box(nat, relaxation_time=1.0, f_ext=(1e-5, 0, 0), precision=prec) as box:
            box.flow_init()
            box.flow_steps(4000, force_on=True)
            _, rho, j = box.flow_get(populations=False)
        out[prec] = (rho, j)
    jx64, jx32 = out[FP64][1][0], out[FP32_DEV][1][0]
    rel = np.max(np.abs(jx32 - jx64)) / np.max(np.abs(jx64))
    assert rel < 1e-4, rel
    assert np.max(np.abs(out[FP32_DEV][0] - out[FP64][0])) < 1e-5


def test_fp32_in_place_and_two_buffer_streaming_agree(monkeypatch):
    """The in-place (AA) and the two-buffer FP32 layouts do the same arithmetic per node, so
    their results are bit-identical after any number of steps, odd or even."""
    nat = geo.porous_spheres(L=16, radius=3.0, porosity=0.65, seed=11)
    out = {}
    for mode in ("ab", "aa"):
        monkeypatch.setenv("LBGPU_FP32_STREAMING", mode)
        with Box(nat, relaxation_time=0.8, f_ext=(1e-5, 2e-6, 0.0), precision=FP32_DEV) as box:
            box.flow_init()
            res = []
            for k in (1, 6, 13):
                box.flow_steps(k, force_on=True)
                res.append(box.flow_get())
        out[mode] = res
    for (na, ra, ja), (nb, rb, jb) in zip(out["ab"], out["aa"]):
        assert np.array_equal(na, nb) and np.array_equal(ra, rb)
        for d in range(3):
            assert np.array_equal(ja[d], jb[d])


@pytest.mark.parametrize("prec", [FP32_DEV, FP64, FP64_FUSED])
def test_flow_set_from_registered_host_memory(prec):
    """lbgpu_flow_set reads host arrays page-locked by lbgpu_host_register in place (an FP32
    context converts the populations straight from host memory, an FP64 one copies them with a
    kernel reading through the mapping); the state is bit-identical to the one staged from
    pageable memory, after the upload and after steps."""
    from laboetie_gb300 import library

    L = library()
    nat = geo.porous_spheres(L=24, radius=3.0, porosity=0.6, seed=5)
    with Box(nat, relaxation_time=0.8, f_ext=(1e-5, 0.0, 0.0)) as b64:
        b64.flow_init()
        b64.flow_steps(30, force_on=True)
        n0, rho0, j0 = b64.flow_get()
    out = {}
    for pinned in (False, True):
        host = [n0.copy(), rho0.copy()] + [x.copy() for x in j0]
        if pinned:
            for h in host:
                assert L.lbgpu_host_register(h.ctypes.data, h.nbytes) == 0
        try:
            with Box(nat, relaxation_time=0.8, f_ext=(1e-5, 0.0, 0.0), precision=prec) as box:
                box.flow_init()
                box.flow_set(host[0], host[1], tuple(host[2:]))
                first = box.flow_get()
                box.flow_steps(7, force_on=True)
                out[pinned] = (first, box.flow_get())
        finally:
            if pinned:
                for h in host:
                    L.lbgpu_host_unregister(h.ctypes.data)
    for (na, ra, ja), (nb, rb, jb) in zip(out[False], out[True]):
        assert np.array_equal(na, nb) and np.array_equal(ra, rb)
        assert all(np.array_equal(ja[d], jb[d]) for d in range(3))


def test_fp32_wide_gather_offsets_bit_identical(monkeypatch):
    """64-bit slot offsets of the in-place layout (taken once 19 Nf reaches 2^32; LBGPU_AA_WIDE=1
    forces them on any box) give the same bits as 32-bit ones: fixed steps, read back after odd
    and even counts (swapped state), and the reference loop with its checks."""
    nat = geo.porous_spheres(L=16, radius=3.0, porosity=0.65, seed=11)
    out = {}
    for wide in ("0", "1"):
        monkeypatch.setenv("LBGPU_AA_WIDE", wide)
        res = []
        with Box(nat, relaxation_time=0.8, f_ext=(1e-5, 2e-6, 0.0), precision=FP32_DEV) as box:
            box.flow_init()
            for k in (1, 6, 13):
                box.flow_steps(k, force_on=True)
                res.append(box.flow_get())
        # the loop's checks on every step, stopped by the step cap (status kept, state readable)
        with Box(nat, relaxation_time=0.8, f_ext=(1e-5, 0.0, 0.0), target_error=1e-12,
                 precision=FP32_DEV) as box:
            box.flow_init()
            steps, hist, rc = box.equilibration(max_steps=3001, hist_cap=3001, check=False)
            res.append((steps, hist, rc, box.flow_get(populations=False)))
        out[wide] = res
    for (na, ra, ja), (nb, rb, jb) in zip(out["0"][:3], out["1"][:3]):
        assert np.array_equal(na, nb) and np.array_equal(ra, rb)
        for d in range(3):
            assert np.array_equal(ja[d], jb[d])
    (sa, ha, ca, (_, ra, ja)), (sb, hb, cb, (_, rb, jb)) = out["0"][3], out["1"][3]
    assert sa == sb == 3001 and ca == cb != 0 and np.array_equal(ha, hb)
    assert np.array_equal(ra, rb) and all(np.array_equal(ja[d], jb[d]) for d in range(3))


@pytest.mark.parametrize("label,make", [(-1, lambda: geo.bulk(9, 9, 9)),
                                        (1, lambda: geo.slit(9, 7, 11))])
def test_equilibration_compensated_force_bit_exact(oracle_mod, label, make):
    """compensate_f_ext (equilibration.f90:388-487): a force on a particle of diameter 3 at the
    box centre, compensated by a background force in the solid-free box."""
    nat = make()
    fe = (1e-4, 2e-5, 0.0)
    ref = oracle_mod.equilibration(nat, tau=1.0, target_error=1e-10, f_ext=fe, max_steps=20000,
                                   compensate_f_ext=True, particle_diameter=3,
                                   geometry_label=label)
    with Box(nat, relaxation_time=1.0, f_ext=fe, target_error=1e-10) as box:
        f = box.compensated_force_field(particle_diameter=3, geometry_label=label)
        for d in range(3):
            assert np.array_equal(f[d], ref["f"][d])
        box.set_force_field(f)
        box.flow_init()
        steps, hist = box.equilibration(max_steps=20000, hist_cap=20000)
        n, rho, j = box.flow_get()
    assert steps == ref["steps"]
    assert np.array_equal(hist, ref["l2err"])
    assert np.array_equal(n, ref["n"])
    for d in range(3):
        assert np.array_equal(j[d], ref["j"][d])


@pytest.mark.parametrize("prec", [FP64, FP32_DEV])
def test_device_profiles_equal_the_reference_profiles(oracle_mod, prec):
    """lbgpu_profiles reduces the reference's profile output (equilibration.f90:154-176) on the
    device in the Fortran SUM order: bit-identical to the oracle's restatement applied to the
    same flow state, along every axis."""
    nat = geo.porous_spheres(L=12, radius=3.0, porosity=0.7, seed=2)
    with Box(nat, relaxation_time=0.9, f_ext=(1e-5, 2e-6, 0.0), precision=prec) as box:
        box.flow_init()
        box.flow_steps(15, force_on=True)
        _, rho, j = box.flow_get(populations=False)
        for axis in range(3):
            flux, dens = box.profiles(axis)
            rf, rd = oracle_mod.profiles(nat, rho, j, axis)
            assert np.array_equal(flux, rf) and np.array_equal(dens, rd)


def test_fp32_reference_loop_tracks_fp64():
    """The reference loop (equilibration.f90:143-491) on an FP32-deviation context: the same
    phase machine, decided on the device before each in-place step.  On the C1 slit with a
    target above the FP32 resolution of j (1e-8; FP32 deviations of ~1e-3 resolve ~1e-10, the
    reference's default target) both precisions converge twice and stop at nearly the same step;
    the l2err history of the first 200 steps and the final velocity profile agree with FP64 to
    1e-4 relative."""
    nat = geo.slit(4, 4, 34)
    out = {}
    for prec in (FP64, FP32_DEV):
        with Box(nat, relaxation_time=1.0, f_ext=(1e-5, 0, 0), target_error=1e-8, precision=prec) as box:
            box.flow_init()
            steps, hist = box.equilibration(max_steps=100000, hist_cap=100000)
            _, rho, j = box.flow_get(populations=False)
        out[prec] = (steps, hist, rho, j)
    s64, h64, r64, j64 = out[FP64]
    s32, h32, r32, j32 = out[FP32_DEV]
    assert abs(s32 - s64) <= 0.05 * s64, (s32, s64)
    assert np.allclose(h32[:200], h64[:200], rtol=1e-4, atol=0)
    assert np.max(np.abs(j32[0] - j64[0])) <= 1e-4 * np.abs(j64[0]).max()
    assert np.max(np.abs(r32 - r64)) < 1e-6


def test_fp32_reference_loop_errors():
    nat = geo.slit(4, 4, 12)
    with Box(nat, relaxation_time=1.0, f_ext=(1e-5, 0, 0), target_error=1e-10, precision=FP32_DEV) as box:
        box.flow_init()
        with pytest.raises(LbgpuError) as e:
            box.equilibration(max_steps=7, hist_cap=7)
        assert e.value.status & (1 << 5)
        n, rho, j = box.flow_get()
        n[2, 4, 1, 1] = np.inf
        box.flow_set(n, rho, j)
        with pytest.raises(LbgpuError) as e:
            box.equilibration(max_steps=100, hist_cap=100)
        assert e.value.status & (1 << 3)
