"""Failure detection and determinism, with every fault made on the host (no GPU fault):
a non-finite population handed in through lbgpu_flow_set stops the reference loop with the
non-finite status; a served request whose force is non-finite leaves with that status while the
requests sharing the device finish bit-identical to their runs alone; a capped request is
flagged; and repeated runs are bit-identical (deterministic reductions, no races)."""
import math

import numpy as np
import pytest

from laboetie_gb300 import FP32_DEV, FP64, Box, LbgpuError
from laboetie_gb300 import geometry as geo
from laboetie_gb300.lbgpu import Batch

pytestmark = pytest.mark.gpu

ERR_NONFINITE = 1 << 3
ERR_STEP_CAP = 1 << 5


def test_injected_nan_stops_the_reference_loop():
    nat = geo.slit(4, 4, 12)
    with Box(nat, relaxation_time=1.0, f_ext=(1e-5, 0, 0), target_error=1e-10) as box:
        box.flow_init()
        n, rho, j = box.flow_get()
        n[3, 5, 2, 1] = np.nan                    # one population of one fluid node
        box.flow_set(n, rho, j)
        with pytest.raises(LbgpuError) as e:
            box.equilibration(max_steps=1000, hist_cap=1000)
        assert e.value.status & ERR_NONFINITE


def test_serving_isolates_a_failing_and_a_capped_request():
    tr = dict(Db=0.01, ka=0.01 * math.e, kd=0.01)
    good = [geo.slit(4, 4, 20), geo.slit(3, 5, 10), geo.cylinder(11, 11, 6)]   # converge fast
    fes = [(1e-5, 0, 0), (1e-5, 0, 0), (0, 0, 1e-5)]
    reqs = [dict(nature=n, arrival=0.001 * k, f_ext=f, tracer=dict(tr, f_ext=f), max_steps=20000,
                 mp_steps=100, moments=True) for k, (n, f) in enumerate(zip(good, fes))]
    reqs.append(dict(nature=geo.slit(4, 4, 16), arrival=0.0, f_ext=(float("nan"), 0.0, 0.0),
                     max_steps=4000, moments=True))                       # fails
    reqs.append(dict(nature=geo.slit(4, 4, 64), arrival=0.0, f_ext=(1e-5, 0.0, 0.0),
                     max_steps=200, moments=True))                        # capped, never converges
    with Batch() as b:
        mix = b.serve(reqs, du_tol=1e-9, check_every=100)
    assert mix[3]["status"] & ERR_NONFINITE and mix[3]["steps"] == 100
    assert mix[4]["status"] == ERR_STEP_CAP and mix[4]["steps"] == 200 and not mix[4]["converged"]
    for k in range(3):
        assert mix[k]["status"] == 0 and mix[k]["converged"]
        with Batch() as b:
            alone = b.serve([dict(reqs[k], arrival=0.0)], du_tol=1e-9, check_every=100)[0]
        assert alone["steps"] == mix[k]["steps"]
        (ra, ja), (rb, jb) = alone["moments"], mix[k]["moments"]
        assert np.array_equal(ra, rb) and all(np.array_equal(ja[d], jb[d]) for d in range(3))
        assert np.array_equal(alone["vacf_sum"], mix[k]["vacf_sum"])


def test_repeated_runs_are_bit_identical():
    nat = geo.porous_spheres(L=40, radius=5.0, porosity=0.6, seed=8)
    runs = []
    for _ in range(2):
        with Box(nat, relaxation_time=0.8, f_ext=(1e-5, 0, 0), precision=FP32_DEV) as box:
            box.flow_init()
            box.flow_steps(120, force_on=True)
            n, rho, j = box.flow_get()
            v0 = box.mp_init(f_ext=(1e-5, 0, 0), Db=0.01, ka=0.02, kd=0.01)
            vac, _ = box.mp_propagate(60)
            P, A = box.mp_get()
        runs.append((n, rho, j, v0, vac, P, A))
    a, b = runs
    for x, y in zip(a, b):
        if isinstance(x, tuple):
            assert all(np.array_equal(p, q) for p, q in zip(x, y))
        else:
            assert np.array_equal(x, y)


def test_tracer_copy_wait_that_runs_out_reports_timeout_promptly(monkeypatch):
    """The FP32 tracer's slab step waits, bounded, for the bulk copies that stage its planes.
    LBGPU_MP_TEST_SKIP_COPIES=1 arms each plane's barrier without issuing its copies (a flag that
    nothing sets: no fault, no hang): every interior tile's wait runs out after 50 ms, the block
    lets nothing else land, leaves its nodes alone and reports LBGPU_ERR_TIMEOUT.  The call returns
    that status after its first step's graph, not after the 5000 steps asked for, and the context
    stays usable."""
    monkeypatch.setenv("LBGPU_MP_TEST_SKIP_COPIES", "1")
    nat = geo.porous_spheres(96, 6.0, 0.7, 11)   # interior 32 x 8 tiles: bulk-copied planes
    fluid = nat == 0
    rho = np.where(fluid, 1.0, 0.0)
    j = [np.where(fluid, 1e-4, 0.0), np.zeros(nat.shape), np.zeros(nat.shape)]
    import time

    with Box(nat, precision=FP32_DEV) as box:
        box.mp_init(moments=(rho, j), Db=0.01)
        t = time.perf_counter()
        with pytest.raises(LbgpuError) as e:
            box.mp_propagate(5000)
        dt = time.perf_counter() - t
        assert e.value.status & (1 << 10)
        assert dt < 30.0
        box.flow_init()                           # the context still runs work
        box.flow_steps(4, force_on=True)
        _, r2, _ = box.flow_get(populations=False)
    assert np.isfinite(r2).all()
