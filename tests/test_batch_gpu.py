"""Batches of boxes and the request server (lbgpu_batch_*, lbgpu_serve) on the GPU.

The batch steps FP32-deviation populations with the force on from the first step, so its
reference points are (a) itself: a box's results must not depend on the other boxes of the
batch, nor on whether it ran in shared memory or in HBM tiles; (b) the single-box FP32 tracer
propagation given the same flow moments; (c) the FP64 oracle's steady state.
"""
import math

import numpy as np
import pytest

from laboetie_gb300 import geometry as geo
from laboetie_gb300.lbgpu import FP32_DEV, Batch, Box, LbgpuError

pytestmark = pytest.mark.gpu

TR = dict(Db=0.01, ka=0.01 * math.e, kd=0.01)


def _cells():
    """Two shared-memory-sized chromatography cells, a slit, a tiled tube and a tiled tube wide
    enough for the tracer's shared-memory slab tiles."""
    return [
        (geo.chromatography_cell(seed=3), (0.0, 0.0, 1e-5)),
        (geo.chromatography_cell(seed=8), (0.0, 0.0, 1e-5)),
        (geo.slit(4, 4, 34), (1e-5, 0.0, 0.0)),
        (geo.modulated_tube(40, n=16, r_mean=5.0, r_amp=2.0), (0.0, 0.0, 1e-5)),
        (geo.modulated_tube(36, n=32, r_mean=9.0, r_amp=3.0), (0.0, 0.0, 1e-5)),
    ]


def _run(cells, idx, flow_steps, mp_steps, du=None):
    """Run the cells idx together; returns {i: (rho, j, mp_get, mp_fields)}.  With a dict du, the
    flow steps end with a checked call whose max|u - u_prev| per box goes into du."""
    out = {}
    with Batch() as b:
        ids = {i: b.add(cells[i][0], relaxation_time=1.0, f_ext=cells[i][1],
                        tracer=dict(TR, f_ext=cells[i][1])) for i in idx}
        if du is None:
            b.steps(flow_steps)
        else:
            b.steps(flow_steps - 100)
            d = b.steps(100, check=True)
            du.update({i: d[ids[i]] for i in idx})
        mom = {i: b.moments(ids[i]) for i in idx}
        for i in idx:
            b.mp_start(ids[i])
        b.steps(mp_steps)
        for i in idx:
            out[i] = mom[i] + (b.mp_get(ids[i]), b.mp_fields(ids[i]))
    return out


def _same(a, b):
    (ra, ja, ma, fa), (rb, jb, mb, fb) = a, b
    assert np.array_equal(ra, rb)
    for d in range(3):
        assert np.array_equal(ja[d], jb[d])
    for x, y in zip(ma[:3], mb[:3]):
        assert np.array_equal(x, y)
    assert ma[3] == mb[3]
    assert np.array_equal(fa[0], fb[0]) and np.array_equal(fa[1], fb[1])


def test_batch_box_alone_equals_box_in_mix():
    cells = _cells()
    mix = _run(cells, range(len(cells)), 300, 200)
    for i in range(len(cells)):
        alone = _run(cells, [i], 300, 200)
        _same(alone[i], mix[i])


def test_batch_boxes_in_both_phases_at_once_equal_their_runs_alone():
    """While some boxes are in the tracer phase and the others still in the flow phase, a call
    runs the two phases' launches as concurrent chains (the shared-memory boxes of each phase on
    their own stream, the tiled boxes' tracer steps on a third stream beside the flow steps): each
    box's moments, VACF and tracer fields are bit-identical to its run alone with the same
    schedule (a shared-memory cell and a tiled tube start their tracer after 100 steps, the rest
    after 300)."""
    cells = _cells()
    early = {0, 3}

    def run(idx):
        out = {}
        with Batch() as b:
            ids = {i: b.add(cells[i][0], relaxation_time=1.0, f_ext=cells[i][1],
                            tracer=dict(TR, f_ext=cells[i][1])) for i in idx}
            b.steps(100)
            mom = {i: b.moments(ids[i]) for i in idx if i in early}
            for i in idx:
                if i in early:
                    b.mp_start(ids[i])
            b.steps(200)                  # both phases in every call
            mom.update({i: b.moments(ids[i]) for i in idx if i not in early})
            for i in idx:
                if i not in early:
                    b.mp_start(ids[i])
            b.steps(100)
            for i in idx:
                out[i] = mom[i] + (b.mp_get(ids[i]), b.mp_fields(ids[i]))
        return out

    mix = run(range(len(cells)))
    for i in range(len(cells)):
        _same(run([i])[i], mix[i])


def test_batch_shared_memory_and_tiled_paths_agree(monkeypatch):
    """The shared-memory and the tiled kernels do the same per-node arithmetic: the flow state
    and the tracer's P and P_ads are bit-identical.  The VACF terms are summed per thread in FP32
    (over a thread's few nodes of the box in shared memory, one node per thread in a tile) before
    the FP64 sums, so the VACF sums differ by that grouping: 1e-6 relative."""
    cells = _cells()[:3]
    res = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("LBGPU_BATCH_SMEM", mode)
        with Batch() as b:
            info_ids = [b.add(c, f_ext=f, tracer=dict(TR, f_ext=f)) for c, f in cells]
            res[mode + "info"] = b.info()["smem_boxes"]
        res[mode] = _run(cells, range(3), 200, 100)
    assert res["1info"] == 3 and res["0info"] == 0
    for i in range(3):
        (ra, ja, ma, fa), (rb, jb, mb, fb) = res["1"][i], res["0"][i]
        assert np.array_equal(ra, rb)
        for d in range(3):
            assert np.array_equal(ja[d], jb[d])
        assert np.array_equal(fa[0], fb[0]) and np.array_equal(fa[1], fb[1]) and np.abs(fa[0]).max() > 0
        for x, y in zip(ma[:3], mb[:3]):
            assert np.allclose(x, y, rtol=1e-6, atol=1e-9 * np.abs(ma[0]).max())


@pytest.mark.parametrize("variant", ["4,1,8", "5,2,32", "6,4,16"])
def test_batch_work_list_launch_equals_one_block_per_tile(monkeypatch, variant):
    """The persistent work-list form of the tiled in-place step (blocks per SM, tiles claimed at a
    time, steps per graph forced through LBGPU_BATCH_AA_LIST) gives every box the same bits as one
    block per tile: the tiles are claimed in another order and by other blocks, but each node's
    arithmetic is the same.  The call's steps also run as several graphs of the tiled launches,
    while the shared-memory boxes step the whole call in one launch of their own: the flow state,
    the convergence measure of a checked call, P, P_ads and the VACF (sum included) are
    bit-identical."""
    cells = _cells()
    du_base, du_listed = {}, {}
    base = _run(cells, range(len(cells)), 300, 200, du_base)
    monkeypatch.setenv("LBGPU_BATCH_AA_LIST", variant)
    with Batch() as b:
        b.add(cells[3][0], f_ext=cells[3][1])
        b.steps(2)
        t = b.tuning()
    minb, tpc, spg = (int(v) for v in variant.split(","))
    assert t["aa_work_list"] == [1, 1] and t["aa_min_blocks"] == [minb, minb]
    assert t["aa_tiles_per_claim"] == [tpc, tpc] and t["steps_per_graph"] == spg
    listed = _run(cells, range(len(cells)), 300, 200, du_listed)
    assert du_listed == du_base and all(v > 0 for v in du_base.values())
    for i in range(len(cells)):
        _same(listed[i], base[i])


def test_batch_flow_reaches_the_fp64_steady_state(oracle_mod):
    """Poiseuille slit 4x4x34, tau 1, f_ext 1e-5: the batch's converged velocity profile
    agrees with the FP64 oracle's converged profile to 1e-4 of its maximum."""
    nat = geo.slit(4, 4, 34)
    ref = oracle_mod.equilibration(nat, tau=1.0, target_error=1e-10, f_ext=(1e-5, 0, 0),
                                   max_steps=100000)
    with Batch() as b:
        box = b.add(nat, f_ext=(1e-5, 0.0, 0.0))
        for _ in range(200):
            du = b.steps(100, check=True)[box]
            if du < 1e-11:
                break
        rho, j = b.moments(box)
    jx_ref = ref["j"][0]
    assert np.max(np.abs(j[0] - jx_ref)) <= 1e-4 * np.abs(jx_ref).max()
    fl = nat == 0
    assert np.max(np.abs(rho[fl] - ref["rho"][fl])) < 1e-5


@pytest.mark.parametrize("make,fe", [
    (lambda: geo.slit(4, 4, 34), (1e-5, 0.0, 0.0)),                                   # shared memory
    (lambda: geo.modulated_tube(48, n=32, r_mean=10.0, r_amp=4.0), (0.0, 0.0, 1e-5)),  # slab tiles
    (lambda: geo.modulated_tube(40, n=16, r_mean=5.0, r_amp=2.0), (0.0, 0.0, 1e-5)),   # node tiles
])
def test_batch_tracer_matches_single_box_fp32(make, fe):
    """Given the batch's own flow moments, the single-box FP32 propagation computes the same V,
    (u*, D) and P step for step: P and P_ads bit-identical after K steps (the batch's node, slab
    and shared-memory kernels do the single box's operations in its order).  VACF(0) agrees to
    1e-12 relative (FP64 sums of the same per-node terms in another order); the per-step VACF is
    summed per thread in FP32 over a few nodes before the FP64 sums, and the kernels group the
    nodes differently, so the VACF sums agree to 1e-6 of the summed magnitudes."""
    nat = make()
    K = 400
    with Batch() as b:
        box = b.add(nat, f_ext=fe, tracer=dict(TR, f_ext=fe))
        b.steps(2000)
        rho, j = b.moments(box)
        b.mp_start(box)
        b.steps(K)
        v0, vs, vl, steps = b.mp_get(box)
        bP, bA = b.mp_fields(box)
    assert steps == K
    with Box(nat, relaxation_time=1.0, f_ext=fe, precision=FP32_DEV) as sb:
        s0 = sb.mp_init(moments=(rho, j), f_ext=fe, **TR)
        vac, _ = sb.mp_propagate(K)
        sP, sA = sb.mp_get()
    assert len(vac) == K
    assert np.array_equal(bP, sP) and np.array_equal(bA, sA) and np.abs(sP).max() > 0
    scale = np.abs(s0).max()
    assert np.max(np.abs(v0 - s0)) <= 1e-12 * scale
    assert np.all(np.abs(vs - vac.sum(axis=0)) <= 1e-6 * np.abs(vac).sum(axis=0))
    assert np.all(np.abs(vl - vac[-1]) <= 1e-6 * np.abs(vac[-1]) + 1e-18)


def test_batch_refusals():
    with Batch() as b:
        with pytest.raises(LbgpuError):
            b.add(np.ones((4, 4, 4), dtype=np.int8))                       # all solid
        with pytest.raises(LbgpuError):
            b.add(geo.slit(4, 4, 8), relaxation_time=0.5)
        with pytest.raises(LbgpuError):
            b.add(geo.slit(4, 4, 8), tracer=dict(Db=0.01, z=1.0))          # charged
        box = b.add(geo.slit(4, 4, 8))
        with pytest.raises(LbgpuError):
            b.mp_start(box)                                                 # no tracer
        with pytest.raises(LbgpuError):
            b.steps(3)                                                      # odd
    with Batch(memory_budget=1 << 20) as b:
        with pytest.raises(LbgpuError) as e:
            b.add(geo.bulk(64, 64, 64))
        assert e.value.status & (1 << 6)


def _requests(seed, n, rate):
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(n):
        t += rng.exponential(1.0 / rate)
        fam = k % 3
        if fam == 0:
            nat, fe = geo.slit(4, 4, int(rng.integers(16, 40))), (1e-5, 0.0, 0.0)
        elif fam == 1:
            nat, fe = geo.chromatography_cell(seed=int(rng.integers(1 << 30))), (0.0, 0.0, 1e-5)
        else:
            L = int(rng.integers(12, 20)) | 1
            nat, fe = geo.cylinder(L, L, 16), (0.0, 0.0, 1e-5)
        out.append(dict(nature=nat, arrival=t, f_ext=fe, tracer=dict(TR, f_ext=fe),
                        max_steps=3000, mp_steps=200, moments=True))
    return out


def test_serve_result_alone_equals_result_in_the_stream():
    """Continuous batching: every request's moments, step count and VACF are the same when it
    is served alone and when it shares the device with the rest of a Poisson stream."""
    reqs = _requests(seed=7, n=9, rate=200.0)
    with Batch() as b:
        mix = b.serve(reqs, du_tol=1e-9, check_every=100)
    # status 0, or 1 << 5 for a flow capped before converging (its tracer steps still ran)
    assert all(r["status"] in (0, 1 << 5) and r["finished"] >= r["admitted"] >= 0 for r in mix)
    overlap = sum(1 for r in mix for q in mix if q is not r and q["admitted"] < r["finished"] and
                  r["admitted"] < q["finished"])
    assert overlap > 0   # the stream really shared the device
    for k in (0, 4, 8):
        with Batch() as b:
            alone = b.serve([dict(reqs[k], arrival=0.0)], du_tol=1e-9, check_every=100)[0]
        assert alone["steps"] == mix[k]["steps"] and alone["mp_steps"] == mix[k]["mp_steps"] == 200
        ra, ja = alone["moments"]
        rb, jb = mix[k]["moments"]
        assert np.array_equal(ra, rb)
        for d in range(3):
            assert np.array_equal(ja[d], jb[d])
        assert np.array_equal(alone["vacf0"], mix[k]["vacf0"])
        assert np.array_equal(alone["vacf_sum"], mix[k]["vacf_sum"])


def test_serve_admission_by_footprint():
    """With a budget of two boxes, the third request waits for a departure; a request larger
    than the budget is rejected with the out-of-memory status and does not block the queue."""
    from laboetie_gb300.lbgpu import footprint, make_cell

    nat = geo.slit(4, 4, 30)
    fp = footprint(make_cell((4, 4, 30)))
    big = geo.bulk(40, 40, 40)
    reqs = [dict(nature=nat, arrival=0.0, f_ext=(1e-5, 0.0, 0.0), max_steps=400) for _ in range(3)]
    reqs.insert(1, dict(nature=big, arrival=0.0, max_steps=400))
    with Batch(memory_budget=2 * fp + 1024) as b:
        res = b.serve(reqs, du_tol=0.0, check_every=100)
    assert res[1]["status"] == 1 << 6 and res[1]["admitted"] < 0
    ok = [res[i] for i in (0, 2, 3)]
    assert all(r["status"] == 1 << 5 and not r["converged"] and r["steps"] == 400 for r in ok)  # capped
    assert ok[2]["admitted"] >= min(ok[0]["finished"], ok[1]["finished"])
