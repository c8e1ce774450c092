"""Box shapes at the edges of the layouts: rows shorter and longer than the 32-node words of the
fluid-only AA layout (x-wrap across words, partial last words), one-node-wide boxes, a single
fluid node, and solid-free boxes.

* FP64 fixed steps against the oracle: bit-identical.
* FP32 in-place (fluid-only AA) against FP32 two-buffer (lattice A/B): bit-identical, since both
  do the same per-node arithmetic and only the addressing differs.
* Batch: a box in shared memory and the same box in compact HBM tiles: bit-identical.
"""
import numpy as np
import pytest

from laboetie_gb300 import FP32_DEV, Box
from laboetie_gb300 import geometry as geo
from laboetie_gb300.lbgpu import Batch

from test_flow_gpu import oracle_fixed_steps

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1, 7), (2, 3, 5), (33, 5, 4), (64, 3, 3), (65, 2, 6), (31, 9, 2), (97, 2, 3)]


def ragged(shape, seed, solid=0.3):
    lx, ly, lz = shape
    rng = np.random.default_rng(seed)
    nat = (rng.random((lz, ly, lx)) < solid).astype(np.int8)
    nat.flat[rng.integers(nat.size)] = 0   # at least one fluid node
    return nat


@pytest.mark.parametrize("shape", SHAPES)
def test_fp64_fixed_steps_bit_exact_on_ragged_shapes(oracle_mod, shape):
    nat = ragged(shape, seed=sum(shape))
    fe = (1e-5, -2e-6, 3e-6)
    K = 9
    with Box(nat, relaxation_time=0.9, f_ext=fe) as box:
        box.flow_init()
        box.flow_steps(K, force_on=True)
        n, rho, j = box.flow_get()
    n_o, rho_o, j_o = oracle_fixed_steps(oracle_mod, nat, 0.9, fe, K)
    assert np.array_equal(n, n_o) and np.array_equal(rho, rho_o)
    for d in range(3):
        assert np.array_equal(j[d], j_o[d])


@pytest.mark.parametrize("shape", SHAPES)
def test_fp32_compact_aa_equals_lattice_ab_on_ragged_shapes(monkeypatch, shape):
    nat = ragged(shape, seed=7 * sum(shape))
    out = {}
    for mode in ("ab", "aa"):
        monkeypatch.setenv("LBGPU_FP32_STREAMING", mode)
        with Box(nat, relaxation_time=0.8, f_ext=(2e-5, 1e-5, -1e-5), precision=FP32_DEV) as box:
            box.flow_init()
            res = []
            for k in (1, 4, 11):
                box.flow_steps(k, force_on=True)
                res.append(box.flow_get())
        out[mode] = res
    for (na, ra, ja), (nb, rb, jb) in zip(out["ab"], out["aa"]):
        assert np.array_equal(na, nb) and np.array_equal(ra, rb)
        for d in range(3):
            assert np.array_equal(ja[d], jb[d])


def test_single_fluid_node_and_solid_free_box(monkeypatch):
    """A fluid node walled in on every side bounces everything back to itself: with no force its
    rest state is a fixed point; a solid-free box keeps its mass exactly under forcing."""
    nat = np.ones((3, 3, 3), dtype=np.int8)
    nat[1, 1, 1] = 0
    with Box(nat, precision=FP32_DEV) as box:
        box.flow_init()
        box.flow_steps(10, force_on=False)
        n, rho, j = box.flow_get()
    assert rho[1, 1, 1] == 1.0 and np.all(rho[nat == 1] == 0.0)
    assert np.all(np.isfinite(n))
    bulk = geo.bulk(40, 3, 2)
    with Box(bulk, f_ext=(1e-5, 0.0, 0.0), precision=FP32_DEV) as box:
        box.flow_init()
        box.flow_steps(50, force_on=True)
        _, rho, j = box.flow_get(populations=False)
    assert abs(rho.sum() - bulk.size) < 1e-9 * bulk.size
    assert np.allclose(j[0], j[0].flat[0], rtol=1e-6)   # uniform acceleration of a periodic box


@pytest.mark.parametrize("shape", [(33, 5, 4), (65, 2, 6), (40, 9, 3)])
def test_batch_shared_memory_and_compact_tiles_agree_on_ragged_shapes(monkeypatch, shape):
    nat = ragged(shape, seed=3 * sum(shape))
    fe = (1e-5, 0.0, 2e-6)
    res = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("LBGPU_BATCH_SMEM", mode)
        with Batch() as b:
            box = b.add(nat, f_ext=fe)
            assert b.info()["smem_boxes"] == (1 if mode == "1" else 0)
            b.steps(26)
            res[mode] = b.moments(box)
    (ra, ja), (rb, jb) = res["1"], res["0"]
    assert np.array_equal(ra, rb)
    for d in range(3):
        assert np.array_equal(ja[d], jb[d])
