"""Geometry builders on the device (lbgpu_geometry, lbgpu_create_label) against the oracle's
restatement of module_geometry.f90: node for node identical for every label over many box
sizes, including boxes with nodes at exactly the threshold distances."""
import numpy as np
import pytest

import oracle
from laboetie_gb300 import Box, LbgpuError
from laboetie_gb300.lbgpu import device_geometry

pytestmark = pytest.mark.gpu

CASES = (
    [(-1, s, None) for s in [(1, 1, 3), (17, 9, 5)]]
    + [(1, s, None) for s in [(1, 1, 3), (4, 4, 34), (33, 7, 5), (64, 64, 64)]]
    + [(2, (n, n, lz), None) for n, lz in [(3, 1), (4, 2), (9, 3), (16, 1), (33, 2), (50, 1), (101, 2), (256, 1)]]
    + [(3, (n, n, n), None) for n in (3, 4, 9, 16, 25, 32, 48, 63, 96)]
    + [(4, (n, n, lz), None) for n, lz in [(3, 1), (9, 2), (15, 1), (31, 1), (51, 2), (201, 1)]]
    + [(5, (lx, ly, 2), None) for lx in (7, 16, 20, 33, 64, 100, 128, 250, 1000) for ly in (9, 11, 21, 31, 63, 99)]
    + [(6, s, None) for s in [(1, 3, 1), (10, 10, 1), (16, 23, 2), (64, 101, 3)]]
    + [(7, (lx, n, n), p) for lx, n in [(20, 9), (40, 21), (7, 4), (33, 16), (120, 64)]
       for p in [(0.5, 0.5), (0.3, 0.6), (0.75, 0.25)]]
    + [(8, (n, n, n), None) for n in (3, 4, 9, 16, 24, 41, 80, 101)]
    + [(9, (n, n, n), None) for n in (3, 9, 15, 21, 31, 51, 75)]
    + [(10, s, None) for s in [(10, 17, 3), (20, 35, 4), (30, 52, 3), (23, 40, 5), (100, 173, 3)]]
)


@pytest.mark.parametrize("label,shape,params", CASES)
def test_device_builder_matches_oracle(label, shape, params):
    lx, ly, lz = shape
    code, ref = oracle.geometry(label, lx, ly, lz, params)
    assert code == 0
    nat = device_geometry(label, lx, ly, lz, params)
    assert np.array_equal(nat, ref), (label, shape, int((nat != ref).sum()))


def test_create_label_equals_create_with_host_nature():
    """A box built by label on the device has the same node classes as the same box created
    from the oracle's nature array."""
    code, ref = oracle.geometry(3, 24, 24, 24)
    assert code == 0
    with Box.from_label(3, 24, 24, 24) as a, Box(ref) as b:
        assert np.array_equal(a.nature, ref)
        assert a.node_counts() == b.node_counts()
        assert np.array_equal(a.interfacial(), b.interfacial())


def test_all_solid_box_is_refused_on_the_device():
    with pytest.raises(LbgpuError, match="All nodes are solid"):
        device_geometry(7, 4, 2, 2, (0.5, 0.1))
    with pytest.raises(LbgpuError, match="All nodes are solid"):
        Box.from_label(7, 4, 2, 2, (0.5, 0.1))


def test_batch_box_by_label_equals_box_from_host_nature(oracle_mod):
    """lbgpu_batch_add_label: the same flow state as lbgpu_batch_add with the oracle's array."""
    from laboetie_gb300.lbgpu import Batch

    code, nat = oracle_mod.geometry(2, 20, 20, 6)
    assert code == 0
    res = []
    with Batch() as b:
        a = b.add_label(2, 20, 20, 6, f_ext=(0.0, 0.0, 1e-5))
        h = b.add(nat, f_ext=(0.0, 0.0, 1e-5))
        b.steps(40)
        res = [b.moments(a), b.moments(h)]
    (ra, ja), (rh, jh) = res
    assert np.array_equal(ra, rh) and all(np.array_equal(ja[d], jh[d]) for d in range(3))
    with Batch() as b:
        with pytest.raises(LbgpuError, match="should have same lx and ly"):
            b.add_label(2, 20, 21, 6)
