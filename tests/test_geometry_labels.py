"""The reference's geometry builders (module_geometry.f90, geometryLabel -1 and 1..10): the C
oracle against the package's numpy restatement, node for node, over many box sizes; known
counts worked out by hand; and the reference's STOP conditions.  No GPU."""
import numpy as np
import pytest

import oracle
from laboetie_gb300 import geometry as geo


def sizes(label):
    if label in (-1, 1):
        return [(1, 1, 3), (4, 4, 34), (7, 5, 3), (10, 10, 4), (3, 13, 6), (16, 2, 9)]
    if label == 6:
        return [(1, 3, 1), (4, 4, 34), (7, 5, 3), (10, 10, 1), (3, 13, 6), (16, 23, 2)]
    if label in (2,):
        return [(3, 3, 1), (4, 4, 2), (9, 9, 3), (16, 16, 1), (33, 33, 2), (50, 50, 1)]
    if label in (3, 8):
        return [(3, 3, 3), (4, 4, 4), (9, 9, 9), (16, 16, 16), (25, 25, 25), (32, 32, 32)]
    if label == 4:
        return [(3, 3, 1), (9, 9, 2), (15, 15, 1), (31, 31, 1), (51, 51, 2)]
    if label == 9:
        return [(3, 3, 3), (9, 9, 9), (15, 15, 15), (21, 21, 21), (31, 31, 31)]
    if label == 5:
        return [(l, w, 1) for l in (7, 16, 20, 33, 64, 100) for w in (9, 11, 21, 31)]
    if label == 7:
        return [(20, 9, 9), (40, 21, 21), (7, 4, 4), (33, 16, 16)]
    if label == 10:
        return [(10, 17, 3), (20, 35, 4), (30, 52, 3), (23, 40, 5)]
    raise AssertionError(label)


@pytest.mark.parametrize("label", [-1, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10])
def test_oracle_builders_match_numpy_restatement(label):
    for (lx, ly, lz) in sizes(label):
        params = (0.5, 0.5) if label == 7 else None
        for p in ([params] if label != 7 else [(0.5, 0.5), (0.3, 0.6), (0.75, 0.25)]):
            code, nat = oracle.geometry(label, lx, ly, lz, p)
            assert code == 0, (label, lx, ly, lz, code)
            ref = geo.build(label, lx, ly, lz, p)
            assert ref.shape == nat.shape and np.array_equal(ref, nat), (label, lx, ly, lz, p)


def test_known_counts():
    # slit: the two walls of a 4 x 4 x 34 box leave 512 fluid nodes
    assert int((oracle.geometry(1, 4, 4, 34)[1] == 0).sum()) == 512
    # cylinder lx = 5: centre (3, 3), radius 2; fluid where the distance is < 2: the centre, its
    # 4 axis neighbours at distance 1 and the 4 diagonal ones at sqrt(2)
    assert int((oracle.geometry(2, 5, 5, 1)[1] == 0).sum()) == 9
    # spherical cavity lx = 3: only the centre is closer than the radius 1
    assert int((oracle.geometry(8, 3, 3, 3)[1] == 0).sum()) == 1
    # Benichou disc lx = 3: radius 1, boundary included (> radius is solid): centre + 4 exits
    assert int((oracle.geometry(4, 3, 3, 1)[1] == 0).sum()) == 5
    # planes with two radii, 10 x 10: rows 1 and 10 solid everywhere; rows 2-3 and 8-9 for x > 5
    nat = oracle.geometry(6, 10, 10, 1)[1]
    assert int((nat == 1).sum()) == 2 * 10 + 4 * 5
    # cylinders between walls: the walls z = 1, lz are solid, the box centre column is fluid
    nat = oracle.geometry(10, 20, 35, 4)[1]
    assert np.all(nat[0] == 1) and np.all(nat[-1] == 1) and nat[1, 17, 9] == 0


@pytest.mark.parametrize("label,shape,code", [
    (2, (4, 5, 1), 1), (2, (2, 2, 1), 1), (3, (4, 4, 5), 1), (4, (8, 8, 1), 1), (4, (9, 7, 1), 1),
    (5, (10, 10, 1), 1), (5, (10, 3, 1), 2), (7, (10, 8, 9), 1), (8, (5, 5, 6), 1), (9, (8, 8, 8), 1),
    (10, (10, 10, 3), 1), (10, (10, 17, 2), 1), (0, (4, 4, 4), 3), (11, (1, 4, 4), 3), (12, (4, 4, 4), 3),
])
def test_reference_stop_conditions(label, shape, code):
    params = (0.5, 0.5) if label == 7 else None
    assert oracle.geometry(label, *shape, params)[0] == code
    with pytest.raises(ValueError):
        geo.build(label, *shape, params)


def test_all_solid_box_is_refused():
    # a tube narrower than one node: every node is solid (supercell_definition.f90:92-94)
    assert oracle.geometry(7, 4, 2, 2, (0.5, 0.1))[0] == 4
    with pytest.raises(ValueError, match="All nodes are solid"):
        geo.build(7, 4, 2, 2, (0.5, 0.1))


def test_pbm_reader(tmp_path):
    p = tmp_path / "geom.pbm"
    p.write_text("P1\n4 3\n1 0 0 1\n0 0 0 0\n1 1 0 0\n")
    nat = geo.read_pbm(str(p), 1, 4, 3)
    assert nat.shape == (3, 4, 1)
    assert nat[:, :, 0].tolist() == [[1, 0, 0, 1], [0, 0, 0, 0], [1, 1, 0, 0]]
    with pytest.raises(ValueError):
        geo.read_pbm(str(p), 2, 4, 3)


@pytest.mark.parametrize("label,shape,params,msg", [
    (2, (4, 5, 1), None, "should have same lx and ly"),
    (3, (4, 4, 5), None, "cubic with lx=ly=lz"),
    (4, (8, 8, 1), None, "lx should be odd"),
    (5, (10, 10, 1), None, "ly should be odd"),
    (7, (10, 8, 9), (0.5, 0.5), "ly should be equal to lz"),
    (7, (10, 9, 9), None, "tube.in cannot be read"),
    (10, (10, 10, 3), None, "ly shoud be lx *sqrt(3)"),
    (0, (4, 4, 4), None, "geom.in on the host"),
    (11, (1, 4, 4), None, "geom.pbm on the host"),
    (13, (4, 4, 4), None, "label tag in input file is invalid"),
])
def test_device_builder_refuses_like_the_reference_without_a_gpu(label, shape, params, msg):
    """The C ABI checks the box before any device work: the reference's STOP message comes back
    through lbgpu_last_error(NULL, ...) on a machine without a GPU too."""
    from laboetie_gb300 import LbgpuError
    from laboetie_gb300.lbgpu import device_geometry
    with pytest.raises(LbgpuError, match="invalid argument") as e:
        device_geometry(label, *shape, params)
    assert msg in str(e.value)
