"""Host logic of the seeded workloads and geometry generators (no GPU)."""
import numpy as np

from laboetie_gb300 import geometry as geo
from laboetie_gb300 import workloads as wl


def test_batched_cells_shapes_and_seed():
    cells = wl.batched_cells(n_cells=32, n_tubes=4)
    again = wl.batched_cells(n_cells=32, n_tubes=4)
    assert len(cells) == 36
    for (a, fa, ka), (b, fb, kb) in zip(cells, again):
        assert ka == kb and fa == fb and np.array_equal(a, b)   # seeded: reproducible
    for nat, fe, fam in cells[:32]:
        assert fam == "cell" and nat.shape == (50, 50, 1) and fe == (0.0, 0.0, wl.FEXT)
        assert np.all(nat[:, 0, 0] == 1) and np.all(nat[:, 49, 0] == 1)   # walls at y = 1, 50
        assert 0 < (nat == 0).sum() < nat.size
    for nat, fe, fam in cells[32:]:
        lz, ly, lx = nat.shape
        assert fam == "tube" and (lx, ly) == (32, 32) and 64 <= lz <= 256
        # radius between 6 and 14: the axis is fluid, the corners solid
        assert np.all(nat[:, 16, 16] == 0) and np.all(nat[:, 0, 0] == 1)


def test_chromatography_discs_do_not_overlap():
    for seed in range(20):
        nat = geo.chromatography_cell(seed=seed, n_discs=8)
        solid = int((nat == 1).sum()) - 2 * 50          # minus the two walls
        # eight discs of radius 5 cover about 8 * 81 nodes when they do not overlap
        assert solid > 8 * 70


def test_serving_stream_arrivals_and_families():
    reqs = wl.serving_stream(seed=3, n=40, rate=10.0, max_steps=1000, mp_steps=100)
    t = [r["arrival"] for r in reqs]
    assert all(b > a for a, b in zip(t, t[1:]))
    assert abs(np.mean(np.diff([0.0] + t)) - 0.1) < 0.05    # Poisson rate 10/s
    for r in reqs:
        nat, fam = r["nature"], r["family"]
        lz, ly, lx = nat.shape
        if fam == "slit":
            assert (lx, ly) == (4, 4) and 16 <= lz <= 128
        elif fam == "cylinder":
            assert lx == ly and 16 <= lx <= 96 and lz == 32
        elif fam == "cc":
            assert lx == ly == lz and 32 <= lx <= 96
        else:
            assert fam == "cavity" and lx == ly == lz and 24 <= lx <= 80
        assert r["tracer"]["Db"] == 0.01 and r["mp_steps"] == 100 and r["max_steps"] == 1000


def test_geometry_known_counts():
    nat = geo.slit(4, 4, 34)                     # C1: 512 fluid nodes between two walls
    assert int((nat == 0).sum()) == 512
    cyl = wl.cylinder_r(20, 3, 20 / 2 - 2)
    assert cyl[0, 9, 0] == 1 and cyl[0, 9, 9] == 0   # (x=1, y=10) is outside radius 8, centre is inside
    cav = geo.spherical_cavity(9, 9, 9)
    assert cav[4, 4, 4] == 0 and cav[0, 0, 0] == 1
    assert np.array_equal(cav, cav[::-1, ::-1, ::-1])   # symmetric about the centre
