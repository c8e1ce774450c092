"""Geometry builders: the reference's geometry labels and seeded synthetic porous media.

All builders return ``nature`` as an int8 array of shape (lz, ly, lx) (x fastest), 0 = fluid,
1 = solid, the layout of ``node%nature`` in module_system.f90.  Indices in the formulas are the
reference's 1-based ones.

The label builders restate module_geometry.f90; distances use gfortran's NORM2 algorithm
(scaled sum of squares) so that nodes at exactly the threshold distance fall on the same side.
The synthetic generators draw from SplitMix64 so that every geometry is reproducible from its
seed on any machine.
"""
from __future__ import annotations

import math

import numpy as np

FLUID, SOLID = 0, 1


def norm2(*comps):
    """gfortran NORM2 of a short vector, element-wise over numpy arrays (scale starts at 1)."""
    comps = [np.asarray(c, dtype=np.float64) for c in comps]
    shape = np.broadcast(*comps).shape
    result = np.zeros(shape)
    scale = np.ones(shape)
    for v in comps:
        v = np.broadcast_to(v, shape)
        nz = v != 0.0
        ax = np.abs(v)
        grow = nz & (scale < ax)
        keep = nz & ~grow
        with np.errstate(divide="ignore", invalid="ignore"):
            val_g = np.where(grow, scale / np.where(ax == 0, 1.0, ax), 0.0)
            val_k = np.where(keep, ax / scale, 0.0)
        result = np.where(grow, 1.0 + result * val_g * val_g, result)
        result = np.where(keep, result + val_k * val_k, result)
        scale = np.where(grow, ax, scale)
    return scale * np.sqrt(result)


def _grid(lx, ly, lz):
    k, j, i = np.meshgrid(np.arange(1, lz + 1), np.arange(1, ly + 1), np.arange(1, lx + 1),
                          indexing="ij")
    return i, j, k


def bulk(lx, ly, lz):
    """geometryLabel = -1: no solid node."""
    return np.zeros((lz, ly, lx), dtype=np.int8)


def slit(lx, ly, lz):
    """geometryLabel = 1: solid walls at z = 1 and z = lz (module_geometry.f90:158-166)."""
    nat = np.zeros((lz, ly, lx), dtype=np.int8)
    nat[0] = SOLID
    nat[-1] = SOLID
    return nat


def cylinder(lx, ly, lz):
    """geometryLabel = 2: cylinder along z of radius (lx-1)/2 (module_geometry.f90:253-277)."""
    if lx != ly or lx < 3:
        raise ValueError("cylinder needs lx == ly >= 3")
    i, j, _ = _grid(lx, ly, lz)
    r = norm2(i - (lx + 1) / 2.0, j - (ly + 1) / 2.0)
    return np.where(r >= (lx - 1) / 2.0, SOLID, FLUID).astype(np.int8)


def cc(lx, ly, lz):
    """geometryLabel = 3: touching solid spheres at the corners and centre of a cubic cell
    (module_geometry.f90:206-245)."""
    if not (lx == ly == lz):
        raise ValueError("cc needs a cubic box")
    i, j, k = _grid(lx, ly, lz)
    centres = [(1, 1, 1), (lx, 1, 1), (1, ly, 1), (1, 1, lz), (lx, ly, 1), (lx, 1, lz),
               (1, ly, lz), (lx, ly, lz), ((lx + 1) / 2.0, (ly + 1) / 2.0, (lz + 1) / 2.0)]
    thr = (lx - 1) * math.sqrt(3.0) / 4.0
    solid = np.zeros(i.shape, dtype=bool)
    for c in centres:
        solid |= norm2(i - c[0], j - c[1], k - c[2]) <= thr
    return solid.astype(np.int8)


def spherical_cavity(lx, ly, lz):
    """geometryLabel = 8: spherical fluid cavity of radius (lx-1)/2 (module_geometry.f90:173-198)."""
    if not (lx == ly == lz) or lx < 3:
        raise ValueError("cavity needs a cubic box with lx >= 3")
    i, j, k = _grid(lx, ly, lz)
    o = (lx + 1) / 2.0
    r = norm2(i - o, j - o, k - o)
    return np.where(r >= (lx - 1) / 2.0, SOLID, FLUID).astype(np.int8)


def tube_varying_diameter(lx, ly, lz, lw_o_lx=0.5, a_o_R=0.5):
    """geometryLabel = 7: tube along x with a wide (radius R = (ly-1)/2) and a narrow (radius
    a_o_R*R) section, the two numbers of tube.in (module_geometry.f90:52-89)."""
    if ly != lz:
        raise ValueError("tube needs ly == lz")
    R = (ly - 1) / 2.0
    a = a_o_R * R
    i, j, k = _grid(lx, ly, lz)
    d = norm2(j - (ly + 1) / 2.0, k - (lz + 1) / 2.0)
    fluid = np.where(i > lw_o_lx * lx, d < a, d < R)
    return np.where(fluid, FLUID, SOLID).astype(np.int8)


def disc_benichou(lx, ly, lz):
    """geometryLabel = 4: a disc of radius (lx-1)/2 with four exits, along z
    (module_geometry.f90:336-378); lx == ly, odd."""
    if lx != ly or lx % 2 == 0:
        raise ValueError("disc needs lx == ly, odd")
    i, j, _ = _grid(lx, ly, lz)
    ox, oy = (lx + 1) / 2.0, (ly + 1) / 2.0
    radius = float(norm2(1.0 - ox, float((lx + 1) // 2) - oy))
    return np.where(norm2(i - ox, j - oy) > radius, SOLID, FLUID).astype(np.int8)


def sinusoidal_walls(lx, ly, lz):
    """geometryLabel = 5: a channel along x between walls y = +-(a sin(2 pi (i-1)/lx) + b) about
    the middle row (module_geometry.f90:122-153); ly odd."""
    if ly % 2 == 0:
        raise ValueError("sinusoidal walls need an odd ly")
    midly = (ly + 1) // 2
    b = float(np.float32(np.float32(2.0) / np.float32(3.0)) * np.float32(midly))   # 2./3.*midly, REAL
    a = float(midly) - b - 1.0
    if a <= 0.0 or b <= 0.0:
        raise ValueError("sinusoidal walls: amplitude or offset not positive")
    nat = np.zeros((lz, ly, lx), dtype=np.int8)
    for i in range(1, lx + 1):
        yi = a * math.sin(2.0 * math.pi * float(i - 1) / float(lx)) + b + float(midly)
        ay = abs(yi)
        ninty = (int(math.floor(ay)) + (1 if ay - math.floor(ay) >= 0.5 else 0)) * (1 if yi >= 0 else -1)   # NINT
        for jj in range(midly, ly + 1):
            v = FLUID if jj < ninty else SOLID
            nat[:, jj - 1, i - 1] = v
            nat[:, 2 * midly - jj - 1, i - 1] = v
    return nat


def planes_two_radii(lx, ly, lz):
    """geometryLabel = 6: walls at y = 1 and y = ly, narrowed by (ly-2)/4 rows on each side for
    x > lx/2 (module_geometry.f90:96-119)."""
    nat = np.zeros((lz, ly, lx), dtype=np.int8)
    nat[:, 0, :] = SOLID
    nat[:, ly - 1, :] = SOLID
    q = (ly - 2) // 4 if ly >= 2 else 0
    for i in range(1, lx + 1):
        if i > lx // 2:
            for jj in range(2, 1 + q + 1):
                nat[:, jj - 1, i - 1] = SOLID
            for jj in range(ly - q, ly):
                nat[:, jj - 1, i - 1] = SOLID
    return nat


def sphere_benichou(lx, ly, lz):
    """geometryLabel = 9: a spherical cavity with six exits (module_geometry.f90:287-331);
    cubic box, odd side."""
    if not (lx == ly == lz) or lx % 2 == 0:
        raise ValueError("sphere needs a cubic box with odd side")
    i, j, k = _grid(lx, ly, lz)
    o = (lx + 1) / 2.0
    radius = float(norm2(1.0 - o, float((ly + 1) // 2) - o, float((lz + 1) // 2) - o))
    return np.where(norm2(i - o, j - o, k - o) > radius, SOLID, FLUID).astype(np.int8)


def cylinders_between_walls(lx, ly, lz):
    """geometryLabel = 10: four cylinders of radius 0.2 lx centred on the edges of an lx x ly
    cell (ly = lx sqrt 3 within 5 %) between walls at z = 1 and z = lz
    (module_geometry.f90:11-49)."""
    s3 = np.float32(math.sqrt(3.0))
    if abs(np.float32(ly) / np.float32(lx) - s3) / s3 >= np.float32(0.05):
        raise ValueError("ly should be lx*sqrt(3)")
    if lz < 3:
        raise ValueError("lz should be greater than 2")
    i, j, _ = _grid(lx, ly, lz)
    midx, midy = (lx + 1) / 2.0, (ly + 1) / 2.0
    radius = 0.2 * lx
    solid = np.zeros(i.shape, dtype=bool)
    for cx, cy in ((1.0, midy), (float(lx), midy), (midx, 1.0), (midx, float(ly))):
        solid |= norm2(i - cx, j - cy) <= radius
    nat = solid.astype(np.int8)
    nat[0] = SOLID
    nat[-1] = SOLID
    return nat


def custom(lx, ly, lz, solid_nodes):
    """geometryLabel = 0: list of 1-based (i, j, k) solid nodes as in geom.in
    (module_geometry.f90:380-426)."""
    nat = np.zeros((lz, ly, lx), dtype=np.int8)
    for (i, j, k) in solid_nodes:
        if not (1 <= i <= lx and 1 <= j <= ly and 1 <= k <= lz):
            raise ValueError(f"geom.in node {(i, j, k)} outside the box")
        nat[k - 1, j - 1, i - 1] = SOLID
    return nat


def read_geom_in(path, lx, ly, lz):
    nodes = []
    with open(path) as fh:
        for line in fh:
            parts = line.split()
            if len(parts) >= 3:
                nodes.append(tuple(int(p) for p in parts[:3]))
    return custom(lx, ly, lz, nodes)


def read_pbm(path, lx, ly, lz):
    """geometryLabel = 11: a plain PBM image (P1) of ly columns and lz lines, '1' = solid, in the
    plane x = 1 (module_geometry.f90:430-511); lx must be 1."""
    if lx != 1:
        raise ValueError("lx must be 1 if geom.pbm is used")
    with open(path) as fh:
        tokens = fh.read().split()
    if not tokens or tokens[0] != "P1":
        raise ValueError("geom.pbm: magic number is not P1")
    ncol, nline = int(tokens[1]), int(tokens[2])
    if ncol != ly or nline != lz:
        raise ValueError("geom.pbm: columns / lines differ from ly / lz")
    pix = "".join(tokens[3:])
    if len(pix) < ncol * nline or set(pix[:ncol * nline]) - {"0", "1"}:
        raise ValueError("geom.pbm: pixels must be 0 or 1")
    nat = np.zeros((lz, ly, 1), dtype=np.int8)
    nat[:, :, 0] = (np.frombuffer(pix[:ncol * nline].encode(), dtype=np.uint8) - ord("0")).reshape(nline, ncol)
    return nat


LABELS = {-1: bulk, 1: slit, 2: cylinder, 3: cc, 4: disc_benichou, 5: sinusoidal_walls,
          6: planes_two_radii, 7: tube_varying_diameter, 8: spherical_cavity, 9: sphere_benichou,
          10: cylinders_between_walls}


def build(label, lx, ly, lz, params=None):
    """The builder of geometryLabel `label` (supercell_definition.f90:52-80); label 7 takes
    params = (lw_o_lx, a_o_R), the two numbers of tube.in.  Labels 0 (geom.in) and 11 (geom.pbm)
    read files: read_geom_in, read_pbm."""
    if label not in LABELS:
        raise ValueError(f"geometryLabel {label}: no builder (0 and 11 read geom.in / geom.pbm)")
    if label == 7:
        lw, ar = params if params is not None else (0.5, 0.5)
        nat = tube_varying_diameter(lx, ly, lz, lw, ar)
    else:
        nat = LABELS[label](lx, ly, lz)
    if not (nat == FLUID).any():
        raise ValueError("All nodes are solid: no fluid, no fluid dynamics!")
    return nat


def write_geom_in(path, nature):
    k, j, i = np.nonzero(nature == SOLID)
    order = np.lexsort((k, j, i))
    with open(path, "w") as fh:
        for q in order:
            fh.write(f"{i[q] + 1}\t{j[q] + 1}\t{k[q] + 1}\n")


# ------------------------------------------------------------------------ synthetic media

class SplitMix64:
    """SplitMix64 (Steele, Lea, Flood 2014), the seeded generator of every synthetic geometry."""

    MASK = (1 << 64) - 1

    def __init__(self, seed: int):
        self.state = seed & self.MASK

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & self.MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & self.MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & self.MASK
        return z ^ (z >> 31)

    def uniform(self) -> float:
        """uniform in [0, 1) with 53 random bits"""
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))

    def randint(self, lo: int, hi: int) -> int:
        """uniform integer in [lo, hi]"""
        return lo + int(self.uniform() * (hi - lo + 1))


def porous_spheres(L=192, radius=8.0, porosity=0.60, seed=20261203):
    """Periodic L^3 box; solid spheres of the given radius (min-image distance <= radius) at
    uniform seeded centres, overlap allowed, added until the porosity is <= the target."""
    rng = SplitMix64(seed)
    solid = np.zeros((L, L, L), dtype=bool)
    r = int(math.ceil(radius))
    off = np.arange(-r, r + 1)
    dz, dy, dx = np.meshgrid(off, off, off, indexing="ij")
    ball = (dx * dx + dy * dy + dz * dz) <= radius * radius
    # offsets taken modulo L and made unique, so a sphere wider than the box counts each node once
    offs = np.unique(np.stack([dz[ball] % L, dy[ball] % L, dx[ball] % L], axis=1), axis=0)
    bz, by, bx = offs[:, 0], offs[:, 1], offs[:, 2]
    total = L ** 3
    n_solid = 0
    while 1.0 - n_solid / total > porosity:
        cx, cy, cz = (int(rng.uniform() * L) for _ in range(3))
        zz = (cz + bz) % L
        yy = (cy + by) % L
        xx = (cx + bx) % L
        new = ~solid[zz, yy, xx]
        n_solid += int(np.count_nonzero(new))
        solid[zz, yy, xx] = True
    return solid.astype(np.int8)


def chromatography_cell(seed, ny=50, nz=50, n_discs=None, radius=5.0):
    """1 x ny x nz cell with solid walls at y = 1 and y = ny and k non-overlapping discs of the
    given radius (k uniform in 1..8 unless given); a node is solid if its periodic distance to a
    disc centre is <= radius (tools/chromato_generator.f90:53-60)."""
    rng = SplitMix64(seed)
    k = n_discs if n_discs is not None else rng.randint(1, 8)
    centres = []
    tries = 0
    while len(centres) < k and tries < 100000:
        tries += 1
        c = (1.0 + rng.uniform() * ny, 1.0 + rng.uniform() * nz)
        ok = True
        for q in centres:
            dy = abs(c[0] - q[0]); dy = min(dy, ny - dy)
            dz = abs(c[1] - q[1]); dz = min(dz, nz - dz)
            if math.hypot(dy, dz) <= 2 * radius:
                ok = False
                break
        if ok:
            centres.append(c)
    nat = np.zeros((nz, ny, 1), dtype=np.int8)
    kk, jj = np.meshgrid(np.arange(1, nz + 1), np.arange(1, ny + 1), indexing="ij")
    for (cy, cz) in centres:
        dy = np.abs(jj - cy); dy = np.minimum(dy, ny - dy)
        dz = np.abs(kk - cz); dz = np.minimum(dz, nz - dz)
        nat[:, :, 0] |= (np.sqrt(dy * dy + dz * dz) <= radius).astype(np.int8)
    nat[:, 0, 0] = SOLID
    nat[:, ny - 1, 0] = SOLID
    return nat


def modulated_tube(L, n=32, r_mean=10.0, r_amp=4.0):
    """n x n x L tube along z, radius r_mean + r_amp sin(2 pi z / L), axis at ((n+1)/2, (n+1)/2)."""
    k, j, i = np.meshgrid(np.arange(1, L + 1), np.arange(1, n + 1), np.arange(1, n + 1),
                          indexing="ij")
    c = (n + 1) / 2.0
    rad = r_mean + r_amp * np.sin(2 * np.pi * k / L)
    d = np.sqrt((i - c) ** 2 + (j - c) ** 2)
    return np.where(d < rad, FLUID, SOLID).astype(np.int8)
