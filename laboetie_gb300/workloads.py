"""Seeded synthetic workloads for the batched and served solvers.

* ``batched_cells``: 1024 two-dimensional chromatography cells of 1 x 50 x 50 (solid walls at
  y = 1 and y = 50, k non-overlapping solid discs of diameter 10, k uniform in 1..8) plus 64
  tubes of 32 x 32 x L (L uniform in 64..256) whose radius is modulated sinusoidally between 6
  and 14 along the axis; tau 1, f_ext 1e-5 along the long (flow) axis.
* ``serving_stream``: Poisson arrivals of solves drawn uniformly from four families -- slit
  (lx = ly = 4, lz in 16..128), cylinder along z (lx = ly in 16..96, radius lx/2 - 2), touching
  spheres at the corners and centre of a cubic cell (32^3..96^3) and spherical cavity
  (24^3..80^3).

Geometries follow the reference's generators (module_geometry.f90, tools/chromato_generator.f90)
as restated in geometry.py.
"""
from __future__ import annotations

import math

import numpy as np

from . import geometry as geo

# Tracer of the batched and served solves: Db 0.01, adsorbing on interfacial fluid nodes with
# Boltzmann factor exp(-beta dF), beta dF = -1 (K = e, kd = 0.01).
TRACER = dict(Db=0.01, ka=0.01 * math.e, kd=0.01)
FEXT = 1e-5


def cylinder_r(n, lz, radius):
    """n x n x lz cylinder along z with the given radius, axis at ((n+1)/2, (n+1)/2)."""
    _, j, i = np.meshgrid(np.arange(1, lz + 1), np.arange(1, n + 1), np.arange(1, n + 1), indexing="ij")
    c = (n + 1) / 2.0
    d = geo.norm2(i - c, j - c)
    return np.where(d >= radius, geo.SOLID, geo.FLUID).astype(np.int8)


def batched_cells(seed=20261203, n_cells=1024, n_tubes=64):
    """[(nature, f_ext, family)]: the chromatography cells first, then the tubes."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_cells):
        nat = geo.chromatography_cell(seed=int(rng.integers(1 << 62)), ny=50, nz=50, radius=5.0)
        out.append((nat, (0.0, 0.0, FEXT), "cell"))
    for k in range(n_tubes):
        L = int(rng.integers(64, 257))
        out.append((geo.modulated_tube(L, n=32, r_mean=10.0, r_amp=4.0), (0.0, 0.0, FEXT), "tube"))
    return out


def serving_family(rng, family):
    """(nature, f_ext) of one solve of the family ('slit', 'cylinder', 'cc', 'cavity')."""
    if family == "slit":
        return geo.slit(4, 4, int(rng.integers(16, 129))), (FEXT, 0.0, 0.0)
    if family == "cylinder":
        n = int(rng.integers(16, 97))
        return cylinder_r(n, 32, n / 2 - 2), (0.0, 0.0, FEXT)
    if family == "cc":
        L = int(rng.integers(32, 97))
        return geo.cc(L, L, L), (FEXT, 0.0, 0.0)
    L = int(rng.integers(24, 81))
    return geo.spherical_cavity(L, L, L), (FEXT, 0.0, 0.0)


def serving_stream(seed, n, rate, max_steps=20000, mp_steps=10000, families=None):
    """n request dicts for Batch.serve with Poisson arrivals at `rate` per second."""
    rng = np.random.default_rng(seed)
    fams = families or ("slit", "cylinder", "cc", "cavity")
    t = 0.0
    out = []
    for _ in range(n):
        t += rng.exponential(1.0 / rate)
        fam = fams[int(rng.integers(len(fams)))]
        nat, fe = serving_family(rng, fam)
        out.append(dict(nature=nat, arrival=t, f_ext=fe, tracer=dict(TRACER, f_ext=fe),
                        max_steps=max_steps, mp_steps=mp_steps, family=fam))
    return out
