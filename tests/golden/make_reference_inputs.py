"""Packs the reference's own input files into tests/golden/reference_inputs.npz.

The reference ships no golden outputs, but it does ship inputs: lb.in (a 1x1x102 slit), geom.in
(a list of solid nodes read by geometryLabel 0), tube.in (the two numbers of geometryLabel 7) and
the chromatography cells tuto/geom.in_chromat_* (1x50x50, walls and 0..8 discs of diameter 10,
made by tools/chromato_generator.f90).  The tests run them through the oracle and the GPU; the GPU
box does not hold the reference, so this script (run where the reference is) records them:

* lb_in: the text of lb.in;
* geom_in: the (x, y, z) triples of geom.in, in file order;
* tube_in: the first two numbers of tube.in;
* cell_names, cell_offsets, cell_nodes: the solid-node triples of every non-empty
  tuto/geom.in_chromat_* file (one empty file, ..._v9, is skipped: the reference's reader has no
  defined result for it, since its first read fails before i, j, k are set).

Run from the repository root:  python tests/golden/make_reference_inputs.py [reference dir]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def triples(path):
    out = []
    with open(path) as fh:
        for line in fh:
            parts = line.split()
            if len(parts) >= 3:
                out.append([int(p) for p in parts[:3]])
    return np.array(out, dtype=np.int16).reshape(-1, 3)


def main(ref):
    lb_in = open(os.path.join(ref, "lb.in")).read()
    geom_in = triples(os.path.join(ref, "geom.in"))
    tube_in = np.array([float(t) for t in open(os.path.join(ref, "tube.in")).read().split()[:2]])
    tuto = os.path.join(ref, "tuto")
    names, offs, nodes = [], [0], []
    for fn in sorted(os.listdir(tuto)):
        if not fn.startswith("geom.in_chromat_"):
            continue
        t = triples(os.path.join(tuto, fn))
        if len(t) == 0:
            continue
        names.append(fn)
        nodes.append(t)
        offs.append(offs[-1] + len(t))
    np.savez_compressed(os.path.join(HERE, "reference_inputs.npz"), lb_in=np.array(lb_in),
                        geom_in=geom_in, tube_in=tube_in, cell_names=np.array(names),
                        cell_offsets=np.array(offs, dtype=np.int64),
                        cell_nodes=np.concatenate(nodes))
    print(len(names), "cells,", len(geom_in), "geom.in nodes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
