"""The reference's own input files, run through both restatements and the GPU.

tests/golden/reference_inputs.npz holds lb.in, geom.in, tube.in and the 80 non-empty
chromatography cells tuto/geom.in_chromat_* of the reference (packed by
tests/golden/make_reference_inputs.py).  They are the only data the reference ships, so they are
the closest available thing to its own test cases:

* lb.in is parsed with the rules of module_input.f90 and run as the reference would: a 1x1x102
  slit (geometryLabel 1), tau 1 (relaxation_time is commented out there), f_ext 0;
* geom.in is read with the rules of module_geometry.f90:380-426 (solid nodes, the rest fluid) in a
  10x10x10 box (the reference's files do not record the box of this geom.in; its nodes span
  x 2..9, y 2..8, z 2..9);
* tube.in gives the two numbers of geometryLabel 7 (a tube whose diameter changes along x);
* every chromatography cell is a 1x50x50 box (the size in its name) with f_ext 1e-5 along z.

CPU tests: the two restatements (oracle/lb_oracle.c and oracle/np_oracle.py) agree on the
classification of every node and on the flow.  GPU tests (-m gpu): the library's interfacial
flags, node counts and FP64 flow are bit-identical to the oracle on every one of them.
"""
import os

import numpy as np
import pytest

from laboetie_gb300 import geometry as geo
from laboetie_gb300.lbin import LbIn, LbInError
from oracle import np_oracle as npo

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "reference_inputs.npz")
REF_DIR = "/root/reference"


def fixture():
    return np.load(FIX)


def cells():
    g = fixture()
    off, nodes = g["cell_offsets"], g["cell_nodes"]
    return [(str(name), geo.custom(1, 50, 50, [tuple(int(v) for v in t) for t in nodes[off[i]:off[i + 1]]]))
            for i, name in enumerate(g["cell_names"])]


def boxes():
    """(name, nature, tau, f_ext) of every reference input."""
    g = fixture()
    p = LbIn(str(g["lb_in"])).flow_params()
    out = [("lb.in", geo.LABELS[p["geometryLabel"]](p["lx"], p["ly"], p["lz"]),
            p["relaxation_time"], p["f_ext"])]
    out.append(("geom.in", geo.custom(10, 10, 10, [tuple(int(v) for v in t) for t in g["geom_in"]]),
                1.0, (1e-5, 0.0, 0.0)))
    out.append(("tube.in", geo.tube_varying_diameter(20, 12, 12, *(float(v) for v in g["tube_in"])),
                1.0, (1e-5, 0.0, 0.0)))
    out += [(name, nat, 1.0, (0.0, 0.0, 1e-5)) for name, nat in cells()]
    return out


# ------------------------------------------------------------------------------------ CPU

def test_lb_in_is_parsed_with_the_reference_rules():
    p = LbIn(str(fixture()["lb_in"])).flow_params()
    assert (p["lx"], p["ly"], p["lz"], p["geometryLabel"]) == (1, 1, 102, 1)
    assert p["relaxation_time"] == 1.0          # commented out: module_collision.f90:38 default
    assert p["f_ext"] == (0.0, 0.0, 0.0) and p["target_error"] == 1e-10 and p["rho0"] == 1.0


def test_lb_in_parser_edge_cases():
    text = ("# a comment line\n"
            "   lx = 7   # trailing comment\n"
            "lxx = 9\n"
            "relaxation_time = 0.8d0\n"
            "f_ext = 1.D-5, 0 ,2e-6\n"
            "print_vacf = false\n"
            "lbmodel = 'D3Q19'\n"
            "target_error =1e-8\n"
            "\n")
    L = LbIn(text)
    assert L.int("lx") == 7 and L.int("lxx") == 9
    assert L.dp("relaxation_time") == 0.8
    assert L.dp3("f_ext") == (1e-5, 0.0, 2e-6)
    assert L.log("print_vacf") is False
    assert L.char("lbmodel") == "D3Q19"
    # the value is read from the 4th character after the tag: "=1e-8" loses its first digit and
    # "e-8" does not read as a real (the reference's READ fails)
    with pytest.raises(LbInError):
        L.dp("target_error")
    assert L.dp("tracer_Db", 0.0) == 0.0
    with pytest.raises(LbInError):
        L.int("ly")


def test_fixture_holds_the_reference_files():
    if not os.path.isdir(REF_DIR):
        pytest.skip("the reference is not on this machine")
    import subprocess
    import sys
    import tempfile

    with tempfile.TemporaryDirectory() as tmp:
        script = os.path.join(HERE, "golden", "make_reference_inputs.py")
        src = open(script).read().replace('HERE = os.path.dirname(os.path.abspath(__file__))',
                                          f'HERE = {tmp!r}')
        tmp_script = os.path.join(tmp, "make.py")
        open(tmp_script, "w").write(src)
        subprocess.run([sys.executable, tmp_script, REF_DIR], check=True, capture_output=True)
        a, b = np.load(os.path.join(tmp, "reference_inputs.npz")), fixture()
        for k in b.files:
            assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("case", range(83))
def test_classification_two_restatements(oracle_mod, case):
    name, nat, _, _ = boxes()[case]
    inter = oracle_mod.detect_interfacial(nat).astype(bool)
    assert np.array_equal(inter, npo.detect_interfacial(nat)), name
    assert (nat == 0).any()


@pytest.mark.parametrize("case", [0, 1, 2, 3, 40, 82])
def test_flow_two_restatements(oracle_mod, case):
    """300 steps of the reference loop (force on from the first convergence) in both."""
    name, nat, tau, f_ext = boxes()[case]
    ref = oracle_mod.equilibration(nat, tau=tau, f_ext=f_ext, max_steps=300, check=False)
    got = npo.equilibration(nat, tau=tau, f_ext=f_ext, max_steps=300)
    assert got["steps"] == ref["steps"]
    assert np.array_equal(got["l2err"], ref["l2err"])
    assert np.array_equal(got["n"], ref["n"])


# ------------------------------------------------------------------------------------ GPU

@pytest.mark.gpu
def test_every_reference_input_on_the_gpu(oracle_mod):
    """Interfacial flags and node counts of every input, and the FP64 reference loop capped at
    300 steps (the state at the cap), bit-identical to the oracle."""
    from laboetie_gb300 import FP64, Box

    for name, nat, tau, f_ext in boxes():
        want = oracle_mod.detect_interfacial(nat)
        ref = oracle_mod.equilibration(nat, tau=tau, f_ext=f_ext, max_steps=300, check=False)
        with Box(nat, relaxation_time=tau, f_ext=f_ext, precision=FP64) as box:
            assert np.array_equal(box.interfacial(), want), name
            cnt = box.node_counts()
            assert cnt["fluid_interfacial"] == int(((nat == 0) & (want == 1)).sum()), name
            box.flow_init()
            steps, hist, rc = box.equilibration(max_steps=300, hist_cap=300, check=False)
            n, rho, j = box.flow_get()
        assert steps == ref["steps"], name
        assert np.array_equal(hist, ref["l2err"]), name
        assert np.array_equal(n, ref["n"]) and np.array_equal(rho, ref["rho"]), name
        assert all(np.array_equal(a, b) for a, b in zip(j, ref["j"])), name


@pytest.mark.gpu
@pytest.mark.parametrize("case", [0, 1, 3, 20, 45, 82])
def test_reference_inputs_converged_flow_on_the_gpu(oracle_mod, case):
    """The whole flow phase (two convergences at the default target 1e-10) of lb.in, geom.in and
    chromatography cells: exit step, l2err history and final state bit-identical."""
    from laboetie_gb300 import FP64, Box

    name, nat, tau, f_ext = boxes()[case]
    ref = oracle_mod.equilibration(nat, tau=tau, f_ext=f_ext, max_steps=400000)
    with Box(nat, relaxation_time=tau, f_ext=f_ext, precision=FP64) as box:
        box.flow_init()
        steps, hist = box.equilibration(max_steps=400000, hist_cap=400000)
        n, rho, j = box.flow_get()
    assert steps == ref["steps"], name
    assert np.array_equal(hist, ref["l2err"]), name
    assert np.array_equal(n, ref["n"]) and all(np.array_equal(a, b) for a, b in zip(j, ref["j"]))
