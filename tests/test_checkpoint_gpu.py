"""Checkpoint and resume of the tracer phase: lbgpu_mp_get, then lbgpu_mp_init + lbgpu_mp_set in a
fresh context.

The reference has no checkpoint (its tracer loop, drop_tracers.f90:40-49, runs to the end in one
process); the library's contract is that a run cut in two and resumed from the checkpoint is the
uninterrupted run: the VACF of every step, P and P_ads bit-identical, in every precision, with
and without adsorption, on a box that takes the FP32 slab step (32 x 32 x 32).  The flow moments
the tracer starts from are the same host arrays in all three contexts.
"""
import math

import numpy as np
import pytest

from laboetie_gb300 import FP32_DEV, FP64, FP64_FUSED, Box
from laboetie_gb300 import geometry as geo
from laboetie_gb300.lbgpu import LbgpuError

pytestmark = pytest.mark.gpu

F_EXT = (1e-5, 0.0, 0.0)


@pytest.fixture(scope="module")
def flow():
    nat = geo.porous_spheres(32, 4, 0.6, 11)
    with Box(nat, relaxation_time=1.0, f_ext=F_EXT, precision=FP64) as box:
        box.flow_init()
        box.flow_steps(400, force_on=True)
        _, rho, j = box.flow_get()
    return nat, rho, j


@pytest.mark.parametrize("ads", [False, True])
@pytest.mark.parametrize("prec", [FP64, FP64_FUSED, FP32_DEV])
def test_tracer_resumed_from_a_checkpoint_is_the_uninterrupted_run(flow, prec, ads):
    nat, rho, j = flow
    tr = dict(f_ext=F_EXT, Db=0.01, ka=0.01 * math.e, kd=0.01) if ads else dict(f_ext=F_EXT, Db=0.01)
    K = 150

    def box():
        b = Box(nat, relaxation_time=1.0, f_ext=F_EXT, precision=prec)
        b.mp_init(moments=(rho, j), **tr)
        return b

    with box() as b:
        v_full, conv = b.mp_propagate(2 * K)
        P_full, A_full = b.mp_get()
    assert not conv and len(v_full) == 2 * K
    with box() as b:
        v1, _ = b.mp_propagate(K)
        P, A = b.mp_get()
    with box() as b:
        b.mp_set(P, A if ads else None, it_next=K + 1)
        v2, _ = b.mp_propagate(K)
        P2, A2 = b.mp_get()
    assert np.array_equal(v1, v_full[:K]) and np.array_equal(v2, v_full[K:])
    assert np.array_equal(P2, P_full) and np.array_equal(A2, A_full)
    assert not np.array_equal(P2, P)   # the resumed steps did move P
    if ads:
        assert np.abs(A_full).sum() > 0


def test_mp_set_refusals(flow):
    nat, rho, j = flow
    with Box(nat, relaxation_time=1.0, f_ext=F_EXT, precision=FP64) as b:
        P = np.zeros(nat.shape + (3,))
        with pytest.raises(LbgpuError):   # no tracer state yet
            b.mp_set(P, None, it_next=1)
        b.mp_init(moments=(rho, j), f_ext=F_EXT, Db=0.01, ka=0.01 * math.e, kd=0.01)
        with pytest.raises(LbgpuError):   # adsorption without P_ads
            b.mp_set(P, None, it_next=1)
        with pytest.raises(LbgpuError):   # the reference's it starts at 1
            b.mp_set(P, P, it_next=0)
