"""FP32-deviation storage against the FP64 strict path: the error of each result the precision
mode is used for (permeability, effective diffusion coefficient, adsorbed fraction of the
propagated quantity and at equilibrium, retention time), on a small porous medium.  Tolerance:
1e-5 relative for each (the measured errors are recorded in the design notes)."""
import math

import numpy as np
import pytest

from laboetie_gb300 import geometry as geo
from laboetie_gb300.lbgpu import FP32_DEV, FP64, Box

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _results(nat, prec, tau, fe, K, KM, tracer):
    with Box(nat, relaxation_time=tau, f_ext=fe, precision=prec) as box:
        box.flow_init()
        box.flow_steps(K, force_on=True)
        _, rho, j = box.flow_get(populations=False)
        v0 = box.mp_init(f_ext=fe, **tracer)
        vac, _ = box.mp_propagate(KM)
        P, A = box.mp_get()
        c = box.node_counts()
    fl = nat == 0
    nu = (tau - 0.5) / 3.0
    kk = tracer["ka"] / tracer["kd"]
    ads = kk * c["fluid_interfacial"] / (c["fluid"] + kk * c["fluid_interfacial"])
    ux = j[0][fl].sum() / rho[fl].sum()
    return dict(permeability=nu * j[0].sum() / nat.size / fe[0],
                d_eff=v0[0] / 2 + vac[:, 0].sum(),
                adsorbed_fraction=A[..., 0].sum() / (P[..., 0].sum() + A[..., 0].sum()),
                equilibrium_adsorbed_fraction=ads,
                retention_time=nat.shape[2] / ((1 - ads) * ux))


def test_fp32_error_statement_porous():
    nat = geo.porous_spheres(L=40, radius=5.0, porosity=0.6, seed=9)
    tracer = dict(Db=0.01, ka=0.01 * math.exp(2.0), kd=0.01)
    r64 = _results(nat, FP64, 0.8, (1e-6, 0.0, 0.0), 6000, 3000, tracer)
    r32 = _results(nat, FP32_DEV, 0.8, (1e-6, 0.0, 0.0), 6000, 3000, tracer)
    for k in r64:
        rel = abs(r32[k] - r64[k]) / abs(r64[k])
        assert rel <= TOL, (k, rel, r32[k], r64[k])
