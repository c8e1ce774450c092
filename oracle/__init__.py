"""CPU oracle for laboetie's lattice-Boltzmann hot path -- TEST INFRASTRUCTURE ONLY.

This package wraps ``lb_oracle.c`` (a plain-C restatement of the reference Fortran, built with
``-ffp-contract=off``) through ctypes.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import it, as the checker.  The product library never does.

Parity status: the reference ships no golden vectors and cannot be compiled where this was
written (no Fortran compiler), so the oracle is pinned by analytic known answers (Poiseuille
profile, mass conservation, diffusion coefficients, closed-form VACF(0)) and by the committed
fixtures in ``tests/golden/`` -- parity against the reference's own outputs is unpinned.

Array conventions follow the reference: Fortran column-major node order (x fastest), flow
populations ``n(x,y,z,l)``, tracer populations ``n(l,x,y,z)``.  Functions take and return numpy
arrays shaped ``(lz, ly, lx)`` for fields and ``(19, lz, ly, lx)`` for flow populations, which
is the same memory order.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "liblboracle.so")
_lib = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i8 = np.ctypeslib.ndpointer(dtype=np.int8, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_vp = C.c_void_p
_int = C.c_int
_d = C.c_double
_pi = C.POINTER(C.c_int)
_pd = C.POINTER(C.c_double)

ORC_ERRORS = {
    0: "ok", 1: "negative population", 2: "step cap reached", 3: "bad input",
    4: "remaining fraction below eps", 5: "not converged", 6: "flux sum not zero",
    7: "charge not conserved",
}


class OracleError(RuntimeError):
    def __init__(self, code, where):
        super().__init__(f"{where}: {ORC_ERRORS.get(code, code)} (code {code})")
        self.code = code


class MPState(C.Structure):
    _fields_ = [
        ("lx", _int), ("ly", _int), ("lz", _int),
        ("ka", _d), ("kd", _d), ("K", _d), ("Db", _d), ("Ds", _d), ("z", _d), ("lam", _d),
        ("consider_adsorption", _int),
        ("vacf", _d * 3),
        ("P_now", _pd), ("P_next", _pd), ("A_now", _pd), ("A_next", _pd),
        ("nthreads", _int),
        ("phi", _pd), ("E", _d * 3),
    ]


class FlowParams(C.Structure):
    _fields_ = [
        ("lx", _int), ("ly", _int), ("lz", _int),
        ("relaxation_time", _d), ("target_error", _d), ("f_ext", _d * 3),
        ("compensate_f_ext", _int), ("particle_diameter", _int), ("particle_coords", _int * 3),
        ("geometry_label", _int), ("max_steps", _int), ("fixed_steps", _int),
        ("nthreads", _int),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with make into oracle/_build/ and return the .so path."""
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < max(
        os.path.getmtime(os.path.join(_HERE, f)) for f in ("lb_oracle.c", "lb_oracle.h")
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _SO


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_SO)
        L.orc_lbm_tables.argtypes = [_vp] * 6
        L.orc_detect_interfacial.argtypes = [_int, _int, _int, _i8, _u8]
        L.orc_init_populations.argtypes = [_int, _int, _int, _i8, _d, _dp, _dp]
        L.orc_collide.argtypes = [_int, _int, _int, _i8, _d] + [_dp] * 8
        L.orc_bounce_back_stream.argtypes = [_int, _int, _int, _i8, _dp, _int]
        L.orc_moments.argtypes = [_int, _int, _int] + [_dp] * 8 + [_pd]
        L.orc_equilibration.argtypes = [C.POINTER(FlowParams), _i8] + [_dp] * 8 + [_vp, _int, _pi]
        L.orc_update_tracer_population.argtypes = [_int, _int, _int, _i8, _dp, _dp, _dp, _dp,
                                                   _pd, _d, _d, _pd, _dp]
        L.orc_mp_init.argtypes = [C.POINTER(MPState), _int, _int, _int, _i8, _u8, _dp, _dp,
                                  _d, _d, _d, _d, _d, _pd]
        L.orc_mp_propagate.argtypes = [C.POINTER(MPState), _int, _i8, _u8, _dp, _dp, _pd, _pi]
        L.orc_mp_free.argtypes = [C.POINTER(MPState)]
        L.orc_mp_init_charged.argtypes = [C.POINTER(MPState), _int, _int, _int, _i8, _u8, _dp, _dp,
                                          _d, _d, _d, _d, _dp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_charges_init.argtypes = [_int, _int, _int, _i8, _u8, _d, _d, _d, _int, _dp, _dp,
                                       _dp, _pd, _pd]
        L.orc_sor.argtypes = [_int, _int, _int, _d, _d, _dp, _dp, _dp, _pd, _pi]
        L.orc_sor_custom.argtypes = [_int, _int, _int, _d, _d, _dp, _dp, _dp, _pd, _d, _d, _int, _pi]
        L.orc_just_eq_smolu.argtypes = [_int, _int, _int, _i8, _dp, _dp, _dp, _d, _d, _d, _d,
                                        _int, _pi]
        L.orc_check_charge_equilibrium.argtypes = [_int] + [_dp] * 6 + [_pd]
        L.orc_charge_test.argtypes = [_int, _i8, _dp, _dp, _d, _pd, _pd]
        L.orc_pnp.argtypes = [_int, _int, _int, _i8, _d, _d, _d, _d, _d, _int, _dp, _dp, _dp,
                              _pd, _int, _pi, _pi]
        L.orc_profiles.argtypes = [_int, _int, _int] + [_dp] * 4 + [_int, _dp, _dp]
        L.orc_geometry.argtypes = [_int, _int, _int, _int, _vp, _vp]
        L.orc_profiles.restype = None
        L.orc_electrostatic_pot.argtypes = [_int, _int, _int, _dp, _vp, _dp]
        L.orc_electrostatic_pot.restype = None
        L.orc_comp_j.argtypes = [_int, _int, _int] + [_dp] * 4
        L.orc_comp_j.restype = None
        L.orc_smolu.argtypes = [_int, _int, _int, _i8, _dp, _dp, _dp, _d, _d, _int, _int, _vp,
                                _vp, _vp, _vp, _dp]
        L.orc_advect.argtypes = [_int, _int, _int, _i8] + [_dp] * 7 + [_vp, _vp]
        _lib = L
    return _lib


def _dims(nature):
    lz, ly, lx = nature.shape
    return lx, ly, lz


def _chk(code, where):
    if code:
        raise OracleError(code, where)


def tables():
    """D3Q19 tables of module_lbmodel.f90: c (19,3), inv, a0, a1, a2, delta."""
    c = np.zeros((19, 3), dtype=np.int32)
    inv = np.zeros(19, dtype=np.int32)
    a0, a1, a2, de = (np.zeros(19) for _ in range(4))
    lib().orc_lbm_tables(*(x.ctypes.data for x in (c, inv, a0, a1, a2, de)))
    return c, inv, a0, a1, a2, de


def detect_interfacial(nature):
    nature = np.ascontiguousarray(nature, dtype=np.int8)
    out = np.zeros(nature.shape, dtype=np.uint8)
    lib().orc_detect_interfacial(*_dims(nature), nature, out)
    return out


def init_populations(nature, svden=1.0):
    nature = np.ascontiguousarray(nature, dtype=np.int8)
    n = np.zeros((19,) + nature.shape)
    rho = np.zeros(nature.shape)
    lib().orc_init_populations(*_dims(nature), nature, svden, n, rho)
    return n, rho


def collide(nature, tau, n, rho, j, f):
    nature = np.ascontiguousarray(nature, dtype=np.int8)
    n = np.array(n, dtype=np.float64, order="C")
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (rho, j[0], j[1], j[2], f[0], f[1], f[2])]
    _chk(lib().orc_collide(*_dims(nature), nature, tau, n, *a), "collide")
    return n


def bounce_back_stream(nature, n, nthreads=1):
    nature = np.ascontiguousarray(nature, dtype=np.int8)
    n = np.array(n, dtype=np.float64, order="C")
    lib().orc_bounce_back_stream(*_dims(nature), nature, n, nthreads)
    return n


def moments(nature, n, f, j_old):
    """Returns (status, rho, (jx,jy,jz), l2err)."""
    shape = nature.shape
    rho = np.zeros(shape)
    jx, jy, jz = (np.array(x, dtype=np.float64, order="C") for x in j_old)
    err = C.c_double(0)
    fx, fy, fz = (np.ascontiguousarray(x, dtype=np.float64) for x in f)
    n = np.ascontiguousarray(n, dtype=np.float64)
    rc = lib().orc_moments(*_dims(nature), n, fx, fy, fz, rho, jx, jy, jz, C.byref(err))
    return rc, rho, (jx, jy, jz), err.value


def equilibration(nature, tau=1.0, target_error=1e-10, f_ext=(0.0, 0.0, 0.0), svden=1.0,
                  max_steps=0, fixed_steps=0, compensate_f_ext=False, particle_diameter=1,
                  particle_coords=(0, 0, 0), geometry_label=0, nthreads=1, hist_cap=None,
                  check=True):
    """Full flow phase of equilibration.f90 from the init_simu.f90 initial state.

    Returns dict(n, rho, j, f, steps, l2err, status); raises on a non-zero status if check."""
    nature = np.ascontiguousarray(nature, dtype=np.int8)
    lx, ly, lz = _dims(nature)
    n, rho = init_populations(nature, svden)
    jx, jy, jz, fx, fy, fz = (np.zeros(nature.shape) for _ in range(6))
    p = FlowParams(lx, ly, lz, tau, target_error, (C.c_double * 3)(*f_ext), int(compensate_f_ext),
                   particle_diameter, (C.c_int * 3)(*particle_coords), geometry_label, max_steps,
                   fixed_steps, nthreads)
    cap = hist_cap if hist_cap is not None else (max_steps or fixed_steps or 1 << 20)
    hist = np.zeros(cap)
    steps = C.c_int(0)
    rc = lib().orc_equilibration(C.byref(p), nature, n, rho, jx, jy, jz, fx, fy, fz,
                                 hist.ctypes.data, cap, C.byref(steps))
    if check:
        _chk(rc, "equilibration")
    return dict(n=n, rho=rho, j=(jx, jy, jz), f=(fx, fy, fz), steps=steps.value,
                l2err=hist[: min(steps.value, cap)], status=rc)


def update_tracer_population(nature, rho, j, f_ext, tracer_z=0.0, tracer_D=0.0,
                             elec_slope=(0.0, 0.0, 0.0)):
    nature = np.ascontiguousarray(nature, dtype=np.int8)
    nmp = np.zeros(nature.shape + (19,))
    fe = (C.c_double * 3)(*f_ext)
    es = (C.c_double * 3)(*elec_slope)
    jx, jy, jz = (np.ascontiguousarray(x, dtype=np.float64) for x in j)
    lib().orc_update_tracer_population(*_dims(nature), nature, np.ascontiguousarray(rho), jx, jy,
                                       jz, fe, tracer_z, tracer_D, es, nmp)
    return nmp


class MomentPropagation:
    """module_moment_propagation.f90 init/propagate on the CPU."""

    def __init__(self, nature, interfacial, rho, n_mp, ka=0.0, kd=0.0, Db=0.01, Ds=0.0, z=0.0,
                 nthreads=1, phi=None, elec_slope=(0.0, 0.0, 0.0)):
        """phi (same shape as nature) with z != 0: a charged tracer (orc_mp_init_charged)."""
        self.nature = np.ascontiguousarray(nature, dtype=np.int8)
        self.inter = np.ascontiguousarray(interfacial, dtype=np.uint8)
        self.rho = np.ascontiguousarray(rho, dtype=np.float64)
        self.nmp = np.ascontiguousarray(n_mp, dtype=np.float64)
        self.s = MPState()
        v0 = (C.c_double * 3)()
        if phi is None:
            rc = lib().orc_mp_init(C.byref(self.s), *_dims(self.nature), self.nature, self.inter,
                                   self.rho, self.nmp, ka, kd, Db, Ds, z, v0)
        else:
            self.phi = np.ascontiguousarray(phi, dtype=np.float64)
            E = (C.c_double * 3)(*elec_slope)
            rc = lib().orc_mp_init_charged(C.byref(self.s), *_dims(self.nature), self.nature,
                                           self.inter, self.rho, self.nmp, ka, kd, Db, z,
                                           self.phi, E, v0)
        _chk(rc, "mp_init")
        self.s.nthreads = nthreads
        self.vacf0 = np.array(list(v0))
        self.N = self.nature.size

    def propagate(self, it):
        v = (C.c_double * 3)()
        conv = C.c_int(0)
        rc = lib().orc_mp_propagate(C.byref(self.s), it, self.nature, self.inter, self.rho,
                                    self.nmp, v, C.byref(conv))
        _chk(rc, "mp_propagate")
        return np.array(list(v)), bool(conv.value)

    def P(self):
        return np.ctypeslib.as_array(self.s.P_now, shape=(self.N * 3,)).copy()

    def Pads(self):
        if not self.s.consider_adsorption:
            return None
        return np.ctypeslib.as_array(self.s.A_now, shape=(self.N * 3,)).copy()

    def close(self):
        if self.s.P_now:
            lib().orc_mp_free(C.byref(self.s))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def charges_init(nature, interfacial, bjl, sigma, lambda_D, charge_distrib="int"):
    nature = np.ascontiguousarray(nature, dtype=np.int8)
    cp, cm, phi = (np.zeros(nature.shape) for _ in range(3))
    an, rc_ = C.c_double(0), C.c_double(0)
    rc = lib().orc_charges_init(*_dims(nature), nature,
                                np.ascontiguousarray(interfacial, dtype=np.uint8), bjl, sigma,
                                lambda_D, int(charge_distrib[:3] == "int"), cp, cm, phi,
                                C.byref(an), C.byref(rc_))
    _chk(rc, "charges_init")
    return cp, cm, phi, an.value, rc_.value


def sor(nature, sigma, bjl, cp, cm, phi, anormf0, omega=None, tol=None, maxiter=500000):
    phi = np.array(phi, dtype=np.float64, order="C")
    an = C.c_double(anormf0)
    it = C.c_int(0)
    lx, ly, lz = _dims(nature)
    cp = np.ascontiguousarray(cp)
    cm = np.ascontiguousarray(cm)
    if omega is None and tol is None:
        rc = lib().orc_sor(lx, ly, lz, sigma, bjl, cp, cm, phi, C.byref(an), C.byref(it))
    else:
        rc = lib().orc_sor_custom(lx, ly, lz, sigma, bjl, cp, cm, phi, C.byref(an),
                                  1.4 if omega is None else omega,
                                  float(np.float32(1e-5)) if tol is None else tol, maxiter,
                                  C.byref(it))
    _chk(rc, "sor")
    return phi, an.value, it.value


def just_eq_smolu(nature, phi, cp, cm, D_plus, D_minus, rho_ch, sigma, loop_bug=True):
    nature = np.ascontiguousarray(nature, dtype=np.int8)
    cp = np.array(cp, dtype=np.float64, order="C")
    cm = np.array(cm, dtype=np.float64, order="C")
    it = C.c_int(0)
    rc = lib().orc_just_eq_smolu(*_dims(nature), nature, np.ascontiguousarray(phi), cp, cm,
                                 D_plus, D_minus, rho_ch, sigma, int(loop_bug), C.byref(it))
    _chk(rc, "just_eq_smolu")
    return cp, cm, it.value


def charge_test(nature, cp, cm, sigma):
    s, f = C.c_double(0), C.c_double(0)
    rc = lib().orc_charge_test(nature.size, np.ascontiguousarray(nature, dtype=np.int8),
                               np.ascontiguousarray(cp), np.ascontiguousarray(cm), sigma,
                               C.byref(s), C.byref(f))
    return rc, s.value, f.value


def pnp(nature, bjl, sigma, D_plus, D_minus, rho_ch, cp, cm, phi, anormf0, loop_bug=True,
        max_outer=10000, check=True):
    nature = np.ascontiguousarray(nature, dtype=np.int8)
    cp = np.array(cp, dtype=np.float64, order="C")
    cm = np.array(cm, dtype=np.float64, order="C")
    phi = np.array(phi, dtype=np.float64, order="C")
    an = C.c_double(anormf0)
    outer, tot = C.c_int(0), C.c_int(0)
    rc = lib().orc_pnp(*_dims(nature), nature, bjl, sigma, D_plus, D_minus, rho_ch,
                       int(loop_bug), cp, cm, phi, C.byref(an), max_outer, C.byref(outer),
                       C.byref(tot))
    if check:
        _chk(rc, "pnp")
    return dict(c_plus=cp, c_minus=cm, phi=phi, anormf0=an.value, outer=outer.value,
                sor_iters=tot.value, status=rc)


def electrostatic_pot(phi, elec_slope):
    lz, ly, lx = phi.shape
    out = np.zeros(phi.shape)
    lib().orc_electrostatic_pot(lx, ly, lz, np.ascontiguousarray(phi, dtype=np.float64),
                                (C.c_double * 3)(*elec_slope), out)
    return out


def comp_j(n, j):
    lz, ly, lx = n.shape[1:]
    jj = [np.array(x, dtype=np.float64, order="C") for x in j]
    lib().orc_comp_j(lx, ly, lz, np.ascontiguousarray(n, dtype=np.float64), *jj)
    return tuple(jj)


def smolu(nature, phi_tot, cp, cm, D_plus, D_minus, time, D_iter, elec_slope, lncb_slope,
          el_curr, ion_curr, solute_force):
    """smolu.f90; returns (status, c+, c-, el_curr, ion_curr, solute_force)."""
    nature = np.ascontiguousarray(nature, dtype=np.int8)
    cp = np.array(cp, dtype=np.float64, order="C")
    cm = np.array(cm, dtype=np.float64, order="C")
    el = (C.c_double * 3)(*el_curr)
    io = (C.c_double * 3)(*ion_curr)
    sf = np.array(solute_force, dtype=np.float64, order="C")
    rc = lib().orc_smolu(*_dims(nature), nature, np.ascontiguousarray(phi_tot), cp, cm, D_plus,
                         D_minus, time, D_iter, (C.c_double * 3)(*elec_slope),
                         (C.c_double * 3)(*lncb_slope), el, io, sf)
    return rc, cp, cm, np.array(list(el)), np.array(list(io)), sf


def advect(nature, j, cp, cm, fp, fm, el_curr, ion_curr):
    """advect.f90; fp, fm: the flux_site arrays carried between calls (updated in place).
    Returns (status, c+, c-, el_curr, ion_curr)."""
    nature = np.ascontiguousarray(nature, dtype=np.int8)
    cp = np.array(cp, dtype=np.float64, order="C")
    cm = np.array(cm, dtype=np.float64, order="C")
    el = (C.c_double * 3)(*el_curr)
    io = (C.c_double * 3)(*ion_curr)
    jx, jy, jz = (np.ascontiguousarray(x, dtype=np.float64) for x in j)
    rc = lib().orc_advect(*_dims(nature), nature, jx, jy, jz, cp, cm, fp, fm, el, io)
    return rc, cp, cm, np.array(list(el)), np.array(list(io))


def profiles(nature, rho, j, axis):
    """equilibration.f90:159-175: (flux (L, 3), mean density (L,)) per plane normal to axis."""
    lx, ly, lz = _dims(nature)
    L = (lx, ly, lz)[axis]
    arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (rho, *j)]
    flux = np.zeros((L, 3))
    dens = np.zeros(L)
    lib().orc_profiles(lx, ly, lz, *arrs, axis, flux, dens)
    return flux, dens


def geometry(label, lx, ly, lz, params=None):
    """module_geometry.f90 builder of geometryLabel `label`: (code, nature (lz, ly, lx) int8);
    code 0, or 1 shape / 2 parameters / 3 label / 4 no fluid node (the reference's STOPs)."""
    nat = np.zeros((lz, ly, lx), dtype=np.int8)
    p = None if params is None else np.ascontiguousarray(params, dtype=np.float64)
    code = lib().orc_geometry(label, lx, ly, lz, None if p is None else p.ctypes.data, nat.ctypes.data)
    return code, nat
