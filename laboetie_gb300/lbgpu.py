"""ctypes binding of liblbgpu (include/lbgpu.h) and a Box class mirroring the reference calls.

Arrays use the reference's memory order: a field f(lx,ly,lz) is a numpy array of shape
(lz, ly, lx) (x fastest), flow populations n(lx,ly,lz,19) are (19, lz, ly, lx) and tracer
quantities P(3,lx,ly,lz) are (lz, ly, lx, 3).  Every call goes to the GPU library; a non-zero
status raises LbgpuError with the library's message.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(HERE, "_build", "liblbgpu.so")

FP64 = 0
FP32_DEV = 1
FP64_FUSED = 2

STATUS = {
    1 << 0: "invalid argument", 1 << 1: "CUDA error", 1 << 2: "negative population",
    1 << 3: "non-finite value", 1 << 4: "remaining fraction below eps", 1 << 5: "step cap",
    1 << 6: "out of device memory", 1 << 7: "flux sum not zero", 1 << 8: "charge not conserved",
    1 << 9: "unsupported", 1 << 10: "device wait timed out",
}
ERR_NEGATIVE_POPULATION = 1 << 2
ERR_NONFINITE = 1 << 3
ERR_FRACTION = 1 << 4
ERR_STEP_CAP = 1 << 5
ERR_OOM = 1 << 6


class LbgpuError(RuntimeError):
    def __init__(self, status: int, message: str):
        names = [v for k, v in STATUS.items() if status & k]
        super().__init__(f"{message} [status {status}: {', '.join(names)}]")
        self.status = status


class Params(C.Structure):
    """lbgpu_params (include/lbgpu.h)."""
    _fields_ = [
        ("lx", C.c_int), ("ly", C.c_int), ("lz", C.c_int), ("precision", C.c_int),
        ("relaxation_time", C.c_double), ("target_error", C.c_double),
        ("f_ext", C.c_double * 3), ("rho0", C.c_double), ("device", C.c_int),
    ]


class Tracer(C.Structure):
    """lbgpu_tracer (include/lbgpu.h): the lb.in tracer tags of drop_tracers.f90 and
    module_moment_propagation.f90."""
    _fields_ = [
        ("Db", C.c_double), ("ka", C.c_double), ("kd", C.c_double), ("Ds", C.c_double),
        ("z", C.c_double), ("f_ext", C.c_double * 3), ("elec_slope", C.c_double * 3),
    ]


class PnpParams(C.Structure):
    """lbgpu_pnp_params (include/lbgpu.h)."""
    _fields_ = [
        ("bjl", C.c_double), ("sigma", C.c_double), ("lambda_D", C.c_double),
        ("D_plus", C.c_double), ("D_minus", C.c_double), ("charge_distrib", C.c_int),
        ("solver", C.c_int), ("omega", C.c_double), ("tol", C.c_double), ("max_iter", C.c_int),
        ("np_loop_bug", C.c_int),
    ]


_lib = None


def library_path() -> str:
    return _LIB_PATH


def library():
    """Load liblbgpu.so (building it first if it is missing).  Raises if it cannot be loaded."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        from . import build as _build

        _build.build()
    L = C.CDLL(_LIB_PATH)
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    pi = C.POINTER(C.c_int)
    L.lbgpu_default_params.argtypes = [C.POINTER(Params), i, i, i]
    L.lbgpu_default_params.restype = None
    L.lbgpu_create.argtypes = [C.POINTER(Params), vp, C.POINTER(vp)]
    L.lbgpu_destroy.argtypes = [vp]
    L.lbgpu_destroy.restype = None
    L.lbgpu_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    L.lbgpu_interfacial.argtypes = [vp, vp]
    L.lbgpu_node_counts.argtypes = [vp, vp]
    L.lbgpu_flow_init.argtypes = [vp]
    L.lbgpu_flow_set.argtypes = [vp] * 6
    L.lbgpu_flow_get.argtypes = [vp] * 6
    L.lbgpu_collide.argtypes = [vp] * 9
    L.lbgpu_bounce_back_stream.argtypes = [vp, vp]
    L.lbgpu_moments.argtypes = [vp] * 10
    L.lbgpu_equilibration.argtypes = [vp, i, vp, i, pi]
    L.lbgpu_flow_steps.argtypes = [vp, i, i]
    L.lbgpu_time_flow_steps.argtypes = [vp, i, i, C.POINTER(C.c_float)]
    L.lbgpu_sync.argtypes = [vp]
    L.lbgpu_host_register.argtypes = [vp, C.c_size_t]
    L.lbgpu_host_unregister.argtypes = [vp]
    for name, args in (
        ("lbgpu_mp_init", [vp, C.POINTER(Tracer), vp, vp, vp, vp, vp]),
        ("lbgpu_mp_init_charged", [vp, C.POINTER(Tracer), vp, vp, vp, vp, vp]),
        ("lbgpu_mp_propagate", [vp, i, vp, pi, pi]),
        ("lbgpu_mp_get", [vp, vp, vp]),
        ("lbgpu_mp_set", [vp, vp, vp, i]),
        ("lbgpu_mp_release", [vp]),
        ("lbgpu_time_mp_steps", [vp, i, C.POINTER(C.c_float)]),
        ("lbgpu_pnp_init", [vp, C.POINTER(PnpParams), C.POINTER(d)]),
        ("lbgpu_pnp_set", [vp, vp, vp, vp, d]),
        ("lbgpu_pnp_get", [vp, vp, vp, vp, C.POINTER(d)]),
        ("lbgpu_sor", [vp, pi]),
        ("lbgpu_just_eq_smolu", [vp, pi]),
        ("lbgpu_poisson_nernst_planck", [vp, i, pi, pi]),
        ("lbgpu_charge_test", [vp, C.POINTER(d), C.POINTER(d)]),
        ("lbgpu_poisson_residual", [vp, C.POINTER(d), C.POINTER(d)]),
        ("lbgpu_electrostatic_pot", [vp, vp]),
        ("lbgpu_comp_j", [vp, vp, vp, vp, vp]),
        ("lbgpu_smolu", [vp, i, i, vp, vp, vp, vp]),
        ("lbgpu_advect", [vp, vp, vp, vp, vp, vp]),
        ("lbgpu_ek_get", [vp, vp, vp]),
        ("lbgpu_moments_noalloc", [i, i, i] + [vp] * 8 + [C.POINTER(d), vp]),
        ("lbgpu_compensated_force_field", [vp, i, vp, i, vp, vp, vp]),
        ("lbgpu_set_force_field", [vp, vp, vp, vp]),
        ("lbgpu_profiles", [vp, i, vp, vp]),
        ("lbgpu_geometry", [i, i, i, i, i, vp, vp]),
        ("lbgpu_create_label", [C.POINTER(Params), i, vp, C.POINTER(vp)]),
    ):
        if hasattr(L, name):
            getattr(L, name).argtypes = args
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data


def _f64(a, shape):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.shape != shape:
        a = a.reshape(shape)
    return a


class Box:
    """One simulation box on the GPU (an lbgpu context).

    ``nature`` is an int8 array of shape (lz, ly, lx) with 0 = fluid, 1 = solid.
    """

    def __init__(self, nature, relaxation_time=1.0, f_ext=(0.0, 0.0, 0.0), target_error=1e-10,
                 rho0=1.0, precision=FP64, device=0):
        self.L = library()
        nature = np.ascontiguousarray(nature, dtype=np.int8)
        if nature.ndim != 3:
            raise ValueError("nature must be (lz, ly, lx)")
        lz, ly, lx = nature.shape
        self._setup(lx, ly, lz, relaxation_time, f_ext, target_error, rho0, precision, device)
        rc = self.L.lbgpu_create(C.byref(self.params), nature.ctypes.data, C.byref(self.ctx))
        if rc:
            raise LbgpuError(rc, self._msg(None))
        self.nature = nature

    @classmethod
    def from_label(cls, label, lx, ly, lz, params=None, relaxation_time=1.0, f_ext=(0.0, 0.0, 0.0),
                   target_error=1e-10, rho0=1.0, precision=FP64, device=0):
        """A box of the reference's geometryLabel `label` built on the device
        (lbgpu_create_label); params: (lw_o_lx, a_o_R) for label 7."""
        self = cls.__new__(cls)
        self.L = library()
        self._setup(lx, ly, lz, relaxation_time, f_ext, target_error, rho0, precision, device)
        par = None if params is None else (C.c_double * len(params))(*params)
        rc = self.L.lbgpu_create_label(C.byref(self.params), label, par, C.byref(self.ctx))
        if rc:
            raise LbgpuError(rc, self._msg(None))
        self.nature = device_geometry(label, lx, ly, lz, params, device)
        return self

    def _setup(self, lx, ly, lz, relaxation_time, f_ext, target_error, rho0, precision, device):
        self.shape = (lz, ly, lx)
        self.N = lx * ly * lz
        p = Params()
        self.L.lbgpu_default_params(C.byref(p), lx, ly, lz)
        p.relaxation_time = relaxation_time
        p.target_error = target_error
        p.f_ext = (C.c_double * 3)(*f_ext)
        p.rho0 = rho0
        p.precision = precision
        p.device = device
        self.params = p
        self.ctx = C.c_void_p()

    # -------------------------------------------------------------- helpers
    def _msg(self, ctx):
        buf = C.create_string_buffer(1024)
        self.L.lbgpu_last_error(ctx, buf, 1024)
        return buf.value.decode(errors="replace")

    def _chk(self, rc, what=""):
        if rc:
            raise LbgpuError(rc, f"{what}: {self._msg(self.ctx)}")

    def close(self):
        if getattr(self, "ctx", None):
            self.L.lbgpu_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -------------------------------------------------------------- geometry
    def interfacial(self):
        out = np.zeros(self.shape, dtype=np.uint8)
        self._chk(self.L.lbgpu_interfacial(self.ctx, out.ctypes.data), "interfacial")
        return out

    def node_counts(self):
        c = (C.c_longlong * 4)()
        self._chk(self.L.lbgpu_node_counts(self.ctx, c), "node_counts")
        return dict(fluid=c[0], solid=c[1], fluid_interfacial=c[2], solid_interfacial=c[3])

    # -------------------------------------------------------------- flow state
    def flow_init(self):
        self._chk(self.L.lbgpu_flow_init(self.ctx), "flow_init")

    def flow_set(self, n, rho, j):
        pshape = (19,) + self.shape
        n = _f64(n, pshape)
        rho = _f64(rho, self.shape)
        jx, jy, jz = (_f64(x, self.shape) for x in j)
        self._chk(self.L.lbgpu_flow_set(self.ctx, _ptr(n), _ptr(rho), _ptr(jx), _ptr(jy), _ptr(jz)),
                  "flow_set")

    def flow_get(self, populations=True):
        n = np.zeros((19,) + self.shape) if populations else None
        rho = np.zeros(self.shape)
        j = [np.zeros(self.shape) for _ in range(3)]
        self._chk(self.L.lbgpu_flow_get(self.ctx, _ptr(n), _ptr(rho), *(_ptr(x) for x in j)),
                  "flow_get")
        return n, rho, tuple(j)

    # -------------------------------------------------------------- reference operators
    def collide(self, n, rho, j, f):
        """module_collision.f90 collide(n, density, jx, jy, jz, f_ext_x, f_ext_y, f_ext_z)."""
        n = np.array(n, dtype=np.float64, order="C").reshape((19,) + self.shape)
        a = [_f64(x, self.shape) for x in (rho, *j, *f)]
        self._chk(self.L.lbgpu_collide(self.ctx, _ptr(n), *(_ptr(x) for x in a)), "collide")
        return n

    def bounce_back_stream(self, n):
        """equilibration.f90:204-243."""
        n = np.array(n, dtype=np.float64, order="C").reshape((19,) + self.shape)
        self._chk(self.L.lbgpu_bounce_back_stream(self.ctx, _ptr(n)), "bounce_back_stream")
        return n

    def moments(self, n, f, j_old):
        """equilibration.f90:248-343: returns (status, rho, j, l2err)."""
        n = _f64(n, (19,) + self.shape)
        f = [_f64(x, self.shape) for x in f]
        j = [np.array(x, dtype=np.float64, order="C").reshape(self.shape) for x in j_old]
        rho = np.zeros(self.shape)
        err = C.c_double(0)
        rc = self.L.lbgpu_moments(self.ctx, _ptr(n), *(_ptr(x) for x in f), _ptr(rho),
                                  *(_ptr(x) for x in j), C.byref(err))
        if rc & ~(ERR_NEGATIVE_POPULATION | ERR_NONFINITE):
            self._chk(rc, "moments")
        return rc, rho, tuple(j), err.value

    # -------------------------------------------------------------- device loop
    def equilibration(self, max_steps=0, hist_cap=0, check=True):
        """equilibration.f90:143-491 on the device.  Returns (steps, l2err history), or
        (steps, history, status) when check is False (the state stays readable after an error)."""
        hist = np.zeros(hist_cap) if hist_cap else None
        steps = C.c_int(0)
        rc = self.L.lbgpu_equilibration(self.ctx, max_steps, _ptr(hist), hist_cap, C.byref(steps))
        h = hist[: min(steps.value, hist_cap)] if hist is not None else None
        if not check:
            return steps.value, h, rc
        self._chk(rc, "equilibration")
        return steps.value, h

    def flow_steps(self, nsteps, force_on=True):
        self._chk(self.L.lbgpu_flow_steps(self.ctx, nsteps, int(force_on)), "flow_steps")

    def time_flow_steps(self, nsteps, force_on=True):
        ms = C.c_float(0)
        self._chk(self.L.lbgpu_time_flow_steps(self.ctx, nsteps, int(force_on), C.byref(ms)),
                  "time_flow_steps")
        return ms.value

    def sync(self):
        self._chk(self.L.lbgpu_sync(self.ctx), "sync")


def _tracer(Db=0.01, ka=0.0, kd=0.0, Ds=0.0, z=0.0, f_ext=(0.0, 0.0, 0.0),
            elec_slope=(0.0, 0.0, 0.0)):
    t = Tracer()
    t.Db, t.ka, t.kd, t.Ds, t.z = Db, ka, kd, Ds, z
    t.f_ext = (C.c_double * 3)(*f_ext)
    t.elec_slope = (C.c_double * 3)(*elec_slope)
    return t


def _mp_init(self, moments=None, charged=False, **tracer):
    """update_tracer_population + moment_propagation::init.  moments = (rho, (jx, jy, jz)) as
    host arrays, or None for the box's own flow state.  charged=True: lbgpu_mp_init_charged (a
    tracer with z != 0 in the box's Poisson-Nernst-Planck potential).  Returns VACF(0)."""
    t = _tracer(**tracer)
    v0 = (C.c_double * 3)()
    init = self.L.lbgpu_mp_init_charged if charged else self.L.lbgpu_mp_init
    if moments is None:
        rc = init(self.ctx, C.byref(t), None, None, None, None, v0)
    else:
        rho, j = moments
        arrs = [_f64(rho, self.shape)] + [_f64(x, self.shape) for x in j]
        rc = init(self.ctx, C.byref(t), *(_ptr(x) for x in arrs), v0)
    self._chk(rc, "mp_init")
    return np.array(list(v0))


def _mp_propagate(self, nsteps):
    """Returns (vacf (steps,3), converged)."""
    v = np.zeros((max(nsteps, 1), 3))
    done, conv = C.c_int(0), C.c_int(0)
    rc = self.L.lbgpu_mp_propagate(self.ctx, nsteps, _ptr(v), C.byref(done), C.byref(conv))
    self._chk(rc, "mp_propagate")
    return v[: done.value], bool(conv.value)


def _mp_get(self):
    P = np.zeros(self.shape + (3,))
    A = np.zeros(self.shape + (3,))
    self._chk(self.L.lbgpu_mp_get(self.ctx, _ptr(P), _ptr(A)), "mp_get")
    return P, A


def _mp_set(self, P, P_ads=None, it_next=1):
    """Resume the tracer phase from (P, P_ads) as mp_get returned them, the next step being the
    reference's step it_next (after mp_init with the same tracer on the same flow)."""
    P = np.ascontiguousarray(P, dtype=np.float64).reshape(self.shape + (3,))
    A = None if P_ads is None else np.ascontiguousarray(P_ads, dtype=np.float64).reshape(self.shape + (3,))
    self._chk(self.L.lbgpu_mp_set(self.ctx, _ptr(P), _ptr(A) if A is not None else None, int(it_next)),
              "mp_set")


def _time_mp_steps(self, nsteps):
    ms = C.c_float(0)
    self._chk(self.L.lbgpu_time_mp_steps(self.ctx, nsteps, C.byref(ms)), "time_mp_steps")
    return ms.value


Box.mp_init = _mp_init
Box.mp_propagate = _mp_propagate
Box.mp_get = _mp_get
Box.mp_set = _mp_set
Box.time_mp_steps = _time_mp_steps
Box.mp_release = lambda self: self._chk(self.L.lbgpu_mp_release(self.ctx), "mp_release")


POISSON_REFERENCE = 0
POISSON_SOR4 = 1
POISSON_JACOBI = 2


def _pnp_init(self, bjl=0.4, sigma=0.0, lambda_D=4.0, D_plus=0.05, D_minus=0.05,
              charge_distrib="int", solver=POISSON_REFERENCE, omega=1.8, tol=1e-10, max_iter=0,
              np_loop_bug=True):
    """charges_init.f90 on the device; returns anormf0."""
    p = PnpParams()
    p.bjl, p.sigma, p.lambda_D, p.D_plus, p.D_minus = bjl, sigma, lambda_D, D_plus, D_minus
    p.charge_distrib = 0 if charge_distrib[:3] == "int" else 1
    p.solver, p.omega, p.tol, p.max_iter, p.np_loop_bug = solver, omega, tol, max_iter, int(np_loop_bug)
    an = C.c_double(0)
    self._chk(self.L.lbgpu_pnp_init(self.ctx, C.byref(p), C.byref(an)), "pnp_init")
    return an.value


def _pnp_get(self):
    cp, cm, phi = (np.zeros(self.shape) for _ in range(3))
    an = C.c_double(0)
    self._chk(self.L.lbgpu_pnp_get(self.ctx, _ptr(cp), _ptr(cm), _ptr(phi), C.byref(an)), "pnp_get")
    return cp, cm, phi, an.value


def _pnp_set(self, cp, cm, phi, anormf0):
    a = [_f64(x, self.shape) for x in (cp, cm, phi)]
    self._chk(self.L.lbgpu_pnp_set(self.ctx, *(_ptr(x) for x in a), C.c_double(anormf0)), "pnp_set")


def _sor(self):
    it = C.c_int(0)
    self._chk(self.L.lbgpu_sor(self.ctx, C.byref(it)), "sor")
    return it.value


def _just_eq_smolu(self):
    it = C.c_int(0)
    self._chk(self.L.lbgpu_just_eq_smolu(self.ctx, C.byref(it)), "just_eq_smolu")
    return it.value


def _pnp(self, max_outer=0, check=True):
    o, t = C.c_int(0), C.c_int(0)
    rc = self.L.lbgpu_poisson_nernst_planck(self.ctx, max_outer, C.byref(o), C.byref(t))
    if not check:
        return o.value, t.value, rc
    self._chk(rc, "poisson_nernst_planck")
    return o.value, t.value


def _poisson_residual(self):
    """(sum |phi* - phi| at the current phi, anormf0)."""
    r, an = C.c_double(0), C.c_double(0)
    self._chk(self.L.lbgpu_poisson_residual(self.ctx, C.byref(r), C.byref(an)), "poisson_residual")
    return r.value, an.value


def _charge_test(self):
    s, f = C.c_double(0), C.c_double(0)
    rc = self.L.lbgpu_charge_test(self.ctx, C.byref(s), C.byref(f))
    return rc, s.value, f.value


def _electrostatic_pot(self, elec_slope=(0.0, 0.0, 0.0)):
    """electrostatic_pot.f90: phi_tot from the box's phi and elec_slope (kept on the device)."""
    self._chk(self.L.lbgpu_electrostatic_pot(self.ctx, (C.c_double * 3)(*elec_slope)),
              "electrostatic_pot")


def _comp_j(self, n, j):
    """comp_j.f90: returns j = 0.5*(j + sum_l n_l c_l)."""
    n = _f64(n, (19,) + self.shape)
    jj = [np.array(x, dtype=np.float64, order="C").reshape(self.shape) for x in j]
    self._chk(self.L.lbgpu_comp_j(self.ctx, _ptr(n), *(_ptr(x) for x in jj)), "comp_j")
    return tuple(jj)


def _smolu(self, time=0, D_iter=-1, elec_slope=(0.0, 0.0, 0.0), lncb_slope=(0.0, 0.0, 0.0),
           el_curr=(0.0, 0.0, 0.0), ion_curr=(0.0, 0.0, 0.0), check=True):
    """smolu.f90 on the box's c+, c-, phi_tot; returns (el_curr, ion_curr), or
    (el_curr, ion_curr, status) when check is False."""
    el, io = (C.c_double * 3)(*el_curr), (C.c_double * 3)(*ion_curr)
    rc = self.L.lbgpu_smolu(self.ctx, int(time), int(D_iter), (C.c_double * 3)(*elec_slope),
                            (C.c_double * 3)(*lncb_slope), el, io)
    out = (np.array(list(el)), np.array(list(io)))
    if not check:
        return out + (rc,)
    self._chk(rc, "smolu")
    return out


def _advect(self, j, el_curr=(0.0, 0.0, 0.0), ion_curr=(0.0, 0.0, 0.0), check=True):
    """advect.f90 of the box's c+, c- by the solvent flux j; returns (el_curr, ion_curr), or
    (el_curr, ion_curr, status) when check is False."""
    jj = [_f64(x, self.shape) for x in j]
    el, io = (C.c_double * 3)(*el_curr), (C.c_double * 3)(*ion_curr)
    rc = self.L.lbgpu_advect(self.ctx, *(_ptr(x) for x in jj), el, io)
    out = (np.array(list(el)), np.array(list(io)))
    if not check:
        return out + (rc,)
    self._chk(rc, "advect")
    return out


def _ek_get(self):
    """(phi_tot, solute_force shaped (3, lz, ly, lx))."""
    phi_tot = np.zeros(self.shape)
    sf = np.zeros((3,) + self.shape)
    self._chk(self.L.lbgpu_ek_get(self.ctx, _ptr(phi_tot), _ptr(sf)), "ek_get")
    return phi_tot, sf


Box.electrostatic_pot = _electrostatic_pot
Box.comp_j = _comp_j
Box.smolu = _smolu
Box.advect = _advect
Box.ek_get = _ek_get
Box.pnp_init = _pnp_init
Box.pnp_get = _pnp_get
Box.pnp_set = _pnp_set
Box.sor = _sor
Box.just_eq_smolu = _just_eq_smolu
Box.poisson_nernst_planck = _pnp
Box.charge_test = _charge_test
Box.poisson_residual = _poisson_residual


def _compensated_force_field(self, particle_diameter=1, particle_coords=(0, 0, 0), geometry_label=0):
    f = [np.zeros(self.shape) for _ in range(3)]
    pc = (C.c_int * 3)(*particle_coords)
    rc = self.L.lbgpu_compensated_force_field(self.ctx, particle_diameter, pc, geometry_label,
                                              *(_ptr(x) for x in f))
    self._chk(rc, "compensated_force_field")
    return f


def _profiles(self, axis):
    """equilibration.f90:154-176: (flux (L, 3), mean density (L,)) per plane normal to axis
    (0 = x, 1 = y, 2 = z), reduced on the device."""
    L = self.shape[2 - axis]
    flux = np.zeros((L, 3))
    dens = np.zeros(L)
    self._chk(self.L.lbgpu_profiles(self.ctx, axis, _ptr(flux), _ptr(dens)), "profiles")
    return flux, dens


Box.profiles = _profiles


def _set_force_field(self, f):
    if f is None:
        self._chk(self.L.lbgpu_set_force_field(self.ctx, None, None, None), "set_force_field")
        return
    a = [_f64(x, self.shape) for x in f]
    self._chk(self.L.lbgpu_set_force_field(self.ctx, *(_ptr(x) for x in a)), "set_force_field")


Box.compensated_force_field = _compensated_force_field
Box.set_force_field = _set_force_field


# ---------------------------------------------------------------- batches of boxes, serving

class Cell(C.Structure):
    """lbgpu_cell (include/lbgpu.h)."""
    _fields_ = [
        ("lx", C.c_int), ("ly", C.c_int), ("lz", C.c_int), ("relaxation_time", C.c_double),
        ("f_ext", C.c_double * 3), ("rho0", C.c_double), ("tracer", Tracer),
    ]


class Request(C.Structure):
    """lbgpu_request (include/lbgpu.h)."""
    _fields_ = [
        ("cell", Cell), ("nature", C.c_void_p), ("arrival", C.c_double), ("max_steps", C.c_int),
        ("mp_steps", C.c_int), ("out_density", C.c_void_p), ("out_jx", C.c_void_p),
        ("out_jy", C.c_void_p), ("out_jz", C.c_void_p),
    ]


class RequestResult(C.Structure):
    """lbgpu_request_result (include/lbgpu.h)."""
    _fields_ = [
        ("admitted", C.c_double), ("finished", C.c_double), ("steps", C.c_int),
        ("converged", C.c_int), ("status", C.c_int), ("mp_steps", C.c_int),
        ("fluid_nodes", C.c_longlong), ("vacf0", C.c_double * 3), ("vacf_sum", C.c_double * 3),
    ]


class BatchTuning(C.Structure):
    """lbgpu_batch_tuning (include/lbgpu.h)."""
    _fields_ = [
        ("tuned", C.c_int), ("aa_work_list", C.c_int * 2), ("aa_min_blocks", C.c_int * 2),
        ("aa_tiles_per_claim", C.c_int * 2), ("smem_threads", C.c_int), ("steps_per_graph", C.c_int),
        ("aa_ms", C.c_float * 2), ("tiled_fluid_nodes", C.c_longlong),
    ]


def make_cell(shape, relaxation_time=1.0, f_ext=(0.0, 0.0, 0.0), rho0=1.0, tracer=None) -> Cell:
    """shape = (lx, ly, lz); tracer = dict of lbgpu_tracer fields (Db, ka, kd, f_ext) or None."""
    c = Cell()
    c.lx, c.ly, c.lz = (int(v) for v in shape)
    c.relaxation_time = relaxation_time
    c.f_ext = (C.c_double * 3)(*f_ext)
    c.rho0 = rho0
    if tracer:
        c.tracer = _tracer(**tracer)
    return c


def _batch_lib():
    L = library()
    vp, i, d, sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t
    pi = C.POINTER(C.c_int)
    for name, args, res in (
        ("lbgpu_batch_create", [i, sz, C.POINTER(vp)], C.c_int),
        ("lbgpu_batch_destroy", [vp], None),
        ("lbgpu_batch_footprint", [C.POINTER(Cell)], C.c_size_t),
        ("lbgpu_batch_add", [vp, C.POINTER(Cell), vp, pi], C.c_int),
        ("lbgpu_batch_add_label", [vp, C.POINTER(Cell), i, vp, pi], C.c_int),
        ("lbgpu_batch_remove", [vp, i], C.c_int),
        ("lbgpu_batch_steps", [vp, i, i, vp], C.c_int),
        ("lbgpu_batch_time_steps", [vp, i, C.POINTER(C.c_float)], C.c_int),
        ("lbgpu_batch_moments", [vp, i, vp, vp, vp, vp], C.c_int),
        ("lbgpu_batch_mp_start", [vp, i], C.c_int),
        ("lbgpu_batch_mp_get", [vp, i, vp, vp, vp, pi], C.c_int),
        ("lbgpu_batch_mp_fields", [vp, i, vp, vp], C.c_int),
        ("lbgpu_batch_info", [vp, pi, C.POINTER(C.c_longlong), pi, C.POINTER(C.c_size_t)], C.c_int),
        ("lbgpu_batch_get_tuning", [vp, C.POINTER(BatchTuning)], C.c_int),
        ("lbgpu_serve", [vp, vp, i, d, i, vp], C.c_int),
    ):
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    return L


def device_geometry(label, lx, ly, lz, params=None, device=0):
    """nature (lz, ly, lx) int8 of the reference's geometryLabel `label`, built on the device
    (lbgpu_geometry); LbgpuError with the reference's message for a box it refuses."""
    L = library()
    nat = np.zeros((lz, ly, lx), dtype=np.int8)
    par = None if params is None else (C.c_double * len(params))(*params)
    rc = L.lbgpu_geometry(device, label, lx, ly, lz, par, nat.ctypes.data)
    if rc:
        buf = C.create_string_buffer(1024)
        L.lbgpu_last_error(None, buf, 1024)
        raise LbgpuError(rc, buf.value.decode(errors="replace"))
    return nat


def footprint(cell: Cell) -> int:
    return int(_batch_lib().lbgpu_batch_footprint(C.byref(cell)))


class Batch:
    """Many independent boxes stepped together (lbgpu_batch_*).  Boxes are identified by the
    slot id add() returns; moments are (rho, (jx, jy, jz)) arrays of shape (lz, ly, lx)."""

    def __init__(self, memory_budget=0, device=0):
        self.L = _batch_lib()
        self.b = C.c_void_p()
        self._natures = {}
        self._shapes = {}
        self._chk(self.L.lbgpu_batch_create(device, memory_budget, C.byref(self.b)), "batch_create")

    def _chk(self, rc, what=""):
        if rc != 0:
            buf = C.create_string_buffer(1024)
            self.L.lbgpu_last_error(None, buf, len(buf))
            raise LbgpuError(rc, f"{what}: {buf.value.decode(errors='replace')}")

    def close(self):
        if getattr(self, "b", None) and self.b.value:
            self.L.lbgpu_batch_destroy(self.b)
            self.b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add(self, nature, relaxation_time=1.0, f_ext=(0.0, 0.0, 0.0), rho0=1.0, tracer=None) -> int:
        nat = np.ascontiguousarray(nature, dtype=np.int8)
        lz, ly, lx = nat.shape
        cell = make_cell((lx, ly, lz), relaxation_time, f_ext, rho0, tracer)
        i = C.c_int(-1)
        self._chk(self.L.lbgpu_batch_add(self.b, C.byref(cell), _ptr(nat), C.byref(i)), "batch_add")
        self._shapes[i.value] = nat.shape
        return i.value

    def add_label(self, label, lx, ly, lz, params=None, relaxation_time=1.0, f_ext=(0.0, 0.0, 0.0),
                  rho0=1.0, tracer=None) -> int:
        """A box of the reference's geometryLabel `label` built on the device
        (lbgpu_batch_add_label); params: (lw_o_lx, a_o_R) for label 7."""
        cell = make_cell((lx, ly, lz), relaxation_time, f_ext, rho0, tracer)
        par = None if params is None else (C.c_double * len(params))(*params)
        i = C.c_int(-1)
        self._chk(self.L.lbgpu_batch_add_label(self.b, C.byref(cell), label, par, C.byref(i)),
                  "batch_add_label")
        self._shapes[i.value] = (lz, ly, lx)
        return i.value

    def remove(self, box: int):
        self._chk(self.L.lbgpu_batch_remove(self.b, box), "batch_remove")
        self._shapes.pop(box, None)

    def steps(self, nsteps: int, check=False):
        """nsteps (even) steps of every box; with check, {slot: max|u - u_prev|} of the flow boxes."""
        n = max(self._shapes) + 1 if self._shapes else 1
        du = np.zeros(n, dtype=np.float32)
        self._chk(self.L.lbgpu_batch_steps(self.b, nsteps, 1 if check else 0,
                                           _ptr(du) if check else None), "batch_steps")
        return {k: float(du[k]) for k in self._shapes} if check else None

    def time_steps(self, nsteps: int) -> float:
        ms = C.c_float(0)
        self._chk(self.L.lbgpu_batch_time_steps(self.b, nsteps, C.byref(ms)), "batch_time_steps")
        return ms.value

    def moments(self, box: int):
        shape = self._shapes[box]
        out = [np.zeros(shape) for _ in range(4)]
        self._chk(self.L.lbgpu_batch_moments(self.b, box, *(_ptr(x) for x in out)), "batch_moments")
        return out[0], tuple(out[1:])

    def mp_start(self, box: int):
        self._chk(self.L.lbgpu_batch_mp_start(self.b, box), "batch_mp_start")

    def mp_get(self, box: int):
        """(vacf0, vacf_sum, vacf_last, steps); D_eff = vacf0/2 + vacf_sum."""
        v = [np.zeros(3) for _ in range(3)]
        st = C.c_int(0)
        self._chk(self.L.lbgpu_batch_mp_get(self.b, box, *(_ptr(x) for x in v), C.byref(st)),
                  "batch_mp_get")
        return v[0], v[1], v[2], st.value

    def mp_fields(self, box: int):
        """(P, P_ads) of a box in its tracer phase, shape (lz, ly, lx, 3), as Box.mp_get."""
        shape = self._shapes[box] + (3,)
        P, A = np.zeros(shape), np.zeros(shape)
        self._chk(self.L.lbgpu_batch_mp_fields(self.b, box, _ptr(P), _ptr(A)), "batch_mp_fields")
        return P, A

    def info(self):
        a, sm = C.c_int(0), C.c_int(0)
        f = C.c_longlong(0)
        by = C.c_size_t(0)
        self._chk(self.L.lbgpu_batch_info(self.b, C.byref(a), C.byref(f), C.byref(sm), C.byref(by)),
                  "batch_info")
        return dict(active=a.value, fluid_nodes=f.value, smem_boxes=sm.value, bytes=by.value)

    def tuning(self):
        """The tuner's choices (lbgpu_batch_get_tuning) as a dict."""
        t = BatchTuning()
        self._chk(self.L.lbgpu_batch_get_tuning(self.b, C.byref(t)), "batch_get_tuning")
        return {"tuned": bool(t.tuned), "aa_work_list": list(t.aa_work_list),
                "aa_min_blocks": list(t.aa_min_blocks), "aa_tiles_per_claim": list(t.aa_tiles_per_claim),
                "smem_threads": t.smem_threads, "steps_per_graph": t.steps_per_graph,
                "aa_ms": [float(x) for x in t.aa_ms], "tiled_fluid_nodes": t.tiled_fluid_nodes}

    def serve(self, requests, du_tol=1e-8, check_every=100):
        """requests: list of dicts {nature, arrival, max_steps, mp_steps, relaxation_time, f_ext,
        rho0, tracer, moments (bool)}.  Returns a list of result dicts (times in seconds after
        the start), with 'moments' = (rho, (jx, jy, jz)) where asked for."""
        n = len(requests)
        reqs = (Request * max(n, 1))()
        keep = []
        outs = []
        for k, r in enumerate(requests):
            nat = np.ascontiguousarray(r["nature"], dtype=np.int8)
            keep.append(nat)
            lz, ly, lx = nat.shape
            q = reqs[k]
            q.cell = make_cell((lx, ly, lz), r.get("relaxation_time", 1.0), r.get("f_ext", (0.0, 0.0, 0.0)),
                               r.get("rho0", 1.0), r.get("tracer"))
            q.nature = _ptr(nat)
            q.arrival = float(r.get("arrival", 0.0))
            q.max_steps = int(r.get("max_steps", 0))
            q.mp_steps = int(r.get("mp_steps", 0))
            m = None
            if r.get("moments"):
                m = [np.zeros(nat.shape) for _ in range(4)]
                q.out_density, q.out_jx, q.out_jy, q.out_jz = (_ptr(x) for x in m)
            outs.append(m)
        res = (RequestResult * max(n, 1))()
        self._chk(self.L.lbgpu_serve(self.b, reqs, n, du_tol, check_every, res), "serve")
        out = []
        for k in range(n):
            x = res[k]
            d = dict(admitted=x.admitted, finished=x.finished, steps=x.steps, converged=bool(x.converged),
                     status=x.status, mp_steps=x.mp_steps, fluid_nodes=x.fluid_nodes,
                     vacf0=np.array(list(x.vacf0)), vacf_sum=np.array(list(x.vacf_sum)))
            if outs[k] is not None:
                d["moments"] = (outs[k][0], tuple(outs[k][1:]))
            out.append(d)
        return out
