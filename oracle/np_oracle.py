"""A second CPU restatement of laboetie's hot path, in numpy -- TEST INFRASTRUCTURE ONLY.

Written from the Fortran sources of the reference, independently of ``lb_oracle.c``, so that a
misreading of the Fortran in one restatement shows up as a difference between the two
(``tests/test_oracle_np.py`` compares them bit for bit).  Only ``tests/`` use it.

How the Fortran's arithmetic is reproduced: every expression is transcribed with the Fortran's
own grouping (left to right within a sum or product, as gfortran evaluates them without
``-ffast-math``); numpy evaluates each elementwise operation as one correctly rounded IEEE
double operation and never fuses a multiply with an add, so a transcription vectorised over the
nodes gives, node by node, the same bits as the scalar Fortran loop.  Whole-array ``SUM`` and the
running sums of the reference's loops are formed sequentially in the reference's element order
(``np.add.accumulate`` is sequential).  Where the reference multiplies by a velocity component
(an integer 0 or +-1 converted to real) the product is formed as well, not skipped.

Arrays: a field f(lx,ly,lz) is a numpy array of shape (lz, ly, lx) (x fastest, the Fortran
element order); flow populations n(lx,ly,lz,19) are (19, lz, ly, lx); tracer populations
n(19,lx,ly,lz) are (lz, ly, lx, 19); P(3,lx,ly,lz) is (lz, ly, lx, 3).
"""
from __future__ import annotations

import math

import numpy as np

FLUID, SOLID = 0, 1

# module_lbmodel.f90:67-86 (D3Q19 velocities, l = 1..19 here 0..18) and 123-147 (weights).
C = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
              [1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, 1], [1, 0, -1],
              [-1, 0, -1], [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1]], dtype=np.int64)
CSQ = 1.0 / 3.0
_A00, _A01, _A02 = 1.0 / 3.0, 1.0 / 18.0, 1.0 / 36.0
_A1 = (_A00 / CSQ, _A01 / CSQ, _A02 / CSQ)
_A2 = (_A00 / (2 * (CSQ * CSQ)), _A01 / (2 * (CSQ * CSQ)), _A02 / (2 * (CSQ * CSQ)))
_CLASS = [0] + [1] * 6 + [2] * 12
A0 = np.array([(_A00, _A01, _A02)[k] for k in _CLASS])
A1 = np.array([_A1[k] for k in _CLASS])
A2 = np.array([_A2[k] for k in _CLASS])
# module_lbmodel.f90:156-162: inv(l) is the velocity with coo = -coo(l)
INV = np.array([next(m for m in range(19) if (C[m] == -C[l]).all()) for l in range(19)])
KBT = 1.0 / 3.0                     # module_system.f90:94
PI = math.acos(-1.0)                # module_constants.f90:19
EPS_DP = float(np.finfo(np.float64).eps)


def _shift(a, c):
    """a(x - c) for every node x of a periodic field shaped (lz, ly, lx): np.roll by +c."""
    return np.roll(a, shift=(int(c[2]), int(c[1]), int(c[0])), axis=(0, 1, 2))


def _at_plus(a, c):
    """a(x + c) (module_system.f90:99-112 pbc, one step across the boundary)."""
    return np.roll(a, shift=(-int(c[2]), -int(c[1]), -int(c[0])), axis=(0, 1, 2))


def _seq_sum(a):
    """Fortran SUM of an array: a single accumulator in array element order."""
    flat = np.ascontiguousarray(a, dtype=np.float64).ravel()
    return float(np.add.accumulate(flat)[-1]) if flat.size else 0.0


# ----------------------------------------------------------------------------------------- flow

def init_populations(nature, svden=1.0):
    """init_simu.f90:31-39: density = svden off the solid, 0 on it; n(:,:,:,l) = density*a0(l)."""
    rho = np.where(nature != SOLID, svden, 0.0)
    return np.stack([rho * A0[l] for l in range(19)]), rho


def collide(nature, tau, n, rho, jx, jy, jz, fx, fy, fz):
    """module_collision.f90:62-108 (second order; first_order_only has no defined result)."""
    fl = nature == FLUID
    with np.errstate(divide="ignore", invalid="ignore"):
        ux = np.where(fl, jx / rho, 0.0)
        uy = np.where(fl, jy / rho, 0.0)
        uz = np.where(fl, jz / rho, 0.0)
    out = n.copy()
    for l in range(19):
        cx, cy, cz = (float(v) for v in C[l])
        a0, a1, a2 = A0[l], A1[l], A2[l]
        neq = a0 * rho \
            + a1 * (cx * jx + cy * jy + cz * jz) \
            + a2 * (jx * ux * (cx ** 2 - CSQ) + jx * uy * cx * cy + jx * uz * cx * cz
                    + jy * ux * cy * cx + jy * uy * (cy ** 2 - CSQ) + jy * uz * cy * cz
                    + jz * ux * cz * cx + jz * uy * cz * cy + jz * uz * (cz ** 2 - CSQ))
        new = (1.0 - 1.0 / tau) * n[l] \
            + (1.0 / tau) * neq \
            + (1.0 - 1.0 / (2.0 * tau)) * (
                a1 * ((cx - ux) * fx + (cy - uy) * fy + (cz - uz) * fz)
                + 2.0 * a2 * (cx * ux + cy * uy + cz * uz) * (cx * fx + cy * fy + cz * fz))
        out[l] = np.where(fl, new, n[l])
    return out


def bounce_back_stream(nature, n):
    """equilibration.f90:204-243: for l = 1, 3, ..., 19 (Fortran numbering) swap n(x,l) with
    n(x+c_l, inv l) where the two natures differ; then n(x+c_l, l) = n_old(x, l) for every l."""
    n = n.copy()
    for l in range(0, 19, 2):            # Fortran l = 1, 3, ..., 19
        c, li = C[l], INV[l]
        diff = nature != _at_plus(nature, c)
        mine = n[l].copy()
        theirs = _at_plus(n[li], c)      # n(x+c_l, inv l) seen from x
        n[l] = np.where(diff, theirs, mine)
        # the partner entries n(x+c, inv l) receive n(x, l): written back at x+c
        back = _shift(np.where(diff, mine, theirs), c)
        n[li] = np.where(_shift(diff, c), back, n[li])
    return np.stack([_shift(n[l], C[l]) for l in range(19)])


def moments(n, fx, fy, fz, jx_old, jy_old, jz_old):
    """equilibration.f90:248-343: (any n<0, density = SUM(n,4), j = f/2 + sum_l n_l c_l, l2err)."""
    negative = bool((n < 0).any())
    rho = n[0].copy()
    for l in range(1, 19):
        rho = rho + n[l]
    jx, jy, jz = fx / 2.0, fy / 2.0, fz / 2.0
    for l in range(19):
        cx, cy, cz = (float(v) for v in C[l])
        jx = jx + n[l] * cx
        jy = jy + n[l] * cy
        jz = jz + n[l] * cz
    l2err = max(np.abs(jx - jx_old).max(), np.abs(jy - jy_old).max(), np.abs(jz - jz_old).max())
    return negative, rho, (jx, jy, jz), float(l2err)


def _norm2(v):
    """gfortran's NORM2 of a short vector: scaled sum of squares, the scale starting at 1."""
    result, scale = 0.0, 1.0
    for x in v:
        if x != 0.0:
            ax = abs(x)
            if scale < ax:
                val = scale / ax
                result = 1.0 + result * val * val
                scale = ax
            else:
                val = ax / scale
                result = result + val * val
    return scale * math.sqrt(result)


def compensated_force_field(nature, f_ext, particle_diameter=1, particle_coords=(0, 0, 0),
                            geometry_label=0):
    """equilibration.f90:388-487 (compensate_f_ext): f_ext on the fluid nodes of a ball of odd
    diameter pd around the particle centre (1-based coordinates; 0 takes the reference's default
    n/2+1), split evenly over its nodes; in a bulk box (geometryLabel -1) every fluid node also
    carries -f_ext / (fluid nodes), so that the total force is zero; 0 on solid nodes."""
    lz, ly, lx = nature.shape
    pd = particle_diameter if particle_diameter > 0 else 1
    if pd % 2 == 0 or lx % 2 == 0 or ly % 2 == 0 or lz % 2 == 0:
        raise ValueError("compensate_f_ext needs an odd particle diameter and odd box sides")
    pdr = pd // 2
    c = [particle_coords[d] if particle_coords[d] > 0 else n // 2 + 1 for d, n in enumerate((lx, ly, lz))]
    f = [np.zeros(nature.shape) for _ in range(3)]
    cnt, err = 0, False
    for i in range(c[0] - pdr, c[0] + pdr + 1):
        for j in range(c[1] - pdr, c[1] + pdr + 1):
            for k in range(c[2] - pdr, c[2] + pdr + 1):
                if _norm2([float(i - c[0]), float(j - c[1]), float(k - c[2])]) > float(pd) / 2.0:
                    continue
                if not (1 <= i <= lx and 1 <= j <= ly and 1 <= k <= lz):
                    raise ValueError("the particle reaches outside the box")
                if nature[k - 1, j - 1, i - 1] != FLUID:
                    err = True
                for d in range(3):
                    f[d][k - 1, j - 1, i - 1] = f_ext[d]
                cnt += 1
    if err:
        raise ValueError("Dominika's particle at a solid node")
    n_fluid = int((nature == FLUID).sum())
    inside = (f[0] == f_ext[0]) & (f[1] == f_ext[1]) & (f[2] == f_ext[2])
    if geometry_label == -1:
        f = [np.where(inside, -f_ext[d] / n_fluid + f[d] / cnt, -f_ext[d] / n_fluid) for d in range(3)]
        if any(abs(_seq_sum(f[d]) / n_fluid) > EPS_DP for d in range(3)):
            raise ValueError("The compensation is not well-implemented")
    else:
        f = [np.where(inside, f[d] / cnt, 0.0) for d in range(3)]
    return tuple(np.where(nature != FLUID, 0.0, f[d]) for d in range(3))


def equilibration(nature, tau=1.0, target_error=1e-10, f_ext=(0.0, 0.0, 0.0), svden=1.0,
                  max_steps=100000, compensate_f_ext=False, particle_diameter=1,
                  particle_coords=(0, 0, 0), geometry_label=0):
    """The time loop of equilibration.f90:143-491: collide, bounce-back, streaming, moments,
    l2err, and the two-phase force machine (from the step after the first convergence the force:
    f_ext on fluid nodes, or the compensated field of compensate_f_ext; exit at the second)."""
    n, rho = init_populations(nature, svden)
    z = np.zeros(nature.shape)
    jx, jy, jz = z.copy(), z.copy(), z.copy()
    fx, fy, fz = z.copy(), z.copy(), z.copy()
    without = with_ = False
    hist = []
    for t in range(1, max_steps + 1):
        n = collide(nature, tau, n, rho, jx, jy, jz, fx, fy, fz)
        n = bounce_back_stream(nature, n)
        negative, rho, (jx2, jy2, jz2), l2err = moments(n, fx, fy, fz, jx, jy, jz)
        if negative:
            raise RuntimeError("In equilibration, the population n(x,y,z,vel) < 0")
        jx, jy, jz = jx2, jy2, jz2
        hist.append(l2err)
        converged = l2err <= target_error and t > 2
        if converged:
            if not without:
                without = True
            else:
                with_ = True
            if without and with_ and t > 2:
                return dict(n=n, rho=rho, j=(jx, jy, jz), steps=t, l2err=np.array(hist),
                            f=(fx, fy, fz))
            if compensate_f_ext:
                fx, fy, fz = compensated_force_field(nature, f_ext, particle_diameter,
                                                     particle_coords, geometry_label)
            else:
                fl = nature == FLUID
                fx = np.where(fl, f_ext[0], fx)
                fy = np.where(fl, f_ext[1], fy)
                fz = np.where(fl, f_ext[2], fz)
    return dict(n=n, rho=rho, j=(jx, jy, jz), steps=max_steps, l2err=np.array(hist), capped=True,
                f=(fx, fy, fz))


def profiles(rho, j, axis):
    """equilibration.f90:153-176 (and :504-516 at the loop's exit): per plane k normal to axis
    (0 = x, 1 = y, 2 = z), SUM(jx), SUM(jy), SUM(jz) and SUM(density) / MAX(COUNT(density > eps),
    1) over the plane's section, each SUM one accumulator in the section's element order (its
    first remaining index fastest).  Returns (flux (L, 3), mean density (L,))."""
    def section(a, k):   # (lz, ly, lx) arrays: x fastest
        if axis == 0:
            return a[:, :, k]
        return a[:, k, :] if axis == 1 else a[k]
    L = rho.shape[2 - axis]
    flux = np.zeros((L, 3))
    dens = np.zeros(L)
    for k in range(L):
        for d in range(3):
            flux[k, d] = _seq_sum(section(j[d], k))
        sd = section(rho, k)
        dens[k] = _seq_sum(sd) / max(int((sd > EPS_DP).sum()), 1)
    return flux, dens


# ------------------------------------------------------------------------ moment propagation

def detect_interfacial(nature):
    """supercell_definition.f90:115-147: a node is interfacial if any of its 18 periodic
    neighbours has another nature."""
    out = np.zeros(nature.shape, dtype=bool)
    for l in range(1, 19):
        out |= nature != _at_plus(nature, C[l])
    return out


def update_tracer_population(nature, rho, j, f_ext, q=0.0, D=0.0, elec_slope=(0.0, 0.0, 0.0)):
    """drop_tracers.f90:94-105: n(l,x) = a0 rho + a1 sum(coo*(flux + f_ext - rho q D E)) on fluid
    nodes, a0 rho + a1 sum(coo*flux) elsewhere.  Returns shape (lz, ly, lx, 19)."""
    fl = nature == FLUID
    out = np.empty(nature.shape + (19,))
    for l in range(19):
        cf = [float(v) for v in C[l]]
        fluid_terms = [cf[d] * (j[d] + f_ext[d] - rho * q * D * elec_slope[d]) for d in range(3)]
        solid_terms = [cf[d] * j[d] for d in range(3)]
        nf = A0[l] * rho + A1[l] * (fluid_terms[0] + fluid_terms[1] + fluid_terms[2])
        ns = A0[l] * rho + A1[l] * (solid_terms[0] + solid_terms[1] + solid_terms[2])
        out[..., l] = np.where(fl, nf, ns)
    return out


def _scattprop(n, rho, w, lam, fermi):
    """module_moment_propagation.f90:341-346: n/rho - w + lambda*w*fermi."""
    with np.errstate(divide="ignore", invalid="ignore"):   # solid nodes (rho = 0) are masked
        return n / rho - w + lam * w * fermi


class MomentPropagation:
    """module_moment_propagation.f90 init (30-160) and propagate (164-289) for a neutral tracer
    (the reference stops on a charged one, :71-79): exp_dphi = 1, fermi = 1/2."""

    def __init__(self, nature, rho, n_mp, ka=0.0, kd=0.0, Db=0.01):
        self.nature = nature
        self.fl = nature == FLUID
        self.inter = detect_interfacial(nature)
        self.rho = rho
        self.n = n_mp
        eps = EPS_DP
        self.ka, self.kd = ka, kd
        K = 0.0 if abs(kd) <= eps else ka / kd
        self.ads = abs(K) > eps
        self.lam = 4.0 * Db / KBT                                  # calc_lambda, :331-337
        self.Db = Db
        nf = int(self.fl.sum())
        nfi = int((self.fl & self.inter).sum())
        pstat = float(nf) + K * float(nfi)                         # :97
        bw = 1.0 / pstat
        fermi = 1.0 / (1.0 + 1.0)
        exp_min_dphi = 1.0 / 1.0
        vacf0 = [0.0, 0.0, 0.0]
        P = np.zeros(nature.shape + (3,))
        # the init loop, DO CONCURRENT over fluid nodes and l = 2..19 (:105-136); the vacf sum
        # runs over nodes in array element order, l inner
        terms = []
        for l in range(1, 19):
            c = C[l]
            nbr_fluid = _at_plus(self.fl, c)
            on = self.fl & nbr_fluid
            sp = _scattprop(self.n[..., l], rho, A0[l], self.lam, fermi)
            li = INV[l]
            sp_p = _scattprop(_at_plus(self.n[..., li], c), _at_plus(rho, c), A0[li], self.lam,
                              1.0 - fermi)
            for d in range(3):
                term = exp_min_dphi * sp_p * float(C[li][d]) * bw
                P[..., d] = np.where(on, P[..., d] + term, P[..., d])
            terms.append([np.where(on, bw * sp * float(c[d]) ** 2, 0.0) for d in range(3)])
        for d in range(3):
            # node-major, l-minor order of the reference's nested loops
            t = np.stack([terms[k][d] for k in range(18)], axis=-1)
            on_all = np.stack([self.fl & _at_plus(self.fl, C[l]) for l in range(1, 19)], axis=-1)
            vacf0[d] = _seq_sum(np.where(on_all, t, 0.0)[on_all])
        self.vacf0 = np.array(vacf0)
        self.P = P
        self.A = np.zeros_like(P) if self.ads else None
        self.fermi = fermi

    def propagate(self, it):
        """One step: returns (vacf(it), is_converged); raises if a remaining fraction < eps."""
        fl, rho, lam, fermi = self.fl, self.rho, self.lam, self.fermi
        Pn = self.P
        Pnext = np.zeros_like(Pn)
        frac = np.ones(fl.shape)
        us = [np.zeros(fl.shape) for _ in range(3)]
        for l in range(1, 19):               # Fortran l = 2..19
            c, li = C[l], INV[l]
            on = fl & _at_plus(fl, c)
            sp = _scattprop(self.n[..., l], rho, A0[l], lam, fermi)
            frac = np.where(on, frac - sp, frac)
            for d in range(3):
                us[d] = np.where(on, us[d] + sp * float(c[d]), us[d])
            sp_p = _scattprop(_at_plus(self.n[..., li], c), _at_plus(rho, c), A0[li], lam,
                              1.0 - fermi)
            for d in range(3):
                Pnext[..., d] = np.where(on, Pnext[..., d] + _at_plus(Pn[..., d], c) * sp_p,
                                         Pnext[..., d])
        vacf = np.array([_seq_sum(np.where(fl, Pn[..., d] * us[d], 0.0)[fl]) for d in range(3)])
        bulk = fl & ~(self.inter & self.ads) if self.ads else fl
        for d in range(3):
            Pnext[..., d] = np.where(bulk, Pnext[..., d] + frac * Pn[..., d], Pnext[..., d])
        if self.ads:
            site = fl & self.inter
            frac = np.where(site, frac - self.ka, frac)
            An = self.A
            Anext = np.zeros_like(An)
            for d in range(3):
                Pnext[..., d] = np.where(site, Pnext[..., d] + frac * Pn[..., d]
                                         + An[..., d] * self.kd, Pnext[..., d])
                Anext[..., d] = np.where(site, An[..., d] * (1.0 - self.kd)
                                         + Pn[..., d] * self.ka, Anext[..., d])
            self.A = Anext
        if (frac[fl] < EPS_DP).any():
            raise RuntimeError("somewhere restpart is negative")
        self.P = Pnext
        lx, ly, lz = fl.shape[2], fl.shape[1], fl.shape[0]
        thr = 1.0 / (2.0 * lx * ly * lz / self.Db)
        conv = it > 2 and bool((np.abs(vacf) < thr).all() and (np.abs(vacf) < float(np.float32(1.e-12))).all())
        return vacf, conv


# ---------------------------------------------------------------------------------- Poisson

def charges_init(nature, interfacial, bjl, sigma, lambda_D):
    """charges_init.f90:3-130 with charge_distrib 'int' (the only distribution the reference
    lets through, :96-100): the surface charge sigma on the interfacial solid nodes, its opposite
    spread over the fluid nodes on top of the salt 0.5 rho_0, phi = 0, and
    anormf0 = 4 pi bjl kBT / 2 * SUM(c+ + c-).  Returns (c+, c-, phi, anormf0, rho_ch)."""
    zeros = np.zeros(nature.shape)
    if bjl <= EPS_DP:
        return zeros, zeros.copy(), zeros.copy(), 0.0, 0.0
    four_pi_bjl = np.float64(4.0) * PI * bjl
    rho_ch = np.float64(1.0) / (four_pi_bjl * (lambda_D * lambda_D))
    rho_0 = 0.0 if abs(lambda_D) <= EPS_DP else float(rho_ch)
    solid, fluid = nature == SOLID, nature == FLUID
    inter = np.asarray(interfacial).astype(bool)
    n_solid_int, n_fluid = int((solid & inter).sum()), int(fluid.sum())
    if abs(sigma) <= EPS_DP:
        return zeros, zeros.copy(), zeros.copy(), 0.0, float(rho_ch)
    sigma_solid = sigma / n_solid_int if n_solid_int != 0 else 0.0
    sigma_fluid = -1.0 * sigma / n_fluid if n_fluid != 0 else 0.0
    p_solid, m_solid = 0.5 * sigma_solid, -0.5 * sigma_solid
    if sigma_fluid > 0.0:
        p_fluid, m_fluid = 0.5 * rho_0 + sigma_fluid, 0.5 * rho_0
    else:
        p_fluid, m_fluid = 0.5 * rho_0, 0.5 * rho_0 - sigma_fluid
    cp = np.where(solid & inter, p_solid, np.where(fluid, p_fluid, 0.0))
    cm = np.where(solid & inter, m_solid, np.where(fluid, m_fluid, 0.0))
    anormf0 = 4.0 * PI * bjl * KBT / 2.0 * _seq_sum(cp + cm)
    return cp, cm, zeros, anormf0, float(rho_ch)


# delta of a link: 1 for a nearest neighbour, sqrt(2) for a next-nearest (module_lbmodel.f90:137,147)
_DELTA = [0.0] + [1.0] * 6 + [math.sqrt(2.0)] * 12


def just_eq_smolu(nature, phi, c_plus, c_minus, D_plus, D_minus, rho_ch, sigma, loop_bug=True):
    """just_eq_smolu.f90:6-135 as poisson_nernst_planck calls it: time is 0 (init_simu.f90:57)
    and D_equil is never set (0), so the first branch holds: eD = 0.1 D, at most 10 iterations.
    Each iteration sums the link fluxes of every fluid-fluid link l = 2, 4, .., 18 (one of each
    pair of opposite velocities) into both of its sites, in the reference's loop order (i outer,
    j, k, l inner; with the reference's loop bounds j and k take only their last value,
    loop_bug), checks that the fluxes add up to zero, adds them to the fluid nodes and forms the
    relative residuals.  Returns (c+, c-, iterations)."""
    lz, ly, lx = nature.shape
    cp = np.array(c_plus, dtype=np.float64)
    cm = np.array(c_minus, dtype=np.float64)
    phi = np.asarray(phi, dtype=np.float64)
    fluid = nature == FLUID
    n_fluid = int(fluid.sum())
    eDp, eDm = 0.1 * D_plus, 0.1 * D_minus
    crit = float(np.float32(5.e-6))
    tot_p = tot_m = float(np.finfo(np.float64).max)
    links = range(1, 19, 2)
    js = [ly - 1] if loop_bug else range(ly)
    ks = [lz - 1] if loop_bug else range(lz)
    it = 0
    while tot_m + tot_p > crit and it < 10:
        fp = np.zeros(nature.shape)
        fm = np.zeros(nature.shape)
        for i in range(lx):
            for j in js:
                for k in ks:
                    for l in links:
                        ip, jp, kp = (i + C[l][0]) % lx, (j + C[l][1]) % ly, (k + C[l][2]) % lz
                        if not (fluid[k, j, i] and fluid[kp, jp, ip]):
                            continue
                        e = math.exp(phi[kp, jp, ip] - phi[k, j, i])
                        em = 1.0 / e
                        flp = 0.5 * (1.0 + em) * (cp[kp, jp, ip] * e - cp[k, j, i])
                        flp = flp * eDp / _DELTA[l]
                        flm = 0.5 * (1.0 + e) * (cm[kp, jp, ip] * em - cm[k, j, i])
                        flm = flm * eDm / _DELTA[l]
                        fp[k, j, i] = fp[k, j, i] + flp
                        fm[k, j, i] = fm[k, j, i] + flm
                        fp[kp, jp, ip] = fp[kp, jp, ip] - flp
                        fm[kp, jp, ip] = fm[kp, jp, ip] - flm
        lim = float(np.float32(1.e-12))
        if abs(_seq_sum(fp)) > lim or abs(_seq_sum(fm)) > lim:
            raise RuntimeError("the sum of all flux does not add up. problem in just_eq_smolu.f90")
        cp = np.where(fluid, cp + fp, cp)
        cm = np.where(fluid, cm + fm, cm)
        if sigma != 0 and eDp != 0.0 and eDm != 0.0:
            tot_p = math.sqrt(_seq_sum((fp * fp)[fluid])) / n_fluid / (0.5 * rho_ch * eDp) / sigma
            tot_m = math.sqrt(_seq_sum((fm * fm)[fluid])) / n_fluid / (0.5 * rho_ch * eDm) / sigma
        it = it + 1
    return cp, cm, it


def sor(nature, sigma, bjl, c_plus, c_minus, phi, anormf0, maxiter=500000):
    """sor.f90:7-91: over-relaxed Jacobi (omega 1.4) over every node, phi* = sum_l a0(l)
    phi(x - c_l) + 4 pi bjl kBT/2 (c+ - c-), stop when sum|phi* - phi| <= 1e-5 anormf0 (the
    sum over i outer, j, k inner); then anormf0 = SUM(|phi|).  Returns (phi, anormf0, iter-1)."""
    if sigma == 0.0:
        return np.zeros(nature.shape), anormf0, 0
    eps = float(np.float32(1.0e-5))
    omega = 1.4
    factor = 4.0 * PI * bjl * KBT / 2.0
    phi = phi.copy()
    rhs = factor * (c_plus - c_minus)
    for it in range(1, maxiter + 1):
        phistar = np.zeros(nature.shape)
        for l in range(19):
            phistar = phistar + A0[l] * _shift(phi, C[l])
        phistar = phistar + rhs
        phitmp = omega * phistar + (1.0 - omega) * phi
        anorm = _seq_sum(np.transpose(np.abs(phistar - phi), (2, 1, 0)))   # k fastest
        phi = phitmp
        if anorm <= eps * anormf0:
            break
    else:
        raise RuntimeError("maximum iterations 500 000 reached without convergence in sor")
    return phi, _seq_sum(np.abs(phi)), it - 1


def check_charge_distribution_equilibrium(phi, phi_old, c_plus, c_plus_old, c_minus, c_minus_old):
    """check_charge_distribution_equilibrium.f90:24-44: for phi, c+ and c-, the mean over the
    nodes whose previous value exceeds 1e-12 in magnitude of |(new - old)/old| (a masked SUM in
    element order over the count); converged when all three are below 1e-12.  Returns
    (converged, (dphi, dcp, dcm))."""
    eps = 1.0e-12
    d = []
    for new, old in ((phi, phi_old), (c_plus, c_plus_old), (c_minus, c_minus_old)):
        mask = np.abs(old) > eps
        n = int(mask.sum())
        rel = np.abs((new[mask] - old[mask]) / old[mask])
        d.append(_seq_sum(rel) / float(n) if n else 0.0)
    return bool(d[0] < eps and d[1] < eps and d[2] < eps), tuple(d)


def charge_test(nature, c_plus, c_minus, sigma):
    """charge_test.f90:6-26: SUM(c+ - c-) over the solid and over the fluid nodes must stay sigma
    and -sigma within the default-real tolerance 1.0e-10.  Returns (ok, solid, fluid)."""
    q = c_plus - c_minus
    solid = _seq_sum(q[nature == SOLID])
    fluid = _seq_sum(q[nature == FLUID])
    tol = float(np.float32(1.0e-10))
    return not (abs(solid - sigma) > tol or abs(fluid + sigma) > tol), solid, fluid


def pnp(nature, bjl, sigma, D_plus, D_minus, rho_ch, c_plus, c_minus, phi, anormf0, loop_bug=True,
        max_outer=10000):
    """poisson_nernst_planck.f90:38-48: until converged, back up phi, c+, c- (backup_phi_c_plus_
    c_minus), solve Poisson (sor, which also refreshes anormf0), one Nernst-Planck update, and
    test convergence (every outer iteration: time stays 0, so modulo(time, 10) is 0).  Stops
    unconverged after max_outer iterations.  Returns the fields, anormf0, the outer count, the
    total of the sweep counts sor reports and whether it converged."""
    cp, cm, ph = (np.array(a, dtype=np.float64) for a in (c_plus, c_minus, phi))
    outer = total = 0
    converged = False
    while not converged and outer < max_outer:
        po, cpo, cmo = ph.copy(), cp.copy(), cm.copy()
        ph, anormf0, it = sor(nature, sigma, bjl, cp, cm, ph, anormf0)
        total += it
        cp, cm, _ = just_eq_smolu(nature, ph, cp, cm, D_plus, D_minus, rho_ch, sigma, loop_bug)
        converged, _ = check_charge_distribution_equilibrium(ph, po, cp, cpo, cm, cmo)
        outer += 1
    return dict(c_plus=cp, c_minus=cm, phi=ph, anormf0=anormf0, outer=outer, sor_iters=total,
                converged=converged)


# --------------------------------------------------------------- coupled electrokinetics

_exp = np.vectorize(math.exp, otypes=[np.float64])   # the C library's exp, as the C oracle's


def electrostatic_pot(phi, elec_slope):
    """electrostatic_pot.f90:7-21."""
    if all(e == 0.0 for e in elec_slope):
        return phi.copy()
    lz, ly, lx = phi.shape
    k, j, i = np.meshgrid(np.arange(1, lz + 1), np.arange(1, ly + 1), np.arange(1, lx + 1),
                          indexing="ij")
    s = np.zeros(phi.shape)
    s = s + elec_slope[0] * i.astype(np.float64)
    s = s + elec_slope[1] * j.astype(np.float64)
    s = s + elec_slope[2] * k.astype(np.float64)
    return phi + s


def comp_j(n, j):
    """comp_j.f90:14-27: j = 0.5*(j + sum(n(:,:,:,l)*coo(l))), the sum from 0 over l."""
    out = []
    for d in range(3):
        s = np.zeros(n.shape[1:])
        for l in range(19):
            s = s + n[l] * float(C[l][d])
        out.append(0.5 * (j[d] + s))
    return tuple(out)


def smolu(nature, phi_tot, cp, cm, D_plus, D_minus, time, D_iter, elec_slope, lncb_slope,
          el_curr, ion_curr, solute_force):
    """smolu.f90:1-144.  Returns (flux sums ok, c+, c-, el_curr, ion_curr, solute_force)."""
    lz, ly, lx = nature.shape
    fl = nature == FLUID
    dit = float(D_iter)
    fp, fm = np.zeros(nature.shape), np.zeros(nature.shape)
    sf = [solute_force[d].copy() for d in range(3)]
    k, jj, i = np.meshgrid(np.arange(lz), np.arange(ly), np.arange(lx), indexing="ij")
    terms = []   # per link, the six current terms at every node (summed below in loop order)
    for l in range(1, 19):
        c = C[l]
        cx, cy, cz = (float(v) for v in c)
        a1 = A1[l]
        fl_p = _at_plus(fl, c)
        both = fl & fl_p
        sol = fl & ~fl_p
        php, cpp, cmp_ = _at_plus(phi_tot, c), _at_plus(cp, c), _at_plus(cm, c)
        e = _exp(php - phi_tot)
        ip, jp, kp = (i + c[0]) % lx, (jj + c[1]) % ly, (k + c[2]) % lz
        for cond, fac in (((i == lx - 1) & (ip == 0), math.exp(elec_slope[0] * lx)),
                          ((jj == ly - 1) & (jp == 0), math.exp(elec_slope[1] * ly)),
                          ((k == lz - 1) & (kp == 0), math.exp(elec_slope[2] * lz)),
                          ((i == 0) & (ip == lx - 1), math.exp(-(elec_slope[0] * lx))),
                          ((jj == 0) & (jp == ly - 1), math.exp(-(elec_slope[1] * ly))),
                          ((k == 0) & (kp == lz - 1), math.exp(-(elec_slope[2] * lz)))):
            e = np.where(cond, e * fac, e)
        em = 1.0 / e
        sl = 0.0
        sl = sl + lncb_slope[0] * cx
        sl = sl + lncb_slope[1] * cy
        sl = sl + lncb_slope[2] * cz
        edl = math.exp(sl)
        emdl = 1.0 / edl
        flp = 0.5 * (1.0 + em * emdl) * (cpp * e * edl - cp)
        flm = 0.5 * (1.0 + e * emdl) * (cmp_ * em * edl - cm)
        elc = flp * D_plus - flm * D_minus
        ionc = flp * D_plus + flm * D_minus
        fpl = 0.5 * (1.0 + em) * (cpp * e - cp)
        fmi = 0.5 * (1.0 + e) * (cmp_ * em - cm)
        fmic = KBT * (fpl + fmi)
        fmic = fmic - KBT * (cpp - cp + cmp_ - cm)
        delta = 1.0 if l < 7 else math.sqrt(2.0)
        flp = flp * (D_plus / delta)
        flm = flm * (D_minus / delta)
        fp = np.where(both, fp + flp, fp)
        fm = np.where(both, fm + flm, fm)
        terms.append([np.where(both, a1 * cd * x / dit, np.nan) for x in (elc, ionc)
                      for cd in (cx, cy, cz)])
        # the force on the solid across a fluid-solid link
        es_ = _exp(php - phi_tot)
        ems = 1.0 / es_
        fmis = KBT * (cp * (1.0 - ems) + cm * (1.0 - es_))
        for d, cd in enumerate((cx, cy, cz)):
            sf[d] = np.where(both, sf[d] + a1 * cd * fmic / dit,
                             np.where(sol, sf[d] + a1 * cd * fmis / dit, sf[d]))
    # the currents, summed over nodes (i outer, j, k inner) and their links in l order
    el, io = list(el_curr), list(ion_curr)
    stack = [np.stack([terms[l][q] for l in range(18)], axis=-1) for q in range(6)]
    order = np.transpose(np.arange(lx * ly * lz).reshape(lz, ly, lx), (2, 1, 0)).ravel()
    for q in range(6):
        t = stack[q].reshape(-1, 18)[order].ravel()
        t = t[~np.isnan(t)]
        acc = el[q] if q < 3 else io[q - 3]
        acc = float(np.add.accumulate(np.concatenate([[acc], t]))[-1]) if t.size else acc
        if q < 3:
            el[q] = acc
        else:
            io[q - 3] = acc
    cp2 = np.where(fl, cp + fp, cp)
    cm2 = np.where(fl, cm + fm, cm)
    if time > 0:
        with np.errstate(divide="ignore", invalid="ignore"):
            el = [v / np.float64(0.0) for v in el]
            io = [v / np.float64(0.0) for v in io]
    ok = not (abs(_seq_sum(fp[fl])) > float(np.float32(1.0e-12))
              or abs(_seq_sum(fm[fl])) > float(np.float32(1.0e-12)))
    return ok, cp2, cm2, np.array(el, dtype=float), np.array(io, dtype=float), np.stack(sf)


def advect(nature, j, cp, cm, fp, fm, el_curr, ion_curr):
    """advect.f90:2-116 as a literal loop (small boxes), the neighbour of link (ix, iy, iz) taken
    as pbc(i + ix) where the reference's ip_all(ix) has no defined result.  fp, fm: flux_site
    arrays carried between calls (updated in place).  Returns (ok, c+, c-, el_curr, ion_curr)."""
    lz, ly, lx = nature.shape
    eps = EPS_DP
    cp, cm = cp.copy(), cm.copy()
    el, io = [float(v) for v in el_curr], [float(v) for v in ion_curr]
    fl = nature == FLUID
    if (np.abs(cp) <= eps).all() and (np.abs(cm) <= eps).all():
        return True, cp, cm, np.array(el), np.array(io)
    if (np.abs(cp - cm) <= eps).all():
        el = [0.0, 0.0, 0.0]
    else:
        el = [-_seq_sum((j[d] * (cp - cm))[fl]) for d in range(3)]
    if (np.abs(cp + cm) <= eps).all():
        el = [0.0, 0.0, 0.0]
    else:
        io = [-_seq_sum((j[d] * (cp + cm))[fl]) for d in range(3)]
    cp_old, cm_old = _seq_sum(cp), _seq_sum(cm)
    for i in range(lx):
        for jj in range(ly):
            for k in range(lz):
                if abs(cp[k, jj, i]) <= eps and abs(cm[k, jj, i]) <= eps:
                    continue
                vx, vy, vz = (float(j[d][k, jj, i]) for d in range(3))
                for ix in (-1, 0, 1):
                    for iy in (-1, 0, 1):
                        for iz in (-1, 0, 1):
                            ip, jp, kp = (i + ix) % lx, (jj + iy) % ly, (k + iz) % lz
                            ax, ay, az = vx * ix, vy * iy, vz * iz
                            if ax >= 0 and ay >= 0 and az >= 0 and nature[k, jj, i] == nature[kp, jp, ip]:
                                fx = 1.0 - abs(vx) if ix == 0 else ax
                                fy = 1.0 - abs(vy) if iy == 0 else ay
                                fz = 1.0 - abs(vz) if iz == 0 else az
                                flp = fx * fy * fz * float(cp[k, jj, i])
                                flm = fx * fy * fz * float(cm[k, jj, i])
                            else:
                                flp = flm = 0.0
                            fm[k, jj, i] = fm[k, jj, i] - flm
                            fm[kp, jp, ip] = fm[kp, jp, ip] + flm
                            fp[k, jj, i] = fp[k, jj, i] - flp
                            fp[kp, jp, ip] = fp[kp, jp, ip] + flp
    cm = np.where(fl, cm + fm, cm)
    cp = np.where(fl, cp + fp, cp)
    ok = not (abs(_seq_sum(cm) - cm_old) > float(np.float32(1.e-8))
              or abs(_seq_sum(cp) - cp_old) > float(np.float32(1.e-8)))
    return ok, cp, cm, np.array(el), np.array(io)
