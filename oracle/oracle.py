"""ctypes front end of the CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  The product package never
imports it.  Parity unpinned: the reference has no tests or fixtures for this
path and cannot be built here (see oracle.c).

Arrays are numpy float64, C order (z, y, x).  Face velocities: u (nz, ny, nx+1),
v (nz, ny+1, nx), w (nz+1, ny, nx).  Face coefficients: cell-shaped low-face
arrays cx, cy, cz (0 on the low walls).
"""
import ctypes as C

import numpy as np

from . import build as _build

_lib = None


class Grid(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double)]


class MGParams(C.Structure):
    _fields_ = [("nu1", C.c_int32), ("nu2", C.c_int32), ("levels", C.c_int32),
                ("coarse_max", C.c_int32), ("max_cycles", C.c_int32), ("smoother", C.c_int32),
                ("blocks", C.c_int32 * 3), ("mean_every_sweep", C.c_int32),
                ("coarse_op", C.c_int32), ("record_history", C.c_int32),
                ("krylov", C.c_int32), ("prolong", C.c_int32), ("coarse_scale", C.c_double)]


class MGStats(C.Structure):
    _fields_ = [("cycles", C.c_int32), ("levels", C.c_int32), ("status", C.c_int32),
                ("coarse_n", C.c_int32), ("rel_residual", C.c_double),
                ("rms_residual", C.c_double), ("history", C.c_double * 256)]


class NSParams(C.Structure):
    _fields_ = [("ghost", C.c_int32), ("bc", C.c_int32 * 6), ("iterations", C.c_int32),
                ("adv_scheme", C.c_int32), ("dt", C.c_double), ("re", C.c_double), ("fr", C.c_double), ("we", C.c_double),
                ("mu_12", C.c_double), ("gx", C.c_double), ("gy", C.c_double),
                ("gz", C.c_double), ("btn_g", C.c_double), ("btn_sf", C.c_double),
                ("p_tol", C.c_double)]


_D = C.POINTER(C.c_double)


def lib():
    global _lib
    if _lib is None:
        so = _build.build()
        L = C.CDLL(so)
        L.or_heaviside.argtypes = [_D, C.c_int64, C.c_double, _D]
        L.or_heaviside_deriv.argtypes = [_D, C.c_int64, C.c_double, _D]
        L.or_rho_from_phi.argtypes = [_D, C.c_int64, C.c_double, C.c_double, C.c_double, _D]
        L.or_face_coef.argtypes = [C.POINTER(Grid), _D, _D, _D, _D]
        L.or_divergence.argtypes = [C.POINTER(Grid), _D, _D, _D, C.c_double, C.c_int, _D]
        L.or_apply.argtypes = [C.POINTER(Grid), _D, _D, _D, _D, _D]
        L.or_residual.argtypes = [C.POINTER(Grid), _D, _D, _D, _D, _D, _D]
        L.or_residual.restype = C.c_double
        L.or_remove_mean.argtypes = [_D, C.c_int64]
        L.or_correct.argtypes = [C.POINTER(Grid), _D, _D, C.c_double, _D, _D, _D]
        L.or_split_rhs.argtypes = [C.POINTER(Grid), _D, _D, _D, _D, _D, C.c_double, C.c_double,
                                   _D]
        L.or_split_correct.argtypes = [C.POINTER(Grid), _D, _D, _D, C.c_double, C.c_double, _D,
                                       _D, _D]
        L.or_div_stats.argtypes = [C.POINTER(Grid), _D, _D, _D, _D, _D]
        L.or_sor_solve.argtypes = [C.POINTER(Grid), _D, _D, _D, _D, _D, C.c_double, C.c_double,
                                   C.c_int64, _D]
        L.or_sor_solve.restype = C.c_int64
        L.or_mg_default.argtypes = [C.POINTER(MGParams)]
        L.or_mg_plan.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int32)]
        L.or_mg_plan.restype = C.c_int
        L.or_mg_solve.argtypes = [C.POINTER(Grid), _D, _D, _D, _D, _D, C.c_double,
                                  C.POINTER(MGParams), C.POINTER(MGStats)]
        L.or_mg_solve.restype = C.c_int
        L.or_mg_level_coef.argtypes = [C.POINTER(Grid), _D, _D, _D, C.POINTER(MGParams), C.c_int,
                                       _D, _D, _D]
        L.or_mg_level_coef.restype = C.c_int
        L.or_adjoint.argtypes = [C.POINTER(Grid), _D, _D, _D, _D, C.c_double, C.c_double,
                                 C.c_double, _D, _D]
        L.or_ls_source.argtypes = [C.POINTER(Grid), _D, _D, _D, _D, _D]
        L.or_ls_advect.argtypes = [C.POINTER(Grid), _D, _D, _D, _D, C.c_double, C.c_int]
        L.or_ls_gradient.argtypes = [C.POINTER(Grid), _D, _D, _D]
        L.or_ls_redistance.argtypes = [C.POINTER(Grid), _D, C.c_double, C.c_double, C.c_double,
                                       C.c_int, C.c_int, _D]
        L.or_ls_redistance.restype = C.c_int
        _G, _N = C.POINTER(Grid), C.POINTER(NSParams)
        L.or_ns_diffusion.argtypes = [_G, _N] + [_D] * 14
        L.or_ns_advance.argtypes = [_G, _N] + [_D] * 18
        L.or_velbc.argtypes = [_G, C.c_int, C.POINTER(C.c_int32), _D, _D, _D]
        L.or_ns_vel_change.argtypes = [_G, C.c_int] + [_D] * 8
        L.or_ns_ab_step.argtypes = ([_G, _N] + [_D] * 22
                                    + [C.POINTER(MGParams), _D, _D, C.POINTER(C.c_int32)])
        L.or_ns_ab_step.restype = C.c_int
        L.or_ccd_decompose.argtypes = [C.c_int, C.c_double, _D, _D, _D, _D]
        L.or_ccd_line.argtypes = [C.c_int, C.c_double, _D, _D, _D, _D, _D, C.c_int64, _D, _D,
                                  C.c_int64]
        L.or_ns_bc.argtypes = [_G, C.c_int, _D]
        L.or_ns_curvature.argtypes = [_G, C.c_int, _D, _D, _D, _D, _D, _D]
        L.or_ns_mass_correct.argtypes = [_G, C.c_int, _D, C.c_double, C.c_double, C.c_double,
                                         C.c_int]
        L.or_ns_mass_correct.restype = C.c_double
        L.or_vof_wlic.argtypes = [_G, C.c_int, _D, _D, _D, _D, _D, _D, C.c_double]
        L.or_ns_ibm.argtypes = [_G, C.c_int, _D, C.c_double, _D, _D, _D]
        L.or_num_threads.restype = C.c_int
        L.or_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous, (a.dtype, a.flags)
    return a.ctypes.data_as(_D)


def grid(shape, spacing):
    nz, ny, nx = shape
    dx, dy, dz = spacing
    return Grid(nx, ny, nz, dx, dy, dz)


def heaviside(phi, eps):
    phi = np.ascontiguousarray(phi, np.float64)
    out = np.empty_like(phi)
    lib().or_heaviside(_p(phi), phi.size, eps, _p(out))
    return out


def heaviside_deriv(phi, eps):
    phi = np.ascontiguousarray(phi, np.float64)
    out = np.empty_like(phi)
    lib().or_heaviside_deriv(_p(phi), phi.size, eps, _p(out))
    return out


def rho_from_phi(phi, eps, rho_pos, rho_neg):
    phi = np.ascontiguousarray(phi, np.float64)
    out = np.empty_like(phi)
    lib().or_rho_from_phi(_p(phi), phi.size, eps, rho_pos, rho_neg, _p(out))
    return out


def face_coef(rho, spacing):
    rho = np.ascontiguousarray(rho, np.float64)
    g = grid(rho.shape, spacing)
    cx, cy, cz = (np.empty_like(rho) for _ in range(3))
    lib().or_face_coef(C.byref(g), _p(rho), _p(cx), _p(cy), _p(cz))
    return cx, cy, cz


def divergence(u, v, w, dt, spacing, remove_mean=True):
    nz, ny, nx1 = u.shape
    shape = (nz, ny, nx1 - 1)
    g = grid(shape, spacing)
    b = np.empty(shape)
    lib().or_divergence(C.byref(g), _p(u), _p(v), _p(w), dt, int(remove_mean), _p(b))
    return b


def apply(coef, p, spacing=(1.0, 1.0, 1.0)):
    cx, cy, cz = coef
    g = grid(p.shape, spacing)
    out = np.empty_like(p)
    lib().or_apply(C.byref(g), _p(cx), _p(cy), _p(cz), _p(p), _p(out))
    return out


def residual(coef, p, b):
    cx, cy, cz = coef
    g = grid(p.shape, (1.0, 1.0, 1.0))
    r = np.empty_like(p)
    s2 = lib().or_residual(C.byref(g), _p(cx), _p(cy), _p(cz), _p(p), _p(b), _p(r))
    return r, s2


def correct(rho, p, dt, u, v, w, spacing):
    g = grid(p.shape, spacing)
    u, v, w = (np.array(a, np.float64, copy=True) for a in (u, v, w))
    lib().or_correct(C.byref(g), _p(rho), _p(p), dt, _p(u), _p(v), _p(w))
    return u, v, w


def split_rhs(rho, u, v, w, p_hat, rho12, dt, spacing):
    """Source of the pressure-split projection (or_split_rhs)."""
    g = grid(rho.shape, spacing)
    src = np.empty_like(rho)
    lib().or_split_rhs(C.byref(g), _p(rho), _p(u), _p(v), _p(w), _p(p_hat), rho12, dt, _p(src))
    return src


def split_correct(rho, p, p_hat, rho12, dt, u, v, w, spacing):
    """ppe_mg_correction on copies of u, v, w (or_split_correct)."""
    g = grid(p.shape, spacing)
    u, v, w = (np.array(a, np.float64, copy=True) for a in (u, v, w))
    lib().or_split_correct(C.byref(g), _p(rho), _p(p), _p(p_hat), rho12, dt, _p(u), _p(v), _p(w))
    return u, v, w


def div_stats(u, v, w, spacing):
    nz, ny, nx1 = u.shape
    g = grid((nz, ny, nx1 - 1), spacing)
    mx, mean = C.c_double(), C.c_double()
    lib().or_div_stats(C.byref(g), _p(u), _p(v), _p(w), C.byref(mx), C.byref(mean))
    return mx.value, mean.value


def sor_solve(coef, b, p0=None, w=1.5, tol=1e-10, max_iter=10**6):
    cx, cy, cz = coef
    p = np.zeros_like(b) if p0 is None else np.array(p0, np.float64, copy=True)
    g = grid(b.shape, (1.0, 1.0, 1.0))
    err = C.c_double()
    it = lib().or_sor_solve(C.byref(g), _p(cx), _p(cy), _p(cz), _p(b), _p(p), w, tol, max_iter,
                            C.byref(err))
    return p, it, err.value


def mg_params(**kw):
    prm = MGParams()
    lib().or_mg_default(C.byref(prm))
    for k, v in kw.items():
        if k == "blocks":
            prm.blocks[:] = list(v)
        else:
            setattr(prm, k, v)
    return prm


def mg_plan(shape, levels=0, coarse_max=64):
    nz, ny, nx = shape
    dims = (C.c_int32 * 96)()
    L = lib().or_mg_plan(nx, ny, nz, levels, coarse_max, dims)
    if L < 1:
        return []
    return [(dims[3 * l + 2], dims[3 * l + 1], dims[3 * l]) for l in range(L)]


def mg_solve(coef, b, p0=None, tol=1e-10, **kw):
    """Returns (p, stats dict).  p is mean-free."""
    cx, cy, cz = coef
    p = np.zeros_like(b) if p0 is None else np.array(p0, np.float64, copy=True)
    g = grid(b.shape, (1.0, 1.0, 1.0))
    prm = mg_params(**kw)
    st = MGStats()
    lib().or_mg_solve(C.byref(g), _p(cx), _p(cy), _p(cz), _p(b), _p(p), tol, C.byref(prm),
                      C.byref(st))
    hist = [st.history[i] for i in range(min(st.cycles, 256))]
    return p, dict(cycles=st.cycles, levels=st.levels, status=st.status, coarse_n=st.coarse_n,
                   rel_residual=st.rel_residual, rms_residual=st.rms_residual, history=hist)


def mg_level_coef(coef, level, **kw):
    cx, cy, cz = coef
    shape = cx.shape
    plan = mg_plan(shape, kw.get("levels", 0), kw.get("coarse_max", 64))
    g = grid(shape, (1.0, 1.0, 1.0))
    prm = mg_params(**kw)
    out = [np.empty(plan[level]) for _ in range(3)]
    rc = lib().or_mg_level_coef(C.byref(g), _p(cx), _p(cy), _p(cz), C.byref(prm), level,
                                *(_p(a) for a in out))
    assert rc == 0
    return out


def adjoint(rho, p, lam, spacing, phi=None, eps=1.0, rho_pos=1.0, rho_neg=1.0):
    """(dJ/drho, dJ/dphi or None) from the solution p and the adjoint lam."""
    g = grid(p.shape, spacing)
    grad_rho = np.empty_like(p)
    grad_phi = np.empty_like(p) if phi is not None else None
    ph = np.ascontiguousarray(phi, np.float64) if phi is not None else None
    lib().or_adjoint(C.byref(g), _p(rho), _p(p), _p(lam), _p(ph), eps, rho_pos, rho_neg,
                     _p(grad_rho), _p(grad_phi))
    return grad_rho, grad_phi


def ls_source(phi, u, v, w, spacing):
    """L(phi) of level_set_rk3_source: WENO-JS split fluxes of u phi (cell-
    centred velocity u, v, w; w ignored for a 2D grid)."""
    phi = np.ascontiguousarray(phi, np.float64)
    g = grid(phi.shape, spacing)
    out = np.empty_like(phi)
    w_ = None if phi.shape[0] == 1 or w is None else np.ascontiguousarray(w, np.float64)
    lib().or_ls_source(C.byref(g), _p(phi), _p(np.ascontiguousarray(u, np.float64)),
                       _p(np.ascontiguousarray(v, np.float64)), _p(w_), _p(out))
    return out


def ls_advect(phi, u, v, w, dt, spacing, steps=1):
    """steps SSP-RK3 steps of level_set_rk3_solver; returns the new phi."""
    phi = np.array(phi, np.float64, order="C", copy=True)
    g = grid(phi.shape, spacing)
    w_ = None if phi.shape[0] == 1 or w is None else np.ascontiguousarray(w, np.float64)
    lib().or_ls_advect(C.byref(g), _p(phi), _p(np.ascontiguousarray(u, np.float64)),
                       _p(np.ascontiguousarray(v, np.float64)), _p(w_), float(dt), int(steps))
    return phi


def ls_gradient(phi, sign, spacing):
    """|grad phi| of level_set_redis_gradient (Godunov upwinding by sign)."""
    phi = np.ascontiguousarray(phi, np.float64)
    g = grid(phi.shape, spacing)
    out = np.empty_like(phi)
    lib().or_ls_gradient(C.byref(g), _p(phi), _p(np.ascontiguousarray(sign, np.float64)), _p(out))
    return out


def ls_redistance(phi, ls_wid, rdt, spacing, rho_12=1e-3, btn=1, max_iter=100000):
    """level_set_rk3_redis(btn); returns (phi, iterations, last max change)."""
    phi = np.array(phi, np.float64, order="C", copy=True)
    g = grid(phi.shape, spacing)
    err = C.c_double(0.0)
    it = lib().or_ls_redistance(C.byref(g), _p(phi), float(ls_wid), float(rdt), float(rho_12),
                                int(btn), int(max_iter), C.byref(err))
    return phi, it, err.value


def set_threads(n):
    lib().or_set_threads(int(n))


def num_threads():
    return lib().or_num_threads()


# --------------------------------------------------------------------------
# Momentum step (admas_bashforth_solver.f90 and its callees).  These arrays
# keep the reference's g ghost layers: padded shape (nz+2g, ny+2g, nx+2g) in 3D,
# (ny+2g, nx+2g) in 2D; element (i, j, k) of the reference's 1-based indices
# at [k-1+g, j-1+g, i-1+g]; u[.., .., i] is the face i+1/2.
# --------------------------------------------------------------------------
NS_OLD = ("u", "v", "w", "rho", "mu", "delta", "phi", "nrm_x", "nrm_y", "nrm_z", "curv")


def ns_params(ghost=3, bc=(1, 1, 1, 1, 1, 1), iterations=4, dt=1e-3, re=1000.0, fr=1.0, we=1.0,
              mu_12=1e-2, gravity=(0.0, -1.0, 0.0), btn_g=1.0, btn_sf=0.0, p_tol=1e-10,
              adv_scheme=0):
    return NSParams(int(ghost), (C.c_int32 * 6)(*[int(b) for b in bc]), int(iterations),
                    int(adv_scheme), float(dt), float(re), float(fr), float(we), float(mu_12),
                    float(gravity[0]), float(gravity[1]), float(gravity[2]), float(btn_g),
                    float(btn_sf), float(p_tol))


def padded_shape(shape, ghost):
    nz, ny, nx = shape
    if nz == 1:
        return (ny + 2 * ghost, nx + 2 * ghost)
    return (nz + 2 * ghost, ny + 2 * ghost, nx + 2 * ghost)


def _pad(a, shape, ghost, name):
    if a is None:
        return None
    a = np.ascontiguousarray(a, np.float64)
    if a.shape != padded_shape(shape, ghost):
        raise ValueError(f"{name}: expected {padded_shape(shape, ghost)}, got {a.shape}")
    return a


def _three(shape):
    return shape[0] > 1


def ns_diffusion(shape, spacing, prm, old):
    """velsrc%tmp of sec_part1..3 from the old fields (dict with NS_OLD keys;
    the normals and curv only needed when btn_sf != 0).  Returns (tu, tv, tw)."""
    g = grid(shape, spacing)
    G = prm.ghost
    f = {k: _pad(old.get(k), shape, G, k) for k in NS_OLD}
    if not _three(shape):
        f["w"] = f["nrm_z"] = None
    out = [np.zeros(padded_shape(shape, G)) for _ in range(3 if _three(shape) else 2)]
    tw = out[2] if _three(shape) else None
    lib().or_ns_diffusion(C.byref(g), C.byref(prm), *[_p(f[k]) for k in NS_OLD],
                          _p(out[0]), _p(out[1]), _p(tw))
    return out[0], out[1], tw


def ns_advance(shape, spacing, prm, old_vel, tmp_vel, diff, src_old):
    """One predictor pass: returns (src_now, vel_now) as tuples of padded arrays
    (vel_now's ghosts are copies of the old velocity's; velbc is separate)."""
    g = grid(shape, spacing)
    G = prm.ghost
    nc = 3 if _three(shape) else 2

    def tri(t, name):
        t = list(t) + [None] * (3 - len(t))
        return [_pad(t[c], shape, G, name) if c < nc else None for c in range(3)]

    o, t, d, so = tri(old_vel, "old"), tri(tmp_vel, "tmp"), tri(diff, "diff"), tri(src_old, "src")
    src = [np.zeros(padded_shape(shape, G)) if c < nc else None for c in range(3)]
    vel = [o[c].copy() if c < nc else None for c in range(3)]
    lib().or_ns_advance(C.byref(g), C.byref(prm), *[_p(a) for a in o + t + d + so + src + vel])
    return tuple(src[:nc]), tuple(vel[:nc])


def velbc(shape, prm, u, v, w=None):
    """velbc in place on padded arrays."""
    g = grid(shape, (1.0, 1.0, 1.0))
    for a in (u, v) + ((w,) if _three(shape) else ()):
        assert a.dtype == np.float64 and a.flags.c_contiguous
    lib().or_velbc(C.byref(g), int(prm.ghost), prm.bc, _p(u), _p(v),
                   _p(w) if _three(shape) else None)


def ns_ab_step(shape, spacing, prm, rho_now, vel, old, src_old, p, **mg_kw):
    """ns_ab_solver_SOR after ppe_sor_init.  vel: (u, v[, w]) padded vel%now
    (start of the linearisation); old: dict of the old padded fields (NS_OLD);
    src_old: velsrc%old; rho_now: compact new density (nz, ny, nx) of the
    pressure operator; p: compact warm start.  Returns a dict with u, v, w,
    su, sv, sw (padded), p, linf, l2f, cycles and status."""
    g = grid(shape, spacing)
    G = prm.ghost
    nc = 3 if _three(shape) else 2
    vel = [np.array(_pad(vel[c], shape, G, "vel"), copy=True) if c < nc else None
           for c in range(3)]
    f = {k: _pad(old.get(k), shape, G, k) for k in NS_OLD}
    so = [_pad(src_old[c], shape, G, "src_old") if c < nc else None for c in range(3)]
    if nc == 2:
        f["w"] = f["nrm_z"] = None
    src = [np.zeros(padded_shape(shape, G)) if c < nc else None for c in range(3)]
    pp = np.array(np.asarray(p, np.float64).reshape(shape), copy=True, order="C")
    rho = np.ascontiguousarray(np.asarray(rho_now, np.float64).reshape(shape))
    mgp = mg_params(**mg_kw)
    linf, l2f, cyc = C.c_double(), C.c_double(), C.c_int32()
    st = lib().or_ns_ab_step(C.byref(g), C.byref(prm), _p(rho), *[_p(a) for a in vel],
                             *[_p(f[k]) for k in ("u", "v", "w")], *[_p(a) for a in src],
                             *[_p(a) for a in so],
                             *[_p(f[k]) for k in ("rho", "mu", "delta", "phi", "nrm_x", "nrm_y",
                                                  "nrm_z", "curv")],
                             _p(pp), C.byref(mgp), C.byref(linf), C.byref(l2f), C.byref(cyc))
    return {"u": vel[0], "v": vel[1], "w": vel[2], "su": src[0], "sv": src[1], "sw": src[2],
            "p": pp, "linf": linf.value, "l2f": l2f.value, "cycles": cyc.value, "status": st}


def ccd_line(f, h):
    """root_solve("ccd") of one line: returns (f', f'')."""
    f = np.ascontiguousarray(f, np.float64)
    L = f.size
    mats = [np.zeros(3 * L) for _ in range(4)]
    lib().or_ccd_decompose(L, float(h), *[_p(m) for m in mats])
    fx, fxx = np.empty(L), np.empty(L)
    lib().or_ccd_line(L, float(h), *[_p(m) for m in mats], _p(f), 1, _p(fx), _p(fxx), 1)
    return fx, fxx


def ns_bc(shape, ghost, a):
    """bc (zero-gradient ghost copies) in place on a padded array."""
    g = grid(shape, (1.0, 1.0, 1.0))
    assert a.dtype == np.float64 and a.flags.c_contiguous
    lib().or_ns_bc(C.byref(g), int(ghost), _p(a))


def ns_curvature(shape, spacing, ghost, phi, want_d2=False):
    """curv + surface_norms on a padded phi: returns (phi_x, phi_y, phi_z or
    None, curv[, d2]) as padded arrays after bc; d2 = (fxx, fyy, fzz, fxy,
    fxz, fyz)."""
    g = grid(shape, spacing)
    phi = _pad(phi, shape, ghost, "phi")
    ps = padded_shape(shape, ghost)
    nx, ny, cv = np.zeros(ps), np.zeros(ps), np.zeros(ps)
    nz = np.zeros(ps) if _three(shape) else None
    d2 = np.zeros((6,) + ps)
    lib().or_ns_curvature(C.byref(g), int(ghost), _p(phi), _p(nx), _p(ny), _p(nz), _p(cv),
                          _p(d2))
    out = (nx, ny, nz, cv)
    return out + (tuple(d2),) if want_d2 else out


def ns_mass_correct(shape, spacing, ghost, phi, ls_wid, rho_12, imass, iterations=2):
    """mass_preserving_level_set on a copy of the padded phi: returns
    (phi, mass measured last); iterations = 0 gives ls_mv's mass only."""
    g = grid(shape, spacing)
    out = np.array(_pad(phi, shape, ghost, "phi"), copy=True)
    m = lib().or_ns_mass_correct(C.byref(g), int(ghost), _p(out), float(ls_wid), float(rho_12),
                                 float(imass), int(iterations))
    return out, m


def vof_wlic(shape, spacing, ghost, vof, vof_old, u, v, w, phi, dt):
    """vof_wlic_solver on a copy of the padded vof; returns it."""
    g = grid(shape, spacing)
    out = np.array(_pad(vof, shape, ghost, "vof"), copy=True)
    args = [_pad(a, shape, ghost, n) if a is not None else None
            for n, a in (("vof_old", vof_old), ("u", u), ("v", v),
                         ("w", w if _three(shape) else None), ("phi", phi))]
    lib().or_vof_wlic(C.byref(g), int(ghost), _p(out), *[_p(a) for a in args], float(dt))
    return out


def ns_ibm(shape, ghost, solid, w_body, u, v, w=None):
    """ibm_bc's forcing in place on padded arrays (solid gets its bc)."""
    g = grid(shape, (1.0, 1.0, 1.0))
    arrs = [solid, u, v] + ([w] if _three(shape) else [])
    for a in arrs:
        assert a.dtype == np.float64 and a.flags.c_contiguous
    lib().or_ns_ibm(C.byref(g), int(ghost), _p(solid), float(w_body), _p(u), _p(v),
                    _p(w) if _three(shape) else None)
