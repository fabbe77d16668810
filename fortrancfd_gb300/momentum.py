"""Host-side mirror of the reference's Adams-Bashforth momentum step, over
libgbmg's C ABI.

The reference's velocity step ("Two phase flows/newOpenMP/2D/src/ns_solver/
admas_bashforth_solver.f90:40-67", 3D "Two phase flows/newOpenMP/3D+IBM/src/
ns_solver/admas_bashforth_solver.f90:43-70") is

    call ppe_sor_init
    do iter = 1, 4
        call ns_linearize      ! vel%tmp = vel%now, find_stag_vel
        call ns_ab_setup       ! velsrc%now = advection + diffusion (+ gravity, tension)
        call ns_ab_predictor   ! vel%now = vel%old + dt (1.5 velsrc%now - 0.5 velsrc%old); velbc
        call ppe_sor_solver(p%glb%p_tol)   ! projection + ns_momentum_correction; velbc
    end do
    call ns_check_convergence_vel

ns_ab_solver(pp, prm, state) runs that loop on the GPU after pp.ppe_init /
pp.rho_mu (ppe_sor_init) with the new density; ns_ab_predictor runs one
predictor pass without the projection and velbc fills the ghost layers.

Arrays keep the reference's ghost cells: every field of `state` except p is
the padded box, shape (nz+2g, ny+2g, nx+2g) (2D: (ny+2g, nx+2g)), with the
reference's element (i, j, k) at [k-1+g, j-1+g, i-1+g] and u[.., .., i] the
face i+1/2 (as the oracle's arrays).  numpy float64 arrays live in host memory,
torch float64 CUDA tensors are used in place; x must be contiguous and all
padded arrays must share their strides.  p is the interior pressure (nz, ny,
nx) (2D (ny, nx)).  state keys: u, v, w (vel%now, in/out), u_old, v_old, w_old,
su, sv, sw (velsrc%now, out), su_old, sv_old, sw_old, rho, mu, delta, phi
(the old fields), nrm_x, nrm_y, nrm_z, curv (only with surface tension) and p.
"""
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .ppe import ConvergenceError, GBMGError, _field, _is_torch

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


@dataclass
class NSParams:
    """The reference's p%glb values the step reads (input/default.txt)."""
    dt: float
    re: float = 1000.0
    fr: float = 1.0
    we: float = 1.0
    mu_12: float = 1e-2
    gravity: tuple = (0.0, -1.0, 0.0)
    btn_g: float = 1.0
    btn_sf: float = 0.0
    ghost: int = 3
    bc: tuple = (1, 1, 1, 1, 1, 1)   # ubc(1:2), vbc(1:2), wbc(1:2): 1 no-slip, 2 slip
    iterations: int = 4
    p_tol: float = 1e-10
    adv_scheme: int = 0   # 0 second-order upwind (the reference's choice), 1 QUICK

    def c_struct(self):
        return _lib.NSParams(int(self.ghost), (C.c_int32 * 6)(*[int(b) for b in self.bc]),
                             int(self.iterations), int(self.adv_scheme), float(self.dt),
                             float(self.re), float(self.fr),
                             float(self.we), float(self.mu_12), float(self.gravity[0]),
                             float(self.gravity[1]), float(self.gravity[2]), float(self.btn_g),
                             float(self.btn_sf), float(self.p_tol))


def padded_shape(shape, ghost):
    nz, ny, nx = shape
    if nz == 1:
        return (ny + 2 * ghost, nx + 2 * ghost)
    return (nz + 2 * ghost, ny + 2 * ghost, nx + 2 * ghost)


# face axis of each velocity-like field (0 = x, 1 = y, 2 = z), None for cells
_AXIS = {"u": 0, "v": 1, "w": 2, "u_old": 0, "v_old": 1, "w_old": 2, "su": 0, "sv": 1, "sw": 2,
         "su_old": 0, "sv_old": 1, "sw_old": 2}


def _padded_field(a, name, shape, g):
    """gbmg_field of a padded array at the address the ABI expects: interior
    cell (1,1,1), or face 0 of its axis for the velocity-like arrays."""
    if a is None:
        return _lib.Field(None, 0, 0), None
    want = padded_shape(shape, g)
    if tuple(a.shape) != want:
        raise ValueError(f"{name}: expected padded shape {want}, got {tuple(a.shape)}")
    three = len(want) == 3
    ix = [g] * len(want)       # numpy index of the reference's (1,1,1): [k, j, i]
    ax = _AXIS.get(name)
    if ax is not None:
        ix[len(want) - 1 - ax] -= 1
    if _is_torch(a):
        if a.dtype != torch.float64 or not a.is_cuda:
            raise TypeError(f"{name}: tensors must be float64 CUDA tensors")
        st = a.stride()
        if st[-1] != 1:
            raise ValueError(f"{name}: x must be contiguous")
        off = sum(i * s for i, s in zip(ix, st))
        sy = st[-2]
        sz = st[0] if three else sy * want[0]
        return _lib.Field(a.data_ptr() + 8 * off, sy, sz), _lib.GBMG_MEM_DEVICE
    if not isinstance(a, np.ndarray) or a.dtype != np.float64:
        raise TypeError(f"{name}: arrays must be float64 numpy arrays or torch tensors")
    st = [s // 8 for s in a.strides]
    if st[-1] != 1:
        raise ValueError(f"{name}: x must be contiguous")
    off = sum(i * s for i, s in zip(ix, st))
    sy = st[-2]
    sz = st[0] if three else sy * want[0]
    return _lib.Field(a.ctypes.data + 8 * off, sy, sz), _lib.GBMG_MEM_HOST


def _fields(pp, prm, state):
    shape = pp.shape
    three = shape[0] > 1
    f = _lib.NSFields()
    mems = set()
    for name in _lib.NS_FIELDS:
        a = state.get(name)
        if name == "p":
            fld, m = _field(a, shape)
        elif not three and name in ("w", "w_old", "sw", "sw_old", "nrm_z"):
            fld, m = _lib.Field(None, 0, 0), None
        elif name in ("nrm_x", "nrm_y", "nrm_z", "curv") and not prm.btn_sf:
            fld, m = _lib.Field(None, 0, 0), None
        else:
            if a is None:
                raise ValueError(f"state['{name}'] is missing")
            fld, m = _padded_field(a, name, shape, prm.ghost)
        setattr(f, name, fld)
        if m is not None:
            mems.add(m)
    if len(mems) != 1:
        raise ValueError("all arrays of one call must be in the same memory (host or CUDA)")
    return f, mems.pop()


def _sync(state):
    if torch is not None and any(_is_torch(a) and a.is_cuda for a in state.values()
                                 if a is not None):
        torch.cuda.current_stream().synchronize()


def ns_ab_solver(pp, prm: NSParams, state, check=True):
    """ns_ab_solver_SOR after ppe_sor_init (call pp.ppe_init(rho_now) or
    pp.rho_mu(phi_now, ...) first): velsrc%tmp, then prm.iterations passes of
    predictor + projection.  Updates u, v, w, su, sv, sw and p of `state` in
    place; returns the statistics (linf, l2f of the last pass, solve cycles,
    worst status).  Raises ConvergenceError where the reference would STOP."""
    f, m = _fields(pp, prm, state)
    _sync(state)
    c = prm.c_struct()
    st = _lib.NSStats()
    rc = pp._L.gbmg_ns_ab_step(pp._h, C.byref(c), C.byref(f), m, C.byref(st))
    stats = st.as_dict()
    if rc in (_lib.GBMG_NOT_CONVERGED, _lib.GBMG_DIVERGED):
        if check:
            raise ConvergenceError(f"ns_ab_solver: pressure solve status {rc}, relative residual "
                                   f"{stats['max_rel_residual']:.3e}", stats)
    elif rc != _lib.GBMG_OK:
        pp._check(rc, "ns_ab_solver")
    return stats


def ns_ab_predictor(pp, prm: NSParams, state):
    """One pass of ns_linearize + ns_ab_setup + ns_ab_predictor + velbc with
    vel%tmp = the given u, v, w (no projection)."""
    f, m = _fields(pp, prm, state)
    _sync(state)
    c = prm.c_struct()
    pp._check(pp._L.gbmg_ns_ab_predict(pp._h, C.byref(c), C.byref(f), m), "ns_ab_predictor")


def velbc(pp, prm: NSParams, u, v, w=None):
    """velbc in place on padded u, v (, w)."""
    three = pp.shape[0] > 1
    fu, m1 = _padded_field(u, "u", pp.shape, prm.ghost)
    fv, m2 = _padded_field(v, "v", pp.shape, prm.ghost)
    fw, m3 = _padded_field(w if three else None, "w", pp.shape, prm.ghost)
    mems = {m for m in (m1, m2, m3) if m is not None}
    if len(mems) != 1:
        raise ValueError("all arrays of one call must be in the same memory (host or CUDA)")
    _sync({"u": u, "v": v, "w": w})
    c = prm.c_struct()
    pp._check(pp._L.gbmg_ns_velbc(pp._h, C.byref(c), fu, fv, fw, mems.pop()), "velbc")


def curv(pp, prm: NSParams, phi, nrm_x, nrm_y, nrm_z, curvature):
    """curv + surface_norms: phi's gradient into nrm_x, nrm_y (nrm_z) and the
    curvature, by compact-difference line solves; padded arrays, in place
    (phi is read only).  nrm_z is ignored in 2D."""
    three = pp.shape[0] > 1
    fs, mems = [], set()
    for name, a in (("phi", phi), ("nrm_x", nrm_x), ("nrm_y", nrm_y),
                    ("nrm_z", nrm_z if three else None), ("curv", curvature)):
        fld, m = _padded_field(a, name, pp.shape, prm.ghost)
        fs.append(fld)
        if m is not None:
            mems.add(m)
    if len(mems) != 1:
        raise ValueError("all arrays of one call must be in the same memory (host or CUDA)")
    _sync({"phi": phi, "x": nrm_x, "y": nrm_y, "z": nrm_z, "c": curvature})
    c = prm.c_struct()
    pp._check(pp._L.gbmg_ns_curvature(pp._h, C.byref(c), *fs, mems.pop()), "curv")


def _one_memory(*pairs):
    mems = {m for _, m in pairs if m is not None}
    if len(mems) != 1:
        raise ValueError("all arrays of one call must be in the same memory (host or CUDA)")
    return mems.pop()


def rho_mu(pp, prm: NSParams, phi, ls_wid, rho_12, rho=None, mu=None, delta=None):
    """ls_funs + rho_mu over the padded box: rho, mu (viscosity ratio
    prm.mu_12) and delta of phi, into the given padded arrays (None skipped)."""
    fs = [_padded_field(a, n, pp.shape, prm.ghost)
          for n, a in (("phi", phi), ("rho", rho), ("mu", mu), ("delta", delta))]
    m = _one_memory(*fs)
    _sync({"phi": phi, "rho": rho, "mu": mu, "delta": delta})
    c = prm.c_struct()
    pp._check(pp._L.gbmg_ns_rho_mu(pp._h, C.byref(c), fs[0][0], float(ls_wid), float(rho_12),
                                   fs[1][0], fs[2][0], fs[3][0], m), "rho_mu")


def bc(pp, prm: NSParams, a):
    """bc: zero-gradient ghost layers of a padded cell array, in place."""
    f = _padded_field(a, "phi", pp.shape, prm.ghost)
    m = _one_memory(f)
    _sync({"a": a})
    c = prm.c_struct()
    pp._check(pp._L.gbmg_ns_bc(pp._h, C.byref(c), f[0], m), "bc")


def mass_preserving_level_set(pp, prm: NSParams, phi, ls_wid, rho_12, imass, iterations=2):
    """mass_preserving_level_set in place on the padded phi; returns the mass
    measured last (iterations=0: ls_mv's mass of phi, no correction)."""
    f = _padded_field(phi, "phi", pp.shape, prm.ghost)
    m = _one_memory(f)
    _sync({"phi": phi})
    c = prm.c_struct()
    mass = C.c_double(0.0)
    pp._check(pp._L.gbmg_ns_mass_correct(pp._h, C.byref(c), f[0], float(ls_wid), float(rho_12),
                                         float(imass), int(iterations), m, C.byref(mass)),
              "mass_preserving_level_set")
    return mass.value


def vof_wlic_solver(pp, prm: NSParams, vof, vof_old, u_old, v_old, w_old, phi):
    """vof_wlic_solver: the CLSVOF volume fraction advanced one step (prm.dt)
    in place; padded arrays (u_old, v_old, w_old the face velocities)."""
    three = pp.shape[0] > 1
    fs = [_padded_field(a, n, pp.shape, prm.ghost)
          for n, a in (("phi", vof), ("phi", vof_old), ("u", u_old), ("v", v_old),
                       ("w", w_old if three else None), ("phi", phi))]
    m = _one_memory(*fs)
    _sync({"vof": vof, "old": vof_old, "u": u_old, "v": v_old, "w": w_old, "phi": phi})
    c = prm.c_struct()
    pp._check(pp._L.gbmg_ns_vof_advect(pp._h, C.byref(c), *[f[0] for f in fs], m),
              "vof_wlic_solver")


def ibm_bc(pp, prm: NSParams, solid, u, v, w=None, w_body=0.0):
    """ibm_bc's forcing: bc on the padded solid fraction, then u, v (, w)
    scaled by (1 - face solid fraction), w (2D: v) plus s w_body; in place."""
    three = pp.shape[0] > 1
    fs = [_padded_field(a, n, pp.shape, prm.ghost)
          for n, a in (("phi", solid), ("u", u), ("v", v), ("w", w if three else None))]
    m = _one_memory(*fs)
    _sync({"s": solid, "u": u, "v": v, "w": w})
    c = prm.c_struct()
    pp._check(pp._L.gbmg_ns_ibm(pp._h, C.byref(c), fs[0][0], float(w_body), fs[1][0], fs[2][0],
                                fs[3][0], m), "ibm_bc")


def ls_mv(pp, prm: NSParams, phi, ls_wid, rho_12):
    """ls_mv's mass sum (H + rho_12 (1 - H)) H dv of a padded phi."""
    return mass_preserving_level_set(pp, prm, phi, ls_wid, rho_12, 0.0, iterations=0)


__all__ = ["NSParams", "ns_ab_solver", "ns_ab_predictor", "velbc", "curv", "rho_mu", "bc",
           "mass_preserving_level_set", "ls_mv", "vof_wlic_solver", "ibm_bc",
           "padded_shape",
           "ConvergenceError", "GBMGError"]
