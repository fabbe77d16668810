"""Level-set transport on the GPU: the advection step of the reference's
interface solver and its redistancing, level_set_rk3_solver ("Two phase flows/newOpenMP/2D/src/
interface_solver/level_set_rk3_solver.f90:1-186"; 3D "Two phase flows/
newOpenMP/3D+IBM/src/interface_solver/level_set_rk3_solver.f90:1-215") and
level_set_rk3_redis (".../level_set_rk3_redis.f90"), through the C ABI
(gbmg_ls_*).  phi is advanced in place, as the reference
advances p%loc%phi%now; u, v, w are the cell-centred velocities (the
reference's nvel; node_velocity() forms them from MAC faces as node_vel
does)."""
import ctypes as C

import numpy as np

from . import _lib
from .ppe import GBMGError, _field, _is_torch, _mem_of

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


def node_velocity(u, v, w=None):
    """Cell-centred velocity from MAC faces, node_vel
    ("Two phase flows/newOpenMP/3D+IBM/src/ns_solver/ns_solvers.f90:128-147"):
    the mean of a cell's two faces along each axis.  u: (nz, ny, nx+1),
    v: (nz, ny+1, nx), w: (nz+1, ny, nx) or None; numpy or torch."""
    un = 0.5 * (u[..., :-1] + u[..., 1:])
    vn = 0.5 * (v[:, :-1, :] + v[:, 1:, :])
    wn = None if w is None else 0.5 * (w[:-1] + w[1:])
    return un, vn, wn


class LevelSet:
    """Level-set advection on one GB300 (FP64, WENO-JS + SSP-RK3).

    shape: (nz, ny, nx) cells (nz = 1 for 2D); spacing: (dx, dy, dz)."""

    def __init__(self, shape, spacing, device=None, stream=None):
        if len(shape) == 2:
            shape = (1,) + tuple(shape)
        self.shape = tuple(int(s) for s in shape)
        if len(spacing) == 2:
            spacing = tuple(spacing) + (1.0,)
        self.spacing = tuple(float(s) for s in spacing)
        nz, ny, nx = self.shape
        L = _lib.load()
        self._L = L
        if device is not None and torch is not None:
            torch.cuda.set_device(int(device))
        g = _lib.Grid(nx, ny, nz, *self.spacing)
        h = C.c_void_p()
        st = getattr(stream, "cuda_stream", stream) or None
        rc = L.gbmg_ls_create(C.byref(g), -1 if device is None else int(device), st, C.byref(h))
        if rc != _lib.GBMG_OK:
            raise GBMGError(f"gbmg_ls_create: {L.gbmg_strerror(rc).decode()}")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.gbmg_ls_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def advect(self, phi, u, v, w=None, dt=1e-3, steps=1):
        """steps SSP-RK3 steps of dt: phi_t + div(u phi) = 0, phi in place.
        Returns phi."""
        fp, m1 = _field(phi, self.shape)
        fu, m2 = _field(u, self.shape)
        fv, m3 = _field(v, self.shape)
        fw, m4 = _field(w if self.shape[0] > 1 else None, self.shape)
        pairs = [(fp, m1), (fu, m2), (fv, m3)] + ([(fw, m4)] if m4 is not None else [])
        m = _mem_of(*pairs)
        if torch is not None and any(_is_torch(a) and a.is_cuda for a in (phi, u, v, w)
                                     if a is not None):
            torch.cuda.current_stream().synchronize()
        rc = self._L.gbmg_ls_advect(self._h, fp, fu, fv, fw, float(dt), int(steps), m)
        if rc != _lib.GBMG_OK:
            msg = self._L.gbmg_ls_last_error(self._h).decode()
            raise GBMGError(f"ls_advect: {self._L.gbmg_strerror(rc).decode()} {msg}".strip())
        return phi

    def redistance(self, phi, ls_wid, rdt, rho_12=1e-3, btn=1, max_iter=100000):
        """level_set_rk3_redis(btn) on phi in place (see gbmg_ls_redistance).
        Returns (phi, iterations, largest change of the last iteration)."""
        fp, m = _field(phi, self.shape)
        if torch is not None and _is_torch(phi) and phi.is_cuda:
            torch.cuda.current_stream().synchronize()
        it = C.c_int32(0)
        ch = C.c_double(0.0)
        rc = self._L.gbmg_ls_redistance(self._h, fp, float(ls_wid), float(rdt), float(rho_12),
                                        int(btn), int(max_iter), m, C.byref(it), C.byref(ch))
        if rc != _lib.GBMG_OK:
            msg = self._L.gbmg_ls_last_error(self._h).decode()
            raise GBMGError(f"ls_redistance: {self._L.gbmg_strerror(rc).decode()} {msg}".strip())
        return phi, it.value, ch.value

    @property
    def kernel_launches(self):
        return int(self._L.gbmg_ls_kernel_launches(self._h))
