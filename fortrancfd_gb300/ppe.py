"""Host-side mirror of the reference's pressure routine, over libgbmg's C ABI.

The reference ("Two phase flows/newOpenMP/{2D,3D+IBM}/src/ns_solver/
ns_ppe_solver.f90") calls, once per Adams-Bashforth sub-iteration,

    call ppe_sor_init                 ! face coefficients 2/(rho_i+rho_nb)/h^2
    call ppe_sor_solver(p%glb%p_tol)  ! b = div(u*)/dt, iterate, then
                                      ! ns_momentum_correction: u -= dt grad(p)/rho_f

PressurePoisson keeps those names and meanings: ppe_init(rho) is
ppe_sor_init, ppe_solver(u, v, w, dt, tol, p) is ppe_sor_solver including the
momentum correction, rho_mu(phi, ...) is the density chain of
interface_solver/others.f90.  Where the reference STOPs the program
(non-convergence, ns_ppe_solver.f90:154-157) this raises ConvergenceError.

Arrays: numpy float64 arrays live in host memory; torch float64 CUDA tensors
are used in place on the device.  Cell arrays have shape (nz, ny, nx) (or
(ny, nx) in 2D); face velocities (nz, ny, nx+1), (nz, ny+1, nx),
(nz+1, ny, nx).  x must be contiguous; y and z strides are free, so views of
ghost-padded arrays work.  All work runs on the handle's own CUDA stream;
every call returns after its work finished.
"""
import ctypes as C

import numpy as np

from . import _lib

try:  # torch is optional for host-memory use
    import torch
except ImportError:  # pragma: no cover
    torch = None


class GBMGError(RuntimeError):
    """A libgbmg call failed (invalid argument, CUDA error, wrong call order)."""


class ConvergenceError(RuntimeError):
    """The solve did not reach the tolerance (the reference STOPs here)."""

    def __init__(self, msg, stats):
        super().__init__(msg)
        self.stats = stats


def _is_torch(a):
    return torch is not None and isinstance(a, torch.Tensor)


def _as3(a):
    if a is None:
        return None
    if a.ndim == 2:
        return a.reshape((1,) + tuple(a.shape)) if not _is_torch(a) else a.unsqueeze(0)
    if a.ndim != 3:
        raise ValueError(f"expected a 2D or 3D array, got shape {tuple(a.shape)}")
    return a


def _field(a, shape):
    """gbmg_field of an array whose logical extent is `shape` (nz, ny, nx)."""
    if a is None:
        return _lib.Field(None, 0, 0), None
    a = _as3(a)
    if tuple(a.shape) != tuple(shape):
        raise ValueError(f"expected shape {tuple(shape)}, got {tuple(a.shape)}")
    if _is_torch(a):
        if a.dtype != torch.float64:
            raise TypeError("tensors must be float64")
        if not a.is_cuda:
            a = a.contiguous().numpy()
        else:
            if a.stride(2) != 1:
                raise ValueError("x must be contiguous")
            return _lib.Field(a.data_ptr(), a.stride(1), a.stride(0)), _lib.GBMG_MEM_DEVICE
    if not isinstance(a, np.ndarray) or a.dtype != np.float64:
        raise TypeError("arrays must be float64 numpy arrays or torch tensors")
    if a.strides[2] != 8:
        raise ValueError("x must be contiguous")
    return _lib.Field(a.ctypes.data, a.strides[1] // 8, a.strides[0] // 8), _lib.GBMG_MEM_HOST


def _krylov_mode(krylov):
    """0 / False: stationary V-cycles; 1 / True / "fcg": flexible CG;
    2 / "fgmres": flexible GMRES(30), each with one V-cycle as preconditioner."""
    if isinstance(krylov, str):
        return {"none": 0, "fcg": 1, "fgmres": 2}[krylov]
    k = int(krylov)
    if k not in (0, 1, 2):
        raise ValueError("krylov must be 0, 1 (flexible CG) or 2 (flexible GMRES)")
    return k


def _mem_of(*pairs):
    mems = {m for _, m in pairs if m is not None}
    if len(mems) != 1:
        raise ValueError("all arrays of one call must be in the same memory (host or CUDA)")
    return mems.pop()


class PressurePoisson:
    """Variable-coefficient pressure-Poisson multigrid on one GB300.

    shape: (nz, ny, nx) cells (nz = 1 for 2D); spacing: (dx, dy, dz).
    precision: "fp64" (FP64 V-cycles) or "mixed" (FP32 V-cycles inside FP64
    defect correction).  krylov=True (or "fcg") wraps one V-cycle per
    iteration in flexible CG, krylov="fgmres" (or 2) in flexible GMRES(30),
    whose residual falls monotonically (faster on smooth right-hand sides such
    as adjoint solves).  stop_rule: "relative" (|b - A p|/|b| < tol),
    "rms" (the DomainDecomposition driver's absolute RMS residual < tol; pass
    p_tol*1e-3) or "increment" (max |p_k - p_(k-1)| < tol between cycles, the
    rule of ppe_sor_solver and PRESS_POISSON; pass p_tol).  zero_wall_faces:
    set the wall-normal faces of u, v, w to zero before the divergence, as
    MPLS_RisingBubble's RHSP does.  use_graph: True (or "loop") runs the
    cycle loop as one CUDA graph with the stopping tests on the device,
    "cycle" replays one graph per cycle and tests on the host, False launches
    each kernel.  inner_cycles: FP32 V-cycles per double-word defect
    correction of the stationary mixed loop (0: four, the last correction
    as many as predicted to reach tol; one under the increment rule).  split_restarts: the DomainDecomposition driver's restarts of a
    stagnating cycle in ppe_mg_solver (at most that many; 0: none).
    """

    def __init__(self, shape, spacing, precision="fp64", nu1=2, nu2=2, levels=0, coarse_max=64,
                 max_cycles=100, krylov=False, use_graph=True, remove_rhs_mean=True, certify=True,
                 device=None, stream=None, stop_rule="relative", zero_wall_faces=False,
                 inner_cycles=0, split_restarts=0):
        if len(shape) == 2:
            shape = (1,) + tuple(shape)
        self.shape = tuple(int(s) for s in shape)
        nz, ny, nx = self.shape
        if len(spacing) == 2:
            spacing = tuple(spacing) + (1.0,)
        self.spacing = tuple(float(s) for s in spacing)
        self.precision = precision
        L = _lib.load()
        self._L = L
        prm = _lib.Params()
        L.gbmg_default_params(C.byref(prm))
        prm.precision = {"fp64": _lib.GBMG_PREC_FP64, "mixed": _lib.GBMG_PREC_MIXED}[precision]
        prm.nu1, prm.nu2 = nu1, nu2
        prm.levels, prm.coarse_max, prm.max_cycles = levels, coarse_max, max_cycles
        prm.krylov = _krylov_mode(krylov)
        prm.use_graph = {True: 1, False: 0, "loop": 1, "cycle": 2}.get(use_graph, use_graph)
        prm.inner_cycles = int(inner_cycles)
        prm.split_restarts = int(split_restarts)
        prm.remove_rhs_mean = int(bool(remove_rhs_mean))
        prm.certify = int(bool(certify))
        prm.stop_rule = {"relative": _lib.GBMG_STOP_RELATIVE, "rms": _lib.GBMG_STOP_RMS,
                         "increment": _lib.GBMG_STOP_INCREMENT}[stop_rule]
        prm.zero_wall_faces = int(bool(zero_wall_faces))
        prm.device = -1 if device is None else int(device)
        # a torch.cuda.Stream, or a raw cudaStream_t handle; None = the handle's own stream
        prm.stream = getattr(stream, "cuda_stream", stream) or None
        if device is not None and torch is not None:
            torch.cuda.set_device(int(device))
        g = _lib.Grid(nx, ny, nz, *self.spacing)
        h = C.c_void_p()
        rc = L.gbmg_create(C.byref(g), C.byref(prm), C.byref(h))
        if rc != _lib.GBMG_OK:
            raise GBMGError(f"gbmg_create: {L.gbmg_strerror(rc).decode()}")
        self._h = h

    # -- lifetime --------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._L.gbmg_destroy(self._h)
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

    # -- helpers ---------------------------------------------------------------
    def _check(self, rc, what):
        if rc != _lib.GBMG_OK:
            msg = self._L.gbmg_last_error(self._h).decode()
            raise GBMGError(f"{what}: {self._L.gbmg_strerror(rc).decode()} {msg}".strip())

    @staticmethod
    def _sync_torch(*arrays):
        if torch is not None and any(_is_torch(a) and a.is_cuda for a in arrays if a is not None):
            torch.cuda.current_stream().synchronize()

    def _faces(self):
        nz, ny, nx = self.shape
        return (nz, ny, nx + 1), (nz, ny + 1, nx), (nz + 1, ny, nx)

    # -- coefficients (ppe_sor_init, rho_mu) -------------------------------------
    @staticmethod
    def _key(a, *extra):
        """Identity of an operator input: a CUDA tensor's storage, offset and
        version counter (so an in-place change is seen), or None."""
        if _is_torch(a) and a.is_cuda:
            return (a.data_ptr(), tuple(a.shape), tuple(a.stride()), a._version) + extra
        return None

    def ppe_init(self, rho):
        """ppe_sor_init: face coefficients 2/(rho_i + rho_nb)/h^2 from cell density."""
        f, m = _field(rho, self.shape)
        self._sync_torch(rho)
        self._op_key = None
        self._check(self._L.gbmg_set_rho(self._h, f, m), "ppe_init")
        self._op_key = self._key(rho, "rho")

    def rho_mu(self, phi, eps, rho_pos=1.0, rho_neg=1e-3):
        """rho_mu + ppe_sor_init: rho = rho_pos H(phi) + rho_neg (1 - H(phi))."""
        f, m = _field(phi, self.shape)
        self._sync_torch(phi)
        self._op_key = None
        self._check(self._L.gbmg_set_phi(self._h, f, eps, rho_pos, rho_neg, m), "rho_mu")
        self._op_key = self._key(phi, "phi", float(eps), float(rho_pos), float(rho_neg))

    def ensure_rho_mu(self, phi, eps, rho_pos=1.0, rho_neg=1e-3):
        """rho_mu, skipped when the operator was last built from this very
        tensor (same storage and version) with the same parameters."""
        key = self._key(phi, "phi", float(eps), float(rho_pos), float(rho_neg))
        if key is None or key != getattr(self, "_op_key", None):
            self.rho_mu(phi, eps, rho_pos, rho_neg)

    def ensure_ppe_init(self, rho):
        """ppe_init, skipped when the operator was last built from this tensor."""
        key = self._key(rho, "rho")
        if key is None or key != getattr(self, "_op_key", None):
            self.ppe_init(rho)

    def set_coef(self, cx, cy, cz):
        """Face coefficients given directly (cell-shaped low-face arrays)."""
        fx, m1 = _field(cx, self.shape)
        fy, m2 = _field(cy, self.shape)
        fz, m3 = _field(cz, self.shape)
        m = _mem_of((fx, m1), (fy, m2), (fz, m3))
        self._sync_torch(cx, cy, cz)
        self._op_key = None
        self._check(self._L.gbmg_set_coef(self._h, fx, fy, fz, m), "set_coef")

    # -- solves ------------------------------------------------------------------
    def solve(self, b, p=None, tol=1e-10, check=True):
        """Solve A p = b (p: initial guess, overwritten with the mean-free
        solution).  Returns (p, stats)."""
        if p is None:
            p = torch.zeros_like(b) if _is_torch(b) else np.zeros_like(b)
        fb, m1 = _field(b, self.shape)
        fp, m2 = _field(p, self.shape)
        m = _mem_of((fb, m1), (fp, m2))
        self._sync_torch(b, p)
        st = _lib.Stats()
        rc = self._L.gbmg_solve(self._h, fb, fp, float(tol), m, C.byref(st))
        stats = st.as_dict()
        self.last_stats = stats
        self._finish(rc, stats, check, "solve")
        return p, stats

    def ppe_solver(self, u, v, w, dt, tol=1e-10, p=None, check=True):
        """ppe_sor_solver + ns_momentum_correction: b = div(u*)/dt, solve, and
        correct u, v, w in place.  Returns (p, stats)."""
        if p is None:
            p = torch.zeros(self.shape, dtype=torch.float64, device=u.device) if _is_torch(u) \
                else np.zeros(self.shape)
        su, sv, sw = self._faces()
        fu, m1 = _field(u, su)
        fv, m2 = _field(v, sv)
        fw, m3 = _field(w if self.shape[0] > 1 else None, sw)
        fp, m4 = _field(p, self.shape)
        m = _mem_of((fu, m1), (fv, m2), (fp, m4), *(((fw, m3),) if m3 is not None else ()))
        self._sync_torch(u, v, w, p)
        st = _lib.Stats()
        rc = self._L.gbmg_project(self._h, fu, fv, fw, fp, float(dt), float(tol), m, C.byref(st))
        stats = st.as_dict()
        self._finish(rc, stats, check, "ppe_solver")
        return p, stats

    def ppe_mg_solver_init(self, rho, rho_12):
        """The pressure-split form of the DomainDecomposition solver
        (ppe_mg_solver_init): store rho and rho_12 and make the operator the
        constant-coefficient Laplacian.  ppe_init / rho_mu switch back."""
        f, m = _field(rho, self.shape)
        self._sync_torch(rho)
        self._op_key = None
        self._check(self._L.gbmg_set_split(self._h, f, float(rho_12), m), "ppe_mg_solver_init")

    def ppe_mg_solver(self, u, v, w, dt, p_hat, tol=1e-10, p=None, check=True):
        """ppe_mg_solver: split source from u* and p_hat, solve the Laplacian
        from p_hat, ppe_mg_correction on u, v, w in place.  Returns (p, stats)."""
        if p is None:
            p = torch.empty_like(p_hat) if _is_torch(p_hat) else np.empty(self.shape)
        su, sv, sw = self._faces()
        fu, m1 = _field(u, su)
        fv, m2 = _field(v, sv)
        fw, m3 = _field(w if self.shape[0] > 1 else None, sw)
        fh, m4 = _field(p_hat, self.shape)
        fp, m5 = _field(p, self.shape)
        m = _mem_of((fu, m1), (fv, m2), (fh, m4), (fp, m5),
                    *(((fw, m3),) if m3 is not None else ()))
        self._sync_torch(u, v, w, p_hat, p)
        st = _lib.Stats()
        rc = self._L.gbmg_project_split(self._h, fu, fv, fw, fh, fp, float(dt), float(tol), m,
                                        C.byref(st))
        stats = st.as_dict()
        self._finish(rc, stats, check, "ppe_mg_solver")
        return p, stats

    def _finish(self, rc, stats, check, what):
        if rc in (_lib.GBMG_OK,):
            return
        if rc in (_lib.GBMG_NOT_CONVERGED, _lib.GBMG_DIVERGED):
            if check:
                raise ConvergenceError(
                    f"{what}: {self._L.gbmg_strerror(rc).decode()} after {stats['cycles']} cycles, "
                    f"relative residual {stats['rel_residual']:.3e}", stats)
            return
        self._check(rc, what)

    def adjoint(self, p, lam, phi=None, eps=1.0, rho_pos=1.0, rho_neg=1e-3):
        """dJ/drho (and dJ/dphi when phi is given) from the solution p and the
        adjoint lam of A lam = dJ/dp, for the current density.  Returns
        (grad_rho, grad_phi or None)."""
        fp, m1 = _field(p, self.shape)
        fl, m2 = _field(lam, self.shape)
        like = (lambda: torch.empty_like(p)) if _is_torch(p) else (lambda: np.empty(self.shape))
        grad_rho = like()
        fr, _ = _field(grad_rho, self.shape)
        grad_phi = None
        fphi, fgp = _lib.Field(None, 0, 0), _lib.Field(None, 0, 0)
        pairs = [(fp, m1), (fl, m2)]
        if phi is not None:
            grad_phi = like()
            fphi, m3 = _field(phi, self.shape)
            fgp, _ = _field(grad_phi, self.shape)
            pairs.append((fphi, m3))
        m = _mem_of(*pairs)
        self._sync_torch(p, lam, phi)
        self._check(self._L.gbmg_adjoint(self._h, fp, fl, fphi, float(eps), float(rho_pos),
                                         float(rho_neg), fr, fgp, m), "adjoint")
        return grad_rho, grad_phi

    # -- diagnostics ------------------------------------------------------------
    def divergence(self, u, v, w, dt, out=None):
        su, sv, sw = self._faces()
        fu, m1 = _field(u, su)
        fv, m2 = _field(v, sv)
        fw, m3 = _field(w if self.shape[0] > 1 else None, sw)
        if out is None:
            out = torch.empty(self.shape, dtype=torch.float64, device=u.device) if _is_torch(u) \
                else np.empty(self.shape)
        fb, m4 = _field(out, self.shape)
        m = _mem_of((fu, m1), (fv, m2), (fb, m4), *(((fw, m3),) if m3 is not None else ()))
        self._sync_torch(u, v, w)
        self._check(self._L.gbmg_divergence(self._h, fu, fv, fw, float(dt), fb, m), "divergence")
        return out

    def residual(self, b, p, out=None, want_r=True):
        fb, m1 = _field(b, self.shape)
        fp, m2 = _field(p, self.shape)
        if want_r and out is None:
            out = torch.empty_like(b) if _is_torch(b) else np.empty(self.shape)
        fr, _ = _field(out, self.shape) if want_r else (_lib.Field(None, 0, 0), None)
        m = _mem_of((fb, m1), (fp, m2))
        n2 = C.c_double()
        self._sync_torch(b, p)
        self._check(self._L.gbmg_residual(self._h, fb, fp, fr, C.byref(n2), m), "residual")
        return out, n2.value

    def div_stats(self, u, v, w):
        su, sv, sw = self._faces()
        fu, m1 = _field(u, su)
        fv, m2 = _field(v, sv)
        fw, m3 = _field(w if self.shape[0] > 1 else None, sw)
        m = _mem_of((fu, m1), (fv, m2), *(((fw, m3),) if m3 is not None else ()))
        mx, mean = C.c_double(), C.c_double()
        self._sync_torch(u, v, w)
        self._check(self._L.gbmg_div_stats(self._h, fu, fv, fw, C.byref(mx), C.byref(mean), m),
                    "div_stats")
        return mx.value, mean.value

    def level_dims(self):
        n = C.c_int32()
        dims = (C.c_int32 * 96)()
        self._L.gbmg_level_dims(self._h, C.byref(n), dims, 32)
        return [(dims[3 * l + 2], dims[3 * l + 1], dims[3 * l]) for l in range(n.value)]

    def level_coef(self, level):
        shape = self.level_dims()[level]
        out = [np.empty(shape) for _ in range(3)]
        f = [_field(a, shape)[0] for a in out]
        self._check(self._L.gbmg_level_coef(self._h, level, *f, _lib.GBMG_MEM_HOST), "level_coef")
        return out

    @property
    def kernel_launches(self):
        return int(self._L.gbmg_kernel_launches(self._h))

    def set_profiling(self, on=True):
        """Time every launch with CUDA events, per kernel class (graphs off)."""
        self._check(self._L.gbmg_set_profiling(self._h, int(bool(on))), "set_profiling")

    def profile(self):
        """{class: (total ms, launches)} since profiling was switched on."""
        n = len(_lib.PROF_CLASSES)
        ms = (C.c_double * n)()
        cnt = (C.c_int64 * n)()
        self._check(self._L.gbmg_profile(self._h, ms, cnt, n), "profile")
        return {name: (ms[i], cnt[i]) for i, name in enumerate(_lib.PROF_CLASSES)}


def div_stats_noalloc(u, v, w, spacing, device=None, stream=None):
    """(max |div u|, mean |div u|) of face velocities in CUDA float64 tensors,
    through gbmg_div_stats_noalloc: no handle and no device allocation (the
    scratch is a static device array).  The first call on a device does a
    one-time set-up; calls from several host threads at once race on the
    shared scratch.  Work runs on `stream` (default: torch's current stream)
    and the call returns after it finished."""
    L = _lib.load()
    if torch is None or not all(_is_torch(a) and a.is_cuda for a in (u, v)):
        raise TypeError("div_stats_noalloc takes CUDA float64 tensors")
    u3, v3 = _as3(u), _as3(v)
    nz, ny, nx1 = u3.shape
    nx = nx1 - 1
    shape = (nz, ny, nx)
    fu, _ = _field(u3, (nz, ny, nx + 1))
    fv, _ = _field(v3, (nz, ny + 1, nx))
    fw, _ = _field(w if nz > 1 else None, (nz + 1, ny, nx))
    dx, dy = spacing[0], spacing[1]
    dz = spacing[2] if len(spacing) > 2 else 1.0
    g = _lib.Grid(nx, ny, nz, dx, dy, dz)
    dev = u3.device.index if device is None else device
    if stream is None:
        stream = torch.cuda.current_stream(u3.device).cuda_stream
    mx, mean = C.c_double(), C.c_double()
    err = C.create_string_buffer(256)
    rc = L.gbmg_div_stats_noalloc(C.byref(g), fu, fv, fw, C.byref(mx), C.byref(mean), dev,
                                  stream, err, len(err))
    if rc != _lib.GBMG_OK:
        raise GBMGError(f"div_stats_noalloc: {L.gbmg_strerror(rc).decode()}: "
                        f"{err.value.decode()} (shape {shape})")
    return mx.value, mean.value
