"""The two-phase solver's time step on one GB300, every field device-resident.

The reference's time loop ("Two phase flows/newOpenMP/2D/src/main.f90:14-40",
3D "Two phase flows/newOpenMP/3D+IBM/src/main.f90") with the classical level
set (interface method 1, "…/src/interface_solver/interface_solver.f90:15-23")
is, per step,

    call p%switch                       ! old <- now for every time-recorded field
    call interface_solver               ! level_set_rk3_solver; level_set_rk3_redis(1)
                                        ! every fifth step; with MPLS (method 2, the
                                        ! input default) mass_preserving_level_set
    call ns_solver                      ! ns_init (rho_mu, curv), ns_ab_solver_SOR,
                                        ! ns_check_convergence_div, node_vel

TwoPhaseStep runs that sequence through the library's entry points: the
level-set advection and redistancing (LevelSet), rho_mu and the CCD curvature
(momentum.rho_mu, momentum.curv), the pressure operator from the new level set
(PressurePoisson.rho_mu), the momentum step with its four predictor-projection
passes (momentum.ns_ab_solver), the divergence statistics and the cell
velocity of the next advection.  Fields keep the reference's ghost layers
(shape (nz+2g, ny+2g, nx+2g); 2D (ny+2g, nx+2g)); torch supplies the device
memory, the switch copies and the cell average of node_vel.
"""
from dataclasses import dataclass

from .levelset import LevelSet, node_velocity
from .momentum import (NSParams, bc, curv, ibm_bc, ls_mv, mass_preserving_level_set,
                       ns_ab_solver, padded_shape, rho_mu, vof_wlic_solver)
from .ppe import PressurePoisson

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


@dataclass
class InterfaceParams:
    ls_wid: float            # smoothed-Heaviside half width (the reference's ls_wid)
    rho_12: float = 1e-3     # density ratio of fluid 2 (phi < 0) to fluid 1
    rdt: float = 0.0         # redistancing pseudo-time step (0: 0.25 dx, the input default)
    redis_every: int = 5     # level_set_rk3_redis(1) every this many steps (0: never)
    method: int = 1          # 1: classical level set, 2: MPLS (+ mass_preserving_level_set),
                             # 3: CLSVOF (VOF transport, rho and mu from the volume fraction)
    recon_every: int = 10    # CLSVOF: clsvof_recon every this many steps (the reference: 10;
                             # redistancing every redis_every = 3 otherwise)


class TwoPhaseStep:
    """shape (nz, ny, nx), spacing (dx, dy, dz); ns: NSParams of the momentum
    step; itf: InterfaceParams.  precision / krylov as PressurePoisson."""

    _TIMED = ("phi", "u", "v", "w", "su", "sv", "sw", "rho", "mu", "delta", "nrm_x", "nrm_y",
              "nrm_z", "curv", "vof")

    def __init__(self, shape, spacing, ns: NSParams, itf: InterfaceParams, precision="mixed",
                 krylov=False, device=None, stream=None):
        if torch is None or not torch.cuda.is_available():
            raise RuntimeError("TwoPhaseStep needs a CUDA device")
        self.shape, self.spacing = tuple(shape), tuple(spacing)
        self.ns, self.itf = ns, itf
        self.three = self.shape[0] > 1
        self.dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.stream = stream
        self.pp = PressurePoisson(shape, spacing, precision=precision, krylov=krylov,
                                  device=self.dev.index, stream=stream)
        self.ls = LevelSet(shape, spacing, device=self.dev.index, stream=stream)
        g = ns.ghost
        ps = padded_shape(shape, g)
        z = lambda: torch.zeros(ps, dtype=torch.float64, device=self.dev)  # noqa: E731
        self.now = {k: z() for k in self._TIMED}
        self.old = {k: z() for k in self._TIMED}
        if not self.three:
            for d in (self.now, self.old):
                d["w"] = d["sw"] = d["nrm_z"] = None
        self.p = torch.zeros(shape if self.three else shape[1:], dtype=torch.float64,
                             device=self.dev)
        self.nvel = None
        self.iter = 0
        self.stats = {}

    # -- views -------------------------------------------------------------------
    def _inner(self, a):
        """interior cells of a padded cell array (a strided view)."""
        g = self.ns.ghost
        nz, ny, nx = self.shape
        if self.three:
            return a[g:g + nz, g:g + ny, g:g + nx]
        return a[g:g + ny, g:g + nx].unsqueeze(0)

    def _faces(self, a, axis):
        """faces 0..n of one axis of a padded face array, interior in the others."""
        g = self.ns.ghost
        nz, ny, nx = self.shape
        sl = {0: (slice(g, g + nz), slice(g, g + ny), slice(g - 1, g + nx)),
              1: (slice(g, g + nz), slice(g - 1, g + ny), slice(g, g + nx)),
              2: (slice(g - 1, g + nz), slice(g, g + ny), slice(g, g + nx))}[axis]
        if self.three:
            return a[sl]
        return a[sl[1:]].unsqueeze(0)

    # -- set-up ------------------------------------------------------------------
    def load(self, phi, u, v, w=None, p=None, vof=None):
        """Initial state (padded arrays, numpy or torch): phi and the face
        velocity; the derived fields (rho, mu, delta, normals, curvature, cell
        velocity) are formed as the reference's problem_init leaves them, and
        velsrc starts at zero."""
        def put(dst, a):
            dst.copy_(torch.as_tensor(a, dtype=torch.float64))
        put(self.now["phi"], phi)
        put(self.now["u"], u)
        put(self.now["v"], v)
        if self.three:
            put(self.now["w"], w)
        if p is not None:
            self.p.copy_(torch.as_tensor(p, dtype=torch.float64).reshape(self.p.shape))
        for k in ("su", "sv", "sw"):
            if self.now[k] is not None:
                self.now[k].zero_()
        if vof is not None:
            put(self.now["vof"], vof)
        elif self.itf.method == 3:  # the smoothed Heaviside of phi
            x = self.now["phi"] / self.itf.ls_wid
            hv = 0.5 * (1.0 + x + torch.sin(torch.pi * x) / torch.pi)
            hv = torch.where(x > 1 - 1e-12, 1.0, torch.where(x < -1 + 1e-12, 0.0, hv))
            self.now["vof"].copy_(hv.clamp(0.0, 1.0))
        self._derived()
        self._node_vel()
        self.iter = 0
        # problem_init's imass: ls_mv of the initial level set
        self.imass = ls_mv(self.pp, self.ns, self.now["phi"], self.itf.ls_wid, self.itf.rho_12)
        self.mass = self.imass

    def _derived(self):
        itf, ns, n = self.itf, self.ns, self.now
        if itf.method == 3:
            # rho_mu with CLSVOF: heavy = vof (others.f90:50-52); delta from phi
            rho_mu(self.pp, ns, n["phi"], itf.ls_wid, itf.rho_12, None, None, n["delta"])
            hv = n["vof"]
            n["rho"].copy_(hv + itf.rho_12 * (1.0 - hv))
            n["mu"].copy_(hv + ns.mu_12 * (1.0 - hv))
        else:
            rho_mu(self.pp, ns, n["phi"], itf.ls_wid, itf.rho_12, n["rho"], n["mu"], n["delta"])
        if ns.btn_sf:
            curv(self.pp, ns, n["phi"], n["nrm_x"], n["nrm_y"], n["nrm_z"], n["curv"])

    def _node_vel(self):
        n = self.now
        u, v = self._faces(n["u"], 0), self._faces(n["v"], 1)
        w = self._faces(n["w"], 2) if self.three else None
        un, vn, wn = node_velocity(u, v, w)
        self.nvel = tuple(x.contiguous() if x is not None else None for x in (un, vn, wn))

    # -- one time step -----------------------------------------------------------
    def step(self, solid=None, w_body=0.0):
        """One time step; returns its statistics (momentum step, divergence).
        solid: a padded cell solid fraction for the 3D solver's immersed
        boundary (ibm_bc after the divergence check), w_body its vertical speed."""
        self.iter += 1
        ns, itf = self.ns, self.itf
        # p%switch
        for k in self._TIMED:
            if self.now[k] is not None:
                self.old[k].copy_(self.now[k])
        nvel_old = self.nvel
        # interface_solver: advection with the previous cell velocity, then
        # redistancing every redis_every steps
        phi = self.now["phi"]
        rdt = itf.rdt or 0.25 * self.spacing[0]
        if itf.method == 3:
            o = self.old
            vof_wlic_solver(self.pp, ns, self.now["vof"], o["vof"], o["u"], o["v"], o["w"], phi)
        self.ls.advect(self._inner(phi), *nvel_old, dt=ns.dt, steps=1)
        bc(self.pp, ns, phi)
        redis = 0
        if itf.method == 3 and itf.recon_every and self.iter % itf.recon_every == 0:
            redis = self._clsvof_recon(rdt)
        elif itf.redis_every and self.iter % itf.redis_every == 0:
            _, redis, _ = self.ls.redistance(self._inner(phi), itf.ls_wid, rdt, itf.rho_12, btn=1)
            bc(self.pp, ns, phi)
        if itf.method == 2:
            self.mass = mass_preserving_level_set(self.pp, ns, phi, itf.ls_wid, itf.rho_12,
                                                  self.imass, iterations=2)
        # ns_init: rho_mu (and the pressure operator from the new level set, or
        # from the volume fraction with CLSVOF), curv
        self._derived()
        if itf.method == 3:
            self.pp.ppe_init(self._inner(self.now["rho"]).contiguous())
        else:
            self.pp.rho_mu(self._inner(phi), itf.ls_wid, 1.0, itf.rho_12)
        # ns_ab_solver_SOR: vel%now starts as vel%old (the switch left it)
        o, n = self.old, self.now
        state = {"u": n["u"], "v": n["v"], "w": n["w"], "u_old": o["u"], "v_old": o["v"],
                 "w_old": o["w"], "su": n["su"], "sv": n["sv"], "sw": n["sw"],
                 "su_old": o["su"], "sv_old": o["sv"], "sw_old": o["sw"], "rho": o["rho"],
                 "mu": o["mu"], "delta": o["delta"], "phi": o["phi"], "nrm_x": o["nrm_x"],
                 "nrm_y": o["nrm_y"], "nrm_z": o["nrm_z"], "curv": o["curv"], "p": self.p}
        st = ns_ab_solver(self.pp, ns, state)
        # ns_check_convergence_div, node_vel
        u, v = self._faces(n["u"], 0), self._faces(n["v"], 1)
        w = self._faces(n["w"], 2) if self.three else None
        div_max, div_mean = self.pp.div_stats(u, v, w)
        if solid is not None:
            ibm_bc(self.pp, ns, solid, n["u"], n["v"], n["w"], w_body=w_body)
        self._node_vel()
        self.stats = dict(st, div_max=div_max, div_mean=div_mean, redistance_iterations=redis,
                          iter=self.iter, mass=self.mass)
        return self.stats

    def _clsvof_recon(self, rdt):
        """clsvof_recon (clsvof.f90:145-192): phi = 2 vof - 1 redistanced from
        scratch (btn 0) for 3 dx of pseudo time, taken where the old |phi| <
        ls_wid, then level_set_rk3_redis(1)."""
        itf, ns = self.itf, self.ns
        phi = self.now["phi"]
        keep = phi.clone()
        phi.copy_(2.0 * self.now["vof"] - 1.0)
        n, t = 0, 0.0
        while True:  # the reference's loop: time += rdt until time > 3 dx
            n += 1
            t += rdt
            if t > 3.0 * self.spacing[0]:
                break
        _, it0, _ = self.ls.redistance(self._inner(phi), itf.ls_wid, rdt, itf.rho_12, btn=0,
                                       max_iter=n)
        bc(self.pp, ns, phi)
        near = keep.abs() < itf.ls_wid
        keep[near] = phi[near]
        phi.copy_(keep)
        _, it1, _ = self.ls.redistance(self._inner(phi), itf.ls_wid, rdt, itf.rho_12, btn=1)
        bc(self.pp, ns, phi)
        return it0 + it1

    def close(self):
        for x in (self.pp, self.ls):
            x.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False
