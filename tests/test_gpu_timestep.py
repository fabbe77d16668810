"""The whole two-phase time step on the GPU (TwoPhaseStep: switch, level-set
advection, redistancing, rho_mu, CCD curvature, momentum step with four
projections, divergence check, cell velocity) against the same sequence of
the oracle's restatements, for a few steps.  The steps contain FP64 solves to
1e-12 and CUDA's sin/cos/pow, so the comparison is to a tolerance."""
import numpy as np
import pytest

from fortrancfd_gb300 import InterfaceParams, NSParams, TwoPhaseStep, inputs, node_velocity
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

G = 3


def _faces(a, axis, shape):
    nz, ny, nx = shape
    g = G
    three = nz > 1
    sl = {0: (slice(g, g + nz), slice(g, g + ny), slice(g - 1, g + nx)),
          1: (slice(g, g + nz), slice(g - 1, g + ny), slice(g, g + nx)),
          2: (slice(g - 1, g + nz), slice(g, g + ny), slice(g, g + nx))}[axis]
    return a[sl] if three else a[sl[1:]][None]


def _inner(a, shape):
    nz, ny, nx = shape
    g = G
    if nz > 1:
        return a[g:g + nz, g:g + ny, g:g + nx]
    return a[g:g + ny, g:g + nx][None]


def _oracle_run(case, st, ns, itf, steps):
    shape, sp = case.shape, case.spacing
    three = shape[0] > 1
    nc = 3 if three else 2
    op = orc.ns_params(ghost=G, bc=ns.bc, iterations=ns.iterations, dt=ns.dt, re=ns.re,
                       fr=ns.fr, we=ns.we, mu_12=ns.mu_12, gravity=ns.gravity, btn_g=ns.btn_g,
                       btn_sf=ns.btn_sf, p_tol=ns.p_tol)
    now = {k: (st[k].copy() if st.get(k) is not None else None)
           for k in ("phi", "u", "v", "w")}
    now["vof"] = orc.heaviside(st["phi"], itf.ls_wid)
    for k in ("su", "sv", "sw")[:nc]:
        now[k] = np.zeros_like(st["phi"])
    p = np.zeros(shape)

    def derived(n):
        H = n["vof"] if itf.method == 3 else orc.heaviside(n["phi"], itf.ls_wid)
        n["rho"] = H + itf.rho_12 * (1.0 - H)
        n["mu"] = H + ns.mu_12 * (1.0 - H)
        n["delta"] = orc.heaviside_deriv(n["phi"], itf.ls_wid)
        n["nrm_x"], n["nrm_y"], n["nrm_z"], n["curv"] = orc.ns_curvature(shape, sp, G, n["phi"])

    def nvel(n):
        f = [_faces(n[k], a, shape) for a, k in enumerate(("u", "v", "w")[:nc])]
        un, vn, wn = node_velocity(f[0], f[1], f[2] if three else None)
        return [np.ascontiguousarray(x) if x is not None else None for x in (un, vn, wn)]

    derived(now)
    vel = nvel(now)
    _, imass = orc.ns_mass_correct(shape, sp, G, now["phi"], itf.ls_wid, itf.rho_12, 0.0, 0)
    for it in range(1, steps + 1):
        old = {k: (a.copy() if a is not None else None) for k, a in now.items()}
        if itf.method == 3:
            now["vof"] = orc.vof_wlic(shape, sp, G, now["vof"], old["vof"], old["u"], old["v"],
                                      old.get("w"), now["phi"], ns.dt)
        phi_in = np.ascontiguousarray(_inner(now["phi"], shape))
        phi_in = orc.ls_advect(phi_in, vel[0], vel[1], vel[2], ns.dt, sp, steps=1)
        _inner(now["phi"], shape)[...] = phi_in
        orc.ns_bc(shape, G, now["phi"])
        if itf.method == 3 and it % itf.recon_every == 0:
            keep = now["phi"].copy()
            now["phi"] = 2.0 * now["vof"] - 1.0
            n, t = 0, 0.0
            while True:
                n += 1
                t += itf.rdt
                if t > 3.0 * sp[0]:
                    break
            phi_in = np.ascontiguousarray(_inner(now["phi"], shape))
            phi_in, _, _ = orc.ls_redistance(phi_in, itf.ls_wid, itf.rdt, sp, rho_12=itf.rho_12,
                                             btn=0, max_iter=n)
            _inner(now["phi"], shape)[...] = phi_in
            orc.ns_bc(shape, G, now["phi"])
            near = np.abs(keep) < itf.ls_wid
            keep[near] = now["phi"][near]
            now["phi"] = keep
            phi_in = np.ascontiguousarray(_inner(now["phi"], shape))
            phi_in, _, _ = orc.ls_redistance(phi_in, itf.ls_wid, itf.rdt, sp, rho_12=itf.rho_12,
                                             btn=1)
            _inner(now["phi"], shape)[...] = phi_in
            orc.ns_bc(shape, G, now["phi"])
        elif itf.redis_every and it % itf.redis_every == 0:
            phi_in = np.ascontiguousarray(_inner(now["phi"], shape))
            phi_in, _, _ = orc.ls_redistance(phi_in, itf.ls_wid, itf.rdt, sp, rho_12=itf.rho_12,
                                             btn=1)
            _inner(now["phi"], shape)[...] = phi_in
            orc.ns_bc(shape, G, now["phi"])
        if itf.method == 2:
            now["phi"], _ = orc.ns_mass_correct(shape, sp, G, now["phi"], itf.ls_wid, itf.rho_12,
                                                imass, 2)
        derived(now)
        if itf.method == 3:
            rho_now = np.ascontiguousarray(_inner(now["rho"], shape))
        else:
            rho_now = orc.rho_from_phi(np.ascontiguousarray(_inner(now["phi"], shape)),
                                       itf.ls_wid, 1.0, itf.rho_12)
        oldf = {k: old[k] for k in orc.NS_OLD}
        out = orc.ns_ab_step(shape, sp, op, rho_now, tuple(now[k] for k in ("u", "v", "w")[:nc]),
                             oldf, tuple(old[k] for k in ("su", "sv", "sw")[:nc]), p, krylov=1)
        for k in ("u", "v", "w", "su", "sv", "sw")[:2 * nc] if three else ("u", "v", "su", "sv"):
            now[k] = out[k]
        p = out["p"]
        vel = nvel(now)
    return now, p


@pytest.mark.parametrize("shape,method", [((1, 32, 32), 1), ((1, 32, 32), 2), ((16, 16, 16), 2),
                                          ((1, 32, 32), 3), ((16, 16, 16), 3)])
def test_time_steps_match_the_oracle_sequence(cuda, shape, method):
    nz, ny, nx = shape
    ext = (1.0, ny / nx, (nz / nx) if nz > 1 else 1.0)
    case = inputs.custom(shape, extent=ext, centers=((0.5, 0.45, 0.5 * ext[2]),), radii=(0.25,),
                         seed=9)
    st = inputs.momentum_state(case, ghost=G, amplitude=0.3)
    h = case.spacing[0]
    ns = NSParams(dt=2e-3, re=100.0, fr=0.5, we=2.0, mu_12=1e-2, btn_sf=1.0, ghost=G,
                  gravity=(0.0, 0.0, -1.0) if nz > 1 else (0.0, -1.0, 0.0), p_tol=1e-12)
    itf = InterfaceParams(ls_wid=1.5 * h, rho_12=1e-3, rdt=0.25 * h, redis_every=2,
                          method=method, recon_every=3)
    steps = 3
    want, p_or = _oracle_run(case, st, ns, itf, steps)
    with TwoPhaseStep(shape, case.spacing, ns, itf, precision="fp64", krylov=True) as ts:
        ts.load(st["phi"], st["u"], st["v"], st["w"],
                vof=orc.heaviside(st["phi"], itf.ls_wid))
        for _ in range(steps):
            stats = ts.step()
        got = {k: (a.cpu().numpy() if a is not None else None) for k, a in ts.now.items()}
        p = ts.p.cpu().numpy().reshape(p_or.shape)
    assert stats["status"] == 0 and stats["iter"] == steps
    assert stats["div_max"] < 1e-6
    scale = np.abs(want["phi"]).max()
    np.testing.assert_allclose(got["phi"], want["phi"], rtol=0, atol=1e-10 * scale)
    for k in ("u", "v", "w") if nz > 1 else ("u", "v"):
        np.testing.assert_allclose(got[k], want[k], rtol=0, atol=1e-7 * np.abs(want[k]).max(),
                                   err_msg=k)
    np.testing.assert_allclose(got["curv"], want["curv"], rtol=0,
                               atol=1e-7 * np.abs(want["curv"]).max())
    np.testing.assert_allclose(p, p_or, rtol=0, atol=1e-6 * np.abs(p_or).max())
    if method == 3:
        np.testing.assert_allclose(got["vof"], want["vof"], rtol=0, atol=1e-10)


@pytest.mark.parametrize("shape", [(1, 40, 48), (16, 16, 24)])
def test_mass_correction_matches_the_oracle(cuda, shape):
    import torch
    from fortrancfd_gb300 import PressurePoisson, ls_mv, mass_preserving_level_set
    nz, ny, nx = shape
    h = 1.0 / nx
    ps = orc.padded_shape(shape, G)
    grids = np.meshgrid(*[(np.arange(m) - G + 0.5) * h for m in ps], indexing="ij")
    phi = 0.22 - np.sqrt(sum((a - 0.4) ** 2 for a in grids))
    sp = (h, h, h)
    prm = NSParams(dt=1.0, ghost=G)
    _, m0 = orc.ns_mass_correct(shape, sp, G, phi, 1.5 * h, 1e-3, 0.0, 0)
    shifted = phi + 0.3 * h
    want, mw = orc.ns_mass_correct(shape, sp, G, shifted, 1.5 * h, 1e-3, m0, 2)
    with PressurePoisson(shape, sp) as pp:
        t = torch.from_numpy(shifted).to(cuda)
        assert ls_mv(pp, prm, torch.from_numpy(phi).to(cuda), 1.5 * h, 1e-3) == \
            pytest.approx(m0, rel=1e-13)
        mg = mass_preserving_level_set(pp, prm, t, 1.5 * h, 1e-3, m0, iterations=2)
        hostarr = shifted.copy()
        mass_preserving_level_set(pp, prm, hostarr, 1.5 * h, 1e-3, m0, iterations=2)
    assert mg == pytest.approx(mw, rel=1e-13)
    np.testing.assert_allclose(t.cpu().numpy(), want, rtol=0, atol=1e-13 * np.abs(want).max())
    np.testing.assert_array_equal(hostarr, t.cpu().numpy())


@pytest.mark.parametrize("shape", [(1, 40, 48), (16, 16, 24)])
def test_vof_transport_matches_the_oracle(cuda, shape):
    import torch
    from fortrancfd_gb300 import PressurePoisson, vof_wlic_solver
    nz, ny, nx = shape
    h = 1.0 / nx
    ps = orc.padded_shape(shape, G)
    grids = np.meshgrid(*[(np.arange(m) - G + 0.5) * h for m in ps], indexing="ij")
    phi = 0.2 - np.sqrt(sum((a - 0.4) ** 2 for a in grids))
    vof = orc.heaviside(phi, 1.5 * h)
    rng = np.random.default_rng(4)
    vel = [0.3 * rng.standard_normal(ps) for _ in range(3 if nz > 1 else 2)]
    dt = 0.1 * h
    want = orc.vof_wlic(shape, (h, h, h), G, vof, vof, *vel, *([None] if nz == 1 else []), phi, dt)
    prm = NSParams(dt=dt, ghost=G)
    with PressurePoisson(shape, (h, h, h)) as pp:
        t = [torch.from_numpy(a).to(cuda) for a in [vof, vof] + vel + [phi]]
        w = t[4] if nz > 1 else None
        vof_wlic_solver(pp, prm, t[0], t[1], t[2], t[3], w, t[-1])
        host = vof.copy()
        vof_wlic_solver(pp, prm, host, vof, *vel, *([None] if nz == 1 else []), phi)
    got = t[0].cpu().numpy()
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-13)
    np.testing.assert_array_equal(host, got)
    assert got.min() >= 0.0 and got.max() <= 1.0


def test_mass_correction_without_an_interface_is_an_error(cuda):
    from fortrancfd_gb300 import GBMGError, PressurePoisson, mass_preserving_level_set
    shape = (1, 16, 16)
    ps = orc.padded_shape(shape, G)
    phi = np.ones(ps)  # no cell within ls_wid of the interface
    with PressurePoisson(shape, (1 / 16, 1 / 16, 1.0)) as pp:
        with pytest.raises(GBMGError, match="no interface cells"):
            mass_preserving_level_set(pp, NSParams(dt=1.0, ghost=G), phi, 1.5 / 16, 1e-3, 1.0)
    assert np.all(phi == 1.0)


def test_stationary_mixed_cycle_certifies_every_solve_of_a_128_cube_step(cuda):
    """The 128^3 sphere's time step (MPLS, dt 2e-4, four warm-started mixed
    projections per step to 1e-10) with the stationary mixed cycle, not a
    Krylov outer iteration: every solve of every step ends certified below
    1e-10 in FP64.  Warm starts run as correction solves from the FP64
    initial residual, and a certification above the tolerance sends the loop
    round again from the certified pressure, so the double-word floor of the
    tracked residual no longer decides the outcome."""
    case = inputs.config(1, 2)
    rho_12 = min(case.rho_pos, case.rho_neg) / max(case.rho_pos, case.rho_neg)
    st = inputs.momentum_state(case, ghost=G, rho_12=rho_12, mu_12=1e-2, amplitude=0.1)
    ns = NSParams(dt=2e-4, re=1000.0, fr=0.4096, we=1000.0, mu_12=1e-2,
                  gravity=(0.0, 0.0, -1.0), btn_g=1.0, btn_sf=1.0, ghost=G, iterations=4,
                  p_tol=1e-10)
    itf = InterfaceParams(ls_wid=case.eps, rho_12=rho_12, rdt=0.25 * case.spacing[0],
                          redis_every=5, method=2)
    with TwoPhaseStep(case.shape, case.spacing, ns, itf, precision="mixed",
                      krylov=False) as ts:
        ts.load(st["phi"], st["u"], st["v"], st["w"])
        for _ in range(4):
            stats = ts.step()
            assert stats["status"] == 0, stats
            assert stats["max_rel_residual"] < 1e-10, stats
    assert stats["div_max"] < 1e-6
