"""The Adams-Bashforth momentum step on the GPU (gbmg_ns_*, momentum.py)
against the CPU oracle's restatement (or_ns_*): the explicit part (sources,
predictor, velbc) is FP64 in the reference's operand order on both sides and
compared bit for bit; the whole step includes pressure solves to p_tol on both
sides and is compared to a tolerance that follows from it."""
import numpy as np
import pytest

from fortrancfd_gb300 import GBMGError, NSParams, PressurePoisson, inputs
from fortrancfd_gb300 import ns_ab_predictor, ns_ab_solver, velbc
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

G = 3


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def _setup(shape, seed=11, extent=None, sf=1.0, noise=0.01):
    nz, ny, nx = shape
    ext = extent or (1.0, ny / nx, (nz / nx) if nz > 1 else 1.0)
    case = inputs.custom(shape, extent=ext, centers=((0.5 * ext[0], 0.45 * ext[1], 0.5 * ext[2]),),
                         radii=(0.25 * min(ext[0], ext[1]),), seed=seed)
    st = inputs.momentum_state(case, ghost=G, amplitude=0.3)
    rng = np.random.default_rng(seed)
    for k in ("u", "v", "w"):  # ghosts as arbitrary as the interior
        if st[k] is not None:
            st[k] = st[k] + noise * rng.standard_normal(st[k].shape)
    st["p"] = 0.01 * rng.standard_normal(shape)
    prm = NSParams(dt=2e-3, re=100.0, fr=0.5, we=2.0, mu_12=1e-2, gravity=(0.3, -0.8, -0.5),
                   btn_g=1.0, btn_sf=sf, ghost=G, p_tol=1e-12)
    return case, st, prm


def _oprm(prm):
    return orc.ns_params(ghost=prm.ghost, bc=prm.bc, iterations=prm.iterations, dt=prm.dt,
                         re=prm.re, fr=prm.fr, we=prm.we, mu_12=prm.mu_12, gravity=prm.gravity,
                         btn_g=prm.btn_g, btn_sf=prm.btn_sf, p_tol=prm.p_tol,
                         adv_scheme=prm.adv_scheme)


def _state_for_lib(st, three):
    s = {"u": st["u"].copy(), "v": st["v"].copy(), "w": st["w"].copy() if three else None,
         "u_old": st["u"], "v_old": st["v"], "w_old": st["w"],
         "su_old": st["su_old"], "sv_old": st["sv_old"], "sw_old": st["sw_old"],
         "rho": st["rho"], "mu": st["mu"], "delta": st["delta"], "phi": st["phi"],
         "nrm_x": st["nrm_x"], "nrm_y": st["nrm_y"], "nrm_z": st["nrm_z"], "curv": st["curv"],
         "p": st["p"].copy()}
    s["su"] = np.zeros_like(st["u"])
    s["sv"] = np.zeros_like(st["v"])
    s["sw"] = np.zeros_like(st["u"]) if three else None
    return s


def _oracle_predict(case, st, prm):
    three = case.shape[0] > 1
    nc = 3 if three else 2
    op = _oprm(prm)
    diff = orc.ns_diffusion(case.shape, case.spacing, op, st)[:nc]
    old = tuple(st[k] for k in ("u", "v", "w")[:nc])
    so = tuple(st[k] for k in ("su_old", "sv_old", "sw_old")[:nc])
    src, vel = orc.ns_advance(case.shape, case.spacing, op, old, old, diff, so)
    vel = [a.copy() for a in vel] + [None] * (3 - nc)
    orc.velbc(case.shape, op, *vel[:nc])
    return src, vel


@pytest.mark.parametrize("shape", [(1, 24, 32), (6, 8, 8), (8, 12, 16)])
@pytest.mark.parametrize("sf", [0.0, 1.0])
def test_predictor_matches_oracle_bitwise(cuda, shape, sf):
    case, st, prm = _setup(shape, sf=sf)
    three = shape[0] > 1
    src, vel = _oracle_predict(case, st, prm)
    s = _state_for_lib(st, three)
    with PressurePoisson(shape, case.spacing) as pp:
        n0 = pp.kernel_launches
        ns_ab_predictor(pp, prm, s)
        assert pp.kernel_launches > n0
    for c, (k, sk) in enumerate(zip(("u", "v", "w"), ("su", "sv", "sw"))):
        if c == 2 and not three:
            break
        assert np.array_equal(_bits(s[k]), _bits(vel[c])), k
        # velsrc%now: interior written, ghosts as given (zeros)
        assert np.array_equal(_bits(s[sk]), _bits(src[c])), sk


@pytest.mark.parametrize("shape", [(1, 8, 5), (4, 8, 8), (6, 8, 10)])
@pytest.mark.parametrize("bc", [(1, 1, 1, 1, 1, 1), (2, 1, 1, 2, 2, 1), (0, 2, 1, 0, 1, 3)])
def test_velbc_matches_oracle_bitwise(cuda, shape, bc):
    import torch
    rng = np.random.default_rng(4)
    three = shape[0] > 1
    ps = orc.padded_shape(shape, G)
    f = [rng.standard_normal(ps) for _ in range(3 if three else 2)]
    want = [a.copy() for a in f]
    prm = NSParams(dt=1.0, ghost=G, bc=bc)
    orc.velbc(shape, _oprm(prm), *want)
    with PressurePoisson(shape, (0.1, 0.1, 0.1)) as pp:
        t = [torch.from_numpy(a).to(cuda) for a in f]
        velbc(pp, prm, *t)
        got = [a.cpu().numpy() for a in t]
        h = [a.copy() for a in f]
        velbc(pp, prm, *h)
    for c in range(len(f)):
        assert np.array_equal(_bits(got[c]), _bits(want[c])), c
        assert np.array_equal(_bits(h[c]), _bits(want[c])), c


def _compare_step(out, s, three, tol):
    for k in ("u", "v", "w")[: 3 if three else 2]:
        scale = np.abs(out[k]).max()
        np.testing.assert_allclose(s[k], out[k], rtol=0, atol=tol * scale, err_msg=k)
    for k in ("su", "sv", "sw")[: 3 if three else 2]:
        scale = np.abs(out[k]).max()
        np.testing.assert_allclose(s[k], out[k], rtol=0, atol=tol * scale, err_msg=k)


@pytest.mark.parametrize("shape", [(1, 32, 32), (16, 16, 16), (1, 48, 64)])
def test_step_matches_oracle(cuda, shape):
    """Whole step with FP64 solves to 1e-12 on both sides: velocities and
    sources agree to 1e-8 of their largest value, the pressure to 1e-7 of
    its, and the change statistics to 1e-6 (they measure a difference of
    iterates, 1e-5 of the velocity)."""
    case, st, prm = _setup(shape, sf=1.0)
    three = shape[0] > 1
    nc = 3 if three else 2
    vel = tuple(st[k] for k in ("u", "v", "w")[:nc])
    so = tuple(st[k] for k in ("su_old", "sv_old", "sw_old")[:nc])
    out = orc.ns_ab_step(case.shape, case.spacing, _oprm(prm), st["rho_now"], vel, st, so,
                         st["p"], krylov=1)
    assert out["status"] == 0
    s = _state_for_lib(st, three)
    with PressurePoisson(shape, case.spacing, krylov=True) as pp:
        pp.ppe_init(st["rho_now"])
        stats = ns_ab_solver(pp, prm, s)
    assert stats["status"] == 0 and stats["max_rel_residual"] < 1e-12
    _compare_step(out, s, three, 1e-8)
    p = s["p"].reshape(out["p"].shape)
    np.testing.assert_allclose(p, out["p"], rtol=0, atol=1e-7 * np.abs(out["p"]).max())
    assert stats["linf"] == pytest.approx(out["linf"], rel=1e-6)
    assert stats["l2f"] == pytest.approx(out["l2f"], rel=1e-6)


def test_step_on_device_tensors_mixed_precision(cuda):
    """Device-resident state (CUDA tensors) with the mixed-precision solve."""
    import torch
    shape = (16, 16, 16)
    case, st, prm = _setup(shape, sf=1.0)
    out = orc.ns_ab_step(case.shape, case.spacing, _oprm(prm), st["rho_now"],
                         (st["u"], st["v"], st["w"]), st, (st["su_old"], st["sv_old"],
                                                         st["sw_old"]), st["p"], krylov=1)
    s = _state_for_lib(st, True)
    t = {k: (torch.from_numpy(np.ascontiguousarray(a)).to(cuda) if a is not None else None)
         for k, a in s.items()}
    with PressurePoisson(shape, case.spacing, precision="mixed", krylov=True) as pp:
        pp.ppe_init(torch.from_numpy(st["rho_now"]).to(cuda))
        stats = ns_ab_solver(pp, prm, t)
    assert stats["status"] == 0
    got = {k: (a.cpu().numpy() if a is not None else None) for k, a in t.items()}
    _compare_step(out, got, True, 1e-8)


def test_step_two_iterations_and_slip_walls(cuda):
    shape = (1, 40, 40)
    case, st, prm = _setup(shape, sf=0.0)
    prm.iterations = 2
    prm.bc = (2, 2, 1, 2, 1, 1)
    op = _oprm(prm)
    out = orc.ns_ab_step(case.shape, case.spacing, op, st["rho_now"], (st["u"], st["v"]), st,
                         (st["su_old"], st["sv_old"]), st["p"], krylov=1)
    s = _state_for_lib(st, False)
    s["nrm_x"] = s["nrm_y"] = s["curv"] = None
    with PressurePoisson(shape, case.spacing, krylov=True) as pp:
        pp.ppe_init(st["rho_now"])
        ns_ab_solver(pp, prm, s)
    _compare_step(out, s, False, 1e-8)


def test_errors(cuda):
    shape = (1, 16, 16)
    case, st, prm = _setup(shape)
    s = _state_for_lib(st, False)
    with PressurePoisson(shape, case.spacing) as pp:
        with pytest.raises(GBMGError, match="density"):
            ns_ab_solver(pp, prm, s)   # no ppe_init yet
        pp.ppe_init(st["rho_now"])
        bad = NSParams(dt=prm.dt, ghost=1)
        with pytest.raises((GBMGError, ValueError)):
            ns_ab_solver(pp, bad, s)
        s2 = dict(s)
        big = np.zeros((s["mu"].shape[0], s["mu"].shape[1] + 4))
        s2["mu"] = big[:, :s["mu"].shape[1]]  # other strides than the rest
        with pytest.raises(GBMGError, match="strides"):
            ns_ab_solver(pp, prm, s2)


def test_two_ghost_layers_and_strided_views(cuda):
    """ghost = 2 (the stencils' minimum) and arrays that are views into larger
    allocations (strides wider than the padded box), on the device."""
    import torch
    g = 2
    shape = (6, 8, 8)
    case = inputs.custom(shape, extent=(1.0, 1.0, 0.75), centers=((0.5, 0.5, 0.4),),
                         radii=(0.25,), seed=3)
    st = inputs.momentum_state(case, ghost=g, amplitude=0.3)
    prm = NSParams(dt=2e-3, re=50.0, fr=0.5, we=2.0, btn_sf=1.0, ghost=g,
                   gravity=(0.0, 0.0, -1.0))
    op = orc.ns_params(ghost=g, dt=prm.dt, re=prm.re, fr=prm.fr, we=prm.we, mu_12=prm.mu_12,
                       gravity=prm.gravity, btn_g=prm.btn_g, btn_sf=prm.btn_sf)
    old = (st["u"], st["v"], st["w"])
    so = (st["su_old"], st["sv_old"], st["sw_old"])
    dif = orc.ns_diffusion(shape, case.spacing, op, st)
    src, vel = orc.ns_advance(shape, case.spacing, op, old, old, dif, so)
    vel = [a.copy() for a in vel]
    orc.velbc(shape, op, *vel)
    ps = orc.padded_shape(shape, g)

    def view(a):  # the padded box inside a wider allocation
        big = torch.full((ps[0], ps[1] + 3, ps[2] + 5), float("nan"), dtype=torch.float64,
                         device=cuda)
        v = big[:, 1:1 + ps[1], 2:2 + ps[2]]
        if a is not None:
            v.copy_(torch.from_numpy(a))
        else:
            v.zero_()
        return v

    s = {k: view(st[k]) for k in ("u", "v", "w", "rho", "mu", "delta", "phi", "nrm_x", "nrm_y",
                                   "nrm_z", "curv", "su_old", "sv_old", "sw_old")}
    s.update(u_old=view(st["u"]), v_old=view(st["v"]), w_old=view(st["w"]),
             su=view(None), sv=view(None), sw=view(None),
             p=torch.zeros(shape, dtype=torch.float64, device=cuda))
    with PressurePoisson(shape, case.spacing) as pp:
        ns_ab_predictor(pp, prm, s)
    for c, (k, sk) in enumerate(zip(("u", "v", "w"), ("su", "sv", "sw"))):
        assert np.array_equal(_bits(s[k].cpu().numpy()), _bits(vel[c])), k
        assert np.array_equal(_bits(s[sk].cpu().numpy()), _bits(src[c])), sk


def test_host_and_device_steps_agree(cuda):
    """The same step through host arrays (staged by the library) and through
    device tensors gives the same doubles."""
    import torch
    shape = (1, 32, 48)
    case, st, prm = _setup(shape, sf=1.0)
    s_host = _state_for_lib(st, False)
    s_dev = {k: (torch.from_numpy(np.ascontiguousarray(a)).to(cuda) if a is not None else None)
             for k, a in _state_for_lib(st, False).items()}
    with PressurePoisson(shape, case.spacing, krylov=True) as pp:
        pp.ppe_init(st["rho_now"])
        a = ns_ab_solver(pp, prm, s_host)
        b = ns_ab_solver(pp, prm, s_dev)
    for k in ("u", "v", "su", "sv", "p"):
        assert np.array_equal(_bits(s_host[k]), _bits(s_dev[k].cpu().numpy())), k
    assert a["linf"] == b["linf"] and a["cycles"] == b["cycles"]


@pytest.mark.parametrize("shape", [(1, 16, 24), (8, 12, 16)])
def test_ibm_forcing_matches_oracle_bitwise(cuda, shape):
    import torch
    from fortrancfd_gb300 import ibm_bc
    rng = np.random.default_rng(6)
    ps = orc.padded_shape(shape, G)
    three = shape[0] > 1
    solid = np.clip(rng.uniform(-0.5, 1.5, ps), 0.0, 1.0)
    vel = [rng.standard_normal(ps) for _ in range(3 if three else 2)]
    want_s, want = solid.copy(), [a.copy() for a in vel]
    orc.ns_ibm(shape, G, want_s, 0.3, *want)
    prm = NSParams(dt=1.0, ghost=G)
    with PressurePoisson(shape, (0.1, 0.1, 0.1)) as pp:
        t = [torch.from_numpy(a).to(cuda) for a in [solid] + vel]
        ibm_bc(pp, prm, t[0], t[1], t[2], t[3] if three else None, w_body=0.3)
        h = [a.copy() for a in [solid] + vel]
        ibm_bc(pp, prm, h[0], h[1], h[2], h[3] if three else None, w_body=0.3)
    for c, a in enumerate([want_s] + want):
        assert np.array_equal(_bits(t[c].cpu().numpy()), _bits(a)), c
        assert np.array_equal(_bits(h[c]), _bits(a)), c


def test_predictor_and_ccd_equal_the_golden_loops(cuda):
    """The GPU's predictor pass and CCD gradient on the stored 2D state equal
    the outputs of the literal loop restatement (tests/golden/
    momentum2d_12x10.npz) bit for bit."""
    import os
    from fortrancfd_gb300 import curv
    f = np.load(os.path.join(os.path.dirname(__file__), "golden", "momentum2d_12x10.npz"))
    g = int(f["ghost"])
    shape = tuple(int(x) for x in f["shape"])
    sp = tuple(float(x) for x in f["spacing"])
    st = {k[3:]: f[k].copy() for k in f.files if k.startswith("in_")}
    prm = NSParams(dt=float(f["prm_dt"]), re=float(f["prm_re"]), fr=float(f["prm_fr"]),
                   we=float(f["prm_we"]), mu_12=float(f["prm_mu_12"]),
                   gravity=(float(f["prm_gx"]), float(f["prm_gy"]), 0.0),
                   btn_g=float(f["prm_btn_g"]), btn_sf=float(f["prm_btn_sf"]), ghost=g,
                   bc=tuple(int(b) for b in f["prm_bc"]) + (1, 1))
    s = {"u": st["u"].copy(), "v": st["v"].copy(), "u_old": st["u"], "v_old": st["v"],
         "su": np.zeros_like(st["u"]), "sv": np.zeros_like(st["v"]), "su_old": st["su_old"],
         "sv_old": st["sv_old"], "rho": st["rho"], "mu": st["mu"], "delta": st["delta"],
         "phi": st["phi"], "nrm_x": st["nrm_x"], "nrm_y": st["nrm_y"], "curv": st["curv"],
         "p": np.zeros(shape[1:])}
    out = [np.zeros_like(st["phi"]) for _ in range(3)]
    with PressurePoisson(shape, sp) as pp:
        ns_ab_predictor(pp, prm, s)
        curv(pp, prm, st["phi"], out[0], out[1], None, out[2])
    for got, key in ((s["su"], "su"), (s["sv"], "sv"), (s["u"], "u_new"), (s["v"], "v_new"),
                     (out[0], "ccd_fx"), (out[1], "ccd_fy")):
        assert np.array_equal(_bits(got), _bits(f[key])), key
    np.testing.assert_allclose(out[2], f["ccd_curv"], rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize("shape", [(1, 24, 32), (8, 12, 16)])
def test_quick_predictor_matches_oracle_bitwise(cuda, shape):
    """The QUICK advection option (ns_ab_adv_source_quick)."""
    case, st, prm = _setup(shape, sf=1.0)
    prm.adv_scheme = 1
    three = shape[0] > 1
    src, vel = _oracle_predict(case, st, prm)
    s = _state_for_lib(st, three)
    with PressurePoisson(shape, case.spacing) as pp:
        ns_ab_predictor(pp, prm, s)
    for c, (k, sk) in enumerate(zip(("u", "v", "w"), ("su", "sv", "sw"))):
        if c == 2 and not three:
            break
        assert np.array_equal(_bits(s[k]), _bits(vel[c])), k
        assert np.array_equal(_bits(s[sk]), _bits(src[c])), sk
