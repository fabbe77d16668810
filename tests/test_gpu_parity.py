"""GPU parity tests: the CUDA path through the C ABI against the CPU oracle on
the same seeded inputs.

Tolerances (floating point):
  * set-up kernels (face coefficients, coarse coefficients, divergence,
    correction formulas) do the oracle's arithmetic in the same order and are
    compared bit for bit, except rho(phi) (CUDA's sin vs the C library's, 1e-14);
  * the residual differs by FMA contraction: 1e-12 relative to max|b|;
  * plain FP64 solve: mean-free pressure within 1e-9 relative L2 of the
    oracle's and the same cycle count +/- 1;
  * mixed precision (FP32 cycles inside FP64 defect correction): the same
    1e-10 relative residual in FP64, pressure within 1e-9 relative L2 of the
    FP64 oracle solution;
  * the FP64 iterate after k = 1, 2, 3 cycles: within 1e-12 relative L2 of the
    oracle's iterate after the same cycles (restriction, prolongation and the
    coarse solve each enter every cycle, so a slip in any shows here);
  * against the reference's own cycle (lexicographic Gauss-Seidel in
    subdomains): pressure within 1e-9 relative L2, cycles within one in 3D.
"""
import numpy as np
import pytest

from fortrancfd_gb300 import ConvergenceError, GBMGError, PressurePoisson, inputs
from oracle import oracle as orc
from tests import cases
from tests.cases import rel_l2

pytestmark = pytest.mark.gpu


def solver(built, **kw):
    return PressurePoisson(built.shape, built.spacing, **kw)


# --- set-up kernels ----------------------------------------------------------------
@pytest.mark.parametrize("idx,scale", [(0, 1), (1, 8), (4, 8)])
def test_face_coefficients_bitwise(cuda, idx, scale):
    c = cases.config(idx, scale)
    with solver(c) as s:
        s.ppe_init(c.rho)
        got = s.level_coef(0)
        for a, b in zip(got, c.coef):
            np.testing.assert_array_equal(a, b)
        for lev, dims in enumerate(s.level_dims()):
            want = orc.mg_level_coef(c.coef, lev)
            got = s.level_coef(lev)
            assert got[0].shape == dims
            for a, b in zip(got, want):
                np.testing.assert_array_equal(a, b)
        assert s.level_dims() == orc.mg_plan(c.shape)


def test_rho_from_phi(cuda):
    c = cases.config(1, 8)
    with solver(c) as s:
        s.rho_mu(c.phi, c.case.eps, c.case.rho_pos, c.case.rho_neg)
        got = s.level_coef(0)
        for a, b in zip(got, c.coef):
            np.testing.assert_allclose(a, b, rtol=1e-13, atol=0)
        # faces between two cells outside the interface band take the
        # precomputed bulk values: those must be bit-identical to the oracle's
        bulk = np.abs(c.phi) > c.case.eps * (1 + 1e-9)
        for ax, (a, b) in enumerate(zip(got, c.coef)):
            axis = 2 - ax
            both = bulk.copy()
            sl_hi = [slice(None)] * 3
            sl_lo = [slice(None)] * 3
            sl_hi[axis] = slice(1, None)
            sl_lo[axis] = slice(None, -1)
            both[tuple(sl_hi)] &= bulk[tuple(sl_lo)]
            assert both.sum() > 0
            np.testing.assert_array_equal(a[both], b[both])


@pytest.mark.parametrize("idx,scale", [(0, 2), (1, 8)])
def test_divergence_bitwise(cuda, idx, scale):
    c = cases.config(idx, scale)
    with solver(c) as s:
        got = s.divergence(c.u, c.v, c.w, c.case.dt)
    want = orc.divergence(c.u, c.v, c.w, c.case.dt, c.spacing, remove_mean=False)
    np.testing.assert_array_equal(got, want)


def test_residual(cuda):
    c = cases.config(1, 8)
    p = np.random.default_rng(7).standard_normal(c.shape)
    with solver(c) as s:
        s.ppe_init(c.rho)
        r, n2 = s.residual(c.b, p)
    r_or, n2_or = orc.residual(c.coef, p, c.b)
    np.testing.assert_allclose(r, r_or, rtol=0, atol=1e-12 * np.abs(c.b).max())
    assert n2 == pytest.approx(n2_or, rel=1e-12)


# --- solves -------------------------------------------------------------------------
@pytest.mark.parametrize("idx,scale", [(0, 1), (1, 4), (1, 2)])
def test_fp64_solve_matches_oracle(cuda, idx, scale):
    c = cases.config(idx, scale)
    p_or, st_or = orc.mg_solve(c.coef, c.b, tol=1e-10)
    assert st_or["status"] == 0
    with solver(c) as s:
        s.ppe_init(c.rho)
        p, st = s.solve(c.b, tol=1e-10)
    assert st["status"] == 0 and st["rel_residual"] < 1e-10
    assert abs(st["cycles"] - st_or["cycles"]) <= 1, (st["cycles"], st_or["cycles"])
    assert rel_l2(p, p_or) <= 1e-9
    assert abs(p.mean()) <= 1e-12 * np.abs(p).max()


@pytest.mark.parametrize("idx,scale", [(0, 1), (1, 4)])
def test_fp64_iterates_after_each_cycle_match_oracle(cuda, idx, scale):
    """The FP64 iterate after k = 1, 2, 3 V(2,2) cycles from zero against the
    oracle's after the same cycles (tol too small to stop).  Every cycle goes
    through restriction, the coarse solve and prolongation on every level, so
    a slip in any of them that still converges within a cycle shows here."""
    c = cases.config(idx, scale)
    scale_b = np.linalg.norm(c.b)
    for k in (1, 2, 3):
        p_or, st_or = orc.mg_solve(c.coef, c.b, tol=1e-300, max_cycles=k)
        assert st_or["cycles"] == k
        with solver(c, max_cycles=k) as s:
            s.ppe_init(c.rho)
            p, st = s.solve(c.b, tol=1e-300, check=False)
        assert st["cycles"] == k and st["status"] == 1, st
        # the iterate is far from converged: compare it and its residual
        assert rel_l2(p - p.mean(), p_or - p_or.mean()) <= 1e-12, k
        assert st["rel_residual"] == pytest.approx(st_or["rel_residual"], rel=1e-9), k
        _, r2 = orc.residual(c.coef, p, c.b)
        assert np.sqrt(r2) / scale_b == pytest.approx(st_or["rel_residual"], rel=1e-9)


@pytest.mark.parametrize("idx,scale,blocks,max_gap", [
    (1, 4, (2, 2, 2), 1), (1, 4, (1, 2, 4), 1), (1, 2, (2, 2, 2), 1), (0, 1, (1, 2, 2), 2)])
def test_fp64_solve_matches_reference_lexicographic_cycle(cuda, idx, scale, blocks, max_gap):
    """The GPU's red-black FP64 cycle against the reference's own cycle: V(2,2)
    with lexicographic Gauss-Seidel inside OpenMP subdomains (the oracle's
    restatement of multigrid_relax over DomainDecomposition's blocks), both
    solved from zero to 1e-10.  The pressures agree to 1e-9 relative L2
    (measured: 2e-11 to 2e-10); the cycle counts differ by at most one in 3D.
    On the 2D bubble the lexicographic cycle converges in two fewer cycles
    (14 against 16): the red-black colouring smooths a little less per sweep
    there."""
    c = cases.config(idx, scale)
    p_lex, st_lex = orc.mg_solve(c.coef, c.b, tol=1e-10, smoother=1, blocks=blocks)
    assert st_lex["status"] == 0
    with solver(c) as s:
        s.ppe_init(c.rho)
        p, st = s.solve(c.b, tol=1e-10)
    assert st["status"] == 0
    gap = rel_l2(p - p.mean(), p_lex - p_lex.mean())
    print(f"lexicographic {blocks}: cycles GPU {st['cycles']} / lex {st_lex['cycles']}, "
          f"relative L2 gap {gap:.2e}")
    assert gap <= 1e-9
    assert abs(st["cycles"] - st_lex["cycles"]) <= max_gap, (st["cycles"], st_lex["cycles"])


@pytest.mark.parametrize("idx,scale", [(1, 4), (0, 1)])
def test_mixed_warm_start_far_from_the_solution(cuda, idx, scale):
    """A warm start whose A p is 10^4 times the right-hand side (as in the later
    passes of a time step, where the predicted velocity is nearly
    divergence-free but the pressure is not small): the mixed solve works on
    the correction from the FP64 initial residual, so the double-word
    operator's rounding scales with the correction, not with p, and the solve
    still certifies 1e-10 in FP64 and meets the oracle's pressure."""
    c = cases.config(idx, scale)
    p_big, _ = orc.mg_solve(c.coef, c.b, tol=1e-12, max_cycles=200)
    b_small = c.b * 1e-4
    want, _ = orc.mg_solve(c.coef, b_small, tol=1e-12, max_cycles=200)
    with solver(c, precision="mixed", max_cycles=100) as s:
        s.ppe_init(c.rho)
        p0 = p_big.copy()
        p, st = s.solve(b_small, p0, tol=1e-10)
    assert st["status"] == 0 and st["rel_residual"] < 1e-10, st
    _, r2 = orc.residual(c.coef, p, b_small)
    assert np.sqrt(r2) / np.linalg.norm(b_small) < 1e-10
    assert rel_l2(p, want) <= 1e-9


@pytest.mark.parametrize("idx,scale", [(0, 1), (1, 4), (1, 2)])
def test_mixed_solve_reaches_fp64_accuracy(cuda, idx, scale):
    c = cases.config(idx, scale)
    p_or, st_or = orc.mg_solve(c.coef, c.b, tol=1e-10)
    with solver(c, precision="mixed") as s:
        s.ppe_init(c.rho)
        p, st = s.solve(c.b, tol=1e-10)
    assert st["status"] == 0 and st["rel_residual"] < 1e-10
    # the true FP64 residual, recomputed by the oracle
    _, r2 = orc.residual(c.coef, p, c.b)
    assert np.sqrt(r2) / np.linalg.norm(c.b) < 1e-10
    assert rel_l2(p, p_or) <= 1e-9
    assert st["cycles"] <= st_or["cycles"] + 2


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_krylov_matches_oracle(cuda, precision):
    c = cases.config(2, 8)
    p_or, st_or = orc.mg_solve(c.coef, c.b, tol=1e-10, krylov=1)
    assert st_or["status"] == 0
    with solver(c, precision=precision, krylov=True) as s:
        s.ppe_init(c.rho)
        p, st = s.solve(c.b, tol=1e-10)
    assert st["status"] == 0 and st["rel_residual"] < 1e-10
    if precision == "fp64":
        assert abs(st["cycles"] - st_or["cycles"]) <= 1, (st["cycles"], st_or["cycles"])
    else:
        assert st["cycles"] <= st_or["cycles"] + 3
    assert rel_l2(p, p_or) <= 1e-9


@pytest.mark.parametrize("precision,idx,scale", [("fp64", 2, 8), ("mixed", 2, 8), ("mixed", 1, 4),
                                             ("fp64", 0, 1)])
def test_fgmres_matches_oracle(cuda, precision, idx, scale):
    """Flexible GMRES(30) around the V-cycle (krylov="fgmres") reaches the
    tolerance in the true FP64 residual and the oracle's FP64 solution."""
    c = cases.config(idx, scale)
    p_or, st_or = orc.mg_solve(c.coef, c.b, tol=1e-10, krylov=1)
    assert st_or["status"] == 0
    with solver(c, precision=precision, krylov="fgmres", max_cycles=200) as s:
        s.ppe_init(c.rho)
        p, st = s.solve(c.b, tol=1e-10)
    assert st["status"] == 0 and st["rel_residual"] < 1e-10
    _, r2 = orc.residual(c.coef, p, c.b)
    assert np.sqrt(r2) / np.linalg.norm(c.b) < 1e-10
    assert rel_l2(p, p_or) <= 1e-9
    assert st["cycles"] <= st_or["cycles"] + 3


def test_fgmres_on_a_smooth_right_hand_side(cuda):
    """The adjoint of J = |p - p_t|^2/2 solves A lam = p - p_t, a smooth
    right-hand side on which flexible CG first raises the residual many-fold
    (measured with the oracle: x61 after the first step on 256^2): flexible
    GMRES, whose residual falls monotonically, needs fewer iterations."""
    c = cases.config(3, 4)
    p_t, _ = orc.mg_solve(c.coef, orc.divergence(*inputs.velocity(c.case, seed=c.case.extra["target_seed"]),
                                                 c.case.dt, c.spacing), tol=1e-10, krylov=1)
    p, _ = orc.mg_solve(c.coef, c.b, tol=1e-10, krylov=1)
    g = p - p_t
    its = {}
    for mode in ("fcg", "fgmres"):
        with solver(c, precision="mixed", krylov=mode, max_cycles=400) as s:
            s.ppe_init(c.rho)
            lam, st = s.solve(g, tol=1e-8)
        assert st["status"] == 0
        its[mode] = st["cycles"]
    assert its["fgmres"] < its["fcg"], its


def test_projection_matches_oracle(cuda):
    c = cases.config(1, 8)
    p_or, _ = orc.mg_solve(c.coef, c.b, tol=1e-12, max_cycles=200)
    u_or, v_or, w_or = orc.correct(c.rho, p_or, c.case.dt, c.u, c.v, c.w, c.spacing)
    u, v, w = c.u.copy(), c.v.copy(), c.w.copy()
    with solver(c, max_cycles=200) as s:
        s.ppe_init(c.rho)
        p, st = s.ppe_solver(u, v, w, c.case.dt, tol=1e-12)
        mx, mean = s.div_stats(u, v, w)
    assert st["status"] == 0
    assert rel_l2(p, p_or) <= 1e-9
    scale = np.abs(c.u).max()
    for a, b in ((u, u_or), (v, v_or), (w, w_or)):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-9 * scale)
    mx0, _ = orc.div_stats(c.u, c.v, c.w, c.spacing)
    assert mx < 1e-9 * mx0
    mx_or, mean_or = orc.div_stats(u, v, w, c.spacing)
    assert mx == pytest.approx(mx_or, rel=1e-12, abs=1e-12 * mx0)


# --- interfaces, layouts, edge cases -------------------------------------------------
def test_ghost_padded_host_arrays(cuda):
    """Fortran-style arrays with 3 ghost cells per side (c_loc(p(1,1,1)) and
    padded strides) give the same answer as dense arrays."""
    c = cases.config(1, 8)
    g = 3
    nz, ny, nx = c.shape

    def padded(a, extra=(0, 0, 0)):
        big = np.full((nz + extra[0] + 2 * g, ny + extra[1] + 2 * g, nx + extra[2] + 2 * g), np.nan)
        view = big[g:g + a.shape[0], g:g + a.shape[1], g:g + a.shape[2]]
        view[...] = a
        return big, view

    with solver(c) as s:
        s.ppe_init(c.rho)
        p_dense, _ = s.solve(c.b, tol=1e-10)
        _, rho_v = padded(c.rho)
        _, b_v = padded(c.b)
        pbig, p_v = padded(np.zeros(c.shape))
        s.ppe_init(rho_v)
        s.solve(b_v, p_v, tol=1e-10)
    np.testing.assert_array_equal(p_v, p_dense)
    assert np.isnan(pbig[0]).all()  # ghosts untouched


def test_device_tensors_in_place(cuda):
    import torch
    c = cases.config(1, 8)
    with solver(c) as s:
        s.ppe_init(c.rho)
        p_host, _ = s.solve(c.b, tol=1e-10)
        rho = torch.from_numpy(c.rho).to(cuda)
        b = torch.from_numpy(c.b).to(cuda)
        p = torch.zeros_like(b)
        s.ppe_init(rho)
        out, st = s.solve(b, p, tol=1e-10)
        assert out is p
    np.testing.assert_array_equal(p.cpu().numpy(), p_host)


def test_deterministic(cuda):
    c = cases.config(1, 4)
    with solver(c, precision="mixed") as s:
        s.ppe_init(c.rho)
        p1, s1 = s.solve(c.b, tol=1e-10)
        p2, s2 = s.solve(c.b, tol=1e-10)
    np.testing.assert_array_equal(p1, p2)
    assert s1["cycles"] == s2["cycles"]


def test_graph_and_eager_paths_agree(cuda):
    c = cases.config(0, 1)
    out = []
    for g in (True, False):
        with solver(c, use_graph=g) as s:
            s.ppe_init(c.rho)
            out.append(s.solve(c.b, tol=1e-10)[0])
    np.testing.assert_array_equal(out[0], out[1])


@pytest.mark.parametrize("shape", [(4, 4, 4), (1, 12, 20), (6, 10, 8), (1, 1, 2)])
def test_small_and_ragged_grids(cuda, shape):
    case = inputs.custom(shape, centers=((0.5, 0.4, 0.5),), radii=(0.3,), seed=3)
    c = cases.Built(case)
    p_or, st_or = orc.mg_solve(c.coef, c.b, tol=1e-10)
    with solver(c) as s:
        s.ppe_init(c.rho)
        assert s.level_dims() == orc.mg_plan(shape)
        p, st = s.solve(c.b, tol=1e-10)
    assert st["status"] == st_or["status"] == 0
    assert abs(st["cycles"] - st_or["cycles"]) <= 1
    assert rel_l2(p, p_or) <= 1e-9


def test_zero_rhs_returns_zero(cuda):
    c = cases.config(1, 8)
    with solver(c) as s:
        s.ppe_init(c.rho)
        p, st = s.solve(np.zeros(c.shape), tol=1e-10)
    assert st["status"] == 0 and st["cycles"] == 0
    assert not p.any()


def test_status_codes(cuda):
    c = cases.config(1, 8)
    with solver(c, max_cycles=1) as s:
        s.ppe_init(c.rho)
        with pytest.raises(ConvergenceError) as e:
            s.solve(c.b, tol=1e-12)
        assert e.value.stats["status"] == 1 and e.value.stats["cycles"] == 1
        _, st = s.solve(c.b, tol=1e-12, check=False)
        assert st["status"] == 1
    with solver(c) as s:
        bad = [a.copy() for a in c.coef]
        bad[0][2, 2, 2] = np.nan
        s.set_coef(*bad)
        _, st = s.solve(c.b, tol=1e-10, check=False)
        assert st["status"] == 2
    with pytest.raises(GBMGError):
        PressurePoisson((10, 14, 18), (0.1, 0.1, 0.1))  # coarsest level 5x7x9 > 64 cells
    with pytest.raises(GBMGError):
        PressurePoisson((8, 8, 8), (0.1, 0.1, 0.1), levels=5)  # not divisible (the reference STOPs)
    with solver(c) as s:
        with pytest.raises(GBMGError):
            s.solve(c.b)  # no coefficients yet


def test_kernels_are_launched(cuda):
    c = cases.config(1, 8)
    with solver(c) as s:
        n0 = s.kernel_launches
        s.ppe_init(c.rho)
        s.solve(c.b, tol=1e-10)
        assert s.kernel_launches > n0 + 20



@pytest.mark.parametrize("precision,idx,scale", [("fp64", 1, 4), ("mixed", 1, 2), ("mixed", 0, 1)])
def test_single_block_bottom_matches_separate_launches(cuda, monkeypatch, precision, idx, scale):
    """The levels of at most 4096 cells run in one block (GBMG_SUBCYCLE=0 runs
    them as separate launches); same cycle, same answer."""
    c = cases.config(idx, scale)
    out = {}
    for flag in ("0", "1"):
        monkeypatch.setenv("GBMG_SUBCYCLE", flag)
        with solver(c, precision=precision) as s:
            s.ppe_init(c.rho)
            out[flag] = s.solve(c.b, tol=1e-10)
    (p0, s0), (p1, s1) = out["0"], out["1"]
    assert s0["cycles"] == s1["cycles"]
    assert rel_l2(p1, p0) <= 1e-12





@pytest.mark.parametrize("idx,scale,krylov", [(1, 2, False), (0, 1, False), (4, 4, True)])
def test_density_form_coefficients(cuda, monkeypatch, idx, scale, krylov):
    """The FP32 finest-level smoother and restriction computing their face
    coefficients from the density (the default for an operator set from rho)
    against the stored FP32 coefficients (GBMG_RHO_COEF=0): the FP32 values
    differ by a few ulp, so the preconditioner changes slightly; both solves
    reach the tolerance, agree with the FP64 oracle to tol-scaled accuracy and
    take the same number of cycles to within two (the stationary loop tests
    its residual once per defect correction, whose length it predicts from
    the last one)."""
    c = cases.config(idx, scale)
    out = {}
    for flag in ("0", "1"):
        monkeypatch.setenv("GBMG_RHO_COEF", flag)
        with solver(c, precision="mixed", krylov=krylov, max_cycles=400) as s:
            s.ppe_init(c.rho)
            out[flag] = s.solve(c.b, tol=1e-10)
    want, _ = orc.mg_solve(c.coef, c.b, tol=1e-13, max_cycles=400, krylov=1)
    for flag, (p, st) in out.items():
        assert st["rel_residual"] < 1e-10, flag
        assert rel_l2(p, want) <= 1e-6, flag
    assert abs(out["0"][1]["cycles"] - out["1"][1]["cycles"]) <= (1 if krylov else 2)


@pytest.mark.parametrize("idx,scale,krylov,shape", [
    (1, 4, False, None), (1, 2, True, None), (0, 1, False, None), (4, 4, True, None),
    (1, 1, False, None), (None, None, False, (8, 8, 512)), (None, None, True, (8, 16, 96)),
    (None, None, False, (16, 16, 12))])
def test_colour_split_layout_is_bit_identical(cuda, monkeypatch, idx, scale, krylov, shape):
    """The colour-split FP32 finest level (the default, with the density
    form) does the natural-layout kernels' arithmetic in the same order
    (GBMG_SPLIT=0 keeps the natural layout): same cycles, same bits.  The
    shapes cover rows of 16 to 256 half cells, a 2D grid, and
    the 16 x 16 x 12 grid with nx % 8 != 0, whose split level keeps the
    colour launches and whose defect runs without TMA."""
    if shape is None:
        c = cases.config(idx, scale)
    else:
        # cubic cells: the extent follows the shape
        nz, ny, nx = shape
        ext = (1.0, ny / nx, nz / nx)
        c = cases.Built(inputs.custom(shape, extent=ext, centers=((0.5, 0.4 * ext[1], 0.5 * ext[2]),),
                                      radii=(0.3 * min(ext),), seed=3))
    out = {}
    monkeypatch.setenv("GBMG_RHO_COEF", "1")
    for name, split in (("natural", "0"), ("colour-split", "1")):
        monkeypatch.setenv("GBMG_SPLIT", split)
        with solver(c, precision="mixed", krylov=krylov, max_cycles=400) as s:
            s.ppe_init(c.rho)
            out[name] = s.solve(c.b, tol=1e-10)
    (p0, s0), (p1, s1) = out["natural"], out["colour-split"]
    assert s0["status"] == 0 and s1["cycles"] == s0["cycles"]
    np.testing.assert_array_equal(p1, p0)



@pytest.mark.parametrize("shape", [(6, 10, 8), (12, 20, 16), (1, 12, 20), (4, 6, 10),
                                   (8, 8, 24)])
def test_mixed_small_and_ragged_grids(cuda, shape):
    """Mixed precision on small grids that take the other code paths: nx % 8
    != 0 (scalar colour-split kernels, defect without TMA), 2D, two-level
    hierarchies."""
    case = inputs.custom(shape, centers=((0.5, 0.4, 0.5),), radii=(0.3,), seed=3)
    c = cases.Built(case)
    p_or, st_or = orc.mg_solve(c.coef, c.b, tol=1e-10)
    with solver(c, precision="mixed") as s:
        s.ppe_init(c.rho)
        p, st = s.solve(c.b, tol=1e-10)
    assert st["status"] == st_or["status"] == 0
    assert st["rel_residual"] < 1e-10
    assert st["cycles"] <= st_or["cycles"] + 2
    assert rel_l2(p, p_or) <= 1e-9
