#!/usr/bin/env python
"""Benchmark: ms per 256^3 pressure-Poisson solve to 1e-10 relative residual,
FP32-in-FP64 multigrid vs FP64 multigrid, on one GB300.

Workload (one step = one pressure solve): the 256^3 rising-bubble projection
case -- one sphere of radius 0.2 at (0.5, 0.5, 0.3) in [0,1]^3, density 1 in
the bubble and 1000 outside through the smoothed Heaviside (half width 1.5 dx),
b = div(u*)/dt with u* ~ N(0,1), dt = 1e-3, Neumann walls, zero-mean pressure.
A step sets the operator from the level set (density, face coefficients,
coarse levels, coarse inverse) and solves from a zero initial guess to
||b - A p|| / ||b|| < 1e-10.

Arms:
  default            this repo's CUDA path (device-resident inputs; value = mixed
                     precision ms per solve, FP64 beside it), plus the e2e run
                     through the C ABI with pinned host buffers, a per-kernel
                     profile pass for the roofline, and the CPU baseline (the
                     oracle on the host cores).
  --impl reference   the reference's own algorithm on the host cores: the FP64
                     multigrid with lexicographic Gauss-Seidel in OpenMP subdomains
                     (the oracle's restatement; the Fortran reference cannot be
                     built here).

Prints one JSON line (rank 0).  Under torchrun each rank solves its own copy
(replicas, weak scaling); value = max-over-ranks time / (steps * ranks).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms per 256³ Poisson solve to 1e-10 rel. residual: FP32-in-FP64 vs FP64 MG"
TOL = 1e-10
NU1, NU2 = 2, 2  # V(2,2), the library's default
# adjoint solves: the right-hand side p - p_t is smooth, so A^+ of it is large
# and the attainable relative residual is higher than the forward's
ADJ_TOL = 1e-8
ADJ_TOL_LOOSE = 1e-7


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1, help="synthetic case index (1 = 256^3 sphere)")
    ap.add_argument("--scale", type=int, default=1, help="divide every axis by this (quick runs)")
    ap.add_argument("--krylov", action="store_true", help="flexible CG around the V-cycle")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU baseline sample budget")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-profile", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-multi", action="store_true", help="skip the 512^3 16-bubble section")
    ap.add_argument("--no-rollout", action="store_true", help="skip the 20-step rollout section")
    ap.add_argument("--no-levelset", action="store_true", help="skip the level-set advection section")
    ap.add_argument("--no-momentum", action="store_true", help="skip the momentum-step section")
    ap.add_argument("--no-timestep", action="store_true", help="skip the whole-time-step section")
    ap.add_argument("--host-loop", action="store_true",
                    help="headline solves with one graph per cycle, tested on the host")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value, device=None):
    """Max of a float over all ranks (the job's time is its slowest rank's);
    the value itself when not distributed."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_desc(case):
    nz, ny, nx = case.shape
    return (f"{nx}x{ny}x{nz}, {len(case.radii)} bubble(s), rho ratio "
            f"{case.rho_pos / case.rho_neg:g}, phi->rho->solve to rel. res. {TOL:g} from p=0")


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.monotonic(), line.strip()))

    def window(self, t0, t1):
        """Keep the samples read between t0 and t1 (the timed region, plus
        one sampling interval of slack for the pipe)."""
        inside = [(t, ln) for t, ln in self.lines if t0 <= t <= t1 + 0.06]
        self.in_window = bool(inside)
        if inside:
            self.lines = inside

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for _, ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm),
                "window": "timed region" if getattr(self, "in_window", False)
                else "warm-up and timed region (no sample read inside the timed region)"}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def traffic_per_cell():
    """dram bytes (read + write) per fine cell processed, per kernel class, from
    an ncu capture summarised in profiles/ (empty when no capture was made)."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# algorithmic bytes per fine cell per launch of each kernel class, mixed solve:
# FP32 cycle arrays (w = 4) and the double-word defect kernel
# per sweep for the smoother (a two-colour sweep is two launches: the bench
# scales by the sweeps a launch covers).  With the density form (the default
# for an operator from rho or phi; GBMG_RHO_COEF=0 stores coefficients) the
# FP32 finest-level kernels read the cell density (w) instead of three
# face-coefficient arrays (3w).
def rho_form():
    return os.environ.get("GBMG_RHO_COEF", "1") != "0"


def algorithmic_bytes_per_cell(cls, w=4, shape=None):
    c = w if rho_form() else 3.0 * w
    return {
        "smooth_fine": 3.0 * w + c,              # one sweep: p, b, coefficients read, p' write
        "restrict_fine": 2.0 * w + c + 2.0 * w / 8,  # p, b, coefficients -> coarse b, sol
        "prolong_fine": 2.0 * w + w / 8,         # p r/w + coarse e
        "residual": 56.0,                        # defect: p(8) + e(4) + b(8) + 3 coefs(24) in,
                                                 # p(8) + r32(4) out
    }.get(cls)


def run_reference(args):
    """The reference's FP64 multigrid on the host cores (oracle restatement)."""
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    from fortrancfd_gb300 import inputs
    from oracle import oracle as orc

    case = inputs.config(args.config, args.scale)
    phi = inputs.level_set(case)
    u, v, w = inputs.velocity(case)
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    blocks = _factor3(threads)
    times, cycles = [], []

    b = orc.divergence(u, v, w, case.dt, case.spacing)

    def step():
        # the same step as the GPU arm: operator from the level set, then the solve
        t0 = time.perf_counter()
        rho = orc.rho_from_phi(phi, case.eps, case.rho_pos, case.rho_neg)
        coef = orc.face_coef(rho, case.spacing)
        p, st = orc.mg_solve(coef, b, tol=TOL, smoother=1, blocks=blocks)
        return (time.perf_counter() - t0) * 1e3, st

    for _ in range(args.warmup):
        step()
    for _ in range(args.steps):
        ms, st = step()
        times.append(ms)
        cycles.append(st["cycles"])
    value = float(np.mean(times))
    sample = (f"{args.steps} full FP64 solves of {case.name}, lexicographic Gauss-Seidel V(2,2) in "
              f"{blocks[0]}x{blocks[1]}x{blocks[2]} OpenMP subdomains, {cycles[-1]} cycles each")
    line = {"metric": METRIC, "value": value, "unit": "ms", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": value, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": workload_desc(case), "grid": list(case.shape[::-1]), "tol": TOL,
                       "cycles": cycles[-1]},
            "cpu_baseline": {"value": value, "unit": "ms", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def _factor3(n):
    """Split n threads into a 3D subdomain grid (largest factors on z, then y)."""
    best = (1, 1, n)
    for a in range(1, n + 1):
        if n % a:
            continue
        for b in range(a, n + 1):
            if (n // a) % b:
                continue
            c = n // a // b
            if c >= b and (c - a) < (best[2] - best[0]):
                best = (a, b, c)
    return best


def cpu_baseline(case, phi, u, v, w, budget_s):
    """The oracle's FP64 multigrid (red-black, all host threads), full solves
    until the sample budget is spent (at least one).  Returns the baseline
    record, the oracle's pressure (for the parity figures) and its (coef, b)."""
    from oracle import oracle as orc

    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    b = orc.divergence(u, v, w, case.dt, case.spacing)
    times = []
    t_start = time.perf_counter()
    while True:
        t0 = time.perf_counter()
        rho = orc.rho_from_phi(phi, case.eps, case.rho_pos, case.rho_neg)
        coef = orc.face_coef(rho, case.spacing)
        p_or, st = orc.mg_solve(coef, b, tol=TOL)
        times.append((time.perf_counter() - t0) * 1e3)
        if time.perf_counter() - t_start > budget_s * 0.5:
            break
    rec = {"value": float(np.mean(times)), "unit": "ms", "cores": threads, "kind": "port",
           "sample": f"{len(times)} full FP64 red-black V(2,2) solve(s) of the same case on "
                     f"{threads} threads, {st['cycles']} cycles each (oracle restatement)"}
    return rec, p_or, st, coef, b


def rel_l2_mean_free(a, b):
    """Relative L2 distance of two pressures after removing each one's mean."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    a = a - a.mean()
    b = b - b.mean()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oracle_parity(p_or, st_or, coef, b, p_mixed, p_fp64, threads):
    """Full-size parity of the GPU pressures against the oracle: the red-black
    FP64 multigrid (the same cycle as the GPU's) and the reference's own cycle
    (lexicographic Gauss-Seidel in OpenMP subdomains, the reference arm's
    algorithm), both solved to the same tolerance from zero."""
    from oracle import oracle as orc

    blocks = _factor3(threads)
    t0 = time.perf_counter()
    p_lex, st_lex = orc.mg_solve(coef, b, tol=TOL, smoother=1, blocks=blocks)
    lex_ms = (time.perf_counter() - t0) * 1e3
    out = {"cycles_oracle": st_or["cycles"],
           "oracle_rel_residual": st_or["rel_residual"],
           "p_rel_l2_mixed_vs_oracle": rel_l2_mean_free(p_mixed, p_or),
           "cycles_lex": st_lex["cycles"],
           "lex_rel_residual": st_lex["rel_residual"],
           "p_rel_l2_mixed_vs_lex": rel_l2_mean_free(p_mixed, p_lex),
           "p_rel_l2_oracle_vs_lex": rel_l2_mean_free(p_or, p_lex),
           "lex_blocks": "x".join(str(x) for x in blocks), "lex_ms": lex_ms}
    if p_fp64 is not None:
        out["p_rel_l2_fp64_vs_oracle"] = rel_l2_mean_free(p_fp64, p_or)
        out["p_rel_l2_fp64_vs_lex"] = rel_l2_mean_free(p_fp64, p_lex)
    # The error of each solution: against the oracle continued from its own
    # solution to a relative residual of 1e-13 (the solves above stop at
    # 1e-10 after different cycle counts, so they differ from one another by
    # about their own errors).
    p_conv, st_conv = orc.mg_solve(coef, b, p0=p_or, tol=1e-13, max_cycles=60)
    out["converged_rel_residual"] = st_conv["rel_residual"]
    out["p_err_oracle"] = rel_l2_mean_free(p_or, p_conv)
    out["p_err_lex"] = rel_l2_mean_free(p_lex, p_conv)
    out["p_err_mixed"] = rel_l2_mean_free(p_mixed, p_conv)
    if p_fp64 is not None:
        out["p_err_fp64"] = rel_l2_mean_free(p_fp64, p_conv)
    return out


def _device_velocity(shape, seed, dev):
    """u*, v*, w* ~ N(0,1) on interior faces, 0 on wall faces, drawn on the
    device from a seeded generator (for the large sections, where host
    generation would dominate the run)."""
    import torch
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    nz, ny, nx = shape
    u = torch.randn((nz, ny, nx + 1), generator=g, device=dev, dtype=torch.float64)
    v = torch.randn((nz, ny + 1, nx), generator=g, device=dev, dtype=torch.float64)
    w = torch.randn((nz + 1, ny, nx), generator=g, device=dev, dtype=torch.float64)
    u[..., 0] = 0.0
    u[..., -1] = 0.0
    v[:, 0, :] = 0.0
    v[:, -1, :] = 0.0
    w[0] = 0.0
    w[-1] = 0.0
    return u, v, w


def multi_bubble_section(dev, stream, scale=1, reps=2, krylov=True, oracle=True):
    """The 512³ sixteen-bubble case: mixed precision (flexible CG around the
    FP32 V-cycle, the mode these small light bubbles need) against the FP64
    GPU solve of the same system.  Flexible GMRES(30) needs 52 iterations
    against 67 here but its Gram-Schmidt over up to 30 vectors of 1 GB costs
    more than it saves (1437 against 938 ms), so flexible CG stays.  With
    `oracle`, the oracle's flexible-CG FP64 solve of the same inputs on the
    host cores gives the pressure error of both GPU solves."""
    import torch

    from fortrancfd_gb300 import PressurePoisson, inputs
    from fortrancfd_gb300.rollout import level_set

    case = inputs.config(2, scale)
    with torch.cuda.stream(stream):
        c = torch.from_numpy(case.centers.copy()).to(dev)
        r = torch.from_numpy(case.radii.copy()).to(dev)
        phi = level_set(c, r, case.shape, case.extent)
        u, v, w = _device_velocity(case.shape, case.seed, dev)
        out = {}
        ps = {}
        for prec in ("mixed", "fp64"):
            s = PressurePoisson(case.shape, case.spacing, precision=prec, krylov=krylov,
                                max_cycles=400, stream=stream)
            b = s.divergence(u, v, w, case.dt)
            p = torch.zeros_like(b)
            times = []
            for it in range(reps + 1):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                p.zero_()
                e0.record(stream)
                s.rho_mu(phi, case.eps, case.rho_pos, case.rho_neg)
                _, st = s.solve(b, p, tol=TOL)
                e1.record(stream)
                torch.cuda.synchronize()
                if it:
                    times.append(e0.elapsed_time(e1))
            out[prec] = {"ms_per_solve": float(np.median(times)), "cycles": st["cycles"],
                         "rel_residual": st["rel_residual"]}
            ps[prec] = p
            s.close()
        out["p_rel_diff_mixed_vs_fp64"] = float((ps["mixed"] - ps["fp64"]).norm() /
                                               ps["fp64"].norm())
        out["mixed_over_fp64"] = out["mixed"]["ms_per_solve"] / out["fp64"]["ms_per_solve"]
        if oracle:
            host = [a.cpu().numpy() for a in (phi, u, v, w)]
            ph = {k: a.cpu().numpy() for k, a in ps.items()}
    del ps
    if oracle:
        # the oracle's flexible-CG FP64 solve of the same system on the host
        # cores (inputs copied from the device, so both sides see the same bytes)
        from oracle import oracle as orc
        orc.set_threads(os.cpu_count() or 1)
        phi_h, u_h, v_h, w_h = host
        t0 = time.perf_counter()
        rho = orc.rho_from_phi(phi_h, case.eps, case.rho_pos, case.rho_neg)
        coef = orc.face_coef(rho, case.spacing)
        b_h = orc.divergence(u_h, v_h, w_h, case.dt, case.spacing)
        del rho, host, phi_h, u_h, v_h, w_h
        p_or, st_or = orc.mg_solve(coef, b_h, tol=TOL, krylov=1, max_cycles=400)
        out["oracle"] = {"ms": (time.perf_counter() - t0) * 1e3, "cycles": st_or["cycles"],
                         "rel_residual": st_or["rel_residual"],
                         "threads": orc.num_threads(),
                         "p_rel_l2_mixed_vs_oracle": rel_l2_mean_free(ph["mixed"], p_or),
                         "p_rel_l2_fp64_vs_oracle": rel_l2_mean_free(ph["fp64"], p_or)}
        del coef, b_h, p_or, ph
    nz, ny, nx = case.shape
    out["workload"] = (f"{case.name}: {nx}x{ny}x{nz} cells, {len(case.radii)} bubbles, density "
                       "ratio 1000, flexible CG around one V(2,2) cycle, tol 1e-10; inputs drawn "
                       "on the device")
    return out


def levelset_section(dev, stream, case, phi_h, u_h, v_h, w_h, steps=5):
    """Level-set advection of the same 256³ case (the interface solver's
    level_set_rk3_solver: WENO-JS split fluxes, SSP-RK3, FP64) with the cell
    velocity of u* (node_vel), timed with CUDA events; one step of the CPU
    oracle on all host cores beside it, and the GPU step compared with it."""
    import torch

    from fortrancfd_gb300 import LevelSet, node_velocity
    from oracle import oracle as orc

    with torch.cuda.stream(stream):
        t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (phi_h, u_h, v_h, w_h)]
        un, vn, wn = (x.contiguous() for x in node_velocity(t[1], t[2], t[3]))
        phi = t[0].clone()
        ls = LevelSet(case.shape, case.spacing, stream=stream)
        ls.advect(phi, un, vn, wn, dt=case.dt, steps=1)  # warm-up, and the step checked below
        torch.cuda.synchronize()
        one = phi.cpu().numpy()
        n0 = ls.kernel_launches
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ls.advect(phi, un, vn, wn, dt=case.dt, steps=steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        launches = (ls.kernel_launches - n0) // steps
        ls.close()
        # redistancing as the reference calls it every fifth step (btn = 1:
        # 3 dx of pseudo time in steps of 0.1 dx, mass-preserving correction)
        h = case.spacing[0]
        ls = LevelSet(case.shape, case.spacing, stream=stream)
        e0.record(stream)
        rho_12 = min(case.rho_pos, case.rho_neg) / max(case.rho_pos, case.rho_neg)
        _, iters, _ = ls.redistance(phi, case.eps, 0.1 * h, rho_12=rho_12, btn=1)
        e1.record(stream)
        torch.cuda.synchronize()
        redis_ms = e0.elapsed_time(e1)
        ls.close()
    un_h, vn_h, wn_h = (x.cpu().numpy() for x in (un, vn, wn))
    t0 = time.perf_counter()
    ref = orc.ls_advect(phi_h, un_h, vn_h, wn_h, case.dt, case.spacing, steps=1)
    cpu_ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    orc.ls_redistance(phi_h, case.eps, 0.1 * case.spacing[0], case.spacing, rho_12=rho_12,
                      btn=1, max_iter=2)
    cpu_redis_it_ms = (time.perf_counter() - t0) * 1e3 / 2
    nz, ny, nx = case.shape
    return {"workload": f"{case.name}: level set of the {nx}x{ny}x{nz} sphere advected by the "
                        f"cell velocity of u*, dt={case.dt}, WENO-JS + SSP-RK3, FP64; then one "
                        "redistancing call (btn=1, rdt=0.1 dx, 3 dx of pseudo time)",
            "ms_per_step": ms, "cell_steps_per_s": nx * ny * nz / (ms * 1e-3),
            "kernels_per_step": launches,
            "cpu_oracle_ms_per_step": cpu_ms, "cpu_threads": orc.num_threads(),
            "gpu_equals_oracle": bool(np.array_equal(one, ref)),
            "redistance_ms": redis_ms, "redistance_iterations": iters,
            "redistance_ms_per_iteration": redis_ms / max(iters, 1),
            "cpu_oracle_redistance_ms_per_iteration": cpu_redis_it_ms}


def momentum_section(dev, stream, case, iterations=4, reps=5):
    """The Adams-Bashforth momentum step of the same case (ns_ab_solver_SOR:
    velsrc%tmp, then `iterations` passes of predictor + mixed-precision
    projection to TOL, velbc, ns_check_convergence_vel) on device-resident
    ghost-padded arrays (g = 3), timed with CUDA events; a profiled step gives
    the momentum kernels' share and roofline; the same step through the C ABI
    with host arrays (e2e) and the CPU oracle's step beside it."""
    import torch

    from fortrancfd_gb300 import (NSParams, PressurePoisson, curv, inputs, ns_ab_predictor,
                                  ns_ab_solver)
    from oracle import oracle as orc

    rho_12 = min(case.rho_pos, case.rho_neg) / max(case.rho_pos, case.rho_neg)
    st = inputs.momentum_state(case, ghost=3, rho_12=rho_12, mu_12=1e-2, amplitude=0.1)
    three = case.dim == 3
    prm = NSParams(dt=case.dt, re=1000.0, fr=0.4096, we=1.0, mu_12=1e-2,
                   gravity=(0.0, 0.0, -1.0) if three else (0.0, -1.0, 0.0), btn_g=1.0,
                   btn_sf=1.0, ghost=3, iterations=iterations, p_tol=TOL)
    names = ("u", "v", "w", "u_old", "v_old", "w_old", "su", "sv", "sw", "su_old", "sv_old",
             "sw_old", "rho", "mu", "delta", "phi", "nrm_x", "nrm_y", "nrm_z", "curv", "p")
    src = {"u": st["u"], "v": st["v"], "w": st["w"], "u_old": st["u"], "v_old": st["v"],
           "w_old": st["w"], "su": np.zeros_like(st["u"]), "sv": np.zeros_like(st["v"]),
           "sw": np.zeros_like(st["u"]) if three else None}
    for k in names:
        src.setdefault(k, st.get(k))
    nz, ny, nx = case.shape
    n = nx * ny * nz
    with torch.cuda.stream(stream):
        t = {k: (torch.from_numpy(np.ascontiguousarray(a)).to(dev) if a is not None else None)
             for k, a in src.items()}
        init = {k: t[k].clone() for k in ("u", "v", "w", "p") if t[k] is not None}
        pp = PressurePoisson(case.shape, case.spacing, precision="mixed", stream=stream,
                             nu1=NU1, nu2=NU2)
        pp.ppe_init(torch.from_numpy(st["rho_now"]).to(dev))

        def reset():
            for k, a in init.items():
                t[k].copy_(a)

        ns_ab_solver(pp, prm, t)  # warm-up
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        times = []
        n0 = pp.kernel_launches
        for _ in range(reps):
            reset()
            torch.cuda.synchronize()
            e0.record(stream)
            stats = ns_ab_solver(pp, prm, t)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        ms = statistics.median(times)
        launches = (pp.kernel_launches - n0) // reps
        gpu_u = {k: t[k].cpu().numpy() for k in ("u", "v", "w") if t[k] is not None}
        # profiled step: the momentum kernels' time against the solves'
        reset()
        pp.set_profiling(True)
        ns_ab_solver(pp, prm, t)
        prof = pp.profile()
        pp.set_profiling(False)
        # one predictor pass without the projection, for the bitwise check
        # against the oracle at full size below
        reset()
        ns_ab_predictor(pp, prm, t)
        pred = {k: t[k].cpu().numpy() for k in ("u", "v", "w", "su", "sv", "sw")
                if t[k] is not None}
        # curv + surface_norms of the same level set (the step's normals and
        # curvature inputs for the next time step), by compact differences
        cv_out = [torch.zeros_like(t["phi"]) for _ in range(4)]
        if not three:
            cv_out[2] = None
        curv(pp, prm, t["phi"], *cv_out)  # warm-up
        ctimes = []
        for _ in range(reps):
            torch.cuda.synchronize()
            e0.record(stream)
            curv(pp, prm, t["phi"], *cv_out)
            e1.record(stream)
            torch.cuda.synchronize()
            ctimes.append(e0.elapsed_time(e1))
        cv_gpu = [a.cpu().numpy() if a is not None else None for a in cv_out]
        # e2e: the same step through the C ABI on host arrays
        host = {k: (np.array(a, copy=True) if a is not None else None) for k, a in src.items()}
        t0 = time.perf_counter()
        ns_ab_solver(pp, prm, host)
        e2e_ms = (time.perf_counter() - t0) * 1e3
        pp.close()
    mom_ms, mom_cnt = prof.get("momentum", (0.0, 0))
    prof_total = sum(v[0] for v in prof.values())
    nc = 3 if three else 2
    # algorithmic bytes (8-byte values per cell): sources once (3 velocities,
    # rho, mu, delta, phi, 3 normals and curv in; 3 out), each pass's fused
    # predictor (old, tmp, velsrc%tmp, velsrc%old in; velsrc%now, vel%now out)
    # and the change statistics (2 x 3 in); velbc touches only the ghost shell
    per_cell = 8 * ((nc + 4 + nc + 1) + nc + iterations * 6 * nc + 2 * nc)
    alg = per_cell * n
    peak, peak_kind = measured_peaks()
    achieved = alg / (mom_ms * 1e-3) / 1e9 if mom_ms else None
    # FP64 divisions the reference writes, per cell (mu/rho counted once):
    # sources about 20 per component in 3D (14 in 2D), each pass 2 per
    # component and axis
    divs = n * ((20 if three else 14) * nc + iterations * 2 * nc * nc)
    # the CPU oracle's step on the host cores
    vel = tuple(st[k] for k in ("u", "v", "w")[:nc])
    so = tuple(st[k] for k in ("su_old", "sv_old", "sw_old")[:nc])
    op = orc.ns_params(ghost=3, bc=prm.bc, iterations=iterations, dt=prm.dt, re=prm.re,
                       fr=prm.fr, we=prm.we, mu_12=prm.mu_12, gravity=prm.gravity,
                       btn_g=prm.btn_g, btn_sf=prm.btn_sf, p_tol=TOL)
    # the predictor pass: oracle sources + advance + velbc, compared bit for bit
    t0 = time.perf_counter()
    dif = orc.ns_diffusion(case.shape, case.spacing, op, st)[:nc]
    osrc, ovel = orc.ns_advance(case.shape, case.spacing, op, vel, vel, dif, so)
    ovel = [a.copy() for a in ovel] + [None] * (3 - nc)
    orc.velbc(case.shape, op, *ovel[:nc])
    cpu_pred_ms = (time.perf_counter() - t0) * 1e3
    pred_equal = all(np.array_equal(pred[k].view(np.int64), ovel[c].view(np.int64))
                     for c, k in enumerate(("u", "v", "w")[:nc]))
    pred_equal = pred_equal and all(
        np.array_equal(pred[k].view(np.int64), osrc[c].view(np.int64))
        for c, k in enumerate(("su", "sv", "sw")[:nc]))
    t0 = time.perf_counter()
    cv_or = orc.ns_curvature(case.shape, case.spacing, 3, st["phi"])
    cpu_curv_ms = (time.perf_counter() - t0) * 1e3
    curv_bitwise = all(np.array_equal(cv_gpu[c].view(np.int64), cv_or[c].view(np.int64))
                       for c in range(nc))
    curv_rel = float(np.abs(cv_gpu[3] - cv_or[3]).max() / np.abs(cv_or[3]).max())
    t0 = time.perf_counter()
    out = orc.ns_ab_step(case.shape, case.spacing, op, st["rho_now"], vel, st, so, st["p"],
                         krylov=1)
    cpu_ms = (time.perf_counter() - t0) * 1e3
    diff = max(float(np.abs(gpu_u[k] - out[k]).max() / np.abs(out[k]).max()) for k in gpu_u)
    return {"workload": f"{case.name}: Adams-Bashforth momentum step on the {nx}x{ny}x{nz} grid "
                        f"(3 ghost layers): sources (viscous, interface viscosity, gravity, "
                        f"surface tension) + {iterations} passes of AB2 predictor, velbc and the "
                        f"mixed-precision projection to {TOL}; FP64 explicit part",
            "ms_per_step": ms, "ms_min": min(times), "cell_steps_per_s": n / (ms * 1e-3),
            "kernels_per_step": launches, "solve_cycles_per_step": stats["cycles"], "linf": stats["linf"], "l2f": stats["l2f"],
            "momentum_kernels_ms": mom_ms, "momentum_launches": mom_cnt,
            "momentum_share": mom_ms / prof_total if prof_total else None,
            "roofline_momentum": {"bound": "fp64 divisions (the reference's operand order kept)",
                                  "achieved_gbs": achieved, "peak_gbs": peak,
                                  "frac_hbm": achieved / peak if achieved else None,
                                  "peak_source": peak_kind, "algorithmic_bytes": alg,
                                  "fp64_divisions": divs,
                                  "divisions_per_ns": divs / (mom_ms * 1e6) if mom_ms else None},
            "e2e_host_arrays_ms": e2e_ms,
            "cpu_oracle_ms_per_step": cpu_ms, "cpu_threads": orc.num_threads(),
            "cpu_oracle_predictor_ms": cpu_pred_ms,
            "predictor_gpu_equals_oracle_bitwise": bool(pred_equal),
            "curvature": {"what": "curv + surface_norms (CCD line solves along every padded line, "
                                  "curvature, zero-gradient ghosts)",
                          "ms": statistics.median(ctimes), "cpu_oracle_ms": cpu_curv_ms,
                          "gradient_equals_oracle_bitwise": bool(curv_bitwise),
                          "curvature_max_rel_diff": curv_rel},
            "gpu_vs_oracle_max_rel_diff": diff}



def timestep_section(dev, stream, case, steps=5):
    """The whole two-phase time step on the 256³ sphere (TwoPhaseStep: switch,
    level-set advection, redistancing every fifth step with rdt = 0.25 dx,
    rho_mu, CCD curvature, the momentum step with four mixed-precision
    projections, divergence check, cell velocity), every field device-resident,
    timed per step with CUDA events after one warm-up step."""
    import torch

    from fortrancfd_gb300 import InterfaceParams, NSParams, TwoPhaseStep, inputs

    rho_12 = min(case.rho_pos, case.rho_neg) / max(case.rho_pos, case.rho_neg)
    st = inputs.momentum_state(case, ghost=3, rho_12=rho_12, mu_12=1e-2, amplitude=0.1)
    three = case.dim == 3
    # explicit time-step limits at 256^3: viscous dx^2/(6 nu) with nu =
    # (mu_12/rho_12)/Re = 0.01 in the light phase is 2.5e-4, so dt = 2e-4 (the
    # case's 1e-3 grows the velocity without bound within four steps); We =
    # 1000 keeps the capillary limit sqrt(We dx^3/(4 pi)) = 2e-3 above it
    dt = 2e-4
    ns = NSParams(dt=dt, re=1000.0, fr=0.4096, we=1000.0, mu_12=1e-2,
                  gravity=(0.0, 0.0, -1.0) if three else (0.0, -1.0, 0.0), btn_g=1.0,
                  btn_sf=1.0, ghost=3, iterations=4, p_tol=TOL)
    itf = InterfaceParams(ls_wid=case.eps, rho_12=rho_12, rdt=0.25 * case.spacing[0],
                          redis_every=5, method=2)
    with torch.cuda.stream(stream):
        ts = TwoPhaseStep(case.shape, case.spacing, ns, itf, precision="mixed", krylov=False,
                          stream=stream)
        ts.load(st["phi"], st["u"], st["v"], st["w"])
        ts.step()  # warm-up (step 1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        times, stats = [], []
        for _ in range(steps):
            torch.cuda.synchronize()
            e0.record(stream)
            stats.append(ts.step())
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        # one profiled MPLS step (CUDA events per kernel class on the pressure
        # handle: the solves' classes and "momentum" for the momentum, CCD,
        # rho_mu, MPLS and bc kernels; the rest of the step is the level set)
        ts.pp.set_profiling(True)
        torch.cuda.synchronize()
        e0.record(stream)
        ts.step()
        e1.record(stream)
        torch.cuda.synchronize()
        step_ms = e0.elapsed_time(e1)
        prof = ts.pp.profile()
        ts.pp.set_profiling(False)
        breakdown = {"step_ms": step_ms,
                     "momentum_ccd_mpls_kernels_ms": prof.get("momentum", (0.0, 0))[0],
                     "pressure_solve_kernels_ms": sum(v[0] for k, v in prof.items()
                                                      if k != "momentum")}
        breakdown["level_set_and_rest_ms"] = (step_ms - breakdown["momentum_ccd_mpls_kernels_ms"]
                                              - breakdown["pressure_solve_kernels_ms"])
        ts.close()
        # the CLSVOF mode (volume-fraction transport; rho and mu from it):
        # steps 2 and 4 without redistancing, 3 with (every third step)
        itf3 = InterfaceParams(ls_wid=case.eps, rho_12=rho_12, rdt=0.25 * case.spacing[0],
                               redis_every=3, method=3, recon_every=10)
        ts = TwoPhaseStep(case.shape, case.spacing, ns, itf3, precision="mixed", krylov=False,
                          stream=stream)
        ts.load(st["phi"], st["u"], st["v"], st["w"])
        ts.step()
        ctimes = []
        for _ in range(3):
            torch.cuda.synchronize()
            e0.record(stream)
            ts.step()
            e1.record(stream)
            torch.cuda.synchronize()
            ctimes.append(e0.elapsed_time(e1))
        ts.close()
    nz, ny, nx = case.shape
    plain = [t for t, s in zip(times, stats) if not s["redistance_iterations"]]
    redis = [(t, s["redistance_iterations"]) for t, s in zip(times, stats)
             if s["redistance_iterations"]]
    return {"workload": f"{case.name}: whole two-phase time step on the {nx}x{ny}x{nz} grid "
                        f"(dt={dt}; MPLS level set, the input default: advection every step, "
                        "redistancing btn=1 every fifth step at rdt=0.25 dx, two mass-preserving "
                        "corrections; rho_mu, CCD curvature, AB2 momentum step "
                        f"with 4 mixed stationary-cycle projections to {TOL}, divergence check)",
            "steps_timed": [s["iter"] for s in stats], "ms_per_step": times,
            "ms_mean": sum(times) / len(times),
            "ms_without_redistancing": statistics.median(plain) if plain else None,
            "ms_with_redistancing": redis[0][0] if redis else None,
            "redistancing_iterations": redis[0][1] if redis else None,
            "div_max": stats[-1]["div_max"], "solve_cycles_last": stats[-1]["cycles"],
            "mass_last": stats[-1]["mass"],
            "clsvof_ms_steps_2_to_4": ctimes,
            "profiled_step": breakdown,
            "velocity_change_linf_last": stats[-1]["linf"]}



def rollout_section(dev, stream, scale=1, steps=20, krylov="fgmres"):
    """The 20-step differentiable projection rollout (128x128x256, 4 bubbles):
    forward (20 mixed solves) and backward (20 adjoint solves and the
    checkpointed level sets) device times, gradient w.r.t. centres and radii.
    Flexible GMRES around the V-cycle (measured: 418 / 495 ms against 542 /
    890 ms with flexible CG, the same gradients)."""
    import torch

    from fortrancfd_gb300 import PressurePoisson, inputs
    from fortrancfd_gb300.rollout import rollout_loss

    case = inputs.config(4, scale)
    with torch.cuda.stream(stream):
        s = PressurePoisson(case.shape, case.spacing, precision="mixed", krylov=krylov,
                            max_cycles=400, stream=stream)
        c = torch.from_numpy(case.centers.copy()).to(dev).requires_grad_(True)
        r = torch.from_numpy(case.radii.copy()).to(dev).requires_grad_(True)
        fw, bw = [], []
        for it in range(2):
            c.grad = None
            r.grad = None
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            J = rollout_loss(c, r, case, s, steps=steps, tol=TOL, adjoint_tol=ADJ_TOL)
            e1.record(stream)
            J.backward()
            e2.record(stream)
            torch.cuda.synchronize()
            if it:
                fw.append(e0.elapsed_time(e1))
                bw.append(e1.elapsed_time(e2))
        s.close()
    nz, ny, nx = case.shape
    outer = {True: "flexible CG", "fcg": "flexible CG", "fgmres": "flexible GMRES(30)"}[krylov]
    return {"workload": f"{case.name}: {nx}x{ny}x{nz} cells, 4 bubbles, {steps} steps, mixed "
                        f"precision, {outer}, tol 1e-10 forward, 1e-8 adjoint",
            "forward_ms": fw[0], "backward_ms": bw[0], "backward_over_forward": bw[0] / fw[0],
            "grad_norm_centres": float(c.grad.norm()), "grad_norm_radii": float(r.grad.norm())}


def adjoint_section(dev, stream, reps=5, scale=1, krylov="fgmres"):
    """The differentiable solve on the 1024^2 eight-circle case: forward
    (operator from phi + mixed-precision solve) and backward (operator rebuild,
    adjoint solve, adjoint kernel) device times, and central differences of
    J = |p - p_t|^2/2 with FP64 solves (step 1e-6, 16 random unit directions
    of phi) against the mixed-precision gradient, and the same gradient from
    FP64 solves (the finite differences of FP64 solves at 1e-12 carry noise
    near 1e-6 themselves: both gradients agree with them equally).  The same
    central differences are also formed from their parts (gradcheck:
    p(phi - h v) and the solve for p(phi + h v) - p(phi - h v)), which removes
    that cancellation noise.  Flexible GMRES around the
    V-cycle by default: on the smooth adjoint right-hand side p - p_t flexible
    CG first raises the residual many-fold and needs 32 iterations against 20."""
    import torch

    from fortrancfd_gb300 import PressurePoisson, inputs
    from fortrancfd_gb300.autograd import pressure_solve
    from fortrancfd_gb300.gradcheck import central_difference

    case = inputs.config(3, scale)
    kw = dict(eps=case.eps, rho_pos=case.rho_pos, rho_neg=case.rho_neg)
    phi = torch.from_numpy(inputs.level_set(case)).to(dev)
    with torch.cuda.stream(stream):
        s = PressurePoisson(case.shape, case.spacing, precision="mixed", krylov=krylov,
                            max_cycles=400, stream=stream)
        s64 = PressurePoisson(case.shape, case.spacing, krylov=True, max_cycles=600, stream=stream)
        tv = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
        b = s.divergence(*[tv(a) for a in inputs.velocity(case)], case.dt)
        bt = s.divergence(*[tv(a) for a in inputs.velocity(case, seed=case.extra["target_seed"])],
                          case.dt)
        p_t = pressure_solve(phi, bt, s, tol=1e-10, **kw).detach()
        fw, bw = [], []
        for it in range(reps + 1):
            x = phi.clone().requires_grad_(True)
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            p = pressure_solve(x, b, s, tol=1e-10, adjoint_tol=ADJ_TOL, **kw)
            e1.record(stream)
            fwd_cycles = s.last_stats["cycles"]
            loss = 0.5 * ((p - p_t) ** 2).sum()
            loss.backward()
            e2.record(stream)
            torch.cuda.synchronize()
            adj_cycles = s.last_stats["cycles"]
            if it:
                fw.append(e0.elapsed_time(e1))
                bw.append(e1.elapsed_time(e2))
        g = x.grad
        # the same timing with the adjoint solved to 1e-7 (the gradient still
        # meets the differences below to well under 1e-6)
        bw_loose = []
        for it in range(reps + 1):
            xl = phi.clone().requires_grad_(True)
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            pl = pressure_solve(xl, b, s, tol=1e-10, adjoint_tol=ADJ_TOL_LOOSE, **kw)
            e1.record(stream)
            (0.5 * ((pl - p_t) ** 2).sum()).backward()
            e2.record(stream)
            torch.cuda.synchronize()
            adj_cycles_loose = s.last_stats["cycles"]
            if it:
                bw_loose.append(e1.elapsed_time(e2))
        g_loose = xl.grad
        # the same gradient from FP64 solves (forward 1e-12, adjoint 3e-9, the
        # adjoint's FP64 floor being about 2.6e-9)
        x64 = phi.clone().requires_grad_(True)
        p64 = pressure_solve(x64, b, s64, tol=1e-12, adjoint_tol=3e-9, **kw)
        (0.5 * ((p64 - p_t) ** 2).sum()).backward()
        g64 = x64.grad

        def J(ph):
            q = pressure_solve(ph, b, s64, tol=1e-12, **kw)
            return 0.5 * ((q - p_t) ** 2).sum()

        rng = np.random.default_rng(7)
        errs, errs64, errs_x, errs_xl = [], [], [], []
        with torch.no_grad():
            for _ in range(16):
                v = torch.from_numpy(rng.standard_normal(case.shape)).to(dev)
                v /= v.norm()
                fd = float((J(phi + 1e-6 * v) - J(phi - 1e-6 * v)) / 2e-6)
                errs.append(abs(fd - float((g * v).sum())) / abs(fd))
                errs64.append(abs(float(((g - g64) * v).sum())) / abs(float((g64 * v).sum())))
                # the same central difference from its parts (no cancellation)
                fdx = central_difference(s64, phi, b, p_t, v, 1e-6, **kw)
                errs_x.append(abs(fdx - float((g * v).sum())) / abs(fdx))
                errs_xl.append(abs(fdx - float((g_loose * v).sum())) / abs(fdx))
        s.close()
        s64.close()
    f, bk = float(np.median(fw)), float(np.median(bw))
    outer = {True: "flexible CG", "fcg": "flexible CG", "fgmres": "flexible GMRES(30)"}[krylov]
    return {"workload": f"{case.name}: {case.shape[2]}x{case.shape[1]} cells, 8 circles, mixed "
                        f"precision, {outer} around one V(2,2) cycle, tol 1e-10 forward, 1e-8 "
                        "adjoint",
            "forward_ms": f, "backward_ms": bk, "backward_over_forward": bk / f,
            "forward_iterations": fwd_cycles, "adjoint_iterations": adj_cycles,
            "fd_max_rel_err": max(errs), "fd_median_rel_err": float(np.median(errs)),
            "fd_directions": len(errs),
            "fd_exact_max_rel_err": max(errs_x),
            "fd_exact_median_rel_err": float(np.median(errs_x)),
            "adjoint_tol": ADJ_TOL,
            "loose_adjoint_tol": ADJ_TOL_LOOSE,
            "loose_backward_ms": float(np.median(bw_loose)),
            "loose_backward_over_forward": float(np.median(bw_loose)) / f,
            "loose_adjoint_iterations": adj_cycles_loose,
            "loose_fd_exact_max_rel_err": max(errs_xl),
            "fp64_gradient_max_rel_diff": max(errs64),
            "fp64_gradient_rel_l2_diff": float((g - g64).norm() / g64.norm())}


def run_ours(args):
    import torch

    from fortrancfd_gb300 import PressurePoisson, inputs

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        # replicas time the headline solve only: the single-GPU sections (and
        # their CPU oracle legs, which would share the host cores) stay at N=1
        for k in ("no_adjoint", "no_multi", "no_rollout", "no_levelset", "no_momentum",
                  "no_timestep"):
            setattr(args, k, True)
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    case = inputs.config(args.config, args.scale)
    phi_h = inputs.level_set(case)
    u_h, v_h, w_h = inputs.velocity(case)
    n = int(np.prod(case.shape))
    stream = torch.cuda.Stream(device=dev)

    def dev_t(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    phi = dev_t(phi_h)
    u, v, w = dev_t(u_h), dev_t(v_h), dev_t(w_h)
    kw = dict(krylov=args.krylov, stream=stream, nu1=NU1, nu2=NU2,
              use_graph="cycle" if args.host_loop else True)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    step_spread = {}

    def timed(solver, steps, warmup, b, p, sample_clocks=False):
        def step():
            p.zero_()
            solver.rho_mu(phi, case.eps, case.rho_pos, case.rho_neg)
            _, st = solver.solve(b, p, tol=TOL)
            return st

        sampler = ClockSampler(dev.index if dev.index is not None else 0)
        # the sampler starts before the warm-up so that nvidia-smi is running
        # when the timed region begins; only the samples inside it are kept
        with torch.cuda.stream(stream), (sampler if sample_clocks else _Null()):
            for _ in range(warmup):
                st = step()
            barrier()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            # an event after every step as well: the spread of the steps
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
            launches0 = solver.kernel_launches
            t0 = time.monotonic()
            e0.record(stream)
            for i in range(steps):
                st = step()
                ev[i].record(stream)
            e1.record(stream)
            torch.cuda.synchronize()
            t1 = time.monotonic()
            barrier()
        ms = e0.elapsed_time(e1)
        per = sorted([e0.elapsed_time(ev[0])] +
                     [ev[i - 1].elapsed_time(ev[i]) for i in range(1, steps)])
        if sample_clocks:  # the headline solve
            step_spread.update(min=per[0], median=per[len(per) // 2], max=per[-1])
        launches = solver.kernel_launches - launches0
        if sample_clocks:
            sampler.window(t0, t1)
        ms = max_over_ranks(ms, dev)
        return ms, st, launches, (sampler.summary() if sample_clocks else None)

    with torch.cuda.stream(stream):
        b = torch.empty(case.shape, dtype=torch.float64, device=dev)
        p = torch.zeros_like(b)
    mixed = PressurePoisson(case.shape, case.spacing, precision="mixed", **kw)
    mixed.divergence(u, v, w, case.dt, out=b)
    ms_mixed, st_mixed, launches, clocks = timed(mixed, args.steps, args.warmup, b, p,
                                                 sample_clocks=True)
    per_solve = ms_mixed / args.steps / world
    p_mixed = p.clone()

    fp64 = p_fp64 = None
    if not args.no_fp64:
        s64 = PressurePoisson(case.shape, case.spacing, precision="fp64", **kw)
        ms64, st64, _, _ = timed(s64, max(1, args.steps // 2), max(1, args.warmup // 2), b, p)
        fp64 = {"ms_per_solve": ms64 / max(1, args.steps // 2) / world, "cycles": st64["cycles"],
                "rel_residual": st64["rel_residual"],
                "p_rel_diff_vs_mixed": float((p - p_mixed).norm() / p.norm())}
        p_fp64 = p.clone()
        s64.close()

    # per-kernel profile pass (eager launches bracketed by CUDA events)
    roofline = None
    prof = None
    if not args.no_profile:
        with torch.cuda.stream(stream):
            mixed.set_profiling(True)
            p.zero_()
            mixed.rho_mu(phi, case.eps, case.rho_pos, case.rho_neg)
            _, st_prof = mixed.solve(b, p, tol=TOL)
            prof = mixed.profile()
            mixed.set_profiling(False)
        total = sum(v[0] for v in prof.values())
        ranked = sorted(((k, v) for k, v in prof.items()
                         if algorithmic_bytes_per_cell(k, 4, case.shape)),
                        key=lambda kv: -kv[1][0])
        cls, (ms_cls, cnt) = ranked[0]
        per_launch_ms = ms_cls / max(cnt, 1)
        # fine cells one launch processes: a smoother launch covers
        # sweeps/launches of a sweep (1/2 for the two-colour launches)
        units = n
        if cls == "smooth_fine":
            units = n * st_prof["cycles"] * (NU1 + NU2) / max(cnt, 1)
        alg = algorithmic_bytes_per_cell(cls, 4, case.shape) * units
        peak, peak_kind = measured_peaks()
        achieved = alg / (per_launch_ms * 1e-3) / 1e9
        tr = traffic_per_cell().get(cls)
        roofline = {"kernel": cls, "bound": "hbm", "achieved": achieved, "peak": peak,
                    "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                    "traffic": (tr * units if tr else None), "launch_ms": per_launch_ms,
                    "share": ms_cls / total if total else None,
                    "algorithmic_bytes_per_launch": alg, "cells_per_launch": units,
                    "bytes_per_cell": algorithmic_bytes_per_cell(cls, 4, case.shape),
                    "coefficients": "density form" if rho_form() else "stored FP32"}

    e2e = None
    if not args.no_e2e:
        # through the C ABI with pinned host buffers: H2D of phi, b and the
        # initial p, D2H of p, every step
        phi_p = torch.from_numpy(np.ascontiguousarray(phi_h)).pin_memory()
        b_p = b.cpu().pin_memory()
        p_p = torch.zeros(case.shape, dtype=torch.float64).pin_memory()
        with torch.cuda.stream(stream):
            def e2e_step():
                p_p.zero_()
                mixed.rho_mu(phi_p, case.eps, case.rho_pos, case.rho_neg)
                _, st = mixed.solve(b_p, p_p, tol=TOL)
                return st
            for _ in range(max(1, args.warmup)):
                e2e_step()
            barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                st_e = e2e_step()
            torch.cuda.synchronize()
            barrier()
            wall = (time.perf_counter() - t0) * 1e3
        wall = max_over_ranks(wall, dev)
        e2e = {"value": wall / args.steps / world, "unit": "ms", "h2d_bytes_per_step": 3 * 8 * n,
               "d2h_bytes_per_step": 8 * n, "timing": "host wall clock around synchronous C-ABI calls",
               "rel_residual": st_e["rel_residual"]}

    adj = None
    if not args.no_adjoint:
        try:
            adj = adjoint_section(dev, stream, scale=max(1, args.scale))
        except Exception as exc:  # report, keep the headline line
            adj = {"error": f"{type(exc).__name__}: {exc}"}

    multi = roll = None
    if not args.no_multi:
        try:
            multi = multi_bubble_section(dev, stream, scale=max(1, args.scale),
                                         oracle=not args.no_cpu and rank == 0)
        except Exception as exc:
            multi = {"error": f"{type(exc).__name__}: {exc}"}
        torch.cuda.empty_cache()
    if not args.no_rollout:
        try:
            roll = rollout_section(dev, stream, scale=max(1, args.scale))
        except Exception as exc:
            roll = {"error": f"{type(exc).__name__}: {exc}"}

    lset = None
    if not args.no_levelset:
        try:
            lset = levelset_section(dev, stream, case, phi_h, u_h, v_h, w_h)
        except Exception as exc:
            lset = {"error": f"{type(exc).__name__}: {exc}"}

    mom = None
    if not args.no_momentum:
        try:
            mom = momentum_section(dev, stream, case)
        except Exception as exc:
            mom = {"error": f"{type(exc).__name__}: {exc}"}
        torch.cuda.empty_cache()

    tstep = None
    if not args.no_timestep:
        try:
            tstep = timestep_section(dev, stream, case)
        except Exception as exc:
            tstep = {"error": f"{type(exc).__name__}: {exc}"}
        torch.cuda.empty_cache()

    cpu = parity = None
    if rank == 0 and not args.no_cpu:
        cpu, p_or, st_or, coef_or, b_or = cpu_baseline(case, phi_h, u_h, v_h, w_h,
                                                       args.cpu_seconds)
        parity = oracle_parity(p_or, st_or, coef_or, b_or, p_mixed.cpu().numpy(),
                               p_fp64.cpu().numpy() if p_fp64 is not None else None,
                               cpu["cores"])
        del p_or, coef_or, b_or

    if rank == 0:
        ws_gb = n * 8 * 9 / 1e9
        line = {"metric": METRIC, "value": per_solve, "unit": "ms", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_solve,
                "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32-in-f64", "data": "synthetic",
                "config": {"workload": workload_desc(case), "grid": list(case.shape[::-1]),
                           "tol": TOL, "cycles": st_mixed["cycles"],
                           "rel_residual": st_mixed["rel_residual"],
                           "precision": "FP32 V(2,2) cycles inside FP64 defect correction",
                           "krylov": bool(args.krylov),
                           "fp64": fp64,
                           "mixed_over_fp64": (per_solve / fp64["ms_per_solve"]) if fp64 else None,
                           "l2": f"inputs larger than L2: working set ~{ws_gb:.2f} GB vs 0.129 GB L2, "
                                 "each FP64 field alone exceeds it",
                           "parallelism": f"replicas x{world}"},
                "parity": parity,
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
                "gpu_launches": launches, "step_ms_spread": step_spread,
                "adjoint": adj, "multi_bubble": multi,
                "rollout": roll, "levelset": lset, "momentum": mom, "timestep": tstep}
        if prof:
            line["profile_ms"] = {k: round(v[0], 4) for k, v in prof.items()}
        line["config"].update(scalar_summary(fp64, parity, adj, multi, roll, tstep))
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def scalar_summary(fp64, parity, adj, multi, roll, tstep):
    """The figures of the nested sections as flat scalar keys (a reader of the
    line that keeps only scalars of `config` still sees them)."""
    out = {}

    def put(key, d, *path):
        for k in path:
            if not isinstance(d, dict) or k not in d:
                return
            d = d[k]
        if isinstance(d, (int, float, str, bool)):
            out[key] = d

    put("ms_fp64", fp64, "ms_per_solve")
    put("cycles_fp64", fp64, "cycles")
    for k in ("p_rel_l2_mixed_vs_oracle", "p_rel_l2_fp64_vs_oracle", "cycles_oracle",
              "p_rel_l2_fp64_vs_lex", "p_rel_l2_mixed_vs_lex", "p_rel_l2_oracle_vs_lex",
              "cycles_lex", "lex_ms", "p_err_mixed", "p_err_fp64", "p_err_oracle", "p_err_lex"):
        put(k, parity, k)
    put("ms_512_mixed", multi, "mixed", "ms_per_solve")
    put("ms_512_fp64", multi, "fp64", "ms_per_solve")
    put("mixed_over_fp64_512", multi, "mixed_over_fp64")
    put("cycles_512_mixed", multi, "mixed", "cycles")
    put("cycles_512_fp64", multi, "fp64", "cycles")
    put("p_rel_l2_512_mixed_vs_fp64", multi, "p_rel_diff_mixed_vs_fp64")
    put("p_rel_l2_512_mixed_vs_oracle", multi, "oracle", "p_rel_l2_mixed_vs_oracle")
    put("p_rel_l2_512_fp64_vs_oracle", multi, "oracle", "p_rel_l2_fp64_vs_oracle")
    put("cycles_512_oracle", multi, "oracle", "cycles")
    put("error_512", multi, "error")
    put("adj_forward_ms", adj, "forward_ms")
    put("adj_backward_ms", adj, "backward_ms")
    put("adj_backward_over_forward", adj, "backward_over_forward")
    put("adj_fd_max_rel", adj, "fd_max_rel_err")
    put("adj_fd_median_rel", adj, "fd_median_rel_err")
    put("adj_fd_directions", adj, "fd_directions")
    put("adj_fd_exact_max_rel", adj, "fd_exact_max_rel_err")
    put("adj_fd_exact_median_rel", adj, "fd_exact_median_rel_err")
    put("adj_loose_tol", adj, "loose_adjoint_tol")
    put("adj_loose_backward_over_forward", adj, "loose_backward_over_forward")
    put("adj_loose_fd_exact_max_rel", adj, "loose_fd_exact_max_rel_err")
    put("adj_vs_fp64_gradient_max_rel", adj, "fp64_gradient_max_rel_diff")
    put("error_adjoint", adj, "error")
    put("rollout_forward_ms", roll, "forward_ms")
    put("rollout_backward_ms", roll, "backward_ms")
    put("rollout_backward_over_forward", roll, "backward_over_forward")
    put("error_rollout", roll, "error")
    put("timestep_ms", tstep, "ms_without_redistancing")
    put("timestep_redistancing_ms", tstep, "ms_with_redistancing")
    put("error_timestep", tstep, "error")
    return out


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
