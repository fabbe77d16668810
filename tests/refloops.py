"""Plain-Python transliterations of the reference's loops, for small cases only.

Test infrastructure: used to pin the C oracle (oracle/oracle.c) against a
second, independent restatement written line by line from the reference's
Fortran, with its 1-based, ghost-padded indexing kept (numpy index = Fortran
index, arrays allocated 0..n+1 on every axis).  Nothing here is fast.

Sources (paths in the reference project):
  ppe_sor_init / ppe_sor_solver / ns_momentum_correction:
      "Two phase flows/newOpenMP/3D+IBM/src/ns_solver/ns_ppe_solver.f90:1-205"
      (2D: "Two phase flows/newOpenMP/2D/src/ns_solver/ns_ppe_solver.f90:1-171")
  bc (zero-gradient ghost copy): "Two phase flows/newOpenMP/2D/src/others/bcs.f90:1-26"
  ls_funs / rho_mu: "Two phase flows/newOpenMP/2D/src/interface_solver/others.f90:1-61"
  multigrid cycle: "DomainDecomposition/3D/src/others/multigrid_solver.f90:1-326"
      (2D: "DomainDecomposition/2D/src/others/multigrid_solver.f90")
  coarse solve: "DomainDecomposition/3D/lib/data/tree_multigrid.f90:1-238"
  outer loop: "DomainDecomposition/3D/src/ns_solver/ns_ppe_mg_solver.f90:17-50"
"""
import math

import numpy as np


def ls_funs_rho(phi, ls_wid, rho_12):
    """rho = heavy + rho_12 (1 - heavy), others.f90:14-27,54 (one value)."""
    eps = 1.0e-12
    x = phi / ls_wid
    if x > 1.0 - eps:
        heavy = 1.0
    elif x < -1.0 + eps:
        heavy = 0.0
    else:
        heavy = 0.5 * (1.0 + x + math.sin(math.pi * x) / math.pi)
    heavy = max(min(heavy, 1.0), 0.0)
    return heavy + rho_12 * (1.0 - heavy)


def pad(a):
    """(nz, ny, nx) numpy -> Fortran-indexed (0..nx+1, 0..ny+1, 0..nz+1) with
    zero-gradient ghosts (bc)."""
    nz, ny, nx = a.shape
    g = np.zeros((nx + 2, ny + 2, nz + 2))
    g[1:nx + 1, 1:ny + 1, 1:nz + 1] = a.transpose(2, 1, 0)
    bc(g)
    return g


def unpad(g):
    return np.ascontiguousarray(g[1:-1, 1:-1, 1:-1].transpose(2, 1, 0))


def bc(g):
    """Zero-gradient ghost copy on every wall (bcs.f90:1-26; job_bc order 0)."""
    g[0, :, :] = g[1, :, :]
    g[-1, :, :] = g[-2, :, :]
    g[:, 0, :] = g[:, 1, :]
    g[:, -1, :] = g[:, -2, :]
    g[:, :, 0] = g[:, :, 1]
    g[:, :, -1] = g[:, :, -2]


def ppe_sor_init(rho_g, nx, ny, nz, dx, dy, dz):
    """ns_ppe_solver.f90:1-65: the seven coefficient arrays r,l,f,b,u,d,c."""
    shp = rho_g.shape
    r, l, f, b, u, d, c = (np.zeros(shp) for _ in range(7))
    three_d = nz > 1
    for k in range(1, nz + 1):
        for j in range(1, ny + 1):
            for i in range(1, nx + 1):
                R = rho_g
                r[i, j, k] = 2.0 / (R[i, j, k] + R[i + 1, j, k]) / dx ** 2.0
                l[i, j, k] = 2.0 / (R[i, j, k] + R[i - 1, j, k]) / dx ** 2.0
                f[i, j, k] = 2.0 / (R[i, j, k] + R[i, j + 1, k]) / dy ** 2.0
                b[i, j, k] = 2.0 / (R[i, j, k] + R[i, j - 1, k]) / dy ** 2.0
                if three_d:
                    u[i, j, k] = 2.0 / (R[i, j, k] + R[i, j, k + 1]) / dz ** 2.0
                    d[i, j, k] = 2.0 / (R[i, j, k] + R[i, j, k - 1]) / dz ** 2.0
                c[i, j, k] = -(r[i, j, k] + l[i, j, k] + f[i, j, k] + b[i, j, k] + u[i, j, k]
                               + d[i, j, k])
                if i == 1:
                    c[i, j, k] += l[i, j, k]; l[i, j, k] = 0.0
                if i == nx:
                    c[i, j, k] += r[i, j, k]; r[i, j, k] = 0.0
                if j == 1:
                    c[i, j, k] += b[i, j, k]; b[i, j, k] = 0.0
                if j == ny:
                    c[i, j, k] += f[i, j, k]; f[i, j, k] = 0.0
                if three_d:
                    if k == 1:
                        c[i, j, k] += d[i, j, k]; d[i, j, k] = 0.0
                    if k == nz:
                        c[i, j, k] += u[i, j, k]; u[i, j, k] = 0.0
    return r, l, f, b, u, d, c


def ppe_apply(coe, p_g, nx, ny, nz):
    """sum coe p_nb + c p_i, the operator ppe_sor_solver relaxes."""
    r, l, f, b, u, d, c = coe
    out = np.zeros((nz, ny, nx))
    for k in range(1, nz + 1):
        for j in range(1, ny + 1):
            for i in range(1, nx + 1):
                P = p_g
                v = (r[i, j, k] * P[i + 1, j, k] + l[i, j, k] * P[i - 1, j, k]
                     + f[i, j, k] * P[i, j + 1, k] + b[i, j, k] * P[i, j - 1, k]
                     + c[i, j, k] * P[i, j, k])
                if nz > 1:
                    v += u[i, j, k] * P[i, j, k + 1] + d[i, j, k] * P[i, j, k - 1]
                out[k - 1, j - 1, i - 1] = v
    return out


def ppe_sor_solver(coe, src, p0, w, tol, max_iter):
    """ns_ppe_solver.f90:93-163 run serially (lexicographic k, j, i): returns
    (p, iterations, err)."""
    nz, ny, nx = src.shape
    r, l, f, b, u, d, c = coe
    P = pad(p0)
    S = pad(src)
    it = 0
    while True:
        it += 1
        tmp = P.copy()
        for k in range(1, nz + 1):
            for j in range(1, ny + 1):
                for i in range(1, nx + 1):
                    v = (S[i, j, k] - r[i, j, k] * P[i + 1, j, k] - l[i, j, k] * P[i - 1, j, k]
                         - f[i, j, k] * P[i, j + 1, k] - b[i, j, k] * P[i, j - 1, k])
                    if nz > 1:
                        v = v - u[i, j, k] * P[i, j, k + 1] - d[i, j, k] * P[i, j, k - 1]
                    P[i, j, k] = v / c[i, j, k]
        inner = P[1:nx + 1, 1:ny + 1, 1:nz + 1]
        sump = inner.sum() / (nx * ny * nz)
        inner -= sump
        inner[...] = w * inner + (1.0 - w) * tmp[1:nx + 1, 1:ny + 1, 1:nz + 1]
        err = np.abs(inner - tmp[1:nx + 1, 1:ny + 1, 1:nz + 1]).max()
        bc(P)
        if err < tol or it >= max_iter:
            break
    return unpad(P), it, err


def momentum_correction(rho, p, u, v, w, dt, dx, dy, dz):
    """ns_momentum_correction (ns_ppe_solver.f90:174-205) on interior faces;
    face arrays in the (nz, ny, nx+1) / (nz, ny+1, nx) / (nz+1, ny, nx) layout."""
    nz, ny, nx = p.shape
    u, v, w = u.copy(), v.copy(), w.copy()
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                if i + 1 < nx:
                    rf = (rho[k, j, i] + rho[k, j, i + 1]) / 2.0
                    px = (p[k, j, i + 1] - p[k, j, i]) / dx
                    u[k, j, i + 1] = u[k, j, i + 1] - dt * px / rf
                if j + 1 < ny:
                    rf = (rho[k, j, i] + rho[k, j + 1, i]) / 2.0
                    py = (p[k, j + 1, i] - p[k, j, i]) / dy
                    v[k, j + 1, i] = v[k, j + 1, i] - dt * py / rf
                if k + 1 < nz:
                    rf = (rho[k, j, i] + rho[k + 1, j, i]) / 2.0
                    pz = (p[k + 1, j, i] - p[k, j, i]) / dz
                    w[k + 1, j, i] = w[k + 1, j, i] - dt * pz / rf
    return u, v, w


# ---------------------------------------------------------------------------
# DomainDecomposition multigrid, one subdomain, constant coefficient.
# wall="ghost": multigrid_relax as written (the wall neighbour is the ghost
#   copied by the sync before the sweep, the diagonal a counts every face);
# wall="folded": the wall term folded into the diagonal as ppe_sor_init does
#   (the form the variable-coefficient solver uses).
# ---------------------------------------------------------------------------
class DDLevel:
    def __init__(self, nx, ny, nz, dx, dy, dz):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.dx, self.dy, self.dz = dx, dy, dz
        shp = (nx + 2, ny + 2, nz + 2)
        self.sol = np.zeros(shp)
        self.src = np.zeros(shp)
        self.res = np.zeros(shp)
        self.pol = np.zeros(shp)


class DDMultigrid:
    def __init__(self, nx, ny, nz, dx, dy, dz, levels, wall="folded"):
        self.three_d = nz > 1
        self.lv = []
        for lev in range(levels):
            f = 2 ** lev
            self.lv.append(DDLevel(nx // f, ny // f, nz // f if nz > 1 else 1, dx * f, dy * f,
                                   dz * f))
        self.wall = wall
        self._setup_coarse()

    def sync(self, a):
        bc(a)

    def relax(self, L, num):
        v = self.lv[L]
        dx2, dy2, dz2 = v.dx ** 2.0, v.dy ** 2.0, v.dz ** 2.0
        for _ in range(num):
            self.sync(v.sol)
            S, B = v.sol, v.src
            for k in range(1, v.nz + 1):
                for j in range(1, v.ny + 1):
                    for i in range(1, v.nx + 1):
                        if self.wall == "ghost":
                            a = -2.0 / dx2 - 2.0 / dy2 - (2.0 / dz2 if self.three_d else 0.0)
                            t = (B[i, j, k] - (S[i + 1, j, k] + S[i - 1, j, k]) / dx2
                                 - (S[i, j + 1, k] + S[i, j - 1, k]) / dy2)
                            if self.three_d:
                                t -= (S[i, j, k + 1] + S[i, j, k - 1]) / dz2
                            S[i, j, k] = t / a
                        else:
                            s, dsum = 0.0, 0.0
                            nb = [(i - 1, j, k, 1 / dx2, i > 1), (i + 1, j, k, 1 / dx2, i < v.nx),
                                  (i, j - 1, k, 1 / dy2, j > 1), (i, j + 1, k, 1 / dy2, j < v.ny)]
                            if self.three_d:
                                nb += [(i, j, k - 1, 1 / dz2, k > 1), (i, j, k + 1, 1 / dz2, k < v.nz)]
                            for (ii, jj, kk, cc, inside) in nb:
                                if inside:
                                    s += cc * S[ii, jj, kk]
                                    dsum += cc
                            S[i, j, k] = (s - B[i, j, k]) / dsum
            self.compat(v.sol, v)
        self.sync(v.sol)

    def compat(self, a, v):
        inner = a[1:v.nx + 1, 1:v.ny + 1, 1:v.nz + 1]
        inner -= inner.sum() / (v.nx * v.ny * v.nz)

    def residual(self, L):
        v = self.lv[L]
        self.sync(v.sol)
        S = v.sol
        tot = 0.0
        for k in range(1, v.nz + 1):
            for j in range(1, v.ny + 1):
                for i in range(1, v.nx + 1):
                    r = (v.src[i, j, k]
                         - (S[i + 1, j, k] - 2.0 * S[i, j, k] + S[i - 1, j, k]) / v.dx ** 2.0
                         - (S[i, j + 1, k] - 2.0 * S[i, j, k] + S[i, j - 1, k]) / v.dy ** 2.0)
                    if self.three_d:
                        r -= (S[i, j, k + 1] - 2.0 * S[i, j, k] + S[i, j, k - 1]) / v.dz ** 2.0
                    v.res[i, j, k] = r
                    tot += r ** 2.0
        return math.sqrt(tot / (v.nx * v.ny * v.nz))

    def restriction(self, L):
        self.relax(L, 2)
        self.residual(L)
        f, c = self.lv[L], self.lv[L + 1]
        for k in range(1, c.nz + 1):
            for j in range(1, c.ny + 1):
                for i in range(1, c.nx + 1):
                    R = f.res
                    if self.three_d:
                        s = (R[2 * i - 1, 2 * j - 1, 2 * k - 1] + R[2 * i, 2 * j - 1, 2 * k - 1]
                             + R[2 * i - 1, 2 * j, 2 * k - 1] + R[2 * i, 2 * j, 2 * k - 1]
                             + R[2 * i - 1, 2 * j - 1, 2 * k] + R[2 * i, 2 * j - 1, 2 * k]
                             + R[2 * i - 1, 2 * j, 2 * k] + R[2 * i, 2 * j, 2 * k]) / 8.0
                    else:
                        s = (R[2 * i - 1, 2 * j - 1, 1] + R[2 * i, 2 * j - 1, 1]
                             + R[2 * i - 1, 2 * j, 1] + R[2 * i, 2 * j, 1]) / 4.0
                    c.src[i, j, k] = s
                    c.sol[i, j, k] = 0.0
        self.compat(c.src, c)

    def _setup_coarse(self):
        """manager_mg_setup (tree_multigrid.f90:1-132), single subdomain."""
        v = self.lv[-1]
        n = v.nx * v.ny * v.nz
        A = np.zeros((n, n))
        node = lambda i, j, k: (k - 1) * v.nx * v.ny + (j - 1) * v.nx + (i - 1)  # noqa: E731
        for k in range(1, v.nz + 1):
            for j in range(1, v.ny + 1):
                for i in range(1, v.nx + 1):
                    q = node(i, j, k)
                    A[q, q] = -2.0 / v.dx ** 2.0 - 2.0 / v.dy ** 2.0
                    if self.three_d:
                        A[q, q] += -2.0 / v.dz ** 2.0
                    for (ii, jj, kk, h, inside) in [
                            (i - 1, j, k, v.dx, i > 1), (i + 1, j, k, v.dx, i < v.nx),
                            (i, j - 1, k, v.dy, j > 1), (i, j + 1, k, v.dy, j < v.ny)] + (
                            [(i, j, k - 1, v.dz, k > 1), (i, j, k + 1, v.dz, k < v.nz)]
                            if self.three_d else []):
                        if inside:
                            A[q, node(ii, jj, kk)] = 1.0 / h ** 2.0
                        else:
                            A[q, q] += 1.0 / h ** 2.0
        self.A = A
        self.node = node

    def final_exact(self):
        """manager_mg_solve_exact + mg_find_error + compatibility_sol.  The
        singular dgesv is replaced by the least-squares (minimum-norm, hence
        mean-free) solution."""
        v = self.lv[-1]
        n = v.nx * v.ny * v.nz
        B = np.zeros(n)
        for k in range(1, v.nz + 1):
            for j in range(1, v.ny + 1):
                for i in range(1, v.nx + 1):
                    B[self.node(i, j, k)] = v.src[i, j, k]
        x = np.linalg.lstsq(self.A, B, rcond=None)[0]
        err = B - self.A @ x
        if np.abs(err).max() > 1e-10:
            x = x + np.linalg.lstsq(self.A, err, rcond=None)[0]
        for k in range(1, v.nz + 1):
            for j in range(1, v.ny + 1):
                for i in range(1, v.nx + 1):
                    v.sol[i, j, k] = x[self.node(i, j, k)]
        self.compat(v.sol, v)

    def prolongation(self, L):
        f, c = self.lv[L], self.lv[L + 1]
        self.sync(c.sol)
        E = c.sol
        for k in range(1, c.nz + 1):
            for j in range(1, c.ny + 1):
                for i in range(1, c.nx + 1):
                    mx = 0.5 * (E[i + 1, j, k] - E[i - 1, j, k])
                    my = 0.5 * (E[i, j + 1, k] - E[i, j - 1, k])
                    if self.three_d:
                        mz = 0.5 * (E[i, j, k + 1] - E[i, j, k - 1])
                        for dk, sz in ((0, -1), (1, 1)):
                            for dj, sy in ((0, -1), (1, 1)):
                                for di, sx in ((0, -1), (1, 1)):
                                    f.pol[2 * i - 1 + di, 2 * j - 1 + dj, 2 * k - 1 + dk] = (
                                        E[i, j, k] + sx * 0.25 * mx + sy * 0.25 * my + sz * 0.25 * mz)
                    else:
                        for dj, sy in ((0, -1), (1, 1)):
                            for di, sx in ((0, -1), (1, 1)):
                                f.pol[2 * i - 1 + di, 2 * j - 1 + dj, 1] = (
                                    E[i, j, k] + sx * 0.25 * mx + sy * 0.25 * my)
        f.sol[1:f.nx + 1, 1:f.ny + 1, 1:f.nz + 1] += f.pol[1:f.nx + 1, 1:f.ny + 1, 1:f.nz + 1]
        self.relax(L, 2)

    def v_cycle(self):
        for L in range(len(self.lv) - 1):
            self.restriction(L)
        self.final_exact()
        for L in range(len(self.lv) - 2, -1, -1):
            self.prolongation(L)

    def solve(self, b, p0, cycles):
        """ppe_mg_solver's loop for a fixed number of cycles; returns p after
        each cycle (mean-free)."""
        f = self.lv[0]
        f.src = pad(b)
        f.sol = pad(p0)
        out = []
        for _ in range(cycles):
            self.v_cycle()
            out.append(unpad(f.sol).copy())
        return out


# ---------------------------------------------------------------------------
# Pressure-split projection of the DomainDecomposition solver
# ("DomainDecomposition/3D/src/ns_solver/ns_ppe_mg_solver.f90"):
# ppe_mg_solver_init :62-136, ppe_mg_solver_src :138-221,
# ppe_mg_correction :223-276, on one subdomain with job_bc ghosts.
# ---------------------------------------------------------------------------
def ppe_mg_split_src(rho, u, v, w, p_hat, rho_12, dt, dx, dy, dz):
    """coe%src of ppe_mg_solver_src (after ppe_mg_solver_init); u, v, w in the
    (nz, ny, nx+1) / (nz, ny+1, nx) / (nz+1, ny, nx) face layout, the
    reference's vel%x(i) being u[k, j, i] with 1-based i (face i+1/2)."""
    nz, ny, nx = rho.shape
    R = pad(rho)
    T = pad(p_hat)
    three_d = nz > 1
    src = np.zeros((nz, ny, nx))
    for k in range(1, nz + 1):
        for j in range(1, ny + 1):
            for i in range(1, nx + 1):
                r = 1.0 - 2.0 * rho_12 / (R[i, j, k] + R[i + 1, j, k])
                l = 1.0 - 2.0 * rho_12 / (R[i, j, k] + R[i - 1, j, k])
                f = 1.0 - 2.0 * rho_12 / (R[i, j, k] + R[i, j + 1, k])
                b = 1.0 - 2.0 * rho_12 / (R[i, j, k] + R[i, j - 1, k])
                r = r / dx ** 2.0
                l = l / dx ** 2.0
                f = f / dy ** 2.0
                b = b / dy ** 2.0
                if three_d:
                    uu = 1.0 - 2.0 * rho_12 / (R[i, j, k] + R[i, j, k + 1])
                    dd = 1.0 - 2.0 * rho_12 / (R[i, j, k] + R[i, j, k - 1])
                    uu = uu / dz ** 2.0
                    dd = dd / dz ** 2.0
                    c = -(r + l + f + b + uu + dd)
                    s = ((u[k - 1, j - 1, i] - u[k - 1, j - 1, i - 1]) / dx
                         + (v[k - 1, j, i - 1] - v[k - 1, j - 1, i - 1]) / dy
                         + (w[k, j - 1, i - 1] - w[k - 1, j - 1, i - 1]) / dz) / dt
                    s = (s * rho_12 + c * T[i, j, k]
                         + r * T[i + 1, j, k] + l * T[i - 1, j, k]
                         + f * T[i, j + 1, k] + b * T[i, j - 1, k]
                         + uu * T[i, j, k + 1] + dd * T[i, j, k - 1])
                else:
                    c = -(r + l + f + b)
                    s = ((u[k - 1, j - 1, i] - u[k - 1, j - 1, i - 1]) / dx
                         + (v[k - 1, j, i - 1] - v[k - 1, j - 1, i - 1]) / dy) / dt
                    s = (s * rho_12 + c * T[i, j, k]
                         + r * T[i + 1, j, k] + l * T[i - 1, j, k]
                         + f * T[i, j + 1, k] + b * T[i, j - 1, k])
                src[k - 1, j - 1, i - 1] = s
    return src


def ppe_mg_split_correction(rho, p, p_hat, u, v, w, rho_12, dt, dx, dy, dz):
    """ppe_mg_correction on copies of u, v, w (every cell's high faces; the
    wall faces see zero differences through the ghosts)."""
    nz, ny, nx = rho.shape
    R, P, T = pad(rho), pad(p), pad(p_hat)
    u, v, w = u.copy(), v.copy(), w.copy()
    for k in range(1, nz + 1):
        for j in range(1, ny + 1):
            for i in range(1, nx + 1):
                s = 1.0 / rho_12 * (P[i + 1, j, k] - P[i, j, k]) / dx
                s = s + (2.0 / (R[i, j, k] + R[i + 1, j, k]) - 1.0 / rho_12) * \
                    (T[i + 1, j, k] - T[i, j, k]) / dx
                u[k - 1, j - 1, i] = u[k - 1, j - 1, i] - s * dt
                s = 1.0 / rho_12 * (P[i, j + 1, k] - P[i, j, k]) / dy
                s = s + (2.0 / (R[i, j, k] + R[i, j + 1, k]) - 1.0 / rho_12) * \
                    (T[i, j + 1, k] - T[i, j, k]) / dy
                v[k - 1, j, i - 1] = v[k - 1, j, i - 1] - s * dt
                if nz > 1:
                    s = 1.0 / rho_12 * (P[i, j, k + 1] - P[i, j, k]) / dz
                    s = s + (2.0 / (R[i, j, k] + R[i, j, k + 1]) - 1.0 / rho_12) * \
                        (T[i, j, k + 1] - T[i, j, k]) / dz
                    w[k, j - 1, i - 1] = w[k, j - 1, i - 1] - s * dt
    return u, v, w


# --- level-set advection ------------------------------------------------------------
# level_set_rk3_solver / level_set_rk3_source_setup / level_set_rk3_source /
# wenojs_flux_split: "Two phase flows/newOpenMP/2D/src/interface_solver/
# level_set_rk3_solver.f90:1-186" (3D: "Two phase flows/newOpenMP/3D+IBM/src/
# interface_solver/level_set_rk3_solver.f90:1-215"); arrays carry ghc = 3
# ghost layers on every axis (numpy index = Fortran index + 3).
LS_GHC = 3


def _sq(x):
    """x**2 as the compiled reference evaluates it: one rounded product."""
    return x * x


def _bc3(a):
    """bc with ghc ghost layers: copy the first/last interior cell outwards."""
    g = LS_GHC
    for ax in range(a.ndim):
        n = a.shape[ax] - 2 * g
        for m in range(1, g + 1):
            lo = [slice(None)] * a.ndim
            src = [slice(None)] * a.ndim
            lo[ax] = g - m
            src[ax] = g
            a[tuple(lo)] = a[tuple(src)]
            hi = [slice(None)] * a.ndim
            srch = [slice(None)] * a.ndim
            hi[ax] = g + n - 1 + m
            srch[ax] = g + n - 1
            a[tuple(hi)] = a[tuple(srch)]


def _wenojs_flux_split(f, g, nn):
    """One line: returns (fp, gm) over i = is-ghc+2 .. ie+ghc-3 (numpy 2 .. nn+2)."""
    eps = 1.0e-13
    fp = [0.0] * len(f)
    gm = [0.0] * len(g)
    for i in range(2, nn + 3):
        b1 = 13.0 * _sq(g[i - 2] - 2.0 * g[i - 1] + g[i]) + 3.0 * _sq(g[i - 2] - 4.0 * g[i - 1] + 3.0 * g[i])
        b2 = 13.0 * _sq(g[i - 1] - 2.0 * g[i] + g[i + 1]) + 3.0 * _sq(g[i - 1] - g[i + 1])
        b3 = 13.0 * _sq(g[i] - 2.0 * g[i + 1] + g[i + 2]) + 3.0 * _sq(3.0 * g[i] - 4.0 * g[i + 1] + g[i + 2])
        a1 = 1.0 / _sq(eps + b1)
        a2 = 6.0 / _sq(eps + b2)
        a3 = 3.0 / _sq(eps + b3)
        w1 = a1 / (a1 + a2 + a3)
        w2 = a2 / (a1 + a2 + a3)
        w3 = a3 / (a1 + a2 + a3)
        gm[i] = (w1 / 3.0 * g[i - 2] - (7.0 * w1 + w2) / 6.0 * g[i - 1]
                 + (11.0 * w1 + 5.0 * w2 + 2.0 * w3) / 6.0 * g[i]
                 + (2.0 * w2 + 5.0 * w3) / 6.0 * g[i + 1] - w3 / 6.0 * g[i + 2])
    for i in range(2, nn + 3):
        b3 = 13.0 * _sq(f[i - 1] - 2.0 * f[i] + f[i + 1]) + 3.0 * _sq(f[i - 1] - 4.0 * f[i] + 3.0 * f[i + 1])
        b2 = 13.0 * _sq(f[i] - 2.0 * f[i + 1] + f[i + 2]) + 3.0 * _sq(f[i] - f[i + 2])
        b1 = 13.0 * _sq(f[i + 1] - 2.0 * f[i + 2] + f[i + 3]) + 3.0 * _sq(3.0 * f[i + 1] - 4.0 * f[i + 2] + f[i + 3])
        a1 = 1.0 / _sq(eps + b1)
        a2 = 6.0 / _sq(eps + b2)
        a3 = 3.0 / _sq(eps + b3)
        w1 = a1 / (a1 + a2 + a3)
        w2 = a2 / (a1 + a2 + a3)
        w3 = a3 / (a1 + a2 + a3)
        fp[i] = (w3 * (-f[i - 1] + 5.0 * f[i] + 2.0 * f[i + 1]) / 6.0
                 + w2 * (2.0 * f[i] + 5.0 * f[i + 1] - f[i + 2]) / 6.0
                 + w1 * (11.0 * f[i + 1] - 7.0 * f[i + 2] + 2.0 * f[i + 3]) / 6.0)
    return fp, gm


def level_set_rk3_solver(phi, u, v, w, dt, dx, dy, dz, steps=1):
    """phi, u, v, w: (nz, ny, nx) cell arrays (w ignored when nz == 1).
    Returns phi after `steps` steps."""
    nz, ny, nx = phi.shape
    three = nz > 1
    g = LS_GHC
    # Fortran (i, j, k) layout: numpy arrays of shape (nx+2g, ny+2g, nz+2g)
    P = np.zeros((nx + 2 * g, ny + 2 * g, nz + 2 * g))
    P[g:g + nx, g:g + ny, g:g + nz] = np.transpose(phi, (2, 1, 0))
    vel = [np.transpose(a, (2, 1, 0)) for a in ((u, v, w) if three else (u, v))]
    h = (dx, dy, dz)
    n = (nx, ny, nz)

    def source():
        S1, S2, SS1, SS2 = [], [], [], []
        for a in range(len(vel)):
            s1 = np.zeros_like(P)
            s2 = np.zeros_like(P)
            for i in range(nx):
                for j in range(ny):
                    for k in range(nz):
                        un = vel[a][i, j, k]
                        ph = P[g + i, g + j, g + k]
                        s1[g + i, g + j, g + k] = 0.5 * (un + abs(un)) * ph
                        s2[g + i, g + j, g + k] = 0.5 * (un - abs(un)) * ph
            _bc3(s1)
            _bc3(s2)
            ss1 = np.zeros_like(P)
            ss2 = np.zeros_like(P)
            # lines along axis a through every interior point of the other axes
            others = [b for b in range(3) if b != a]
            for p0 in range(n[others[0]]):
                for p1 in range(n[others[1]]):
                    idx = [0, 0, 0]
                    idx[others[0]] = g + p0
                    idx[others[1]] = g + p1
                    sl = list(idx)
                    sl[a] = slice(None)
                    fp, gm = _wenojs_flux_split(list(s2[tuple(sl)]), list(s1[tuple(sl)]), n[a])
                    ss2[tuple(sl)] = fp
                    ss1[tuple(sl)] = gm
            SS1.append(ss1)
            SS2.append(ss2)
        out = np.zeros((nx, ny, nz))
        for i in range(nx):
            for j in range(ny):
                for k in range(nz):
                    I, J, K = g + i, g + j, g + k
                    s = -(SS1[0][I, J, K] + SS2[0][I, J, K] - SS1[0][I - 1, J, K] - SS2[0][I - 1, J, K]) / dx \
                        - (SS1[1][I, J, K] + SS2[1][I, J, K] - SS1[1][I, J - 1, K] - SS2[1][I, J - 1, K]) / dy
                    if three:
                        s = s - (SS1[2][I, J, K] + SS2[2][I, J, K] - SS1[2][I, J, K - 1]
                                 - SS2[2][I, J, K - 1]) / dz
                    out[i, j, k] = s
        return out

    for _ in range(steps):
        l1 = source()
        P[g:g + nx, g:g + ny, g:g + nz] = P[g:g + nx, g:g + ny, g:g + nz] + l1 * dt
        _bc3(P)
        l2 = source()
        P[g:g + nx, g:g + ny, g:g + nz] = P[g:g + nx, g:g + ny, g:g + nz] + ((-3.0 * l1 + l2) / 4.0) * dt
        _bc3(P)
        l3 = source()
        P[g:g + nx, g:g + ny, g:g + nz] = (P[g:g + nx, g:g + ny, g:g + nz]
                                          + ((-l1 - l2 + 8.0 * l3) / 12.0) * dt)
        _bc3(P)
    return np.ascontiguousarray(np.transpose(P[g:g + nx, g:g + ny, g:g + nz], (2, 1, 0)))


# --- level-set redistancing ---------------------------------------------------------
# level_set_rk3_redis / level_set_redis_init / level_set_redis_stable /
# level_set_rk3_redis_solver / level_set_redis_gradient / wenojs_flux /
# level_set_redis_lambda: "Two phase flows/newOpenMP/2D/src/interface_solver/
# level_set_rk3_redis.f90:1-361" (3D: "Two phase flows/newOpenMP/3D+IBM/src/
# interface_solver/level_set_rk3_redis.f90"); ls_funs: ".../3D+IBM/src/
# interface_solver/others.f90:1-37".  Fortran (i, j, k) arrays with ghc = 3.
def _ls_funs(P, ls_wid):
    eps = 1.0e-12
    pi = math.acos(-1.0)
    H = np.zeros_like(P)
    D = np.zeros_like(P)
    S = np.zeros_like(P)
    for idx in np.ndindex(P.shape):
        x = P[idx] / ls_wid
        if x > 1.0 - eps:
            heavy, hp = 1.0, 0.0
        elif x < -1.0 + eps:
            heavy, hp = 0.0, 0.0
        else:
            heavy = 0.5 * (1.0 + x + math.sin(pi * x) / pi)
            hp = 0.5 * (1.0 + math.cos(pi * x)) / ls_wid
        heavy = max(min(heavy, 1.0), 0.0)
        H[idx], D[idx], S[idx] = heavy, hp, 2.0 * heavy - 1.0
    return H, D, S


def _wenojs_flux(f, nn):
    """One line: (fp, fm) over i = is-1 .. ie (numpy 2 .. nn+2), EPS = 1e-10."""
    eps = 1.0e-10
    fp = [0.0] * len(f)
    fm = [0.0] * len(f)
    for i in range(2, nn + 3):
        b1 = 13.0 * _sq(f[i - 2] - 2.0 * f[i - 1] + f[i]) + 3.0 * _sq(f[i - 2] - 4.0 * f[i - 1] + 3.0 * f[i])
        b2 = 13.0 * _sq(f[i - 1] - 2.0 * f[i] + f[i + 1]) + 3.0 * _sq(f[i - 1] - f[i + 1])
        b3 = 13.0 * _sq(f[i] - 2.0 * f[i + 1] + f[i + 2]) + 3.0 * _sq(3.0 * f[i] - 4.0 * f[i + 1] + f[i + 2])
        a1 = 1.0 / _sq(eps + b1)
        a2 = 6.0 / _sq(eps + b2)
        a3 = 3.0 / _sq(eps + b3)
        w1 = a1 / (a1 + a2 + a3)
        w2 = a2 / (a1 + a2 + a3)
        w3 = a3 / (a1 + a2 + a3)
        fm[i] = (w1 / 3.0 * f[i - 2] - (7.0 * w1 + w2) / 6.0 * f[i - 1]
                 + (11.0 * w1 + 5.0 * w2 + 2.0 * w3) / 6.0 * f[i]
                 + (2.0 * w2 + 5.0 * w3) / 6.0 * f[i + 1] - w3 / 6.0 * f[i + 2])
        b3 = 13.0 * _sq(f[i - 1] - 2.0 * f[i] + f[i + 1]) + 3.0 * _sq(f[i - 1] - 4.0 * f[i] + 3.0 * f[i + 1])
        b2 = 13.0 * _sq(f[i] - 2.0 * f[i + 1] + f[i + 2]) + 3.0 * _sq(f[i] - f[i + 2])
        b1 = 13.0 * _sq(f[i + 1] - 2.0 * f[i + 2] + f[i + 3]) + 3.0 * _sq(3.0 * f[i + 1] - 4.0 * f[i + 2] + f[i + 3])
        a1 = 1.0 / _sq(eps + b1)
        a2 = 6.0 / _sq(eps + b2)
        a3 = 3.0 / _sq(eps + b3)
        w1 = a1 / (a1 + a2 + a3)
        w2 = a2 / (a1 + a2 + a3)
        w3 = a3 / (a1 + a2 + a3)
        fp[i] = (w3 * (-f[i - 1] + 5.0 * f[i] + 2.0 * f[i + 1]) / 6.0
                 + w2 * (2.0 * f[i] + 5.0 * f[i + 1] - f[i + 2]) / 6.0
                 + w1 * (11.0 * f[i + 1] - 7.0 * f[i + 2] + 2.0 * f[i + 3]) / 6.0)
    return fp, fm


def level_set_rk3_redis(phi, ls_wid, rdt, dx, dy, dz, rho_12=1e-3, btn=1, max_iter=100000):
    """phi: (nz, ny, nx).  Returns (phi, iterations, last error)."""
    nz, ny, nx = phi.shape
    three = nz > 1
    g = LS_GHC
    n = (nx, ny, nz)
    h = (dx, dy, dz)
    axes = 3 if three else 2
    P = np.zeros((nx + 2 * g, ny + 2 * g, nz + 2 * g))
    P[g:g + nx, g:g + ny, g:g + nz] = np.transpose(phi, (2, 1, 0))
    _bc3(P)
    inner = (slice(g, g + nx), slice(g, g + ny), slice(g, g + nz))

    def gradient(sign_tmp):
        S1, S2 = [], []
        for a in range(axes):
            N = np.zeros_like(P)
            for i in range(nx):
                for j in range(ny):
                    for k in range(nz):
                        c = [g + i, g + j, g + k]
                        m = list(c)
                        m[a] -= 1
                        N[tuple(c)] = (P[tuple(c)] - P[tuple(m)]) / h[a]
            _bc3(N)
            s1 = np.zeros_like(P)
            s2 = np.zeros_like(P)
            others = [b for b in range(3) if b != a]
            for p0 in range(n[others[0]]):
                for p1 in range(n[others[1]]):
                    idx = [0, 0, 0]
                    idx[others[0]] = g + p0
                    idx[others[1]] = g + p1
                    sl = list(idx)
                    sl[a] = slice(None)
                    fp, fm = _wenojs_flux(list(N[tuple(sl)]), n[a])
                    s1[tuple(sl)] = fp
                    s2[tuple(sl)] = fm
            S1.append(s1)
            S2.append(s2)
        G = np.zeros_like(P)
        for i in range(nx):
            for j in range(ny):
                for k in range(nz):
                    I = (g + i, g + j, g + k)
                    tot = 0.0
                    for a in range(axes):
                        pm = -min(S1[a][I], 0.0)
                        pp = max(S1[a][I], 0.0)
                        mm = -min(S2[a][I], 0.0)
                        mp = max(S2[a][I], 0.0)
                        t = max(pm, mp) if sign_tmp[I] >= 0.0 else max(pp, mm)
                        tot = _sq(t) if a == 0 else tot + _sq(t)
                    G[I] = math.sqrt(tot)
        return G

    def lam_s1(sign_tmp, G):
        if btn == 0:
            return np.zeros_like(P)
        H, D, _ = _ls_funs(P, ls_wid)
        s2 = np.zeros_like(P)
        s3 = np.zeros_like(P)
        for I in np.ndindex(nx, ny, nz):
            J = (g + I[0], g + I[1], g + I[2])
            lam = (2.0 * (1.0 - rho_12) * H[J] + rho_12) * D[J] if three else D[J]
            s2[J] = lam * sign_tmp[J] * (G[J] - 1.0)
            s3[J] = G[J] * D[J] * lam
        _bc3(s2)
        _bc3(s3)
        out = np.zeros_like(P)
        wgt = 51.0 if three else 16.0
        kr = (-1, 0, 1) if three else (0,)
        for I in np.ndindex(nx, ny, nz):
            J = (g + I[0], g + I[1], g + I[2])
            a = wgt * s2[J]
            b = wgt * s3[J]
            for kk in kr:
                for jj in (-1, 0, 1):
                    for ii in (-1, 0, 1):
                        K = (J[0] + ii, J[1] + jj, J[2] + kk)
                        a = a + s2[K]
                        b = b + s3[K]
            out[J] = a / b * D[J] if abs(b) > 1.0e-12 else 0.0
        return out

    _, _, sign_tmp = _ls_funs(P, ls_wid)
    if btn == 0:
        sign_tmp = P.copy()
        G = gradient(sign_tmp)
        gmax = 0.0
        for I in np.ndindex(nx, ny, nz):
            gmax = max(gmax, G[g + I[0], g + I[1], g + I[2]])
        P[inner] = P[inner] / gmax
        _bc3(P)
    ext = max(nx * dx, ny * dy, nz * dz) if three else max(nx * dx, ny * dy)
    timestop = 1.5 * ext if btn == 0 else 3.0 * dx
    tol = 1.0e-5 if three else 1.0e-8
    it = 0
    time = 0.0
    error = 0.0
    while it < max_iter:
        it += 1
        time = time + rdt
        tmp = P[inner].copy()
        l1 = l2 = None
        for stage in (1, 2, 3):
            G = gradient(sign_tmp)
            S1 = lam_s1(sign_tmp, G)
            L = (sign_tmp[inner] - S1[inner]) * G[inner] - sign_tmp[inner]
            if stage == 1:
                l1 = L
                src = L
            elif stage == 2:
                l2 = L
                src = (-3.0 * l1 + L) / 4.0
            else:
                src = (-l1 - l2 + 8.0 * L) / 12.0
            P[inner] = P[inner] - rdt * src
            _bc3(P)
        error = float(np.abs(tmp - P[inner]).max())
        if time > timestop or error <= tol:
            break
    return np.ascontiguousarray(np.transpose(P[inner], (2, 1, 0))), it, error


# ---------------------------------------------------------------------------
# Momentum step of the Adams-Bashforth solver, literally:
#   ns_ab_adv_source_sec  "Two phase flows/newOpenMP/2D/src/ns_solver/ns_ab_adv.f90:1-42"
#                         (3D: ".../3D+IBM/src/ns_solver/ns_ab_adv.f90:1-73")
#   sec_part1..3          ".../2D/src/ns_solver/ns_ab_diff.f90:10-135" (3D :10-199)
#   ns_ab_setup, ns_ab_predictor
#                         ".../2D/src/ns_solver/admas_bashforth_solver.f90:19-93"
#   find_stag_vel, velbc  ".../2D/src/others/bcs.f90:28-148,265-400" (3D :44-257,464-774)
# Arrays are the reference's ghost-padded boxes (numpy shape (ny+2g, nx+2g) or
# (nz+2g, ny+2g, nx+2g)); R[i, j(, k)] reads them with the Fortran indices.
# ---------------------------------------------------------------------------
class R:
    def __init__(self, a, g):
        self.a, self.g, self.three = a, g, a.ndim == 3

    def _ix(self, ijk):
        g = self.g
        if self.three:
            i, j, k = ijk
            return (k - 1 + g, j - 1 + g, i - 1 + g)
        i, j = ijk
        return (j - 1 + g, i - 1 + g)

    def __getitem__(self, ijk):
        return float(self.a[self._ix(ijk)])

    def __setitem__(self, ijk, val):
        self.a[self._ix(ijk)] = val


def ns_ab_diff_sec_2d(uo, vo, rho, mu, delta, phi, nrm_x, nrm_y, curv, g, nx, ny, dx, dy, re,
                      mu_12, gx, gy, btn_g, btn_sf, fr, we):
    """velsrc%tmp (x, y) of sec_part1 + sec_part2 + sec_part3, 2D."""
    U, V, RO, MU, DE, PH = (R(a, g) for a in (uo, vo, rho, mu, delta, phi))
    NX, NY, CU = R(nrm_x, g), R(nrm_y, g), R(curv, g)
    tx, ty = np.zeros_like(uo), np.zeros_like(vo)
    TX, TY = R(tx, g), R(ty, g)
    for j in range(1, ny + 1):
        for i in range(1, nx + 1):
            rho_ = 0.5 * (RO[i, j] + RO[i + 1, j])
            mu_ = 0.5 * (MU[i, j] + MU[i + 1, j])
            xx = (U[i + 1, j] - 2.0 * U[i, j] + U[i - 1, j]) / _sq(dx)
            yy = (U[i, j + 1] - 2.0 * U[i, j] + U[i, j - 1]) / _sq(dy)
            dif_x = mu_ / rho_ * xx / re
            dif_y = mu_ / rho_ * yy / re
            TX[i, j] = dif_x + dif_y
            rho_ = 0.5 * (RO[i, j] + RO[i, j + 1])
            mu_ = 0.5 * (MU[i, j] + MU[i, j + 1])
            xx = (V[i + 1, j] - 2.0 * V[i, j] + V[i - 1, j]) / _sq(dx)
            yy = (V[i, j + 1] - 2.0 * V[i, j] + V[i, j - 1]) / _sq(dy)
            dif_x = mu_ / rho_ * xx / re
            dif_y = mu_ / rho_ * yy / re
            TY[i, j] = dif_x + dif_y
    for j in range(1, ny + 1):
        for i in range(1, nx + 1):
            rho_ = 0.5 * (RO[i, j] + RO[i + 1, j])
            delta_ = 0.5 * (DE[i, j] + DE[i + 1, j])
            ux = 0.5 * (U[i + 1, j] - U[i - 1, j]) / dx
            uy = 0.5 * (U[i, j + 1] - U[i, j - 1]) / dy
            vx = 0.5 * (V[i + 1, j] - V[i, j] + V[i + 1, j - 1] - V[i, j - 1]) / dx
            phix = (PH[i + 1, j] - PH[i, j]) / dx
            phiy = 0.25 * (PH[i + 1, j + 1] - PH[i + 1, j - 1] + PH[i, j + 1] - PH[i, j - 1]) / dy
            dif_x = (1.0 - mu_12) * delta_ * phix * 2.0 * ux / (rho_ * re)
            dif_y = (1.0 - mu_12) * delta_ * phiy * (uy + vx) / (rho_ * re)
            TX[i, j] = TX[i, j] + dif_x + dif_y
            rho_ = 0.5 * (RO[i, j] + RO[i, j + 1])
            delta_ = 0.5 * (DE[i, j] + DE[i, j + 1])
            vx = 0.5 * (V[i + 1, j] - V[i - 1, j]) / dx
            vy = 0.5 * (V[i, j + 1] - V[i, j - 1]) / dy
            uy = 0.5 * (U[i, j + 1] - U[i, j] + U[i - 1, j + 1] - U[i - 1, j]) / dy
            phix = 0.25 * (PH[i + 1, j] - PH[i - 1, j] + PH[i + 1, j + 1] - PH[i - 1, j + 1]) / dx
            phiy = (PH[i, j + 1] - PH[i, j]) / dy
            dif_x = (1.0 - mu_12) * delta_ * phix * (uy + vx) / (rho_ * re)
            dif_y = (1.0 - mu_12) * delta_ * phiy * 2.0 * vy / (rho_ * re)
            TY[i, j] = TY[i, j] + dif_x + dif_y
    for j in range(1, ny + 1):
        for i in range(1, nx + 1):
            rho_ = 0.5 * (RO[i, j] + RO[i + 1, j])
            delta_ = 0.5 * (DE[i, j] + DE[i + 1, j])
            curv_ = (CU[i, j] + CU[i + 1, j]) / 2.0
            phix = 0.5 * (NX[i, j] + NX[i + 1, j])
            TX[i, j] = TX[i, j] + gx * btn_g / fr - btn_sf * curv_ * delta_ * phix / (we * rho_)
            rho_ = 0.5 * (RO[i, j] + RO[i, j + 1])
            delta_ = 0.5 * (DE[i, j] + DE[i, j + 1])
            curv_ = (CU[i, j] + CU[i, j + 1]) / 2.0
            phiy = 0.5 * (NY[i, j] + NY[i, j + 1])
            TY[i, j] = TY[i, j] + gy * btn_g / fr - btn_sf * curv_ * delta_ * phiy / (we * rho_)
    return tx, ty


def ns_ab_diff_sec_3d(uo, vo, wo, rho, mu, delta, phi, nrm_x, nrm_y, nrm_z, curv, g, nx, ny, nz,
                      dx, dy, dz, re, mu_12, gx, gy, gz, btn_g, btn_sf, fr, we):
    """velsrc%tmp (x, y, z) of sec_part1 + sec_part2 + sec_part3, 3D."""
    U, V, W, RO, MU, DE, PH = (R(a, g) for a in (uo, vo, wo, rho, mu, delta, phi))
    NX, NY, NZ, CU = R(nrm_x, g), R(nrm_y, g), R(nrm_z, g), R(curv, g)
    tx, ty, tz = np.zeros_like(uo), np.zeros_like(vo), np.zeros_like(wo)
    TX, TY, TZ = R(tx, g), R(ty, g), R(tz, g)
    rng = [(i, j, k) for k in range(1, nz + 1) for j in range(1, ny + 1) for i in range(1, nx + 1)]
    for i, j, k in rng:
        for (T, F, o) in ((TX, U, (1, 0, 0)), (TY, V, (0, 1, 0)), (TZ, W, (0, 0, 1))):
            a, b, c = i + o[0], j + o[1], k + o[2]
            rho_ = 0.5 * (RO[i, j, k] + RO[a, b, c])
            mu_ = 0.5 * (MU[i, j, k] + MU[a, b, c])
            xx = (F[i + 1, j, k] - 2.0 * F[i, j, k] + F[i - 1, j, k]) / _sq(dx)
            yy = (F[i, j + 1, k] - 2.0 * F[i, j, k] + F[i, j - 1, k]) / _sq(dy)
            zz = (F[i, j, k + 1] - 2.0 * F[i, j, k] + F[i, j, k - 1]) / _sq(dz)
            dif_x = mu_ / rho_ * xx / re
            dif_y = mu_ / rho_ * yy / re
            dif_z = mu_ / rho_ * zz / re
            T[i, j, k] = dif_x + dif_y + dif_z
    for i, j, k in rng:
        rho_ = 0.5 * (RO[i, j, k] + RO[i + 1, j, k])
        delta_ = 0.5 * (DE[i, j, k] + DE[i + 1, j, k])
        ux = 0.5 * (U[i + 1, j, k] - U[i - 1, j, k]) / dx
        uy = 0.5 * (U[i, j + 1, k] - U[i, j - 1, k]) / dy
        uz = 0.5 * (U[i, j, k + 1] - U[i, j, k - 1]) / dz
        vx = 0.5 * (V[i + 1, j, k] - V[i, j, k] + V[i + 1, j - 1, k] - V[i, j - 1, k]) / dx
        wx = 0.5 * (W[i + 1, j, k] - W[i, j, k] + W[i + 1, j, k - 1] - W[i, j, k - 1]) / dx
        phix = (PH[i + 1, j, k] - PH[i, j, k]) / dx
        phiy = 0.25 * (PH[i + 1, j + 1, k] - PH[i + 1, j - 1, k] + PH[i, j + 1, k] - PH[i, j - 1, k]) / dy
        phiz = 0.25 * (PH[i + 1, j, k + 1] - PH[i + 1, j, k - 1] + PH[i, j, k + 1] - PH[i, j, k - 1]) / dz
        dif_x = (1.0 - mu_12) * delta_ * phix * 2.0 * ux / (rho_ * re)
        dif_y = (1.0 - mu_12) * delta_ * phiy * (uy + vx) / (rho_ * re)
        dif_z = (1.0 - mu_12) * delta_ * phiz * (uz + wx) / (rho_ * re)
        TX[i, j, k] = TX[i, j, k] + dif_x + dif_y + dif_z
        rho_ = 0.5 * (RO[i, j, k] + RO[i, j + 1, k])
        delta_ = 0.5 * (DE[i, j, k] + DE[i, j + 1, k])
        vx = 0.5 * (V[i + 1, j, k] - V[i - 1, j, k]) / dx
        vy = 0.5 * (V[i, j + 1, k] - V[i, j - 1, k]) / dy
        vz = 0.5 * (V[i, j, k + 1] - V[i, j, k - 1]) / dz
        uy = 0.5 * (U[i, j + 1, k] - U[i, j, k] + U[i - 1, j + 1, k] - U[i - 1, j, k]) / dy
        wy = 0.5 * (W[i, j + 1, k] - W[i, j, k] + W[i, j + 1, k - 1] - W[i, j, k - 1]) / dy
        phix = 0.25 * (PH[i + 1, j, k] - PH[i - 1, j, k] + PH[i + 1, j + 1, k] - PH[i - 1, j + 1, k]) / dx
        phiy = (PH[i, j + 1, k] - PH[i, j, k]) / dy
        phiz = 0.25 * (PH[i, j + 1, k + 1] - PH[i, j + 1, k - 1] + PH[i, j, k + 1] - PH[i, j, k - 1]) / dz
        dif_x = (1.0 - mu_12) * delta_ * phix * (uy + vx) / (rho_ * re)
        dif_y = (1.0 - mu_12) * delta_ * phiy * 2.0 * vy / (rho_ * re)
        dif_z = (1.0 - mu_12) * delta_ * phiz * (wy + vz) / (rho_ * re)
        TY[i, j, k] = TY[i, j, k] + dif_x + dif_y + dif_z
        rho_ = 0.5 * (RO[i, j, k] + RO[i, j, k + 1])
        delta_ = 0.5 * (DE[i, j, k] + DE[i, j, k + 1])
        wx = 0.5 * (W[i + 1, j, k] - W[i - 1, j, k]) / dx
        wy = 0.5 * (W[i, j + 1, k] - W[i, j - 1, k]) / dy
        wz = 0.5 * (W[i, j, k + 1] - W[i, j, k - 1]) / dz
        uz = 0.5 * (U[i, j, k + 1] - U[i, j, k] + U[i - 1, j, k + 1] - U[i - 1, j, k]) / dz
        vz = 0.5 * (V[i, j, k + 1] - V[i, j, k] + V[i, j - 1, k + 1] - V[i, j - 1, k]) / dz
        phix = 0.25 * (PH[i + 1, j, k + 1] - PH[i - 1, j, k + 1] + PH[i + 1, j, k] - PH[i - 1, j, k]) / dx
        phiy = 0.25 * (PH[i, j + 1, k + 1] - PH[i, j - 1, k + 1] + PH[i, j + 1, k] - PH[i, j - 1, k]) / dy
        phiz = (PH[i, j, k + 1] - PH[i, j, k]) / dz
        dif_x = (1.0 - mu_12) * delta_ * phix * (uz + wx) / (rho_ * re)
        dif_y = (1.0 - mu_12) * delta_ * phiy * (vz + wy) / (rho_ * re)
        dif_z = (1.0 - mu_12) * delta_ * phiz * 2.0 * wz / (rho_ * re)
        TZ[i, j, k] = TZ[i, j, k] + dif_x + dif_y + dif_z
    for i, j, k in rng:
        for (T, N, o, gg) in ((TX, NX, (1, 0, 0), gx), (TY, NY, (0, 1, 0), gy),
                              (TZ, NZ, (0, 0, 1), gz)):
            a, b, c = i + o[0], j + o[1], k + o[2]
            rho_ = 0.5 * (RO[i, j, k] + RO[a, b, c])
            delta_ = 0.5 * (DE[i, j, k] + DE[a, b, c])
            curv_ = (CU[i, j, k] + CU[a, b, c]) / 2.0
            phin = 0.5 * (N[i, j, k] + N[a, b, c])
            T[i, j, k] = T[i, j, k] + gg * btn_g / fr - btn_sf * curv_ * delta_ * phin / (we * rho_)
    return tx, ty, tz


def find_stag_vel(us, vs, ws, g, nx, ny, nz):
    """The interior averages of find_stag_vel: returns (V, W, U, WW, UU, VV) =
    (y%s1, z%s1, x%s1, z%s2, x%s2, y%s2) as dicts keyed by (i, j[, k])."""
    three = us.ndim == 3
    Us, Vs = R(us, g), R(vs, g)
    out = [dict() for _ in range(6)]
    if not three:
        for j in range(1, ny + 1):
            for i in range(1, nx + 1):
                out[0][i, j] = 0.25 * (Vs[i, j] + Vs[i, j - 1] + Vs[i + 1, j] + Vs[i + 1, j - 1])
                out[2][i, j] = 0.25 * (Us[i, j] + Us[i - 1, j] + Us[i, j + 1] + Us[i - 1, j + 1])
        return out
    Ws = R(ws, g)
    for k in range(1, nz + 1):
        for j in range(1, ny + 1):
            for i in range(1, nx + 1):
                out[0][i, j, k] = 0.25 * (Vs[i, j, k] + Vs[i, j - 1, k] + Vs[i + 1, j, k] + Vs[i + 1, j - 1, k])
                out[1][i, j, k] = 0.25 * (Ws[i, j, k] + Ws[i, j, k - 1] + Ws[i + 1, j, k] + Ws[i + 1, j, k - 1])
                out[2][i, j, k] = 0.25 * (Us[i, j, k] + Us[i - 1, j, k] + Us[i, j + 1, k] + Us[i - 1, j + 1, k])
                out[3][i, j, k] = 0.25 * (Ws[i, j, k] + Ws[i, j, k - 1] + Ws[i, j + 1, k] + Ws[i, j + 1, k - 1])
                out[4][i, j, k] = 0.25 * (Us[i, j, k] + Us[i - 1, j, k] + Us[i, j, k + 1] + Us[i - 1, j, k + 1])
                out[5][i, j, k] = 0.25 * (Vs[i, j, k] + Vs[i, j - 1, k] + Vs[i, j, k + 1] + Vs[i, j - 1, k + 1])
    return out


def ns_ab_adv_predictor(old, tmp, diff, src_old, g, n, h, dt):
    """ns_linearize's find_stag_vel, ns_ab_adv_source_sec, ns_ab_setup and
    ns_ab_predictor (without velbc).  old/tmp/diff/src_old: tuples of padded
    arrays (u, v[, w]); n = (nx, ny[, nz]); h = (dx, dy[, dz]).  Returns
    (velsrc%now, vel%now) tuples; vel%now starts as a copy of vel%old."""
    three = len(old) == 3
    nx, ny = n[0], n[1]
    nz = n[2] if three else 1
    st = find_stag_vel(tmp[0], tmp[1], tmp[2] if three else None, g, nx, ny, nz)
    src = [np.zeros_like(a) for a in old]
    vel = [a.copy() for a in old]
    O = [R(a, g) for a in old]
    T = [R(a, g) for a in tmp]
    S = [R(a, g) for a in src]
    D = [R(a, g) for a in diff]
    SO = [R(a, g) for a in src_old]
    VN = [R(a, g) for a in vel]

    def d1(F, ix, ax, hh):
        e = [0, 0, 0][:len(ix)]
        e[ax] = 1
        p1 = tuple(a + b for a, b in zip(ix, e))
        p2 = tuple(a + 2 * b for a, b in zip(ix, e))
        m1 = tuple(a - b for a, b in zip(ix, e))
        m2 = tuple(a - 2 * b for a, b in zip(ix, e))
        p = 0.5 * (-F[p2] + 4.0 * F[p1] - 3.0 * F[ix]) / hh
        m = 0.5 * (F[m2] - 4.0 * F[m1] + 3.0 * F[ix]) / hh
        return p, m

    pts = ([(i, j, k) for k in range(1, nz + 1) for j in range(1, ny + 1) for i in range(1, nx + 1)]
           if three else [(i, j) for j in range(1, ny + 1) for i in range(1, nx + 1)])
    for ix in pts:
        if three:
            adv = [(T[0][ix], st[0][ix], st[1][ix]), (st[2][ix], T[1][ix], st[3][ix]),
                   (st[4][ix], st[5][ix], T[2][ix])]
        else:
            adv = [(T[0][ix], st[0][ix]), (st[2][ix], T[1][ix])]
        for c in range(len(old)):
            a = adv[c]
            xp, xm = d1(O[c], ix, 0, h[0])
            yp, ym = d1(O[c], ix, 1, h[1])
            u, v = a[0], a[1]
            s = - ((u + abs(u)) * xm + (u - abs(u)) * xp) / 2.0 \
                - ((v + abs(v)) * ym + (v - abs(v)) * yp) / 2.0
            if three:
                zp, zm = d1(O[c], ix, 2, h[2])
                w = a[2]
                s = s - ((w + abs(w)) * zm + (w - abs(w)) * zp) / 2.0
            S[c][ix] = s
            S[c][ix] = S[c][ix] + D[c][ix]
            srcv = 1.50 * S[c][ix] - 0.5 * SO[c][ix]
            VN[c][ix] = O[c][ix] + dt * srcv
    return tuple(src), tuple(vel)


def velbc(u, v, w, g, nx, ny, nz, ubc, vbc, wbc=(0, 0)):
    """velbc in place (2D when w is None)."""
    three = w is not None
    U, V = R(u, g), R(v, g)
    W = R(w, g) if three else None
    ks = list(range(1 - g, nz + g + 1)) if three else [None]

    def at(F, i, j, k):
        return (i, j, k) if three else (i, j)

    comps = [(U, 0), (V, 1)] + ([(W, 2)] if three else [])
    for side, t in ((0, ubc[0]), (1, ubc[1])):
        if t not in (1, 2):
            continue
        for k in ks:
            for j in range(1 - g, ny + g + 1):
                for m in range(1, g + 1):
                    for F, c in comps:
                        if side == 0:
                            s_ = (1 - 2 + m) if c == 0 else (1 - 1 + m)
                            F[at(F, 1 - m, j, k)] = F[at(F, s_, j, k)] if t == 2 else -F[at(F, s_, j, k)]
                        else:
                            s_ = (nx - m) if c == 0 else (nx + 1 - m)
                            F[at(F, nx + m, j, k)] = F[at(F, s_, j, k)] if t == 2 else -F[at(F, s_, j, k)]
                U[at(U, 0 if side == 0 else nx, j, k)] = 0.0
    for side, t in ((0, vbc[0]), (1, vbc[1])):
        if t not in (1, 2):
            continue
        for k in ks:
            for i in range(1 - g, nx + g + 1):
                for m in range(1, g + 1):
                    for F, c in comps:
                        if side == 0:
                            s_ = (1 - 2 + m) if c == 1 else (1 - 1 + m)
                            F[at(F, i, 1 - m, k)] = F[at(F, i, s_, k)] if t == 2 else -F[at(F, i, s_, k)]
                        else:
                            s_ = (ny - m) if c == 1 else (ny + 1 - m)
                            F[at(F, i, ny + m, k)] = F[at(F, i, s_, k)] if t == 2 else -F[at(F, i, s_, k)]
                V[at(V, i, 0 if side == 0 else ny, k)] = 0.0
    if not three:
        return
    for side, t in ((0, wbc[0]), (1, wbc[1])):
        if t not in (1, 2):
            continue
        for j in range(1 - g, ny + g + 1):
            for i in range(1 - g, nx + g + 1):
                for m in range(1, g + 1):
                    for F, c in comps:
                        if side == 0:
                            s_ = (1 - 2 + m) if c == 2 else (1 - 1 + m)
                            F[i, j, 1 - m] = F[i, j, s_] if t == 2 else -F[i, j, s_]
                        else:
                            s_ = (nz - m) if c == 2 else (nz + 1 - m)
                            F[i, j, nz + m] = F[i, j, s_] if t == 2 else -F[i, j, s_]
                W[i, j, 0 if side == 0 else nz] = 0.0


# ---------------------------------------------------------------------------
# Compact-difference normals and curvature, literally:
#   working_matrix_bc / init_ccd / asgn_src_ccd / root_solve("ccd")
#       "Two phase flows/newOpenMP/2D/lib/solver/ccd_solvers.f90:76-159,287-306,379-399"
#   TWIN_DEC, TWIN_BKS  ".../2D/lib/solver/matrix_solver.f90:6-78"
#   surface_norms, curv ".../2D/src/interface_solver/others_normals.f90:1-103"
#                       (3D ".../3D+IBM/src/interface_solver/others_normals.f90")
#   bc                  ".../2D/src/others/bcs.f90:1-26"
# Matrices are dicts keyed (row, i) with i the Fortran index is..ie.
# ---------------------------------------------------------------------------
def _twin_dec(A, B, AA, BB, IS, IE):
    A[1, IS] = 0.0; AA[1, IS] = 0.0; A[3, IE] = 0.0; AA[3, IE] = 0.0
    B[1, IS] = 0.0; BB[1, IS] = 0.0; B[3, IE] = 0.0; BB[3, IE] = 0.0
    for i in range(IS + 1, IE + 1):
        Den = A[2, i - 1] * BB[2, i - 1] - AA[2, i - 1] * B[2, i - 1]
        SC1 = -(AA[2, i - 1] * B[1, i] - A[1, i] * BB[2, i - 1]) / Den
        SC2 = (B[1, i] * A[2, i - 1] - B[2, i - 1] * A[1, i]) / Den
        A[1, i] = SC1
        A[2, i] = A[2, i] - (SC1 * A[3, i - 1] + SC2 * AA[3, i - 1])
        B[1, i] = SC2
        B[2, i] = B[2, i] - (SC1 * B[3, i - 1] + SC2 * BB[3, i - 1])
        SC1 = -(AA[2, i - 1] * BB[1, i] - AA[1, i] * BB[2, i - 1]) / Den
        SC2 = (BB[1, i] * A[2, i - 1] - B[2, i - 1] * AA[1, i]) / Den
        AA[1, i] = SC1
        AA[2, i] = AA[2, i] - (SC1 * A[3, i - 1] + SC2 * AA[3, i - 1])
        BB[1, i] = SC2
        BB[2, i] = BB[2, i] - (SC1 * B[3, i - 1] + SC2 * BB[3, i - 1])


def _twin_bks(A, B, AA, BB, S, SS, IS, IE):
    for i in range(IS + 1, IE + 1):
        S[i] = S[i] - (A[1, i] * S[i - 1] + B[1, i] * SS[i - 1])
        SS[i] = SS[i] - (AA[1, i] * S[i - 1] + BB[1, i] * SS[i - 1])
    Den = A[2, IE] * BB[2, IE] - AA[2, IE] * B[2, IE]
    SolS = -(B[2, IE] * SS[IE] - BB[2, IE] * S[IE]) / Den
    SolSS = (A[2, IE] * SS[IE] - AA[2, IE] * S[IE]) / Den
    S[IE] = SolS
    SS[IE] = SolSS
    for i in range(IE - 1, IS - 1, -1):
        S[i] = S[i] - (A[3, i] * SolS + B[3, i] * SolSS)
        SS[i] = SS[i] - (AA[3, i] * SolS + BB[3, i] * SolSS)
        Den = A[2, i] * BB[2, i] - AA[2, i] * B[2, i]
        SolS = -(B[2, i] * SS[i] - BB[2, i] * S[i]) / Den
        SolSS = (A[2, i] * SS[i] - AA[2, i] * S[i]) / Den
        S[i] = SolS
        SS[i] = SolSS


def ccd_solve(f, dx):
    """root_solve("ccd"): f a list over is..ie (here 0..L-1); returns (fx, fxx)."""
    IS, IE = 0, len(f) - 1
    A, B, AA, BB = {}, {}, {}, {}
    # working_matrix_bc
    A[2, IS] = 1.0; B[2, IS] = 0.0; AA[2, IS] = 0.0; BB[2, IS] = 1.0
    A[3, IS] = 2.0; B[3, IS] = - dx; AA[3, IS] = -2.5 / dx; BB[3, IS] = 8.5
    A[2, IE] = 1.0; B[2, IE] = 0.0; AA[2, IE] = 0.0; BB[2, IE] = 1.0
    A[1, IE] = 2.0; B[1, IE] = dx; AA[1, IE] = 2.5 / dx; BB[1, IE] = 8.5
    # working_matrix_init_ccd
    for i in range(IS + 1, IE):
        A[1, i] = 7.0 / 16.0; A[2, i] = 1.0; A[3, i] = 7.0 / 16.0
        B[1, i] = dx / 16.0; B[2, i] = 0.0; B[3, i] = - dx / 16.0
        AA[1, i] = - 9.0 / 8.0 / dx; AA[2, i] = 0.0; AA[3, i] = 9.0 / 8.0 / dx
        BB[1, i] = - 1.0 / 8.0; BB[2, i] = 1.0; BB[3, i] = - 1.0 / 8.0
    _twin_dec(A, B, AA, BB, IS, IE)
    S, SS = {}, {}
    S[IS] = (-3.5 * f[IS] + 4.0 * f[IS + 1] - 0.5 * f[IS + 2]) / dx
    SS[IS] = (34.0 / 3.0 * f[IS] - 83.0 / 4.0 * f[IS + 1] + 10.0 * f[IS + 2]
              - 7.0 / 12.0 * f[IS + 3]) / _sq(dx)
    for i in range(IS + 1, IE):
        S[i] = 15.0 / 16.0 * (-f[i - 1] + f[i + 1]) / dx
        SS[i] = (3.0 * f[i - 1] - 6.0 * f[i] + 3.0 * f[i + 1]) / _sq(dx)
    S[IE] = -(-3.5 * f[IE] + 4.0 * f[IE - 1] - 0.5 * f[IE - 2]) / dx
    SS[IE] = (34.0 / 3.0 * f[IE] - 83.0 / 4.0 * f[IE - 1] + 10.0 * f[IE - 2]
              - 7.0 / 12.0 * f[IE - 3]) / _sq(dx)
    _twin_bks(A, B, AA, BB, S, SS, IS, IE)
    return [S[i] for i in range(IS, IE + 1)], [SS[i] for i in range(IS, IE + 1)]


def _ccd_lines(a, axis, h):
    """CCD along numpy axis `axis` (0 = slowest) of every line of a padded array."""
    fx, fxx = np.empty_like(a), np.empty_like(a)
    moved = np.moveaxis(a, axis, -1)
    ox, oxx = np.moveaxis(fx, axis, -1), np.moveaxis(fxx, axis, -1)
    for idx in np.ndindex(moved.shape[:-1]):
        d1, d2 = ccd_solve([float(x) for x in moved[idx]], h)
        ox[idx] = d1
        oxx[idx] = d2
    return fx, fxx


def _bc_copy(a):
    """bc: zero-gradient copies from the boundary interior, x then y (then z)."""
    g = _bc_copy.g
    for ax in range(a.ndim - 1, -1, -1):
        m = np.moveaxis(a, ax, -1)
        n = m.shape[-1] - 2 * g
        for k in range(1, g + 1):
            m[..., g - k] = m[..., g]
            m[..., g + n - 1 + k] = m[..., g + n - 1]


def curv(phi, g, dx, dy, dz=None):
    """surface_norms + curv on a padded phi (2D (ny+2g, nx+2g) or 3D).  Returns
    (fx, fy, fz or None, curv) after bc."""
    _bc_copy.g = g
    three = phi.ndim == 3
    ax = {"x": phi.ndim - 1, "y": phi.ndim - 2, "z": 0}
    fx, fxx = _ccd_lines(phi, ax["x"], dx)
    fy, fyy = _ccd_lines(phi, ax["y"], dy)
    fxy, _ = _ccd_lines(fx, ax["y"], dy)
    if three:
        fz, fzz = _ccd_lines(phi, ax["z"], dz)
        fxz, _ = _ccd_lines(fx, ax["z"], dz)
        fyz, _ = _ccd_lines(fy, ax["z"], dz)
        arrs = (fx, fxx, fy, fyy, fz, fzz, fxy, fxz, fyz)
    else:
        fz = None
        arrs = (fx, fxx, fy, fyy, fxy)
    for a in arrs:
        _bc_copy(a)
    cv = np.zeros_like(phi)
    inner = tuple(slice(g, s - g) for s in phi.shape)
    it = np.ndindex(*[s - 2 * g for s in phi.shape])
    for rel in it:
        q = tuple(r + g for r in rel)
        Fx, Fy = float(fx[q]), float(fy[q])
        if not three:
            cv[q] = (float(fyy[q]) * _sq(Fx) + float(fxx[q]) * _sq(Fy)
                     - 2.0 * float(fxy[q]) * Fx * Fy) / (_sq(Fx) + _sq(Fy) + 1.0e-12) ** 1.5
        else:
            Fz = float(fz[q])
            cv[q] = ((float(fyy[q]) + float(fzz[q])) * _sq(Fx) + (float(fxx[q]) + float(fzz[q])) * _sq(Fy)
                     + (float(fxx[q]) + float(fyy[q])) * _sq(Fz)
                     - 2.0 * (float(fxy[q]) * Fx * Fy + float(fxz[q]) * Fx * Fz + float(fyz[q]) * Fy * Fz)) \
                / (_sq(Fx) + _sq(Fy) + _sq(Fz) + 1.0e-12) ** 1.5
    del inner
    _bc_copy(cv)
    return fx, fy, fz, cv


def ns_ab_adv_source_quick_2d(uo, vo, ut, vt, g, nx, ny, dx, dy):
    """ns_ab_adv_source_quick, 2D ("Two phase flows/newOpenMP/2D/src/ns_solver/
    ns_ab_adv.f90:44-114"), literally: returns velsrc%now (x, y)."""
    U, V, UT, VT = R(uo, g), R(vo, g), R(ut, g), R(vt, g)
    xs1, xs2, ys1, ys2 = {}, {}, {}, {}
    for j in range(0, ny + 1):
        for i in range(0, nx + 1):
            uh = 0.5 * (UT[i, j] + UT[i + 1, j])
            vh = 0.5 * (VT[i, j] + VT[i + 1, j])
            if uh >= 0.0:
                xs1[i, j] = (-U[i - 1, j] + 6.0 * U[i, j] + 3.0 * U[i + 1, j]) / 8.0
            else:
                xs1[i, j] = (-U[i + 2, j] + 6.0 * U[i + 1, j] + 3.0 * U[i, j]) / 8.0
            if vh >= 0.0:
                xs2[i, j] = (-U[i, j - 1] + 6.0 * U[i, j] + 3.0 * U[i, j + 1]) / 8.0
            else:
                xs2[i, j] = (-U[i, j + 2] + 6.0 * U[i, j + 1] + 3.0 * U[i, j]) / 8.0
            uh = 0.5 * (UT[i, j] + UT[i, j + 1])
            vh = 0.5 * (VT[i, j] + VT[i, j + 1])
            if uh >= 0.0:
                ys1[i, j] = (-V[i - 1, j] + 6.0 * V[i, j] + 3.0 * V[i + 1, j]) / 8.0
            else:
                ys1[i, j] = (-V[i + 2, j] + 6.0 * V[i + 1, j] + 3.0 * V[i, j]) / 8.0
            if vh >= 0.0:
                ys2[i, j] = (-V[i, j - 1] + 6.0 * V[i, j] + 3.0 * V[i, j + 1]) / 8.0
            else:
                ys2[i, j] = (-V[i, j + 2] + 6.0 * V[i, j + 1] + 3.0 * V[i, j]) / 8.0
    sx, sy = np.zeros_like(uo), np.zeros_like(vo)
    SX, SY = R(sx, g), R(sy, g)
    for j in range(1, ny + 1):
        for i in range(1, nx + 1):
            uh = 0.5 * (UT[i, j] + UT[i + 1, j])
            vh = 0.5 * (VT[i, j] + VT[i + 1, j])
            SX[i, j] = - uh * (xs1[i, j] - xs1[i - 1, j]) / dx - vh * (xs2[i, j] - xs2[i, j - 1]) / dy
            uh = 0.5 * (UT[i, j] + UT[i, j + 1])
            vh = 0.5 * (VT[i, j] + VT[i, j + 1])
            SY[i, j] = - uh * (ys1[i, j] - ys1[i - 1, j]) / dx - vh * (ys2[i, j] - ys2[i, j - 1]) / dy
    return sx, sy
