"""Seeded synthetic inputs for the projection step: bubbles -> level set phi,
and MAC face velocities u* ~ N(0, 1).

The reference benchmarks no public dataset; these stand in for the rising-bubble
set-ups of the two-phase solvers (a signed-distance level set, negative inside
the bubble, "Two phase flows/newOpenMP/2D/src/interface_solver/others.f90" for
the density chain).  Arrays are float64, C order (z, y, x) == the reference's
Fortran (i, j, k) order without ghosts.  Face velocities: u (nz, ny, nx+1),
v (nz, ny+1, nx), w (nz+1, ny, nx); wall-normal faces are 0 (as velbc / RHSP
leave them).  All randomness comes from numpy.random.default_rng(seed).
"""
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Case:
    name: str
    shape: tuple            # (nz, ny, nx); nz == 1 for 2D
    extent: tuple           # physical lengths (Lx, Ly, Lz)
    centers: np.ndarray     # (nb, 3) bubble centres (x, y, z)
    radii: np.ndarray       # (nb,)
    dt: float = 1e-3
    rho_pos: float = 1000.0  # density where phi > 0 (outside the bubbles)
    rho_neg: float = 1.0     # density where phi < 0 (inside)
    eps_cells: float = 1.5   # smoothed-Heaviside half width in cells
    seed: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def spacing(self):
        nz, ny, nx = self.shape
        Lx, Ly, Lz = self.extent
        return (Lx / nx, Ly / ny, Lz / nz)

    @property
    def eps(self):
        return self.eps_cells * self.spacing[0]

    @property
    def dim(self):
        return 2 if self.shape[0] == 1 else 3


def cell_centers(shape, extent):
    nz, ny, nx = shape
    Lx, Ly, Lz = extent
    x = (np.arange(nx) + 0.5) * (Lx / nx)
    y = (np.arange(ny) + 0.5) * (Ly / ny)
    z = (np.arange(nz) + 0.5) * (Lz / nz)
    return x, y, z


def level_set(case: Case) -> np.ndarray:
    """phi = min over bubbles of (distance to centre - radius); negative inside."""
    x, y, z = cell_centers(case.shape, case.extent)
    nz, ny, nx = case.shape
    phi = np.full(case.shape, np.inf)
    two_d = case.dim == 2
    for c, r in zip(case.centers, case.radii):
        d2 = (x[None, None, :] - c[0]) ** 2 + (y[None, :, None] - c[1]) ** 2
        if not two_d:
            d2 = d2 + (z[:, None, None] - c[2]) ** 2
        np.minimum(phi, np.sqrt(d2) - r, out=phi)
    return phi


def velocity(case: Case, seed=None):
    """Face velocities u*, v*, w* ~ N(0,1) on interior faces, 0 on walls."""
    rng = np.random.default_rng(case.seed if seed is None else seed)
    nz, ny, nx = case.shape
    u = rng.standard_normal((nz, ny, nx + 1))
    v = rng.standard_normal((nz, ny + 1, nx))
    if case.dim == 3:
        w = rng.standard_normal((nz + 1, ny, nx))
        w[0] = 0.0
        w[-1] = 0.0
    else:
        w = np.zeros((nz + 1, ny, nx))
    u[..., 0] = 0.0
    u[..., -1] = 0.0
    v[:, 0, :] = 0.0
    v[:, -1, :] = 0.0
    return u, v, w


def _place_bubbles(rng, n, rmin, rmax, extent, dim, wall_gap, gap=0.0, zrange=None,
                   max_tries=100000):
    """Seeded rejection sampling of non-overlapping bubbles, each at least
    `wall_gap` from every wall (surface to wall)."""
    centers, radii = [], []
    tries = 0
    while len(centers) < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("bubble placement failed")
        r = rng.uniform(rmin, rmax) if rmax > rmin else rmin
        c = np.array([rng.uniform(r + wall_gap, L - r - wall_gap) for L in extent])
        if dim == 2:
            c[2] = 0.5 * extent[2]
        if zrange is not None:
            c[2] = rng.uniform(*zrange)
        ok = True
        for c2, r2 in zip(centers, radii):
            d = np.linalg.norm((c - c2)[:dim])
            if d < r + r2 + gap:
                ok = False
                break
        if ok:
            centers.append(c)
            radii.append(r)
    return np.array(centers), np.array(radii)


def config(index: int, scale: int = 1) -> Case:
    """The five synthetic cases of the pressure-solve benchmark, numbered as the
    benchmark configuration list (0: 2D 128^2 one bubble, 1: 3D 256^3 one
    sphere, 2: 3D 512^3 16 spheres, 3: 2D 1024^2 8 circles, 4: 128x128x256
    four spheres).  `scale` > 1 divides every axis by `scale` (a smaller case
    with the same geometry, for tests)."""
    def sh(*n):
        return tuple(max(1, a // scale) if a > 1 else 1 for a in n)

    if index == 0:
        return Case("bubble2d_128", sh(1, 128, 128), (1.0, 1.0, 1.0),
                    np.array([[0.5, 0.5, 0.5]]), np.array([0.25]), seed=0)
    if index == 1:
        return Case("sphere3d_256", sh(256, 256, 256), (1.0, 1.0, 1.0),
                    np.array([[0.5, 0.5, 0.3]]), np.array([0.2]), seed=1)
    if index == 2:
        rng = np.random.default_rng(2002)
        c, r = _place_bubbles(rng, 16, 0.03, 0.08, (1.0, 1.0, 1.0), 3, 0.02)
        return Case("spheres16_512", sh(512, 512, 512), (1.0, 1.0, 1.0), c, r, seed=2)
    if index == 3:
        rng = np.random.default_rng(3003)
        c, r = _place_bubbles(rng, 8, 0.03, 0.1, (1.0, 1.0, 1.0), 2, 0.0)
        return Case("circles8_1024", sh(1, 1024, 1024), (1.0, 1.0, 1.0), c, r, seed=3,
                    extra=dict(target_seed=33))
    if index == 4:
        rng = np.random.default_rng(4004)
        c, r = _place_bubbles(rng, 4, 0.1, 0.1, (1.0, 1.0, 2.0), 3, 0.0, zrange=(0.3, 0.7))
        return Case("spheres4_128x128x256", sh(256, 128, 128), (1.0, 1.0, 2.0), c, r,
                    dt=2e-3, seed=4, extra=dict(steps=20, shift=(0.0, 0.0, 0.5)))
    raise ValueError(index)


def custom(shape, extent=(1.0, 1.0, 1.0), centers=((0.5, 0.5, 0.5),), radii=(0.25,),
           seed=0, **kw) -> Case:
    return Case("custom", tuple(shape), tuple(extent), np.asarray(centers, float),
                np.asarray(radii, float), seed=seed, **kw)
