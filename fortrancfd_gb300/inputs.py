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


def padded_shape(shape, ghost):
    """The reference's ghost-padded box of an interior (nz, ny, nx):
    (nz+2g, ny+2g, nx+2g), or (ny+2g, nx+2g) in 2D."""
    nz, ny, nx = shape
    if nz == 1:
        return (ny + 2 * ghost, nx + 2 * ghost)
    return (nz + 2 * ghost, ny + 2 * ghost, nx + 2 * ghost)


def velbc_numpy(u, v, w, ghost, bc):
    """velbc ("Two phase flows/newOpenMP/2D/src/others/bcs.f90:28-132",
    3D "…/3D+IBM/src/others/bcs.f90:44-257") on padded numpy arrays, for
    building consistent synthetic states: ghosts mirror the interior (negated
    for bc 1, no-slip; copied for bc 2, slip), the wall-normal face is 0.
    Passes x, y, z in order over the whole padded extent."""
    g = ghost
    comps = [u, v] + ([w] if w is not None else [])
    ax_of = {0: -1, 1: -2, 2: -3}
    for axis in range(len(comps)):
        ax = ax_of[axis]
        for side in (0, 1):
            t = bc[2 * axis + side]
            if t not in (1, 2):
                continue
            s = -1.0 if t == 1 else 1.0
            for c, f in enumerate(comps):
                n = f.shape[ax] - 2 * g
                a = np.moveaxis(f, ax, -1)
                stag = c == axis
                for m in range(1, g + 1):
                    if side == 0:  # ghost index 1-m <- 1-2+m (staggered) or m
                        src = (m - 1) if stag else m
                        a[..., g - m] = s * a[..., g + src - 1]
                    else:          # ghost n+m <- n-m (staggered) or n+1-m
                        src = (n - m) if stag else (n + 1 - m)
                        a[..., g + n + m - 1] = s * a[..., g + src - 1]
                if stag:
                    a[..., g - 1 if side == 0 else g + n - 1] = 0.0
    return u, v, w


def momentum_state(case: Case, ghost=3, rho_12=1e-3, mu_12=1e-2, amplitude=0.1, seed=None):
    """Seeded synthetic state of one Adams-Bashforth momentum step, every array
    on the reference's ghost-padded box: the old level set phi (signed distance
    to the case's bubbles) and from it heavy/delta (ls_funs with half width
    eps), rho = H + rho_12 (1 - H), mu = H + mu_12 (1 - H), unit normals and
    their divergence (curvature) by central differences; a smooth old
    velocity (a few random Fourier modes, velbc no-slip applied) and a smooth
    old source velsrc%old.  Returns a dict of float64 arrays plus 'rho_now'
    (the interior density of the same phi, for the pressure operator)."""
    rng = np.random.default_rng(case.seed + 17 if seed is None else seed)
    nz, ny, nx = case.shape
    dx, dy, dz = case.spacing
    g = ghost
    three = nz > 1
    ps = padded_shape(case.shape, g)
    xs = (np.arange(nx + 2 * g) - g + 0.5) * dx
    ys = (np.arange(ny + 2 * g) - g + 0.5) * dy
    if three:
        zs = (np.arange(nz + 2 * g) - g + 0.5) * dz
        Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    else:
        Y, X = np.meshgrid(ys, xs, indexing="ij")
        Z = np.full(X.shape, 0.5 * case.extent[2])
    phi = np.full(Z.shape, np.inf)
    for c, r in zip(case.centers, case.radii):
        d2 = (X - c[0]) ** 2 + (Y - c[1]) ** 2
        if three:
            d2 = d2 + (Z - c[2]) ** 2
        np.minimum(phi, np.sqrt(d2) - r, out=phi)
    # negative inside the bubbles: phi > 0 is the heavy fluid 1 of the reference
    eps = case.eps
    x = phi / eps
    heavy = np.where(x > 1 - 1e-12, 1.0, np.where(x < -1 + 1e-12, 0.0,
                                                 0.5 * (1.0 + x + np.sin(np.pi * x) / np.pi)))
    delta = np.where(np.abs(x) < 1 - 1e-12, 0.5 * (1.0 + np.cos(np.pi * x)) / eps, 0.0)
    heavy = np.clip(heavy, 0.0, 1.0)
    rho = heavy + rho_12 * (1.0 - heavy)
    mu = heavy + mu_12 * (1.0 - heavy)
    grads = np.gradient(phi, *((dz, dy, dx) if three else (dy, dx)))
    mag = np.sqrt(sum(gr * gr for gr in grads)) + 1e-12
    nrm = [gr / mag for gr in grads]  # (z, y, x) or (y, x) order
    curv = sum(np.gradient(nrm[a], (dz, dy, dx)[a] if three else (dy, dx)[a], axis=a)
               for a in range(len(nrm)))
    nrm_x, nrm_y = nrm[-1], nrm[-2]
    nrm_z = nrm[0] if three else None

    def smooth():
        f = np.zeros(Z.shape)
        for _ in range(4):
            kx, ky, kz = rng.integers(1, 4, size=3)
            ph = rng.uniform(0, 2 * np.pi, size=3)
            f += rng.standard_normal() * (np.sin(kx * np.pi * X + ph[0])
                                          * np.sin(ky * np.pi * Y + ph[1])
                                          * (np.sin(kz * np.pi * Z + ph[2]) if three else 1.0))
        return amplitude * f

    u, v = smooth(), smooth()
    w = smooth() if three else None
    bc = (1, 1, 1, 1, 1, 1)
    velbc_numpy(u, v, w, g, bc)
    su, sv = smooth(), smooth()
    sw = smooth() if three else None
    sl = (slice(g, g + nz),) if three else ()
    rho_now = rho[sl + (slice(g, g + ny), slice(g, g + nx))].reshape(case.shape).copy()
    out = dict(u=u, v=v, w=w, su_old=su, sv_old=sv, sw_old=sw, rho=rho, mu=mu, delta=delta,
               phi=phi, nrm_x=nrm_x, nrm_y=nrm_y, nrm_z=nrm_z, curv=curv, rho_now=rho_now,
               p=np.zeros(case.shape))
    for k, a in out.items():
        if a is not None:
            out[k] = np.ascontiguousarray(a, np.float64)
            assert k in ("rho_now", "p") or out[k].shape == ps, (k, out[k].shape, ps)
    return out
