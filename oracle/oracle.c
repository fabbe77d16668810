/*
 * oracle.c -- CPU restatement (FP64, C11 + OpenMP) of the pressure-Poisson
 * path of ntu-d09525007/FortranCFD.  TEST INFRASTRUCTURE ONLY: the product
 * (fortrancfd_gb300/) never links, loads or calls this file; it is used by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, as
 * the checker and the timed CPU reference.
 *
 * PARITY UNPINNED: the reference ships no tests, golden vectors or fixtures
 * for this path, and it cannot be built here (Fortran + Intel MKL only).  The
 * restatement is pinned instead by known-answer properties (manufactured
 * solutions, operator symmetry and null space, convergence of the multigrid to
 * the fully converged point-relaxation fixed point) in tests/.
 *
 * Every function cites the reference loop it follows.  Paths are relative to
 * the reference project:
 *   NO2 = "Two phase flows/newOpenMP/2D", NO3 = "Two phase flows/newOpenMP/3D+IBM"
 *   MP3 = "MPLS_RisingBubble/20190612",  DD3 = "DomainDecomposition/3D"
 *
 * Layout (shared with the CUDA path): every cell array is dense, C order
 * (z, y, x) with x fastest, which is the Fortran column-major (i, j, k) order
 * of the reference without its ghost cells.  Face coefficients are stored in
 * cell-shaped "low face" arrays: cx[k][j][i] couples cell (i-1,j,k) and
 * (i,j,k); cx[..][..][0] is the x=0 wall and is 0.  The high wall of the last
 * cell has no entry and is implicitly 0.  Zero wall coefficients are the
 * Neumann folding of ppe_sor_init (NO3/src/ns_solver/ns_ppe_solver.f90:30-58):
 * the wall term moves into the diagonal and vanishes from the sum, which is
 * the same as a zero-gradient ghost (NO2/src/others/bcs.f90:1-26).
 *
 * Build: gcc -O3 -fopenmp -ffp-contract=off -fPIC -shared (see oracle/build.py);
 * -ffp-contract=off keeps results bit-identical on x86_64 and aarch64.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  int32_t nx, ny, nz;
  double dx, dy, dz;
} or_grid;

/* Multigrid parameters.  Defaults in or_mg_default(). */
typedef struct {
  int32_t nu1, nu2;          /* pre/post sweeps per level: DD3 multigrid_solver.f90:57,158 use 2,2 */
  int32_t levels;            /* 0 = auto (coarsen until <= coarse_max cells) */
  int32_t coarse_max;        /* auto mode: stop coarsening at or below this many cells */
  int32_t max_cycles;        /* DD3 ns_ppe_mg_solver.f90:17 uses 100 */
  int32_t smoother;          /* 0 = red-black GS, 1 = lexicographic GS in blocks (DD3 relax) */
  int32_t blocks[3];         /* lexicographic mode: subdomain grid (DD3 input/default.txt:5-6) */
  int32_t mean_every_sweep;  /* 1 = compatibility_sol after every sweep (DD3 :43) */
  int32_t coarse_op;         /* 0 = arithmetic face average, 1 = series-harmonic along the normal */
  int32_t record_history;    /* fill stats->history with the per-cycle relative residual */
  int32_t krylov;            /* 0 = stationary V-cycles (the reference's loop), 1 = flexible PCG
                                with one V-cycle as the preconditioner */
  int32_t prolong;           /* 0 = central-slope linear (DD3 :106-160), 1 = piecewise constant */
  double coarse_scale;       /* multiplies the coarse correction before it is added */
} or_mg_params;

typedef struct {
  int32_t cycles;
  int32_t levels;
  int32_t status;            /* 0 ok, 1 not converged, 2 diverged, 3 bad argument */
  int32_t coarse_n;
  double rel_residual;       /* ||b - A p||_2 / ||b||_2 */
  double rms_residual;       /* sqrt(sum r^2 / n), the reference's l2norm (DD3 :204) */
  double history[256];
} or_mg_stats;

#define OR_OK 0
#define OR_NOT_CONVERGED 1
#define OR_DIVERGED 2
#define OR_BAD_ARG 3

static inline size_t cells_of(int nx, int ny, int nz) { return (size_t)nx * ny * nz; }

/* ------------------------------------------------------------------------- */
/* a1: smoothed Heaviside and density.                                        */
/* ls_funs / rho_mu, NO2/src/interface_solver/others.f90:1-37,39-61:          */
/*   x = phi/eps; H = 1 if x > 1-1e-12, 0 if x < -1+1e-12,                    */
/*   else 0.5(1 + x + sin(pi x)/pi); H clipped to [0,1];                      */
/*   rho = H + rho_12 (1 - H)  (heavy fluid where phi > 0).                   */
/* Generalised here to rho = rho_pos H + rho_neg (1 - H); the reference is     */
/* rho_pos = 1, rho_neg = rho_12.                                             */
/* ------------------------------------------------------------------------- */
void or_heaviside(const double* phi, int64_t n, double eps, double* H) {
  const double pi = acos(-1.0);
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < n; ++q) {
    double x = phi[q] / eps, h;
    if (x > 1.0 - 1e-12) h = 1.0;
    else if (x < -1.0 + 1e-12) h = 0.0;
    else h = 0.5 * (1.0 + x + sin(pi * x) / pi);
    H[q] = fmax(fmin(h, 1.0), 0.0);
  }
}

/* Derivative of the smoothed Heaviside (others.f90:24: hp = (1+cos(pi x))/(2 eps)). */
void or_heaviside_deriv(const double* phi, int64_t n, double eps, double* dH) {
  const double pi = acos(-1.0);
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < n; ++q) {
    double x = phi[q] / eps;
    dH[q] = (x > 1.0 - 1e-12 || x < -1.0 + 1e-12) ? 0.0 : 0.5 * (1.0 + cos(pi * x)) / eps;
  }
}

void or_rho_from_phi(const double* phi, int64_t n, double eps, double rho_pos, double rho_neg,
                     double* rho) {
  or_heaviside(phi, n, eps, rho);
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < n; ++q) rho[q] = rho_pos * rho[q] + rho_neg * (1.0 - rho[q]);
}

/* ------------------------------------------------------------------------- */
/* a2: face coefficients, ppe_sor_init (NO3/src/ns_solver/ns_ppe_solver.f90:1-65; */
/* 2D NO2 :1-48): coe_f = 2/(rho_i + rho_nb)/h^2, walls folded to 0.           */
/* ------------------------------------------------------------------------- */
void or_face_coef(const or_grid* g, const double* rho, double* cx, double* cy, double* cz) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const double dx2 = g->dx * g->dx, dy2 = g->dy * g->dy, dz2 = g->dz * g->dz;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        size_t q = ((size_t)k * ny + j) * nx + i;
        cx[q] = (i > 0) ? 2.0 / (rho[q] + rho[q - 1]) / dx2 : 0.0;
        cy[q] = (j > 0) ? 2.0 / (rho[q] + rho[q - nx]) / dy2 : 0.0;
        cz[q] = (k > 0) ? 2.0 / (rho[q] + rho[q - (size_t)nx * ny]) / dz2 : 0.0;
      }
}

/* ------------------------------------------------------------------------- */
/* a3: RHS b = div(u*)/dt (NO3 ns_ppe_solver.f90:77-89; NO2 :60-69).          */
/* Face velocities: u has shape (nz, ny, nx+1), u[.][.][f] on the x-face at    */
/* x = f dx (reference u(f) with cells 1-based); v (nz, ny+1, nx); w (nz+1,    */
/* ny, nx).  remove_mean subtracts the mean of b (the synthetic configs ask    */
/* for a mean-free b; the reference relies on zero wall fluxes instead).       */
/* ------------------------------------------------------------------------- */
void or_divergence(const or_grid* g, const double* u, const double* v, const double* w, double dt,
                   int remove_mean, double* b) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        size_t q = ((size_t)k * ny + j) * nx + i;
        size_t qu = ((size_t)k * ny + j) * (nx + 1) + i;
        size_t qv = ((size_t)k * (ny + 1) + j) * nx + i;
        size_t qw = ((size_t)k * ny + j) * nx + i;
        double d = (u[qu + 1] - u[qu]) / g->dx + (v[qv + nx] - v[qv]) / g->dy;
        if (nz > 1 || w) d += (w[qw + (size_t)nx * ny] - w[qw]) / g->dz;
        b[q] = d / dt;
        s += b[q];
      }
  if (remove_mean) {
    size_t n = cells_of(nx, ny, nz);
    s /= (double)n;
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < n; ++q) b[q] -= s;
  }
}

/* ------------------------------------------------------------------------- */
/* Operator: (A p)_i = sum_f coe_f (p_nb - p_i), the sign convention of every  */
/* reference PPE (NO3 ns_ppe_solver.f90:104-111 solves p_i = (src - sum coe    */
/* p_nb)/c with c = -sum coe).                                                */
/* ------------------------------------------------------------------------- */
static inline double stencil_sum(int nx, int ny, int nz, const double* cx, const double* cy,
                                 const double* cz, const double* p, int i, int j, int k,
                                 double* diag) {
  size_t q = ((size_t)k * ny + j) * nx + i;
  size_t sy = nx, sz = (size_t)nx * ny;
  double s = 0.0, d = 0.0, c;
  if (i > 0) { c = cx[q]; s += c * p[q - 1]; d += c; }
  if (i < nx - 1) { c = cx[q + 1]; s += c * p[q + 1]; d += c; }
  if (j > 0) { c = cy[q]; s += c * p[q - sy]; d += c; }
  if (j < ny - 1) { c = cy[q + sy]; s += c * p[q + sy]; d += c; }
  if (k > 0) { c = cz[q]; s += c * p[q - sz]; d += c; }
  if (k < nz - 1) { c = cz[q + sz]; s += c * p[q + sz]; d += c; }
  *diag = d;
  return s;
}

void or_apply(const or_grid* g, const double* cx, const double* cy, const double* cz,
              const double* p, double* Ap) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        double d, s = stencil_sum(nx, ny, nz, cx, cy, cz, p, i, j, k, &d);
        size_t q = ((size_t)k * ny + j) * nx + i;
        Ap[q] = s - d * p[q];
      }
}

/* r = b - A p; returns sum r^2 (multigrid_residual, DD3 multigrid_solver.f90:162-222).
 * The flux form b - sum_f coe_f (p_nb - p_i) (differences first) keeps the
 * rounding relative to each flux, so tight tolerances stay reachable. */
double or_residual(const or_grid* g, const double* cx, const double* cy, const double* cz,
                   const double* p, const double* b, double* r) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const size_t sy = nx, sz = (size_t)nx * ny;
  double s2 = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s2)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        size_t q = ((size_t)k * ny + j) * nx + i;
        const double pc = p[q];
        double s = 0.0;
        if (i > 0) s += cx[q] * (p[q - 1] - pc);
        if (i < nx - 1) s += cx[q + 1] * (p[q + 1] - pc);
        if (j > 0) s += cy[q] * (p[q - sy] - pc);
        if (j < ny - 1) s += cy[q + sy] * (p[q + sy] - pc);
        if (k > 0) s += cz[q] * (p[q - sz] - pc);
        if (k < nz - 1) s += cz[q + sz] * (p[q + sz] - pc);
        double rr = b[q] - s;
        if (r) r[q] = rr;
        s2 += rr * rr;
      }
  return s2;
}

static double sum_of(const double* a, size_t n) {
  double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s)
  for (size_t q = 0; q < n; ++q) s += a[q];
  return s;
}

/* compatibility_sol / compatibility_src (DD3 multigrid_solver.f90:224-308): a -= mean(a). */
void or_remove_mean(double* a, int64_t n) {
  double m = sum_of(a, (size_t)n) / (double)n;
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < n; ++q) a[q] -= m;
}

/* ------------------------------------------------------------------------- */
/* a12: projection, ns_momentum_correction (NO3 ns_ppe_solver.f90:174-205):   */
/* u_f -= dt (p_nb - p_i)/h / rho_f with rho_f = (rho_i + rho_nb)/2.  Wall     */
/* faces are left untouched (velbc keeps them 0).  Face layout as in           */
/* or_divergence.                                                             */
/* ------------------------------------------------------------------------- */
void or_correct(const or_grid* g, const double* rho, const double* p, double dt, double* u,
                double* v, double* w) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        size_t q = ((size_t)k * ny + j) * nx + i;
        if (i > 0) {
          double rf = (rho[q] + rho[q - 1]) / 2.0;
          double px = (p[q] - p[q - 1]) / g->dx;
          u[((size_t)k * ny + j) * (nx + 1) + i] -= dt * px / rf;
        }
        if (j > 0) {
          double rf = (rho[q] + rho[q - nx]) / 2.0;
          double py = (p[q] - p[q - nx]) / g->dy;
          v[((size_t)k * (ny + 1) + j) * nx + i] -= dt * py / rf;
        }
        if (k > 0 && w) {
          size_t sz = (size_t)nx * ny;
          double rf = (rho[q] + rho[q - sz]) / 2.0;
          double pz = (p[q] - p[q - sz]) / g->dz;
          w[q] -= dt * pz / rf;
        }
      }
}

/* ------------------------------------------------------------------------- */
/* Pressure-split projection of the DomainDecomposition solver                */
/* (DomainDecomposition/3D/src/ns_solver/ns_ppe_mg_solver.f90): the constant- */
/* coefficient Laplacian is solved for p with the split source               */
/*   src = rho_12 div(u*)/dt + c p^_i + sum_f coe_f p^_nb                      */
/* (ppe_mg_solver_init :62-136, ppe_mg_solver_src :138-221): coe_f =          */
/* (1 - 2 rho_12/(rho_i + rho_nb))/h^2 on all six faces, c = -(r+l+f+b+u+d),  */
/* with the zero-gradient ghosts of job_bc (DomainDecomposition/3D/lib/data/  */
/* branches.f90:243-288) for rho and p^ at the walls; the terms are added in  */
/* the reference's order.  nz == 1 drops the z terms (the 2D form).           */
/* ------------------------------------------------------------------------- */
void or_split_rhs(const or_grid* g, const double* rho, const double* u, const double* v,
                  const double* w, const double* ph, double rho12, double dt, double* src) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const double dx2 = g->dx * g->dx, dy2 = g->dy * g->dy, dz2 = g->dz * g->dz;
  const int three = nz > 1;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t sz = (size_t)nx * ny;
        const size_t q = ((size_t)k * ny + j) * nx + i;
        /* neighbour indices with the walls clamped to the cell (ghost = copy) */
        const size_t qr = i < nx - 1 ? q + 1 : q, ql = i > 0 ? q - 1 : q;
        const size_t qf = j < ny - 1 ? q + nx : q, qb = j > 0 ? q - nx : q;
        const size_t qu = k < nz - 1 ? q + sz : q, qd = k > 0 ? q - sz : q;
        const double r = (1.0 - 2.0 * rho12 / (rho[q] + rho[qr])) / dx2;
        const double l = (1.0 - 2.0 * rho12 / (rho[q] + rho[ql])) / dx2;
        const double f = (1.0 - 2.0 * rho12 / (rho[q] + rho[qf])) / dy2;
        const double b = (1.0 - 2.0 * rho12 / (rho[q] + rho[qb])) / dy2;
        double up = 0.0, dn = 0.0, c;
        if (three) {
          up = (1.0 - 2.0 * rho12 / (rho[q] + rho[qu])) / dz2;
          dn = (1.0 - 2.0 * rho12 / (rho[q] + rho[qd])) / dz2;
          c = -(r + l + f + b + up + dn);
        } else {
          c = -(r + l + f + b);
        }
        const size_t fu = ((size_t)k * ny + j) * (nx + 1) + i;
        const size_t fv = ((size_t)k * (ny + 1) + j) * nx + i;
        double d = (u[fu + 1] - u[fu]) / g->dx + (v[fv + nx] - v[fv]) / g->dy;
        if (three) d += (w[q + sz] - w[q]) / g->dz;
        d = d / dt;
        double sv = d * rho12 + c * ph[q] + r * ph[qr] + l * ph[ql] + f * ph[qf] + b * ph[qb];
        if (three) sv = sv + up * ph[qu] + dn * ph[qd];
        src[q] = sv;
      }
}

/* ppe_mg_correction (ns_ppe_mg_solver.f90:223-276) on the interior faces:    */
/*   u_f -= dt [ (1/rho_12)(p_nb - p_i)/h + (2/(rho_i+rho_nb) - 1/rho_12)      */
/*               (p^_nb - p^_i)/h ]                                           */
/* (wall faces get p and p^ differences of zero from the ghosts and stay).    */
void or_split_correct(const or_grid* g, const double* rho, const double* p, const double* ph,
                      double rho12, double dt, double* u, double* v, double* w) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const size_t sz = (size_t)nx * ny;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t q = ((size_t)k * ny + j) * nx + i;
        if (i < nx - 1) {
          double s = 1.0 / rho12 * (p[q + 1] - p[q]) / g->dx;
          s = s + (2.0 / (rho[q] + rho[q + 1]) - 1.0 / rho12) * (ph[q + 1] - ph[q]) / g->dx;
          u[((size_t)k * ny + j) * (nx + 1) + i + 1] -= s * dt;
        }
        if (j < ny - 1) {
          double s = 1.0 / rho12 * (p[q + nx] - p[q]) / g->dy;
          s = s + (2.0 / (rho[q] + rho[q + nx]) - 1.0 / rho12) * (ph[q + nx] - ph[q]) / g->dy;
          v[((size_t)k * (ny + 1) + j + 1) * nx + i] -= s * dt;
        }
        if (k < nz - 1 && w) {
          double s = 1.0 / rho12 * (p[q + sz] - p[q]) / g->dz;
          s = s + (2.0 / (rho[q] + rho[q + sz]) - 1.0 / rho12) * (ph[q + sz] - ph[q]) / g->dz;
          w[q + sz] -= s * dt;
        }
      }
}

/* a13: max and mean |div u| (ns_check_convergence_div, NO2/src/ns_solver/ns_solvers.f90:55-83). */
void or_div_stats(const or_grid* g, const double* u, const double* v, const double* w,
                  double* out_max, double* out_mean) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  double mx = 0.0, sm = 0.0;
#pragma omp parallel for schedule(static) reduction(max : mx) reduction(+ : sm)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        size_t qu = ((size_t)k * ny + j) * (nx + 1) + i;
        size_t qv = ((size_t)k * (ny + 1) + j) * nx + i;
        size_t qw = ((size_t)k * ny + j) * nx + i;
        double d = (u[qu + 1] - u[qu]) / g->dx + (v[qv + nx] - v[qv]) / g->dy;
        if (w) d += (w[qw + (size_t)nx * ny] - w[qw]) / g->dz;
        d = fabs(d);
        mx = d > mx ? d : mx;
        sm += d;
      }
  *out_max = mx;
  *out_mean = sm / (double)cells_of(nx, ny, nz);
}

/* ------------------------------------------------------------------------- */
/* Faithful point relaxation, ppe_sor_solver (NO2 ns_ppe_solver.f90:73-135;   */
/* NO3 :93-163).  The reference sweeps in place under OpenMP (a data race);    */
/* this serial restatement sweeps lexicographically.  Per iteration:           */
/*   tmp = p; p_i = (src - sum coe p_nb)/c in place; p -= mean(p);             */
/*   p = w p + (1-w) tmp; err = max|p - tmp|; stop when err < tol.             */
/* max_iter replaces the reference's STOP (err > 10 after 1e5 sweeps).         */
/* Returns the sweep count (negative if max_iter was reached).                 */
/* ------------------------------------------------------------------------- */
int64_t or_sor_solve(const or_grid* g, const double* cx, const double* cy, const double* cz,
                     const double* b, double* p, double w, double tol, int64_t max_iter,
                     double* out_err) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const size_t n = cells_of(nx, ny, nz);
  double* tmp = (double*)malloc(n * sizeof(double));
  int64_t it = 0;
  double err = 0.0;
  for (;;) {
    ++it;
    memcpy(tmp, p, n * sizeof(double));
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          double d, s = stencil_sum(nx, ny, nz, cx, cy, cz, p, i, j, k, &d);
          size_t q = ((size_t)k * ny + j) * nx + i;
          p[q] = (b[q] - s) / (-d);
        }
    double m = sum_of(p, n) / (double)n;
    err = 0.0;
    for (size_t q = 0; q < n; ++q) {
      p[q] -= m;
      p[q] = w * p[q] + (1.0 - w) * tmp[q];
      double e = fabs(p[q] - tmp[q]);
      err = e > err ? e : err;
    }
    if (err < tol) break;
    if (it >= max_iter) { it = -it; break; }
  }
  free(tmp);
  if (out_err) *out_err = err;
  return it;
}

/* ------------------------------------------------------------------------- */
/* Multigrid: the cycle of DD3 (multigrid_solver.f90:1-326, tree_multigrid.f90) */
/* applied to the variable-coefficient operator of ppe_sor_init.              */
/* ------------------------------------------------------------------------- */
typedef struct {
  int nx, ny, nz;
  int fx, fy, fz; /* coarsening factor from this level to the next (1 or 2) */
  double *cx, *cy, *cz;
  double *sol, *src, *res, *snap;
} or_level;

typedef struct {
  int L;
  or_level lv[32];
  int nc;          /* coarsest cell count */
  double* Minv;    /* nc x nc inverse of the mean-constrained coarsest operator */
  double* Adense;  /* nc x nc coarsest operator (for the refinement step) */
} or_mg;

void or_mg_default(or_mg_params* prm) {
  memset(prm, 0, sizeof(*prm));
  prm->nu1 = 2;
  prm->nu2 = 2;
  prm->levels = 0;
  prm->coarse_max = 64;
  prm->max_cycles = 100;
  prm->smoother = 0;
  prm->blocks[0] = prm->blocks[1] = prm->blocks[2] = 1;
  prm->mean_every_sweep = 1;
  prm->coarse_op = 0;
  prm->record_history = 1;
  prm->krylov = 0;
  prm->prolong = 0;
  prm->coarse_scale = 1.0;
}

/* Level plan.  Each axis with more than one cell is halved per level; an axis
 * of one cell (nz = 1 in 2D) is never coarsened.  Explicit levels require
 * divisibility as manager_init does (DD3/lib/data/branches.f90:172-216);
 * auto mode stops when the next halving is impossible or the level already
 * has <= coarse_max cells.  Returns the level count or -1. */
int or_mg_plan(int nx, int ny, int nz, int levels, int coarse_max, int32_t* dims_out) {
  int L = 1;
  int n[3] = {nx, ny, nz};
  if (nx < 1 || ny < 1 || nz < 1) return -1;
  if (dims_out) { dims_out[0] = nx; dims_out[1] = ny; dims_out[2] = nz; }
  for (;;) {
    if (levels > 0 && L >= levels) break;
    if (levels <= 0 && (long)n[0] * n[1] * n[2] <= coarse_max) break;
    int ok = 1, any = 0;
    for (int a = 0; a < 3; ++a)
      if (n[a] > 1) { any = 1; if (n[a] % 2) ok = 0; }
    if (!ok || !any) {
      if (levels > 0) return -1;
      break;
    }
    for (int a = 0; a < 3; ++a)
      if (n[a] > 1) n[a] /= 2;
    if (dims_out) { dims_out[3 * L] = n[0]; dims_out[3 * L + 1] = n[1]; dims_out[3 * L + 2] = n[2]; }
    ++L;
    if (L >= 32) return -1;
  }
  return L;
}

/* Coarse face coefficients from the fine ones.  No reference counterpart (its
 * multigrid is constant-coefficient, DD3 multigrid_solver.f90:12); the coarse
 * operator is rediscretised with spacing 2h:
 *   coarse_op 0: beta_c = mean of the fine face betas covering the coarse face;
 *   coarse_op 1: along the normal, the fine links between the two coarse
 *     centres in series (half, full, half link), averaged over the tangential
 *     children: coe_c = mean_t 1/(1/c_{2I-1} + 2/c_{2I} + 1/c_{2I+1}).
 * Both reduce to coe_c = coe/4 for constant coefficients. */
static void coarsen_coef(const or_level* f, or_level* c, int op) {
  const int nx = c->nx, ny = c->ny, nz = c->nz;
  const int fx = f->fx, fy = f->fy, fz = f->fz;
  const int fnx = f->nx, fny = f->ny;
  const double tang = 1.0 / (double)(fx * fy * fz);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        size_t q = ((size_t)k * ny + j) * nx + i;
        for (int a = 0; a < 3; ++a) {
          const double* fc = a == 0 ? f->cx : (a == 1 ? f->cy : f->cz);
          double* cc = a == 0 ? c->cx : (a == 1 ? c->cy : c->cz);
          int idx = a == 0 ? i : (a == 1 ? j : k);
          int fa = a == 0 ? fx : (a == 1 ? fy : fz);
          if (idx == 0 || fa == 1) { cc[q] = 0.0; continue; }
          size_t fs = a == 0 ? 1 : (a == 1 ? (size_t)fnx : (size_t)fnx * fny);
          double acc = 0.0;
          for (int dz = 0; dz < fz; ++dz)
            for (int dy = 0; dy < fy; ++dy)
              for (int dx = 0; dx < fx; ++dx) {
                /* children that touch the coarse low face along axis a only */
                if ((a == 0 && dx) || (a == 1 && dy) || (a == 2 && dz)) continue;
                size_t fq = ((size_t)(fz * k + dz) * fny + (fy * j + dy)) * fnx + (fx * i + dx);
                if (op == 0 || op == 2) {
                  acc += fc[fq];
                } else {
                  double c1 = fc[fq - fs], c2 = fc[fq], c3 = fc[fq + fs];
                  acc += (c1 > 0.0 && c2 > 0.0 && c3 > 0.0) ? 1.0 / (1.0 / c1 + 2.0 / c2 + 1.0 / c3) : 0.0;
                }
              }
          /* fa children along the normal were skipped: the count is fx*fy*fz/fa */
          acc *= tang * fa;
          /* op 2: Galerkin R A P with piecewise-constant P and averaging R:
           * sum of the crossing fine coefficients / 2^d = mean / fa */
          cc[q] = op == 0 ? acc / (double)(fa * fa) : (op == 2 ? acc / (double)fa : acc);
        }
      }
}

static double* dalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

/* Dense solve of the coarsest level (manager_mg_setup / manager_mg_solve_exact /
 * mg_find_error / mg_solve_correct, DD3 tree_multigrid.f90:1-238).  The
 * reference LU-factors the singular Neumann matrix with dgesv; here the null
 * space is removed first: M = A - s 11^T/n (s = mean diagonal), which is
 * non-singular and gives the mean-free solution for a mean-free right-hand
 * side.  M is inverted once per operator by Gauss-Jordan with partial
 * pivoting; each cycle applies the inverse, does the reference's one
 * refinement step when max|b - A x| > 1e-10, and projects the mean. */
static int build_coarse(or_mg* mg) {
  or_level* c = &mg->lv[mg->L - 1];
  const int nx = c->nx, ny = c->ny, nz = c->nz;
  const int n = nx * ny * nz;
  mg->nc = n;
  double* A = dalloc((size_t)n * n);
  double* M = dalloc((size_t)n * 2 * n);
  mg->Minv = dalloc((size_t)n * n);
  mg->Adense = A;
  double dsum = 0.0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        int q = (k * ny + j) * nx + i;
        double d = 0.0, cc;
        if (i > 0) { cc = c->cx[q]; A[(size_t)q * n + q - 1] += cc; d += cc; }
        if (i < nx - 1) { cc = c->cx[q + 1]; A[(size_t)q * n + q + 1] += cc; d += cc; }
        if (j > 0) { cc = c->cy[q]; A[(size_t)q * n + q - nx] += cc; d += cc; }
        if (j < ny - 1) { cc = c->cy[q + nx]; A[(size_t)q * n + q + nx] += cc; d += cc; }
        if (k > 0) { cc = c->cz[q]; A[(size_t)q * n + q - nx * ny] += cc; d += cc; }
        if (k < nz - 1) { cc = c->cz[q + nx * ny]; A[(size_t)q * n + q + nx * ny] += cc; d += cc; }
        A[(size_t)q * n + q] -= d;
        dsum += d;
      }
  double s = (n > 0 ? dsum / n : 1.0);
  if (s <= 0.0) s = 1.0;
  for (int r = 0; r < n; ++r) {
    for (int q = 0; q < n; ++q) M[(size_t)r * 2 * n + q] = A[(size_t)r * n + q] - s / n;
    M[(size_t)r * 2 * n + n + r] = 1.0;
  }
  for (int col = 0; col < n; ++col) {
    int piv = col;
    double best = fabs(M[(size_t)col * 2 * n + col]);
    for (int r = col + 1; r < n; ++r) {
      double v = fabs(M[(size_t)r * 2 * n + col]);
      if (v > best) { best = v; piv = r; }
    }
    if (best == 0.0) { free(M); return OR_BAD_ARG; }
    if (piv != col)
      for (int q = 0; q < 2 * n; ++q) {
        double t = M[(size_t)col * 2 * n + q];
        M[(size_t)col * 2 * n + q] = M[(size_t)piv * 2 * n + q];
        M[(size_t)piv * 2 * n + q] = t;
      }
    double inv = 1.0 / M[(size_t)col * 2 * n + col];
    for (int q = 0; q < 2 * n; ++q) M[(size_t)col * 2 * n + q] *= inv;
    for (int r = 0; r < n; ++r) {
      if (r == col) continue;
      double f = M[(size_t)r * 2 * n + col];
      if (f == 0.0) continue;
      for (int q = 0; q < 2 * n; ++q) M[(size_t)r * 2 * n + q] -= f * M[(size_t)col * 2 * n + q];
    }
  }
  for (int r = 0; r < n; ++r)
    for (int q = 0; q < n; ++q) mg->Minv[(size_t)r * n + q] = M[(size_t)r * 2 * n + n + q];
  free(M);
  return OR_OK;
}

static void v_cycle(or_mg* mg, const or_mg_params* prm);
static void coarse_solve(or_mg* mg) {
  or_level* c = &mg->lv[mg->L - 1];
  const int n = mg->nc;
  double* x = c->sol;
  const double* b = c->src;
  double* e = dalloc(n);
  for (int r = 0; r < n; ++r) {
    double a = 0.0;
    for (int q = 0; q < n; ++q) a += mg->Minv[(size_t)r * n + q] * b[q];
    x[r] = a;
  }
  /* mg_find_error: error = b - A x; refine once when max|error| > 1e-10 */
  double emax = 0.0;
  for (int r = 0; r < n; ++r) {
    double a = b[r];
    for (int q = 0; q < n; ++q) a -= mg->Adense[(size_t)r * n + q] * x[q];
    e[r] = a;
    emax = fabs(a) > emax ? fabs(a) : emax;
  }
  if (emax > 1e-10) {
    for (int r = 0; r < n; ++r) {
      double a = 0.0;
      for (int q = 0; q < n; ++q) a += mg->Minv[(size_t)r * n + q] * e[q];
      x[r] += a;
    }
  }
  free(e);
  or_remove_mean(x, n); /* multigrid_final_exact: compatibility_sol (DD3 :100) */
}

static int mg_setup(or_mg* mg, const or_grid* g, const double* cx, const double* cy,
                    const double* cz, const or_mg_params* prm) {
  int32_t dims[96];
  int L = or_mg_plan(g->nx, g->ny, g->nz, prm->levels, prm->coarse_max, dims);
  if (L < 1) return OR_BAD_ARG;
  memset(mg, 0, sizeof(*mg));
  mg->L = L;
  for (int l = 0; l < L; ++l) {
    or_level* v = &mg->lv[l];
    v->nx = dims[3 * l];
    v->ny = dims[3 * l + 1];
    v->nz = dims[3 * l + 2];
    size_t n = cells_of(v->nx, v->ny, v->nz);
    if (l + 1 < L) {
      v->fx = v->nx / dims[3 * l + 3];
      v->fy = v->ny / dims[3 * l + 4];
      v->fz = v->nz / dims[3 * l + 5];
    } else {
      v->fx = v->fy = v->fz = 1;
    }
    if (l == 0) {
      v->cx = (double*)cx; v->cy = (double*)cy; v->cz = (double*)cz;
      v->src = NULL; v->sol = NULL;
    } else {
      v->cx = dalloc(n); v->cy = dalloc(n); v->cz = dalloc(n);
      v->src = dalloc(n); v->sol = dalloc(n);
    }
    v->res = dalloc(n);
    v->snap = dalloc(n);
  }
  for (int l = 1; l < L; ++l) coarsen_coef(&mg->lv[l - 1], &mg->lv[l], prm->coarse_op);
  return build_coarse(mg);
}

static void mg_free(or_mg* mg) {
  for (int l = 0; l < mg->L; ++l) {
    or_level* v = &mg->lv[l];
    if (l > 0) { free(v->cx); free(v->cy); free(v->cz); free(v->src); free(v->sol); }
    free(v->res);
    free(v->snap);
  }
  free(mg->Minv);
  free(mg->Adense);
}

/* One smoothing sweep.  Red-black: all cells with (i+j+k) even, then odd,
 * each colour from the latest values (deterministic, order-free).  Blocked
 * lexicographic: the reference's multigrid_relax (DD3 multigrid_solver.f90:1-49)
 * runs an in-place lexicographic Gauss-Seidel inside each OpenMP subdomain and
 * reads neighbouring subdomains through halos refreshed only before the sweep
 * (ptrmgpart_sync, DD3/lib/pointer/ptr_roots.f90:437-606); blocks = 1x1x1 is a
 * plain serial lexicographic sweep. */
static void smooth_sweep(or_level* v, const or_mg_params* prm, int reverse) {
  const int nx = v->nx, ny = v->ny, nz = v->nz;
  double* p = v->sol;
  const double* b = v->src;
  if (prm->smoother == 0) {
    for (int cc = 0; cc < 2; ++cc) {
      const int color = reverse ? 1 - cc : cc;
#pragma omp parallel for schedule(static)
      for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
          for (int i = (j + k + color) & 1; i < nx; i += 2) {
            double d, s = stencil_sum(nx, ny, nz, v->cx, v->cy, v->cz, p, i, j, k, &d);
            size_t q = ((size_t)k * ny + j) * nx + i;
            p[q] = (s - b[q]) / d;
          }
    }
  } else {
    const size_t n = cells_of(nx, ny, nz);
    memcpy(v->snap, p, n * sizeof(double));
    const int bx = prm->blocks[0] > 0 ? prm->blocks[0] : 1;
    const int by = prm->blocks[1] > 0 ? prm->blocks[1] : 1;
    const int bz = prm->blocks[2] > 0 ? prm->blocks[2] : 1;
    const int nb = bx * by * bz;
#pragma omp parallel for schedule(static)
    for (int id = 0; id < nb; ++id) {
      int ib = id % bx, jb = (id / bx) % by, kb = id / (bx * by);
      int i0 = (int)((long)nx * ib / bx), i1 = (int)((long)nx * (ib + 1) / bx);
      int j0 = (int)((long)ny * jb / by), j1 = (int)((long)ny * (jb + 1) / by);
      int k0 = (int)((long)nz * kb / bz), k1 = (int)((long)nz * (kb + 1) / bz);
      const size_t sy = nx, sz = (size_t)nx * ny;
      for (int k = k0; k < k1; ++k)
        for (int j = j0; j < j1; ++j)
          for (int i = i0; i < i1; ++i) {
            size_t q = ((size_t)k * ny + j) * nx + i;
            double s = 0.0, d = 0.0, c;
            /* neighbours inside the block: latest values; outside: the halo snapshot */
            if (i > 0) { c = v->cx[q]; s += c * (i - 1 >= i0 ? p[q - 1] : v->snap[q - 1]); d += c; }
            if (i < nx - 1) { c = v->cx[q + 1]; s += c * (i + 1 < i1 ? p[q + 1] : v->snap[q + 1]); d += c; }
            if (j > 0) { c = v->cy[q]; s += c * (j - 1 >= j0 ? p[q - sy] : v->snap[q - sy]); d += c; }
            if (j < ny - 1) { c = v->cy[q + sy]; s += c * (j + 1 < j1 ? p[q + sy] : v->snap[q + sy]); d += c; }
            if (k > 0) { c = v->cz[q]; s += c * (k - 1 >= k0 ? p[q - sz] : v->snap[q - sz]); d += c; }
            if (k < nz - 1) { c = v->cz[q + sz]; s += c * (k + 1 < k1 ? p[q + sz] : v->snap[q + sz]); d += c; }
            p[q] = (s - b[q]) / d;
          }
    }
  }
}

/* multigrid_relax (DD3 :1-49): num sweeps, each followed by compatibility_sol.
 * reverse = 1 runs the red-black colours black-first (post-smoothing of the
 * symmetric V-cycle used as a Krylov preconditioner). */
static void relax(or_level* v, int num, const or_mg_params* prm, int reverse) {
  const size_t n = cells_of(v->nx, v->ny, v->nz);
  for (int s = 0; s < num; ++s) {
    smooth_sweep(v, prm, reverse);
    if (prm->mean_every_sweep) or_remove_mean(v->sol, (int64_t)n);
  }
}

static double level_residual(or_level* v) {
  or_grid g = {v->nx, v->ny, v->nz, 1, 1, 1};
  return or_residual(&g, v->cx, v->cy, v->cz, v->sol, v->src, v->res);
}

/* multigrid_restriction (DD3 :51-90): relax, residual, coarse src = mean of the
 * children's residuals, coarse sol = 0, compatibility_src. */
static void restrict_level(or_mg* mg, int l, const or_mg_params* prm) {
  or_level* f = &mg->lv[l];
  or_level* c = &mg->lv[l + 1];
  relax(f, prm->nu1, prm, 0);
  level_residual(f);
  const int fx = f->fx, fy = f->fy, fz = f->fz, fnx = f->nx, fny = f->ny;
  const double w = 1.0 / (double)(fx * fy * fz);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < c->nz; ++k)
    for (int j = 0; j < c->ny; ++j)
      for (int i = 0; i < c->nx; ++i) {
        double s = 0.0;
        for (int dz = 0; dz < fz; ++dz)
          for (int dy = 0; dy < fy; ++dy)
            for (int dx = 0; dx < fx; ++dx)
              s += f->res[((size_t)(fz * k + dz) * fny + (fy * j + dy)) * fnx + (fx * i + dx)];
        size_t q = ((size_t)k * c->ny + j) * c->nx + i;
        c->src[q] = s * w;
        c->sol[q] = 0.0;
      }
  or_remove_mean(c->src, (int64_t)cells_of(c->nx, c->ny, c->nz));
}

/* multigrid_prolongation (DD3 :106-160): central slopes of the coarse solution
 * with zero-gradient ghosts (ptrmgpart_sync copies the first interior cell into
 * the wall ghost), child = e_c +/- m_x/4 +/- m_y/4 +/- m_z/4 on coarsened axes,
 * sol += child value, then relax. */
static void prolong_level(or_mg* mg, int l, const or_mg_params* prm) {
  or_level* f = &mg->lv[l];
  or_level* c = &mg->lv[l + 1];
  const int cnx = c->nx, cny = c->ny, cnz = c->nz;
  const size_t csy = cnx, csz = (size_t)cnx * cny;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < f->nz; ++k)
    for (int j = 0; j < f->ny; ++j)
      for (int i = 0; i < f->nx; ++i) {
        int I = i / f->fx, J = j / f->fy, K = k / f->fz;
        size_t cq = ((size_t)K * cny + J) * cnx + I;
        const double* e = c->sol;
        double ec = e[cq], val = ec;
        if (prm->prolong == 1) {
          f->sol[((size_t)k * f->ny + j) * f->nx + i] += prm->coarse_scale * val;
          continue;
        }
        if (f->fx == 2) {
          double em = I > 0 ? e[cq - 1] : ec, ep = I < cnx - 1 ? e[cq + 1] : ec;
          double m = 0.5 * (ep - em);
          val += (i & 1) ? 0.25 * m : -0.25 * m;
        }
        if (f->fy == 2) {
          double em = J > 0 ? e[cq - csy] : ec, ep = J < cny - 1 ? e[cq + csy] : ec;
          double m = 0.5 * (ep - em);
          val += (j & 1) ? 0.25 * m : -0.25 * m;
        }
        if (f->fz == 2) {
          double em = K > 0 ? e[cq - csz] : ec, ep = K < cnz - 1 ? e[cq + csz] : ec;
          double m = 0.5 * (ep - em);
          val += (k & 1) ? 0.25 * m : -0.25 * m;
        }
        f->sol[((size_t)k * f->ny + j) * f->nx + i] += prm->coarse_scale == 1.0 ? val : prm->coarse_scale * val;
      }
  relax(f, prm->nu2, prm, prm->krylov ? 1 : 0);
}

/* multigrid_v_cycle (DD3 :310-326). */
static void v_cycle(or_mg* mg, const or_mg_params* prm) {
  for (int l = 0; l < mg->L - 1; ++l) restrict_level(mg, l, prm);
  coarse_solve(mg);
  for (int l = mg->L - 2; l >= 0; --l) prolong_level(mg, l, prm);
}

static double dot(const double* a, const double* b, size_t n) {
  double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s)
  for (size_t q = 0; q < n; ++q) s += a[q] * b[q];
  return s;
}

/* Flexible preconditioned CG (Polak-Ribiere beta), preconditioner = one V-cycle
 * from a zero initial guess on the residual.  No reference counterpart: an
 * optional acceleration for many-bubble cases where the stationary cycle
 * stalls on the near-null modes of isolated light bubbles.  A and the V-cycle
 * are both negative (semi)definite; the signs cancel in alpha and beta. */
static int pcg_loop(or_mg* mg, const or_mg_params* prm, const or_grid* g, double* p,
                    const double* b, double bnorm, double tol, or_mg_stats* st, int* cyc_out,
                    double* rel_out, double* r2_out) {
  const size_t n = cells_of(g->nx, g->ny, g->nz);
  or_level* f = &mg->lv[0];
  double* r = dalloc(n);
  double* z = dalloc(n);
  double* zold = dalloc(n);
  double* d = dalloc(n);
  double* q = dalloc(n);
  double* x = f->sol; /* == p */
  double r2 = or_residual(g, f->cx, f->cy, f->cz, x, b, r);
  double rel = sqrt(r2) / (bnorm > 0 ? bnorm : 1.0);
  int status = OR_NOT_CONVERGED, it;
  double rz = 0.0;
  /* the V-cycle works on level 0's (sol, src) = (z, r) */
  f->src = r;
  for (it = 1; it <= prm->max_cycles; ++it) {
    memset(z, 0, n * sizeof(double));
    f->sol = z;
    v_cycle(mg, prm);
    or_remove_mean(z, (int64_t)n);
    double rz_new = dot(r, z, n);
    if (it == 1) {
      memcpy(d, z, n * sizeof(double));
    } else {
      double beta = (rz_new - dot(r, zold, n)) / rz;
#pragma omp parallel for schedule(static)
      for (size_t k = 0; k < n; ++k) d[k] = z[k] + beta * d[k];
    }
    rz = rz_new;
    memcpy(zold, z, n * sizeof(double));
    or_apply(g, f->cx, f->cy, f->cz, d, q);
    double alpha = rz / dot(d, q, n);
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n; ++k) { x[k] += alpha * d[k]; r[k] -= alpha * q[k]; }
    /* true residual for the stopping test, as the stationary loop does */
    r2 = or_residual(g, f->cx, f->cy, f->cz, x, b, r);
    rel = sqrt(r2) / (bnorm > 0 ? bnorm : 1.0);
    if (prm->record_history && it <= 256) st->history[it - 1] = rel;
    if (!isfinite(rel) || rel > 1e3) { status = OR_DIVERGED; break; }
    if (rel < tol) { status = OR_OK; break; }
  }
  if (it > prm->max_cycles) it = prm->max_cycles;
  f->sol = p;
  f->src = (double*)b;
  free(r); free(z); free(zold); free(d); free(q);
  *cyc_out = it;
  *rel_out = rel;
  *r2_out = r2;
  return status;
}

/* The solve.  Outer loop as ppe_mg_solver (DD3/src/ns_solver/ns_ppe_mg_solver.f90:
 * 17-50): V-cycles until the relative residual ||b - A p||_2/||b||_2 < tol, at
 * most max_cycles.  p is the initial guess on entry (warm start) and the
 * mean-free solution on exit.  b must be mean-free (compatible). */
int or_mg_solve(const or_grid* g, const double* cx, const double* cy, const double* cz,
                const double* b, double* p, double tol, const or_mg_params* prm_in,
                or_mg_stats* st) {
  or_mg_params prm;
  if (prm_in) prm = *prm_in; else or_mg_default(&prm);
  or_mg mg;
  or_mg_stats local;
  if (!st) st = &local;
  memset(st, 0, sizeof(*st));
  int rc = mg_setup(&mg, g, cx, cy, cz, &prm);
  if (rc) { st->status = OR_BAD_ARG; return OR_BAD_ARG; }
  st->levels = mg.L;
  st->coarse_n = mg.nc;
  or_level* f = &mg.lv[0];
  f->sol = p;
  f->src = (double*)b;
  const size_t n = cells_of(g->nx, g->ny, g->nz);
  double b2 = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : b2)
  for (size_t q = 0; q < n; ++q) b2 += b[q] * b[q];
  const double bnorm = sqrt(b2);
  double r2 = level_residual(f);
  double rel = bnorm > 0 ? sqrt(r2) / bnorm : sqrt(r2);
  int status = OR_NOT_CONVERGED;
  int cyc = 0;
  if (prm.krylov && !(rel < tol)) {
    status = pcg_loop(&mg, &prm, g, p, b, bnorm, tol, st, &cyc, &rel, &r2);
  } else if (!(rel < tol)) {
    for (cyc = 1; cyc <= prm.max_cycles; ++cyc) {
      v_cycle(&mg, &prm);
      r2 = level_residual(f);
      rel = bnorm > 0 ? sqrt(r2) / bnorm : sqrt(r2);
      if (prm.record_history && cyc <= 256) st->history[cyc - 1] = rel;
      if (!isfinite(rel) || rel > 1e3) { status = OR_DIVERGED; break; }
      if (rel < tol) { status = OR_OK; break; }
    }
    if (cyc > prm.max_cycles) cyc = prm.max_cycles;
  } else {
    status = OR_OK;
  }
  or_remove_mean(p, (int64_t)n);
  st->cycles = cyc;
  st->status = status;
  st->rel_residual = rel;
  st->rms_residual = sqrt(r2 / (double)n);
  mg_free(&mg);
  return status;
}

/* Coarse-level coefficients (for tests of the coarsening rule): writes level
 * `level`'s cx, cy, cz into the caller's arrays sized by or_mg_plan. */
int or_mg_level_coef(const or_grid* g, const double* cx, const double* cy, const double* cz,
                     const or_mg_params* prm, int level, double* ocx, double* ocy, double* ocz) {
  or_mg mg;
  if (mg_setup(&mg, g, cx, cy, cz, prm)) return OR_BAD_ARG;
  if (level < 0 || level >= mg.L) { mg_free(&mg); return OR_BAD_ARG; }
  or_level* v = &mg.lv[level];
  size_t n = cells_of(v->nx, v->ny, v->nz);
  memcpy(ocx, v->cx, n * sizeof(double));
  memcpy(ocy, v->cy, n * sizeof(double));
  memcpy(ocz, v->cz, n * sizeof(double));
  mg_free(&mg);
  return OR_OK;
}

/* ------------------------------------------------------------------------- */
/* Adjoint of the solve (no reference counterpart; the FP64 host reference of  */
/* the differentiable solve).  With (A p)_i = sum_f coe_f (p_nb - p_i) and the */
/* adjoint lam solving A lam = dJ/dp (mean-free):                              */
/*   dJ/dcoe_f   = (lam_nb - lam_i)(p_nb - p_i)                                */
/*   dcoe_f/drho = -2/(rho_i + rho_nb)^2/h^2 for both cells of the face        */
/*   dJ/drho_i   = sum over the faces of cell i of the two products            */
/* and through rho = rho_pos H(phi/eps) + rho_neg (1 - H):                      */
/*   dJ/dphi_i   = dJ/drho_i (rho_pos - rho_neg) H'(phi_i)                      */
/* phi may be NULL (grad_phi then not written).                                */
/* ------------------------------------------------------------------------- */
void or_adjoint(const or_grid* g, const double* rho, const double* p, const double* lam,
                const double* phi, double eps, double rho_pos, double rho_neg, double* grad_rho,
                double* grad_phi) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const size_t sy = nx, sz = (size_t)nx * ny;
  const double h2[3] = {g->dx * g->dx, g->dy * g->dy, g->dz * g->dz};
  const double pi = acos(-1.0);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t q = (size_t)k * sz + (size_t)j * sy + i;
        double acc = 0.0;
        const int has[6] = {i > 0, i < nx - 1, j > 0, j < ny - 1, k > 0, k < nz - 1};
        const long off[6] = {-1, 1, -(long)sy, (long)sy, -(long)sz, (long)sz};
        for (int f = 0; f < 6; ++f) {
          if (!has[f]) continue;
          const size_t n = (size_t)((long)q + off[f]);
          const double s = rho[q] + rho[n];
          const double dcoe = -2.0 / (s * s) / h2[f / 2];
          acc += (lam[n] - lam[q]) * (p[n] - p[q]) * dcoe;
        }
        grad_rho[q] = acc;
        if (phi && grad_phi) {
          const double x = phi[q] / eps;
          const double hp = (x > 1.0 - 1e-12 || x < -1.0 + 1e-12) ? 0.0 : 0.5 * (1.0 + cos(pi * x)) / eps;
          grad_phi[q] = acc * (rho_pos - rho_neg) * hp;
        }
      }
}

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void or_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ------------------------------------------------------------------------- */
/* Level-set advection, level_set_rk3_solver (NO2 src/interface_solver/       */
/* level_set_rk3_solver.f90:1-128; NO3 :1-160): phi_t + div(u phi) = 0 with   */
/* the cell-centred velocity, the flux split into u+ phi and u- phi           */
/* (level_set_rk3_source_setup), each part reconstructed at the faces by      */
/* WENO-JS (wenojs_flux_split, NO2 :131-186, EPS = 1e-13), zero-gradient      */
/* ghosts for the split fluxes (bc, NO2 src/others/bcs.f90:1-26) and three    */
/* stages of SSP-RK3 in the reference's incremental form.  nz = 1 is the 2D   */
/* solver (no z term).                                                        */
/* ------------------------------------------------------------------------- */
static inline double ls_sq(double x) { return x * x; }

/* value at face i+1/2 of g(i-2..i+2) = g0..g4, biased to the left */
static double or_weno_left(double g0, double g1, double g2, double g3, double g4, double eps) {
  const double b1 = 13.0 * ls_sq((g0 - 2.0 * g1) + g2) + 3.0 * ls_sq((g0 - 4.0 * g1) + 3.0 * g2);
  const double b2 = 13.0 * ls_sq((g1 - 2.0 * g2) + g3) + 3.0 * ls_sq(g1 - g3);
  const double b3 = 13.0 * ls_sq((g2 - 2.0 * g3) + g4) + 3.0 * ls_sq((3.0 * g2 - 4.0 * g3) + g4);
  const double a1 = 1.0 / ls_sq(eps + b1), a2 = 6.0 / ls_sq(eps + b2), a3 = 3.0 / ls_sq(eps + b3);
  const double s = (a1 + a2) + a3;
  const double w1 = a1 / s, w2 = a2 / s, w3 = a3 / s;
  double v = w1 / 3.0 * g0;
  v = v - (7.0 * w1 + w2) / 6.0 * g1;
  v = v + ((11.0 * w1 + 5.0 * w2) + 2.0 * w3) / 6.0 * g2;
  v = v + (2.0 * w2 + 5.0 * w3) / 6.0 * g3;
  v = v - w3 / 6.0 * g4;
  return v;
}

/* value at face i+1/2 of f(i-1..i+3) = f0..f4, biased to the right */
static double or_weno_right(double f0, double f1, double f2, double f3, double f4, double eps) {
  const double b3 = 13.0 * ls_sq((f0 - 2.0 * f1) + f2) + 3.0 * ls_sq((f0 - 4.0 * f1) + 3.0 * f2);
  const double b2 = 13.0 * ls_sq((f1 - 2.0 * f2) + f3) + 3.0 * ls_sq(f1 - f3);
  const double b1 = 13.0 * ls_sq((f2 - 2.0 * f3) + f4) + 3.0 * ls_sq((3.0 * f2 - 4.0 * f3) + f4);
  const double a1 = 1.0 / ls_sq(eps + b1), a2 = 6.0 / ls_sq(eps + b2), a3 = 3.0 / ls_sq(eps + b3);
  const double s = (a1 + a2) + a3;
  const double w1 = a1 / s, w2 = a2 / s, w3 = a3 / s;
  double v = w3 * ((-f0 + 5.0 * f1) + 2.0 * f2) / 6.0;
  v = v + w2 * ((2.0 * f1 + 5.0 * f2) - f3) / 6.0;
  v = v + w1 * ((11.0 * f2 - 7.0 * f3) + 2.0 * f4) / 6.0;
  return v;
}

static inline int ls_clamp(int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); }

/* split flux of cell c along one axis: sgn +1 -> u+ phi, -1 -> u- phi */
static inline double ls_split(const double* phi, const double* vel, size_t c, int sgn) {
  const double a = vel[c];
  return sgn > 0 ? 0.5 * (a + fabs(a)) * phi[c] : 0.5 * (a - fabs(a)) * phi[c];
}

/* L(phi) = -sum over axes of (ss1(i) + ss2(i) - ss1(i-1) - ss2(i-1))/h
 * (level_set_rk3_source): ss1 the left-biased value of u+ phi, ss2 the
 * right-biased value of u- phi at face i+1/2 */
void or_ls_source(const or_grid* g, const double* phi, const double* u, const double* v,
                  const double* w, double* out) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const double eps = 1.0e-13;
  const int dims[3] = {nx, ny, nz};
  const size_t strides[3] = {1, (size_t)nx, (size_t)nx * ny};
  const double* vel[3] = {u, v, w};
  const double h[3] = {g->dx, g->dy, g->dz};
  const int naxes = nz > 1 ? 3 : 2;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int idx[3] = {i, j, k};
        const size_t q = ((size_t)k * ny + j) * nx + i;
        double src = 0.0;
        for (int a = 0; a < naxes; ++a) {
          const int n = dims[a], c = idx[a];
          const size_t base = q - (size_t)c * strides[a];
          double ss1[2], ss2[2];
          for (int f = 0; f < 2; ++f) {  /* faces c-1/2 (f = 0) and c+1/2 (f = 1) */
            const int fi = c - 1 + f;     /* the face is fi+1/2 */
            double gv[5], fv[5];
            for (int m = 0; m < 5; ++m) {
              const size_t cg = base + (size_t)ls_clamp(fi - 2 + m, n) * strides[a];
              const size_t cf = base + (size_t)ls_clamp(fi - 1 + m, n) * strides[a];
              gv[m] = ls_split(phi, vel[a], cg, 1);
              fv[m] = ls_split(phi, vel[a], cf, -1);
            }
            ss1[f] = or_weno_left(gv[0], gv[1], gv[2], gv[3], gv[4], eps);
            ss2[f] = or_weno_right(fv[0], fv[1], fv[2], fv[3], fv[4], eps);
          }
          const double d = ((ss1[1] + ss2[1]) - ss1[0]) - ss2[0];
          src = a == 0 ? -(d / h[a]) : src - d / h[a];
        }
        out[q] = src;
      }
}

/* steps SSP-RK3 steps (level_set_rk3_solver); l1..l3: scratch of n cells */
void or_ls_advect(const or_grid* g, double* phi, const double* u, const double* v,
                  const double* w, double dt, int steps) {
  const size_t n = cells_of(g->nx, g->ny, g->nz);
  double* l1 = (double*)malloc(n * sizeof(double));
  double* l2 = (double*)malloc(n * sizeof(double));
  double* l3 = (double*)malloc(n * sizeof(double));
  for (int s = 0; s < steps; ++s) {
    or_ls_source(g, phi, u, v, w, l1);
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < n; ++q) phi[q] = phi[q] + l1[q] * dt;
    or_ls_source(g, phi, u, v, w, l2);
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < n; ++q) {
      const double src = (-3.0 * l1[q] + l2[q]) / 4.0;
      phi[q] = phi[q] + src * dt;
    }
    or_ls_source(g, phi, u, v, w, l3);
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < n; ++q) {
      const double src = ((-l1[q] - l2[q]) + 8.0 * l3[q]) / 12.0;
      phi[q] = phi[q] + src * dt;
    }
  }
  free(l1);
  free(l2);
  free(l3);
}

/* ------------------------------------------------------------------------- */
/* Level-set redistancing, level_set_rk3_redis (NO2 src/interface_solver/     */
/* level_set_rk3_redis.f90:1-361; NO3 :1-420 for nz > 1).  phi_tau +          */
/* S (|grad phi| - 1) = 0 in pseudo time rdt with the sign S fixed at the    */
/* start (ls_funs: S = 2H - 1; btn = 0, level_set_redis_stable: S = phi and  */
/* phi is first divided by max |grad phi|), the Godunov gradient of WENO-JS  */
/* one-sided derivatives of the backward differences (level_set_redis_       */
/* gradient, wenojs_flux with EPS = 1e-10), and for btn = 1 the mass-        */
/* preserving correction lambda (level_set_redis_lambda: 2D lam = delta,     */
/* weight 16 over a 3x3 block; 3D lam = (2(1 - rho_12)H + rho_12) delta,     */
/* weight 51 over 3x3x3).  Three SSP-RK3 stages per iteration; stop when    */
/* the time passes 3 dx (btn = 1) or 1.5 x the largest extent (btn = 0), or */
/* when max |change| <= 1e-8 (2D) / 1e-5 (3D).                               */
/* ------------------------------------------------------------------------- */
static void or_ls_funs1(double phi, double ls_wid, double* heavy, double* delta, double* sgn) {
  const double eps = 1.0e-12, pi = acos(-1.0);
  const double x = phi / ls_wid;
  double h, hp;
  if (x > 1.0 - eps) {
    h = 1.0;
    hp = 0.0;
  } else if (x < -1.0 + eps) {
    h = 0.0;
    hp = 0.0;
  } else {
    h = 0.5 * ((1.0 + x) + sin(pi * x) / pi);
    hp = 0.5 * (1.0 + cos(pi * x)) / ls_wid;
  }
  h = h < 1.0 ? h : 1.0;
  h = h > 0.0 ? h : 0.0;
  *heavy = h;
  *delta = hp;
  *sgn = 2.0 * h - 1.0;
}

/* backward difference of phi at cell m of a line (zero-gradient ghosts) */
static inline double ls_nrm(const double* phi, size_t base, size_t stride, int m, int n, double h) {
  const int c = ls_clamp(m, n);
  const int cm = c > 0 ? c - 1 : 0;
  return (phi[base + (size_t)c * stride] - phi[base + (size_t)cm * stride]) / h;
}

static inline double ls_max(double a, double b) { return a > b ? a : b; }
static inline double ls_min(double a, double b) { return a < b ? a : b; }

/* |grad phi| per cell, Godunov upwinding by the sign s (level_set_redis_gradient) */
void or_ls_gradient(const or_grid* g, const double* phi, const double* s, double* grad) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const int dims[3] = {nx, ny, nz};
  const size_t strides[3] = {1, (size_t)nx, (size_t)nx * ny};
  const double h[3] = {g->dx, g->dy, g->dz};
  const int naxes = nz > 1 ? 3 : 2;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int idx[3] = {i, j, k};
        const size_t q = ((size_t)k * ny + j) * nx + i;
        double sum = 0.0;
        for (int a = 0; a < naxes; ++a) {
          const int n = dims[a], c = idx[a];
          const size_t base = q - (size_t)c * strides[a];
          double f[6];
          for (int m = 0; m < 6; ++m) f[m] = ls_nrm(phi, base, strides[a], c - 2 + m, n, h[a]);
          const double s1 = or_weno_right(f[1], f[2], f[3], f[4], f[5], 1.0e-10);
          const double s2 = or_weno_left(f[0], f[1], f[2], f[3], f[4], 1.0e-10);
          const double pm = -ls_min(s1, 0.0), pp = ls_max(s1, 0.0);
          const double mm = -ls_min(s2, 0.0), mp = ls_max(s2, 0.0);
          const double t = s[q] >= 0.0 ? ls_max(pm, mp) : ls_max(pp, mm);
          sum = a == 0 ? t * t : sum + t * t;
        }
        grad[q] = sqrt(sum);
      }
}

/* the mass-preserving correction s1 (level_set_redis_lambda, btn = 1) */
static void or_ls_lambda(const or_grid* g, const double* phi, const double* s, const double* grad,
                         double ls_wid, double rho_12, double* s2, double* s3, double* s1) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const size_t n = cells_of(nx, ny, nz);
  const int three = nz > 1;
#pragma omp parallel for schedule(static)
  for (size_t q = 0; q < n; ++q) {
    double hv, dl, sg;
    or_ls_funs1(phi[q], ls_wid, &hv, &dl, &sg);
    const double lam = three ? (2.0 * (1.0 - rho_12) * hv + rho_12) * dl : dl;
    s2[q] = lam * s[q] * (grad[q] - 1.0);
    s3[q] = grad[q] * dl * lam;
  }
  const double wgt = three ? 51.0 : 16.0;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t q = ((size_t)k * ny + j) * nx + i;
        double a = wgt * s2[q], b = wgt * s3[q];
        for (int kk = three ? -1 : 0; kk <= (three ? 1 : 0); ++kk)
          for (int jj = -1; jj <= 1; ++jj)
            for (int ii = -1; ii <= 1; ++ii) {
              const size_t r = ((size_t)ls_clamp(k + kk, nz) * ny + ls_clamp(j + jj, ny)) * nx +
                               ls_clamp(i + ii, nx);
              a = a + s2[r];
              b = b + s3[r];
            }
        double hv, dl, sg;
        or_ls_funs1(phi[q], ls_wid, &hv, &dl, &sg);
        s1[q] = fabs(b) > 1.0e-12 ? a / b * dl : 0.0;
      }
}

int or_ls_redistance(const or_grid* g, double* phi, double ls_wid, double rdt, double rho_12,
                     int btn, int max_iter, double* last_error) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const size_t n = cells_of(nx, ny, nz);
  const int three = nz > 1;
  double* s = (double*)malloc(n * sizeof(double));
  double* grad = (double*)malloc(n * sizeof(double));
  double* s1 = (double*)calloc(n, sizeof(double));
  double* s2 = (double*)malloc(n * sizeof(double));
  double* s3 = (double*)malloc(n * sizeof(double));
  double* l1 = (double*)malloc(n * sizeof(double));
  double* l2 = (double*)malloc(n * sizeof(double));
  double* tmp = (double*)malloc(n * sizeof(double));
  /* level_set_redis_init */
  for (size_t q = 0; q < n; ++q) {
    double hv, dl;
    or_ls_funs1(phi[q], ls_wid, &hv, &dl, &s[q]);
  }
  if (btn == 0) { /* level_set_redis_stable */
    for (size_t q = 0; q < n; ++q) s[q] = phi[q];
    or_ls_gradient(g, phi, s, grad);
    double gm = 0.0;
    for (size_t q = 0; q < n; ++q) gm = ls_max(gm, grad[q]);
    for (size_t q = 0; q < n; ++q) phi[q] = phi[q] / gm;
  }
  const double ext = three ? ls_max(ls_max(nx * g->dx, ny * g->dy), nz * g->dz)
                           : ls_max(nx * g->dx, ny * g->dy);
  const double timestop = btn == 0 ? 1.5 * ext : 3.0 * g->dx;
  const double tol = three ? 1.0e-5 : 1.0e-8;
  double time = 0.0, error = 0.0;
  int iter = 0;
  while (iter < max_iter) {
    ++iter;
    time = time + rdt;
    memcpy(tmp, phi, n * sizeof(double));
    for (int stage = 1; stage <= 3; ++stage) {
      or_ls_gradient(g, phi, s, grad);
      if (btn == 0) {
        memset(s1, 0, n * sizeof(double));
      } else {
        or_ls_lambda(g, phi, s, grad, ls_wid, rho_12, s2, s3, s1);
      }
      for (size_t q = 0; q < n; ++q) {
        const double l = (s[q] - s1[q]) * grad[q] - s[q];
        double src;
        if (stage == 1) {
          l1[q] = l;
          src = l;
        } else if (stage == 2) {
          l2[q] = l;
          src = (-3.0 * l1[q] + l) / 4.0;
        } else {
          src = ((-l1[q] - l2[q]) + 8.0 * l) / 12.0;
        }
        phi[q] = phi[q] - rdt * src;
      }
    }
    error = 0.0;
    for (size_t q = 0; q < n; ++q) error = ls_max(error, fabs(tmp[q] - phi[q]));
    if (time > timestop || error <= tol) break;
  }
  if (last_error) *last_error = error;
  free(s); free(grad); free(s1); free(s2); free(s3); free(l1); free(l2); free(tmp);
  return iter;
}

/* ------------------------------------------------------------------------- */
/* Momentum step of the Adams-Bashforth solver (NO2/NO3 src/ns_solver/        */
/* admas_bashforth_solver.f90: ns_ab_solver_SOR, ns_ab_setup,                */
/* ns_ab_predictor; ns_ab_adv.f90: ns_ab_adv_source_sec; ns_ab_diff.f90:     */
/* sec_part1..3; ns_solvers.f90: ns_linearize, ns_check_convergence_vel;     */
/* src/others/bcs.f90: velbc, find_stag_vel).                                 */
/*                                                                           */
/* These arrays keep the reference's ghost cells: every array is the padded  */
/* box of the reference, (nx+2g)(ny+2g)(nz+2g) (2D: (nx+2g)(ny+2g)), C order  */
/* (z, y, x), and element (i, j, k) in the reference's 1-based indices sits   */
/* at ((k-1+gz)(ny+2g) + j-1+g)(nx+2g) + i-1+g with gz = g in 3D, 0 in 2D.    */
/* u(i,j,k) is the x-face i+1/2 of cell (i,j,k), v and w likewise.  Every     */
/* expression keeps the reference's operand order, and the file is built     */
/* without contraction, so each result is the reference's double rounding.   */
/* ------------------------------------------------------------------------- */
typedef struct {
  int32_t ghost;       /* g, >= 2 */
  int32_t bc[6];       /* velbc: ubc(1), ubc(2), vbc(1), vbc(2), wbc(1), wbc(2) */
  int32_t iterations;  /* predictor-projection passes (the reference: 4) */
  int32_t adv_scheme;  /* 0 second-order upwind (ns_ab_adv_source_sec), 1 QUICK */
  double dt, re, fr, we, mu_12, gx, gy, gz, btn_g, btn_sf, p_tol;
} or_ns_params;

typedef struct {
  int nx, ny, nz, g, gz;
  size_t px, py;
} ns_box;

static ns_box ns_box_of(const or_grid* gr, int g) {
  ns_box b;
  b.nx = gr->nx; b.ny = gr->ny; b.nz = gr->nz; b.g = g;
  b.gz = gr->nz > 1 ? g : 0;
  b.px = (size_t)gr->nx + 2 * (size_t)g;
  b.py = (size_t)gr->ny + 2 * (size_t)g;
  return b;
}

static inline size_t NI(const ns_box* b, int i, int j, int k) {
  return ((size_t)(k - 1 + b->gz) * b->py + (size_t)(j - 1 + b->g)) * b->px + (size_t)(i - 1 + b->g);
}

static size_t ns_span(const ns_box* b) {
  return b->px * b->py * (b->nz > 1 ? (size_t)b->nz + 2 * (size_t)b->g : 1);
}

/* velsrc%tmp: the diffusion, interface-viscosity, gravity and surface-tension
 * terms (sec_part1 + sec_part2 + sec_part3, NO2 ns_ab_diff.f90:10-135, NO3
 * :10-199) from the old fields.  The surface-tension term is added only when
 * btn_sf != 0 (the reference computes the curvature only then, ns_solvers.f90
 * ns_init); nrm and curv may be NULL otherwise. */
void or_ns_diffusion(const or_grid* gr, const or_ns_params* prm, const double* U, const double* V,
                     const double* W, const double* R, const double* M, const double* D,
                     const double* P, const double* N1, const double* N2, const double* N3,
                     const double* CV, double* TU, double* TV, double* TW) {
  const ns_box b = ns_box_of(gr, prm->ghost);
  const int three = gr->nz > 1;
  const double dx = gr->dx, dy = gr->dy, dz = gr->dz;
  const double dx2 = dx * dx, dy2 = dy * dy, dz2 = dz * dz;
  const double re = prm->re, c1 = 1.0 - prm->mu_12;
  const int sf = prm->btn_sf != 0.0;
  const size_t sx = 1, sy = b.px, sz = b.px * b.py;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 1; k <= gr->nz; ++k)
    for (int j = 1; j <= gr->ny; ++j)
      for (int i = 1; i <= gr->nx; ++i) {
        const size_t q = NI(&b, i, j, k);
        double rho, mu, delta, curv, xx, yy, zz, t;
        double ux, uy, uz, vx, vy, vz, wx, wy, wz, phix, phiy, phiz, dxx, dyy, dzz;
        /* ---- x: u at (i+1/2, j, k) ---- */
        rho = 0.5 * (R[q] + R[q + sx]);
        mu = 0.5 * (M[q] + M[q + sx]);
        xx = ((U[q + sx] - 2.0 * U[q]) + U[q - sx]) / dx2;
        yy = ((U[q + sy] - 2.0 * U[q]) + U[q - sy]) / dy2;
        t = ((mu / rho) * xx) / re + ((mu / rho) * yy) / re;
        if (three) {
          zz = ((U[q + sz] - 2.0 * U[q]) + U[q - sz]) / dz2;
          t = t + ((mu / rho) * zz) / re;
        }
        delta = 0.5 * (D[q] + D[q + sx]);
        ux = 0.5 * (U[q + sx] - U[q - sx]) / dx;
        uy = 0.5 * (U[q + sy] - U[q - sy]) / dy;
        vx = 0.5 * (((V[q + sx] - V[q]) + V[q + sx - sy]) - V[q - sy]) / dx;
        phix = (P[q + sx] - P[q]) / dx;
        phiy = 0.25 * (((P[q + sx + sy] - P[q + sx - sy]) + P[q + sy]) - P[q - sy]) / dy;
        dxx = c1 * delta * phix * 2.0 * ux / (rho * re);
        dyy = c1 * delta * phiy * (uy + vx) / (rho * re);
        t = (t + dxx) + dyy;
        if (three) {
          uz = 0.5 * (U[q + sz] - U[q - sz]) / dz;
          wx = 0.5 * (((W[q + sx] - W[q]) + W[q + sx - sz]) - W[q - sz]) / dx;
          phiz = 0.25 * (((P[q + sx + sz] - P[q + sx - sz]) + P[q + sz]) - P[q - sz]) / dz;
          dzz = c1 * delta * phiz * (uz + wx) / (rho * re);
          t = t + dzz;
        }
        t = t + prm->gx * prm->btn_g / prm->fr;
        if (sf) {
          curv = (CV[q] + CV[q + sx]) / 2.0;
          phix = 0.5 * (N1[q] + N1[q + sx]);
          t = t - prm->btn_sf * curv * delta * phix / (prm->we * rho);
        }
        TU[q] = t;
        /* ---- y: v at (i, j+1/2, k) ---- */
        rho = 0.5 * (R[q] + R[q + sy]);
        mu = 0.5 * (M[q] + M[q + sy]);
        xx = ((V[q + sx] - 2.0 * V[q]) + V[q - sx]) / dx2;
        yy = ((V[q + sy] - 2.0 * V[q]) + V[q - sy]) / dy2;
        t = ((mu / rho) * xx) / re + ((mu / rho) * yy) / re;
        if (three) {
          zz = ((V[q + sz] - 2.0 * V[q]) + V[q - sz]) / dz2;
          t = t + ((mu / rho) * zz) / re;
        }
        delta = 0.5 * (D[q] + D[q + sy]);
        vx = 0.5 * (V[q + sx] - V[q - sx]) / dx;
        vy = 0.5 * (V[q + sy] - V[q - sy]) / dy;
        uy = 0.5 * (((U[q + sy] - U[q]) + U[q - sx + sy]) - U[q - sx]) / dy;
        phix = 0.25 * (((P[q + sx] - P[q - sx]) + P[q + sx + sy]) - P[q - sx + sy]) / dx;
        phiy = (P[q + sy] - P[q]) / dy;
        dxx = c1 * delta * phix * (uy + vx) / (rho * re);
        dyy = c1 * delta * phiy * 2.0 * vy / (rho * re);
        t = (t + dxx) + dyy;
        if (three) {
          vz = 0.5 * (V[q + sz] - V[q - sz]) / dz;
          wy = 0.5 * (((W[q + sy] - W[q]) + W[q + sy - sz]) - W[q - sz]) / dy;
          phiz = 0.25 * (((P[q + sy + sz] - P[q + sy - sz]) + P[q + sz]) - P[q - sz]) / dz;
          dzz = c1 * delta * phiz * (wy + vz) / (rho * re);
          t = t + dzz;
        }
        t = t + prm->gy * prm->btn_g / prm->fr;
        if (sf) {
          curv = (CV[q] + CV[q + sy]) / 2.0;
          phiy = 0.5 * (N2[q] + N2[q + sy]);
          t = t - prm->btn_sf * curv * delta * phiy / (prm->we * rho);
        }
        TV[q] = t;
        if (!three) continue;
        /* ---- z: w at (i, j, k+1/2) ---- */
        rho = 0.5 * (R[q] + R[q + sz]);
        mu = 0.5 * (M[q] + M[q + sz]);
        xx = ((W[q + sx] - 2.0 * W[q]) + W[q - sx]) / dx2;
        yy = ((W[q + sy] - 2.0 * W[q]) + W[q - sy]) / dy2;
        zz = ((W[q + sz] - 2.0 * W[q]) + W[q - sz]) / dz2;
        t = (((mu / rho) * xx) / re + ((mu / rho) * yy) / re) + ((mu / rho) * zz) / re;
        delta = 0.5 * (D[q] + D[q + sz]);
        wx = 0.5 * (W[q + sx] - W[q - sx]) / dx;
        wy = 0.5 * (W[q + sy] - W[q - sy]) / dy;
        wz = 0.5 * (W[q + sz] - W[q - sz]) / dz;
        uz = 0.5 * (((U[q + sz] - U[q]) + U[q - sx + sz]) - U[q - sx]) / dz;
        vz = 0.5 * (((V[q + sz] - V[q]) + V[q - sy + sz]) - V[q - sy]) / dz;
        phix = 0.25 * (((P[q + sx + sz] - P[q - sx + sz]) + P[q + sx]) - P[q - sx]) / dx;
        phiy = 0.25 * (((P[q + sy + sz] - P[q - sy + sz]) + P[q + sy]) - P[q - sy]) / dy;
        phiz = (P[q + sz] - P[q]) / dz;
        dxx = c1 * delta * phix * (uz + wx) / (rho * re);
        dyy = c1 * delta * phiy * (vz + wy) / (rho * re);
        dzz = c1 * delta * phiz * 2.0 * wz / (rho * re);
        t = ((t + dxx) + dyy) + dzz;
        t = t + prm->gz * prm->btn_g / prm->fr;
        if (sf) {
          curv = (CV[q] + CV[q + sz]) / 2.0;
          phiz = 0.5 * (N3[q] + N3[q + sz]);
          t = t - prm->btn_sf * curv * delta * phiz / (prm->we * rho);
        }
        TW[q] = t;
      }
}

/* One predictor pass after ns_linearize (vel%tmp = the advecting velocity Ut,
 * Vt, Wt): find_stag_vel's four-point averages of the other components at
 * each face (bcs.f90), the second-order upwind advection of the old velocity
 * (ns_ab_adv_source_sec, NO2 ns_ab_adv.f90:1-42, NO3 :1-73),
 * velsrc%now = advection + velsrc%tmp (ns_ab_setup) and the AB2 predictor
 * vel%now = vel%old + dt (1.5 velsrc%now - 0.5 velsrc%old) (ns_ab_predictor)
 * over the reference's interior loops i = 1..nx etc. (which include the high
 * wall face; velbc zeroes it).  Ghosts are not written. */
static inline double ns_upwind(double a, double m, double p) {
  return (a + fabs(a)) * m + (a - fabs(a)) * p;
}

void or_ns_advance(const or_grid* gr, const or_ns_params* prm, const double* U, const double* V,
                   const double* W, const double* Ut, const double* Vt, const double* Wt,
                   const double* TU, const double* TV, const double* TW, const double* SUo,
                   const double* SVo, const double* SWo, double* SU, double* SV, double* SW,
                   double* Un, double* Vn, double* Wn) {
  const ns_box b = ns_box_of(gr, prm->ghost);
  const int three = gr->nz > 1;
  const double dx = gr->dx, dy = gr->dy, dz = gr->dz, dt = prm->dt;
  const size_t sx = 1, sy = b.px, sz = b.px * b.py;
  const double* F[3] = {U, V, W};
  double* S[3] = {SU, SV, SW};
  double* O[3] = {Un, Vn, Wn};
  const double* T[3] = {TU, TV, TW};
  const double* SO[3] = {SUo, SVo, SWo};
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 1; k <= gr->nz; ++k)
    for (int j = 1; j <= gr->ny; ++j)
      for (int i = 1; i <= gr->nx; ++i) {
        const size_t q = NI(&b, i, j, k);
        for (int c = 0; c < (three ? 3 : 2); ++c) {
          double a[3];
          if (c == 0) {
            a[0] = Ut[q];
            a[1] = 0.25 * (((Vt[q] + Vt[q - sy]) + Vt[q + sx]) + Vt[q + sx - sy]);
            if (three) a[2] = 0.25 * (((Wt[q] + Wt[q - sz]) + Wt[q + sx]) + Wt[q + sx - sz]);
          } else if (c == 1) {
            a[0] = 0.25 * (((Ut[q] + Ut[q - sx]) + Ut[q + sy]) + Ut[q - sx + sy]);
            a[1] = Vt[q];
            if (three) a[2] = 0.25 * (((Wt[q] + Wt[q - sz]) + Wt[q + sy]) + Wt[q + sy - sz]);
          } else {
            a[0] = 0.25 * (((Ut[q] + Ut[q - sx]) + Ut[q + sz]) + Ut[q - sx + sz]);
            a[1] = 0.25 * (((Vt[q] + Vt[q - sy]) + Vt[q + sz]) + Vt[q - sy + sz]);
            a[2] = Wt[q];
          }
          const double* f = F[c];
          const size_t st[3] = {sx, sy, sz};
          const double h[3] = {dx, dy, dz};
          double src = 0.0;
          if (prm->adv_scheme == 1) {
            /* ns_ab_adv_source_quick (NO2 ns_ab_adv.f90:44-114, NO3 :75-199) */
            const double* Tv[3] = {Ut, Vt, Wt};
            const size_t ec = st[c];
            for (int d = 0; d < (three ? 3 : 2); ++d) {
              const size_t s = st[d];
              double sv[2], ah = 0.0;
              for (int m = 0; m < 2; ++m) { /* positions q - e_d (m = 0) and q (m = 1) */
                const size_t pq = m == 0 ? q - s : q;
                const double av = 0.5 * (Tv[d][pq] + Tv[d][pq + ec]);
                sv[m] = av >= 0.0 ? ((-f[pq - s] + 6.0 * f[pq]) + 3.0 * f[pq + s]) / 8.0
                                  : ((-f[pq + 2 * s] + 6.0 * f[pq + s]) + 3.0 * f[pq]) / 8.0;
                if (m == 1) ah = av;
              }
              const double term = ah * (sv[1] - sv[0]) / h[d];
              src = d == 0 ? -term : src - term;
            }
          } else {
            for (int d = 0; d < (three ? 3 : 2); ++d) {
              const size_t s = st[d];
              const double fp = 0.5 * ((-f[q + 2 * s] + 4.0 * f[q + s]) - 3.0 * f[q]) / h[d];
              const double fm = 0.5 * ((f[q - 2 * s] - 4.0 * f[q - s]) + 3.0 * f[q]) / h[d];
              const double term = ns_upwind(a[d], fm, fp) / 2.0;
              src = d == 0 ? -term : src - term;
            }
          }
          src = src + T[c][q];
          S[c][q] = src;
          O[c][q] = F[c][q] + dt * (1.5 * src - 0.5 * SO[c][q]);
        }
      }
}

/* velbc (NO2 bcs.f90:28-148, NO3 :44-257): for each wall with bc 1 (no-slip)
 * or 2 (slip) the g ghost layers mirror the interior, negated for no-slip;
 * the normal component's wall face is set to 0.  Passes in the reference's
 * order: x (low, high), then y, then z, each over the whole padded extent of
 * the other axes.  Other bc values leave that wall's ghosts. */
void or_velbc(const or_grid* gr, int g, const int32_t bc[6], double* U, double* V, double* W) {
  const ns_box b = ns_box_of(gr, g);
  const int three = gr->nz > 1;
  const int nx = gr->nx, ny = gr->ny, nz = gr->nz;
  const int k0 = three ? 1 - g : 1, k1 = three ? nz + g : 1;
  double* F[3] = {U, V, W};
  const int nc = three ? 3 : 2;
  /* x */
  for (int side = 0; side < 2; ++side) {
    const int t = bc[side];
    if (t != 1 && t != 2) continue;
    for (int k = k0; k <= k1; ++k)
      for (int j = 1 - g; j <= ny + g; ++j) {
        for (int m = 1; m <= g; ++m)
          for (int c = 0; c < nc; ++c) {
            double* f = F[c];
            if (side == 0) {
              const int src = c == 0 ? 1 - 2 + m : 1 - 1 + m;
              const double v = f[NI(&b, src, j, k)];
              f[NI(&b, 1 - m, j, k)] = t == 1 ? -v : v;
            } else {
              const int src = c == 0 ? nx - m : nx + 1 - m;
              const double v = f[NI(&b, src, j, k)];
              f[NI(&b, nx + m, j, k)] = t == 1 ? -v : v;
            }
          }
        U[NI(&b, side == 0 ? 0 : nx, j, k)] = 0.0;
      }
  }
  /* y */
  for (int side = 0; side < 2; ++side) {
    const int t = bc[2 + side];
    if (t != 1 && t != 2) continue;
    for (int k = k0; k <= k1; ++k)
      for (int i = 1 - g; i <= nx + g; ++i) {
        for (int m = 1; m <= g; ++m)
          for (int c = 0; c < nc; ++c) {
            double* f = F[c];
            if (side == 0) {
              const int src = c == 1 ? 1 - 2 + m : 1 - 1 + m;
              const double v = f[NI(&b, i, src, k)];
              f[NI(&b, i, 1 - m, k)] = t == 1 ? -v : v;
            } else {
              const int src = c == 1 ? ny - m : ny + 1 - m;
              const double v = f[NI(&b, i, src, k)];
              f[NI(&b, i, ny + m, k)] = t == 1 ? -v : v;
            }
          }
        V[NI(&b, i, side == 0 ? 0 : ny, k)] = 0.0;
      }
  }
  if (!three) return;
  /* z */
  for (int side = 0; side < 2; ++side) {
    const int t = bc[4 + side];
    if (t != 1 && t != 2) continue;
    for (int j = 1 - g; j <= ny + g; ++j)
      for (int i = 1 - g; i <= nx + g; ++i) {
        for (int m = 1; m <= g; ++m)
          for (int c = 0; c < 3; ++c) {
            double* f = F[c];
            if (side == 0) {
              const int src = c == 2 ? 1 - 2 + m : 1 - 1 + m;
              const double v = f[NI(&b, i, j, src)];
              f[NI(&b, i, j, 1 - m)] = t == 1 ? -v : v;
            } else {
              const int src = c == 2 ? nz - m : nz + 1 - m;
              const double v = f[NI(&b, i, j, src)];
              f[NI(&b, i, j, nz + m)] = t == 1 ? -v : v;
            }
          }
        W[NI(&b, i, j, side == 0 ? 0 : nz)] = 0.0;
      }
  }
}

/* linf and l2f of vel%now - vel%tmp over the interior loops
 * (ns_check_convergence_vel, NO2 ns_solvers.f90:85-115, NO3 :92-126):
 * l2f = sqrt(sum / (2 nx ny)) in 2D, sqrt(sum / (3 nx ny nz)) in 3D. */
void or_ns_vel_change(const or_grid* gr, int g, const double* Un, const double* Vn,
                      const double* Wn, const double* Ut, const double* Vt, const double* Wt,
                      double* linf, double* l2f) {
  const ns_box b = ns_box_of(gr, g);
  const int three = gr->nz > 1;
  double mx = 0.0, s = 0.0;
  for (int k = 1; k <= gr->nz; ++k)
    for (int j = 1; j <= gr->ny; ++j)
      for (int i = 1; i <= gr->nx; ++i) {
        const size_t q = NI(&b, i, j, k);
        const double du = Un[q] - Ut[q], dv = Vn[q] - Vt[q];
        mx = fmax(mx, fabs(du));
        mx = fmax(mx, fabs(dv));
        if (three) mx = fmax(mx, fabs(Wn[q] - Wt[q]));
        s = s + du * du;
        s = s + dv * dv;
        if (three) s = s + (Wn[q] - Wt[q]) * (Wn[q] - Wt[q]);
      }
  *linf = mx;
  *l2f = three ? sqrt(s / (3.0 * gr->nx * gr->ny * gr->nz)) : sqrt(s / (2.0 * gr->nx * gr->ny));
}

/* The pressure step inside the loop: ppe_sor_solver + ns_momentum_correction
 * on the padded velocity (faces 0..n of each axis), with the multigrid of this
 * file in place of the point relaxation; then velbc. */
static int ns_project(const or_grid* gr, const or_ns_params* prm, const double* rho,
                      const double* cx, const double* cy, const double* cz, double* Un, double* Vn,
                      double* Wn, double* p, const or_mg_params* mgp, or_mg_stats* st) {
  const ns_box b = ns_box_of(gr, prm->ghost);
  const int three = gr->nz > 1;
  const int nx = gr->nx, ny = gr->ny, nz = gr->nz;
  const size_t n = cells_of(nx, ny, nz);
  double* u = dalloc((size_t)(nx + 1) * ny * nz);
  double* v = dalloc((size_t)nx * (ny + 1) * nz);
  double* w = three ? dalloc((size_t)nx * ny * (nz + 1)) : NULL;
  double* rhs = dalloc(n);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int f = 0; f <= nx; ++f) u[((size_t)k * ny + j) * (nx + 1) + f] = Un[NI(&b, f, j + 1, k + 1)];
  for (int k = 0; k < nz; ++k)
    for (int f = 0; f <= ny; ++f)
      for (int i = 0; i < nx; ++i) v[((size_t)k * (ny + 1) + f) * nx + i] = Vn[NI(&b, i + 1, f, k + 1)];
  if (three)
    for (int f = 0; f <= nz; ++f)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) w[((size_t)f * ny + j) * nx + i] = Wn[NI(&b, i + 1, j + 1, f)];
  or_divergence(gr, u, v, w, prm->dt, 1, rhs);
  const int rc = or_mg_solve(gr, cx, cy, cz, rhs, p, prm->p_tol, mgp, st);
  or_correct(gr, rho, p, prm->dt, u, v, w);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int f = 1; f < nx; ++f) Un[NI(&b, f, j + 1, k + 1)] = u[((size_t)k * ny + j) * (nx + 1) + f];
  for (int k = 0; k < nz; ++k)
    for (int f = 1; f < ny; ++f)
      for (int i = 0; i < nx; ++i) Vn[NI(&b, i + 1, f, k + 1)] = v[((size_t)k * (ny + 1) + f) * nx + i];
  if (three)
    for (int f = 1; f < nz; ++f)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) Wn[NI(&b, i + 1, j + 1, f)] = w[((size_t)f * ny + j) * nx + i];
  free(u);
  free(v);
  free(w);
  free(rhs);
  or_velbc(gr, prm->ghost, prm->bc, Un, Vn, Wn);
  return rc;
}

/* ns_ab_solver_SOR after ppe_sor_init (NO2 admas_bashforth_solver.f90:40-67, NO3 :43-70):
 * velsrc%tmp once (it depends on the old fields only), then `iterations`
 * passes of ns_linearize, ns_ab_setup, ns_ab_predictor (+ velbc) and the
 * pressure step, then ns_check_convergence_vel.  rho is the new cell density
 * (compact) of the pressure operator; p the compact pressure (warm start in,
 * result out); the velocity, source and old fields are padded.  Returns the
 * worst solve status; cycles (may be NULL) receives the total cycles. */
int or_ns_ab_step(const or_grid* gr, const or_ns_params* prm, const double* rho, double* Un,
                  double* Vn, double* Wn, const double* U, const double* V, const double* W,
                  double* SU, double* SV, double* SW, const double* SUo, const double* SVo,
                  const double* SWo, const double* R, const double* M, const double* D,
                  const double* P, const double* N1, const double* N2, const double* N3,
                  const double* CV, double* p, const or_mg_params* mgp, double* linf,
                  double* l2f, int32_t* cycles) {
  const ns_box b = ns_box_of(gr, prm->ghost);
  const int three = gr->nz > 1;
  const size_t span = ns_span(&b), n = cells_of(gr->nx, gr->ny, gr->nz);
  double* T[3] = {dalloc(span), dalloc(span), three ? dalloc(span) : NULL};
  double* Tm[3] = {dalloc(span), dalloc(span), three ? dalloc(span) : NULL};
  double* cx = dalloc(n);
  double* cy = dalloc(n);
  double* cz = dalloc(n);
  or_face_coef(gr, rho, cx, cy, cz);
  or_ns_diffusion(gr, prm, U, V, W, R, M, D, P, N1, N2, N3, CV, T[0], T[1], T[2]);
  double* Nw[3] = {Un, Vn, Wn};
  int worst = OR_OK, total = 0;
  for (int it = 0; it < prm->iterations; ++it) {
    for (int c = 0; c < (three ? 3 : 2); ++c) memcpy(Tm[c], Nw[c], span * sizeof(double));
    or_ns_advance(gr, prm, U, V, W, Tm[0], Tm[1], Tm[2], T[0], T[1], T[2], SUo, SVo, SWo, SU, SV,
                  SW, Un, Vn, Wn);
    or_velbc(gr, prm->ghost, prm->bc, Un, Vn, Wn);
    or_mg_stats st;
    const int rc = ns_project(gr, prm, rho, cx, cy, cz, Un, Vn, Wn, p, mgp, &st);
    total += st.cycles;
    if (rc > worst) worst = rc;
  }
  or_ns_vel_change(gr, prm->ghost, Un, Vn, Wn, Tm[0], Tm[1], Tm[2], linf, l2f);
  if (cycles) *cycles = total;
  for (int c = 0; c < 3; ++c) {
    free(T[c]);
    free(Tm[c]);
  }
  free(cx);
  free(cy);
  free(cz);
  return worst;
}

/* ------------------------------------------------------------------------- */
/* Interface normals and curvature from combined compact differences          */
/* (curv + surface_norms, NO2 src/interface_solver/others_normals.f90:1-103,   */
/* NO3 :1-166; the "ccd" scheme of NO2 lib/solver/ccd_solvers.f90:76-159,     */
/* 287-306, 379-399 with TWIN_DEC / TWIN_BKS of lib/solver/matrix_solver.f90). */
/* Every line of the padded box (g ghosts each side, L = n + 2g points) is    */
/* one 2x2-block tridiagonal system for (f', f''); the matrix depends only on */
/* L and h, so it is decomposed once per axis.  dx**2.0d0 is dx*dx (a real    */
/* exponent of integral value is an integer power in gfortran).               */
/* ------------------------------------------------------------------------- */
/* A, B, AA, BB: 3 x L each, row r (1..3 in the reference) at [(r-1)*L + i]. */
void or_ccd_decompose(int L, double h, double* A, double* B, double* AA, double* BB) {
#define M_(X, r, i) X[((r) - 1) * L + (i)]
  const int is = 0, ie = L - 1;
  /* working_matrix_bc */
  M_(A, 2, is) = 1.0; M_(B, 2, is) = 0.0; M_(AA, 2, is) = 0.0; M_(BB, 2, is) = 1.0;
  M_(A, 3, is) = 2.0; M_(B, 3, is) = -h; M_(AA, 3, is) = -(2.5 / h); M_(BB, 3, is) = 8.5;
  M_(A, 2, ie) = 1.0; M_(B, 2, ie) = 0.0; M_(AA, 2, ie) = 0.0; M_(BB, 2, ie) = 1.0;
  M_(A, 1, ie) = 2.0; M_(B, 1, ie) = h; M_(AA, 1, ie) = 2.5 / h; M_(BB, 1, ie) = 8.5;
  /* working_matrix_init_ccd */
  for (int i = is + 1; i <= ie - 1; ++i) {
    M_(A, 1, i) = 7.0 / 16.0; M_(A, 2, i) = 1.0; M_(A, 3, i) = 7.0 / 16.0;
    M_(B, 1, i) = h / 16.0; M_(B, 2, i) = 0.0; M_(B, 3, i) = -(h / 16.0);
    M_(AA, 1, i) = -(9.0 / 8.0 / h); M_(AA, 2, i) = 0.0; M_(AA, 3, i) = 9.0 / 8.0 / h;
    M_(BB, 1, i) = -(1.0 / 8.0); M_(BB, 2, i) = 1.0; M_(BB, 3, i) = -(1.0 / 8.0);
  }
  /* TWIN_DEC */
  M_(A, 1, is) = 0.0; M_(AA, 1, is) = 0.0; M_(A, 3, ie) = 0.0; M_(AA, 3, ie) = 0.0;
  M_(B, 1, is) = 0.0; M_(BB, 1, is) = 0.0; M_(B, 3, ie) = 0.0; M_(BB, 3, ie) = 0.0;
  for (int i = is + 1; i <= ie; ++i) {
    const double den = M_(A, 2, i - 1) * M_(BB, 2, i - 1) - M_(AA, 2, i - 1) * M_(B, 2, i - 1);
    double sc1 = -((M_(AA, 2, i - 1) * M_(B, 1, i) - M_(A, 1, i) * M_(BB, 2, i - 1)) / den);
    double sc2 = (M_(B, 1, i) * M_(A, 2, i - 1) - M_(B, 2, i - 1) * M_(A, 1, i)) / den;
    M_(A, 1, i) = sc1;
    M_(A, 2, i) = M_(A, 2, i) - (sc1 * M_(A, 3, i - 1) + sc2 * M_(AA, 3, i - 1));
    M_(B, 1, i) = sc2;
    M_(B, 2, i) = M_(B, 2, i) - (sc1 * M_(B, 3, i - 1) + sc2 * M_(BB, 3, i - 1));
    sc1 = -((M_(AA, 2, i - 1) * M_(BB, 1, i) - M_(AA, 1, i) * M_(BB, 2, i - 1)) / den);
    sc2 = (M_(BB, 1, i) * M_(A, 2, i - 1) - M_(B, 2, i - 1) * M_(AA, 1, i)) / den;
    M_(AA, 1, i) = sc1;
    M_(AA, 2, i) = M_(AA, 2, i) - (sc1 * M_(A, 3, i - 1) + sc2 * M_(AA, 3, i - 1));
    M_(BB, 1, i) = sc2;
    M_(BB, 2, i) = M_(BB, 2, i) - (sc1 * M_(B, 3, i - 1) + sc2 * M_(BB, 3, i - 1));
  }
#undef M_
}

/* One line: f at f[i*sf], i = 0..L-1, into fx, fxx at [i*so]
 * (working_matrix_asgn_src_ccd, then TWIN_BKS). */
void or_ccd_line(int L, double h, const double* A, const double* B, const double* AA,
                 const double* BB, const double* f, int64_t sf, double* S, double* SS,
                 int64_t so) {
#define M_(X, r, i) X[((r) - 1) * L + (i)]
#define F(i) f[(int64_t)(i) * sf]
#define S_(i) S[(int64_t)(i) * so]
#define SS_(i) SS[(int64_t)(i) * so]
  const int is = 0, ie = L - 1;
  const double h2 = h * h;
  S_(is) = ((-3.5 * F(is) + 4.0 * F(is + 1)) - 0.5 * F(is + 2)) / h;
  SS_(is) = (((34.0 / 3.0 * F(is) - 83.0 / 4.0 * F(is + 1)) + 10.0 * F(is + 2)) -
             7.0 / 12.0 * F(is + 3)) / h2;
  for (int i = is + 1; i <= ie - 1; ++i) {
    S_(i) = 15.0 / 16.0 * (-F(i - 1) + F(i + 1)) / h;
    SS_(i) = ((3.0 * F(i - 1) - 6.0 * F(i)) + 3.0 * F(i + 1)) / h2;
  }
  S_(ie) = -(((-3.5 * F(ie) + 4.0 * F(ie - 1)) - 0.5 * F(ie - 2)) / h);
  SS_(ie) = (((34.0 / 3.0 * F(ie) - 83.0 / 4.0 * F(ie - 1)) + 10.0 * F(ie - 2)) -
             7.0 / 12.0 * F(ie - 3)) / h2;
  /* TWIN_BKS */
  for (int i = is + 1; i <= ie; ++i) {
    const double sp = S_(i - 1), ssp = SS_(i - 1);
    S_(i) = S_(i) - (M_(A, 1, i) * sp + M_(B, 1, i) * ssp);
    SS_(i) = SS_(i) - (M_(AA, 1, i) * sp + M_(BB, 1, i) * ssp);
  }
  double den = M_(A, 2, ie) * M_(BB, 2, ie) - M_(AA, 2, ie) * M_(B, 2, ie);
  double sol = -((M_(B, 2, ie) * SS_(ie) - M_(BB, 2, ie) * S_(ie)) / den);
  double sol2 = (M_(A, 2, ie) * SS_(ie) - M_(AA, 2, ie) * S_(ie)) / den;
  S_(ie) = sol;
  SS_(ie) = sol2;
  for (int i = ie - 1; i >= is; --i) {
    S_(i) = S_(i) - (M_(A, 3, i) * sol + M_(B, 3, i) * sol2);
    SS_(i) = SS_(i) - (M_(AA, 3, i) * sol + M_(BB, 3, i) * sol2);
    den = M_(A, 2, i) * M_(BB, 2, i) - M_(AA, 2, i) * M_(B, 2, i);
    sol = -((M_(B, 2, i) * SS_(i) - M_(BB, 2, i) * S_(i)) / den);
    sol2 = (M_(A, 2, i) * SS_(i) - M_(AA, 2, i) * S_(i)) / den;
    S_(i) = sol;
    SS_(i) = sol2;
  }
#undef M_
#undef F
#undef S_
#undef SS_
}

/* all lines along one axis of the padded box */
static void ccd_axis(const ns_box* b, int axis, double h, const double* f, double* fx,
                     double* fxx) {
  const int three = b->nz > 1;
  const size_t px = b->px, py = b->py, pz = three ? (size_t)b->nz + 2 * (size_t)b->g : 1;
  const size_t ext[3] = {px, py, pz};
  const int64_t st[3] = {1, (int64_t)px, (int64_t)(px * py)};
  const int L = (int)ext[axis];
  double* A = dalloc(3 * (size_t)L);
  double* B = dalloc(3 * (size_t)L);
  double* AA = dalloc(3 * (size_t)L);
  double* BB = dalloc(3 * (size_t)L);
  or_ccd_decompose(L, h, A, B, AA, BB);
  const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
  const size_t n1 = ext[a1], n2 = ext[a2];
#pragma omp parallel for collapse(2) schedule(static)
  for (size_t i2 = 0; i2 < n2; ++i2)
    for (size_t i1 = 0; i1 < n1; ++i1) {
      const size_t base = i1 * (size_t)st[a1] + i2 * (size_t)st[a2];
      or_ccd_line(L, h, A, B, AA, BB, f + base, st[axis], fx + base, fxx + base, st[axis]);
    }
  free(A);
  free(B);
  free(AA);
  free(BB);
}

/* bc (NO2 src/others/bcs.f90:1-26, NO3 :1-42): zero-gradient copies of the
 * boundary values into the ghosts, x then y then z passes. */
void or_ns_bc(const or_grid* gr, int g, double* a) {
  const ns_box b = ns_box_of(gr, g);
  const int three = gr->nz > 1;
  const int k0 = three ? 1 - g : 1, k1 = three ? gr->nz + g : 1;
  for (int k = k0; k <= k1; ++k)
    for (int j = 1 - g; j <= gr->ny + g; ++j)
      for (int m = 1; m <= g; ++m) {
        a[NI(&b, 1 - m, j, k)] = a[NI(&b, 1, j, k)];
        a[NI(&b, gr->nx + m, j, k)] = a[NI(&b, gr->nx, j, k)];
      }
  for (int k = k0; k <= k1; ++k)
    for (int i = 1 - g; i <= gr->nx + g; ++i)
      for (int m = 1; m <= g; ++m) {
        a[NI(&b, i, 1 - m, k)] = a[NI(&b, i, 1, k)];
        a[NI(&b, i, gr->ny + m, k)] = a[NI(&b, i, gr->ny, k)];
      }
  if (!three) return;
  for (int j = 1 - g; j <= gr->ny + g; ++j)
    for (int i = 1 - g; i <= gr->nx + g; ++i)
      for (int m = 1; m <= g; ++m) {
        a[NI(&b, i, j, 1 - m)] = a[NI(&b, i, j, 1)];
        a[NI(&b, i, j, gr->nz + m)] = a[NI(&b, i, j, gr->nz)];
      }
}

/* curv: the derivatives of phi by compact lines (x, y, z of phi; y of phi_x,
 * z of phi_x and of phi_y), bc on each, then on the interior
 *   2D  curv = (fyy fx^2 + fxx fy^2 - 2 fxy fx fy) / (fx^2 + fy^2 + 1e-12)^1.5
 *   3D  curv = ((fyy+fzz) fx^2 + (fxx+fzz) fy^2 + (fxx+fyy) fz^2
 *               - 2 (fxy fx fy + fxz fx fz + fyz fy fz)) / (|grad phi|^2 + 1e-12)^1.5
 * and bc.  nx, ny, nz receive phi_x, phi_y, phi_z (the reference's normals%x..z,
 * not normalised); d2 (may be NULL) receives fxx, fyy, fzz, fxy, fxz, fyz,
 * six padded arrays one after another. */
void or_ns_curvature(const or_grid* gr, int g, const double* phi, double* nx, double* ny,
                     double* nz, double* curv, double* d2) {
  const ns_box b = ns_box_of(gr, g);
  const int three = gr->nz > 1;
  const size_t span = ns_span(&b);
  double* own = d2 ? NULL : dalloc(6 * span);
  double* D = d2 ? d2 : own;
  double *fxx = D, *fyy = D + span, *fzz = D + 2 * span, *fxy = D + 3 * span,
         *fxz = D + 4 * span, *fyz = D + 5 * span;
  double* dummy = dalloc(span);
  ccd_axis(&b, 0, gr->dx, phi, nx, fxx);
  ccd_axis(&b, 1, gr->dy, phi, ny, fyy);
  if (three) ccd_axis(&b, 2, gr->dz, phi, nz, fzz);
  ccd_axis(&b, 1, gr->dy, nx, fxy, dummy);
  if (three) {
    ccd_axis(&b, 2, gr->dz, nx, fxz, dummy);
    ccd_axis(&b, 2, gr->dz, ny, fyz, dummy);
  }
  double* bcs[9] = {nx, fxx, ny, fyy, nz, fzz, fxy, fxz, fyz};
  for (int a = 0; a < 9; ++a) {
    if (!three && (a == 4 || a == 5 || a == 7 || a == 8)) continue;
    or_ns_bc(gr, g, bcs[a]);
  }
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 1; k <= gr->nz; ++k)
    for (int j = 1; j <= gr->ny; ++j)
      for (int i = 1; i <= gr->nx; ++i) {
        const size_t q = NI(&b, i, j, k);
        const double fx = nx[q], fy = ny[q];
        if (!three) {
          const double num = (fyy[q] * (fx * fx) + fxx[q] * (fy * fy)) - 2.0 * fxy[q] * fx * fy;
          curv[q] = num / pow((fx * fx + fy * fy) + 1.0e-12, 1.5);
        } else {
          const double fz = nz[q];
          const double num = (((fyy[q] + fzz[q]) * (fx * fx) + (fxx[q] + fzz[q]) * (fy * fy)) +
                              (fxx[q] + fyy[q]) * (fz * fz)) -
                             2.0 * ((fxy[q] * fx * fy + fxz[q] * fx * fz) + fyz[q] * fy * fz);
          curv[q] = num / pow(((fx * fx + fy * fy) + fz * fz) + 1.0e-12, 1.5);
        }
      }
  or_ns_bc(gr, g, curv);
  free(own);
  free(dummy);
}

/* mass_preserving_level_set (NO2 src/interface_solver/
 * mass_preserving_level_set.f90:1-48, NO3 the same with dz): `iterations`
 * times ls_mv's mass (ls_mv, NO2 others.f90:63-113: sum (H + rho_12 (1-H)) H dv)
 * and surface_norms' compact gradient, then phi += lam delta |grad phi| with
 * lam = (imass - mass) / sum delta^2 |grad phi| (2 (1 - rho_12) H + rho_12) dv,
 * and bc.  Returns the mass measured last (iterations = 0: ls_mv only).  Sums
 * in loop order (the reference's OpenMP reductions have no fixed order). */
double or_ns_mass_correct(const or_grid* gr, int g, double* phi, double ls_wid, double rho_12,
                          double imass, int iterations) {
  const ns_box b = ns_box_of(gr, g);
  const int three = gr->nz > 1;
  const size_t span = ns_span(&b);
  const double pi = acos(-1.0);
  double* gx[3] = {dalloc(span), dalloc(span), three ? dalloc(span) : NULL};
  double* dummy = dalloc(span);
  const double dv = three ? gr->dx * gr->dy * gr->dz : gr->dx * gr->dy;
  double mass = 0.0;
  const int passes = iterations > 0 ? iterations : 1;
  for (int it = 0; it < passes; ++it) {
    const int correct = iterations > 0;
    if (correct) {
      ccd_axis(&b, 0, gr->dx, phi, gx[0], dummy);
      ccd_axis(&b, 1, gr->dy, phi, gx[1], dummy);
      if (three) ccd_axis(&b, 2, gr->dz, phi, gx[2], dummy);
    }
    double m = 0.0, den = 0.0;
    for (int k = 1; k <= gr->nz; ++k)
      for (int j = 1; j <= gr->ny; ++j)
        for (int i = 1; i <= gr->nx; ++i) {
          const size_t q = NI(&b, i, j, k);
          const double x = phi[q] / ls_wid;
          double heavy, delta;
          if (x > 1.0 - 1e-12) { heavy = 1.0; delta = 0.0; }
          else if (x < -1.0 + 1e-12) { heavy = 0.0; delta = 0.0; }
          else {
            heavy = 0.5 * (1.0 + x + sin(pi * x) / pi);
            delta = 0.5 * (1.0 + cos(pi * x)) / ls_wid;
          }
          heavy = fmax(fmin(heavy, 1.0), 0.0);
          const double rho = heavy + rho_12 * (1.0 - heavy);
          m = m + rho * heavy * dv;
          if (!correct) continue;
          const double g2 = three ? (gx[0][q] * gx[0][q] + gx[1][q] * gx[1][q]) + gx[2][q] * gx[2][q]
                                  : gx[0][q] * gx[0][q] + gx[1][q] * gx[1][q];
          double plam = delta * delta * sqrt(g2);
          plam = plam * (2.0 * (1.0 - rho_12) * heavy + rho_12) * gr->dx * gr->dy;
          if (three) plam = plam * gr->dz;
          den = den + plam;
        }
    mass = m;
    if (!correct) break;
    const double lam = (imass - m) / den;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k <= gr->nz; ++k)
      for (int j = 1; j <= gr->ny; ++j)
        for (int i = 1; i <= gr->nx; ++i) {
          const size_t q = NI(&b, i, j, k);
          const double x = phi[q] / ls_wid;
          double delta = 0.0;
          if (!(x > 1.0 - 1e-12) && !(x < -1.0 + 1e-12)) delta = 0.5 * (1.0 + cos(pi * x)) / ls_wid;
          const double g2 = three ? (gx[0][q] * gx[0][q] + gx[1][q] * gx[1][q]) + gx[2][q] * gx[2][q]
                                  : gx[0][q] * gx[0][q] + gx[1][q] * gx[1][q];
          phi[q] = phi[q] + lam * delta * sqrt(g2);
        }
    or_ns_bc(gr, g, phi);
  }
  for (int c = 0; c < 3; ++c) free(gx[c]);
  free(dummy);
  return mass;
}

/* ------------------------------------------------------------------------- */
/* CLSVOF's volume-fraction transport, vof_wlic_solver (NO2 src/interface_     */
/* solver/clsvof.f90:1-143; NO3 adds the z sweep): directional sweeps x, y(, z) */
/* of the WLIC flux (a THINC profile of slope beta = 2.3 weighted by the       */
/* normal's share |n_d|/|n|_1 against the upwind flux vof u dt), each followed */
/* by the cell update with the divergence correction vof_old dt du/dx and bc; */
/* after the last sweep vof is clipped to 0 below 1e-12 and 1 above 1 - 1e-12.  */
/* The normals are surface_norms2's central differences of phi (others_       */
/* normals.f90:47-74) with zero-gradient ghosts.  Padded arrays as the        */
/* momentum step's; u, v, w are vel%old.                                      */
/* ------------------------------------------------------------------------- */
static inline int clampn(int x, int n) { return x < 1 ? 1 : (x > n ? n : x); }

void or_vof_wlic(const or_grid* gr, int g, double* vof, const double* vof_old, const double* U,
                 const double* V, const double* W, const double* phi, double dt) {
  const ns_box b = ns_box_of(gr, g);
  const int three = gr->nz > 1;
  const int n[3] = {gr->nx, gr->ny, gr->nz};
  const double h[3] = {gr->dx, gr->dy, gr->dz};
  const double* vel[3] = {U, V, W};
  const double eps = 1.0e-12, beta = 2.3;
  const size_t span = ns_span(&b);
  double* flux = dalloc(span);
  for (int ax = 0; ax < (three ? 3 : 2); ++ax) {
    const double* uu = vel[ax];
    const int k0 = three ? 0 : 1;
    /* fluxes at faces 0..n of the axis, rows js-1..je (ks-1..ke) of the others */
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = k0; k <= gr->nz; ++k)
      for (int j = 0; j <= gr->ny; ++j)
        for (int i = 0; i <= gr->nx; ++i) {
          int ix[3] = {i, j, k};
          const size_t q = NI(&b, i, j, k);
          const double u = uu[q];
          int cc[3] = {i, j, k};
          double isgn;
          if (u > 0.0) { isgn = 1.0; } else { cc[ax] = ix[ax] + 1; isgn = 0.0; }
          const size_t qi = NI(&b, cc[0], cc[1], cc[2]);
          const double f = vof[qi];
          double l;
          if (f > 1.0 - eps || f < eps) {
            l = f * u * dt;
          } else {
            int cb[3] = {cc[0], cc[1], cc[2]}, cp[3] = {cc[0], cc[1], cc[2]};
            cb[ax] = cc[ax] - 1 < 1 ? 1 : cc[ax] - 1;
            cp[ax] = cc[ax] + 1;
            const double alpha = vof[NI(&b, cb[0], cb[1], cb[2])] < vof[NI(&b, cp[0], cp[1], cp[2])] ? 1.0 : -1.0;
            const double a1 = exp(beta * (2.0 * f - 1.0) / alpha);
            const double a3 = exp(beta);
            const double xc = 0.5 / beta * log((a3 * a3 - a1 * a3) / (a1 * a3 - 1.0));
            const double a4 = cosh(beta * ((isgn - u * dt / h[ax]) - xc));
            const double a5 = cosh(beta * (isgn - xc));
            /* surface_norms2 at the (zero-gradient clamped) upwind cell */
            const int c0 = clampn(cc[0], n[0]), c1 = clampn(cc[1], n[1]), c2 = three ? clampn(cc[2], n[2]) : 1;
            const size_t qc = NI(&b, c0, c1, c2);
            const size_t sy = b.px, sz = b.px * b.py;
            double nrm[3];
            nrm[0] = 0.5 * (phi[qc + 1] - phi[qc - 1]) / gr->dx;
            nrm[1] = 0.5 * (phi[qc + sy] - phi[qc - sy]) / gr->dy;
            nrm[2] = three ? 0.5 * (phi[qc + sz] - phi[qc - sz]) / gr->dz : 0.0;
            double w = three ? (fabs(nrm[0]) + fabs(nrm[1])) + fabs(nrm[2]) : fabs(nrm[0]) + fabs(nrm[1]);
            w = fabs(nrm[ax]) / w;
            l = 0.5 * (u * dt - alpha * h[ax] / beta * log(a4 / a5));
            l = l * w + (1.0 - w) * f * u * dt;
          }
          flux[q] = l;
        }
    const size_t st = ax == 0 ? 1 : (ax == 1 ? b.px : b.px * b.py);
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k <= gr->nz; ++k)
      for (int j = 1; j <= gr->ny; ++j)
        for (int i = 1; i <= gr->nx; ++i) {
          const size_t q = NI(&b, i, j, k);
          double f = vof[q] - (flux[q] - flux[q - st]) / h[ax] +
                     vof_old[q] * dt * (uu[q] - uu[q - st]) / h[ax];
          if (ax == (three ? 2 : 1)) {
            if (f < eps) f = 0.0;
            if (f > 1.0 - eps) f = 1.0;
          }
          vof[q] = f;
        }
    or_ns_bc(gr, g, vof);
  }
  free(flux);
}

/* ibm_bc's forcing (NO3 src/ns_solver/ns_solvers.f90:150-211) with a given
 * solid fraction: bc(solid), then u = (1 - s) u, v = (1 - s) v,
 * w = (1 - s) w + s w_body on the interior faces (s the face average; in 2D
 * v takes the body velocity). */
void or_ns_ibm(const or_grid* gr, int g, double* S, double w_body, double* U, double* V,
               double* W) {
  const ns_box b = ns_box_of(gr, g);
  const int three = gr->nz > 1;
  or_ns_bc(gr, g, S);
  const size_t sy = b.px, sz = b.px * b.py;
  for (int k = 1; k <= gr->nz; ++k)
    for (int j = 1; j <= gr->ny; ++j)
      for (int i = 1; i <= gr->nx; ++i) {
        const size_t q = NI(&b, i, j, k);
        double s = 0.5 * (S[q] + S[q + 1]);
        U[q] = (1.0 - s) * U[q];
        s = 0.5 * (S[q] + S[q + sy]);
        V[q] = three ? (1.0 - s) * V[q] : (1.0 - s) * V[q] + s * w_body;
        if (!three) continue;
        s = 0.5 * (S[q] + S[q + sz]);
        W[q] = (1.0 - s) * W[q] + s * w_body;
      }
}
