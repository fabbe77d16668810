/*
 * gbmg.h -- C ABI of the GB300 pressure-Poisson multigrid.
 *
 * Drop-in for the pressure routine of the reference's two-phase solvers
 * (ntu-d09525007/FortranCFD).  The reference has no C interface: its pressure
 * step is a set of Fortran subroutines over module state, called as
 *     call ppe_sor_init                      ("Two phase flows/newOpenMP/3D+IBM/
 *     call ppe_sor_solver(p%glb%p_tol)         src/ns_solver/admas_bashforth_solver.f90:50,62")
 * with ppe_sor_solver ending in ns_momentum_correction
 * ("Two phase flows/newOpenMP/3D+IBM/src/ns_solver/ns_ppe_solver.f90:1-205"),
 * or as CALL SOLVE_PRESSURE_POISSON() ("MPLS_RisingBubble/20190612/SOLVE_NS.F90:35").
 * Each entry point below names the routine it replaces.  Plain pointers and
 * sizes only; a Fortran host binds them with ISO_C_BINDING.
 *
 * Arrays.  Every array is a gbmg_field: the address of element (0,0,0) plus
 * the element strides of y and z; x is contiguous.  Cell arrays hold
 * nx*ny*nz interior cells.  Face velocities follow the reference's MAC layout:
 * u(f, j, k) is the x-face at x = f*dx for f = 0..nx (the reference's
 * u(i,j,k) on face i+1/2 with 1-based cells), v(i, f, k) with f = 0..ny,
 * w(i, j, f) with f = 0..nz.  A Fortran caller with ghost width g passes
 * c_loc(p(1,1,1)) with sy = nx+2g, sz = (nx+2g)*(ny+2g), and c_loc(u(0,1,1))
 * with the same strides.  Memory is host or device memory (GBMG_MEM_*).
 *
 * Operator: (A p)_i = sum over faces f of coe_f (p_nb - p_i), coe_f =
 * 2/(rho_i + rho_nb)/h^2, zero on walls (homogeneous Neumann, folded as in
 * ppe_sor_init).  The solve finds the mean-free p with A p = b to a relative
 * residual ||b - A p||_2/||b||_2 < tol (or the reference's own stopping rules,
 * gbmg_params.stop_rule).
 *
 * Errors never abort: every call returns a gbmg_status.  A solve that reaches
 * max_cycles returns GBMG_NOT_CONVERGED with the best iterate in p (the
 * reference STOPs the program instead, ns_ppe_solver.f90:154-157).
 * Threading: a handle is not re-entrant; use one handle per host thread.  All
 * work runs on the handle's stream and every call returns after it finished.
 */
#ifndef GBMG_H
#define GBMG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GBMG_OK = 0,
  GBMG_NOT_CONVERGED = 1,
  GBMG_DIVERGED = 2,
  GBMG_INVALID_ARG = 3,
  GBMG_CUDA_ERROR = 4,
  GBMG_NO_DEVICE = 5,
  GBMG_OUT_OF_MEMORY = 6,
  GBMG_STATE_ERROR = 7
} gbmg_status;

enum { GBMG_PREC_FP64 = 0, GBMG_PREC_MIXED = 1 };
/* When a solve stops (gbmg_params.stop_rule):
 *   GBMG_STOP_RELATIVE   ||b - A p||_2 / ||b||_2 < tol (the default);
 *   GBMG_STOP_RMS        sqrt(sum r^2 / n) < tol, the absolute RMS residual of
 *                        the reference's multigrid driver ppe_mg_solver, which
 *                        stops at l2norm < p_tol*0.001 ("DomainDecomposition/3D/
 *                        src/ns_solver/ns_ppe_mg_solver.f90:42-43"): pass
 *                        tol = p_tol*1e-3;
 *   GBMG_STOP_INCREMENT  max over the cells of |p_k - p_(k-1)| < tol between
 *                        successive V-cycles, the increment max-norm with which
 *                        ppe_sor_solver ("Two phase flows/newOpenMP/3D+IBM/src/
 *                        ns_solver/ns_ppe_solver.f90:143,152") and PRESS_POISSON
 *                        ("MPLS_RisingBubble/20190612/SOLVE_PRESSURE_POISSON.F90:
 *                        158-164") stop their sweeps: pass tol = p_tol.  The
 *                        reference measures it per SOR sweep, this library per
 *                        V-cycle.  Stationary cycles only (krylov = 0). */
enum { GBMG_STOP_RELATIVE = 0, GBMG_STOP_RMS = 1, GBMG_STOP_INCREMENT = 2 };
enum { GBMG_MEM_HOST = 0, GBMG_MEM_DEVICE = 1 };

typedef struct {
  int32_t nx, ny, nz; /* interior cells; nz = 1 for a 2D problem */
  double dx, dy, dz;  /* cell sizes (dz ignored when nz = 1) */
} gbmg_grid;

typedef struct {
  int32_t precision;       /* GBMG_PREC_FP64: FP64 V-cycles; GBMG_PREC_MIXED: FP32 V-cycles
                              inside FP64 defect correction */
  int32_t nu1, nu2;        /* red-black Gauss-Seidel sweeps before/after the coarse correction */
  int32_t levels;          /* 0 = automatic; else the reference's "Multigrid level" count */
  int32_t coarse_max;      /* automatic levels: coarsen until at most this many cells (<= 64) */
  int32_t max_cycles;      /* cycle (or Krylov iteration) limit */
  int32_t krylov;          /* 0: stationary V-cycles; 1: flexible CG, 2: flexible GMRES(30)
                              (residual falls monotonically), one V-cycle as preconditioner */
  int32_t use_graph;       /* 1 (default): the cycle loop as one CUDA graph whose stopping tests
                              run on the device (one host wait per solve); 2: one captured graph
                              per cycle, tested on the host; 0: no graphs */
  int32_t remove_rhs_mean; /* 1: project the mean out of b before solving (compatibility) */
  int32_t certify;         /* mixed precision: 1 = recompute the final residual in native FP64
                              (the cycle loop tracks it in double-word FP32 pairs) */
  int32_t device;          /* CUDA device ordinal; -1 = the current device */
  void* stream;            /* cudaStream_t to run on; NULL = the handle creates its own */
  int32_t stop_rule;       /* GBMG_STOP_* (default GBMG_STOP_RELATIVE) */
  int32_t zero_wall_faces; /* 1: gbmg_project and gbmg_divergence first set the wall-normal
                              faces of u, v, w to zero in the caller's arrays (u at f = 0
                              and nx, v at 0 and ny, w at 0 and nz), as RHSP does before
                              its divergence ("MPLS_RisingBubble/20190612/
                              SOLVE_PRESSURE_POISSON.F90:16-41"); 0 (default): the faces
                              are read as given */
  int32_t inner_cycles;    /* mixed precision, stationary loop: FP32 V-cycles per double-word
                              defect correction (the residual is tested after each correction);
                              0 (default): four, and for the last correction the number the
                              last reduction predicts will reach tol (one under
                              GBMG_STOP_INCREMENT); 1..8: that many; at most 8 */
  int32_t split_restarts;  /* gbmg_project_split, stationary cycle: the DomainDecomposition
                              driver's restarts ("DomainDecomposition/3D/src/ns_solver/
                              ns_ppe_mg_solver.f90:29-44"): a cycle that does not cut the
                              residual by 1% (or raises it) ends the solve, p^ becomes
                              1.5 p - 0.5 p^, the source is rebuilt and the solve starts again
                              from the new p^, at most split_restarts times; after the last one
                              a stagnating cycle stops once the residual is under 1000 tol.
                              One V-cycle per iteration (also in mixed precision); 0 (default):
                              no restarts; at most 100 */
} gbmg_params;

typedef struct {
  int32_t status;       /* gbmg_status of the solve */
  int32_t cycles;       /* V-cycles (or Krylov iterations) done */
  int32_t levels;       /* multigrid levels used */
  int32_t coarse_n;     /* cells on the coarsest level (solved directly) */
  double rel_residual;  /* ||b - A p||_2 / ||b||_2 at exit (FP64) */
  double rms_residual;  /* sqrt(sum r^2 / n): the reference's multigrid norm */
  double res0;          /* relative residual of the initial guess */
  double ms;            /* device time of the call (CUDA events on the handle's stream) */
  double bytes;         /* algorithmic HBM bytes of the call */
  double increment;     /* GBMG_STOP_INCREMENT: max |p_k - p_(k-1)| of the last cycle (the
                           reference's ppe_linf); 0 under the other rules */
  int32_t device_loop;  /* 1: the cycles ran as one graph with the stopping tests on the device */
  int32_t restarts;     /* gbmg_project_split with split_restarts: restarts made (cycles counts
                           all of them) */
} gbmg_stats;

typedef struct {
  double* data; /* address of element (0,0,0) */
  int64_t sy;   /* element stride between y rows */
  int64_t sz;   /* element stride between z planes */
} gbmg_field;

typedef struct gbmg_handle gbmg_handle;

/* Defaults: FP64, V(2,2), automatic levels, coarse_max 64, 100 cycles,
 * stationary cycles, graphs on, mean projection of b on, FP64 certification
 * on, current device, relative-residual stopping rule, wall faces as given. */
void gbmg_default_params(gbmg_params* prm);

/* Allocates the device hierarchy for one grid.  Replaces the level set-up of
 * manager_init ("DomainDecomposition/3D/lib/data/branches.f90:172-216").
 * Returns GBMG_INVALID_ARG for a grid the hierarchy cannot coarsen as asked. */
int gbmg_create(const gbmg_grid* grid, const gbmg_params* prm, gbmg_handle** out);

int gbmg_destroy(gbmg_handle* h);

/* Face coefficients from the cell density rho: ppe_sor_init
 * ("Two phase flows/newOpenMP/3D+IBM/src/ns_solver/ns_ppe_solver.f90:1-65";
 * 2D "Two phase flows/newOpenMP/2D/src/ns_solver/ns_ppe_solver.f90:1-48").
 * Also builds every coarse level and the coarse-level inverse.  Returns once
 * rho has been read (the caller may then reuse it); the set-up kernels run on
 * on the handle's stream, and every later call on the handle is ordered after
 * them (a kernel failure there is reported by the next call). */
int gbmg_set_rho(gbmg_handle* h, gbmg_field rho, int mem);

/* Density from the level set, then as gbmg_set_rho: rho_mu + ls_funs
 * ("Two phase flows/newOpenMP/2D/src/interface_solver/others.f90:1-61"):
 * rho = rho_pos*H + rho_neg*(1-H), H the smoothed Heaviside of half width eps.
 * The reference is rho_pos = 1, rho_neg = rho_12.  Returns once phi has been
 * read, as gbmg_set_rho. */
int gbmg_set_phi(gbmg_handle* h, gbmg_field phi, double eps, double rho_pos, double rho_neg,
                 int mem);

/* Face coefficients given directly as cell-shaped low-face arrays (cx(i,j,k)
 * couples cells i-1 and i; cx(0,j,k) is ignored and taken as the wall). */
int gbmg_set_coef(gbmg_handle* h, gbmg_field cx, gbmg_field cy, gbmg_field cz, int mem);

/* Solve A p = b.  p is the initial guess on entry (the reference warm-starts
 * from the previous pressure) and the mean-free solution on exit.  Replaces
 * the iteration of ppe_sor_solver (ns_ppe_solver.f90:93-163) and of
 * ppe_mg_solver ("DomainDecomposition/3D/src/ns_solver/ns_ppe_mg_solver.f90:1-60"). */
int gbmg_solve(gbmg_handle* h, gbmg_field b, gbmg_field p, double tol, int mem,
               gbmg_stats* stats);

/* The whole projection, ppe_sor_solver + ns_momentum_correction
 * (ns_ppe_solver.f90:67-205): b = div(u*)/dt, solve, then
 * u_f -= dt (p_nb - p_i)/h / rho_f with rho_f the face average of rho (from the
 * last gbmg_set_rho / gbmg_set_phi).  u, v, w are corrected in place; wall
 * faces are left as given. */
int gbmg_project(gbmg_handle* h, gbmg_field u, gbmg_field v, gbmg_field w, gbmg_field p,
                 double dt, double tol, int mem, gbmg_stats* stats);

/* Pressure-split projection, the form of the DomainDecomposition solver's
 * pressure step ("DomainDecomposition/3D/src/ns_solver/ns_ppe_mg_solver.f90"):
 * the multigrid solves the constant-coefficient Laplacian
 *     lap p = rho_12 div(u*)/dt + div((1 - rho_12 beta) grad p_hat)
 * (ppe_mg_solver_init :62-136 and ppe_mg_solver_src :138-221, with beta =
 * 2/(rho_i + rho_nb) and zero-gradient ghosts at the walls), then corrects
 *     u_f -= dt [ (p_nb - p_i)/(rho_12 h) + (beta_f - 1/rho_12)(p_hat_nb - p_hat_i)/h ]
 * (ppe_mg_correction :223-276).  gbmg_set_split stores the cell density and
 * rho_12 and makes the handle's operator the Laplacian (coe = 1/h^2, walls
 * folded); gbmg_set_rho/phi/coef switch back.  gbmg_project_split starts the
 * solve from p_hat (the reference extrapolates p_hat = 2 p^n - p^{n-1} after
 * its third step and uses p^n before) and writes the mean-free pressure to
 * p; wall faces of u, v, w are left as given.  By default the solve runs to
 * tol under the handle's stop rule; with gbmg_params.split_restarts > 0 it
 * follows the reference driver's restarts of a stagnating cycle
 * (ns_ppe_mg_solver.f90:29-44: p_hat <- 1.5 p - 0.5 p_hat and the source
 * rebuilt), and the correction uses the last p_hat. */
int gbmg_set_split(gbmg_handle* h, gbmg_field rho, double rho_12, int mem);
int gbmg_project_split(gbmg_handle* h, gbmg_field u, gbmg_field v, gbmg_field w,
                       gbmg_field p_hat, gbmg_field p, double dt, double tol, int mem,
                       gbmg_stats* stats);

/* b = div(u)/dt (the right-hand side of ppe_sor_solver, ns_ppe_solver.f90:77-89),
 * without mean removal. */
int gbmg_divergence(gbmg_handle* h, gbmg_field u, gbmg_field v, gbmg_field w, double dt,
                    gbmg_field b, int mem);

/* r = b - A p with the current coefficients; *norm2 = sum r^2 (FP64).  r may
 * have data == NULL (norm only).  The residual of multigrid_residual
 * ("DomainDecomposition/3D/src/others/multigrid_solver.f90:162-222"). */
int gbmg_residual(gbmg_handle* h, gbmg_field b, gbmg_field p, gbmg_field r, double* norm2,
                  int mem);

/* max and mean |div u| over the cells: ns_check_convergence_div
 * ("Two phase flows/newOpenMP/2D/src/ns_solver/ns_solvers.f90:55-83"). */
int gbmg_div_stats(gbmg_handle* h, gbmg_field u, gbmg_field v, gbmg_field w, double* max_div,
                   double* mean_div, int mem);

/* gbmg_div_stats without a handle and without allocating (no counterpart in
 * the reference; the statistics are those of ns_check_convergence_div).  For
 * callers that must not allocate device memory while they run: a time loop
 * that checks the divergence after every step while other streams keep working
 * (cudaFree synchronizes the whole device, so an allocating check would stall
 * them each step), and a code whose device memory is committed to its own
 * fields, with no room for the multigrid hierarchy gbmg_create allocates.
 * u, v, w: DEVICE arrays in the MAC layout above (w ignored when nz = 1);
 * device: CUDA device (-1 = current); stream: cudaStream_t (NULL = default);
 * err: optional buffer (err_len bytes) for the error text.
 * The scratch is a static 33 KB device array: partial sums of at most 2048
 * blocks (the call needs 8 per SM) plus result slots; grids whose rows of
 * cells (ny*nz) exceed 2^31 - 1, or a device whose reduction needs more than
 * 2048 blocks, are rejected with GBMG_INVALID_ARG and a message in err.
 * Every call looks up the scratch's address on its device (no cached address,
 * so a cudaDeviceReset in between is safe) and zeroes the scratch's completion
 * counter on the stream before its launch, so a launch that failed earlier
 * leaves nothing behind.  The first call on a device may load the library's
 * module there: make it before any stream capture on that device.  Calls
 * share the one scratch of their device: two calls in
 * flight at once (from two host threads) race and corrupt each other's sums.
 * Every call returns after its stream has finished it. */
int gbmg_div_stats_noalloc(const gbmg_grid* grid, gbmg_field u, gbmg_field v, gbmg_field w,
                           double* max_div, double* mean_div, int device, void* stream,
                           char* err, size_t err_len);

/* Adjoint of the solve (no reference counterpart: the differentiable
 * projection of this library).  Given the solution p of A p = b and the
 * adjoint lam of A lam = dJ/dp (both from gbmg_solve with the current
 * operator), writes dJ/drho_i = sum over the faces of cell i of
 * (lam_nb - lam_i)(p_nb - p_i) * (-2/(rho_i + rho_nb)^2/h^2) into grad_rho,
 * and, when phi.data is not NULL, dJ/dphi = dJ/drho (rho_pos - rho_neg) H'(phi)
 * into grad_phi.  dJ/db is lam itself.  Uses the density of the last
 * gbmg_set_rho / gbmg_set_phi. */
int gbmg_adjoint(gbmg_handle* h, gbmg_field p, gbmg_field lam, gbmg_field phi, double eps,
                 double rho_pos, double rho_neg, gbmg_field grad_rho, gbmg_field grad_phi, int mem);

/* ---- Adams-Bashforth momentum step ------------------------------------------
 * The velocity step around the projection, ns_ab_solver_SOR after
 * ppe_sor_init ("Two phase flows/newOpenMP/2D/src/ns_solver/
 * admas_bashforth_solver.f90:40-67"; 3D "Two phase flows/newOpenMP/3D+IBM/
 * src/ns_solver/admas_bashforth_solver.f90:43-70"): velsrc%tmp from the old
 * fields (sec_part1..3 of ns_ab_diff.f90: viscous term mu/rho lap(u)/Re, the
 * interface-viscosity term (1 - mu_12) delta grad(phi).grad(u)/(rho Re),
 * gravity btn_g g/Fr and surface tension btn_sf curv delta n/(We rho)), then
 * `iterations` passes (the reference: 4) of
 *   ns_linearize     vel%tmp = vel%now (the advecting velocity), averaged to
 *                    each face by find_stag_vel (bcs.f90),
 *   ns_ab_setup      velsrc%now = second-order upwind advection of vel%old
 *                    (ns_ab_adv_source_sec) + velsrc%tmp,
 *   ns_ab_predictor  vel%now = vel%old + dt (1.5 velsrc%now - 0.5 velsrc%old),
 *                    velbc,
 *   the projection   gbmg_project's solve and correction with the handle's
 *                    operator (set it from rho%now first: gbmg_set_rho /
 *                    gbmg_set_phi, the reference's ppe_sor_init), velbc,
 * and ns_check_convergence_vel (linf, l2f of vel%now - vel%tmp of the last
 * pass).  All arithmetic of the explicit part is FP64 in the reference's
 * operand order, so velsrc%now and the predicted velocity are the reference
 * formulas' own doubles; the projection solves to p_tol.
 *
 * Arrays keep the reference's ghost cells: each is the padded box of `ghost`
 * layers around the interior, and all of them (except p) share one pair of
 * strides (a Fortran caller's arrays of one shape).  Addresses follow the
 * layout above: a cell array at its interior cell (1,1,1) (c_loc(phi(1,1,1))),
 * u at c_loc(u(0,1,1)), v at c_loc(v(1,0,1)), w at c_loc(w(1,1,0)).  velbc
 * (bcs.f90:28-148, 3D :44-257) fills every ghost layer: per wall, bc 1
 * (no-slip) mirrors the interior negated, 2 (slip) copies it, and the
 * wall-normal face is set to 0; other values leave that wall's ghosts.  The
 * surface-tension term is added only when btn_sf != 0 (the reference computes
 * the curvature only then); nrm_* and curv may be NULL otherwise.  In 2D
 * (nz = 1) the w arrays, nrm_z and gz are ignored.  p is an interior cell
 * array with its own strides (ghosts untouched).  Needs ghost >= 2 and at
 * least ghost + 1 cells per axis. */
typedef struct {
  int32_t ghost;       /* ghost layers of every array (the reference's ghc) */
  int32_t bc[6];       /* velbc of the walls x-, x+, y-, y+, z-, z+: ubc(1:2), vbc(1:2), wbc(1:2) */
  int32_t iterations;  /* predictor-projection passes */
  int32_t adv_scheme;  /* momentum advection: 0 second-order upwind (ns_ab_adv_source_sec, the
                          reference's active choice), 1 QUICK (ns_ab_adv_source_quick) */
  double dt;
  double re, fr, we;   /* Reynolds, Froude and Weber numbers */
  double mu_12;        /* viscosity ratio */
  double gx, gy, gz;   /* gravity direction */
  double btn_g, btn_sf; /* gravity and surface-tension switches */
  double p_tol;        /* relative residual of each pressure solve */
} gbmg_ns_params;

typedef struct {
  gbmg_field u, v, w;                   /* vel%now: in, the first linearisation; out, the step */
  gbmg_field u_old, v_old, w_old;       /* vel%old */
  gbmg_field su, sv, sw;                /* velsrc%now (out: interior written) */
  gbmg_field su_old, sv_old, sw_old;    /* velsrc%old */
  gbmg_field rho, mu, delta, phi;       /* rho%old, mu%old, delta%old, phi%old */
  gbmg_field nrm_x, nrm_y, nrm_z, curv; /* normals%{x,y,z,curv}%old */
  gbmg_field p;                         /* p%now: warm start in, pressure out */
} gbmg_ns_fields;

typedef struct {
  int32_t status;          /* worst gbmg_status of the pressure solves */
  int32_t cycles;          /* cycles (or Krylov iterations) of all solves */
  double max_rel_residual; /* largest final relative residual of the solves */
  double linf, l2f;        /* ns_check_convergence_vel of the last pass */
  double ms;               /* device time of the call */
} gbmg_ns_stats;

int gbmg_ns_ab_step(gbmg_handle* h, const gbmg_ns_params* prm, const gbmg_ns_fields* f, int mem,
                    gbmg_ns_stats* stats);

/* One predictor pass without the projection: velsrc%tmp, ns_linearize,
 * ns_ab_setup, ns_ab_predictor and velbc (su, sv, sw and u, v, w written). */
int gbmg_ns_ab_predict(gbmg_handle* h, const gbmg_ns_params* prm, const gbmg_ns_fields* f,
                       int mem);

/* velbc alone on u, v, w (uses prm->ghost and prm->bc). */
int gbmg_ns_velbc(gbmg_handle* h, const gbmg_ns_params* prm, gbmg_field u, gbmg_field v,
                  gbmg_field w, int mem);

/* Interface normals and curvature, the reference's curv + surface_norms
 * ("Two phase flows/newOpenMP/2D/src/interface_solver/others_normals.f90";
 * 3D "…/3D+IBM/src/interface_solver/others_normals.f90") with the combined
 * compact difference scheme "ccd" ("…/2D/lib/solver/ccd_solvers.f90",
 * block tridiagonal solver "…/2D/lib/solver/matrix_solver.f90"): phi_x,
 * phi_y (phi_z) and the second and cross derivatives of phi by compact line
 * solves over the whole padded box, then on the interior
 *   curv = (fyy fx^2 + fxx fy^2 - 2 fxy fx fy) / (fx^2 + fy^2 + 1e-12)^1.5
 * (3D: the three-term form) and zero-gradient ghosts (bc) on nrm_x, nrm_y,
 * nrm_z and curv.  nrm_* receive phi's gradient (the reference's
 * normals%x..z, not normalised): the nrm_* and curv inputs of the momentum
 * step at the next time step.  Padded arrays as gbmg_ns_fields (prm->ghost
 * layers, one pair of strides); the derivatives equal the reference formulas'
 * doubles, the curvature's power uses CUDA's pow. */
int gbmg_ns_curvature(gbmg_handle* h, const gbmg_ns_params* prm, gbmg_field phi,
                      gbmg_field nrm_x, gbmg_field nrm_y, gbmg_field nrm_z, gbmg_field curv,
                      int mem);

/* ls_funs + rho_mu over the whole padded box ("Two phase flows/newOpenMP/2D/
 * src/interface_solver/others.f90:1-61"): with x = phi/ls_wid, heavy = 1 for
 * x > 1 - 1e-12, 0 for x < -1 + 1e-12, else (1 + x + sin(pi x)/pi)/2 clipped
 * to [0, 1]; delta = (1 + cos(pi x))/(2 ls_wid) inside the band, else 0;
 * rho = heavy + rho_12 (1 - heavy), mu = heavy + prm->mu_12 (1 - heavy): the
 * rho, mu and delta of the momentum step (as its old fields one step later).
 * Padded arrays as gbmg_ns_fields; CUDA's sin and cos; NULL outputs skipped. */
int gbmg_ns_rho_mu(gbmg_handle* h, const gbmg_ns_params* prm, gbmg_field phi, double ls_wid,
                   double rho_12, gbmg_field rho, gbmg_field mu, gbmg_field delta, int mem);

/* mass_preserving_level_set ("Two phase flows/newOpenMP/2D/src/interface_
 * solver/mass_preserving_level_set.f90:1-48"; 3D "…/3D+IBM/…"), the correction
 * of the MPLS interface method, in place on the padded phi: `iterations`
 * times (the reference: 2) measure ls_mv's mass = sum (H + rho_12 (1 - H)) H dv
 * and the compact gradient of phi (surface_norms), then
 *     phi += lam delta |grad phi|,  lam = (imass - mass) /
 *            sum delta^2 |grad phi| (2 (1 - rho_12) H + rho_12) dv
 * on the interior, and bc.  *mass receives the mass measured last (before the
 * last correction, as the reference leaves p%glb%mass); iterations = 0 only
 * measures it (ls_mv, e.g. imass at the start).  H, delta from ls_funs with
 * half width ls_wid (CUDA's sin and cos); sums in a fixed order.  Returns
 * GBMG_INVALID_ARG, phi unchanged by that pass, when no cell lies in the
 * interface band (the reference would divide by zero). */
int gbmg_ns_mass_correct(gbmg_handle* h, const gbmg_ns_params* prm, gbmg_field phi,
                         double ls_wid, double rho_12, double imass, int iterations, int mem,
                         double* mass);

/* vof_wlic_solver ("Two phase flows/newOpenMP/2D/src/interface_solver/
 * clsvof.f90:1-143"; 3D "…/3D+IBM/…"), the volume-fraction transport of the
 * CLSVOF interface method, in place on the padded vof: sweeps along x, y (z),
 * each the WLIC flux at every face (a THINC profile with beta = 2.3, weighted
 * by |n_d|/|n|_1 of surface_norms2's central-difference normal of phi, against
 * the upwind flux vof u dt), the update vof -= d(flux)/dx_d - vof_old dt du/dx_d
 * and bc; vof is clipped to [0, 1] (1e-12 margins) after the last sweep.
 * u_old, v_old, w_old are the face velocities (vel%old), prm->dt the step;
 * padded arrays as gbmg_ns_fields.  CUDA's exp, log and cosh. */
int gbmg_ns_vof_advect(gbmg_handle* h, const gbmg_ns_params* prm, gbmg_field vof,
                       gbmg_field vof_old, gbmg_field u_old, gbmg_field v_old, gbmg_field w_old,
                       gbmg_field phi, int mem);

/* ibm_bc's forcing ("Two phase flows/newOpenMP/3D+IBM/src/ns_solver/
 * ns_solvers.f90:150-211"), after ns_check_convergence_div: bc on the padded
 * cell solid fraction (in place), then on the interior faces, with s the face
 * average of the solid fraction, u = (1 - s) u, v = (1 - s) v and
 * w = (1 - s) w + s w_body (the body's vertical speed; in 2D v takes it).
 * The reference samples one gate geometry into the solid fraction; here the
 * caller supplies the field.  Ghost faces are not touched, as there. */
int gbmg_ns_ibm(gbmg_handle* h, const gbmg_ns_params* prm, gbmg_field solid, double w_body,
                gbmg_field u, gbmg_field v, gbmg_field w, int mem);

/* bc ("Two phase flows/newOpenMP/2D/src/others/bcs.f90:1-26"): zero-gradient
 * ghost layers of one padded cell array, in place. */
int gbmg_ns_bc(gbmg_handle* h, const gbmg_ns_params* prm, gbmg_field a, int mem);

/* Copies level `level`'s face coefficients (FP64) into cell-shaped arrays of
 * that level's size (gbmg_level_dims).  For tests of the coarsening rule. */
int gbmg_level_coef(gbmg_handle* h, int level, gbmg_field cx, gbmg_field cy, gbmg_field cz,
                    int mem);

/* Level count and per-level sizes (dims[3*l+0..2] = nx, ny, nz). */
int gbmg_level_dims(gbmg_handle* h, int32_t* levels, int32_t* dims, int32_t max_levels);

/* Number of kernels this handle launched since creation (graph replays count
 * every kernel node). */
int64_t gbmg_kernel_launches(gbmg_handle* h);

/* Per-kernel-class timing (no reference counterpart; the reference only
 * accumulates the wall time of the whole pressure step, ns_ppe_solver.f90:
 * 75,167-168).  With profiling on, graphs are bypassed and every launch is
 * bracketed by CUDA events on the handle's stream.  Classes: GBMG_PROF_*. */
enum {
  GBMG_PROF_SMOOTH_FINE = 0,   /* smoother on the finest level */
  GBMG_PROF_SMOOTH_COARSE = 1, /* smoother on the other levels */
  GBMG_PROF_RESTRICT_FINE = 2, /* residual + restriction out of the finest level */
  GBMG_PROF_RESTRICT_COARSE = 3,
  GBMG_PROF_PROLONG_FINE = 4,  /* prolongation + correction into the finest level */
  GBMG_PROF_PROLONG_COARSE = 5,
  GBMG_PROF_COARSE_SOLVE = 6,
  GBMG_PROF_RESIDUAL = 7,      /* FP64 (or double-word) residual + norm on the finest level */
  GBMG_PROF_VECTOR = 8,        /* mean projection, p += e, Krylov vector kernels */
  GBMG_PROF_SETUP = 9,         /* coefficients, coarse operators, coarse inverse */
  GBMG_PROF_CERTIFY = 10,      /* native FP64 residual after a mixed-precision solve */
  GBMG_PROF_MOMENTUM = 11,     /* momentum step: sources, predictor, velbc, velocity change */
  GBMG_PROF_CLASSES = 12
};
int gbmg_set_profiling(gbmg_handle* h, int on);
/* ms[c] = summed device time, launches[c] = launch count of class c since
 * profiling was switched on (arrays of n >= GBMG_PROF_CLASSES entries). */
int gbmg_profile(gbmg_handle* h, double* ms, int64_t* launches, int32_t n);

/* ---- Level-set transport (the interface solver's advection step) ---------
 * level_set_rk3_solver ("Two phase flows/newOpenMP/2D/src/interface_solver/
 * level_set_rk3_solver.f90:1-186"; 3D "Two phase flows/newOpenMP/3D+IBM/src/
 * interface_solver/level_set_rk3_solver.f90:1-215"): phi_t + div(u phi) = 0
 * with the cell-centred velocity (the reference's nvel, node_vel of the MAC
 * faces), WENO-JS reconstruction of the split fluxes u+ phi and u- phi
 * (wenojs_flux_split), zero-gradient ghosts (bc) and three stages of SSP-RK3,
 * all in FP64.  A separate handle owns its device scratch (phi, u, v, w, two
 * stage arrays and six face arrays: 12 n doubles). */
typedef struct gbmg_ls gbmg_ls;

/* device: CUDA device (-1 = current); stream: cudaStream_t (NULL = own). */
int gbmg_ls_create(const gbmg_grid* grid, int device, void* stream, gbmg_ls** out);
int gbmg_ls_destroy(gbmg_ls* ls);

/* steps time steps of dt on phi, in place (host or device memory, the
 * gbmg_field layout of the cell arrays above); u, v, w cell-centred (w
 * ignored when nz = 1).  Returns after the stream has finished. */
int gbmg_ls_advect(gbmg_ls* ls, gbmg_field phi, gbmg_field u, gbmg_field v, gbmg_field w,
                   double dt, int steps, int mem);

/* Redistancing, level_set_rk3_redis(btn) ("Two phase flows/newOpenMP/2D/src/
 * interface_solver/level_set_rk3_redis.f90:1-361"; 3D "Two phase flows/
 * newOpenMP/3D+IBM/src/interface_solver/level_set_rk3_redis.f90"), phi in
 * place: phi_tau + S (|grad phi| - 1) = 0 in pseudo-time steps rdt with the
 * Godunov gradient of WENO-JS one-sided derivatives and three SSP-RK3
 * stages.  btn = 1 (every few time steps in the reference): S = 2H - 1 of the
 * level set (H the smoothed Heaviside of half width ls_wid) and the
 * mass-preserving correction (3D: weighted by the density ratio rho_12),
 * for 3 dx of pseudo time.  btn = 0 (initialisation): S = phi, phi first
 * divided by max |grad phi|, for 1.5 x the largest extent of the domain
 * (n h per axis).  Both stop earlier when the largest change of an
 * iteration is at most 1e-8 (2D) or 1e-5 (3D), or after max_iter
 * iterations.  *iters and *last_change report the iterations done and that
 * change.  The sign and the Heaviside use CUDA's sin and cos. */
int gbmg_ls_redistance(gbmg_ls* ls, gbmg_field phi, double ls_wid, double rdt, double rho_12,
                       int btn, int max_iter, int mem, int32_t* iters, double* last_change);

/* Kernels launched by this handle since creation. */
int64_t gbmg_ls_kernel_launches(gbmg_ls* ls);

/* Text of the last error on this handle ("" if none). */
const char* gbmg_ls_last_error(gbmg_ls* ls);

const char* gbmg_strerror(int status);

/* Text of the last error on this handle ("" if none). */
const char* gbmg_last_error(gbmg_handle* h);

#ifdef __cplusplus
}
#endif

#endif /* GBMG_H */
