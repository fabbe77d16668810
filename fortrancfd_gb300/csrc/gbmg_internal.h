// Internal declarations shared by the CUDA translation units of libgbmg.
//
// Device layout: every level stores dense cell arrays in C order (z, y, x),
// x fastest, with strides sy = nx and sz = nx*ny.  Face coefficients are
// cell-shaped low-face arrays (cx[q] couples cells q-1 and q along x; the low
// wall entries are 0 and the high wall is implicit), so every array of a level
// has the same index map and alignment.
#pragma once

#include "schedule.h"
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace gbmg {

constexpr int kMaxCoarse = 64;    // largest coarsest level solved by the dense inverse
constexpr int kMaxLevels = 24;

// One multigrid level seen by the kernels, in arithmetic type T.
template <typename T>
struct LevelView {
  int nx, ny, nz;
  int fx, fy, fz;        // coarsening factor to the next level per axis (1 or 2)
  const T* cx;
  const T* cy;
  const T* cz;
  const T* idiag;        // 1/diagonal, or nullptr (computed on the fly)
  T* sol;
  T* src;
  // Coefficients from the cell density (FP32 finest level): when rho is set,
  // the face coefficient between cells a and b along axis x is
  // kx / (rho_a + rho_b) with kx = 2/dx^2, and cx, cy, cz are not read.
  const T* rho = nullptr;
  T kx = T(0), ky = T(0), kz = T(0);
  // sol, src and rho in the colour-split layout (FP32 finest level, density
  // form, nx even): cell (i,j,k) at ((i+j+k)&1)*hstride + q/2, q the natural
  // index, hstride >= n/2 the distance between the two colour halves
  int split = 0;
  size_t hstride = 0;
  // traverse the z planes from the top (split kernels): consecutive launches
  // on the finest level alternate direction, so each starts on the planes the
  // previous one touched last, which are still in L2
  int zrev = 0;
};

// Deterministic single-pass grid reduction scratch: per-block partial sums,
// a completion counter and result slots (see reduce.cuh).
struct ReduceScratch {
  double* partials;      // kRedValues * max_blocks
  unsigned int* counter; // 1 word, returns to 0 after each reduction
  double* result;        // result slots
  int max_blocks;
};

constexpr int kRedValues = 2;   // values reduced together per launch
constexpr int kRedSlots = 16;   // result slots

// State of the cycle loop run on the device (k_cycle_ctl after each cycle):
// the host's stopping tests, in the same order and arithmetic.
struct CycleCtl {
  double scale;      // ||b|| (1 when b = 0)
  double tol;        // threshold of the residual test (or of the increment)
  double guard;      // divergence bound on the relative residual
  double best;       // lowest relative residual so far (the flat test)
  double r2, rel;    // last cycle: sum r^2 and ||r|| / scale
  double inc;        // last cycle: max |p_k - p_(k-1)| (increment rule)
  int max_cycles;
  int step;          // cycles per iteration (FP32 cycles per defect correction)
  int iters;         // iterations done
  int by_inc;        // stop on the increment instead of the residual
  int flat_stop;     // stop after four cycles without a lower residual
  int cyc;           // cycles done
  int flat;          // cycles since the last new lowest residual
  int status;        // kCtlRunning / kCtlConverged / kCtlDiverged
  int stalled;       // the flat test ended the loop
  int adaptive;      // end the loop when fewer than `step` cycles will do (tail_cycles)
  int tail;          // ... and the cycles of that last correction
};

// tail_cycles (the adaptive mixed loop's schedule): schedule.h
enum : int { kCtlRunning = 0, kCtlConverged = 1, kCtlDiverged = 2 };

// Result slot assignment.
enum : int {
  kSlotNorm = 0,     // sum r^2 of the last residual
  kSlotSumB = 2,     // sum b, sum (b - mean)^2
  kSlotSum = 4,      // generic sum / sum of squares
  kSlotMax = 6,      // max |div| (bit pattern, atomicMax)
  kSlotDot = 8,      // Krylov dot products (2 values)
  kSlotDot2 = 10,
  kSlotInc = 12,     // max |p_k - p_(k-1)| of the last cycle (bit pattern, atomicMax)
  kSlotIncSum = 14,  // sum of p_k - p_(k-1) (its mean is removed first)
};

// ---- the bottom of the cycle in one block (subcycle.cu) ----------------------
constexpr int kSubMaxCells = 4096;  // levels this small run inside one block
constexpr int kSubMaxLevels = 8;
template <typename T>
struct SubLevel {
  int nx, ny, nz;
  int fx, fy, fz;
  const T* cx;
  const T* cy;
  const T* cz;
  int lx, ly;  // log2 of nx and ny when both are powers of two (index by shifts), else -1
};
template <typename T>
struct SubCycle {
  int nlev, nu1, nu2, reverse, n_coarse;
  SubLevel<T> lv[kSubMaxLevels];   // the levels from the first small one down
  int off[kSubMaxLevels + 1];      // shared-memory offsets (elements): sol, src per level
  const T* src_in;                 // right-hand side of the first small level (global)
  T* sol_out;                      // its result (global)
  const T* minv;
  const T* adense;
};
template <typename T>
size_t subcycle_smem(const SubCycle<T>& S);
template <typename T>
int subcycle_init(size_t smem);
template <typename T>
void launch_subcycle(cudaStream_t s, const SubCycle<T>& S);

// ---- launchers (kernels_mg.cu) ---------------------------------------------
// zero_guess: the level's current values are taken as zero (first colour of
// the first sweep after the coarse unknown was started at zero)
template <typename T>
void launch_smooth(cudaStream_t s, const LevelView<T>& L, int color, bool zero_guess = false);
// zero_sol: also set the coarse unknown to zero (not needed when its first
// sweep starts from a zero guess)
template <typename T>
void launch_restrict(cudaStream_t s, const LevelView<T>& F, const LevelView<T>& C, bool zero_sol);
// live >= 0 (split finest level only): correct only the cells of colour live,
// when the next sweep's first colour launch overwrites the other colour unread
template <typename T>
void launch_prolong(cudaStream_t s, const LevelView<T>& F, const LevelView<T>& C, int live = -1);
// r = src - A sol on a level; writes r (type TO, may be null) and sum r^2 into slot.
template <typename TO>
void launch_residual_norm(cudaStream_t s, const LevelView<double>& L, TO* r,
                          const ReduceScratch& R, int slot);
template <typename T>
void launch_coarse_solve(cudaStream_t s, int n, const T* minv, const T* adense, const T* b, T* x);
// work: 2 n^2 + n doubles of scratch (n = cells of the coarsest level)
void launch_coarse_invert(cudaStream_t s, const LevelView<double>& C, double* minv,
                          double* adense, float* minv32, float* adense32, double* work);
// three optional float outputs
struct Float3Out {
  float* p[3];
};
void launch_coarsen(cudaStream_t s, const LevelView<double>& F, double* cx, double* cy,
                    double* cz, int cnx, int cny, int cnz, Float3Out c32 = Float3Out{});
void launch_idiag(cudaStream_t s, const LevelView<double>& L, double* idiag);
void launch_to_float(cudaStream_t s, const double* a, float* b, size_t n);

// ---- launchers (kernels_flow.cu) -------------------------------------------
struct Strided {
  const double* data;
  int64_t sy, sz;
};
void launch_rho_from_phi(cudaStream_t s, int nx, int ny, int nz, Strided phi, double eps,
                         double rho_pos, double rho_neg, double* rho);
void launch_copy_in(cudaStream_t s, int nx, int ny, int nz, Strided src, double* dst);
void launch_copy_out(cudaStream_t s, int nx, int ny, int nz, const double* src, double* dst,
                     int64_t sy, int64_t sz);
// c32 / cw: optional arrays of 3 pointers (x, y, z) for the FP32 and
// double-word copies, written in the same pass.
// ---- pressure-split projection (psplit.cu) ----
// src = rho_12 div(u*)/dt + the split term of p^ (ppe_mg_solver_src)
void launch_psplit_rhs(cudaStream_t s, int nx, int ny, int nz, const double* rho, Strided u,
                       Strided v, Strided w, const double* ph, double rho12, double dx, double dy,
                       double dz, double dt, double* src);
// u_f -= dt ((1/rho_12) dp/h + (beta_f - 1/rho_12) dp^/h) (ppe_mg_correction)
// ph = w p + (1 - w) ph
void launch_guess_update(cudaStream_t s, const double* p, double* ph, size_t n, double w);
void launch_psplit_correct(cudaStream_t s, int nx, int ny, int nz, const double* rho,
                           const double* p, const double* ph, double rho12, double dx, double dy,
                           double dz, double dt, double* u, int64_t usy, int64_t usz, double* v,
                           int64_t vsy, int64_t vsz, double* w, int64_t wsy, int64_t wsz);
// constant-coefficient Laplacian: coe = 1/h^2 on interior faces (c32, cw optional)
void launch_face_const(cudaStream_t s, int nx, int ny, int nz, double dx2, double dy2, double dz2,
                       double* cx, double* cy, double* cz, float* const* c32, float2* const* cw);

// ---- density-form FP32 arithmetic (the finest level of the mixed cycle) ----
// Approximate reciprocal (rcp.approx.ftz: one MUFU.RCP, within 1 ulp; +inf ->
// +0, so a wall neighbour given density +inf contributes a zero coefficient).
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
// The roundings of the density-form FP32 arithmetic are pinned with explicit
// _rn intrinsics (no contraction left to the compiler), so that every kernel
// that relaxes a cell -- natural layout, colour-split layout, one colour per
// launch or a whole sweep per launch -- gives the same bits.
// face coefficient k/(rho_a + rho_b), k = 2/h^2
__device__ __forceinline__ float rho_face32(float k, float ra, float rb) {
  return __fmul_rn(k, rcp_approx(__fadd_rn(ra, rb)));
}
// one face of the smoother's sums: s += c p_nb, d += c
__device__ __forceinline__ void rho_acc32(float c, float pn, float& s, float& d) {
  s = __fmaf_rn(c, pn, s);
  d = __fadd_rn(d, c);
}
// the smoother's update (s - b)/d
__device__ __forceinline__ float rho_update32(float v, float d) {
  return __fmul_rn(v, rcp_approx(d));
}
__device__ __forceinline__ float rho_relax32(float s, float b, float d) {
  return rho_update32(__fsub_rn(s, b), d);
}

// ---- colour-split FP32 finest level (kernels_split.cu) ----
void launch_smooth_split(cudaStream_t s, const LevelView<float>& L, int color, bool zero_guess);
void launch_restrict_split(cudaStream_t s, const LevelView<float>& F, const LevelView<float>& C,
                           bool zero_sol);
void launch_prolong_split(cudaStream_t s, const LevelView<float>& F, const LevelView<float>& C,
                          int live);
void launch_to_split(cudaStream_t s, const double* a, float* out, int nx, int ny, int nz,
                     size_t hstride);
void launch_from_split(cudaStream_t s, const float* a, double* out, int nx, int ny, int nz,
                       size_t hstride);
// elements reserved past n in each split FP32 finest-level array for the pad
constexpr size_t kSplitPadMax = 65536;

// bulk_rho: the two bulk densities (rho_pos, rho_neg of the level set), or
// null; faces between two bulk cells use host-computed values.
void launch_face_coef(cudaStream_t s, int nx, int ny, int nz, double dx2, double dy2, double dz2,
                      const double* rho, double* cx, double* cy, double* cz, float* const* c32,
                      float2* const* cw, const double* bulk_rho, float* rho32 = nullptr,
                      size_t hstride = 0);
void launch_divergence(cudaStream_t s, int nx, int ny, int nz, Strided u, Strided v, Strided w,
                       double dx, double dy, double dz, double dt, double* b);
void launch_correct(cudaStream_t s, int nx, int ny, int nz, const double* rho, const double* p,
                    double dx, double dy, double dz, double dt, double* u, int64_t usy,
                    int64_t usz, double* v, int64_t vsy, int64_t vsz, double* w, int64_t wsy,
                    int64_t wsz);
// dJ/drho (and dJ/dphi when grad_phi != nullptr) from p and the adjoint lam.
void launch_adjoint(cudaStream_t s, int nx, int ny, int nz, double dx2, double dy2, double dz2,
                    const double* rho, const double* p, const double* lam, Strided phi,
                    double eps, double rpos, double rneg, double* grad_rho, double* grad_phi);
void launch_div_stats(cudaStream_t s, int nx, int ny, int nz, Strided u, Strided v, Strided w,
                      double dx, double dy, double dz, const ReduceScratch& R);
// The mean-free increment of a cycle: d = x - y (y null: d = x) over the
// cells (colour-split when hstride > 0); R.result[slot_sum] <- sum d,
// R.result[slot_out] <- max |d - mean d| (bit pattern of a non-negative double)
// *flag (a result slot, as bits) = nonzero when any x[q] is nonzero
void launch_nonzero(cudaStream_t s, const double* x, size_t n, double* flag);
// One thread: applies the stopping tests to the cycle just finished and
// sets the graph conditionals `loop` (and `next` when has_next) to 1 to go on
// or 0 to stop.  Only inside a graph that owns these handles.
void launch_cycle_ctl(cudaStream_t s, CycleCtl* c, const double* result,
                      cudaGraphConditionalHandle loop, cudaGraphConditionalHandle next,
                      int has_next);
template <typename T>
void launch_increment(cudaStream_t s, const T* x, const T* y, size_t n, size_t hstride,
                      const ReduceScratch& R, int slot_sum, int slot_out);
// u at f = 0 and nx, v at 0 and ny, w (if not null) at 0 and nz set to zero
void launch_zero_wall_faces(cudaStream_t s, int nx, int ny, int nz, double* u, int64_t usy,
                            int64_t usz, double* v, int64_t vsy, int64_t vsz, double* w,
                            int64_t wsy, int64_t wsz);
// slot <- sum x, slot+1 <- sum x^2
void launch_sum(cudaStream_t s, const double* x, size_t n, const ReduceScratch& R, int slot);
// y = x - result[slot]/n ; result[slot2] <- sum y^2 (slot2 < 0: no norm)
void launch_shift_by_mean(cudaStream_t s, const double* x, double* y, size_t n,
                          const ReduceScratch& R, int slot, int slot2);
void launch_add_float(cudaStream_t s, double* p, const float* e, size_t n);
// Flexible-CG helpers.  Slots: kSlotDot = r.z, kSlotDot+1 = r.z_old,
// kSlotDot2 = d.(A d), kSlotDot2+1 = r.z of the previous iteration.
void launch_dot2(cudaStream_t s, const double* a, const double* b, const double* c, size_t n,
                 const ReduceScratch& R, int slot);
void launch_pcg_direction(cudaStream_t s, double* d, double* zold, const double* z, size_t n,
                          const ReduceScratch& R, int first);
void launch_pcg_step(cudaStream_t s, double* x, const double* d, size_t n, const ReduceScratch& R);
// q = A d on a level and d.q into slot (kernels_mg.cu)
void launch_apply_dot(cudaStream_t s, const LevelView<double>& L, const double* d, double* q,
                      const ReduceScratch& R, int slot);
void launch_float_to_double(cudaStream_t s, const float* a, double* b, size_t n);
// flexible GMRES vector kernels (krylov.cu): out[i] = V_i . w for i < cnt
// (basis V_i at V + i*ld; partials: cnt * max_blocks doubles), w += sign *
// sum_i coef[i] V_i, out = alpha * in
void launch_mdot(cudaStream_t s, const double* V, size_t ld, int cnt, const double* w, size_t n,
                 double* partials, int max_blocks, double* out);
void launch_maxpy(cudaStream_t s, double* w, const double* V, size_t ld, const double* coef,
                  int cnt, double sign, size_t n);
void launch_scale_copy(cudaStream_t s, double* out, const double* in, double alpha, size_t n);
void launch_scale_rsqrt(cudaStream_t s, double* w, const double* nrm2, size_t n);  // w /= |w|
void launch_double_to_float(cudaStream_t s, const double* a, float* b, size_t n);

int reduce_blocks_for(size_t n);

// ---- double-word (float-float) operator of the finest level (kernels_dw.cu) ----
struct DwOperator {
  int nx, ny, nz;
  const float2* cx;
  const float2* cy;
  const float2* cz;
  const float2* b;
};
dim3 defect_grid(int nx, int ny, int nz);
// p_out = p_in + e (e may be null), r32 = float(b - A p_out), slot <- sum r^2;
// split: e and r32 in the colour-split layout
void launch_defect(cudaStream_t s, const DwOperator& A, const float2* pin, float2* pout,
                   const float* e, float* r32, const ReduceScratch& R, int slot, size_t hstride);
// TMA-fed k_defect (finest level with nx % 4 == 0): maps of p, e, b, cx, cy, cz.
struct DefectMaps {
  CUtensorMap p, e, b, cx, cy, cz;
  CUtensorMap e1;  // colour-split e: e holds the colour-0 half, e1 the colour-1 half
};
bool make_defect_maps(DefectMaps* m, const float2* p, const float* e, const float2* b,
                      const float2* cx, const float2* cy, const float2* cz, int nx, int ny,
                      int nz, size_t split_hstride);
int defect_tma_init();
void launch_defect_tma(cudaStream_t s, const DefectMaps& maps, int nx, int ny, int nz, bool use_e,
                       float2* pout, float* r32, const ReduceScratch& R, int slot, int* err,
                       size_t hstride);
void launch_to_dw(cudaStream_t s, const double* a, float2* out, size_t n);
// result[slot] = sum of x, summed in double-word per thread (FP32 pipes)
void launch_sum_dw(cudaStream_t s, const double* x, size_t n, const ReduceScratch& R, int slot);
// b -= result[mslot]/n (mslot < 0: unchanged), sum b^2 -> result[slot2], and
// when given the double-word copy bw and float(b) into r32 (colour-split when
// hstride != 0): one pass
void launch_rhs_prep(cudaStream_t s, double* b, size_t n, const ReduceScratch& R, int mslot,
                     int slot2, float2* bw, float* r32, int nx, int ny, size_t hstride);
void launch_dw_sum(cudaStream_t s, const float2* p, size_t n, const ReduceScratch& R, int slot);
// out += double(d)
void launch_dw_accumulate(cudaStream_t s, const float2* d, double* out, size_t n);
// out = double(p) - result[slot]/n
void launch_dw_out(cudaStream_t s, const float2* p, double* out, size_t n, const ReduceScratch& R,
                   int slot);

// ---- Adams-Bashforth momentum step (momentum.cu) ------------------------------
// Geometry and constants of one step.  Arrays are ghost-padded boxes sharing
// the strides sy, sz; kernels take the address of the reference's element
// (1,1,1) of each.
struct NsArgs {
  int nx, ny, nz, g;
  int64_t sy, sz;
  double dx, dy, dz, dt, re, fr, we, mu_12, gx, gy, gz, btn_g, btn_sf;
  // RN reciprocals of the constant divisors (dx, dy, dz, their squares, re)
  // and fast = 1 when all of them allow the division-free quotient
  // (fdiv.cuh); gterm = (g_d btn_g)/fr per axis, the gravity source
  double rdx, rdy, rdz, rdx2, rdy2, rdz2, rre;
  double gterm[3];
  int fast;
  int scheme;  // momentum advection: 0 second-order upwind, 1 QUICK
};
struct NsBc {
  int b[6];  // velbc type of the walls x-, x+, y-, y+, z-, z+ (1 no-slip, 2 slip, else none)
};
void launch_ns_diffusion(cudaStream_t s, const NsArgs& a, const double* const vel[3],
                         const double* rho, const double* mu, const double* delta,
                         const double* phi, const double* const nrm[3], const double* curv,
                         double* const out[3]);
void launch_ns_advance(cudaStream_t s, const NsArgs& a, const double* const old[3],
                       const double* const tmp[3], const double* const diff[3],
                       const double* const src_old[3], double* const src[3],
                       double* const now[3]);
void launch_velbc(cudaStream_t s, const NsArgs& a, const NsBc& bc, double* const vel[3]);
// ibm_bc's velocity forcing by the solid fraction (arrays at element (1,1,1))
void launch_ns_ibm(cudaStream_t s, const NsArgs& a, const double* solid, double w_body,
                   double* const vel[3]);
// ls_funs + rho_mu over the padded box (null outputs skipped)
void launch_ns_rho_mu(cudaStream_t s, const NsArgs& a, const double* phi, double ls_wid,
                      double rho_12, double* rho, double* mu, double* delta);
// max |now - tmp| -> R.result[kSlotMax] (bit pattern), sum (now - tmp)^2 -> R.result[kSlotSum]
void launch_ns_change(cudaStream_t s, const NsArgs& a, const double* const now[3],
                      const double* const tmp[3], const ReduceScratch& R);

// ---- compact-difference normals and curvature (ccd.cu) ------------------------
// One axis of CCD line solves over the padded box: L points per line, st
// apart; lines i1 + n1 i2 start at i1 s1 + i2 s2 from the box origin.
struct CcdArgs {
  int L, n1, n2;
  int64_t st, s1, s2;
  double h, h2, rh, rh2;  // spacing, its square and their RN reciprocals
  int fast;               // 1: quotients by h, h^2 from the reciprocals
};
// factor table of the CCD matrix for L points (14 doubles per point); work: 12 L doubles
void launch_ccd_decompose(cudaStream_t s, int L, double h, double* work, double* table);
// Up to three independent line passes in one launch (the grid's y index
// picks the pass): f' into S and f'' into SS along every line of each pass
// (box-origin pointers).
struct CcdBatch {
  int n;
  CcdArgs c[3];
  const double* table[3];
  const double* f[3];
  double* S[3];
  double* SS[3];
};
void launch_ccd_lines(cudaStream_t s, const CcdBatch& b);
// zero-gradient ghosts (bc) of up to four arrays at element (1,1,1) (null = none)
void launch_ccd_bc(cudaStream_t s, const NsArgs& a, double* const f[4]);
// curvature on the interior from phi_x, phi_y, phi_z and the second derivatives
// fxx, fyy, fzz, fxy, fxz, fyz (arrays at element (1,1,1))
void launch_curvature(cudaStream_t s, const NsArgs& a, const double* const d1[3],
                      const double* const d2[6], double* curv);
// mass_preserving_level_set: result[kSlotSum] = ls_mv mass, [kSlotSum + 1] =
// the lambda denominator; g = the compact gradient of phi (g[2] null in 2D)
void launch_mpls_sums(cudaStream_t s, const NsArgs& a, const double* phi, const double* const g[3],
                      double ls_wid, double rho_12, double dv, const ReduceScratch& R);
// one sweep of vof_wlic_solver along axis ax (flux, then the cell update;
// the caller applies bc): arrays at element (1,1,1), flux a padded scratch
void launch_wlic(cudaStream_t s, const NsArgs& a, int ax, double* vof, const double* vof_old,
                 const double* vel, const double* phi, double* flux);
// phi += lam delta |grad phi| on the interior
void launch_mpls_update(cudaStream_t s, const NsArgs& a, double* phi, const double* const g[3],
                        double ls_wid, double lam);

}  // namespace gbmg
