// Host side and C ABI of the momentum step and the interface entry points:
// gbmg_ns_ab_step / gbmg_ns_ab_predict (ns_ab_solver_SOR, "Two phase flows/
// newOpenMP/2D/src/ns_solver/admas_bashforth_solver.f90:19-92"), velbc,
// the CCD normals and curvature (curv, surface_norms), rho_mu, bc, the MPLS
// mass correction, the CLSVOF volume-fraction transport and the immersed-
// boundary forcing, on the handle of the pressure solve (handle.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "fdiv.cuh"
#include "handle.h"

using namespace gbmg;
using namespace gbmg::host;

namespace {


// ---- Adams-Bashforth momentum step -------------------------------------------
// Arrays of the step, in the order of gbmg_ns_fields.
enum NsSlot {
  kNsU, kNsV, kNsW, kNsUo, kNsVo, kNsWo, kNsSu, kNsSv, kNsSw, kNsSuo, kNsSvo, kNsSwo,
  kNsRho, kNsMu, kNsDelta, kNsPhi, kNsNx, kNsNy, kNsNz, kNsCurv, kNsFields
};
// scratch buffers after the staging slots: vel%tmp (3), velsrc%tmp (3)
constexpr int kNsTmp = kNsFields, kNsDiff = kNsFields + 3;

const gbmg_field& ns_field(const gbmg_ns_fields* f, int slot) {
  const gbmg_field* all[kNsFields] = {&f->u,      &f->v,      &f->w,      &f->u_old, &f->v_old,
                                      &f->w_old,  &f->su,     &f->sv,     &f->sw,    &f->su_old,
                                      &f->sv_old, &f->sw_old, &f->rho,    &f->mu,    &f->delta,
                                      &f->phi,    &f->nrm_x,  &f->nrm_y,  &f->nrm_z, &f->curv};
  return *all[slot];
}

// Offset of element (1,1,1) of the reference's indices from a field's
// address: faces are addressed at their face 0 (u(0,1,1), v(1,0,1), w(1,1,0)).
int64_t ns_origin(int slot, int64_t sy, int64_t sz) {
  const int axis = slot < kNsRho ? slot % 3 : -1;
  return axis == 0 ? 1 : axis == 1 ? sy : axis == 2 ? sz : 0;
}

struct NsPlan {
  NsArgs a{};
  NsBc bc{};
  int64_t lo = 0, hi = 0;  // element offsets of the padded box from element (1,1,1)
  double* base[kNsFields + 6] = {};
  bool used[kNsFields] = {};
};

int ns_buffer(gbmg_handle* h, int slot, size_t n) {
  if (h->ns_n[slot] < n) {
    dfree(h->ns_buf[slot]);
    h->ns_n[slot] = 0;
    GB_TRY(dmalloc(h, &h->ns_buf[slot], n));
    h->ns_n[slot] = n;
  }
  return GBMG_OK;
}

// Validate the arrays a call uses, fill the kernel arguments and make every
// used array device-resident (host memory: staged copies of the padded box).
int ns_prepare(gbmg_handle* h, const gbmg_ns_params* prm, const gbmg_ns_fields* f, int mem,
               const bool (&used)[kNsFields], const bool (&copy_in)[kNsFields], NsPlan* P,
               bool step_scratch = true) {
  const gbmg_grid& g = h->grid;
  const bool three = g.nz > 1;
  if (!prm || !f) { h->err = "null parameters"; return GBMG_INVALID_ARG; }
  const int gh = prm->ghost;
  if (gh < 2 || g.nx < gh + 1 || g.ny < gh + 1 || (three && g.nz < gh + 1)) {
    h->err = "the momentum step needs ghost >= 2 and at least ghost + 1 cells per axis";
    return GBMG_INVALID_ARG;
  }
  if (!(prm->dt > 0) || !(prm->re > 0) || !(prm->fr > 0) || (prm->btn_sf != 0 && !(prm->we > 0))) {
    h->err = "dt, re, fr (and we with surface tension) must be > 0";
    return GBMG_INVALID_ARG;
  }
  int64_t sy = 0, sz = 0;
  for (int i = 0; i < kNsFields; ++i) {
    if (!used[i]) continue;
    const gbmg_field& fi = ns_field(f, i);
    if (!fi.data) { h->err = "a field the momentum step reads or writes is NULL"; return GBMG_INVALID_ARG; }
    if (!sy) { sy = fi.sy; sz = fi.sz; }
    if (fi.sy != sy || (three && fi.sz != sz)) {
      h->err = "the arrays of the momentum step must share their strides";
      return GBMG_INVALID_ARG;
    }
  }
  if (sy < g.nx + 2 * gh || (three && sz < sy * (g.ny + 2 * gh))) {
    h->err = "strides too small for the ghost-padded box";
    return GBMG_INVALID_ARG;
  }
  NsArgs& a = P->a;
  a.nx = g.nx; a.ny = g.ny; a.nz = g.nz; a.g = gh;
  a.sy = sy; a.sz = three ? sz : 0;
  a.dx = g.dx; a.dy = g.dy; a.dz = g.dz;
  a.dt = prm->dt; a.re = prm->re; a.fr = prm->fr; a.we = prm->we; a.mu_12 = prm->mu_12;
  a.gx = prm->gx; a.gy = prm->gy; a.gz = prm->gz; a.btn_g = prm->btn_g; a.btn_sf = prm->btn_sf;
  // reciprocals of the constant divisors (IEEE divisions, so RN(1/b)), and
  // the gravity source (g_d btn_g)/fr as the reference evaluates it per cell
  const double dvs[7] = {g.dx, g.dy, g.dz, g.dx * g.dx, g.dy * g.dy, g.dz * g.dz, prm->re};
  double* rcp[7] = {&a.rdx, &a.rdy, &a.rdz, &a.rdx2, &a.rdy2, &a.rdz2, &a.rre};
  a.fast = 1;
  for (int i = 0; i < 7; ++i) {
    *rcp[i] = 1.0 / dvs[i];
    if (!fdiv_divisor_ok(dvs[i])) a.fast = 0;
  }
  a.scheme = prm->adv_scheme;
  if (a.scheme != 0 && a.scheme != 1) {
    h->err = "adv_scheme must be 0 (second-order upwind) or 1 (QUICK)";
    return GBMG_INVALID_ARG;
  }
  a.gterm[0] = prm->gx * prm->btn_g / prm->fr;
  a.gterm[1] = prm->gy * prm->btn_g / prm->fr;
  a.gterm[2] = prm->gz * prm->btn_g / prm->fr;
  for (int i = 0; i < 6; ++i) P->bc.b[i] = prm->bc[i];
  P->lo = -(int64_t)gh - gh * a.sy - (three ? gh * a.sz : 0);
  P->hi = (int64_t)(g.nx + gh - 1) + (g.ny + gh - 1) * a.sy + (three ? (g.nz + gh - 1) * a.sz : 0);
  const size_t span = (size_t)(P->hi - P->lo + 1);
  for (int i = 0; i < kNsFields; ++i) {
    P->used[i] = used[i];
    if (!used[i]) continue;
    double* b = ns_field(f, i).data + ns_origin(i, a.sy, a.sz);
    if (mem == GBMG_MEM_DEVICE) {
      P->base[i] = b;
      continue;
    }
    GB_TRY(ns_buffer(h, i, span));
    if (copy_in[i])
      GB_CUDA(h, cudaMemcpyAsync(h->ns_buf[i], b + P->lo, span * sizeof(double),
                                 cudaMemcpyHostToDevice, h->stream));
    P->base[i] = h->ns_buf[i] - P->lo;
  }
  // vel%tmp and velsrc%tmp of the momentum step (not for the other calls)
  for (int c = 0; c < 6 && step_scratch; ++c) {
    if (!three && c % 3 == 2) continue;
    GB_TRY(ns_buffer(h, kNsTmp + c, span));
    P->base[kNsTmp + c] = h->ns_buf[kNsTmp + c] - P->lo;
  }
  return GBMG_OK;
}

int ns_finish(gbmg_handle* h, const gbmg_ns_fields* f, int mem, const NsPlan& P,
              const bool (&copy_out)[kNsFields]) {
  if (mem != GBMG_MEM_HOST) return GBMG_OK;
  const size_t span = (size_t)(P.hi - P.lo + 1);
  for (int i = 0; i < kNsFields; ++i) {
    if (!P.used[i] || !copy_out[i]) continue;
    double* b = ns_field(f, i).data + ns_origin(i, P.a.sy, P.a.sz);
    GB_CUDA(h, cudaMemcpyAsync(b + P.lo, P.base[i] + P.lo, span * sizeof(double),
                               cudaMemcpyDeviceToHost, h->stream));
  }
  return GBMG_OK;
}

// ns_linearize (vel%tmp = vel%now over the padded box), ns_ab_setup and
// ns_ab_predictor, then velbc on vel%now.
int ns_pass(gbmg_handle* h, const NsPlan& P) {
  const cudaStream_t s = h->stream;
  const bool three = P.a.nz > 1;
  const size_t span = (size_t)(P.hi - P.lo + 1);
  for (int c = 0; c < (three ? 3 : 2); ++c)
    GB_CUDA(h, cudaMemcpyAsync(P.base[kNsTmp + c] + P.lo, P.base[kNsU + c] + P.lo,
                               span * sizeof(double), cudaMemcpyDeviceToDevice, s));
  const double* old[3] = {P.base[kNsUo], P.base[kNsVo], P.base[kNsWo]};
  const double* tmp[3] = {P.base[kNsTmp], P.base[kNsTmp + 1], P.base[kNsTmp + 2]};
  const double* diff[3] = {P.base[kNsDiff], P.base[kNsDiff + 1], P.base[kNsDiff + 2]};
  const double* so[3] = {P.base[kNsSuo], P.base[kNsSvo], P.base[kNsSwo]};
  double* src[3] = {P.base[kNsSu], P.base[kNsSv], P.base[kNsSw]};
  double* now[3] = {P.base[kNsU], P.base[kNsV], P.base[kNsW]};
  LAUNCH(h, GBMG_PROF_MOMENTUM, launch_ns_advance(s, P.a, old, tmp, diff, so, src, now));
  LAUNCH(h, GBMG_PROF_MOMENTUM, launch_velbc(s, P.a, P.bc, now));
  return check_launch(h, "momentum predictor");
}

int ns_diffusion(gbmg_handle* h, const NsPlan& P) {
  const double* vel[3] = {P.base[kNsUo], P.base[kNsVo], P.base[kNsWo]};
  const double* nrm[3] = {P.base[kNsNx], P.base[kNsNy], P.base[kNsNz]};
  double* out[3] = {P.base[kNsDiff], P.base[kNsDiff + 1], P.base[kNsDiff + 2]};
  LAUNCH(h, GBMG_PROF_MOMENTUM,
         launch_ns_diffusion(h->stream, P.a, vel, P.base[kNsRho], P.base[kNsMu],
                             P.base[kNsDelta], P.base[kNsPhi], nrm, P.base[kNsCurv], out));
  return check_launch(h, "momentum sources");
}

void ns_used(const gbmg_grid& g, const gbmg_ns_params* prm, bool (&used)[kNsFields],
             bool (&in)[kNsFields], bool (&out)[kNsFields]) {
  const bool three = g.nz > 1, sf = prm && prm->btn_sf != 0.0;
  for (int i = 0; i < kNsFields; ++i) {
    const bool is_w = i < kNsRho && i % 3 == 2;
    used[i] = !(is_w && !three) && !(i == kNsNz && !three) &&
              !(i >= kNsNx && i <= kNsCurv && !sf);
    in[i] = used[i];  // velsrc%now round-trips its ghosts
    out[i] = used[i] && (i <= kNsW || (i >= kNsSu && i <= kNsSw));
  }
}

// Compact-difference normals and curvature (curv + surface_norms): scratch
// slots after the momentum step's: the six second derivatives and a dummy
// second derivative, then a factor table per axis and the factoring work.
constexpr int kCcdD2 = kNsDiff + 3, kCcdDummy = kCcdD2 + 6, kCcdTable = kCcdDummy + 1,
              kCcdWork = kCcdTable + 3, kCcdSpare = kCcdWork + 1;  // two spare fields

// One CCD line pass: its arguments, and the axis's factor table (made by
// one sequential thread, so once, and kept while the line length and spacing
// stay the same).
int ccd_pass(gbmg_handle* h, const NsPlan& P, int axis, CcdArgs* out) {
  const NsArgs& a = P.a;
  const bool three = a.nz > 1;
  const int px = a.nx + 2 * a.g, py = a.ny + 2 * a.g, pz = three ? a.nz + 2 * a.g : 1;
  const int ext[3] = {px, py, pz};
  const int64_t str[3] = {1, a.sy, three ? a.sz : 0};
  const double hs[3] = {a.dx, a.dy, a.dz};
  CcdArgs c{};
  c.L = ext[axis];
  c.st = str[axis];
  const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
  c.n1 = ext[a1]; c.s1 = str[a1];
  c.n2 = ext[a2]; c.s2 = str[a2];
  c.h = hs[axis];
  c.h2 = c.h * c.h;
  c.rh = 1.0 / c.h;
  c.rh2 = 1.0 / c.h2;
  c.fast = fdiv_divisor_ok(c.h) && fdiv_divisor_ok(c.h2);
  if (h->ccd_L[axis] != c.L || h->ccd_h[axis] != c.h) {
    h->ccd_L[axis] = 0;
    GB_TRY(ns_buffer(h, kCcdTable + axis, (size_t)14 * c.L));
    GB_TRY(ns_buffer(h, kCcdWork, (size_t)12 * c.L));
    LAUNCH(h, GBMG_PROF_MOMENTUM,
           launch_ccd_decompose(h->stream, c.L, c.h, h->ns_buf[kCcdWork],
                                h->ns_buf[kCcdTable + axis]));
    GB_TRY(check_launch(h, "ccd factors"));
    h->ccd_L[axis] = c.L;
    h->ccd_h[axis] = c.h;
  }
  *out = c;
  return GBMG_OK;
}

// Independent line passes (axis, f -> f', f'') in one launch; arrays at
// element (1,1,1), the second-derivative outputs distinct.
int ccd_passes(gbmg_handle* h, const NsPlan& P, int n, const int* axes,
               const double* const* f, double* const* S, double* const* SS) {
  CcdBatch b{};
  b.n = n;
  for (int i = 0; i < n; ++i) {
    GB_TRY(ccd_pass(h, P, axes[i], &b.c[i]));
    b.table[i] = h->ns_buf[kCcdTable + axes[i]];
    b.f[i] = f[i] + P.lo;
    b.S[i] = S[i] + P.lo;
    b.SS[i] = SS[i] + P.lo;
  }
  LAUNCH(h, GBMG_PROF_MOMENTUM, launch_ccd_lines(h->stream, b));
  return check_launch(h, "ccd lines");
}

// Padded cell arrays of the momentum step's layout: the plan of ns_prepare
// for the given slots (prm supplies the ghost count and mu_12).
int ns_cells(gbmg_handle* h, const gbmg_ns_params* prm, gbmg_ns_fields* f, int mem,
             const int* slots, const bool* outs, int n, NsPlan* P, bool (&out)[kNsFields]) {
  if (!prm) { h->err = "null parameters"; return GBMG_INVALID_ARG; }
  bool used[kNsFields] = {}, in[kNsFields] = {};
  for (int i = 0; i < kNsFields; ++i) out[i] = false;
  for (int i = 0; i < n; ++i) {
    used[slots[i]] = in[slots[i]] = true;
    out[slots[i]] = outs[i];
  }
  gbmg_ns_params q = *prm;
  q.dt = q.re = q.fr = 1.0;
  q.btn_sf = 0.0;
  return ns_prepare(h, &q, f, mem, used, in, P, false);
}

}  // namespace

extern "C" {

int gbmg_ns_ab_step(gbmg_handle* h, const gbmg_ns_params* prm, const gbmg_ns_fields* f, int mem,
                    gbmg_ns_stats* stats) {
  GB_TRY(begin(h));
  gbmg_ns_stats local{};
  gbmg_ns_stats* st = stats ? stats : &local;
  std::memset(st, 0, sizeof(*st));
  if (!prm || !f) { h->err = "null parameters"; return GBMG_INVALID_ARG; }
  if (!h->coef_ready || !h->rho_ready) {
    h->err = "the momentum step needs the new density: call gbmg_set_rho or gbmg_set_phi first";
    return GBMG_STATE_ERROR;
  }
  const gbmg_grid& g = h->grid;
  const bool three = g.nz > 1;
  bool used[kNsFields], in[kNsFields], out[kNsFields];
  ns_used(g, prm, used, in, out);
  if (prm->iterations < 1 || !(prm->p_tol > 0)) {
    h->err = "iterations must be >= 1 and p_tol > 0";
    return GBMG_INVALID_ARG;
  }
  GB_TRY(validate_field(h, f->p, "p"));
  const cudaStream_t s = h->stream;
  GB_CUDA(h, cudaEventRecord(h->ev0, s));
  NsPlan P;
  GB_TRY(ns_prepare(h, prm, f, mem, used, in, &P));
  GB_TRY(upload(h, f->p, g.nx, g.ny, g.nz, mem, h->p));
  GB_TRY(ns_diffusion(h, P));
  gbmg_field dfield[3] = {{P.base[kNsU] - 1, P.a.sy, P.a.sz},
                          {P.base[kNsV] - P.a.sy, P.a.sy, P.a.sz},
                          {three ? P.base[kNsW] - P.a.sz : nullptr, P.a.sy, P.a.sz}};
  double* now[3] = {P.base[kNsU], P.base[kNsV], P.base[kNsW]};
  int worst = GBMG_OK;
  for (int it = 0; it < prm->iterations; ++it) {
    GB_TRY(ns_pass(h, P));
    gbmg_stats ps{};
    const int rc = project_device(h, dfield, three, prm->dt, prm->p_tol, &ps);
    if (rc != GBMG_OK && rc != GBMG_NOT_CONVERGED && rc != GBMG_DIVERGED) return rc;
    if (rc > worst) worst = rc;
    st->cycles += ps.cycles;
    st->max_rel_residual = std::max(st->max_rel_residual, ps.rel_residual);
    LAUNCH(h, GBMG_PROF_MOMENTUM, launch_velbc(s, P.a, P.bc, now));
    GB_TRY(check_launch(h, "velbc"));
  }
  const double* tmp[3] = {P.base[kNsTmp], P.base[kNsTmp + 1], P.base[kNsTmp + 2]};
  const double* nowc[3] = {now[0], now[1], now[2]};
  LAUNCH(h, GBMG_PROF_MOMENTUM, launch_ns_change(s, P.a, nowc, tmp, h->red));
  GB_TRY(check_launch(h, "velocity change"));
  GB_CUDA(h, cudaMemcpyAsync(h->host_res, h->red.result, kRedSlots * sizeof(double),
                             cudaMemcpyDeviceToHost, s));
  GB_TRY(ns_finish(h, f, mem, P, out));
  GB_TRY(download(h, h->p, g.nx, g.ny, g.nz, mem, f->p));
  GB_CUDA(h, cudaEventRecord(h->ev1, s));
  GB_CUDA(h, cudaEventSynchronize(h->ev1));
  double mx = 0.0;
  std::memcpy(&mx, &h->host_res[kSlotMax], sizeof(double));
  const double cnt = (three ? 3.0 : 2.0) * g.nx * g.ny * g.nz;
  st->linf = mx;
  st->l2f = std::sqrt(h->host_res[kSlotSum] / cnt);
  st->status = worst;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  st->ms = ms;
  return worst;
}

int gbmg_ns_ab_predict(gbmg_handle* h, const gbmg_ns_params* prm, const gbmg_ns_fields* f,
                       int mem) {
  GB_TRY(begin(h));
  bool used[kNsFields], in[kNsFields], out[kNsFields];
  ns_used(h->grid, prm, used, in, out);
  NsPlan P;
  GB_TRY(ns_prepare(h, prm, f, mem, used, in, &P));
  GB_TRY(ns_diffusion(h, P));
  GB_TRY(ns_pass(h, P));
  GB_TRY(ns_finish(h, f, mem, P, out));
  GB_CUDA(h, cudaStreamSynchronize(h->stream));
  return GBMG_OK;
}

int gbmg_ns_velbc(gbmg_handle* h, const gbmg_ns_params* prm, gbmg_field u, gbmg_field v,
                  gbmg_field w, int mem) {
  GB_TRY(begin(h));
  gbmg_ns_fields f{};
  f.u = u; f.v = v; f.w = w;
  bool used[kNsFields] = {}, in[kNsFields] = {}, out[kNsFields] = {};
  const bool three = h->grid.nz > 1;
  for (int c = 0; c < (three ? 3 : 2); ++c) used[c] = in[c] = out[c] = true;
  NsPlan P;
  gbmg_ns_params q = prm ? *prm : gbmg_ns_params{};
  if (prm) { q.dt = q.re = q.fr = 1.0; q.btn_sf = 0.0; }  // velbc reads only ghost and bc
  GB_TRY(ns_prepare(h, prm ? &q : nullptr, &f, mem, used, in, &P, false));
  double* now[3] = {P.base[kNsU], P.base[kNsV], P.base[kNsW]};
  LAUNCH(h, GBMG_PROF_MOMENTUM, launch_velbc(h->stream, P.a, P.bc, now));
  GB_TRY(check_launch(h, "velbc"));
  GB_TRY(ns_finish(h, &f, mem, P, out));
  GB_CUDA(h, cudaStreamSynchronize(h->stream));
  return GBMG_OK;
}

int gbmg_ns_curvature(gbmg_handle* h, const gbmg_ns_params* prm, gbmg_field phi,
                      gbmg_field nrm_x, gbmg_field nrm_y, gbmg_field nrm_z, gbmg_field curv,
                      int mem) {
  GB_TRY(begin(h));
  if (!prm) { h->err = "null parameters"; return GBMG_INVALID_ARG; }
  const bool three = h->grid.nz > 1;
  gbmg_ns_fields f{};
  f.phi = phi; f.nrm_x = nrm_x; f.nrm_y = nrm_y; f.nrm_z = nrm_z; f.curv = curv;
  bool used[kNsFields] = {}, in[kNsFields] = {}, out[kNsFields] = {};
  const int slots[5] = {kNsPhi, kNsNx, kNsNy, kNsNz, kNsCurv};
  for (int i = 0; i < 5; ++i) {
    if (slots[i] == kNsNz && !three) continue;
    used[slots[i]] = in[slots[i]] = true;
    out[slots[i]] = slots[i] != kNsPhi;
  }
  gbmg_ns_params q = *prm;
  q.dt = q.re = q.fr = 1.0;  // only ghost is read
  q.btn_sf = 0.0;
  NsPlan P;
  GB_TRY(ns_prepare(h, &q, &f, mem, used, in, &P, false));
  const size_t span = (size_t)(P.hi - P.lo + 1);
  double* d2[9];
  for (int i = 0; i < 9; ++i) {
    const int slot = i < 7 ? kCcdD2 + i : kCcdSpare + (i - 7);
    GB_TRY(ns_buffer(h, slot, span));
    d2[i] = h->ns_buf[slot] - P.lo;
  }
  double* nx = P.base[kNsNx];
  double* ny = P.base[kNsNy];
  double* nz = three ? P.base[kNsNz] : nullptr;
  const double* ph = P.base[kNsPhi];
  // surface_norms: first and second derivatives of phi along each axis (one
  // launch), then the cross derivatives from phi_x and phi_y before any bc
  // (one launch; their second derivatives are discarded, each its own buffer)
  {
    const int axes[3] = {0, 1, 2};
    const double* src[3] = {ph, ph, ph};
    double* S[3] = {nx, ny, nz};
    double* SS[3] = {d2[0], d2[1], d2[2]};
    GB_TRY(ccd_passes(h, P, three ? 3 : 2, axes, src, S, SS));
  }
  {
    const int axes[3] = {1, 2, 2};
    const double* src[3] = {nx, nx, ny};
    double* S[3] = {d2[3], d2[4], d2[5]};
    double* SS[3] = {d2[6], d2[7], d2[8]};
    GB_TRY(ccd_passes(h, P, three ? 3 : 1, axes, src, S, SS));
  }
  const double* d1c[3] = {nx, ny, nz};
  const double* d2c[6] = {d2[0], d2[1], d2[2], d2[3], d2[4], d2[5]};
  LAUNCH(h, GBMG_PROF_MOMENTUM, launch_curvature(h->stream, P.a, d1c, d2c, P.base[kNsCurv]));
  double* bcs[4] = {nx, ny, nz, P.base[kNsCurv]};
  LAUNCH(h, GBMG_PROF_MOMENTUM, launch_ccd_bc(h->stream, P.a, bcs));
  GB_TRY(check_launch(h, "curvature"));
  GB_TRY(ns_finish(h, &f, mem, P, out));
  GB_CUDA(h, cudaStreamSynchronize(h->stream));
  return GBMG_OK;
}

int gbmg_ns_rho_mu(gbmg_handle* h, const gbmg_ns_params* prm, gbmg_field phi, double ls_wid,
                   double rho_12, gbmg_field rho, gbmg_field mu, gbmg_field delta, int mem) {
  GB_TRY(begin(h));
  if (!(ls_wid > 0) || !(rho_12 > 0)) { h->err = "ls_wid and rho_12 must be > 0"; return GBMG_INVALID_ARG; }
  gbmg_ns_fields f{};
  f.phi = phi; f.rho = rho; f.mu = mu; f.delta = delta;
  int slots[4] = {kNsPhi};
  bool outs[4] = {false};
  int n = 1;
  const gbmg_field* o[3] = {&rho, &mu, &delta};
  const int os[3] = {kNsRho, kNsMu, kNsDelta};
  for (int i = 0; i < 3; ++i)
    if (o[i]->data) { slots[n] = os[i]; outs[n++] = true; }
  NsPlan P;
  bool out[kNsFields];
  GB_TRY(ns_cells(h, prm, &f, mem, slots, outs, n, &P, out));
  LAUNCH(h, GBMG_PROF_MOMENTUM,
         launch_ns_rho_mu(h->stream, P.a, P.base[kNsPhi], ls_wid, rho_12, P.base[kNsRho],
                          P.base[kNsMu], P.base[kNsDelta]));
  GB_TRY(check_launch(h, "rho_mu"));
  GB_TRY(ns_finish(h, &f, mem, P, out));
  GB_CUDA(h, cudaStreamSynchronize(h->stream));
  return GBMG_OK;
}

int gbmg_ns_bc(gbmg_handle* h, const gbmg_ns_params* prm, gbmg_field a, int mem) {
  GB_TRY(begin(h));
  gbmg_ns_fields f{};
  f.phi = a;
  const int slots[1] = {kNsPhi};
  const bool outs[1] = {true};
  NsPlan P;
  bool out[kNsFields];
  GB_TRY(ns_cells(h, prm, &f, mem, slots, outs, 1, &P, out));
  double* arr[4] = {P.base[kNsPhi], nullptr, nullptr, nullptr};
  LAUNCH(h, GBMG_PROF_MOMENTUM, launch_ccd_bc(h->stream, P.a, arr));
  GB_TRY(check_launch(h, "bc"));
  GB_TRY(ns_finish(h, &f, mem, P, out));
  GB_CUDA(h, cudaStreamSynchronize(h->stream));
  return GBMG_OK;
}

int gbmg_ns_mass_correct(gbmg_handle* h, const gbmg_ns_params* prm, gbmg_field phi,
                         double ls_wid, double rho_12, double imass, int iterations, int mem,
                         double* mass) {
  GB_TRY(begin(h));
  if (!(ls_wid > 0) || !(rho_12 > 0) || iterations < 0) {
    h->err = "ls_wid and rho_12 must be > 0 and iterations >= 0";
    return GBMG_INVALID_ARG;
  }
  const bool three = h->grid.nz > 1;
  gbmg_ns_fields f{};
  f.phi = phi;
  const int slots[1] = {kNsPhi};
  const bool outs[1] = {iterations > 0};
  NsPlan P;
  bool out[kNsFields];
  GB_TRY(ns_cells(h, prm, &f, mem, slots, outs, 1, &P, out));
  const size_t span = (size_t)(P.hi - P.lo + 1);
  double* gr[3] = {nullptr, nullptr, nullptr};
  for (int c = 0; c < (three ? 3 : 2); ++c) {
    GB_TRY(ns_buffer(h, kCcdD2 + c, span));
    gr[c] = h->ns_buf[kCcdD2 + c] - P.lo;
  }
  GB_TRY(ns_buffer(h, kCcdD2 + 6, span));
  GB_TRY(ns_buffer(h, kCcdSpare, span));
  GB_TRY(ns_buffer(h, kCcdSpare + 1, span));
  double* dummy = h->ns_buf[kCcdD2 + 6] - P.lo;
  double* dummy2 = h->ns_buf[kCcdSpare] - P.lo;
  double* dummy3 = h->ns_buf[kCcdSpare + 1] - P.lo;
  double* ph = P.base[kNsPhi];
  const gbmg_grid& g = h->grid;
  const double dv = three ? g.dx * g.dy * g.dz : g.dx * g.dy;
  const cudaStream_t s = h->stream;
  double m = 0.0;
  const int passes = iterations > 0 ? iterations : 1;
  for (int it = 0; it < passes; ++it) {
    // ls_mv, and before a correction surface_norms' gradient of phi
    const bool correct = iterations > 0;
    if (correct) {
      const int axes[3] = {0, 1, 2};
      const double* src[3] = {ph, ph, ph};
      double* SS[3] = {dummy, dummy2, dummy3};
      GB_TRY(ccd_passes(h, P, three ? 3 : 2, axes, src, gr, SS));
    }
    const double* gc[3] = {correct ? gr[0] : nullptr, gr[1], gr[2]};
    LAUNCH(h, GBMG_PROF_MOMENTUM, launch_mpls_sums(s, P.a, ph, gc, ls_wid, rho_12, dv, h->red));
    GB_TRY(check_launch(h, "mass sums"));
    GB_CUDA(h, cudaMemcpyAsync(h->host_res, h->red.result, kRedSlots * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    GB_CUDA(h, cudaStreamSynchronize(s));
    m = h->host_res[kSlotSum];
    if (!correct) break;
    const double den = h->host_res[kSlotSum + 1];
    if (!(den > 0.0) || !std::isfinite(den)) {
      // no cell inside the interface band (or a non-finite field): the
      // reference's lambda would be a division by zero
      h->err = "mass correction: no interface cells (sum of delta^2 |grad phi| is not > 0)";
      return GBMG_INVALID_ARG;
    }
    const double lam = (imass - m) / den;
    const double* gcc[3] = {gr[0], gr[1], gr[2]};
    LAUNCH(h, GBMG_PROF_MOMENTUM, launch_mpls_update(s, P.a, ph, gcc, ls_wid, lam));
    double* arr[4] = {ph, nullptr, nullptr, nullptr};
    LAUNCH(h, GBMG_PROF_MOMENTUM, launch_ccd_bc(s, P.a, arr));
    GB_TRY(check_launch(h, "mass correction"));
  }
  // the mass measured last: before the last correction, as the reference
  // leaves p%glb%mass (or of phi itself when iterations = 0)
  if (mass) *mass = m;
  GB_TRY(ns_finish(h, &f, mem, P, out));
  GB_CUDA(h, cudaStreamSynchronize(s));
  return GBMG_OK;
}

int gbmg_ns_vof_advect(gbmg_handle* h, const gbmg_ns_params* prm, gbmg_field vof,
                       gbmg_field vof_old, gbmg_field u_old, gbmg_field v_old, gbmg_field w_old,
                       gbmg_field phi, int mem) {
  GB_TRY(begin(h));
  if (!prm || !(prm->dt > 0)) { h->err = "dt must be > 0"; return GBMG_INVALID_ARG; }
  const bool three = h->grid.nz > 1;
  // the cell arrays ride in the plan's cell slots (vof, vof_old, phi), the
  // face velocities in the old-velocity slots
  gbmg_ns_fields f{};
  f.rho = vof; f.mu = vof_old; f.phi = phi;
  f.u_old = u_old; f.v_old = v_old; f.w_old = w_old;
  int slots[6] = {kNsRho, kNsMu, kNsPhi, kNsUo, kNsVo, kNsWo};
  const bool outs[6] = {true, false, false, false, false, false};
  NsPlan P;
  bool out[kNsFields];
  GB_TRY(ns_cells(h, prm, &f, mem, slots, outs, three ? 6 : 5, &P, out));
  P.a.dt = prm->dt;
  const size_t span = (size_t)(P.hi - P.lo + 1);
  GB_TRY(ns_buffer(h, kCcdD2, span));
  double* flux = h->ns_buf[kCcdD2] - P.lo;
  double* vf = P.base[kNsRho];
  const double* vel[3] = {P.base[kNsUo], P.base[kNsVo], P.base[kNsWo]};
  for (int ax = 0; ax < (three ? 3 : 2); ++ax) {
    LAUNCH(h, GBMG_PROF_MOMENTUM,
           launch_wlic(h->stream, P.a, ax, vf, P.base[kNsMu], vel[ax], P.base[kNsPhi], flux));
    double* arr[4] = {vf, nullptr, nullptr, nullptr};
    LAUNCH(h, GBMG_PROF_MOMENTUM, launch_ccd_bc(h->stream, P.a, arr));
    GB_TRY(check_launch(h, "vof sweep"));
  }
  GB_TRY(ns_finish(h, &f, mem, P, out));
  GB_CUDA(h, cudaStreamSynchronize(h->stream));
  return GBMG_OK;
}

int gbmg_ns_ibm(gbmg_handle* h, const gbmg_ns_params* prm, gbmg_field solid, double w_body,
                gbmg_field u, gbmg_field v, gbmg_field w, int mem) {
  GB_TRY(begin(h));
  const bool three = h->grid.nz > 1;
  gbmg_ns_fields f{};
  f.rho = solid; f.u = u; f.v = v; f.w = w;
  const int slots[4] = {kNsRho, kNsU, kNsV, kNsW};
  const bool outs[4] = {true, true, true, true};
  NsPlan P;
  bool out[kNsFields];
  GB_TRY(ns_cells(h, prm, &f, mem, slots, outs, three ? 4 : 3, &P, out));
  double* arr[4] = {P.base[kNsRho], nullptr, nullptr, nullptr};
  LAUNCH(h, GBMG_PROF_MOMENTUM, launch_ccd_bc(h->stream, P.a, arr));  // bc(solid)
  double* vel[3] = {P.base[kNsU], P.base[kNsV], P.base[kNsW]};
  LAUNCH(h, GBMG_PROF_MOMENTUM, launch_ns_ibm(h->stream, P.a, P.base[kNsRho], w_body, vel));
  GB_TRY(check_launch(h, "ibm"));
  GB_TRY(ns_finish(h, &f, mem, P, out));
  GB_CUDA(h, cudaStreamSynchronize(h->stream));
  return GBMG_OK;
}

}  // extern "C"
