// cbns_kernels.cu — sm_103a kernels of one RK3 stage of the cbns3d right-hand side.
//
// One stage (src/cbns3d.cpp:203-240) is five launches over a flattened tile
// table that may span many solves:
//   k_inviscid<0,1,2>  characteristic WENO5 + Roe eigenvectors + local Lax-Friedrichs
//                      flux at every face normal to x, y, z (Block3d::rec_riemann_x/y/z)
//   k_viscous          4th-order velocity/temperature gradients, Sutherland mu, and the
//                      nine distinct terms of the viscous fluxes Ev, Fv, Gv (six
//                      stresses, three energy fluxes) on the NGV ring
//                      (calc_viscous_terms + calc_viscous_flux)
//   k_update           flux differences + 4th-order viscous divergence, SSP-RK3 update,
//   (k_update_f32)     then the periodic ghost fill and the primitive recovery of the
//                      new state, written to the cell and all its ghost images
//                      (calc_viscous_flux_contribution tail, update_rk3,
//                      boundary_condition, calc_primitive)
// plus, once per step, k_dt_reduce + k_dt_finalize (calc_dt, the MIN all-reduce,
// the clip to t_end and is_finished).
//
// Binary64 solves run the kernels in binary64.  GB300 issues binary64 at about
// 1/64 of the binary32 rate (about 2 DFMA per clock per SM), so these kernels
// are bound by the FP64 pipe and are written to issue few binary64
// instructions: the eigenvector products use the structure of L and R for
// axis-aligned normals, the stencil projections are shared by the two biased
// reconstructions of a face, WENO5 works on first differences, the ten WENO
// normalisations of a face share one division, and divisions by constants
// become multiplications.  These rewrites change rounding only (a few ulp per
// operation); the results stay within the 1e-11 relative tolerance of the
// reference after 100 steps.  FP32-mixed solves run the same kernels
// instantiated for binary32 on a perturbation of the state about the free
// stream, with the binary64 state and its RK3 combination kept in binary64;
// their face kernels (k_inviscid_x2<D>) compute two faces per thread in the
// lanes of packed binary32x2 instructions, and their binary32 arrays are packed
// per cell so that a stencil point is one or two 16-byte loads.  CBNS_FP64_FF
// solves keep the binary64 state and RK3 combination (k_update<double, S, true>,
// k_dt_reduce<double, true>) and take their faces and viscous terms from the
// float-float kernels of cbns_ff_kernels.cu.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "../../include/cbns_gpu.h"
#include "cbns_device.cuh"
#include "cbns_ff.cuh"
#include "cbns_modes.h"
#include "cbns_prof.h"

namespace cbns {

// ---------------------------------------------------------------------------
// Division, reciprocal and square root by compute type.  Binary64 keeps IEEE
// division and square root.  The binary32 paths of FP32-mixed use the fast
// approximations (a couple of ulp): their results are stored and differenced in
// binary32 anyway, whose rounding dominates.

__device__ __forceinline__ double fma_(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double div_(double a, double b) { return a / b; }
__device__ __forceinline__ float div_(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double sqrt_(double a) { return sqrt(a); }
__device__ __forceinline__ float sqrt_(float a) { return a * rsqrtf(a); }

// ---------------------------------------------------------------------------
// Primitive recovery (Block3d::calc_primitive, src/Block3d.cpp:359-385) of one
// conserved state, written at padded offset o.

__device__ __forceinline__ int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

struct Prims64 {
  double u, v, w, p, T, sr, H;
};

// Binary64 primitives of one state (Block3d::calc_primitive, src/Block3d.cpp:359-385),
// with 1/rho and sqrt(rho) from one reciprocal square root (a few ulp from the
// reference's division and square root).  The start-up fill and the update
// both use it, so a solve restarted from its own state continues bitwise.
__device__ __forceinline__ Prims64 prims64(const SolveDev& s, double r, double ru, double rv, double rw, double E) {
  const double rs = rsqrt(r);
  const double ir = rs * rs;
  Prims64 q;
  q.u = ru * ir;
  q.v = rv * ir;
  q.w = rw * ir;
  const double q2 = q.u * q.u + q.v * q.v + q.w * q.w;
  q.p = s.gam1 * (E - 0.5 * r * q2);
  q.T = s.gM2 * q.p * ir;
  q.sr = r * rs;
  q.H = s.cd.gamma_gam1_inv * q.p * ir + 0.5 * q2;
  return q;
}

__device__ __forceinline__ void store_prims(const SolveDev& s, long long o, double r, double ru,
                                            double rv, double rw, double E) {
  const Prims64 q = prims64(s, r, ru, rv, rw, E);
  const long long V = s.V;
  at(s, s.pd.rho, V, o) = r;
  at(s, s.pd.u, V, o) = q.u;
  at(s, s.pd.v, V, o) = q.v;
  at(s, s.pd.w, V, o) = q.w;
  at(s, s.pd.p, V, o) = q.p;
  at(s, s.pd.T, V, o) = q.T;
  at(s, s.pd.srho, V, o) = q.sr;
  at(s, s.pd.H, V, o) = q.H;
}

// The split of a state into the float-float perturbation CBNS_FP64_FF kernels
// read: (rho - rho_ref, rho u, rho v, rho w, E - E_ref), the differences taken in
// binary64.
__device__ __forceinline__ float2 ff_split_state(const SolveDev& s, int n, double q) {
  return ff_split(n == 0 ? q - s.rho_ref : (n == NEQ - 1 ? q - s.E_ref : q));
}

// CBNS_FP64_FF solves: the float-float copies the face and viscous kernels
// read, of a cell's state (into QFo, the copy of the array the state went to,
// as the perturbation above) and of its primitives sqrt(rho), H, u, v, w, T
// (split on the integer pipe).
__device__ __forceinline__ void store_ff(const SolveDev& s, float2* QFo, long long d, const double (&q)[NEQ],
                                         double sr, double H, double u, double v, double w, double T) {
  const long long V = s.V, n5 = NEQ * V, np = kFFPrims * V;
#pragma unroll
  for (int n = 0; n < NEQ; ++n) at(s, QFo, n5, n * V + d) = ff_split_state(s, n, q[n]);
  float2* P = s.PF;
  at(s, P, np, d) = ff_split(sr);
  at(s, P, np, V + d) = ff_split(H);
  at(s, P, np, 2 * V + d) = ff_split(u);
  at(s, P, np, 3 * V + d) = ff_split(v);
  at(s, P, np, 4 * V + d) = ff_split(w);
  at(s, P, np, 5 * V + d) = ff_split(T);
}

// CBNS_FP64_FF: the primitives of a state in float-float (prims64's formulas),
// from the float-float perturbation q' = (rho - rho_ref, rho u, rho v, rho w,
// E - E_ref): p = p_ref + (gamma - 1) (E' - rho q^2 / 2), as (gamma - 1) E_ref
// = p_ref.
struct PrimsFF {
  ff u, v, w, p, T, sr, H;
};

__device__ __forceinline__ PrimsFF prims_ff(const SolveDev& s, const ff (&q)[NEQ]) {
  auto cf = [](float2 v) { return ff{v.x, v.y}; };
  const ff rho = q[0] + cf(s.ff_rho_ref);
  const ff rs = ff_rsqrt(rho);
  const ff ir = ff_sqr(rs);
  PrimsFF r;
  r.u = q[1] * ir;
  r.v = q[2] * ir;
  r.w = q[3] * ir;
  const ff q2 = ff_sqr_add_acc(r.w, ff_sqr_add_acc(r.v, ff_sqr(r.u)));  // no cancellation
  r.p = cf(s.ff_gam1) * (q[4] - ff_scale(rho * q2, 0.5f)) + cf(s.ff_p_ref);
  r.T = (cf(s.ff_gM2) * r.p) * ir;
  r.sr = rho * rs;
  r.H = ff_fma(cf(s.ff_ggam1) * r.p, ir, ff_scale(q2, 0.5f));
  return r;
}

// FP32-mixed: the binary32 perturbation state and primitives of a binary64 state.
// rho' = rho - rho_ref and E' = E - E_ref are formed in binary64 before rounding,
// so binary32 keeps 24 bits of the fluctuations; p' = p - p_ref and
// T' = T - T_ref follow from them without touching the large means.  sqrt(rho)
// for the Roe weights is taken in binary64 where rho is below 1% of rho_ref.
struct MixedCell {
  float U[NEQ];
  float rho, u, v, w, p, T, srho, H;
};

// sqrt(rho) in binary64 for the rare cells below the low-density threshold.
// Kept out of line so that the common path does not evaluate it: a select
// between the two square roots would cost every cell a binary64 square root.
__device__ __noinline__ float low_density_srho(double rho) { return (float)sqrt(rho); }

__device__ __forceinline__ MixedCell mixed_cell(const SolveDev& s, const double (&q)[NEQ]) {
  MixedCell m;
  const Consts<float>& C = s.cf;
  const float rp = (float)(q[0] - s.cd.rho_ref);
  const float Ep = (float)(q[4] - s.cd.E_ref);
  const float r = C.rho_ref + rp;  // binary32 density without another conversion
  m.U[0] = rp;
  m.U[1] = (float)q[1];
  m.U[2] = (float)q[2];
  m.U[3] = (float)q[3];
  m.U[4] = Ep;
  const float ir = div_(1.0f, r);
  const float uu = m.U[1] * ir, vv = m.U[2] * ir, ww = m.U[3] * ir;
  const float q2 = uu * uu + vv * vv + ww * ww;
  const float pp = C.gam1 * (Ep - 0.5f * r * q2);
  m.rho = r;
  m.u = uu;
  m.v = vv;
  m.w = ww;
  m.p = pp;
  m.T = C.gM2 * ir * (pp - C.pref_over_rref * rp);
  if (r < C.low_rho) {
    m.srho = low_density_srho(q[0]);
  } else {
    m.srho = sqrt_(r);
  }
  m.H = C.gamma_gam1_inv * (C.p_ref + pp) * ir + 0.5f * q2;
  return m;
}

// The packed binary32 state and primitives of one cell: four 16-byte stores and
// one 4-byte store.
__device__ __forceinline__ void store_mixed(const SolveDev& s, long long o, const MixedCell& m) {
  at(s, s.U4, s.V, o) = make_float4(m.U[0], m.U[1], m.U[2], m.U[3]);
  at(s, s.UE, s.V, o) = m.U[4];
  at(s, s.PA, s.V, o) = make_float4(m.u, m.v, m.w, m.T);
  at(s, s.PB, s.V, o) = make_float4(m.rho, m.p, m.srho, m.H);
}

__global__ void k_aos_to_soa(const SolveDev* __restrict__ solves, int sidx, const double* __restrict__ aos,
                             double* __restrict__ soa) {
  const SolveDev& s = solves[sidx];
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < s.V;
       o += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int n = 0; n < NEQ; ++n) at(s, soa, NEQ * s.V, n * s.V + o) = at(s, aos, NEQ * s.V, NEQ * o + n);
  }
}

__global__ void k_soa_to_aos(const SolveDev* __restrict__ solves, int sidx, const double* __restrict__ soa,
                             double* __restrict__ aos) {
  const SolveDev& s = solves[sidx];
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < s.V;
       o += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int n = 0; n < NEQ; ++n) at(s, aos, NEQ * s.V, NEQ * o + n) = at(s, soa, NEQ * s.V, n * s.V + o);
  }
}

// Start-up: ghost fill, primitives, Q_p = Q, mu = 1 (src/cbns3d.cpp:149-153 and
// src/Block3d.cpp:265).  Over the padded domain; each cell reads only its
// interior source, so ghosts and interior are written without races.
__global__ void k_prepare(const SolveDev* __restrict__ solves, const TileRef* __restrict__ tiles,
                          int ntiles) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    TileCell tc = tile_cell(tiles[t], -NG);
    const SolveDev& s = solves[tc.s];
    if (tc.i >= s.IM + NG || tc.j >= s.JM + NG) continue;
    const long long o = pad_off(s, tc.i, tc.j, tc.k);
    const long long src = pad_off(s, wrap(tc.i, s.IM), wrap(tc.j, s.JM), wrap(tc.k, s.KM));
    double q[NEQ];
#pragma unroll
    for (int n = 0; n < NEQ; ++n) q[n] = at(s, s.Q, NEQ * s.V, n * s.V + src);
#pragma unroll
    for (int n = 0; n < NEQ; ++n) {
      at(s, s.Q, NEQ * s.V, n * s.V + o) = q[n];
      at(s, s.Qp, NEQ * s.V, n * s.V + o) = q[n];
    }
    store_prims(s, o, q[0], q[1], q[2], q[3], q[4]);
    if (s.mixed) store_mixed(s, o, mixed_cell(s, q));
    if (s.ffaces) {
      const Prims64 pr = prims64(s, q[0], q[1], q[2], q[3], q[4]);
      store_ff(s, s.QF, o, q, pr.sr, pr.H, pr.u, pr.v, pr.w, pr.T);
      store_ff(s, s.QpF, o, q, pr.sr, pr.H, pr.u, pr.v, pr.w, pr.T);
    }
    const bool interior = tc.i >= 0 && tc.i < s.IM && tc.j >= 0 && tc.j < s.JM && tc.k >= 0 && tc.k < s.KM;
    if (interior) {
      at(s, s.pd.mu, s.V, o) = 1.0;
      if (s.mixed) at(s, s.muf, s.V, o) = 1.0f;
    }
  }
}

// Device initial condition (no host state): the Taylor-Green fields of
// Block3d::initial_condition (src/Block3d.cpp:237-271) on gen_mesh's mesh
// (src/Block3d.cpp:208-235), plus the project's solenoidal perturbation, then
// calc_conservative (src/Block3d.cpp:273-300), written to the interior of Q.
// The device sin/cos differ from the host libm in the last place at most.
constexpr int kMaxModes = 64;
struct ModeTable {
  int n;
  PerturbMode m[kMaxModes];
};

__global__ void k_init_tgv(const SolveDev* __restrict__ solves, int sidx, const TileRef* __restrict__ tiles,
                           int ntiles, double p_inf, ModeTable modes) {
  const SolveDev& s = solves[sidx];
  const double half_pi2 = 3.14159265358979323846;  // (2 pi) / 2, gen_mesh's offset
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    TileCell tc = tile_cell(tiles[t], 0);
    if (tc.i >= s.IM || tc.j >= s.JM) continue;
    const double xl = (tc.i * s.dx - half_pi2) + 0.5 * s.dx;
    const double yl = (tc.j * s.dy - half_pi2) + 0.5 * s.dy;
    const double zl = (tc.k * s.dz - half_pi2) + 0.5 * s.dz;
    double u = sin(xl) * cos(yl) * cos(zl);
    double v = -cos(xl) * sin(yl) * cos(zl);
    double w = 0.0;
    for (int m = 0; m < modes.n; ++m) {
      const PerturbMode& md = modes.m[m];
      const double c = cos(md.k[0] * xl + md.k[1] * yl + md.k[2] * zl + md.phase);
      u += md.a[0] * c;
      v += md.a[1] * c;
      w += md.a[2] * c;
    }
    const double p = p_inf + (cos(2.0 * xl) + cos(2.0 * yl)) * (cos(2.0 * zl) + 2.0) / 16.0;
    const double r = s.gM2 * p;
    const long long o = pad_off(s, tc.i, tc.j, tc.k);
    const long long n5 = NEQ * s.V;
    at(s, s.Q, n5, o) = r;
    at(s, s.Q, n5, s.V + o) = r * u;
    at(s, s.Q, n5, 2 * s.V + o) = r * v;
    at(s, s.Q, n5, 3 * s.V + o) = r * w;
    at(s, s.Q, n5, 4 * s.V + o) = p / s.gam1 + 0.5 * r * (u * u + v * v + w * w);
  }
}

// Binary64 primitives of the current Q for output (FP32-mixed solves keep
// binary32 primitives only while stepping).
__global__ void k_prims_double(const SolveDev* __restrict__ solves, const TileRef* __restrict__ tiles,
                               int ntiles) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    TileCell tc = tile_cell(tiles[t], -NG);
    const SolveDev& s = solves[tc.s];
    if (tc.i >= s.IM + NG || tc.j >= s.JM + NG) continue;
    const long long o = pad_off(s, tc.i, tc.j, tc.k);
    const long long n5 = NEQ * s.V;
    store_prims(s, o, at(s, s.Q, n5, o), at(s, s.Q, n5, s.V + o), at(s, s.Q, n5, 2 * s.V + o),
                at(s, s.Q, n5, 3 * s.V + o), at(s, s.Q, n5, 4 * s.V + o));
  }
}

// ---------------------------------------------------------------------------
// Time step: Block3d::calc_dt (src/Block3d.cpp:515-553) as a max-reduction, then
// the MIN all-reduce (trivial on one block), clip to t_end and is_finished
// (src/cbns3d.cpp:178-194, src/Block3d.cpp:502-513).

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// The reference's per-cell sum over x, y, z of |u_d| + c/h_d + fv/h_d^2 with
// c = sqrt(gamma p / rho) and fv = 2 mu C_dt_v |u| / (rho c), regrouped as
//   (|u| + |v| + |w|) + c (1/hx + 1/hy + 1/hz) + fv (1/hx^2 + 1/hy^2 + 1/hz^2),
// with one reciprocal square root: z = 1/sqrt(gamma p rho) = 1/(rho c) and
// c = gamma p z.
template <typename R>
__device__ __forceinline__ R dt_speed(const SolveDev& s, long long o) {
  const Consts<R>& C = consts_of<R>(s);
  R rr, uu, vv, ww, pp, mu;
  if constexpr (sizeof(R) == 4) {
    const float4 a = at(s, s.PA, s.V, o), b = at(s, s.PB, s.V, o);
    rr = b.x, uu = a.x, vv = a.y, ww = a.z;
    pp = C.p_ref + b.y;
    mu = at(s, s.muf, s.V, o);
  } else {
    const PrimSet<double>& P = s.pd;
    const long long V = s.V;
    rr = at(s, P.rho, V, o), uu = at(s, P.u, V, o), vv = at(s, P.v, V, o), ww = at(s, P.w, V, o);
    pp = at(s, P.p, V, o);
    mu = at(s, P.mu, V, o);
  }
  const R gp = C.gamma * pp;
  const R z = rsqrt(gp * rr);
  const R c = gp * z;
  const R q2 = fma_(ww, ww, fma_(vv, vv, uu * uu));
  const R q = (sizeof(R) == 4 && !(q2 > (R)0)) ? (R)0 : sqrt_(q2);  // binary32 sqrt_ is q2 * rsqrt(q2)
  const R fv = (C.C_dt_v2 * mu) * q * z;
  return (fabs(uu) + fabs(vv) + fabs(ww)) + fma_(c, C.sum_ih, fv * C.sum_ih2);
}

// CBNS_FP64_FF: the same speed in float-float, from the float-float primitives
// (rho = sqrt(rho)^2, p = rho T / (gamma M^2)) and the binary64 mu, widened once.
__device__ __forceinline__ double dt_speed_ff(const SolveDev& s, long long o) {
  const long long V = s.V, np = kFFPrims * V;
  auto ld = [&](int b) {
    const float2 v = at(s, s.PF, np, b * V + o);
    return ff{v.x, v.y};
  };
  auto cf = [](float2 v) { return ff{v.x, v.y}; };
  const ff sr = ld(0), uu = ld(2), vv = ld(3), ww = ld(4), TT = ld(5);
  const float2 m2 = ff_split(at(s, s.pd.mu, V, o));
  const ff mu{m2.x, m2.y};
  const ff rr = ff_sqr(sr);
  const ff gp = cf(s.ff_gamma) * ((rr * TT) * cf(s.ff_igM2));
  const ff z = ff_rsqrt(gp * rr);
  const ff c = gp * z;
  const ff q2 = ff_sqr_add(ww, ff_sqr_add_acc(vv, ff_sqr(uu)));
  const ff q = q2.hi > 0.0f ? q2 * ff_rsqrt(q2) : ff{0.0f, 0.0f};
  const ff fv = ((cf(s.ff_Cdt2) * mu) * q) * z;
  const ff a = (ff_abs(uu) + ff_abs(vv)) + ff_abs(ww);
  return ff_to_double(a + ff_fma(c, cf(s.ff_sum_ih), fv * cf(s.ff_sum_ih2)));
}

// Each CTA walks its tiles (grid stride) keeping a running per-thread maximum,
// and folds it into the solve's control block (one block reduction and one
// atomicMax) only when the next tile belongs to another solve or the walk ends.
// Tiles of one solve are contiguous in the table, so a bounded grid issues
// about one atomic per CTA instead of one per tile.  The running maximum stays
// in the compute type and is widened once per fold (exact and monotonic, so
// the same maximum); whether the solve has finished is tested once per solve.
template <typename R, bool FF>
__global__ void __launch_bounds__(kMaxThreads) k_dt_reduce(const SolveDev* __restrict__ solves,
                                                           const TileRef* __restrict__ tiles, int ntiles,
                                                           double t_end, int use_t_end, int skip_finished) {
  __shared__ double red[kMaxThreads / 32];
  const int nwarps = (int)(blockDim.x / 32);
  R run = (R)0;
  int live_solve = -1;
  bool live = false;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    TileCell tc = tile_cell(tiles[t], 0);
    const SolveDev& s = solves[tc.s];
    if (tc.s != live_solve) {  // uniform over the CTA
      const SolveCtl* ctl = s.ctl;
      const double te = use_t_end ? t_end : ctl->t_end;
      live = !(skip_finished && ctl->t_cur + 1.0e-5 > te);
      live_solve = tc.s;
    }
    if (live && tc.i < s.IM && tc.j < s.JM) {
      R sum;
      if constexpr (FF)
        sum = dt_speed_ff(s, pad_off(s, tc.i, tc.j, tc.k));
      else
        sum = dt_speed<R>(s, pad_off(s, tc.i, tc.j, tc.k));
      if (sum > run) run = sum;  // a NaN is skipped, as the reference's ternary does
    }
    const int tn = t + (int)gridDim.x;
    const bool flush = tn >= ntiles || tiles[tn].solve != tiles[t].solve;  // uniform over the CTA
    if (flush) {
      double m = warp_max((double)run);
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
      __syncthreads();
      if (threadIdx.x == 0) {
        for (int a = 1; a < nwarps; ++a) m = fmax(m, red[a]);
        // Positive doubles order like their bit patterns.
        if (m > 0.0) atomicMax(&s.ctl->smax_bits, (unsigned long long)__double_as_longlong(m));
      }
      __syncthreads();
      run = (R)0;
    }
  }
}

__global__ void k_dt_finalize(const SolveDev* __restrict__ solves, int nsolves, double t_end,
                              int use_t_end) {
  int si = blockIdx.x * blockDim.x + threadIdx.x;
  if (si >= nsolves) return;
  SolveCtl* ctl = solves[si].ctl;
  if (use_t_end) ctl->t_end = t_end;
  double smax = __longlong_as_double((long long)ctl->smax_bits);
  ctl->smax_bits = 0ull;
  if (ctl->t_cur + 1.0e-5 > ctl->t_end) {
    ctl->active = 0;
    return;
  }
  double dt = solves[si].CFL / smax;
  if (ctl->t_end - ctl->t_cur < dt) dt = ctl->t_end - ctl->t_cur;
  ctl->t_cur += dt;
  ctl->dt = dt;
  ctl->cdt[0] = (float)(0.25 * dt);
  ctl->cdt[1] = (float)((2.0 / 3.0) * dt);
  ctl->active = 1;
  ctl->steps += 1;
}

// calc_dt's value alone (cbns_calc_dt): CFL / max, no clip, no time advance.
__global__ void k_dt_raw(const SolveDev* __restrict__ solves, int sidx, double* __restrict__ out) {
  SolveCtl* ctl = solves[sidx].ctl;
  out[0] = solves[sidx].CFL / __longlong_as_double((long long)ctl->smax_bits);
  ctl->smax_bits = 0ull;
}

// The control block of a solve restarting at time t (the asynchronous upload:
// no host buffer is read while earlier work may still be queued).
__global__ void k_reset_ctl(SolveCtl* __restrict__ ctl, double t, double t_end) {
  SolveCtl c{};
  c.t_cur = t;
  c.t_end = t_end;
  c.active = 1;
  *ctl = c;
}

// Explicit dt for a single stage called from the host (cbns_stage).
__global__ void k_set_dt(const SolveDev* __restrict__ solves, int sidx, double dt) {
  SolveCtl* ctl = solves[sidx].ctl;
  ctl->dt = dt;
  ctl->cdt[0] = (float)(0.25 * dt);
  ctl->cdt[1] = (float)((2.0 / 3.0) * dt);
  ctl->active = 1;
}

// ---------------------------------------------------------------------------
// WENO5 (src/weno.cpp:25-56).  The reference forms w_k = d_k / (eps + IS_k)^2
// and returns (sum w_k f_k) / (sum w_k).  Here:
// * every quantity is written in the first differences d_m = v_{m+1} - v_m of
//   the six values v0..v5 of a face (cells c-3 .. c+2);
// * the result is v2 + (sum w_k g_k) / (sum w_k) with g_k = f_k - v2 (the
//   candidates' deviations are two-term combinations of the d_m);
// * the indicators are taken four times over, 4 (eps + IS_k) =
//   13/3 D_k^2 + e_k^2 + 4 eps (exact: a power-of-two scaling that cancels in
//   the ratio);
// * numerator and denominator are multiplied by 10 a1 a2 a3, a_k = (4 (eps + IS_k))^2,
//     num = a2 a3 g1 + 6 a1 a3 g2 + 3 a1 a2 g3,  den = a2 a3 + 6 a1 a3 + 3 a1 a2,
//   and the division is deferred so the ten of a face share one.
// (4 (eps + IS_k) >= 4e-6, so den >= 2.56e-22: inside binary32's normal range.)

template <typename R>
struct Weno {
  R num, den;
};

// One biased stencil: D_k the second differences (C_k = 13/3 D_k), e_k the
// one-sided differences of the indicators, g1 = f1 - v2, g2s = 6 (f2 - v2) and
// g3s = 3 (f3 - v2) (the linear weights 0.1 : 0.6 : 0.3, times 10, folded in).
template <typename R>
__device__ __forceinline__ void weno5_side(R D1, R C1, R D2, R C2, R D3, R C3, R e1, R e2, R e3, R g1, R g2s,
                                           R g3s, Weno<R>& out) {
  const R eps4 = (R)4.0e-6;
  const R is1 = fma_(C1, D1, fma_(e1, e1, eps4));
  const R is2 = fma_(C2, D2, fma_(e2, e2, eps4));
  const R is3 = fma_(C3, D3, fma_(e3, e3, eps4));
  const R a1 = is1 * is1, a2 = is2 * is2, a3 = is3 * is3;
  const R p1 = a2 * a3, q2 = a1 * a3, q3 = a1 * a2;
  out.den = fma_((R)6, q2, fma_((R)3, q3, p1));
  out.num = fma_(q2, g2s, fma_(q3, g3s, p1 * g1));
}

// Both reconstructions of one characteristic field at a face: the left-biased
// stencil (v0..v4, result v2 + num/den) and the mirrored right-biased one
// (v5..v1, result v3 + num/den).  With d_m as above,
//   left:  D = d1-d0, d2-d1, d3-d2;  e = 3 d1 - d0, d1 + d2, d3 - 3 d2;
//          6 g1 = 5 d1 - 2 d0,  6 g2 = d1 + 2 d2,  6 g3 = 4 d2 - d3;
//   right: D = d4-d3, d3-d2, d2-d1;  e = d4 - 3 d3, d2 + d3, 3 d2 - d1;
//          6 g1 = 2 d4 - 5 d3,  6 g2 = -(d3 + 2 d2),  6 g3 = d1 - 4 d2
// (the sign of an e_k is immaterial: it is squared).  The middle second
// differences D2, D3 serve both stencils.
template <typename R>
__device__ __forceinline__ void weno5_pair(const R (&v)[6], Weno<R>& L, Weno<R>& Rt) {
  const R d0 = v[1] - v[0], d1 = v[2] - v[1], d2 = v[3] - v[2], d3 = v[4] - v[3], d4 = v[5] - v[4];
  const R D1 = d1 - d0, D2 = d2 - d1, D3 = d3 - d2, D4 = d4 - d3;
  const R c13 = (R)(13.0 / 3.0);
  const R C1 = c13 * D1, C2 = c13 * D2, C3 = c13 * D3, C4 = c13 * D4;
  const R k56 = (R)(5.0 / 6.0), k13 = (R)(1.0 / 3.0);
  // 3 g3 of both stencils from one 2 d2 (exact): 2 d2 - d3/2 and d1/2 - 2 d2
  const R t2 = d2 + d2;
  weno5_side<R>(D1, C1, D2, C2, D3, C3, fma_((R)3, d1, -d0), d1 + d2, fma_((R)-3, d2, d3),
                fma_(k56, d1, -k13 * d0), fma_((R)2, d2, d1), fma_((R)-0.5, d3, t2), L);
  weno5_side<R>(D4, C4, D3, C3, D2, C2, fma_((R)-3, d3, d4), d2 + d3, fma_((R)3, d2, -d1),
                fma_(-k56, d3, k13 * d4), fma_((R)-2, d2, -d3), fma_((R)0.5, d1, -t2), Rt);
}

// r[n] = base[n] + num[n] / den[n] for ten parts (both states of a face).
// Binary64: one division (Montgomery's simultaneous inversion).  Every den is
// positive and at least 2.56e-22; the batch is used while the product of each
// half lies in about [1e-150, 1e150] (biased exponent 525 .. 1520, tested on the
// integer pipe), which keeps every partial product and partial reciprocal in
// the normal range; otherwise each quotient is divided on its own.  (The
// binary32 faces multiply by per-face reciprocals: face_core_x2.)
__device__ __forceinline__ void weno_divide10(const Weno<double> (&w)[10], const double (&base)[10],
                                              double (&r)[10]) {
  // Two halves of five: prefix products within each half, one reciprocal of the
  // whole product, then 1/(half product) = reciprocal x (other half's product).
  // The same 28 multiplications as one chain of ten, at half its depth.
  double pa[5], pb[5];
  pa[0] = w[0].den;
  pb[0] = w[5].den;
#pragma unroll
  for (int n = 1; n < 5; ++n) {
    pa[n] = pa[n - 1] * w[n].den;
    pb[n] = pb[n - 1] * w[5 + n].den;
  }
  const unsigned ea = (unsigned)((unsigned long long)__double_as_longlong(pa[4]) >> 52);
  const unsigned eb = (unsigned)((unsigned long long)__double_as_longlong(pb[4]) >> 52);
  if (ea - 525u < 996u && eb - 525u < 996u) {
    const double inv = rcp64(pa[4] * pb[4]);
    double ia = inv * pb[4], ib = inv * pa[4];  // 1/pa[4], 1/pb[4]
#pragma unroll
    for (int n = 4; n > 0; --n) {
      r[n] = fma(w[n].num, ia * pa[n - 1], base[n]);
      r[5 + n] = fma(w[5 + n].num, ib * pb[n - 1], base[5 + n]);
      ia *= w[n].den;
      ib *= w[5 + n].den;
    }
    r[0] = fma(w[0].num, ia, base[0]);
    r[5] = fma(w[5].num, ib, base[5]);
  } else {
#pragma unroll
    for (int n = 0; n < 10; ++n) r[n] = base[n] + w[n].num / w[n].den;
  }
}

// ---------------------------------------------------------------------------
// Numerical flux at one face (src/Block3d.cpp:566-616 and its y/z twins).
//
// Eigenvectors (src/eigenvectors_roe.cpp:32-171).  For a face normal to axis D
// the tangent vectors l, m are the other two axes up to sign, so with the Roe
// state (U, H, c), K = (gamma-1)/(2c^2) and t = q^2/2 f0 - U.m + f4 (m the
// momentum of the projected conserved vector f):
//   L f = ( A + B, f0 - 2A, A - B, f_t1 - U_t1 f0, f_t2 - U_t2 f0 ),
//   A = K t,  B = (U_D f0 - f_D) / (2c)
// (the signs of the two shear fields are dropped: WENO5 is odd, R flips them back).
// R r, with s = r0 + r2 and d = r2 - r0:
//   rho = s + r1,  m_D = U_D rho + c d,  m_ti = U_ti rho + r_ti,
//   E = H s + U_D c d + q^2/2 r1 + U_t1 r3 + U_t2 r4.
// The Roe average (ratio = sqrt(rho_R/rho_L)) is formed from per-cell sqrt(rho).
// lf_flux (src/lf_flux.cpp:32-99) takes the reconstructed conserved states.
// Binary64; the FP32-mixed faces are face_core_x2 below.

// The stencil of one binary64 face normal to D: the conserved state of the six
// cells c-3 .. c+2 (W[m][n], field n of cell c-3+m) and, of the two cells
// either side (l = c - st, r = c), sqrt(rho), H and the velocity.
struct FaceSide {
  double sr, h, u, v, w;
};

__device__ __forceinline__ FaceSide face_side(const SolveDev& s, long long o) {
  const PrimSet<double>& P = s.pd;
  const long long V = s.V;
  return FaceSide{at(s, P.srho, V, o), at(s, P.H, V, o), at(s, P.u, V, o), at(s, P.v, V, o), at(s, P.w, V, o)};
}

template <int D>
__device__ __forceinline__ void face_core(const SolveDev& s, const double (&W)[6][NEQ], const FaceSide& Ls,
                                          const FaceSide& Rs, double (&out)[NEQ]) {
  using R = double;
  constexpr int T1 = (D + 1) % 3;
  constexpr int T2 = (D + 2) % 3;
  const Consts<R>& C = consts_of<R>(s);
  const R gam1 = C.gam1, gamma = C.gamma;

  // Roe-averaged state of the two cells either side (src/eigenvectors_roe.cpp:87-106).
  // (sqrt(rho_L) f_L + sqrt(rho_R) f_R) / (sqrt(rho_L) + sqrt(rho_R)) = f_R + wL (f_L - f_R).
  R Uv[3], HH;
  {
    const R sl = Ls.sr, sr = Rs.sr, hl = Ls.h, hr = Rs.h;
    const R ul = Ls.u, ur = Rs.u, vl = Ls.v, vr = Rs.v, wl = Ls.w, wr = Rs.w;
    const R wL = sl * rcp64(sl + sr);
    Uv[0] = fma_(wL, ul - ur, ur);
    Uv[1] = fma_(wL, vl - vr, vr);
    Uv[2] = fma_(wL, wl - wr, wr);
    HH = fma_(wL, hl - hr, hr);
  }
  const R q2 = Uv[0] * Uv[0] + Uv[1] * Uv[1] + Uv[2] * Uv[2];
  const R hq2 = (R)0.5 * q2;
  const R c2 = gam1 * (HH - hq2);
  const R ic = rsqrt(c2);  // 1/c; c = c^2 * (1/c)
  const R cc = c2 * ic;
  const R K = (C.hgam1 * ic) * ic;
  const R hic = (R)0.5 * ic;
  const R un = Uv[D], u1 = Uv[T1], u2 = Uv[T2];

  // Characteristic projections of the six cells c-3 .. c+2 (shared by both
  // biased stencils).
  R w[NEQ][6];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const R f0 = W[m][0], f1 = W[m][1], f2 = W[m][2], f3 = W[m][3], f4 = W[m][4];
    const R fm[3] = {f1, f2, f3};
    const R t = fma_(-Uv[2], f3, fma_(-Uv[1], f2, fma_(-Uv[0], f1, fma_(hq2, f0, f4))));
    const R A = K * t;
    const R g = fma_(un, f0, -fm[D]);  // B = g / (2c)
    w[0][m] = fma_(hic, g, A);
    w[1][m] = fma_((R)-2, A, f0);
    w[2][m] = fma_(-hic, g, A);
    w[3][m] = fma_(-u1, f0, fm[T1]);
    w[4][m] = fma_(-u2, f0, fm[T2]);
  }

  // Left-biased (cells -3..+1) and right-biased mirrored (+2..-2) reconstructions
  // (src/Block3d.cpp:591-607, src/weno.cpp:77-152).
  R rl[NEQ], rr[NEQ];
  {
    Weno<R> wp[2 * NEQ];
#pragma unroll
    for (int n = 0; n < NEQ; ++n) weno5_pair<R>(w[n], wp[n], wp[NEQ + n]);
    R base[2 * NEQ], q[2 * NEQ];
#pragma unroll
    for (int n = 0; n < NEQ; ++n) {
      base[n] = w[n][2];
      base[NEQ + n] = w[n][3];
    }
    weno_divide10(wp, base, q);
#pragma unroll
    for (int n = 0; n < NEQ; ++n) {
      rl[n] = q[n];
      rr[n] = q[NEQ + n];
    }
  }

  // Back to conserved variables.
  R rhoL, mL[3], EL, rhoR, mR[3], ER;
  {
    R sp = rl[0] + rl[2], dm = rl[2] - rl[0];
    rhoL = sp + rl[1];
    mL[D] = un * rhoL + cc * dm;
    mL[T1] = u1 * rhoL + rl[3];
    mL[T2] = u2 * rhoL + rl[4];
    EL = HH * sp + (un * cc) * dm + hq2 * rl[1] + u1 * rl[3] + u2 * rl[4];
  }
  {
    R sp = rr[0] + rr[2], dm = rr[2] - rr[0];
    rhoR = sp + rr[1];
    mR[D] = un * rhoR + cc * dm;
    mR[T1] = u1 * rhoR + rr[3];
    mR[T2] = u2 * rhoR + rr[4];
    ER = HH * sp + (un * cc) * dm + hq2 * rr[1] + u1 * rr[3] + u2 * rr[4];
  }

  // Local Lax-Friedrichs flux (src/lf_flux.cpp:32-99); both 1/rho from one division.
  // The stored flux is twice the reference's: the halves are folded into the
  // flux difference's 0.5/h (an exact power-of-two scaling).
  const R ip = rcp64(rhoL * rhoR);
  const R iL = ip * rhoR, iR = ip * rhoL;
  R vL[3], vR[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    vL[a] = mL[a] * iL;
    vR[a] = mR[a] * iR;
  }
  // rho q^2 = m . v; p = (gamma - 1) (E - rho q^2 / 2).
  const R kL = fma_(mL[2], vL[2], fma_(mL[1], vL[1], mL[0] * vL[0]));
  const R kR = fma_(mR[2], vR[2], fma_(mR[1], vR[1], mR[0] * vR[0]));
  const R pL = gam1 * fma_((R)-0.5, kL, EL);
  const R pR = gam1 * fma_((R)-0.5, kR, ER);
  const R c2L = (gamma * iL) * pL, c2R = (gamma * iR) * pR;
  const R cL = c2L * rsqrt(c2L), cR = c2R * rsqrt(c2R);
  const R alpha = fmax(fabs(vR[D]) + cR, fabs(vL[D]) + cL);
  const R fL = mL[D], fR = mR[D];  // mass fluxes rho*q_n
  out[0] = fma_(-alpha, rhoR - rhoL, fL + fR);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const R fLa = (a == D) ? fma_(fL, vL[a], pL + pR) : fL * vL[a];
    out[1 + a] = fma_(-alpha, mR[a] - mL[a], fma_(fR, vR[a], fLa));
  }
  // rho q_n H = q_n (E + p).
  out[4] = fma_(-alpha, ER - EL, fma_(vR[D], ER + pR, vL[D] * (EL + pL)));
}

// One face from memory: the six stencil cells of U and the two sides' primitives.
template <int D, typename R>
__device__ __forceinline__ void face_flux(const SolveDev& s, const R* __restrict__ U, long long c,
                                          R (&out)[NEQ]) {
  static_assert(sizeof(R) == 8, "binary64 faces; FP32-mixed faces are face_core_x2");
  const long long st = D == 0 ? 1ll : (D == 1 ? (long long)s.nx : (long long)s.nx * s.ny);
  const long long V = s.V;
  double W[6][NEQ];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const long long o = c + (m - 3) * st;
#pragma unroll
    for (int n = 0; n < NEQ; ++n) W[m][n] = at(s, U, NEQ * V, n * V + o);
  }
  face_core<D>(s, W, face_side(s, c - st), face_side(s, c), out);
}

// ---------------------------------------------------------------------------
// FP32-mixed faces two at a time.  The binary32 face kernel is bound by
// instruction issue, and every operation of a face is the same for all faces, so
// a thread computes the faces of two rows (j, j+1) in the two lanes of
// Blackwell's packed binary32 instructions (fma/add/mul .f32x2), which do two
// faces' arithmetic per issued instruction.  Loads, the reciprocal and
// reciprocal square roots (MUFU), abs/max and the stores stay per face.  Each
// lane performs face_flux's operations in binary32 on the perturbation form:
// f is the perturbation (rho', m, E') of the reference state; L and R are
// linear and WENO5 reproduces constants, so reconstructing the perturbation and
// adding rho_ref, E_ref back is the same scheme; the momentum flux drops the
// constant p_ref (it cancels in every flux difference), so every binary32 flux
// component is O(1) instead of O(p_ref); the energy flux is rho q_n H with H
// from the full sound speed.  Subtractions are fma(b, -1, a) (the same rounding
// as a - b), and terms whose sign a scalar fma takes for free are formed with
// the opposite sign where that leaves the result unchanged (a squared e_k; the
// right-biased numerator negated together with its reciprocal; alpha times
// (L - R) instead of -alpha times (R - L)).

struct f2 {
  float2 v;
};
__device__ __forceinline__ f2 bc(float a) { return {make_float2(a, a)}; }
__device__ __forceinline__ f2 lanes(float a, float b) { return {make_float2(a, b)}; }
__device__ __forceinline__ f2 add2(f2 a, f2 b) { return {__fadd2_rn(a.v, b.v)}; }
__device__ __forceinline__ f2 sub2(f2 a, f2 b) { return {__ffma2_rn(b.v, make_float2(-1.0f, -1.0f), a.v)}; }
__device__ __forceinline__ f2 mul2(f2 a, f2 b) { return {__fmul2_rn(a.v, b.v)}; }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) { return {__ffma2_rn(a.v, b.v, c.v)}; }
__device__ __forceinline__ f2 rcp2(f2 a) { return {make_float2(__fdividef(1.0f, a.v.x), __fdividef(1.0f, a.v.y))}; }
__device__ __forceinline__ f2 rsqrt2(f2 a) { return {make_float2(rsqrtf(a.v.x), rsqrtf(a.v.y))}; }

// One biased stencil (weno5_side); num is returned with the sign sg of its g's.
__device__ __forceinline__ void weno5_side_x2(f2 D1, f2 C1, f2 D2, f2 C2, f2 D3, f2 C3, f2 e1, f2 e2, f2 e3,
                                              f2 g1, f2 g2s, f2 g3s, f2& num, f2& den) {
  const f2 eps4 = bc(4.0e-6f);
  const f2 is1 = fma2(C1, D1, fma2(e1, e1, eps4));
  const f2 is2 = fma2(C2, D2, fma2(e2, e2, eps4));
  const f2 is3 = fma2(C3, D3, fma2(e3, e3, eps4));
  const f2 a1 = mul2(is1, is1), a2 = mul2(is2, is2), a3 = mul2(is3, is3);
  const f2 p1 = mul2(a2, a3), q2 = mul2(a1, a3), q3 = mul2(a1, a2);
  den = fma2(bc(6.0f), q2, fma2(bc(3.0f), q3, p1));
  num = fma2(q2, g2s, fma2(q3, g3s, mul2(p1, g1)));
}

// weno5_pair on two faces: the left-biased result v2 + numL/denL and the
// right-biased v3 - numRn/denR (numRn the negated numerator).
__device__ __forceinline__ void weno5_pair_x2(const f2 (&v)[6], f2& numL, f2& denL, f2& numRn, f2& denR) {
  const f2 d0 = sub2(v[1], v[0]), d1 = sub2(v[2], v[1]), d2 = sub2(v[3], v[2]), d3 = sub2(v[4], v[3]),
           d4 = sub2(v[5], v[4]);
  const f2 D1 = sub2(d1, d0), D2 = sub2(d2, d1), D3 = sub2(d3, d2), D4 = sub2(d4, d3);
  const f2 c13 = bc((float)(13.0 / 3.0));
  const f2 C1 = mul2(c13, D1), C2 = mul2(c13, D2), C3 = mul2(c13, D3), C4 = mul2(c13, D4);
  const f2 k56 = bc((float)(5.0 / 6.0)), mk13 = bc((float)(-1.0 / 3.0));
  const f2 m3 = bc(-3.0f), two = bc(2.0f), mhalf = bc(-0.5f);
  // left: e = d0 - 3 d1 (sign immaterial), d1 + d2, d3 - 3 d2;
  //       g1 = 5/6 d1 - 1/3 d0, g2s = 2 d2 + d1, g3s = 2 d2 - 0.5 d3
  weno5_side_x2(D1, C1, D2, C2, D3, C3, fma2(m3, d1, d0), add2(d1, d2), fma2(m3, d2, d3),
                fma2(k56, d1, mul2(mk13, d0)), fma2(two, d2, d1), fma2(two, d2, mul2(mhalf, d3)), numL, denL);
  // right, numerator negated: e = d4 - 3 d3, d2 + d3, d1 - 3 d2 (sign immaterial);
  //       -g1 = 5/6 d3 - 1/3 d4, -g2s = 2 d2 + d3, -g3s = 2 d2 - 0.5 d1
  weno5_side_x2(D4, C4, D3, C3, D2, C2, fma2(m3, d3, d4), add2(d2, d3), fma2(m3, d2, d1),
                fma2(k56, d3, mul2(mk13, d4)), fma2(two, d2, d3), fma2(two, d2, mul2(mhalf, d1)), numRn, denR);
}

// The side of a face the Roe average takes from a cell, for both lanes:
// velocity, sqrt(rho) and total enthalpy.
struct SideX2 {
  f2 u, v, w, sr, h;
};

__device__ __forceinline__ SideX2 side_x2(const float4& a0, const float4& b0, const float4& a1, const float4& b1) {
  return SideX2{lanes(a0.x, a1.x), lanes(a0.y, a1.y), lanes(a0.z, a1.z), lanes(b0.z, b1.z), lanes(b0.w, b1.w)};
}

// Two binary32 faces normal to D in the lanes of f2: the Roe sides L and R of
// each face and, through cell(m, f), the perturbation state f[0..4] of stencil
// cell m = 0..5 (cells c-3 .. c+2 of each face's high cell c).
template <int D, class CellFn>
__device__ __forceinline__ void face_core_x2(const Consts<float>& C, const SideX2& Ls, const SideX2& Rs, CellFn cell,
                                             f2 (&out)[NEQ]) {
  constexpr int T1 = (D + 1) % 3;
  constexpr int T2 = (D + 2) % 3;
  const f2 gam1 = bc(C.gam1), half = bc(0.5f), mone = bc(-1.0f);

  // Roe average of the cells either side of each face
  f2 Uv[3], HH;
  {
    const f2 sl = Ls.sr, sr = Rs.sr;
    const f2 ssum = add2(sl, sr);
    const f2 wL = lanes(__fdividef(sl.v.x, ssum.v.x), __fdividef(sl.v.y, ssum.v.y));
    const f2 ur = Rs.u, vr = Rs.v, wr = Rs.w, hr = Rs.h;
    Uv[0] = fma2(wL, sub2(Ls.u, ur), ur);
    Uv[1] = fma2(wL, sub2(Ls.v, vr), vr);
    Uv[2] = fma2(wL, sub2(Ls.w, wr), wr);
    HH = fma2(wL, sub2(Ls.h, hr), hr);
  }
  const f2 q2 = fma2(Uv[2], Uv[2], fma2(Uv[1], Uv[1], mul2(Uv[0], Uv[0])));
  const f2 hq2 = mul2(half, q2);
  const f2 c2 = mul2(gam1, sub2(HH, hq2));
  const f2 ic = rsqrt2(c2);
  const f2 cc = mul2(c2, ic);
  const f2 K = mul2(mul2(bc(0.5f * C.gam1), ic), ic);
  const f2 hic = mul2(half, ic), nhic = mul2(bc(-0.5f), ic);
  const f2 un = Uv[D], u1 = Uv[T1], u2 = Uv[T2];
  const f2 nU0 = mul2(mone, Uv[0]), nU1 = mul2(mone, Uv[1]), nU2 = mul2(mone, Uv[2]);
  const f2 nun = mul2(mone, un), nu1 = mul2(mone, u1), nu2 = mul2(mone, u2);

  // characteristic projections of the six cells c-3 .. c+2 of each face
  f2 w[NEQ][6];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    f2 fc[NEQ];
    cell(m, fc);
    const f2 f0 = fc[0], f1 = fc[1], f2v = fc[2], f3 = fc[3], f4 = fc[4];
    const f2 fm[3] = {f1, f2v, f3};
    const f2 t = fma2(nU2, f3, fma2(nU1, f2v, fma2(nU0, f1, fma2(hq2, f0, f4))));
    const f2 A = mul2(K, t);
    const f2 gn = fma2(nun, f0, fm[D]);  // -g = f_D - U_D f0
    w[0][m] = fma2(nhic, gn, A);
    w[1][m] = fma2(bc(-2.0f), A, f0);
    w[2][m] = fma2(hic, gn, A);
    w[3][m] = fma2(nu1, f0, fm[T1]);
    w[4][m] = fma2(nu2, f0, fm[T2]);
  }

  // both biased reconstructions of every field (src/weno.cpp:77-152)
  f2 rl[NEQ], rr[NEQ];
#pragma unroll
  for (int n = 0; n < NEQ; ++n) {
    f2 numL, denL, numRn, denR;
    weno5_pair_x2(w[n], numL, denL, numRn, denR);
    rl[n] = fma2(numL, rcp2(denL), w[n][2]);
    rr[n] = fma2(numRn, mul2(mone, rcp2(denR)), w[n][3]);
  }

  // back to conserved perturbations
  f2 rhoL, mL[3], EL, rhoR, mR[3], ER;
  const f2 uncc = mul2(un, cc);
  {
    const f2 sp = add2(rl[0], rl[2]), dm = sub2(rl[2], rl[0]);
    rhoL = add2(sp, rl[1]);
    mL[D] = fma2(un, rhoL, mul2(cc, dm));
    mL[T1] = fma2(u1, rhoL, rl[3]);
    mL[T2] = fma2(u2, rhoL, rl[4]);
    EL = fma2(u2, rl[4], fma2(u1, rl[3], fma2(hq2, rl[1], fma2(uncc, dm, mul2(HH, sp)))));
  }
  {
    const f2 sp = add2(rr[0], rr[2]), dm = sub2(rr[2], rr[0]);
    rhoR = add2(sp, rr[1]);
    mR[D] = fma2(un, rhoR, mul2(cc, dm));
    mR[T1] = fma2(u1, rhoR, rr[3]);
    mR[T2] = fma2(u2, rhoR, rr[4]);
    ER = fma2(u2, rr[4], fma2(u1, rr[3], fma2(hq2, rr[1], fma2(uncc, dm, mul2(HH, sp)))));
  }

  // local Lax-Friedrichs flux, doubled (src/lf_flux.cpp:32-99)
  const f2 rref = bc(C.rho_ref), pref = bc(C.p_ref), gamma = bc(C.gamma);
  const f2 dL = add2(rref, rhoL), dR = add2(rref, rhoR);
  const f2 ip = rcp2(mul2(dL, dR));
  const f2 iL = mul2(ip, dR), iR = mul2(ip, dL);
  f2 vL[3], vR[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    vL[a] = mul2(mL[a], iL);
    vR[a] = mul2(mR[a], iR);
  }
  const f2 kL = fma2(mL[2], vL[2], fma2(mL[1], vL[1], mul2(mL[0], vL[0])));
  const f2 kR = fma2(mR[2], vR[2], fma2(mR[1], vR[1], mul2(mR[0], vR[0])));
  const f2 pL = mul2(gam1, fma2(bc(-0.5f), kL, EL));
  const f2 pR = mul2(gam1, fma2(bc(-0.5f), kR, ER));
  const f2 c2L = mul2(mul2(gamma, iL), add2(pref, pL)), c2R = mul2(mul2(gamma, iR), add2(pref, pR));
  const f2 cL = mul2(c2L, rsqrt2(c2L)), cR = mul2(c2R, rsqrt2(c2R));
  const f2 alpha = lanes(fmaxf(fabsf(vR[D].v.x) + cR.v.x, fabsf(vL[D].v.x) + cL.v.x),
                         fmaxf(fabsf(vR[D].v.y) + cR.v.y, fabsf(vL[D].v.y) + cL.v.y));
  const f2 fL = mL[D], fR = mR[D];
  out[0] = fma2(alpha, sub2(rhoL, rhoR), add2(fL, fR));
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const f2 fLa = (a == D) ? fma2(fL, vL[a], add2(pL, pR)) : mul2(fL, vL[a]);
    out[1 + a] = fma2(alpha, sub2(mL[a], mR[a]), fma2(fR, vR[a], fLa));
  }
  const f2 gi = bc(C.gam1_inv);
  const f2 HLf = fma2(c2L, gi, mul2(half, mul2(kL, iL)));
  const f2 HRf = fma2(c2R, gi, mul2(half, mul2(kR, iR)));
  out[4] = fma2(alpha, sub2(EL, ER), fma2(fR, HRf, mul2(fL, HLf)));
}

// Threads of 32 x (tile_rows / 2): a thread takes rows j and j+1 of its tile
// (the tile table is the one of the other stage kernels).  When JM is odd the
// last row's partner lane repeats the row and is not stored.
template <int D>
__global__ void __maxnreg__(128) k_inviscid_x2(const SolveDev* __restrict__ solves,
                                               const TileRef* __restrict__ tiles, int ntiles) {
  const int rows = 2 * (int)(blockDim.x / TILE_X);
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const TileRef tr = tiles[t];
    const SolveDev& s = solves[tr.solve];
    if (!s.ctl->active) continue;
    const int i = tr.ti * TILE_X + (int)(threadIdx.x % TILE_X);
    const int j = tr.tj * rows + 2 * (int)(threadIdx.x / TILE_X);
    const int k = tr.tk;
    if (i >= s.IM || j >= s.JM) continue;
    const bool pair = j + 1 < s.JM;
    const long long c0 = pad_off(s, i, j, k);
    const long long st = D == 0 ? 1ll : (D == 1 ? (long long)s.nx : (long long)s.nx * s.ny);
    // y faces: row j+1's stencil is row j's shifted by one cell, so its offsets
    // are written as row j's (c0 + k st), and the five shared cells' loads are
    // the same expressions.  An unpaired last row's partner lane then reads the
    // ghost row JM (inside the padding) and is not stored.
    const long long c1 = (D == 1 || pair) ? c0 + s.nx : c0;
    const long long V = s.V;
    const long long l1 = D == 1 ? c0 : c1 - st, r1 = D == 1 ? c0 + st : c1;
    const SideX2 Ls = side_x2(at(s, s.PA, V, c0 - st), at(s, s.PB, V, c0 - st), at(s, s.PA, V, l1),
                              at(s, s.PB, V, l1));
    const SideX2 Rs = side_x2(at(s, s.PA, V, c0), at(s, s.PB, V, c0), at(s, s.PA, V, r1), at(s, s.PB, V, r1));
    auto cell = [&](int m, f2(&fc)[NEQ]) {
      const long long o0 = c0 + (m - 3) * st, o1 = D == 1 ? c0 + (m - 2) * st : c1 + (m - 3) * st;
      const float4 a0 = at(s, s.U4, V, o0), a1 = at(s, s.U4, V, o1);
      fc[0] = lanes(a0.x, a1.x);
      fc[1] = lanes(a0.y, a1.y);
      fc[2] = lanes(a0.z, a1.z);
      fc[3] = lanes(a0.w, a1.w);
      fc[4] = lanes(at(s, s.UE, V, o0), at(s, s.UE, V, o1));
    };
    f2 f[NEQ];
    face_core_x2<D>(s.cf, Ls, Rs, cell, f);
    // Packed for the update's loads: equations 0-3 as one float4 per face, then
    // the energy flux in a block of its own (SolveDev::Ff).
    float4* F4 = reinterpret_cast<float4*>(s.Ff[D]);
    float* FE = s.Ff[D] + 4 * s.IV;
    const long long fo = int_off(s, i, j, k);
    at(s, F4, s.IV, fo) = make_float4(f[0].v.x, f[1].v.x, f[2].v.x, f[3].v.x);
    at(s, FE, s.IV, fo) = f[4].v.x;
    if (pair) {
      at(s, F4, s.IV, fo + s.IM) = make_float4(f[0].v.y, f[1].v.y, f[2].v.y, f[3].v.y);
      at(s, FE, s.IV, fo + s.IM) = f[4].v.y;
    }
  }
}

// Binary64 faces, one per thread.  Register cap 128 (16 warps per SM at 128
// threads per CTA; measured 3.4% faster than the same kernel under
// __launch_bounds__(256)).
template <int D, typename R>
__global__ void __maxnreg__(128) k_inviscid(const SolveDev* __restrict__ solves, const TileRef* __restrict__ tiles,
                                            int ntiles, int stage) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    TileCell tc = tile_cell(tiles[t], 0);
    const SolveDev& s = solves[tc.s];
    if (!s.ctl->active) continue;
    if (tc.i >= s.IM || tc.j >= s.JM) continue;
    const R* U = stage == 1 ? s.Q : s.Qp;
    R* F = s.F[D];
    R f[NEQ];
    face_flux<D, R>(s, U, pad_off(s, tc.i, tc.j, tc.k), f);
    const long long fo = int_off(s, tc.i, tc.j, tc.k);
#pragma unroll
    for (int n = 0; n < NEQ; ++n) at(s, F, NEQ * s.IV, n * s.IV + fo) = f[n];
  }
}

// ---------------------------------------------------------------------------
// Viscous fluxes on the NGV ring (src/calc_gradient.cpp:17-66,
// src/Block3d.cpp:750-868).  d/dx f = ((f[-2]-f[+2])/12 + (f[+1]-f[-1])*2/3) / dx,
// evaluated with the 1/dx folded into the two weights.
// FP32-mixed: T is stored as T - T_ref; its derivatives are the same.

template <typename R>
__device__ __forceinline__ R d4v(R m2, R p2, R m1, R p1, R c12h, R c23h) {
  if constexpr (sizeof(R) == 8) {
    return fma(m2 - p2, c12h, (p1 - m1) * c23h);
  } else {
    return (m2 - p2) * c12h + (p1 - m1) * c23h;
  }
}
template <typename R>
__device__ __forceinline__ R d4(const SolveDev& s, const R* __restrict__ f, long long o, long long st, R c12h,
                               R c23h) {
  const long long V = s.V;
  return d4v<R>(at(s, f, V, o - 2 * st), at(s, f, V, o + 2 * st), at(s, f, V, o - st), at(s, f, V, o + st), c12h,
                c23h);
}
// Register caps: 64 for binary64 (FP64-pipe bound; lower caps measured no
// faster) and 40 for binary32 (memory bound; 4% faster than at 48, spills at 32).
template <typename R>
__global__ void __maxnreg__(sizeof(R) == 4 ? 40 : 64) k_viscous(const SolveDev* __restrict__ solves,
                                                                const TileRef* __restrict__ tiles, int ntiles) {
  constexpr bool MIXED = sizeof(R) == 4;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    TileCell tc;
    if constexpr (MIXED) {
      // row tiles (32 x rows), the overhang of each row idle
      tc = tile_cell(tiles[t], -NGV);
      if (!solves[tc.s].ctl->active) continue;
      if (tc.i >= solves[tc.s].IM + NGV || tc.j >= solves[tc.s].JM + NGV) continue;
    } else {
      // Binary64 (FP64-pipe bound): plane tiles over the NGV ring, consecutive
      // points of a k-plane, so no lane idles at the end of a row (rx = IM + 4
      // is rarely a multiple of 32).  Row tiles measured faster for binary32.
      const TileRef tr = tiles[t];
      const SolveDev& sp = solves[tr.solve];
      if (!sp.ctl->active) continue;
      const long long p = plane_tile_first(tr, (int)blockDim.x) + threadIdx.x;
      if (p >= (long long)sp.rx * sp.ry) continue;
      tc.s = tr.solve;
      tc.j = (int)(p / sp.rx);
      tc.i = (int)(p - (long long)tc.j * sp.rx) - NGV;
      tc.j -= NGV;
      tc.k = (int)tr.tk - NGV;
    }
    const SolveDev& s = solves[tc.s];
    const long long o = pad_off(s, tc.i, tc.j, tc.k);
    const long long sy = s.nx, sz = (long long)s.nx * s.ny;
    const Consts<R>& CS = consts_of<R>(s);
    const R ax = CS.c12x, bx = CS.c23x, ay = CS.c12y, by = CS.c23y, az = CS.c12z, bz = CS.c23z;
    R ux, uy, uz, vx, vy, vz, wx, wy, wz, Tx, Ty, Tz, Tl, uu, vv, ww;
    if constexpr (MIXED) {
      // (u, v, w, T - T_ref) packed: four 16-byte loads per direction
      auto grad = [&](long long st, float c12h, float c23h, float& gu, float& gv, float& gw, float& gT) {
        const float4 m2 = at(s, s.PA, s.V, o - 2 * st), p2 = at(s, s.PA, s.V, o + 2 * st),
                     m1 = at(s, s.PA, s.V, o - st), p1 = at(s, s.PA, s.V, o + st);
        gu = d4v(m2.x, p2.x, m1.x, p1.x, c12h, c23h);
        gv = d4v(m2.y, p2.y, m1.y, p1.y, c12h, c23h);
        gw = d4v(m2.z, p2.z, m1.z, p1.z, c12h, c23h);
        gT = d4v(m2.w, p2.w, m1.w, p1.w, c12h, c23h);
      };
      grad(1, ax, bx, ux, vx, wx, Tx);
      grad(sy, ay, by, uy, vy, wy, Ty);
      grad(sz, az, bz, uz, vz, wz, Tz);
      const float4 a = at(s, s.PA, s.V, o);
      uu = a.x, vv = a.y, ww = a.z;
      Tl = CS.T_ref + a.w;
    } else {
      const PrimSet<double>& P = s.pd;
      ux = d4<R>(s, P.u, o, 1, ax, bx), uy = d4<R>(s, P.u, o, sy, ay, by), uz = d4<R>(s, P.u, o, sz, az, bz);
      vx = d4<R>(s, P.v, o, 1, ax, bx), vy = d4<R>(s, P.v, o, sy, ay, by), vz = d4<R>(s, P.v, o, sz, az, bz);
      wx = d4<R>(s, P.w, o, 1, ax, bx), wy = d4<R>(s, P.w, o, sy, ay, by), wz = d4<R>(s, P.w, o, sz, az, bz);
      Tx = d4<R>(s, P.T, o, 1, ax, bx), Ty = d4<R>(s, P.T, o, sy, ay, by), Tz = d4<R>(s, P.T, o, sz, az, bz);
      uu = at(s, P.u, s.V, o), vv = at(s, P.v, s.V, o), ww = at(s, P.w, s.V, o);
      Tl = at(s, P.T, s.V, o);
    }
    const R C = CS.C_T_inf;
    // Sutherland's law, (1 + C) / (T + C) * T^1.5 (src/Block3d.cpp:777), as
    // (1 + C) T^2 / sqrt(T (T + C)^2): one reciprocal square root, no division.
    const R TC = Tl + C;
    const R C1 = sizeof(R) == 8 ? (R)s.C_T_inf1 : (R)1 + C;  // 1 + C (binary64: formed once on the host)
    const R mu = (C1 * (Tl * Tl)) * rsqrt(Tl * (TC * TC));
    if (tc.i >= 0 && tc.i < s.IM && tc.j >= 0 && tc.j < s.JM && tc.k >= 0 && tc.k < s.KM) {
      if constexpr (MIXED) {
        at(s, s.muf, s.V, o) = mu;
      } else {
        at(s, s.pd.mu, s.V, o) = mu;
      }
    }
    const R mr = mu * CS.Re_inv;
    const R m23 = (R)(2.0 / 3.0) * mr;
    const R txx = m23 * ((R)2 * ux - vy - wz);
    const R tyy = m23 * ((R)2 * vy - ux - wz);
    const R tzz = m23 * ((R)2 * wz - ux - vy);
    const R txy = mr * (uy + vx);
    const R txz = mr * (uz + wx);
    const R tyz = mr * (vz + wy);
    const R mk = mr * CS.kappa;
    const long long r = ring_off(s, tc.i, tc.j, tc.k);
    const long long RV = s.RV;
    // Ev, Fv, Gv (src/Block3d.cpp:812-868) share their stresses: nine terms.
    const R ex = uu * txx + vv * txy + ww * txz - mk * Tx;
    const R ey = uu * txy + vv * tyy + ww * tyz - mk * Ty;
    const R ez = uu * txz + vv * tyz + ww * tzz - mk * Tz;
    if constexpr (MIXED) {
      // grouped by differencing direction: Ev, Fv, Gv as one float4 each
      at(s, s.Tvg, 3 * RV, r) = make_float4(txx, txy, txz, ex);
      at(s, s.Tvg, 3 * RV, RV + r) = make_float4(txy, tyy, tyz, ey);
      at(s, s.Tvg, 3 * RV, 2 * RV + r) = make_float4(txz, tyz, tzz, ez);
    } else {
      const long long n9 = kViscTerms * RV;
      at(s, s.Tv, n9, TXX * RV + r) = txx;
      at(s, s.Tv, n9, TYY * RV + r) = tyy;
      at(s, s.Tv, n9, TZZ * RV + r) = tzz;
      at(s, s.Tv, n9, TXY * RV + r) = txy;
      at(s, s.Tv, n9, TXZ * RV + r) = txz;
      at(s, s.Tv, n9, TYZ * RV + r) = tyz;
      at(s, s.Tv, n9, EX * RV + r) = ex;
      at(s, s.Tv, n9, EY * RV + r) = ey;
      at(s, s.Tv, n9, EZ * RV + r) = ez;
    }
  }
}

// ---------------------------------------------------------------------------
// RK3 stage update fused with the periodic ghost fill and the primitive
// recovery (src/Block3d.cpp:870-962, src/boundary_condition.cpp:4-231,
// src/Block3d.cpp:359-385).  Each interior cell writes its new state and
// primitives to itself and to every ghost cell that is its periodic image, which
// is exactly what the reference's x, y, z halo sweeps leave there.
// FP32-mixed: the flux differences are binary32, the RK3 accumulation of the
// conserved state binary64.

// STAGE 1..3 makes the stage a compile-time constant, so each launch's code
// holds one RK3 combination and no cell evaluates another stage's arithmetic
// (the binary64 update); STAGE 0 takes it at run time from rstage (the FP32-mixed
// update, whose per-launch weights already keep one combination per cell and
// which allocates registers better this way).
template <typename R, int STAGE, bool FF = false>
__device__ __forceinline__ void update_tiles(const SolveDev* __restrict__ solves, const TileRef* __restrict__ tiles,
                                             int ntiles, int rstage) {
  const int stage = STAGE ? STAGE : rstage;
  constexpr bool MIXED = sizeof(R) == 4;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    TileCell tc = tile_cell(tiles[t], 0);
    const SolveDev& s = solves[tc.s];
    SolveCtl* ctl = s.ctl;
    if (!ctl->active) continue;
    const int i = tc.i, j = tc.j, k = tc.k;
    if (i >= s.IM || j >= s.JM) continue;
    const double dt = ctl->dt;
    const long long o = pad_off(s, i, j, k);
    const long long fo = int_off(s, i, j, k);
    const long long fx = int_off(s, i + 1 == s.IM ? 0 : i + 1, j, k);
    const long long fy = int_off(s, i, j + 1 == s.JM ? 0 : j + 1, k);
    const long long fz = int_off(s, i, j, k + 1 == s.KM ? 0 : k + 1);
    const long long r = ring_off(s, i, j, k);
    const long long ry = s.rx, rz = (long long)s.rx * s.ry;
    const long long IV = s.IV, V = s.V, RV = s.RV;
    const R* F0;
    const R* F1;
    const R* F2;
    if constexpr (MIXED) {
      F0 = s.Ff[0], F1 = s.Ff[1], F2 = s.Ff[2];
    } else {
      F0 = s.F[0], F1 = s.F[1], F2 = s.F[2];
    }
    // The face fluxes are stored doubled: hf = 0.5 / h.
    const R idx = consts_of<R>(s).hfx, idy = consts_of<R>(s).hfy, idz = consts_of<R>(s).hfz;

    const Consts<R>& CS = consts_of<R>(s);
    // FP32-mixed stages 2 and 3: the binary32 weight of dt df (1/4 or 2/3 of dt,
    // formed once per step with dt).
    const float cdt = MIXED && stage != 1 ? ctl->cdt[stage - 2] : 0.0f;
    // FP32-mixed stages 2 and 3: the weights of q0 and qp (one pair per launch,
    // so each cell evaluates one combination).
    const double ca = stage == 2 ? 0.75 : 1.0 / 3.0, cb = stage == 2 ? 0.25 : 2.0 / 3.0;
    // FP32-mixed: minus the 4th-order central divergence of the viscous fluxes
    // (src/Block3d.cpp:887-910, calc_viscous_flux_contribution:
    // ((f[-2]-f[+2])/12 + (f[+1]-f[-1])*2/3) / h per direction) of equations
    // 1..4, one direction at a time from its grouped terms: four 16-byte loads
    // per direction.
    float dv[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if constexpr (MIXED) {
      // g: the direction's block of the grouped terms plus this ring point
      auto direction = [&](long long g, long long st, float c12, float c23) {
        const long long n3 = 3 * RV;
        const float4 m2 = at(s, s.Tvg, n3, g - 2 * st), p2 = at(s, s.Tvg, n3, g + 2 * st),
                     m1 = at(s, s.Tvg, n3, g - st), p1 = at(s, s.Tvg, n3, g + st);
        dv[0] = fmaf(p1.x - m1.x, -c23, fmaf(m2.x - p2.x, -c12, dv[0]));
        dv[1] = fmaf(p1.y - m1.y, -c23, fmaf(m2.y - p2.y, -c12, dv[1]));
        dv[2] = fmaf(p1.z - m1.z, -c23, fmaf(m2.z - p2.z, -c12, dv[2]));
        dv[3] = fmaf(p1.w - m1.w, -c23, fmaf(m2.w - p2.w, -c12, dv[3]));
      };
      direction(r, 1, CS.c12x, CS.c23x);
      direction(RV + r, ry, CS.c12y, CS.c23y);
      direction(2 * RV + r, rz, CS.c12z, CS.c23z);
    }
    // FP32-mixed: then the inviscid flux differences along x, y, z, each
    // equation's chain in that order; per direction the cell's and its
    // neighbour's face are a float4 (equations 0-3) and a float (equation 4).
    float dfm[NEQ];
    if constexpr (MIXED) {
      const float* Fd[3] = {F0, F1, F2};
      const long long fn[3] = {fx, fy, fz};
      const float hd[3] = {idx, idy, idz};
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float4* F4 = reinterpret_cast<const float4*>(Fd[d]);
        const float* FE = Fd[d] + 4 * IV;
        const float4 a = at(s, F4, IV, fo), b = at(s, F4, IV, fn[d]);
        const float ea = at(s, FE, IV, fo), eb = at(s, FE, IV, fn[d]);
        const float dif[NEQ] = {b.x - a.x, b.y - a.y, b.z - a.z, b.w - a.w, eb - ea};
#pragma unroll
        for (int n = 0; n < NEQ; ++n)
          dfm[n] = fmaf(dif[n], hd[d], d > 0 ? dfm[n] : (n > 0 ? dv[n - 1] : 0.0f));
      }
    }
    // CBNS_FP64_FF: every equation's chain of the binary64 update below (the
    // inviscid flux differences along x, y, z, then minus the 4th-order viscous
    // divergence along x, y, z) in float-float arithmetic, all equations at
    // once: per direction, the faces' fluxes are three 16-byte loads per face and
    // the four terms differenced along it two 16-byte loads per ring point.
    // Accumulated without renormalising, rounded to binary64 once per equation.
    double dff[NEQ];
    if constexpr (FF) {
      auto cf = [](float2 v) { return ff{v.x, v.y}; };
      ff acc[NEQ];
      const long long n3 = 3 * IV, n6 = 6 * RV;
      const long long fn[3] = {fx, fy, fz}, rs[3] = {1, ry, rz};
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float4* G = s.FFa[d];
        const float4 o0 = at(s, G, n3, 3 * fo), o1 = at(s, G, n3, 3 * fo + 1), o2 = at(s, G, n3, 3 * fo + 2);
        const float4 x0 = at(s, G, n3, 3 * fn[d]), x1 = at(s, G, n3, 3 * fn[d] + 1),
                     x2 = at(s, G, n3, 3 * fn[d] + 2);
        const ff dif[NEQ] = {ff{x0.x, x0.y} - ff{o0.x, o0.y}, ff{x0.z, x0.w} - ff{o0.z, o0.w},
                             ff{x1.x, x1.y} - ff{o1.x, o1.y}, ff{x1.z, x1.w} - ff{o1.z, o1.w},
                             ff{x2.x, x2.y} - ff{o2.x, o2.y}};
        const ff h = cf(s.ff_hf[d]);
#pragma unroll
        for (int n = 0; n < NEQ; ++n) acc[n] = d == 0 ? dif[n] * h : ff_fma_acc(dif[n], h, acc[n]);
      }
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float4* T = s.TvG;
        const long long b0 = 2 * (d * RV + r), sd = 2 * rs[d];
        const float4 m2a = at(s, T, n6, b0 - 2 * sd), m2b = at(s, T, n6, b0 - 2 * sd + 1);
        const float4 p2a = at(s, T, n6, b0 + 2 * sd), p2b = at(s, T, n6, b0 + 2 * sd + 1);
        const float4 m1a = at(s, T, n6, b0 - sd), m1b = at(s, T, n6, b0 - sd + 1);
        const float4 p1a = at(s, T, n6, b0 + sd), p1b = at(s, T, n6, b0 + sd + 1);
        const ff m2[4] = {ff{m2a.x, m2a.y}, ff{m2a.z, m2a.w}, ff{m2b.x, m2b.y}, ff{m2b.z, m2b.w}};
        const ff p2[4] = {ff{p2a.x, p2a.y}, ff{p2a.z, p2a.w}, ff{p2b.x, p2b.y}, ff{p2b.z, p2b.w}};
        const ff m1[4] = {ff{m1a.x, m1a.y}, ff{m1a.z, m1a.w}, ff{m1b.x, m1b.y}, ff{m1b.z, m1b.w}};
        const ff p1[4] = {ff{p1a.x, p1a.y}, ff{p1a.z, p1a.w}, ff{p1b.x, p1b.y}, ff{p1b.z, p1b.w}};
        const ff c12 = -cf(s.ff_c12[d]), c23 = -cf(s.ff_c23[d]);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          acc[1 + q] = ff_fma_acc(m2[q] - p2[q], c12, acc[1 + q]);
          acc[1 + q] = ff_fma_acc(p1[q] - m1[q], c23, acc[1 + q]);
        }
      }
#pragma unroll
      for (int n = 0; n < NEQ; ++n) dff[n] = ff_to_double(acc[n]);
    }
    double qn[NEQ];
#pragma unroll
    for (int n = 0; n < NEQ; ++n) {
      R df;
      if constexpr (MIXED) {
        df = dfm[n];
      } else if constexpr (FF) {
        df = dff[n];
      } else {
        // Inviscid flux differences, then minus the viscous divergence, as one
        // chain of fused multiply-adds with the 1/h-folded weights negated.
        const long long n5 = NEQ * IV;
        df = (at(s, F0, n5, n * IV + fx) - at(s, F0, n5, n * IV + fo)) * idx;
        df = fma_(at(s, F1, n5, n * IV + fy) - at(s, F1, n5, n * IV + fo), idy, df);
        df = fma_(at(s, F2, n5, n * IV + fz) - at(s, F2, n5, n * IV + fo), idz, df);
        if (n > 0) {
          // the term differenced along x, y, z in this equation: its block plus r
          const long long n9 = kViscTerms * RV;
          const long long vx = visc_term(n, 0) * RV + r, vy = visc_term(n, 1) * RV + r,
                          vz = visc_term(n, 2) * RV + r;
          const double* Tv = s.Tv;
          df = fma_(at(s, Tv, n9, vx - 2) - at(s, Tv, n9, vx + 2), -CS.c12x, df);
          df = fma_(at(s, Tv, n9, vx + 1) - at(s, Tv, n9, vx - 1), -CS.c23x, df);
          df = fma_(at(s, Tv, n9, vy - 2 * ry) - at(s, Tv, n9, vy + 2 * ry), -CS.c12y, df);
          df = fma_(at(s, Tv, n9, vy + ry) - at(s, Tv, n9, vy - ry), -CS.c23y, df);
          df = fma_(at(s, Tv, n9, vz - 2 * rz) - at(s, Tv, n9, vz + 2 * rz), -CS.c12z, df);
          df = fma_(at(s, Tv, n9, vz + rz) - at(s, Tv, n9, vz - rz), -CS.c23z, df);
        }
      }
      const double q0 = at(s, s.Q, NEQ * V, n * V + o);
      if (MIXED && stage != 1) {
        // FP32-mixed stages 2 and 3: the increment c dt df in binary32 (df has
        // binary32 accuracy), the combination of the binary64 states in binary64:
        // 3/4 q0 + 1/4 qp - 1/4 dt df and 1/3 q0 + 2/3 qp - 2/3 dt df.
        const double qp = at(s, s.Qp, NEQ * V, n * V + o);
        const double inc = (double)(cdt * (float)df);
        qn[n] = fma(ca, q0, fma(cb, qp, -inc));
      } else {
        const double dfd = (double)df;
        if (stage == 1) {
          qn[n] = q0 - dt * dfd;
        } else if (stage == 2) {
          qn[n] = 0.75 * q0 + 0.25 * (at(s, s.Qp, NEQ * V, n * V + o) - dt * dfd);
        } else {
          qn[n] = (q0 + 2.0 * (at(s, s.Qp, NEQ * V, n * V + o) - dt * dfd)) * (1.0 / 3.0);
        }
      }
    }
    double* out = stage == 3 ? s.Q : s.Qp;

    // Primitives of the new state (once), then the cell and its ghost images.
    double uu = 0, vv = 0, ww = 0, pp = 0, TT = 0, sr = 0, HH = 0;
    MixedCell mc;
    ff fq[NEQ];
    PrimsFF pf;
    if constexpr (MIXED) {
      mc = mixed_cell(s, qn);
      if (!(mc.rho > 0.0f) || !(s.cf.p_ref + mc.p > 0.0f)) atomicOr(&ctl->status, kStatusNonphysical);
    } else if constexpr (FF) {
      // CBNS_FP64_FF: the float-float split of the state (its perturbation of
      // the reference state) and its float-float primitives, the only copies
      // the float-float kernels read (binary64 primitives are formed on demand
      // for output)
#pragma unroll
      for (int n = 0; n < NEQ; ++n) {
        const float2 t2 = ff_split_state(s, n, qn[n]);
        fq[n] = ff{t2.x, t2.y};
      }
      pf = prims_ff(s, fq);
      if (!(qn[0] > 0.0) || !(pf.p.hi > 0.0f)) atomicOr(&ctl->status, kStatusNonphysical);
    } else {
      const Prims64 q = prims64(s, qn[0], qn[1], qn[2], qn[3], qn[4]);
      uu = q.u, vv = q.v, ww = q.w, pp = q.p, TT = q.T, sr = q.sr, HH = q.H;
      if (!(qn[0] > 0.0) || !(pp > 0.0)) atomicOr(&ctl->status, kStatusNonphysical);
    }

    // The cell itself, then its periodic images in the ghost layers: along each
    // axis a cell within NG of either end has one image (two when the extent is
    // below 2*NG).  Most cells have none, and take the first branch only.
    auto store = [&](long long d) {
#pragma unroll
      for (int n = 0; n < NEQ; ++n) at(s, out, NEQ * V, n * V + d) = qn[n];
      if constexpr (MIXED) {
        store_mixed(s, d, mc);
      } else if constexpr (FF) {
        const long long n5 = NEQ * V, np = kFFPrims * V;
        float2* QFo = stage == 3 ? s.QF : s.QpF;
#pragma unroll
        for (int n = 0; n < NEQ; ++n) at(s, QFo, n5, n * V + d) = make_float2(fq[n].hi, fq[n].lo);
        const ff pv[kFFPrims] = {pf.sr, pf.H, pf.u, pf.v, pf.w, pf.T};
#pragma unroll
        for (int b2 = 0; b2 < kFFPrims; ++b2) at(s, s.PF, np, b2 * V + d) = make_float2(pv[b2].hi, pv[b2].lo);
      } else {
        // the PrimSet arrays are consecutive blocks of V values from pd.rho
        double* b = s.pd.rho;
        const long long n8 = 8 * V;
        at(s, b, n8, d) = qn[0];
        at(s, b, n8, V + d) = uu;
        at(s, b, n8, 2 * V + d) = vv;
        at(s, b, n8, 3 * V + d) = ww;
        at(s, b, n8, 4 * V + d) = pp;
        at(s, b, n8, 5 * V + d) = TT;
        at(s, b, n8, 6 * V + d) = sr;
        at(s, b, n8, 7 * V + d) = HH;
      }
    };
    store(o);
    const bool xl = i < NG, xh = i >= s.IM - NG, yl = j < NG, yh = j >= s.JM - NG, zl = k < NG,
               zh = k >= s.KM - NG;
    if (xl || xh || yl || yh || zl || zh) {
      // Image m = a + 3 b + 9 c (m = 0 is the cell itself); per axis, slot 0 =
      // the cell's own coordinate, 1 = + extent (used when near the low end),
      // 2 = - extent (near the high end).  A rolled loop keeps few registers live.
      const long long sy = s.nx, sz = (long long)s.nx * s.ny;
#pragma unroll 1
      for (int m = 1; m < 27; ++m) {
        const int a = m % 3, b = (m / 3) % 3, c = m / 9;
        const bool use = (a == 0 || (a == 1 ? xl : xh)) && (b == 0 || (b == 1 ? yl : yh)) &&
                         (c == 0 || (c == 1 ? zl : zh));
        if (!use) continue;
        const long long ox = a == 0 ? 0 : (a == 1 ? (long long)s.IM : -(long long)s.IM);
        const long long oy = b == 0 ? 0 : (b == 1 ? (long long)s.JM : -(long long)s.JM);
        const long long oz = c == 0 ? 0 : (c == 1 ? (long long)s.KM : -(long long)s.KM);
        store(o + ox + oy * sy + oz * sz);
      }
    }
  }
}

// Register caps, measured at 256^3: the binary64 update (FP64-pipe bound) runs
// 11% faster at 80 registers (24 warps per SM, a few spills) than unconstrained
// (126 registers); the binary32 one (memory-latency bound) 12% faster at 64
// (32 warps per SM) than at 80.
// FF: CBNS_FP64_FF solves (float-float flux differences and copies).  That
// kernel is bound by memory latency, so its cap is set for occupancy: at 64
// registers eight 128-thread CTAs fit per SM (32 warps) against four at 128, and
// the launch took 1.34 instead of 1.67 ms at 256^3 despite 4-32 bytes of spill
// (80 registers: 1.46 ms); results bitwise the same.
template <typename R, int STAGE, bool FF>
__global__ void __maxnreg__(FF ? 64 : 80) k_update(const SolveDev* __restrict__ solves,
                                         const TileRef* __restrict__ tiles, int ntiles) {
  update_tiles<R, STAGE, FF>(solves, tiles, ntiles, STAGE);
}
__global__ void __maxnreg__(64) k_update_f32(const SolveDev* __restrict__ solves,
                                              const TileRef* __restrict__ tiles, int ntiles, int stage) {
  update_tiles<float, 0>(solves, tiles, ntiles, stage);
}

// ---------------------------------------------------------------------------
// Diagnostics (project-defined): kinetic energy and enstrophy with compensated
// binary64 sums.  Each CTA reduces its tiles to one (sum, error) pair per
// quantity in `partials` (scratch, 4 doubles per CTA); k_diag_finalize folds them
// in a fixed order, so the result is deterministic.

struct Comp {
  double s, e;
};

__device__ __forceinline__ Comp comp_add(Comp a, Comp b) {
  double t = a.s + b.s;
  double z = t - a.s;
  double err = (a.s - (t - z)) + (b.s - z);
  Comp r;
  r.s = t;
  r.e = a.e + b.e + err;
  return r;
}

__device__ __forceinline__ Comp warp_comp(Comp v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    Comp other;
    other.s = __shfl_down_sync(0xffffffffu, v.s, o);
    other.e = __shfl_down_sync(0xffffffffu, v.e, o);
    v = comp_add(v, other);
  }
  return v;
}

__device__ __forceinline__ double vel(const SolveDev& s, const double* Q, long long V, long long o, int n) {
  return at(s, Q, NEQ * V, n * V + o) / at(s, Q, NEQ * V, o);
}
__device__ __forceinline__ double dvel(const SolveDev& s, const double* Q, long long V, long long o, long long st,
                                       int n, double inv_h) {
  const double c12 = 1.0 / 12.0, c23 = 2.0 / 3.0;
  return ((vel(s, Q, V, o - 2 * st, n) - vel(s, Q, V, o + 2 * st, n)) * c12 +
          (vel(s, Q, V, o + st, n) - vel(s, Q, V, o - st, n)) * c23) * inv_h;
}

__global__ void __launch_bounds__(TILE_THREADS) k_diag(const SolveDev* __restrict__ solves, int sidx,
                                                       const TileRef* __restrict__ tiles, int ntiles,
                                                       double* __restrict__ partials) {
  __shared__ Comp red[2][TILE_THREADS / 32];
  const SolveDev& s = solves[sidx];
  Comp ke{0.0, 0.0}, en{0.0, 0.0};
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    TileCell tc = tile_cell(tiles[t], 0);
    if (tc.i >= s.IM || tc.j >= s.JM) continue;
    const long long o = pad_off(s, tc.i, tc.j, tc.k);
    const long long V = s.V, sy = s.nx, sz = (long long)s.nx * s.ny;
    const double* Q = s.Q;
    const double r = at(s, Q, NEQ * V, o);
    const double u = vel(s, Q, V, o, 1), v = vel(s, Q, V, o, 2), w = vel(s, Q, V, o, 3);
    const double wxc = dvel(s, Q, V, o, sy, 3, s.inv_dy) - dvel(s, Q, V, o, sz, 2, s.inv_dz);
    const double wyc = dvel(s, Q, V, o, sz, 1, s.inv_dz) - dvel(s, Q, V, o, 1, 3, s.inv_dx);
    const double wzc = dvel(s, Q, V, o, 1, 2, s.inv_dx) - dvel(s, Q, V, o, sy, 1, s.inv_dy);
    ke = comp_add(ke, Comp{0.5 * r * (u * u + v * v + w * w), 0.0});
    en = comp_add(en, Comp{0.5 * r * (wxc * wxc + wyc * wyc + wzc * wzc), 0.0});
  }
  ke = warp_comp(ke);
  en = warp_comp(en);
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = ke;
    red[1][threadIdx.x >> 5] = en;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    Comp a = red[0][0], b = red[1][0];
    for (int q = 1; q < TILE_THREADS / 32; ++q) {
      a = comp_add(a, red[0][q]);
      b = comp_add(b, red[1][q]);
    }
    partials[4 * blockIdx.x + 0] = a.s;
    partials[4 * blockIdx.x + 1] = a.e;
    partials[4 * blockIdx.x + 2] = b.s;
    partials[4 * blockIdx.x + 3] = b.e;
  }
}

__global__ void k_diag_finalize(const double* __restrict__ partials, int nparts, double inv_n,
                                double* __restrict__ out) {
  __shared__ Comp red[2][32];
  Comp ke{0.0, 0.0}, en{0.0, 0.0};
  for (int q = threadIdx.x; q < nparts; q += blockDim.x) {
    ke = comp_add(ke, Comp{partials[4 * q], partials[4 * q + 1]});
    en = comp_add(en, Comp{partials[4 * q + 2], partials[4 * q + 3]});
  }
  ke = warp_comp(ke);
  en = warp_comp(en);
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = ke;
    red[1][threadIdx.x >> 5] = en;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    Comp a = red[0][0], b = red[1][0];
    for (int q = 1; q < (int)(blockDim.x / 32); ++q) {
      a = comp_add(a, red[0][q]);
      b = comp_add(b, red[1][q]);
    }
    out[0] = (a.s + a.e) * inv_n;
    out[1] = (b.s + b.e) * inv_n;
  }
}

// ---------------------------------------------------------------------------
// Host-side launchers.  Each launch is bracketed by the profiler's events when
// profiling is on (pf may be null).

static int grid_for(int ntiles, int max_ctas) {
  if (ntiles <= 0) return 0;
  return max_ctas > 0 && ntiles > max_ctas ? max_ctas : ntiles;
}

// cbns_ff_kernels.cu
void launch_faces_ff(const SolveDev* d, const TileRef* tiles, int ntiles, int stage, int g, int nt,
                     cudaStream_t st, Profiler* pf);
void launch_viscous_ff(const SolveDev* d, const TileRef* ring, int nring, int g, int nt, cudaStream_t st,
                       Profiler* pf);

#define CBNS_LAUNCH(pf, id, st, ...) \
  do {                               \
    if (pf) (pf)->before(id, st);    \
    __VA_ARGS__;                     \
    if (pf) (pf)->after(st);         \
  } while (0)

cudaError_t launch_prepare(const SolveDev* d, const TileRef* tiles, int ntiles, cudaStream_t st, Profiler* pf) {
  if (ntiles == 0) return cudaSuccess;
  CBNS_LAUNCH(pf, KID_PREPARE, st, (k_prepare<<<grid_for(ntiles, 0), TILE_THREADS, 0, st>>>(d, tiles, ntiles)));
  return cudaGetLastError();
}

cudaError_t launch_layout(const SolveDev* d, int sidx, const double* src, double* dst, bool to_soa,
                          long long V, cudaStream_t st, Profiler* pf) {
  int blocks = (int)((V + 255) / 256);
  if (blocks > 65535) blocks = 65535;
  if (to_soa)
    CBNS_LAUNCH(pf, KID_LAYOUT, st, (k_aos_to_soa<<<blocks, 256, 0, st>>>(d, sidx, src, dst)));
  else
    CBNS_LAUNCH(pf, KID_LAYOUT, st, (k_soa_to_aos<<<blocks, 256, 0, st>>>(d, sidx, src, dst)));
  return cudaGetLastError();
}

cudaError_t launch_init_tgv(const SolveDev* d, int sidx, const TileRef* tiles, int ntiles, double p_inf,
                            const PerturbMode* modes, int nmodes, cudaStream_t st) {
  if (nmodes < 0 || nmodes > kMaxModes) return cudaErrorInvalidValue;
  ModeTable mt;
  mt.n = nmodes;
  for (int m = 0; m < nmodes; ++m) mt.m[m] = modes[m];
  k_init_tgv<<<grid_for(ntiles, 0), TILE_THREADS, 0, st>>>(d, sidx, tiles, ntiles, p_inf, mt);
  return cudaGetLastError();
}

cudaError_t launch_prims_double(const SolveDev* d, const TileRef* tiles, int ntiles, cudaStream_t st) {
  if (ntiles == 0) return cudaSuccess;
  k_prims_double<<<grid_for(ntiles, 0), TILE_THREADS, 0, st>>>(d, tiles, ntiles);
  return cudaGetLastError();
}

// The reduction runs persistent whatever the stage kernels do: a few CTAs per SM
// keep the atomics on the control block few.
constexpr int kDtReduceCtas = 152 * 8;

template <typename R, bool FF>
static void dt_reduce_ty(const SolveDev* d, const TileRef* tiles, int ntiles, double t_end, int use_t_end, int skip,
                         const LaunchCfg& cfg, cudaStream_t st, Profiler* pf) {
  const int g = grid_for(ntiles, (cfg.max_ctas > 0 && cfg.max_ctas < kDtReduceCtas) ? cfg.max_ctas : kDtReduceCtas);
  CBNS_LAUNCH(pf, KID_DT_REDUCE, st,
              (k_dt_reduce<R, FF><<<g, 32 * cfg.tile_rows, 0, st>>>(d, tiles, ntiles, t_end, use_t_end, skip)));
}

static void dt_reduce_prec(const SolveDev* d, const TileRef* tiles, int ntiles, double t_end, int use_t_end,
                           int skip, int precision, const LaunchCfg& cfg, cudaStream_t st, Profiler* pf) {
  if (precision == CBNS_FP32_MIXED)
    dt_reduce_ty<float, false>(d, tiles, ntiles, t_end, use_t_end, skip, cfg, st, pf);
  else if (precision == CBNS_FP64_FF)
    dt_reduce_ty<double, true>(d, tiles, ntiles, t_end, use_t_end, skip, cfg, st, pf);
  else
    dt_reduce_ty<double, false>(d, tiles, ntiles, t_end, use_t_end, skip, cfg, st, pf);
}

cudaError_t launch_dt(const SolveDev* d, int nsolves, const TileRef* tiles, int ntiles, double t_end,
                      bool use_t_end, int precision, const LaunchCfg& cfg, cudaStream_t st, Profiler* pf) {
  if (ntiles > 0) dt_reduce_prec(d, tiles, ntiles, t_end, use_t_end ? 1 : 0, 1, precision, cfg, st, pf);
  CBNS_LAUNCH(pf, KID_DT_FINALIZE, st,
              (k_dt_finalize<<<(nsolves + 127) / 128, 128, 0, st>>>(d, nsolves, t_end, use_t_end ? 1 : 0)));
  return cudaGetLastError();
}

cudaError_t launch_dt_raw(const SolveDev* d, int sidx, const TileRef* tiles, int ntiles, double* out,
                          int precision, const LaunchCfg& cfg, cudaStream_t st, Profiler* pf) {
  if (ntiles > 0) dt_reduce_prec(d, tiles, ntiles, 0.0, 0, 0, precision, cfg, st, pf);
  CBNS_LAUNCH(pf, KID_DT_FINALIZE, st, (k_dt_raw<<<1, 1, 0, st>>>(d, sidx, out)));
  return cudaGetLastError();
}

cudaError_t launch_reset_ctl(SolveCtl* ctl, double t, double t_end, cudaStream_t st) {
  k_reset_ctl<<<1, 1, 0, st>>>(ctl, t, t_end);
  return cudaGetLastError();
}

cudaError_t launch_set_dt(const SolveDev* d, int sidx, double dt, cudaStream_t st) {
  k_set_dt<<<1, 1, 0, st>>>(d, sidx, dt);
  return cudaGetLastError();
}

template <typename R>
static void stage_ty(const SolveDev* d, const StageTables& T, int stage, const LaunchCfg& cfg, bool ff,
                     cudaStream_t st, Profiler* pf) {
  const TileRef* tiles = T.tiles;
  const int ntiles = T.ntiles;
  const int g = grid_for(ntiles, cfg.max_ctas);
  const int nt = 32 * cfg.tile_rows;
  if constexpr (sizeof(R) == 4) {
    const int nt2 = 16 * cfg.tile_rows;  // two rows per thread
    CBNS_LAUNCH(pf, KID_INVISCID_X, st, (k_inviscid_x2<0><<<g, nt2, 0, st>>>(d, tiles, ntiles)));
    CBNS_LAUNCH(pf, KID_INVISCID_Y, st, (k_inviscid_x2<1><<<g, nt2, 0, st>>>(d, tiles, ntiles)));
    CBNS_LAUNCH(pf, KID_INVISCID_Z, st, (k_inviscid_x2<2><<<g, nt2, 0, st>>>(d, tiles, ntiles)));
  } else if (ff) {
    launch_faces_ff(d, tiles, ntiles, stage, g, nt, st, pf);
  } else {
    CBNS_LAUNCH(pf, KID_INVISCID_X, st, (k_inviscid<0, R><<<g, nt, 0, st>>>(d, tiles, ntiles, stage)));
    CBNS_LAUNCH(pf, KID_INVISCID_Y, st, (k_inviscid<1, R><<<g, nt, 0, st>>>(d, tiles, ntiles, stage)));
    CBNS_LAUNCH(pf, KID_INVISCID_Z, st, (k_inviscid<2, R><<<g, nt, 0, st>>>(d, tiles, ntiles, stage)));
  }
  if (ff)
    launch_viscous_ff(d, T.ring, T.nring, grid_for(T.nring, cfg.max_ctas), nt, st, pf);
  else
    CBNS_LAUNCH(pf, KID_VISCOUS, st,
                (k_viscous<R><<<grid_for(T.nring, cfg.max_ctas), nt, 0, st>>>(d, T.ring, T.nring)));
  if constexpr (sizeof(R) == 4) {
    CBNS_LAUNCH(pf, KID_UPDATE, st, (k_update_f32<<<g, nt, 0, st>>>(d, tiles, ntiles, stage)));
  } else {
    if (ff) {
      if (stage == 1) CBNS_LAUNCH(pf, KID_UPDATE, st, (k_update<R, 1, true><<<g, nt, 0, st>>>(d, tiles, ntiles)));
      else if (stage == 2) CBNS_LAUNCH(pf, KID_UPDATE, st, (k_update<R, 2, true><<<g, nt, 0, st>>>(d, tiles, ntiles)));
      else CBNS_LAUNCH(pf, KID_UPDATE, st, (k_update<R, 3, true><<<g, nt, 0, st>>>(d, tiles, ntiles)));
    } else {
      if (stage == 1) CBNS_LAUNCH(pf, KID_UPDATE, st, (k_update<R, 1, false><<<g, nt, 0, st>>>(d, tiles, ntiles)));
      else if (stage == 2) CBNS_LAUNCH(pf, KID_UPDATE, st, (k_update<R, 2, false><<<g, nt, 0, st>>>(d, tiles, ntiles)));
      else CBNS_LAUNCH(pf, KID_UPDATE, st, (k_update<R, 3, false><<<g, nt, 0, st>>>(d, tiles, ntiles)));
    }
  }
}

cudaError_t launch_stage(const SolveDev* d, const StageTables& T, int stage, const LaunchCfg& cfg, int precision,
                         cudaStream_t st, Profiler* pf) {
  if (T.ntiles == 0) return cudaSuccess;
  if (precision == CBNS_FP32_MIXED) stage_ty<float>(d, T, stage, cfg, false, st, pf);
  else stage_ty<double>(d, T, stage, cfg, precision == CBNS_FP64_FF, st, pf);
  return cudaGetLastError();
}

cudaError_t launch_diag(const SolveDev* d, int sidx, const TileRef* tiles, int ntiles, double* partials,
                        int nparts, double inv_n, double* out, cudaStream_t st, Profiler* pf) {
  CBNS_LAUNCH(pf, KID_DIAG, st, (k_diag<<<nparts, TILE_THREADS, 0, st>>>(d, sidx, tiles, ntiles, partials)));
  CBNS_LAUNCH(pf, KID_DIAG, st, (k_diag_finalize<<<1, 1024, 0, st>>>(partials, nparts, inv_n, out)));
  return cudaGetLastError();
}

}  // namespace cbns
