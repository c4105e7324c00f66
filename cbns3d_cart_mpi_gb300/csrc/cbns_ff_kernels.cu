// cbns_ff_kernels.cu — the float-float kernels of CBNS_FP64_FF solves, on the
// binary32 pipes (arithmetic: cbns_ff.cuh):
//   k_inviscid_ff<D>  the inviscid face fluxes, one face per thread: the binary64
//                     face kernel's scheme (Roe-averaged characteristic WENO5 with
//                     local Lax-Friedrichs splitting; src/Block3d.cpp:555-748,
//                     src/eigenvectors_roe.cpp, src/weno.cpp, src/lf_flux.cpp)
//   k_viscous_ff      the viscous terms on the NGV ring (src/calc_gradient.cpp:17-66,
//                     src/Block3d.cpp:750-868)
// Their inputs are the float-float copies of the state (its perturbation of the
// reference state) and of the primitives sqrt(rho), H, u, v, w, T that the update
// writes with the binary64 state; their
// outputs are float-float pairs packed for the update's 16-byte loads
// (SolveDev::FFa, TvG), and mu in binary64 for the time step.  Each step is the
// binary64 kernels' (cbns_kernels.cu: face_core, k_viscous), operation for
// operation where the float-float forms allow; the notes there give the algebra.
#include <cuda_runtime.h>

#include <mutex>

#include "cbns_device.cuh"
#include "cbns_ff.cuh"
#include "cbns_prof.h"

namespace cbns {

namespace {

__device__ __forceinline__ ff ld(const SolveDev& s, const float2* p, long long n, long long i) {
  const float2 v = at(s, p, n, i);
  return ff{v.x, v.y};
}

__device__ __forceinline__ ff cst(float2 v) { return ff{v.x, v.y}; }

// sqrt(rho), H and the velocity of one cell beside a face.
struct SideFF {
  ff sr, h, u, v, w;
};

__device__ __forceinline__ SideFF side_ff(const SolveDev& s, long long o) {
  const long long V = s.V, n5 = kFFPrims * V;
  const float2* P = s.PF;
  return SideFF{ld(s, P, n5, o), ld(s, P, n5, V + o), ld(s, P, n5, 2 * V + o), ld(s, P, n5, 3 * V + o),
                ld(s, P, n5, 4 * V + o)};
}

struct WenoFF {
  ff num, den;
};

// One biased WENO5 stencil as the binary64 weno5_side: the indicators taken four
// times over, 4 (eps + IS_k) = 13/3 D_k^2 + e_k^2 + 4 eps, a_k their squares,
// num = a2 a3 g1 + 6 a1 a3 g2 + 3 a1 a2 g3 and den = a2 a3 + 6 a1 a3 + 3 a1 a2.
__device__ __forceinline__ void weno5_side_ff(ff D1, ff C1, ff D2, ff C2, ff D3, ff C3, ff e1, ff e2, ff e3,
                                              ff g1, ff g2s, ff g3s, WenoFF& out) {
  constexpr ff eps4 = ff_const(4.0e-6);
  // the indicators and the denominator are sums of positive terms (no
  // cancellation), left unrenormalised like products
  // (C_k = 13/3 D_k, so C_k D_k >= 0: every sum here is of non-negative terms)
  const ff is1 = ff_fma_acc<true>(C1, D1, ff_sqr_add_acc(e1, eps4));
  const ff is2 = ff_fma_acc<true>(C2, D2, ff_sqr_add_acc(e2, eps4));
  const ff is3 = ff_fma_acc<true>(C3, D3, ff_sqr_add_acc(e3, eps4));
  const ff a1 = ff_sqr(is1), a2 = ff_sqr(is2), a3 = ff_sqr(is3);
  const ff p1 = a2 * a3, q2 = a1 * a3, q3 = a1 * a2;
  out.den = ff_fma_acc<true>(6.0f, q2, ff_fma_acc<true>(3.0f, q3, p1));
  out.num = ff_fma(q2, g2s, ff_fma_acc(q3, g3s, p1 * g1));
}

// Both reconstructions of one characteristic field (the binary64 weno5_pair):
// with d_m = v_{m+1} - v_m and the arguments g1, 6 g2, 3 g3,
//   left:  D = d1-d0, d2-d1, d3-d2;  e = 3 d1 - d0, d1 + d2, d3 - 3 d2;
//          g1 = 5/6 d1 - 1/3 d0,  6 g2 = d1 + 2 d2,  3 g3 = 2 d2 - d3/2;
//   right: D = d4-d3, d3-d2, d2-d1;  e = d4 - 3 d3, d2 + d3, 3 d2 - d1;
//          g1 = 1/3 d4 - 5/6 d3,  6 g2 = -(d3 + 2 d2),  3 g3 = d1/2 - 2 d2.
__device__ __forceinline__ void weno5_pair_ff(const ff (&v)[6], WenoFF& L, WenoFF& Rt) {
  const ff d0 = v[1] - v[0], d1 = v[2] - v[1], d2 = v[3] - v[2], d3 = v[4] - v[3], d4 = v[5] - v[4];
  const ff D1 = d1 - d0, D2 = d2 - d1, D3 = d3 - d2, D4 = d4 - d3;
  constexpr ff c13 = ff_const(13.0 / 3.0);
  const ff C1 = c13 * D1, C2 = c13 * D2, C3 = c13 * D3, C4 = c13 * D4;
  constexpr ff k56 = ff_const(5.0 / 6.0), k13 = ff_const(1.0 / 3.0);
  const ff t2 = ff_scale(d2, 2.0f);
  weno5_side_ff(D1, C1, D2, C2, D3, C3, ff_fma(3.0f, d1, -d0), d1 + d2, ff_fma(-3.0f, d2, d3),
                ff_fma(k56, d1, -(k13 * d0)), t2 + d1, t2 - ff_scale(d3, 0.5f), L);
  weno5_side_ff(D4, C4, D3, C3, D2, C2, ff_fma(-3.0f, d3, d4), d2 + d3, ff_fma(3.0f, d2, -d1),
                ff_fma(-k56, d3, k13 * d4), -(t2 + d3), ff_scale(d1, 0.5f) - t2, Rt);
}

// Per-thread float-float slots in shared memory: slot k of thread tid is the
// 8-byte word {hi, lo} k T + tid of a thread-minor float2 array, so a slot is
// one 64-bit access and a warp's accesses to one slot are 32 consecutive words
// (no bank conflicts).  A thread touches only its own slots, so no barrier is
// needed.
struct Slots {
  float2* base;
  int T, tid;
  __device__ __forceinline__ void put(int k, ff v) const { base[k * T + tid] = make_float2(v.hi, v.lo); }
  __device__ __forceinline__ ff get(int k) const {
    const float2 w = base[k * T + tid];
    return ff{w.x, w.y};
  }
};
constexpr int kFaceSlots = NEQ * 6;  // the characteristic fields of the six stencil cells

// The face flux (binary64 face_core's steps; the stored flux is twice the
// reference's, the halves folded into the update's 0.5/h).  A face is about
// 6,000 binary32 instructions; written out in full for the six stencil cells
// and five fields it overflows the instruction cache, so the projections (per
// cell) and the reconstructions (per field) run as loops over the thread's
// shared-memory slots, one copy of each body.  U: the stage input's float-float
// copy, c the face's cell (the face between c - st and c).
template <int D>
__device__ __forceinline__ void face_ff(const SolveDev& s, const float2* __restrict__ U, long long c,
                                        long long st, const Slots& sl, ff (&out)[NEQ]) {
  constexpr int T1 = (D + 1) % 3;
  constexpr int T2 = (D + 2) % 3;
  const long long V = s.V, n5 = NEQ * V;
  const ff gam1 = cst(s.ff_gam1), gamma = cst(s.ff_gamma), hgam1 = cst(s.ff_hgam1);

  // Roe average: f_R + wL (f_L - f_R), wL = sqrt(rho_L) / (sqrt(rho_L) + sqrt(rho_R)).
  ff Uv[3], HH;
  {
    const SideFF Ls = side_ff(s, c - st), Rs = side_ff(s, c);
    const ff wL = Ls.sr * ff_rcp(Ls.sr + Rs.sr);
    Uv[0] = ff_fma(wL, Ls.u - Rs.u, Rs.u);
    Uv[1] = ff_fma(wL, Ls.v - Rs.v, Rs.v);
    Uv[2] = ff_fma(wL, Ls.w - Rs.w, Rs.w);
    HH = ff_fma(wL, Ls.h - Rs.h, Rs.h);
  }
  const ff q2 = ff_sqr_add_acc(Uv[2], ff_sqr_add_acc(Uv[1], ff_sqr(Uv[0])));  // no cancellation
  const ff hq2 = ff_scale(q2, 0.5f);
  const ff c2 = gam1 * (HH - hq2);
  const ff ic = ff_rsqrt(c2);  // 1/c
  const ff cc = c2 * ic;
  const ff K = (hgam1 * ic) * ic;
  const ff hic = ff_scale(ic, 0.5f);
  const ff un = Uv[D], u1 = Uv[T1], u2 = Uv[T2];

  // Characteristic projections of the six stencil cells c-3 .. c+2 into slots
  // 6 n + m; the next cell's state is loaded while this one is projected.
  ff f[NEQ];
#pragma unroll
  for (int n = 0; n < NEQ; ++n) f[n] = ld(s, U, n5, n * V + c - 3 * st);
#pragma unroll 1
  for (int m = 0; m < 6; ++m) {
    ff g5[NEQ];
    const long long o = c + (m - 2) * st;  // the next cell (not loaded after the last)
#pragma unroll
    for (int n = 0; n < NEQ; ++n) g5[n] = m < 5 ? ld(s, U, n5, n * V + o) : f[n];
    const ff f0 = f[0], f4 = f[4];
    const ff fm[3] = {f[1], f[2], f[3]};
    const ff t =
        ff_fma(-Uv[2], fm[2], ff_fma_acc(-Uv[1], fm[1], ff_fma_acc(-Uv[0], fm[0], ff_fma_acc(hq2, f0, f4))));
    const ff A = K * t;
    const ff g = ff_fma(un, f0, -fm[D]);
    // the characteristic values enter the reconstructions only through
    // differences and as addends: stored unrenormalised
    sl.put(m, ff_fma_acc(hic, g, A));
    sl.put(6 + m, ff_add_acc(f0, ff_scale(A, -2.0f)));
    sl.put(12 + m, ff_fma_acc(-hic, g, A));
    sl.put(18 + m, ff_fma_acc(-u1, f0, fm[T1]));
    sl.put(24 + m, ff_fma_acc(-u2, f0, fm[T2]));
#pragma unroll
    for (int n = 0; n < NEQ; ++n) f[n] = g5[n];
  }

  // Left- and right-biased reconstructions of each field, r = base + num / den,
  // into the field's slots 6 n (left) and 6 n + 1 (right).
#pragma unroll 1
  for (int n = 0; n < NEQ; ++n) {
    ff v[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) v[m] = sl.get(6 * n + m);
    WenoFF a, b;
    weno5_pair_ff(v, a, b);
    sl.put(6 * n, ff_fma(a.num, ff_rcp(a.den), v[2]));
    sl.put(6 * n + 1, ff_fma(b.num, ff_rcp(b.den), v[3]));
  }
  ff rl[NEQ], rr[NEQ];
#pragma unroll
  for (int n = 0; n < NEQ; ++n) {
    rl[n] = sl.get(6 * n);
    rr[n] = sl.get(6 * n + 1);
  }

  // Back to conserved variables.
  const ff uncc = un * cc;
  ff rhoL, mL[3], EL, rhoR, mR[3], ER;
  {
    const ff sp = rl[0] + rl[2], dm = rl[2] - rl[0];
    rhoL = sp + rl[1];
    mL[D] = ff_fma(un, rhoL, cc * dm);
    mL[T1] = ff_fma(u1, rhoL, rl[3]);
    mL[T2] = ff_fma(u2, rhoL, rl[4]);
    EL = ff_fma_acc(HH, sp, ff_fma_acc(uncc, dm, ff_fma_acc(hq2, rl[1], ff_fma_acc(u1, rl[3], u2 * rl[4]))));
  }
  {
    const ff sp = rr[0] + rr[2], dm = rr[2] - rr[0];
    rhoR = sp + rr[1];
    mR[D] = ff_fma(un, rhoR, cc * dm);
    mR[T1] = ff_fma(u1, rhoR, rr[3]);
    mR[T2] = ff_fma(u2, rhoR, rr[4]);
    ER = ff_fma_acc(HH, sp, ff_fma_acc(uncc, dm, ff_fma_acc(hq2, rr[1], ff_fma_acc(u1, rr[3], u2 * rr[4]))));
  }

  // Local Lax-Friedrichs flux.  The reconstructed states are perturbations
  // (rho', m, E') of the reference state (the inputs are, and the projections and
  // WENO5 are linear and reproduce constants); rho = rho_ref + rho' for the
  // velocities and the sound speed, and p' = p - p_ref = (gamma - 1)(E' - rho q^2
  // / 2).  The momentum flux carries p' instead of p: the constant p_ref cancels
  // in every flux difference.  Both 1/rho from one reciprocal.
  const ff rref = cst(s.ff_rho_ref), pref = cst(s.ff_p_ref);
  const ff rhoLf = rhoL + rref, rhoRf = rhoR + rref;
  const ff ip = ff_rcp(rhoLf * rhoRf);
  const ff iL = ip * rhoRf, iR = ip * rhoLf;
  ff vL[3], vR[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    vL[a] = mL[a] * iL;
    vR[a] = mR[a] * iR;
  }
  const ff kL = ff_fma_acc(mL[2], vL[2], ff_fma_acc(mL[1], vL[1], mL[0] * vL[0]));
  const ff kR = ff_fma_acc(mR[2], vR[2], ff_fma_acc(mR[1], vR[1], mR[0] * vR[0]));
  const ff pL = gam1 * (EL - ff_scale(kL, 0.5f));  // p - p_ref
  const ff pR = gam1 * (ER - ff_scale(kR, 0.5f));
  const ff c2L = (gamma * iL) * (pL + pref), c2R = (gamma * iR) * (pR + pref);
  const ff cL = c2L * ff_rsqrt(c2L), cR = c2R * ff_rsqrt(c2R);
  const ff alpha = ff_max(ff_abs(vR[D]) + cR, ff_abs(vL[D]) + cL);
  const ff fL = mL[D], fR = mR[D];
  // the fluxes are stored unrenormalised: the update only differences them
  out[0] = ff_fma_acc(-alpha, rhoR - rhoL, ff_add_acc(fL, fR));
  const ff pLR = ff_add_acc(pL, pR);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const ff fLa = (a == D) ? ff_fma_acc(fL, vL[a], pLR) : fL * vL[a];
    out[1 + a] = ff_fma_acc(-alpha, mR[a] - mL[a], ff_fma_acc(fR, vR[a], fLa));
  }
  // q_n (E + p) with E + p = (E' + p') + (E_ref + p_ref)
  const ff epref = cst(s.ff_Ep_ref);
  out[4] = ff_fma_acc(-alpha, ER - EL,
                      ff_fma_acc(vR[D], (ER + pR) + epref, vL[D] * ((EL + pL) + epref)));
}

// One face per thread over the interior tiles (the binary64 k_inviscid's walk).
// The stage input is Q's float-float copy in stage 1 and Q_p's in stages 2-3.
// Dynamic shared memory: kFaceSlots float-float slots per thread.  Register cap
// 80 (no spills): six 128-thread CTAs per SM, where 128 registers fit four;
// measured 0.5-3% faster, the results bitwise the same.
template <int D>
__global__ void __maxnreg__(80) k_inviscid_ff(const SolveDev* __restrict__ solves,
                                               const TileRef* __restrict__ tiles, int ntiles, int stage) {
  extern __shared__ float2 face_slots[];
  const Slots sl{face_slots, (int)blockDim.x, (int)threadIdx.x};
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const TileCell tc = tile_cell(tiles[t], 0);
    const SolveDev& s = solves[tc.s];
    if (!s.ctl->active) continue;
    if (tc.i >= s.IM || tc.j >= s.JM) continue;
    const float2* U = stage == 1 ? s.QF : s.QpF;
    const long long st = D == 0 ? 1ll : (D == 1 ? (long long)s.nx : (long long)s.nx * s.ny);
    ff f[NEQ];
    face_ff<D>(s, U, pad_off(s, tc.i, tc.j, tc.k), st, sl, f);
    const long long fo = int_off(s, tc.i, tc.j, tc.k);
    float4* F = s.FFa[D];
    const long long n3 = 3 * s.IV;
    at(s, F, n3, 3 * fo) = make_float4(f[0].hi, f[0].lo, f[1].hi, f[1].lo);
    at(s, F, n3, 3 * fo + 1) = make_float4(f[2].hi, f[2].lo, f[3].hi, f[3].lo);
    at(s, F, n3, 3 * fo + 2) = make_float4(f[4].hi, f[4].lo, 0.0f, 0.0f);
  }
}

// ---------------------------------------------------------------------------
// Viscous terms on the NGV ring (the binary64 k_viscous in float-float: the
// 4th-order gradients of u, v, w, T, Sutherland mu, the six stresses and three
// energy fluxes; src/calc_gradient.cpp:17-66, src/Block3d.cpp:750-868).  The
// terms are float-float, grouped by differencing direction (SolveDev::TvG); mu
// (interior, lagged into the time step) is stored in binary64.  Plane tiles over
// the ring, as the binary64 kernel.

__device__ __forceinline__ ff d4_ff(const SolveDev& s, const float2* f, long long n, long long o, long long st,
                                    ff c12, ff c23) {
  // ((f[-2] - f[+2]) c12 + (f[+1] - f[-1]) c23), the 1/h folded into the weights;
  // unrenormalised: the gradients enter the stresses through sums, and the
  // energy fluxes as multiplicands with a low part within a few ulps
  return ff_fma_acc(ld(s, f, n, o - 2 * st) - ld(s, f, n, o + 2 * st), c12,
                    (ld(s, f, n, o + st) - ld(s, f, n, o - st)) * c23);
}

__global__ void __launch_bounds__(256) k_viscous_ff(const SolveDev* __restrict__ solves,
                                                    const TileRef* __restrict__ tiles, int ntiles) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const TileRef tr = tiles[t];
    const SolveDev& s = solves[tr.solve];
    if (!s.ctl->active) continue;
    const long long p = plane_tile_first(tr, (int)blockDim.x) + threadIdx.x;
    if (p >= (long long)s.rx * s.ry) continue;
    const int jr = (int)(p / s.rx);
    const int i = (int)(p - (long long)jr * s.rx) - NGV, j = jr - NGV, k = (int)tr.tk - NGV;
    const long long V = s.V;
    const long long o = pad_off(s, i, j, k);
    const long long sy = s.nx, sz = (long long)s.nx * s.ny;
    const float2* P = s.PF;
    const float2 *Pu = P + 2 * V, *Pv = P + 3 * V, *Pw = P + 4 * V, *PT = P + 5 * V;
    const long long nb = V;  // each block's extent (the checked build's bound)
    const ff ax = cst(s.ff_c12[0]), bx = cst(s.ff_c23[0]), ay = cst(s.ff_c12[1]), by = cst(s.ff_c23[1]),
             az = cst(s.ff_c12[2]), bz = cst(s.ff_c23[2]);
    const ff ux = d4_ff(s, Pu, nb, o, 1, ax, bx), uy = d4_ff(s, Pu, nb, o, sy, ay, by),
             uz = d4_ff(s, Pu, nb, o, sz, az, bz);
    const ff vx = d4_ff(s, Pv, nb, o, 1, ax, bx), vy = d4_ff(s, Pv, nb, o, sy, ay, by),
             vz = d4_ff(s, Pv, nb, o, sz, az, bz);
    const ff wx = d4_ff(s, Pw, nb, o, 1, ax, bx), wy = d4_ff(s, Pw, nb, o, sy, ay, by),
             wz = d4_ff(s, Pw, nb, o, sz, az, bz);
    const ff Tx = d4_ff(s, PT, nb, o, 1, ax, bx), Ty = d4_ff(s, PT, nb, o, sy, ay, by),
             Tz = d4_ff(s, PT, nb, o, sz, az, bz);
    const ff uu = ld(s, Pu, nb, o), vv = ld(s, Pv, nb, o), ww = ld(s, Pw, nb, o), Tl = ld(s, PT, nb, o);
    // Sutherland's law as (1 + C) T^2 / sqrt(T (T + C)^2).
    const ff TC = Tl + cst(s.ff_C);
    const ff mu = (cst(s.ff_C1) * ff_sqr(Tl)) * ff_rsqrt(Tl * ff_sqr(TC));
    if (i >= 0 && i < s.IM && j >= 0 && j < s.JM && k >= 0 && k < s.KM) at(s, s.pd.mu, V, o) = ff_to_double(mu);
    const ff mr = mu * cst(s.ff_Re_inv);
    const ff m23 = ff_const(2.0 / 3.0) * mr;
    const ff txx = m23 * ((ff_scale(ux, 2.0f) - vy) - wz);
    const ff tyy = m23 * ((ff_scale(vy, 2.0f) - ux) - wz);
    const ff tzz = m23 * ((ff_scale(wz, 2.0f) - ux) - vy);
    const ff txy = mr * (uy + vx);
    const ff txz = mr * (uz + wx);
    const ff tyz = mr * (vz + wy);
    const ff mk = mr * cst(s.ff_kappa);
    const ff ex = ff_fma_acc(ww, txz, ff_fma_acc(vv, txy, uu * txx)) - mk * Tx;
    const ff ey = ff_fma_acc(ww, tyz, ff_fma_acc(vv, tyy, uu * txy)) - mk * Ty;
    const ff ez = ff_fma_acc(ww, tzz, ff_fma_acc(vv, tyz, uu * txz)) - mk * Tz;
    // grouped by differencing direction: the four terms of equations 1..4
    // differenced along d, two float4 per direction and ring point
    const long long r = ring_off(s, i, j, k), RV = s.RV, n6 = 6 * RV;
    const ff terms[kViscTerms] = {txx, tyy, tzz, txy, txz, tyz, ex, ey, ez};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const ff a = terms[visc_term(1, d)], b = terms[visc_term(2, d)], c = terms[visc_term(3, d)],
               e = terms[visc_term(4, d)];
      at(s, s.TvG, n6, 2 * (d * RV + r)) = make_float4(a.hi, a.lo, b.hi, b.lo);
      at(s, s.TvG, n6, 2 * (d * RV + r) + 1) = make_float4(c.hi, c.lo, e.hi, e.lo);
    }
  }
}

}  // namespace

// The three face launches of a stage (grid g, nt threads: the binary64 tiles).
void launch_faces_ff(const SolveDev* d, const TileRef* tiles, int ntiles, int stage, int g, int nt,
                     cudaStream_t st, Profiler* pf) {
  // shared memory for kFaceSlots float-float slots per thread, up to 256 threads
  // (above the 48 KB default): the kernels' attribute, set once per device
  constexpr int kMaxBytes = 256 * kFaceSlots * (int)sizeof(float2);
  constexpr int kMaxDevices = 64;
  static std::mutex mu;
  static bool opted[kMaxDevices] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < kMaxDevices) {
    std::lock_guard<std::mutex> lock(mu);
    if (!opted[dev]) {
      // and the largest shared-memory carveout, so that the slots of as many
      // CTAs as the registers allow fit on an SM
      for (const void* k : {(const void*)k_inviscid_ff<0>, (const void*)k_inviscid_ff<1>,
                             (const void*)k_inviscid_ff<2>}) {
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxBytes);
        cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
      }
      opted[dev] = true;
    }
  }
  const size_t smem = (size_t)nt * kFaceSlots * sizeof(float2);
  auto run = [&](int id, auto kern) {
    if (pf) pf->before(id, st);
    kern<<<g, nt, smem, st>>>(d, tiles, ntiles, stage);
    if (pf) pf->after(st);
  };
  run(KID_INVISCID_X, k_inviscid_ff<0>);
  run(KID_INVISCID_Y, k_inviscid_ff<1>);
  run(KID_INVISCID_Z, k_inviscid_ff<2>);
}

// The viscous launch of a stage over the ring's plane tiles (grid g, nt threads).
void launch_viscous_ff(const SolveDev* d, const TileRef* ring, int nring, int g, int nt, cudaStream_t st,
                       Profiler* pf) {
  if (pf) pf->before(KID_VISCOUS, st);
  k_viscous_ff<<<g, nt, 0, st>>>(d, ring, nring);
  if (pf) pf->after(st);
}

}  // namespace cbns
