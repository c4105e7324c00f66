// cbns_device.cuh — device-side data model of the GB300 right-hand-side library.
//
// A "solve" is one periodic block (the reference's Block3d).  Its arrays live in
// HBM as structure-of-arrays, padded by NG = 4 ghost layers on every side like
// the reference's (include/Block3d.h:169-199), so stencils need no wrap logic:
//
//   padded cell (i,j,k), i in [-NG, IM+NG):  off = (i+NG) + nx*((j+NG) + ny*(k+NG))
//   Q[n*V + off], n = 0..4 (rho, rho*u, rho*v, rho*w, E);  V = nx*ny*nz
//
// Face fluxes are stored per direction at the cell on the face's high side (face
// i-1/2 at cell i), over the interior only: the periodic face IM-1/2... +1/2 is
// face -1/2 (same stencil values), so F[IM] reads F[0].
//
// Work is cut into tiles of TILE_X x TILE_Y x 1 cells; a batch of solves is one
// flattened table of tiles, so a single launch covers every solve of a batch.
#pragma once

#include <cstdint>

#include <vector_types.h>

namespace cbns {

constexpr int NEQ = 5;
constexpr int NG = 4;
constexpr int NGV = 2;
// Viscous terms kept on the NGV ring: six stresses and three energy fluxes.
constexpr int kViscTerms = 9;
enum ViscTerm { TXX = 0, TYY, TZZ, TXY, TXZ, TYZ, EX, EY, EZ };
// The term differenced along direction d in the equation of momentum component
// n - 1 (n = 1..3) or energy (n = 4): the components of Ev, Fv, Gv
// (src/Block3d.cpp:812-868).
__host__ __device__ constexpr int visc_term(int n, int d) {
  return n == 1 ? (d == 0 ? TXX : d == 1 ? TXY : TXZ)
       : n == 2 ? (d == 0 ? TXY : d == 1 ? TYY : TYZ)
       : n == 3 ? (d == 0 ? TXZ : d == 1 ? TYZ : TZZ)
                : (d == 0 ? EX : d == 1 ? EY : EZ);
}
constexpr int TILE_X = 32;
constexpr int TILE_Y = 4;
constexpr int TILE_THREADS = TILE_X * TILE_Y;

// Per-solve time control, kept on the device so a replayed step graph needs no
// host round trip (the loop of src/cbns3d.cpp:176-198).
struct SolveCtl {
  double t_cur;
  double t_end;
  double dt;
  unsigned long long smax_bits;  // running max of calc_dt's wave-speed sum (bits of a double >= 0)
  int active;                    // 0 once is_finished held: later kernels of the step do nothing
  int status;                    // CBNS_ERR_NONPHYSICAL bit pattern once a stage met a bad state
  unsigned int steps;            // steps taken since upload
  int pad;
  float cdt[2];                  // binary32 dt/4 and 2 dt/3: FP32-mixed stages 2 and 3
  float pad2[2];
};

// Cell-centred binary64 primitive fields of a stage input, one array each.  The
// arrays are consecutive blocks of V values of one allocation, in member order
// (the update kernel's stores address them from the first).
template <typename R>
struct PrimSet {
  R* rho;
  R* u;
  R* v;
  R* w;
  R* p;
  R* T;
  R* srho;  // sqrt(rho): Roe weights
  R* H;     // total enthalpy
  R* mu;    // Sutherland viscosity, interior; lagged into calc_dt like the reference
};

// Per-solve constants in the precision a kernel computes in, derived once on the
// host so no thread converts or re-derives them.
template <typename R>
struct Consts {
  R gamma, gam1, gam1_inv, gM2, Re_inv, kappa, C_T_inf, C_dt_v;
  R hgam1;  // (gamma - 1) / 2
  R inv_dx, inv_dy, inv_dz;
  R hfx, hfy, hfz;  // 0.5 / h: the inviscid face fluxes are stored doubled
  R sum_ih, sum_ih2;  // 1/hx + 1/hy + 1/hz and 1/hx^2 + 1/hy^2 + 1/hz^2 (time step)
  R C_dt_v2;          // 2 C_dt_v
  // 4th-order central difference weights with 1/h folded in:
  // d/dx f = (f[-2] - f[+2]) * c12x + (f[+1] - f[-1]) * c23x
  R c12x, c23x, c12y, c23y, c12z, c23z;
  R rho_ref, p_ref, E_ref, T_ref;
  R gamma_gam1_inv;  // gamma / (gamma - 1)
  R pref_over_rref;  // p_ref / rho_ref
  R low_rho;         // below this density the Roe weights' sqrt is taken in binary64
};

struct SolveDev {
  int IM, JM, KM;      // interior extents
  int nx, ny, nz;      // padded extents (IM + 2*NG ...)
  long long V;         // padded volume
  int rx, ry, rz;      // NGV-ring extents (IM + 2*NGV ...)
  long long RV;        // ring volume
  long long IV;        // interior volume
  int mixed;           // 0: binary64 throughout; 1: FP32-mixed
  // conserved state (SoA, padded), binary64 in both modes
  double* Q;
  double* Qp;
  // binary64 primitives (binary64 mode; in FP32-mixed mode filled on demand for output)
  PrimSet<double> pd;
  // binary64 mode: face fluxes (interior, 5 components) and the viscous terms on
  // the NGV ring: 9 blocks of RV values, the stresses txx, tyy, tzz, txy, txz,
  // tyz and the energy fluxes ex, ey, ez -- the 9 distinct components of
  // Ev = (txx, txy, txz, ex), Fv = (txy, tyy, tyz, ey), Gv = (txz, tyz, tzz, ez)
  double* F[3];
  double* Tv;
  // FP32-mixed mode: the stage input as a binary32 perturbation of the reference
  // state (rho - rho_ref, rho*u, rho*v, rho*w, E - E_ref), its primitives, and
  // binary32 face fluxes and viscous terms.  The viscous terms are grouped by the
  // direction d they are differenced along: block d (RV float4 values) holds at
  // each ring point the terms of the x-, y-, z-momentum and energy equations,
  // (visc_term(1,d), visc_term(2,d), visc_term(3,d), visc_term(4,d)), so the
  // update reads a direction's four terms with one 16-byte load per offset.
  //
  // The binary32 state and primitives are packed per cell, so a stencil point
  // costs one or two 16-byte loads instead of a load per field.  rho, u, v, w,
  // sqrt(rho), H and mu are absolute; p and T are perturbations p - p_ref and
  // T - T_ref (binary32 keeps 24 bits of the O(0.1) fluctuations instead of the
  // O(70) mean pressure).
  float4* U4;   // (rho - rho_ref, rho*u, rho*v, rho*w), padded
  float* UE;    // E - E_ref, padded
  float4* PA;   // (u, v, w, T - T_ref), padded
  float4* PB;   // (rho, p - p_ref, sqrt(rho), H), padded
  float* muf;   // Sutherland mu, interior; lagged into calc_dt like the reference
  // per direction, the face fluxes: IV float4 of equations 0-3, then IV floats
  // of equation 4 (5 IV floats in all)
  float* Ff[3];
  float4* Tvg;
  // reference state of the perturbation form (u_ref = 0, E_ref = p_ref/(gamma-1))
  double rho_ref, p_ref, E_ref, T_ref;
  // parameters (src/read_input.cpp:78-90)
  double gamma, gam1, gam1_inv, gM2, Re_inv, kappa, C_T_inf, CFL, C_dt_v;
  double dx, dy, dz, inv_dx, inv_dy, inv_dz;
  Consts<double> cd;
  Consts<float> cf;
  SolveCtl* ctl;
  double C_T_inf1;  // 1 + C_T_inf, Sutherland's law (binary64 viscous terms)
  // CBNS_FP64_FF solves: the binary64 state, RK3 and primitives, with the face
  // fluxes, the viscous terms and the flux differences in float-float
  // arithmetic.  Its inputs as float-float pairs {hi, lo}, written with the
  // binary64 state by the update and start-up kernels: the state Q and Q_p (5
  // blocks of V each) and the primitives sqrt(rho), H, u, v, w, T (kFFPrims
  // blocks of V).  The face fluxes and viscous terms are float-float pairs in
  // the bytes of F[d] and Tv (8 bytes a value in both forms).  Float-float
  // constants: gamma - 1, gamma, (gamma - 1)/2; 0.5/h, the 4th-order weights
  // c12 and c23 per direction; 1/Re, kappa, C and 1 + C of Sutherland's law.
  // Null / unused otherwise.
  int ffaces;
  float2* QF;
  float2* QpF;
  float2* PF;
  float2 ff_gam1, ff_gamma, ff_hgam1;
  float2 ff_hf[3], ff_c12[3], ff_c23[3];
  float2 ff_Re_inv, ff_kappa, ff_C, ff_C1;
  // the primitives and time step of CBNS_FP64_FF: gamma M^2, 1/(gamma M^2),
  // gamma/(gamma - 1), 2 C_dt_v, sum 1/h, sum 1/h^2
  float2 ff_gM2, ff_igM2, ff_ggam1, ff_Cdt2, ff_sum_ih, ff_sum_ih2;
  // CBNS_FP64_FF face fluxes and viscous terms, packed so the update reads them
  // with 16-byte loads (F and Tv are unused in this mode):
  //   FFa[d]: per interior cell, the five float-float fluxes of its face normal
  //   to d as three float4 {f0, f1}, {f2, f3}, {f4, 0};
  //   TvG: per direction d and ring point, the four terms differenced along d
  //   (visc_term(1..4, d)) as two float4 {t1, t2}, {t3, t4}: element
  //   (d RV + r) 2 + h.
  float4* FFa[3];
  float4* TvG;
  // CBNS_FP64_FF state copies are perturbations of the reference state: QF and
  // QpF hold (rho - rho_ref, rho u, rho v, rho w, E - E_ref), the differences
  // taken in binary64 before the split, so float-float's 47 bits are spent on
  // the fluctuations rather than on E_ref ~ 1/(gamma (gamma-1) M^2).  The
  // constants rho_ref, p_ref and E_ref + p_ref in float-float:
  float2 ff_rho_ref, ff_p_ref, ff_Ep_ref;
};

// Blocks of SolveDev::PF: sqrt(rho), H, u, v, w, T.
constexpr int kFFPrims = 6;

template <typename R>
__host__ __device__ inline const Consts<R>& consts_of(const SolveDev& s);
template <>
__host__ __device__ inline const Consts<double>& consts_of<double>(const SolveDev& s) {
  return s.cd;
}
template <>
__host__ __device__ inline const Consts<float>& consts_of<float>(const SolveDev& s) {
  return s.cf;
}

// Bits of SolveCtl::status.
constexpr int kStatusNonphysical = 1;  // a stage produced rho <= 0, p <= 0 or a NaN
constexpr int kStatusBounds = 2;       // bounds-checked build: an index left its array

// Element i of an array of n elements that belongs to solve s.  Every global
// access of the stage kernels goes through here.  Built with CBNS_BOUNDS_CHECK,
// an index outside [0, n) sets the solve's kStatusBounds bit and the access goes
// to element 0 instead: no access outside the array is made and nothing traps,
// so the host reads the bit after the launch.  Otherwise it is plain indexing.
template <class T>
__device__ __forceinline__ T& at(const SolveDev& s, T* base, long long n, long long i) {
#ifdef CBNS_BOUNDS_CHECK
  if (i < 0 || i >= n) {
    atomicOr(&s.ctl->status, kStatusBounds);
    i = 0;
  }
#endif
  return base[i];
}

// Reciprocal of a positive, normal binary64 value (the face kernel's three
// divisions: the Roe weight, the shared WENO normalisation, the two 1/rho of
// the Lax-Friedrichs flux).  From the hardware's reciprocal estimate y (PTX
// rcp.approx.ftz.f64, which reads the operand's upper 32 bits and returns about
// 20 good bits) one third-order step of the series 1/x = y / (1 - e) =
// y (1 + e + e^2 + O(e^3)), e = 1 - x y: the estimate's relative error cubed,
// far below an ulp, so the result is within one ulp of 1/x.  A division a/x in
// IEEE binary64 costs about 9 FP64 issue slots and 1/x about 6 (measured); this
// is one estimate and three fused multiply-adds.
__device__ __forceinline__ double rcp64(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double e = fma(-x, y, 1.0);
  return fma(y, fma(e, e, e), y);
}

// Fill cd and cf from the binary64 parameters (host side, once per solve).
inline void fill_consts(SolveDev& s) {
  Consts<double>& c = s.cd;
  c.gamma = s.gamma;
  c.gam1 = s.gam1;
  c.gam1_inv = s.gam1_inv;
  c.hgam1 = 0.5 * s.gam1;
  c.gM2 = s.gM2;
  c.Re_inv = s.Re_inv;
  c.kappa = s.kappa;
  c.C_T_inf = s.C_T_inf;
  c.C_dt_v = s.C_dt_v;
  c.inv_dx = s.inv_dx;
  c.inv_dy = s.inv_dy;
  c.inv_dz = s.inv_dz;
  c.hfx = 0.5 * s.inv_dx;
  c.hfy = 0.5 * s.inv_dy;
  c.hfz = 0.5 * s.inv_dz;
  c.sum_ih = s.inv_dx + s.inv_dy + s.inv_dz;
  c.sum_ih2 = s.inv_dx * s.inv_dx + s.inv_dy * s.inv_dy + s.inv_dz * s.inv_dz;
  c.C_dt_v2 = 2.0 * s.C_dt_v;
  c.c12x = (1.0 / 12.0) * s.inv_dx;
  c.c23x = (2.0 / 3.0) * s.inv_dx;
  c.c12y = (1.0 / 12.0) * s.inv_dy;
  c.c23y = (2.0 / 3.0) * s.inv_dy;
  c.c12z = (1.0 / 12.0) * s.inv_dz;
  c.c23z = (2.0 / 3.0) * s.inv_dz;
  c.rho_ref = s.rho_ref;
  c.p_ref = s.p_ref;
  c.E_ref = s.E_ref;
  c.T_ref = s.T_ref;
  c.gamma_gam1_inv = s.gamma * s.gam1_inv;
  c.pref_over_rref = s.p_ref / s.rho_ref;
  c.low_rho = 0.01 * s.rho_ref;
  Consts<float>& f = s.cf;
  f.gamma = (float)c.gamma;
  f.gam1 = (float)c.gam1;
  f.gam1_inv = (float)c.gam1_inv;
  f.hgam1 = (float)c.hgam1;
  f.gM2 = (float)c.gM2;
  f.Re_inv = (float)c.Re_inv;
  f.kappa = (float)c.kappa;
  f.C_T_inf = (float)c.C_T_inf;
  f.C_dt_v = (float)c.C_dt_v;
  f.inv_dx = (float)c.inv_dx;
  f.inv_dy = (float)c.inv_dy;
  f.inv_dz = (float)c.inv_dz;
  f.hfx = (float)c.hfx;
  f.hfy = (float)c.hfy;
  f.hfz = (float)c.hfz;
  f.sum_ih = (float)c.sum_ih;
  f.sum_ih2 = (float)c.sum_ih2;
  f.C_dt_v2 = (float)c.C_dt_v2;
  f.c12x = (float)c.c12x;
  f.c23x = (float)c.c23x;
  f.c12y = (float)c.c12y;
  f.c23y = (float)c.c23y;
  f.c12z = (float)c.c12z;
  f.c23z = (float)c.c23z;
  f.rho_ref = (float)c.rho_ref;
  f.p_ref = (float)c.p_ref;
  f.E_ref = (float)c.E_ref;
  f.T_ref = (float)c.T_ref;
  f.gamma_gam1_inv = (float)c.gamma_gam1_inv;
  f.pref_over_rref = (float)c.pref_over_rref;
  f.low_rho = (float)c.low_rho;
}

struct TileRef {
  uint16_t solve;
  uint16_t ti;
  uint16_t tj;
  uint16_t tk;
};

// A plane tile: blockDim.x consecutive points of one k-plane of a box of
// extents ex x ey, numbered p = i + ex j (so every warp is full whatever ex is);
// the tile number within the plane is ti + 65536 tj, the plane tk.
__host__ __device__ inline long long plane_tile_first(const TileRef& t, int threads) {
  return ((long long)t.ti + 65536ll * t.tj) * threads;
}

// ---------------------------------------------------------------------------
// Tile walk.  Every kernel loops over its tile table with a grid stride, so it
// runs either one tile per CTA or persistently with fewer CTAs than tiles.

struct TileCell {
  int s;  // solve index
  int i, j, k;
};

// A tile is TILE_X cells along i by blockDim.x/32 rows along j (one CTA).  The
// row count is a launch-time choice (the batch autotuner picks 2, 4 or 8), not a
// template parameter, so every launch shape runs the same compiled kernel and
// therefore the same arithmetic: results do not depend on the launch shape.
constexpr int kMaxThreads = 256;

__device__ __forceinline__ TileCell tile_cell(const TileRef& t, int origin) {
  TileCell c;
  c.s = t.solve;
  c.i = origin + t.ti * TILE_X + (int)(threadIdx.x % TILE_X);
  c.j = origin + t.tj * (int)(blockDim.x / TILE_X) + (int)(threadIdx.x / TILE_X);
  c.k = origin + t.tk;
  return c;
}

__host__ __device__ inline long long pad_off(const SolveDev& s, int i, int j, int k) {
  return (long long)(i + NG) + (long long)s.nx * ((long long)(j + NG) + (long long)s.ny * (k + NG));
}
__host__ __device__ inline long long ring_off(const SolveDev& s, int i, int j, int k) {
  return (long long)(i + NGV) + (long long)s.rx * ((long long)(j + NGV) + (long long)s.ry * (k + NGV));
}
__host__ __device__ inline long long int_off(const SolveDev& s, int i, int j, int k) {
  return (long long)i + (long long)s.IM * ((long long)j + (long long)s.JM * k);
}

enum Domain { DOM_INTERIOR = 0, DOM_RING = 1, DOM_PADDED = 2 };

// The work tables of one stage: interior tiles (face and update kernels) and
// NGV-ring tiles (viscous terms).
struct StageTables {
  const TileRef* tiles;
  int ntiles;
  const TileRef* ring;
  int nring;
};

// Launch shape of the stage and dt kernels: tile rows (CTA = 32 x tile_rows
// threads) and, when > 0, a persistent grid of max_ctas CTAs walking the table.
struct LaunchCfg {
  int tile_rows = TILE_Y;
  int max_ctas = 0;
};

}  // namespace cbns
