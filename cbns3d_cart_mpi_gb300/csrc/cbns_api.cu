// cbns_api.cu — the C ABI of include/cbns_gpu.h over the kernels of cbns_kernels.cu.
//
// A handle owns one solve: a single device arena holding the padded state, the
// primitives, the face and viscous fluxes, the control block and the tile
// tables, plus a CUDA stream.  The host never sees device pointers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cbns_gpu.h"
#include "cbns_internal.h"
#include "cbns_modes.h"

namespace cbns {
cudaError_t launch_prepare(const SolveDev* d, const TileRef* tiles, int ntiles, cudaStream_t st, Profiler* pf);
cudaError_t launch_layout(const SolveDev* d, int sidx, const double* src, double* dst, bool to_soa,
                          long long V, cudaStream_t st, Profiler* pf);
cudaError_t launch_prims_double(const SolveDev* d, const TileRef* tiles, int ntiles, cudaStream_t st);
cudaError_t launch_init_tgv(const SolveDev* d, int sidx, const TileRef* tiles, int ntiles, double p_inf,
                            const PerturbMode* modes, int nmodes, cudaStream_t st);
cudaError_t launch_dt(const SolveDev* d, int nsolves, const TileRef* tiles, int ntiles, double t_end,
                      bool use_t_end, int precision, const LaunchCfg& cfg, cudaStream_t st, Profiler* pf);
cudaError_t launch_dt_raw(const SolveDev* d, int sidx, const TileRef* tiles, int ntiles, double* out,
                          int precision, const LaunchCfg& cfg, cudaStream_t st, Profiler* pf);
cudaError_t launch_set_dt(const SolveDev* d, int sidx, double dt, cudaStream_t st);
cudaError_t launch_reset_ctl(SolveCtl* ctl, double t, double t_end, cudaStream_t st);
cudaError_t launch_stage(const SolveDev* d, const StageTables& T, int stage, const LaunchCfg& cfg, int precision,
                         cudaStream_t st, Profiler* pf);
cudaError_t launch_diag(const SolveDev* d, int sidx, const TileRef* tiles, int ntiles, double* partials,
                        int nparts, double inv_n, double* out, cudaStream_t st, Profiler* pf);
}  // namespace cbns

using namespace cbns;

namespace {

thread_local std::string g_last_error;

cbns_status fail(cbns_status st, const std::string& msg) {
  g_last_error = msg;
  return st;
}

cbns_status cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return CBNS_ERR_OUT_OF_MEMORY;
  return CBNS_ERR_CUDA;
}

// The error a solve's device status word stands for (0: none).
cbns_status ctl_fail(int status, const char* fn) {
  if (status & kStatusBounds)
    return fail(CBNS_ERR_BOUNDS, std::string(fn) + ": a kernel index left its array (bounds-checked build)");
  return fail(CBNS_ERR_NONPHYSICAL, std::string(fn) + ": non-physical state (rho <= 0, p <= 0 or NaN)");
}

#define CBNS_CUDA(call)                                   \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
  } while (0)

// Tiles of TILE_X x rows x 1 cells over a box of extents ex, ey, ez.
void append_tiles(std::vector<TileRef>& out, int solve, int ex, int ey, int ez, int rows = TILE_Y) {
  const int tx = (ex + TILE_X - 1) / TILE_X, ty = (ey + rows - 1) / rows;
  for (int k = 0; k < ez; ++k)
    for (int j = 0; j < ty; ++j)
      for (int i = 0; i < tx; ++i)
        out.push_back(TileRef{(uint16_t)solve, (uint16_t)i, (uint16_t)j, (uint16_t)k});
}

size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

// Plane tiles of 32 x rows consecutive points of each k-plane of an ex x ey x ez
// box (the NGV ring of the viscous kernel): the tile number within the plane
// is split into the 16-bit ti (low) and tj (high) fields.
void append_plane_tiles(std::vector<TileRef>& out, int solve, int ex, int ey, int ez, int rows = TILE_Y) {
  const long long per = (long long)TILE_X * rows;
  const long long n = ((long long)ex * ey + per - 1) / per;
  for (int k = 0; k < ez; ++k)
    for (long long q = 0; q < n; ++q)
      out.push_back(TileRef{(uint16_t)solve, (uint16_t)(q & 0xffff), (uint16_t)(q >> 16), (uint16_t)k});
}

size_t plane_tile_count(long long ex, long long ey, long long ez, int rows = TILE_Y) {
  const long long per = (long long)TILE_X * rows;
  return (size_t)((ex * ey + per - 1) / per) * (size_t)ez;
}

// Tile coordinates are 16-bit (TileRef): the padded extent along k (one tile
// per plane) and the tile counts along i and j must stay below 65536.  With
// 2-row tiles (the smallest the batches use) this caps every extent at
// 65535 - 2 NG cells along k, and more along i and j; memory runs out far below.
constexpr uint32_t kMaxExtent = 65535 - 2 * NG;
bool block_extents_ok(uint32_t IM, uint32_t JM, uint32_t KM) {
  return IM <= kMaxExtent && JM <= kMaxExtent && KM <= kMaxExtent;
}

size_t tile_count(long long ex, long long ey, long long ez, int rows = TILE_Y) {
  return (size_t)((ex + TILE_X - 1) / TILE_X) * (size_t)((ey + rows - 1) / rows) * (size_t)ez;
}

// The viscous kernel's NGV ring: plane tiles for binary64, row tiles for the
// binary32 kernel (each walk measured the faster for its precision).
void append_ring_tiles(std::vector<TileRef>& out, int solve, int ex, int ey, int ez, bool mixed, int rows = TILE_Y) {
  if (mixed)
    append_tiles(out, solve, ex, ey, ez, rows);
  else
    append_plane_tiles(out, solve, ex, ey, ez, rows);
}

size_t ring_tile_count(long long ex, long long ey, long long ez, bool mixed) {
  return mixed ? tile_count(ex, ey, ez) : plane_tile_count(ex, ey, ez);
}

// Byte offsets of everything a solve's arena holds (see cbns_create).
struct ArenaLayout {
  size_t oQ, oQp, oStage, oPrim, oF[3], oTv, oFf[3], oTv32, oU32, oP32, oQF, oQpF, oPF, oFFa[3], oTvG, oCtl, oDesc,
      oTi, oTr, oTp, oPart, oOut, total;
};

ArenaLayout arena_layout(const SolveDev& s, int precision, size_t n_int, size_t n_ring, size_t n_pad, int nparts) {
  const bool mixed = precision == CBNS_FP32_MIXED;
  ArenaLayout L{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += align_up(bytes);
    return o;
  };
  const size_t dV = sizeof(double) * (size_t)s.V, fV = sizeof(float) * (size_t)s.V;
  L.oQ = take(NEQ * dV);
  L.oQp = take(NEQ * dV);
  L.oStage = take(NEQ * dV);
  L.oPrim = take(9 * dV);
  if (precision == CBNS_FP64_FF) {
    const size_t f2V = sizeof(float2) * (size_t)s.V;
    L.oQF = take(NEQ * f2V);
    L.oQpF = take(NEQ * f2V);
    L.oPF = take(kFFPrims * f2V);
    for (int d = 0; d < 3; ++d) L.oFFa[d] = take(sizeof(float4) * 3 * (size_t)s.IV);
    L.oTvG = take(sizeof(float4) * 6 * (size_t)s.RV);
  } else if (!mixed) {
    for (int d = 0; d < 3; ++d) L.oF[d] = take(sizeof(double) * NEQ * (size_t)s.IV);
    L.oTv = take(sizeof(double) * kViscTerms * (size_t)s.RV);
  } else {
    L.oU32 = take(NEQ * fV);  // U4 (4 values per cell), then UE
    L.oP32 = take(9 * fV);    // PA and PB (4 values per cell each), then mu
    for (int d = 0; d < 3; ++d) L.oFf[d] = take(sizeof(float) * NEQ * (size_t)s.IV);
    L.oTv32 = take(sizeof(float4) * 3 * (size_t)s.RV);
  }
  L.oCtl = take(sizeof(SolveCtl));
  L.oDesc = take(sizeof(SolveDev));
  L.oTi = take(sizeof(TileRef) * n_int);
  L.oTr = take(sizeof(TileRef) * n_ring);
  L.oTp = take(sizeof(TileRef) * n_pad);
  L.oPart = take(sizeof(double) * 4 * nparts);
  L.oOut = take(sizeof(double) * 8);
  L.total = off;
  return L;
}

void set_extents(SolveDev& s, uint32_t IM, uint32_t JM, uint32_t KM) {
  s.IM = IM;
  s.JM = JM;
  s.KM = KM;
  s.nx = IM + 2 * NG;
  s.ny = JM + 2 * NG;
  s.nz = KM + 2 * NG;
  s.V = (long long)s.nx * s.ny * s.nz;
  s.rx = IM + 2 * NGV;
  s.ry = JM + 2 * NGV;
  s.rz = KM + 2 * NGV;
  s.RV = (long long)s.rx * s.ry * s.rz;
  s.IV = (long long)IM * JM * KM;
}

constexpr int kDiagParts = 1024;

}  // namespace

namespace cbns {
// Lets other translation units of the library report through cbns_last_error().
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace cbns



extern "C" {

const char* cbns_last_error(void) { return g_last_error.c_str(); }
const char* cbns_version(void) { return "cbns3d-gb300 0.1.0 (sm_103a)"; }

cbns_status cbns_params_derive(cbns_params* p) {
  if (!p) return fail(CBNS_ERR_INVALID_ARG, "cbns_params_derive: null params");
  // src/read_input.cpp:78-90
  p->Mach2 = p->Mach * p->Mach;
  p->Re_inv = 1.0 / p->Re;
  p->Pr_inv = 1.0 / p->Pr;
  p->gam1 = p->gamma - 1.0;
  p->gM2 = p->gamma * p->Mach2;
  p->gam1_inv = 1.0 / p->gam1;
  p->p_inf = 1.0 / p->gM2;
  p->C_T_inf = 110.5 / p->T_inf;
  double a = 4.0 / 3.0, g = p->gamma * p->Pr_inv;
  p->C_dt_v = (a < g ? g : a) * p->Re_inv;
  return CBNS_OK;
}

cbns_status cbns_destroy(cbns_handle* h) {
  if (!h) return CBNS_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->up_stream) cudaStreamSynchronize(h->up_stream);
  if (h->down_stream) cudaStreamSynchronize(h->down_stream);
  if (h->step_graph) cudaGraphExecDestroy(h->step_graph);
  if (h->d_stage_out) cudaFree(h->d_stage_out);
  for (cudaEvent_t ev : {h->ev_in_ready, h->ev_in_free, h->ev_out_ready, h->ev_out_free})
    if (ev) cudaEventDestroy(ev);
  if (h->up_stream) cudaStreamDestroy(h->up_stream);
  if (h->down_stream) cudaStreamDestroy(h->down_stream);
  if (h->arena) cudaFree(h->arena);
  if (h->h_ctl) cudaFreeHost(h->h_ctl);
  if (h->h_out) cudaFreeHost(h->h_out);
  for (int b = 0; b < 2; ++b) {
    if (h->h_chunk[b]) cudaFreeHost(h->h_chunk[b]);
    if (h->ev_chunk[b]) cudaEventDestroy(h->ev_chunk[b]);
  }
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return CBNS_OK;
}

cbns_status cbns_create(const cbns_params* p, uint32_t IM, uint32_t JM, uint32_t KM, int precision,
                        cbns_handle** out) {
  if (!p || !out) return fail(CBNS_ERR_INVALID_ARG, "cbns_create: null argument");
  *out = nullptr;
  if (precision != CBNS_FP64 && precision != CBNS_FP32_MIXED && precision != CBNS_FP64_FF)
    return fail(CBNS_ERR_INVALID_ARG, "cbns_create: unknown precision");
  // The reference's halo exchange sends NG interior layers; a block narrower than
  // NG would send ghost cells.  Above that, the extents are limited by the 16-bit
  // tile coordinates (block_extents_ok) and by device memory (checked against
  // cbns_footprint's arena size below); every offset is 64-bit.
  if (IM < (uint32_t)NG || JM < (uint32_t)NG || KM < (uint32_t)NG)
    return fail(CBNS_ERR_BAD_DIMS, "cbns_create: every extent must be >= 4 (NG)");
  if (!block_extents_ok(IM, JM, KM))
    return fail(CBNS_ERR_BAD_DIMS, "cbns_create: an extent exceeds " + std::to_string(kMaxExtent) +
                                       " cells (16-bit tile coordinates)");
  if (!(p->gamma > 1.0) || !(p->Re > 0.0) || !(p->Mach > 0.0) || !(p->Pr > 0.0) || !(p->CFL > 0.0) ||
      !(p->T_inf > 0.0) || p->IM == 0 || p->JM == 0 || p->KM == 0)
    return fail(CBNS_ERR_INVALID_ARG, "cbns_create: parameters out of range (gamma>1, Re, Mach, Pr, CFL, T_inf > 0)");
  // One GPU holds the whole grid: the spacing (gen_mesh, from p->IM/JM/KM) and the
  // periodic ghost images (from the block's own extents) must describe one grid.
  if (p->IM != IM || p->JM != JM || p->KM != KM)
    return fail(CBNS_ERR_BAD_DIMS, "cbns_create: the block extents must equal the grid's (p->IM, p->JM, p->KM): "
                                   "one GPU holds the whole periodic grid");

  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(CBNS_ERR_NO_DEVICE, "cbns_create: no CUDA device");
  }
  // The calling thread's current device, unless CBNS_DEVICE names one.
  int dev = 0;
  if (const char* e = std::getenv("CBNS_DEVICE")) {
    dev = std::atoi(e);
  } else if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    dev = 0;
  }
  if (dev < 0 || dev >= ndev) return fail(CBNS_ERR_NO_DEVICE, "cbns_create: CBNS_DEVICE out of range");
  cudaDeviceProp prop;
  CBNS_CUDA(cudaGetDeviceProperties(&prop, dev));
  if (prop.major != 10 || prop.minor != 3)
    return fail(CBNS_ERR_NO_DEVICE, std::string("cbns_create: built for sm_103a, device is ") + prop.name);

  cbns_handle* h = new cbns_handle();
  h->device = dev;
  h->precision = precision;
  h->params = *p;
  cbns_params_derive(&h->params);
  h->IM = IM;
  h->JM = JM;
  h->KM = KM;
  auto bail = [&](cbns_status s) {
    cbns_destroy(h);
    return s;
  };
  if (cudaSetDevice(dev) != cudaSuccess) return bail(cuda_fail(cudaGetLastError(), "cudaSetDevice"));
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(cuda_fail(cudaGetLastError(), "cudaStreamCreate"));

  SolveDev& s = h->desc;
  set_extents(s, IM, JM, KM);

  // Arena layout.  Both modes hold the binary64 state (Q, Q_p, staging) and
  // binary64 primitives; binary64 solves add binary64 face/viscous fluxes,
  // FP32-mixed solves the binary32 perturbation state, primitives and fluxes.
  // The size is checked against free device memory before any table is built.
  const bool mixed = precision == CBNS_FP32_MIXED;
  s.mixed = mixed ? 1 : 0;
  h->nparts = kDiagParts;
  const size_t nt_int = tile_count(IM, JM, KM), nt_ring = ring_tile_count(s.rx, s.ry, s.rz, mixed),
               nt_pad = tile_count(s.nx, s.ny, s.nz);
  const ArenaLayout L = arena_layout(s, precision, nt_int, nt_ring, nt_pad, h->nparts);
  const size_t off = L.total;
  {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && off > free_b)
      return bail(fail(CBNS_ERR_OUT_OF_MEMORY, "cbns_create: the block needs " + std::to_string(off) +
                                                   " device bytes, " + std::to_string(free_b) + " are free"));
    cudaGetLastError();
  }
  std::vector<TileRef> t_int, t_ring, t_pad;
  append_tiles(t_int, 0, IM, JM, KM);
  append_ring_tiles(t_ring, 0, s.rx, s.ry, s.rz, mixed);
  append_tiles(t_pad, 0, s.nx, s.ny, s.nz);
  h->n_int = (int)t_int.size();
  h->n_ring = (int)t_ring.size();
  h->n_pad = (int)t_pad.size();

  const size_t oQ = L.oQ, oQp = L.oQp, oStage = L.oStage, oPrim = L.oPrim, oU32 = L.oU32, oP32 = L.oP32;
  const size_t oCtl = L.oCtl, oDesc = L.oDesc, oTi = L.oTi, oTr = L.oTr, oTp = L.oTp, oPart = L.oPart,
               oOut = L.oOut;
  const size_t *oF = L.oF, *oFf = L.oFf;
  h->arena_bytes = off;
  cudaError_t e = cudaMalloc(&h->arena, off);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc(arena)"));
  e = cudaMemsetAsync(h->arena, 0, off, h->stream);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMemset(arena)"));

  char* A = h->arena;
  s.Q = (double*)(A + oQ);
  s.Qp = (double*)(A + oQp);
  h->d_stage = (double*)(A + oStage);
  double* prim = (double*)(A + oPrim);
  s.pd = PrimSet<double>{prim + 0 * s.V, prim + 1 * s.V, prim + 2 * s.V, prim + 3 * s.V, prim + 4 * s.V,
                         prim + 5 * s.V, prim + 6 * s.V, prim + 7 * s.V, prim + 8 * s.V};
  if (!mixed) {
    s.ffaces = precision == CBNS_FP64_FF ? 1 : 0;
    for (int d = 0; d < 3; ++d) {
      s.F[d] = s.ffaces ? nullptr : (double*)(A + oF[d]);
      s.FFa[d] = s.ffaces ? (float4*)(A + L.oFFa[d]) : nullptr;
      s.Ff[d] = nullptr;
    }
    s.Tv = s.ffaces ? nullptr : (double*)(A + L.oTv);
    s.TvG = s.ffaces ? (float4*)(A + L.oTvG) : nullptr;
    s.Tvg = nullptr;
    s.U4 = nullptr;
    s.UE = nullptr;
    s.PA = s.PB = nullptr;
    s.muf = nullptr;
    s.QF = s.ffaces ? (float2*)(A + L.oQF) : nullptr;
    s.QpF = s.ffaces ? (float2*)(A + L.oQpF) : nullptr;
    s.PF = s.ffaces ? (float2*)(A + L.oPF) : nullptr;
  } else {
    s.ffaces = 0;
    for (int d = 0; d < 3; ++d) s.FFa[d] = nullptr;
    s.TvG = nullptr;
    s.QF = s.QpF = s.PF = nullptr;
    s.U4 = (float4*)(A + oU32);
    s.UE = (float*)(s.U4 + s.V);
    s.PA = (float4*)(A + oP32);
    s.PB = s.PA + s.V;
    s.muf = (float*)(s.PB + s.V);
    for (int d = 0; d < 3; ++d) {
      s.Ff[d] = (float*)(A + oFf[d]);
      s.F[d] = nullptr;
    }
    s.Tvg = (float4*)(A + L.oTv32);
    s.Tv = nullptr;
  }
  const cbns_params& P = h->params;
  // Reference state of the FP32-mixed perturbation form: the reference's
  // free stream, rho = 1, p = 1/(gamma M^2) (src/read_input.cpp:88), u = 0.
  s.p_ref = P.p_inf;
  s.rho_ref = P.gM2 * P.p_inf;
  s.E_ref = P.p_inf * P.gam1_inv;
  s.T_ref = P.gM2 * s.p_ref / s.rho_ref;
  s.gamma = P.gamma;
  s.gam1 = P.gam1;
  s.gam1_inv = P.gam1_inv;
  s.gM2 = P.gM2;
  s.Re_inv = P.Re_inv;
  s.kappa = -P.Pr_inv * P.gam1_inv / P.Mach2;  // src/Block3d.cpp:766-767
  s.C_T_inf = P.C_T_inf;
  s.C_T_inf1 = 1.0 + P.C_T_inf;
  s.CFL = P.CFL;
  s.C_dt_v = P.C_dt_v;
  // gen_mesh (src/Block3d.cpp:215-219): spacing from the global grid size.
  const double two_pi = 2.0 * 3.14159265358979323846;
  s.dx = two_pi / P.IM;
  s.dy = two_pi / P.JM;
  s.dz = two_pi / P.KM;
  s.inv_dx = 1.0 / s.dx;
  s.inv_dy = 1.0 / s.dy;
  s.inv_dz = 1.0 / s.dz;
  fill_consts(s);
  {
    // float-float constants of CBNS_FP64_FF faces: hi = x rounded to binary32,
    // lo = the rest rounded
    auto split = [](double x) {
      const float hi = (float)x;
      return make_float2(hi, (float)(x - (double)hi));
    };
    s.ff_gam1 = split(s.gam1);
    s.ff_gamma = split(s.gamma);
    s.ff_hgam1 = split(0.5 * s.gam1);
    const Consts<double>& c = s.cd;
    const double hf[3] = {c.hfx, c.hfy, c.hfz}, c12[3] = {c.c12x, c.c12y, c.c12z},
                 c23[3] = {c.c23x, c.c23y, c.c23z};
    for (int d = 0; d < 3; ++d) {
      s.ff_hf[d] = split(hf[d]);
      s.ff_c12[d] = split(c12[d]);
      s.ff_c23[d] = split(c23[d]);
    }
    s.ff_Re_inv = split(s.Re_inv);
    s.ff_kappa = split(s.kappa);
    s.ff_C = split(s.C_T_inf);
    s.ff_C1 = split(s.C_T_inf1);
    s.ff_gM2 = split(s.gM2);
    s.ff_igM2 = split(1.0 / s.gM2);
    s.ff_ggam1 = split(c.gamma_gam1_inv);
    s.ff_Cdt2 = split(c.C_dt_v2);
    s.ff_sum_ih = split(c.sum_ih);
    s.ff_sum_ih2 = split(c.sum_ih2);
    s.ff_rho_ref = split(s.rho_ref);
    s.ff_p_ref = split(s.p_ref);
    s.ff_Ep_ref = split(s.E_ref + s.p_ref);
  }
  h->d_ctl = (SolveCtl*)(A + oCtl);
  s.ctl = h->d_ctl;
  h->d_desc = (SolveDev*)(A + oDesc);
  h->d_tiles_int = (TileRef*)(A + oTi);
  h->d_tiles_ring = (TileRef*)(A + oTr);
  h->d_tiles_pad = (TileRef*)(A + oTp);
  h->d_partials = (double*)(A + oPart);
  h->d_out = (double*)(A + oOut);

  if ((e = cudaMallocHost(&h->h_ctl, sizeof(SolveCtl))) != cudaSuccess) return bail(cuda_fail(e, "cudaMallocHost"));
  if ((e = cudaMallocHost(&h->h_out, sizeof(double) * 8)) != cudaSuccess) return bail(cuda_fail(e, "cudaMallocHost"));
  std::memset(h->h_ctl, 0, sizeof(SolveCtl));
  h->h_ctl->t_cur = P.t_cur;
  h->h_ctl->t_end = P.t_end;

  if ((e = cudaMemcpyAsync(h->d_desc, &h->desc, sizeof(SolveDev), cudaMemcpyHostToDevice, h->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(h->d_tiles_int, t_int.data(), sizeof(TileRef) * t_int.size(), cudaMemcpyHostToDevice,
                           h->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(h->d_tiles_ring, t_ring.data(), sizeof(TileRef) * t_ring.size(),
                           cudaMemcpyHostToDevice, h->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(h->d_tiles_pad, t_pad.data(), sizeof(TileRef) * t_pad.size(), cudaMemcpyHostToDevice,
                           h->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(h->d_ctl, h->h_ctl, sizeof(SolveCtl), cudaMemcpyHostToDevice, h->stream)) != cudaSuccess)
    return bail(cuda_fail(e, "cudaMemcpyAsync(setup)"));

  if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return bail(cuda_fail(e, "cudaStreamSynchronize"));
  *out = h;
  return CBNS_OK;
}

static cbns_status check_handle(cbns_handle* h, const char* fn) {
  if (!h) return fail(CBNS_ERR_INVALID_ARG, std::string(fn) + ": null handle");
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  return CBNS_OK;
}

cbns_status cbns_upload_Q(cbns_handle* h, const double* Q, double t) {
  cbns_status st = check_handle(h, "cbns_upload_Q");
  if (st != CBNS_OK) return st;
  if (!Q) return fail(CBNS_ERR_INVALID_ARG, "cbns_upload_Q: null Q");
  // The host array goes to the staging buffer as-is, then becomes the state.
  CBNS_CUDA(cudaMemcpyAsync(h->d_stage, Q, sizeof(double) * NEQ * (size_t)h->desc.V, cudaMemcpyHostToDevice,
                            h->stream));
  return cbns::adopt_staged(h, t);
}

cbns_status cbns_init_tgv(cbns_handle* h, uint64_t seed, double amp, int nmodes, int kmax, double t) {
  cbns_status st = check_handle(h, "cbns_init_tgv");
  if (st != CBNS_OK) return st;
  if (nmodes < 0 || nmodes > 64 || (nmodes > 0 && kmax < 1))
    return fail(CBNS_ERR_INVALID_ARG, "cbns_init_tgv: nmodes must be in [0, 64] and kmax >= 1");
  std::vector<PerturbMode> modes;
  if (nmodes > 0) modes = draw_modes(seed, amp, nmodes, kmax);
  CBNS_CUDA(launch_init_tgv(h->d_desc, 0, h->d_tiles_int, h->n_int, h->params.p_inf, modes.data(), nmodes,
                            h->stream));
  CBNS_CUDA(launch_prepare(h->d_desc, h->d_tiles_pad, h->n_pad, h->stream, h->pf()));
  std::memset(h->h_ctl, 0, sizeof(SolveCtl));
  h->h_ctl->t_cur = t;
  h->h_ctl->t_end = h->params.t_end;
  h->h_ctl->active = 1;
  CBNS_CUDA(cudaMemcpyAsync(h->d_ctl, h->h_ctl, sizeof(SolveCtl), cudaMemcpyHostToDevice, h->stream));
  CBNS_CUDA(cudaStreamSynchronize(h->stream));
  return CBNS_OK;
}

static cbns_status download_state(cbns_handle* h, const double* src, double* dst, const char* fn) {
  cbns_status st = check_handle(h, fn);
  if (st != CBNS_OK) return st;
  if (!dst) return fail(CBNS_ERR_INVALID_ARG, std::string(fn) + ": null output");
  const SolveDev& s = h->desc;
  CBNS_CUDA(launch_layout(h->d_desc, 0, src, h->d_stage, false, s.V, h->stream, h->pf()));
  CBNS_CUDA(cudaMemcpyAsync(dst, h->d_stage, sizeof(double) * NEQ * (size_t)s.V, cudaMemcpyDeviceToHost, h->stream));
  CBNS_CUDA(cudaStreamSynchronize(h->stream));
  return CBNS_OK;
}

cbns_status cbns_download_Q(cbns_handle* h, double* Q) {
  if (!h) return fail(CBNS_ERR_INVALID_ARG, "cbns_download_Q: null handle");
  return download_state(h, h->desc.Q, Q, "cbns_download_Q");
}

cbns_status cbns_download_Q_p(cbns_handle* h, double* Qp) {
  if (!h) return fail(CBNS_ERR_INVALID_ARG, "cbns_download_Q_p: null handle");
  return download_state(h, h->desc.Qp, Qp, "cbns_download_Q_p");
}

cbns_status cbns_download_prims(cbns_handle* h, double* rho, double* u, double* v, double* w, double* p,
                                double* T) {
  cbns_status st = check_handle(h, "cbns_download_prims");
  if (st != CBNS_OK) return st;
  const SolveDev& s = h->desc;
  const size_t bytes = sizeof(double) * (size_t)s.V;
  // FP32-mixed solves step with binary32 primitives and CBNS_FP64_FF solves with
  // float-float ones; form the binary64 ones of Q.
  if (s.mixed || s.ffaces) CBNS_CUDA(launch_prims_double(h->d_desc, h->d_tiles_pad, h->n_pad, h->stream));
  double* dst[6] = {rho, u, v, w, p, T};
  double* src[6] = {s.pd.rho, s.pd.u, s.pd.v, s.pd.w, s.pd.p, s.pd.T};
  for (int a = 0; a < 6; ++a)
    if (dst[a]) CBNS_CUDA(cudaMemcpyAsync(dst[a], src[a], bytes, cudaMemcpyDeviceToHost, h->stream));
  CBNS_CUDA(cudaStreamSynchronize(h->stream));
  return CBNS_OK;
}

cbns_status cbns_calc_dt(cbns_handle* h, double* dt) {
  cbns_status st = check_handle(h, "cbns_calc_dt");
  if (st != CBNS_OK) return st;
  if (!dt) return fail(CBNS_ERR_INVALID_ARG, "cbns_calc_dt: null output");
  CBNS_CUDA(launch_dt_raw(h->d_desc, 0, h->d_tiles_int, h->n_int, h->d_out, h->precision, LaunchCfg{},
                          h->stream, h->pf()));
  CBNS_CUDA(cudaMemcpyAsync(h->h_out, h->d_out, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CBNS_CUDA(cudaStreamSynchronize(h->stream));
  *dt = h->h_out[0];
  return CBNS_OK;
}

static cbns_status enqueue_stage(cbns_handle* h, int stage) {
  const StageTables T{h->d_tiles_int, h->n_int, h->d_tiles_ring, h->n_ring};
  CBNS_CUDA(launch_stage(h->d_desc, T, stage, LaunchCfg{}, h->precision, h->stream, h->pf()));
  return CBNS_OK;
}

cbns_status cbns_stage(cbns_handle* h, double dt, int stage) {
  cbns_status st = check_handle(h, "cbns_stage");
  if (st != CBNS_OK) return st;
  if (stage < 1 || stage > 3) return fail(CBNS_ERR_INVALID_ARG, "cbns_stage: stage must be 1, 2 or 3");
  CBNS_CUDA(launch_set_dt(h->d_desc, 0, dt, h->stream));
  if ((st = enqueue_stage(h, stage)) != CBNS_OK) return st;
  CBNS_CUDA(cudaStreamSynchronize(h->stream));
  return CBNS_OK;
}

static cbns_status enqueue_step(cbns_handle* h, double t_end, bool use_t_end) {
  CBNS_CUDA(launch_dt(h->d_desc, 1, h->d_tiles_int, h->n_int, t_end, use_t_end, h->precision, LaunchCfg{},
                      h->stream, h->pf()));
  for (int s = 1; s <= 3; ++s) {
    cbns_status st = enqueue_stage(h, s);
    if (st != CBNS_OK) return st;
  }
  return CBNS_OK;
}

cbns_status cbns_step(cbns_handle* h, double t_end, double* dt_out, double* t_out) {
  cbns_status st = check_handle(h, "cbns_step");
  if (st != CBNS_OK) return st;
  if ((st = enqueue_step(h, t_end, true)) != CBNS_OK) return st;
  CBNS_CUDA(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, h->stream));
  CBNS_CUDA(cudaStreamSynchronize(h->stream));
  if (dt_out) *dt_out = h->h_ctl->dt;
  if (t_out) *t_out = h->h_ctl->t_cur;
  if (h->h_ctl->status) return ctl_fail(h->h_ctl->status, "cbns_step");
  return h->h_ctl->active ? CBNS_OK : CBNS_FINISHED;
}

// The step of enqueue_step captured as a CUDA graph for this t_end (rebuilt when
// t_end changes).
static cbns_status ensure_step_graph(cbns_handle* h, double t_end) {
  if (h->step_graph && h->graph_t_end == t_end) return CBNS_OK;
  if (h->step_graph) {
    cudaGraphExecDestroy(h->step_graph);
    h->step_graph = nullptr;
  }
  cudaGraph_t g;
  CBNS_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  cbns_status st = enqueue_step(h, t_end, true);
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  if (st != CBNS_OK) return st;
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&h->step_graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  h->graph_t_end = t_end;
  return CBNS_OK;
}

cbns_status cbns_run(cbns_handle* h, uint32_t nsteps, double t_end, uint32_t* steps_done) {
  cbns_status st = check_handle(h, "cbns_run");
  if (st != CBNS_OK) return st;
  CBNS_CUDA(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, h->stream));
  CBNS_CUDA(cudaStreamSynchronize(h->stream));
  const unsigned start = h->h_ctl->steps;
  if (h->prof.on) {
    // Profiling: direct launches, each bracketed by events.
    for (uint32_t n = 0; n < nsteps; ++n)
      if ((st = enqueue_step(h, t_end, true)) != CBNS_OK) return st;
  } else if ((st = ensure_step_graph(h, t_end)) != CBNS_OK) {
    return st;
  }
  if (!h->prof.on)
    for (uint32_t n = 0; n < nsteps; ++n) CBNS_CUDA(cudaGraphLaunch(h->step_graph, h->stream));
  CBNS_CUDA(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, h->stream));
  CBNS_CUDA(cudaStreamSynchronize(h->stream));
  if (steps_done) *steps_done = h->h_ctl->steps - start;
  if (h->h_ctl->status) return ctl_fail(h->h_ctl->status, "cbns_run");
  return CBNS_OK;
}

// ---------------------------------------------------------------------------
// Asynchronous entry points.  Work goes to three streams of the handle: kernels
// on h->stream, host-to-device copies on h->up_stream and device-to-host copies
// on h->down_stream, ordered by events, through two staging buffers (uploads
// through d_stage, downloads through d_stage_out).  The upload of the next
// state then runs under the current step's kernels, and the download of a
// result under the next step's.

// Each piece is made once; a call that failed part-way resumes where it stopped.
static cbns_status ensure_async(cbns_handle* h) {
  if (h->down_stream) return CBNS_OK;
  if (!h->d_stage_out) {
    const size_t bytes = sizeof(double) * NEQ * (size_t)h->desc.V;
    cudaError_t e = cudaMalloc(&h->d_stage_out, bytes);
    if (e != cudaSuccess) {
      h->d_stage_out = nullptr;
      return cuda_fail(e, "cudaMalloc(download staging)");
    }
    h->arena_bytes += bytes;
  }
  for (cudaEvent_t* ev : {&h->ev_in_ready, &h->ev_in_free, &h->ev_out_ready, &h->ev_out_free})
    if (!*ev) CBNS_CUDA(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
  if (!h->up_stream) CBNS_CUDA(cudaStreamCreateWithFlags(&h->up_stream, cudaStreamNonBlocking));
  // Both staging buffers start free.
  CBNS_CUDA(cudaEventRecord(h->ev_in_free, h->stream));
  CBNS_CUDA(cudaEventRecord(h->ev_out_free, h->stream));
  CBNS_CUDA(cudaStreamCreateWithFlags(&h->down_stream, cudaStreamNonBlocking));  // last: marks set-up done
  return CBNS_OK;
}

cbns_status cbns_upload_Q_async(cbns_handle* h, const double* Q, double t) {
  cbns_status st = check_handle(h, "cbns_upload_Q_async");
  if (st != CBNS_OK) return st;
  if (!Q) return fail(CBNS_ERR_INVALID_ARG, "cbns_upload_Q_async: null Q");
  if ((st = ensure_async(h)) != CBNS_OK) return st;
  const SolveDev& s = h->desc;
  // upload stream: wait until the last upload's transpose has read the staging
  // buffer, then copy the host state into it
  CBNS_CUDA(cudaStreamWaitEvent(h->up_stream, h->ev_in_free, 0));
  CBNS_CUDA(cudaMemcpyAsync(h->d_stage, Q, sizeof(double) * NEQ * (size_t)s.V, cudaMemcpyHostToDevice,
                            h->up_stream));
  CBNS_CUDA(cudaEventRecord(h->ev_in_ready, h->up_stream));
  // compute stream: the start-up sequence of cbns_upload_Q once the copy is in
  CBNS_CUDA(cudaStreamWaitEvent(h->stream, h->ev_in_ready, 0));
  CBNS_CUDA(launch_layout(h->d_desc, 0, h->d_stage, s.Q, true, s.V, h->stream, nullptr));
  CBNS_CUDA(cudaEventRecord(h->ev_in_free, h->stream));
  CBNS_CUDA(launch_prepare(h->d_desc, h->d_tiles_pad, h->n_pad, h->stream, nullptr));
  CBNS_CUDA(launch_reset_ctl(h->d_ctl, t, h->params.t_end, h->stream));
  return CBNS_OK;
}

cbns_status cbns_step_async(cbns_handle* h, double t_end) {
  cbns_status st = check_handle(h, "cbns_step_async");
  if (st != CBNS_OK) return st;
  if ((st = ensure_step_graph(h, t_end)) != CBNS_OK) return st;
  CBNS_CUDA(cudaGraphLaunch(h->step_graph, h->stream));
  return CBNS_OK;
}

cbns_status cbns_download_Q_async(cbns_handle* h, double* Q) {
  cbns_status st = check_handle(h, "cbns_download_Q_async");
  if (st != CBNS_OK) return st;
  if (!Q) return fail(CBNS_ERR_INVALID_ARG, "cbns_download_Q_async: null output");
  if ((st = ensure_async(h)) != CBNS_OK) return st;
  const SolveDev& s = h->desc;
  // compute stream: wait until the last download has left the staging buffer,
  // then transpose the current state into it
  CBNS_CUDA(cudaStreamWaitEvent(h->stream, h->ev_out_free, 0));
  CBNS_CUDA(launch_layout(h->d_desc, 0, s.Q, h->d_stage_out, false, s.V, h->stream, nullptr));
  CBNS_CUDA(cudaEventRecord(h->ev_out_ready, h->stream));
  // download stream: the device-to-host copy, overlapping later kernels
  CBNS_CUDA(cudaStreamWaitEvent(h->down_stream, h->ev_out_ready, 0));
  CBNS_CUDA(cudaMemcpyAsync(Q, h->d_stage_out, sizeof(double) * NEQ * (size_t)s.V, cudaMemcpyDeviceToHost,
                            h->down_stream));
  CBNS_CUDA(cudaEventRecord(h->ev_out_free, h->down_stream));
  return CBNS_OK;
}

cbns_status cbns_wait(cbns_handle* h, double* dt_last, double* t_cur) {
  cbns_status st = check_handle(h, "cbns_wait");
  if (st != CBNS_OK) return st;
  CBNS_CUDA(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, h->stream));
  CBNS_CUDA(cudaStreamSynchronize(h->stream));
  if (h->up_stream) CBNS_CUDA(cudaStreamSynchronize(h->up_stream));
  if (h->down_stream) CBNS_CUDA(cudaStreamSynchronize(h->down_stream));
  if (dt_last) *dt_last = h->h_ctl->dt;
  if (t_cur) *t_cur = h->h_ctl->t_cur;
  if (h->h_ctl->status) return ctl_fail(h->h_ctl->status, "cbns_wait");
  return h->h_ctl->active ? CBNS_OK : CBNS_FINISHED;
}

cbns_status cbns_poll(cbns_handle* h, int* done) {
  cbns_status st = check_handle(h, "cbns_poll");
  if (st != CBNS_OK) return st;
  if (!done) return fail(CBNS_ERR_INVALID_ARG, "cbns_poll: null output");
  cudaError_t e = cudaStreamQuery(h->stream);
  if (e == cudaSuccess && h->up_stream) e = cudaStreamQuery(h->up_stream);
  if (e == cudaSuccess && h->down_stream) e = cudaStreamQuery(h->down_stream);
  if (e == cudaErrorNotReady) {
    *done = 0;
    return CBNS_OK;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cbns_poll");
  *done = 1;
  return CBNS_OK;
}

cbns_status cbns_get_time(cbns_handle* h, double* t_cur, double* dt_last) {
  cbns_status st = check_handle(h, "cbns_get_time");
  if (st != CBNS_OK) return st;
  CBNS_CUDA(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, h->stream));
  CBNS_CUDA(cudaStreamSynchronize(h->stream));
  if (t_cur) *t_cur = h->h_ctl->t_cur;
  if (dt_last) *dt_last = h->h_ctl->dt;
  return CBNS_OK;
}

cbns_status cbns_diagnostics(cbns_handle* h, double* ke, double* enstrophy) {
  cbns_status st = check_handle(h, "cbns_diagnostics");
  if (st != CBNS_OK) return st;
  const double inv_n = 1.0 / ((double)h->IM * (double)h->JM * (double)h->KM);
  CBNS_CUDA(launch_diag(h->d_desc, 0, h->d_tiles_int, h->n_int, h->d_partials, h->nparts, inv_n, h->d_out,
                        h->stream, h->pf()));
  CBNS_CUDA(cudaMemcpyAsync(h->h_out, h->d_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CBNS_CUDA(cudaStreamSynchronize(h->stream));
  if (ke) *ke = h->h_out[0];
  if (enstrophy) *enstrophy = h->h_out[1];
  return CBNS_OK;
}

cbns_status cbns_check_state(cbns_handle* h) {
  cbns_status st = check_handle(h, "cbns_check_state");
  if (st != CBNS_OK) return st;
  CBNS_CUDA(cudaMemcpyAsync(h->h_ctl, h->d_ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, h->stream));
  CBNS_CUDA(cudaStreamSynchronize(h->stream));
  if (const int bits = h->h_ctl->status) {
    h->h_ctl->status = 0;
    CBNS_CUDA(cudaMemcpyAsync(&h->d_ctl->status, &h->h_ctl->status, sizeof(int), cudaMemcpyHostToDevice,
                              h->stream));
    CBNS_CUDA(cudaStreamSynchronize(h->stream));
    return ctl_fail(bits, "cbns_check_state (since the last check)");
  }
  return CBNS_OK;
}

void* cbns_stream(cbns_handle* h) { return h ? (void*)h->stream : nullptr; }

cbns_status cbns_profile_begin(cbns_handle* h) {
  cbns_status st = check_handle(h, "cbns_profile_begin");
  if (st != CBNS_OK) return st;
  h->prof.reset();
  h->prof.on = true;
  return CBNS_OK;
}

cbns_status cbns_profile_end(cbns_handle* h, cbns_kernel_time* out, int cap, int* n) {
  cbns_status st = check_handle(h, "cbns_profile_end");
  if (st != CBNS_OK) return st;
  CBNS_CUDA(cudaStreamSynchronize(h->stream));
  double total[KID_COUNT] = {0};
  unsigned count[KID_COUNT] = {0};
  for (const Profiler::Rec& r : h->prof.recs) {
    if (!r.b) continue;
    float ms = 0.f;
    CBNS_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
    total[r.id] += ms;
    count[r.id] += 1;
  }
  h->prof.on = false;
  h->prof.reset();
  int k = 0;
  for (int id = 0; id < KID_COUNT; ++id) {
    if (!count[id]) continue;
    if (out && k < cap) {
      std::memset(out[k].name, 0, sizeof out[k].name);
      std::strncpy(out[k].name, kernel_name(id), sizeof out[k].name - 1);
      out[k].launches = count[id];
      out[k].total_ms = total[id];
    }
    ++k;
  }
  if (n) *n = k < cap ? k : cap;
  return CBNS_OK;
}

// ---------------------------------------------------------------------------
// Batches.

}  // extern "C"

namespace {
constexpr int kRowsOptions[3] = {2, 4, 8};
int rows_index(int rows) { return rows == 2 ? 0 : (rows == 8 ? 2 : 1); }
}  // namespace


static cbns_status batch_enqueue_step(cbns_batch* b) {
  const int ri = rows_index(b->cfg.tile_rows);
  const int n = (int)b->handles.size();
  CBNS_CUDA(launch_dt(b->d_descs, n, b->d_int[ri], b->n_int[ri], 0.0, false, b->precision, b->cfg, b->stream, nullptr));
  const StageTables T{b->d_int[ri], b->n_int[ri], b->d_ring[ri], b->n_ring[ri]};
  for (int st = 1; st <= 3; ++st)
    CBNS_CUDA(launch_stage(b->d_descs, T, st, b->cfg, b->precision, b->stream, nullptr));
  return CBNS_OK;
}

static cbns_status batch_graph(cbns_batch* b) {
  if (b->graph && b->graph_rows == b->cfg.tile_rows && b->graph_ctas == b->cfg.max_ctas) return CBNS_OK;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  cudaGraph_t g;
  CBNS_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  cbns_status st = batch_enqueue_step(b);
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (st != CBNS_OK) return st;
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture(batch)");
  e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate(batch)");
  b->graph_rows = b->cfg.tile_rows;
  b->graph_ctas = b->cfg.max_ctas;
  return CBNS_OK;
}

extern "C" {

cbns_status cbns_batch_destroy(cbns_batch* b) {
  if (!b) return CBNS_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->arena) cudaFree(b->arena);
  if (b->h_ctl) cudaFreeHost(b->h_ctl);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return CBNS_OK;
}

cbns_status cbns_batch_create(cbns_handle* const* handles, int n, cbns_batch** out) {
  if (!handles || !out || n <= 0) return fail(CBNS_ERR_INVALID_ARG, "cbns_batch_create: no handles");
  *out = nullptr;
  if (n > 65535) return fail(CBNS_ERR_INVALID_ARG, "cbns_batch_create: at most 65535 solves");
  for (int i = 0; i < n; ++i) {
    if (!handles[i]) return fail(CBNS_ERR_INVALID_ARG, "cbns_batch_create: null handle");
    if (handles[i]->device != handles[0]->device || handles[i]->precision != handles[0]->precision)
      return fail(CBNS_ERR_INVALID_ARG, "cbns_batch_create: handles differ in device or precision");
  }
  {
    // A handle listed twice would put its tiles in the table twice: two CTAs
    // would update the same cells and control block in every stage.
    std::vector<cbns_handle*> sorted(handles, handles + n);
    std::sort(sorted.begin(), sorted.end());
    if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
      return fail(CBNS_ERR_INVALID_ARG, "cbns_batch_create: a handle appears more than once");
  }
  cbns_batch* b = new cbns_batch();
  auto bail = [&](cbns_status st) {
    cbns_batch_destroy(b);
    return st;
  };
  b->device = handles[0]->device;
  b->mixed = handles[0]->precision == CBNS_FP32_MIXED;
  b->precision = handles[0]->precision;
  b->handles.assign(handles, handles + n);
  cudaError_t e = cudaSetDevice(b->device);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaSetDevice"));
  if ((e = cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device)) != cudaSuccess)
    return bail(cuda_fail(e, "cudaDeviceGetAttribute"));
  if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(cuda_fail(e, "cudaStreamCreate(batch)"));
  std::vector<SolveDev> descs(n);
  std::vector<TileRef> ti[3], tr[3];
  for (int i = 0; i < n; ++i) {
    const SolveDev& s = handles[i]->desc;
    descs[i] = s;
    for (int r = 0; r < 3; ++r) {
      append_tiles(ti[r], i, s.IM, s.JM, s.KM, kRowsOptions[r]);
      append_ring_tiles(tr[r], i, s.rx, s.ry, s.rz, b->mixed, kRowsOptions[r]);
    }
  }
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += align_up(bytes);
    return o;
  };
  size_t oD = take(sizeof(SolveDev) * n), oI[3], oR[3];
  for (int r = 0; r < 3; ++r) {
    oI[r] = take(sizeof(TileRef) * ti[r].size());
    oR[r] = take(sizeof(TileRef) * tr[r].size());
  }
  if ((e = cudaMalloc(&b->arena, off)) != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc(batch)"));
  b->d_descs = (SolveDev*)(b->arena + oD);
  if ((e = cudaMemcpyAsync(b->d_descs, descs.data(), sizeof(SolveDev) * n, cudaMemcpyHostToDevice, b->stream)) !=
      cudaSuccess)
    return bail(cuda_fail(e, "cudaMemcpyAsync(batch descs)"));
  for (int r = 0; r < 3; ++r) {
    b->d_int[r] = (TileRef*)(b->arena + oI[r]);
    b->d_ring[r] = (TileRef*)(b->arena + oR[r]);
    b->n_int[r] = (int)ti[r].size();
    b->n_ring[r] = (int)tr[r].size();

    if ((e = cudaMemcpyAsync(b->d_int[r], ti[r].data(), sizeof(TileRef) * ti[r].size(), cudaMemcpyHostToDevice,
                             b->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b->d_ring[r], tr[r].data(), sizeof(TileRef) * tr[r].size(), cudaMemcpyHostToDevice,
                             b->stream)) != cudaSuccess)
      return bail(cuda_fail(e, "cudaMemcpyAsync(batch tiles)"));
  }
  if ((e = cudaMallocHost(&b->h_ctl, sizeof(SolveCtl) * n)) != cudaSuccess)
    return bail(cuda_fail(e, "cudaMallocHost(batch)"));
  // Work queued on the handles' own streams comes first.
  for (int i = 0; i < n; ++i)
    if ((e = cudaStreamSynchronize(handles[i]->stream)) != cudaSuccess) return bail(cuda_fail(e, "sync"));
  b->start_steps.assign(n, 0);
  for (int i = 0; i < n; ++i)
    if ((e = cudaMemcpyAsync(&b->h_ctl[i], handles[i]->d_ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost,
                             b->stream)) != cudaSuccess)
      return bail(cuda_fail(e, "cudaMemcpyAsync(batch ctl)"));
  if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess) return bail(cuda_fail(e, "sync(batch)"));
  for (int i = 0; i < n; ++i) b->start_steps[i] = b->h_ctl[i].steps;
  *out = b;
  return CBNS_OK;
}

cbns_status cbns_batch_set_config(cbns_batch* b, const cbns_launch_config* cfg) {
  if (!b || !cfg) return fail(CBNS_ERR_INVALID_ARG, "cbns_batch_set_config: null argument");
  if (cfg->tile_rows != 2 && cfg->tile_rows != 4 && cfg->tile_rows != 8)
    return fail(CBNS_ERR_INVALID_ARG, "cbns_batch_set_config: tile_rows must be 2, 4 or 8");
  if (cfg->ctas_per_sm < 0 || cfg->ctas_per_sm > 64)
    return fail(CBNS_ERR_INVALID_ARG, "cbns_batch_set_config: ctas_per_sm must be in [0, 64]");
  b->cfg.tile_rows = cfg->tile_rows;
  b->ctas_per_sm = cfg->ctas_per_sm;
  b->cfg.max_ctas = cfg->ctas_per_sm * b->sm_count;
  return CBNS_OK;
}

cbns_status cbns_batch_get_config(cbns_batch* b, cbns_launch_config* cfg) {
  if (!b || !cfg) return fail(CBNS_ERR_INVALID_ARG, "cbns_batch_get_config: null argument");
  cfg->tile_rows = b->cfg.tile_rows;
  cfg->ctas_per_sm = b->ctas_per_sm;
  return CBNS_OK;
}

void* cbns_batch_stream(cbns_batch* b) { return b ? (void*)b->stream : nullptr; }

cbns_status cbns_batch_run(cbns_batch* b, uint32_t nsteps, uint32_t* steps_out) {
  if (!b) return fail(CBNS_ERR_INVALID_ARG, "cbns_batch_run: null batch");
  CBNS_CUDA(cudaSetDevice(b->device));
  cbns_status st = batch_graph(b);
  if (st != CBNS_OK) return st;
  for (uint32_t k = 0; k < nsteps; ++k) CBNS_CUDA(cudaGraphLaunch(b->graph, b->stream));
  const int n = (int)b->handles.size();
  for (int i = 0; i < n; ++i)
    CBNS_CUDA(cudaMemcpyAsync(&b->h_ctl[i], b->handles[i]->d_ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost,
                              b->stream));
  CBNS_CUDA(cudaStreamSynchronize(b->stream));
  int bits = 0;
  for (int i = 0; i < n; ++i) {
    if (steps_out) steps_out[i] = b->h_ctl[i].steps - b->start_steps[i];
    bits |= b->h_ctl[i].status;
  }
  if (bits) return ctl_fail(bits, "cbns_batch_run (a solve of the batch)");
  return CBNS_OK;
}

cbns_status cbns_batch_autotune(cbns_batch* b, int reps, double* ms_out, int cap, int* ncand) {
  if (!b || reps < 1) return fail(CBNS_ERR_INVALID_ARG, "cbns_batch_autotune: bad arguments");
  CBNS_CUDA(cudaSetDevice(b->device));
  const int n = (int)b->handles.size();
  // Snapshot every solve's whole device arena so the timing steps leave no trace.
  std::vector<char*> snap(n, nullptr);
  auto release = [&]() {
    for (char* p : snap)
      if (p) cudaFree(p);
  };
  for (int i = 0; i < n; ++i) {
    cudaError_t e = cudaMalloc(&snap[i], b->handles[i]->arena_bytes);
    if (e != cudaSuccess) {
      release();
      return cuda_fail(e, "cudaMalloc(autotune snapshot)");
    }
    e = cudaMemcpyAsync(snap[i], b->handles[i]->arena, b->handles[i]->arena_bytes, cudaMemcpyDeviceToDevice,
                        b->stream);
    if (e != cudaSuccess) {
      release();
      return cuda_fail(e, "cudaMemcpyAsync(autotune snapshot)");
    }
  }
  const int cps_options[4] = {0, 2, 4, 8};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 1e300;
  cbns_launch_config best_cfg{b->cfg.tile_rows, b->ctas_per_sm};
  int k = 0;
  cbns_status st = CBNS_OK;
  for (int r = 0; r < 3 && st == CBNS_OK; ++r)
    for (int c = 0; c < 4 && st == CBNS_OK; ++c) {
      cbns_launch_config cand{kRowsOptions[r], cps_options[c]};
      cbns_batch_set_config(b, &cand);
      if ((st = batch_graph(b)) != CBNS_OK) break;
      cudaGraphLaunch(b->graph, b->stream);  // warm-up
      cudaEventRecord(e0, b->stream);
      for (int q = 0; q < reps; ++q) cudaGraphLaunch(b->graph, b->stream);
      cudaEventRecord(e1, b->stream);
      cudaError_t e = cudaEventSynchronize(e1);
      if (e != cudaSuccess) {
        st = cuda_fail(e, "autotune step");
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      double per = ms / reps;
      if (ms_out && k < cap) ms_out[k] = per;
      ++k;
      if (per < best) {
        best = per;
        best_cfg = cand;
      }
      // Restore the state before the next candidate.
      for (int i = 0; i < n; ++i)
        cudaMemcpyAsync(b->handles[i]->arena, snap[i], b->handles[i]->arena_bytes, cudaMemcpyDeviceToDevice,
                        b->stream);
    }
  cudaError_t e = cudaStreamSynchronize(b->stream);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  release();
  if (st != CBNS_OK) return st;
  if (e != cudaSuccess) return cuda_fail(e, "autotune restore");
  cbns_batch_set_config(b, &best_cfg);
  if (ncand) *ncand = k;
  return CBNS_OK;
}

cbns_status cbns_footprint(uint32_t IM, uint32_t JM, uint32_t KM, int precision, uint64_t* bytes) {
  if (!bytes) return fail(CBNS_ERR_INVALID_ARG, "cbns_footprint: null output");
  if (IM < (uint32_t)NG || JM < (uint32_t)NG || KM < (uint32_t)NG || !block_extents_ok(IM, JM, KM))
    return fail(CBNS_ERR_BAD_DIMS, "cbns_footprint: every extent must be in [4, " + std::to_string(kMaxExtent) + "]");
  SolveDev s{};
  set_extents(s, IM, JM, KM);
  const bool mixed = precision == CBNS_FP32_MIXED;
  ArenaLayout L = arena_layout(s, precision, tile_count(IM, JM, KM), ring_tile_count(s.rx, s.ry, s.rz, mixed),
                               tile_count(s.nx, s.ny, s.nz), kDiagParts);
  *bytes = L.total;
  return CBNS_OK;
}

cbns_status cbns_get_info(cbns_handle* h, uint32_t dims[3], uint64_t* device_bytes, int* precision) {
  if (!h) return fail(CBNS_ERR_INVALID_ARG, "cbns_get_info: null handle");
  if (dims) {
    dims[0] = h->IM;
    dims[1] = h->JM;
    dims[2] = h->KM;
  }
  if (device_bytes) *device_bytes = h->arena_bytes;
  if (precision) *precision = h->precision;
  return CBNS_OK;
}

}  // extern "C"

namespace cbns {
cbns_status enter(cbns_handle* h, const char* fn) { return check_handle(h, fn); }

cbns_status cuda_error(cudaError_t e, const char* what) { return cuda_fail(e, what); }

// The AoS state in h->d_stage becomes the solve's state at time t: transposed
// into Q (SoA), then the start-up kernel fills ghosts, primitives, Q_p and mu
// (src/cbns3d.cpp:149-153), and the control block restarts at t.
cbns_status adopt_staged(cbns_handle* h, double t) {
  const SolveDev& s = h->desc;
  CBNS_CUDA(launch_layout(h->d_desc, 0, h->d_stage, s.Q, true, s.V, h->stream, h->pf()));
  CBNS_CUDA(launch_prepare(h->d_desc, h->d_tiles_pad, h->n_pad, h->stream, h->pf()));
  std::memset(h->h_ctl, 0, sizeof(SolveCtl));
  h->h_ctl->t_cur = t;
  h->h_ctl->t_end = h->params.t_end;
  h->h_ctl->active = 1;
  CBNS_CUDA(cudaMemcpyAsync(h->d_ctl, h->h_ctl, sizeof(SolveCtl), cudaMemcpyHostToDevice, h->stream));
  CBNS_CUDA(cudaStreamSynchronize(h->stream));
  return CBNS_OK;
}

// Q in the reference's AoS layout in h->d_stage, enqueued on h->stream.
cbns_status stage_state(cbns_handle* h) {
  CBNS_CUDA(launch_layout(h->d_desc, 0, h->desc.Q, h->d_stage, false, h->desc.V, h->stream, h->pf()));
  return CBNS_OK;
}
}  // namespace cbns
