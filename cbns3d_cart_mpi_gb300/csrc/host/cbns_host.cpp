// cbns_host.cpp — host-side pieces of the solver kept on the CPU (include/cbns_host.h).
#include "../../../include/cbns_host.h"
#include "../cbns_modes.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace {

constexpr uint32_t NEQ = CBNS_NEQ;
constexpr uint32_t NG = CBNS_NG;
constexpr double PI = 3.14159265358979323846;  // include/constants.h:19

inline size_t pidx(uint32_t IM_G, uint32_t JM_G, long i, long j, long k) {
  return (size_t)(NG + i) + (size_t)IM_G * ((size_t)(NG + j) + (size_t)JM_G * (size_t)(NG + k));
}

// Cell-centred primitive fields of the Taylor-Green vortex
// (src/Block3d.cpp:241-269), then conserved variables (src/Block3d.cpp:277-298).
void tgv_state(const cbns_params* p, uint32_t IM, uint32_t JM, uint32_t KM, uint32_t i0, uint32_t j0,
               uint32_t k0, std::vector<double>& u, std::vector<double>& v, std::vector<double>& w,
               std::vector<double>& pr, std::vector<double>& rho) {
  std::vector<double> x(IM + 1), y(JM + 1), z(KM + 1);
  cbns_host_gen_mesh(p, IM, JM, KM, i0, j0, k0, x.data(), y.data(), z.data());
  const double dx = 2.0 * PI / p->IM, dy = 2.0 * PI / p->JM, dz = 2.0 * PI / p->KM;
  const size_t n = (size_t)IM * JM * KM;
  u.assign(n, 0.0);
  v.assign(n, 0.0);
  w.assign(n, 0.0);
  pr.assign(n, 0.0);
  rho.assign(n, 0.0);
  for (uint32_t k = 0; k < KM; k++) {
    double zl = z[k] + 0.5 * dz;
    for (uint32_t j = 0; j < JM; j++) {
      double yl = y[j] + 0.5 * dy;
      for (uint32_t i = 0; i < IM; i++) {
        double xl = x[i] + 0.5 * dx;
        size_t c = i + (size_t)IM * (j + (size_t)JM * k);
        u[c] = std::sin(xl) * std::cos(yl) * std::cos(zl);
        v[c] = -std::cos(xl) * std::sin(yl) * std::cos(zl);
        w[c] = 0.0;
        pr[c] = p->p_inf + (std::cos(2.0 * xl) + std::cos(2.0 * yl)) * (std::cos(2.0 * zl) + 2.0) / 16.0;
        rho[c] = p->gM2 * pr[c];
      }
    }
  }
}

void conservative(const cbns_params* p, uint32_t IM, uint32_t JM, uint32_t KM, const std::vector<double>& u,
                  const std::vector<double>& v, const std::vector<double>& w, const std::vector<double>& pr,
                  const std::vector<double>& rho, double* Q) {
  const uint32_t IM_G = IM + 2 * NG, JM_G = JM + 2 * NG, KM_G = KM + 2 * NG;
  std::memset(Q, 0, sizeof(double) * NEQ * IM_G * JM_G * KM_G);
  for (uint32_t k = 0; k < KM; k++)
    for (uint32_t j = 0; j < JM; j++)
      for (uint32_t i = 0; i < IM; i++) {
        size_t c = i + (size_t)IM * (j + (size_t)JM * k);
        size_t q = NEQ * pidx(IM_G, JM_G, i, j, k);
        double rr = rho[c], uu = u[c], vv = v[c], ww = w[c], pp = pr[c];
        Q[q] = rr;
        Q[q + 1] = rr * uu;
        Q[q + 2] = rr * vv;
        Q[q + 3] = rr * ww;
        Q[q + 4] = pp / p->gam1 + 0.5 * rr * (uu * uu + vv * vv + ww * ww);
      }
}

// src/read_input.cpp:78-90 (a host-only copy; the GPU library exports the same
// computation as cbns_params_derive).
void derive(cbns_params* p) {
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
}

}  // namespace

extern "C" {

cbns_status cbns_host_read_input(const char* path, cbns_params* out) {
  if (!path || !out) return CBNS_ERR_INVALID_ARG;
  std::ifstream fh(path);
  if (!fh) return CBNS_ERR_IO;
  cbns_params p;
  std::memset(&p, 0, sizeof p);
  std::string fname;
  unsigned long IM, JM, KM, nstep, ckf, nout;
  long restart;
  // src/read_input.cpp:24-72, in order.
  if (!(fh >> fname >> p.CFL >> p.t_cur >> p.t_end >> p.Pr >> p.gamma >> p.Mach >> p.Re >> p.T_inf >> p.L >> IM >>
        JM >> KM >> nstep >> ckf >> nout >> restart))
    return CBNS_ERR_FORMAT;
  if (fname.size() >= sizeof p.checkpoint_fname) return CBNS_ERR_FORMAT;
  std::memcpy(p.checkpoint_fname, fname.c_str(), fname.size() + 1);
  p.IM = (uint32_t)IM;
  p.JM = (uint32_t)JM;
  p.KM = (uint32_t)KM;
  p.nstep_max = (uint32_t)nstep;
  p.checkpoint_freq = (uint32_t)ckf;
  p.num_output = (uint32_t)nout;
  p.is_restart = restart != 0;
  derive(&p);
  *out = p;
  return CBNS_OK;
}

cbns_status cbns_host_gen_mesh(const cbns_params* p, uint32_t IM, uint32_t JM, uint32_t KM, uint32_t i0,
                               uint32_t j0, uint32_t k0, double* x, double* y, double* z) {
  if (!p || !x || !y || !z) return CBNS_ERR_INVALID_ARG;
  double tmp = 2.0 * PI;
  const double dx = tmp / p->IM, dy = tmp / p->JM, dz = tmp / p->KM;
  tmp /= 2.0;
  for (uint32_t i = 0; i < IM + 1; i++) x[i] = (i0 + i) * dx - tmp;
  for (uint32_t j = 0; j < JM + 1; j++) y[j] = (j0 + j) * dy - tmp;
  for (uint32_t k = 0; k < KM + 1; k++) z[k] = (k0 + k) * dz - tmp;
  return CBNS_OK;
}

cbns_status cbns_host_initial_condition(const cbns_params* p, uint32_t IM, uint32_t JM, uint32_t KM, uint32_t i0,
                                        uint32_t j0, uint32_t k0, double* Q) {
  if (!p || !Q) return CBNS_ERR_INVALID_ARG;
  if (IM == 0 || JM == 0 || KM == 0) return CBNS_ERR_BAD_DIMS;
  std::vector<double> u, v, w, pr, rho;
  tgv_state(p, IM, JM, KM, i0, j0, k0, u, v, w, pr, rho);
  conservative(p, IM, JM, KM, u, v, w, pr, rho, Q);
  return CBNS_OK;
}

cbns_status cbns_host_initial_condition_perturbed(const cbns_params* p, uint32_t IM, uint32_t JM, uint32_t KM,
                                                  uint64_t seed, double amp, int nmodes, int kmax, double* Q) {
  if (!p || !Q || nmodes < 0 || kmax < 1) return CBNS_ERR_INVALID_ARG;
  if (IM == 0 || JM == 0 || KM == 0) return CBNS_ERR_BAD_DIMS;
  std::vector<double> u, v, w, pr, rho;
  tgv_state(p, IM, JM, KM, 0, 0, 0, u, v, w, pr, rho);
  const std::vector<cbns::PerturbMode> modes = cbns::draw_modes(seed, amp, nmodes, kmax);
  std::vector<double> x(IM + 1), y(JM + 1), z(KM + 1);
  cbns_host_gen_mesh(p, IM, JM, KM, 0, 0, 0, x.data(), y.data(), z.data());
  const double dx = 2.0 * PI / p->IM, dy = 2.0 * PI / p->JM, dz = 2.0 * PI / p->KM;
  for (uint32_t k = 0; k < KM; k++)
    for (uint32_t j = 0; j < JM; j++)
      for (uint32_t i = 0; i < IM; i++) {
        double xc[3] = {x[i] + 0.5 * dx, y[j] + 0.5 * dy, z[k] + 0.5 * dz};
        size_t c = i + (size_t)IM * (j + (size_t)JM * k);
        for (const cbns::PerturbMode& m : modes) {
          double ph = m.k[0] * xc[0] + m.k[1] * xc[1] + m.k[2] * xc[2] + m.phase;
          double cph = std::cos(ph);
          u[c] += m.a[0] * cph;
          v[c] += m.a[1] * cph;
          w[c] += m.a[2] * cph;
        }
      }
  conservative(p, IM, JM, KM, u, v, w, pr, rho, Q);
  return CBNS_OK;
}

cbns_status cbns_host_output_bin(const char* fname, double t_cur, uint32_t IM, uint32_t JM, uint32_t KM,
                                 const double* Q) {
  if (!fname || !Q) return CBNS_ERR_INVALID_ARG;
  FILE* fh = std::fopen(fname, "wb");
  if (!fh) return CBNS_ERR_IO;
  uint32_t dims[3] = {IM + 2 * NG, JM + 2 * NG, KM + 2 * NG};
  size_t n = (size_t)NEQ * dims[0] * dims[1] * dims[2];
  bool ok = std::fwrite(&t_cur, sizeof(double), 1, fh) == 1 && std::fwrite(dims, sizeof(uint32_t), 3, fh) == 3 &&
            std::fwrite(Q, sizeof(double), n, fh) == n;
  ok = (std::fclose(fh) == 0) && ok;
  return ok ? CBNS_OK : CBNS_ERR_IO;
}

cbns_status cbns_host_read_bin(const char* fname, uint32_t IM, uint32_t JM, uint32_t KM, double* Q, double* t_cur) {
  if (!fname || !Q) return CBNS_ERR_INVALID_ARG;
  FILE* fh = std::fopen(fname, "rb");
  if (!fh) return CBNS_ERR_IO;
  double t = 0.0;
  uint32_t dims[3];
  const uint32_t want[3] = {IM + 2 * NG, JM + 2 * NG, KM + 2 * NG};
  cbns_status st = CBNS_OK;
  if (std::fread(&t, sizeof(double), 1, fh) != 1 || std::fread(dims, sizeof(uint32_t), 3, fh) != 3) {
    st = CBNS_ERR_FORMAT;
  } else if (dims[0] != want[0] || dims[1] != want[1] || dims[2] != want[2]) {
    st = CBNS_ERR_FORMAT;  // "The dimensions do not match." (src/Block3d.cpp:334-338)
  } else {
    size_t n = (size_t)NEQ * want[0] * want[1] * want[2];
    if (std::fread(Q, sizeof(double), n, fh) != n) st = CBNS_ERR_FORMAT;
  }
  std::fclose(fh);
  if (st == CBNS_OK && t_cur) *t_cur = t;
  return st;
}

cbns_status cbns_host_output_vtk_xml(const char* dir, const char* fname, int rank, uint32_t num_blocks,
                                     uint32_t IM, uint32_t JM, uint32_t KM, const double* x, const double* y,
                                     const double* z, const double* rho, const double* u, const double* v,
                                     const double* w, const double* p) {
  if (!dir || !fname || !x || !y || !z || !rho || !u || !v || !w || !p) return CBNS_ERR_INVALID_ARG;
  const uint32_t IM_G = IM + 2 * NG, JM_G = JM + 2 * NG;
  char rk[16];
  std::snprintf(rk, sizeof rk, "%03d", rank);
  std::string base = std::string(dir) + "/" + fname;
  FILE* fh = std::fopen((base + rk + ".vtr").c_str(), "w");
  if (!fh) return CBNS_ERR_IO;
  // Block3d::output_vtr (src/Block3d.cpp:396-469).
  std::fprintf(fh, "<?xml version=\"1.0\"?>\n");
  std::fprintf(fh, "<VTKFile type=\"RectilinearGrid\" version=\"1.0\" byte_order=\"LittleEndian\">\n");
  std::fprintf(fh, "  <RectilinearGrid WholeExtent=\"0 %d 0 %d 0 %d\">\n", (int)IM, (int)JM, (int)KM);
  std::fprintf(fh, "    <Piece Extent=\"0 %d 0 %d 0 %d\">\n", (int)IM, (int)JM, (int)KM);
  std::fprintf(fh, "    <CellData>\n");
  auto cell_data = [&](const char* name, const double* arr) {
    std::fprintf(fh, "      <DataArray type=\"Float64\" Name=\"%s\" format=\"ascii\">\n", name);
    std::fprintf(fh, "        ");
    uint32_t cnt = 0;
    for (uint32_t k = 0; k < KM; k++)
      for (uint32_t j = 0; j < JM; j++)
        for (uint32_t i = 0; i < IM; i++) {
          std::fprintf(fh, "%e ", arr[pidx(IM_G, JM_G, i, j, k)]);
          if (4 == cnt++ % 5) std::fprintf(fh, "\n        ");
        }
    if (0 != cnt % 5) std::fprintf(fh, "\n");
    std::fprintf(fh, "      </DataArray>\n");
  };
  cell_data("rho", rho);
  cell_data("u", u);
  cell_data("v", v);
  cell_data("w", w);
  cell_data("p", p);
  std::fprintf(fh, "    </CellData>\n");
  std::fprintf(fh, "    <Coordinates>\n");
  auto coord = [&](const char* name, uint32_t n, const double* arr) {
    std::fprintf(fh, "      <DataArray type=\"Float64\" Name=\"%s\" format=\"ascii\">\n", name);
    std::fprintf(fh, "        ");
    for (uint32_t i = 0; i < n; i++) {
      std::fprintf(fh, "%e ", arr[i]);
      if (4 == i % 5) std::fprintf(fh, "\n        ");
    }
    if (0 != n % 5) std::fprintf(fh, "\n");
    std::fprintf(fh, "      </DataArray>\n");
  };
  coord("x", IM + 1, x);
  coord("y", JM + 1, y);
  coord("z", KM + 1, z);
  std::fprintf(fh, "    </Coordinates>\n");
  std::fprintf(fh, "    </Piece>\n");
  std::fprintf(fh, "  </RectilinearGrid>\n");
  std::fprintf(fh, "</VTKFile>\n");
  bool ok = std::fclose(fh) == 0;
  if (!ok) return CBNS_ERR_IO;
  if (rank == 0) {
    // Block3d::output_vtm (src/Block3d.cpp:471-500).
    FILE* fm = std::fopen((base + ".vtm").c_str(), "w");
    if (!fm) return CBNS_ERR_IO;
    std::fprintf(fm, "<?xml version=\"1.0\"?>\n");
    std::fprintf(fm, "<VTKFile type=\"vtkMultiBlockDataSet\" version=\"1.0\" byte_order=\"LittleEndian\">\n");
    std::fprintf(fm, "  <vtkMultiBlockDataSet>\n");
    for (uint32_t b = 0; b < num_blocks; b++)
      std::fprintf(fm, "    <DataSet index=\"%d\" file=\"%s%.3i.vtr\"/>\n", (int)b, fname, (int)b);
    std::fprintf(fm, "  </vtkMultiBlockDataSet>\n");
    std::fprintf(fm, "</VTKFile>\n");
    if (std::fclose(fm) != 0) return CBNS_ERR_IO;
  }
  return CBNS_OK;
}

}  // extern "C"
