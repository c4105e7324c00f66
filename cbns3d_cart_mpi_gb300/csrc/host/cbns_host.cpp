// cbns_host.cpp — host-side pieces of the solver kept on the CPU (include/cbns_host.h).
#include "../../../include/cbns_host.h"
#include "../cbns_modes.h"

#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <new>
#include <sstream>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

namespace {

constexpr uint32_t NEQ = CBNS_NEQ;
constexpr uint32_t NG = CBNS_NG;
constexpr double PI = 3.14159265358979323846;  // include/constants.h:19

inline size_t pidx(uint32_t IM_G, uint32_t JM_G, long i, long j, long k) {
  return (size_t)(NG + i) + (size_t)IM_G * ((size_t)(NG + j) + (size_t)JM_G * (size_t)(NG + k));
}

// ---------------------------------------------------------------------------
// VTK text.  The reference prints every value with printf("%e ", x)
// (src/Block3d.cpp:420): 7 significant digits, correctly rounded.  At 256^3 a
// .vtr file holds 84 million of them, ~20 s of snprintf on one core, so the
// writer formats the numbers itself and spreads them over the host cores.

// 10^k for k in [-300, 300], each correctly rounded (strtod of "1eK").
struct DecimalPowers {
  double v[601];
  DecimalPowers() {
    char b[16];
    for (int k = -300; k <= 300; k++) {
      std::snprintf(b, sizeof b, "1e%d", k);
      v[k + 300] = std::strtod(b, nullptr);
    }
  }
  double operator()(int k) const { return v[k + 300]; }
};
const DecimalPowers& decimal_powers() {
  static const DecimalPowers t;
  return t;
}

// The text of printf("%e ", x) into out (at most 24 bytes); returns its length.
// y = |x| * 10^(6-e) (e the decimal exponent) carries the 7 digits in its integer
// part; one correctly rounded power and one product leave y within 2.3e-16
// relative, 2.3e-9 absolute below 1e7, of the exact value.  So y's rounding to
// an integer is the exact one whenever its fraction lies farther than 1e-6 from
// one half; otherwise (a tie or near-tie), and for zero, subnormal, very large
// or non-finite x, the text comes from snprintf itself.
inline int put_e(char* out, double x) {
  const double a = std::fabs(x);
  if (!(a > 1e-290 && a < 1e290)) return std::snprintf(out, 24, "%e ", x);
  const DecimalPowers& P = decimal_powers();
  int e2;
  std::frexp(a, &e2);  // 2^(e2-1) <= a < 2^e2
  // floor((e2-1) log10 2) is the decimal exponent of a or one below it
  int e10 = (int)std::floor((e2 - 1) * 0.30102999566398120);
  double y = a * P(6 - e10);
  if (y >= 1e7) {
    e10++;
    y = a * P(6 - e10);
  }
  const double r = std::floor(y), f = y - r;
  if (std::fabs(f - 0.5) < 1e-6) return std::snprintf(out, 24, "%e ", x);
  uint32_t d = (uint32_t)r + (f > 0.5 ? 1u : 0u);
  if (d == 10000000u) {  // 9.9999995... rounds up to the next decade
    d = 1000000u;
    e10++;
  }
  if (d < 1000000u || d > 9999999u) return std::snprintf(out, 24, "%e ", x);
  char* o = out;
  if (std::signbit(x)) *o++ = '-';
  o[0] = (char)('0' + d / 1000000u);
  o[1] = '.';
  uint32_t m = d % 1000000u;
  for (int i = 7; i >= 2; i--) {
    o[i] = (char)('0' + m % 10u);
    m /= 10u;
  }
  o[8] = 'e';
  o += 9;
  int ex = e10 < 0 ? -e10 : e10;
  *o++ = e10 < 0 ? '-' : '+';
  if (ex >= 100) {
    *o++ = (char)('0' + ex / 100);
    ex %= 100;
  }
  *o++ = (char)('0' + ex / 10);
  *o++ = (char)('0' + ex % 10);
  *o++ = ' ';
  return (int)(o - out);
}

constexpr char kLineBreak[] = "\n        ";  // after every fifth value (src/Block3d.cpp:421)
// A value is at most 15 characters ("-1.234567e+308 "), a line break 9 per five
// values; put_e's snprintf may be told of 24 bytes, hence the slack.
constexpr size_t kCharsPerValue = 17;
constexpr size_t kPutSlack = 32;

// Values c0..c1-1 (i fastest) of one cell-data array in the reference's line
// layout; c0 is a multiple of 5, so the text starts a line.  Returns the length.
size_t format_cells(char* out, const double* arr, uint32_t IM, uint32_t JM, uint32_t IM_G, uint32_t JM_G,
                    uint64_t c0, uint64_t c1) {
  char* o = out;
  uint64_t i = c0 % IM, j = (c0 / IM) % JM, k = c0 / ((uint64_t)IM * JM);
  for (uint64_t c = c0; c < c1; c++) {
    o += put_e(o, arr[pidx(IM_G, JM_G, (long)i, (long)j, (long)k)]);
    if (c % 5 == 4) {
      std::memcpy(o, kLineBreak, sizeof kLineBreak - 1);
      o += sizeof kLineBreak - 1;
    }
    if (++i == IM) {
      i = 0;
      if (++j == JM) {
        j = 0;
        k++;
      }
    }
  }
  return (size_t)(o - out);
}

// Host threads for the text: CBNS_HOST_THREADS if set, else every core.
unsigned text_threads() {
  if (const char* e = std::getenv("CBNS_HOST_THREADS")) {
    long n = std::strtol(e, nullptr, 10);
    if (n >= 1) return (unsigned)std::min(n, 1024L);
  }
  unsigned n = std::thread::hardware_concurrency();
  return n ? n : 1;
}

// The <CellData> arrays of a .vtr file.  Worker threads format chunks of
// kChunkValues values (a multiple of 5) into a ring of kRing buffers; the calling
// thread writes the chunks in order, so the file is the serial writer's byte for
// byte.  A worker takes chunk c only once chunk c - kRing has been written.
bool write_cell_data(FILE* fh, const char* const names[5], const double* const arrs[5], uint32_t IM,
                     uint32_t JM, uint32_t KM) {
  constexpr uint64_t kChunkValues = 5 * 3276;
  const uint32_t IM_G = IM + 2 * NG, JM_G = JM + 2 * NG;
  const uint64_t n = (uint64_t)IM * JM * KM;
  const uint64_t per_field = (n + kChunkValues - 1) / kChunkValues, total = 5 * per_field;
  const unsigned want = (unsigned)std::min<uint64_t>(text_threads(), std::max<uint64_t>(total, 1));
  const size_t kRing = 2 * (size_t)want + 2;
  std::vector<std::vector<char>> ring(kRing, std::vector<char>(kChunkValues * kCharsPerValue + kPutSlack));
  std::vector<size_t> len(kRing, 0);
  std::vector<char> ready(kRing, 0);
  std::mutex mu;
  std::condition_variable cv_take, cv_ready;
  uint64_t next = 0, written = 0;
  auto format = [&](uint64_t c) {
    const uint64_t f = c / per_field, c0 = (c % per_field) * kChunkValues, c1 = std::min(c0 + kChunkValues, n);
    return format_cells(ring[c % kRing].data(), arrs[f], IM, JM, IM_G, JM_G, c0, c1);
  };
  auto worker = [&] {
    for (;;) {
      uint64_t c;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_take.wait(lk, [&] { return next >= total || next < written + kRing; });
        if (next >= total) return;
        c = next++;
      }
      const size_t l = format(c);
      {
        std::lock_guard<std::mutex> lk(mu);
        len[c % kRing] = l;
        ready[c % kRing] = 1;
      }
      cv_ready.notify_all();
    }
  };
  std::vector<std::thread> pool;
  try {
    for (unsigned t = 0; t < want && total > 0; t++) pool.emplace_back(worker);
  } catch (const std::system_error&) {
    // fewer threads than asked: the ones started (or, with none, this thread) do the work
  }
  bool ok = true;
  for (int f = 0; f < 5; f++) {
    ok = std::fprintf(fh, "      <DataArray type=\"Float64\" Name=\"%s\" format=\"ascii\">\n        ", names[f]) > 0 && ok;
    for (uint64_t q = 0; q < per_field; q++) {
      const uint64_t c = (uint64_t)f * per_field + q;
      const size_t s = c % kRing;
      if (pool.empty()) {
        len[s] = format(c);
      } else {
        std::unique_lock<std::mutex> lk(mu);
        cv_ready.wait(lk, [&] { return ready[s] != 0; });
      }
      ok = std::fwrite(ring[s].data(), 1, len[s], fh) == len[s] && ok;
      {
        std::lock_guard<std::mutex> lk(mu);
        ready[s] = 0;
        written = c + 1;
      }
      cv_take.notify_all();
    }
    if (n % 5 != 0) ok = std::fputc('\n', fh) != EOF && ok;
    ok = std::fprintf(fh, "      </DataArray>\n") > 0 && ok;
  }
  for (std::thread& t : pool) t.join();
  return ok;
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
  const char* const names[5] = {"rho", "u", "v", "w", "p"};
  const double* const arrs[5] = {rho, u, v, w, p};
  bool ok;
  try {
    ok = write_cell_data(fh, names, arrs, IM, JM, KM);
  } catch (const std::bad_alloc&) {
    ok = false;
  }
  std::fprintf(fh, "    </CellData>\n");
  std::fprintf(fh, "    <Coordinates>\n");
  auto coord = [&](const char* name, uint32_t n, const double* arr) {
    std::fprintf(fh, "      <DataArray type=\"Float64\" Name=\"%s\" format=\"ascii\">\n", name);
    std::fprintf(fh, "        ");
    char b[kPutSlack];
    for (uint32_t i = 0; i < n; i++) {
      std::fwrite(b, 1, (size_t)put_e(b, arr[i]), fh);
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
  ok = (std::fclose(fh) == 0) && ok;
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
