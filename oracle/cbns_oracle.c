/*
 * cbns_oracle.c — CPU restatement of the reference solver's hot path.
 *
 * TEST INFRASTRUCTURE.  Only the tests, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load this file's library, and only as the checker or as the
 * timed CPU baseline; the product path never calls it.
 *
 * It restates, in plain C and in the reference's own operation order, the
 * FP64 arithmetic of chenbei102/cbns3d_cart_mpi (each function cites the file:line
 * it follows), so that on the same input it reproduces the reference's binary64
 * results bit for bit.  That claim is pinned: tests compare this port against
 * the reference itself, compiled unmodified (oracle/build.py), and against
 * the golden states made from it (tests/golden/).  Build with
 * -ffp-contract=off and without -ffast-math so no multiply-add is fused.
 *
 * The periodic halo exchange of the one-rank periodic Cartesian topology
 * (src/boundary_condition.cpp) is restated as the copies it amounts to.  Loops
 * over k run on OpenMP threads; every cell's arithmetic is independent of the
 * thread count, and calc_dt's maximum is order-independent, so results do not
 * depend on it.
 *
 * Project-defined additions (absent from the reference): oracle_diagnostics
 * (kinetic energy and enstrophy), and the perturbed initial states used by the
 * ensemble tests (oracle_set_Q takes any state).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/cbns_gpu.h"

#define NEQ 5
#define NG 4
#define NGV 2

typedef struct oracle_block {
  cbns_params sp;
  long IM, JM, KM, IM_G, JM_G, KM_G, IM_GV, JM_GV, KM_GV;
  double dx, dy, dz;
  double *x, *y, *z;
  double *u, *v, *w, *rho, *T, *p, *mu;
  double *Q, *Q_p;
  double *Ep, *Fp, *Gp;
  double *u_x, *v_x, *w_x, *u_y, *v_y, *w_y, *u_z, *v_z, *w_z, *T_x, *T_y, *T_z;
  double *tau_xx, *tau_yy, *tau_zz, *tau_xy, *tau_xz, *tau_yz, *q_x, *q_y, *q_z;
  double *Ev, *Fv, *Gv, *dfv;
} oracle_block;

/* Index maps of include/Block3d.h:169-199 (64-bit here; identical where the
 * reference's 32-bit size_type does not overflow). */
static inline long idx(const oracle_block* b, long i, long j, long k) {
  return (NG + i) + b->IM_G * ((NG + j) + b->JM_G * (NG + k));
}
static inline long idx_ux(const oracle_block* b, long i, long j, long k) {
  return (NGV + i) + b->IM_GV * ((NGV + j) + b->JM_GV * (NGV + k));
}
static inline long idx_Q(const oracle_block* b, long n, long i, long j, long k) {
  return n + NEQ * idx(b, i, j, k);
}
static inline long idx_Ep(const oracle_block* b, long n, long i, long j, long k) {
  return n + NEQ * (i + (b->IM + 1) * (j + b->JM * k));
}
static inline long idx_Fp(const oracle_block* b, long n, long i, long j, long k) {
  return n + NEQ * (i + b->IM * (j + (b->JM + 1) * k));
}
static inline long idx_Gp(const oracle_block* b, long n, long i, long j, long k) {
  return n + NEQ * (i + b->IM * (j + b->JM * k));
}
static inline long idx_Ev(const oracle_block* b, long n, long i, long j, long k) {
  return n + (NEQ - 1) * idx_ux(b, i, j, k);
}
static inline long idx_dfv(const oracle_block* b, long n, long i, long j, long k) {
  return n + (NEQ - 1) * (i + b->IM * (j + b->JM * k));
}

/* src/read_input.cpp:78-90 */
void oracle_params_derive(cbns_params* p) {
  p->Mach2 = p->Mach * p->Mach;
  p->Re_inv = 1.0 / p->Re;
  p->Pr_inv = 1.0 / p->Pr;
  p->gam1 = p->gamma - 1.0;
  p->gM2 = p->gamma * p->Mach2;
  p->gam1_inv = 1.0 / p->gam1;
  p->p_inf = 1.0 / p->gM2;
  p->C_T_inf = 110.5 / p->T_inf;
  double a = 4.0 / 3.0, g = p->gamma * p->Pr_inv;
  p->C_dt_v = (a < g ? g : a) * p->Re_inv; /* std::max(a, g) */
}

static double* zalloc(long n) { return (double*)calloc((size_t)n, sizeof(double)); }

void oracle_destroy(oracle_block* b);

/* Block3d ctor + allocate_mem (src/Block3d.cpp:11-135) and gen_mesh
 * (src/Block3d.cpp:208-235) with block origin 0. */
oracle_block* oracle_create(const cbns_params* sp, long IM, long JM, long KM) {
  if (IM < NG || JM < NG || KM < NG) return NULL;
  oracle_block* b = (oracle_block*)calloc(1, sizeof(oracle_block));
  if (!b) return NULL;
  b->sp = *sp;
  b->IM = IM; b->JM = JM; b->KM = KM;
  b->IM_G = IM + 2 * NG; b->JM_G = JM + 2 * NG; b->KM_G = KM + 2 * NG;
  b->IM_GV = IM + 2 * NGV; b->JM_GV = JM + 2 * NGV; b->KM_GV = KM + 2 * NGV;
  long ng = b->IM_G * b->JM_G * b->KM_G, ngv = b->IM_GV * b->JM_GV * b->KM_GV;
  b->x = zalloc(IM + 1); b->y = zalloc(JM + 1); b->z = zalloc(KM + 1);
  b->u = zalloc(ng); b->v = zalloc(ng); b->w = zalloc(ng); b->rho = zalloc(ng);
  b->T = zalloc(ng); b->p = zalloc(ng); b->mu = zalloc(ng);
  double** g[] = {&b->u_x, &b->v_x, &b->w_x, &b->u_y, &b->v_y, &b->w_y, &b->u_z, &b->v_z,
                  &b->w_z, &b->T_x, &b->T_y, &b->T_z, &b->tau_xx, &b->tau_yy, &b->tau_zz,
                  &b->tau_xy, &b->tau_xz, &b->tau_yz, &b->q_x, &b->q_y, &b->q_z};
  for (size_t a = 0; a < sizeof g / sizeof g[0]; ++a) *g[a] = zalloc(ngv);
  b->Q = zalloc(NEQ * ng); b->Q_p = zalloc(NEQ * ng);
  b->Ev = zalloc((NEQ - 1) * ngv); b->Fv = zalloc((NEQ - 1) * ngv); b->Gv = zalloc((NEQ - 1) * ngv);
  b->dfv = zalloc((NEQ - 1) * IM * JM * KM);
  b->Ep = zalloc(NEQ * (IM + 1) * JM * KM);
  b->Fp = zalloc(NEQ * IM * (JM + 1) * KM);
  b->Gp = zalloc(NEQ * IM * JM * (KM + 1));
  if (!b->Gp || !b->Ep || !b->Q_p || !b->tau_yz || !b->dfv) {
    oracle_destroy(b);
    return NULL;
  }
  double tmp = 2.0 * 3.14159265358979323846; /* constant::PI, include/constants.h:19 */
  b->dx = tmp / sp->IM;
  b->dy = tmp / sp->JM;
  b->dz = tmp / sp->KM;
  tmp /= 2.0;
  for (long i = 0; i < IM + 1; i++) b->x[i] = (0 + i) * b->dx - tmp;
  for (long j = 0; j < JM + 1; j++) b->y[j] = (0 + j) * b->dy - tmp;
  for (long k = 0; k < KM + 1; k++) b->z[k] = (0 + k) * b->dz - tmp;
  return b;
}

void oracle_destroy(oracle_block* b) {
  if (!b) return;
  double* all[] = {b->x, b->y, b->z, b->u, b->v, b->w, b->rho, b->T, b->p, b->mu, b->Q,
                   b->Q_p, b->Ep, b->Fp, b->Gp, b->u_x, b->v_x, b->w_x, b->u_y, b->v_y,
                   b->w_y, b->u_z, b->v_z, b->w_z, b->T_x, b->T_y, b->T_z, b->tau_xx,
                   b->tau_yy, b->tau_zz, b->tau_xy, b->tau_xz, b->tau_yz, b->q_x, b->q_y,
                   b->q_z, b->Ev, b->Fv, b->Gv, b->dfv};
  for (size_t a = 0; a < sizeof all / sizeof all[0]; ++a) free(all[a]);
  free(b);
}

/* Block3d::initial_condition + calc_conservative (src/Block3d.cpp:237-300). */
void oracle_initial_condition(oracle_block* b) {
  const cbns_params* sp = &b->sp;
  for (long k = 0; k < b->KM; k++) {
    double z_l = b->z[k] + 0.5 * b->dz;
    for (long j = 0; j < b->JM; j++) {
      double y_l = b->y[j] + 0.5 * b->dy;
      for (long i = 0; i < b->IM; i++) {
        double x_l = b->x[i] + 0.5 * b->dx;
        long i1 = idx(b, i, j, k);
        b->u[i1] = sin(x_l) * cos(y_l) * cos(z_l);
        b->v[i1] = -cos(x_l) * sin(y_l) * cos(z_l);
        b->w[i1] = 0.0;
        b->p[i1] = sp->p_inf + (cos(2.0 * x_l) + cos(2.0 * y_l)) * (cos(2.0 * z_l) + 2.0) / 16.0;
        b->rho[i1] = sp->gM2 * b->p[i1];
        b->T[i1] = 1.0;
        b->mu[i1] = 1.0;
      }
    }
  }
  for (long k = 0; k < b->KM; k++)
    for (long j = 0; j < b->JM; j++)
      for (long i = 0; i < b->IM; i++) {
        long i1 = idx(b, i, j, k), i2 = idx_Q(b, 0, i, j, k);
        double rr = b->rho[i1], uu = b->u[i1], vv = b->v[i1], ww = b->w[i1], pp = b->p[i1];
        b->Q[i2] = rr;
        b->Q[i2 + 1] = rr * uu;
        b->Q[i2 + 2] = rr * vv;
        b->Q[i2 + 3] = rr * ww;
        b->Q[i2 + 4] = pp / sp->gam1 + 0.5 * rr * (uu * uu + vv * vv + ww * ww);
      }
}

/* src/boundary_condition.cpp:4-231 on one periodic rank: every neighbour is the
 * rank itself, so each ghost layer receives the opposite interior layers. The
 * x sweep covers interior j,k; the y sweep covers all i; the z sweep all i,j,
 * which fills edges and corners. */
void oracle_boundary_condition(oracle_block* b, double* Q) {
  const long IM = b->IM, JM = b->JM, KM = b->KM;
#pragma omp parallel for schedule(static)
  for (long k = 0; k < KM; k++)
    for (long j = 0; j < JM; j++)
      for (long i = 0; i < NG; i++) {
        long dl = idx_Q(b, 0, i - NG, j, k), sl = idx_Q(b, 0, IM - NG + i, j, k);
        long dr = idx_Q(b, 0, IM + i, j, k), sr = idx_Q(b, 0, i, j, k);
        for (int n = 0; n < NEQ; n++) { Q[dl + n] = Q[sl + n]; Q[dr + n] = Q[sr + n]; }
      }
#pragma omp parallel for schedule(static)
  for (long k = 0; k < KM; k++)
    for (long i = -NG; i < IM + NG; i++)
      for (long j = 0; j < NG; j++) {
        long dd = idx_Q(b, 0, i, j - NG, k), sd = idx_Q(b, 0, i, JM - NG + j, k);
        long du = idx_Q(b, 0, i, JM + j, k), su = idx_Q(b, 0, i, j, k);
        for (int n = 0; n < NEQ; n++) { Q[dd + n] = Q[sd + n]; Q[du + n] = Q[su + n]; }
      }
#pragma omp parallel for schedule(static)
  for (long j = -NG; j < JM + NG; j++)
    for (long i = -NG; i < IM + NG; i++)
      for (long k = 0; k < NG; k++) {
        long db = idx_Q(b, 0, i, j, k - NG), sb = idx_Q(b, 0, i, j, KM - NG + k);
        long df = idx_Q(b, 0, i, j, KM + k), sf = idx_Q(b, 0, i, j, k);
        for (int n = 0; n < NEQ; n++) { Q[db + n] = Q[sb + n]; Q[df + n] = Q[sf + n]; }
      }
}

/* Block3d::calc_primitive (src/Block3d.cpp:359-385), whole padded array. */
void oracle_calc_primitive(oracle_block* b, const double* Q) {
  const long n = b->IM_G * b->JM_G * b->KM_G;
  const double gam1 = b->sp.gam1, gM2 = b->sp.gM2;
#pragma omp parallel for schedule(static)
  for (long i1 = 0; i1 < n; i1++) {
    long i2 = NEQ * i1;
    double rr = Q[i2];
    double uu = Q[i2 + 1] / rr;
    double vv = Q[i2 + 2] / rr;
    double ww = Q[i2 + 3] / rr;
    double pp = gam1 * (Q[i2 + 4] - 0.5 * rr * (uu * uu + vv * vv + ww * ww));
    b->rho[i1] = rr; b->u[i1] = uu; b->v[i1] = vv; b->w[i1] = ww; b->p[i1] = pp;
    b->T[i1] = gM2 * pp / rr;
  }
}

/* Block3d::calc_dt (src/Block3d.cpp:515-553). */
double oracle_calc_dt(oracle_block* b) {
  const cbns_params* sp = &b->sp;
  const double dx = b->dx, dy = b->dy, dz = b->dz;
  double s_max = 0.0;
#pragma omp parallel
  {
    double s_loc = 0.0;
#pragma omp for schedule(static)
    for (long k = 0; k < b->KM; k++)
      for (long j = 0; j < b->JM; j++)
        for (long i = 0; i < b->IM; i++) {
          long i1 = idx(b, i, j, k);
          double rr = b->rho[i1], uu = b->u[i1], vv = b->v[i1], ww = b->w[i1], pp = b->p[i1];
          double c = sqrt(sp->gamma * pp / rr);
          double factor_v = 2.0 * b->mu[i1] * sp->C_dt_v * sqrt(uu * uu + vv * vv + ww * ww) / c / rr;
          double t1 = fabs(uu) + c / dx;
          t1 += factor_v / dx / dx;
          double t2 = fabs(vv) + c / dy;
          t2 += factor_v / dy / dy;
          double t3 = fabs(ww) + c / dz;
          t3 += factor_v / dz / dz;
          s_loc = ((s_loc < t1 + t2 + t3) ? (t1 + t2 + t3) : s_loc);
        }
#pragma omp critical
    s_max = ((s_max < s_loc) ? s_loc : s_max);
  }
  return sp->CFL / s_max;
}

/* calc_eigenvectors (src/eigenvectors_roe.cpp:32-171). */
static void eigenvectors(double gamma, double rho_L, double u_L, double v_L, double w_L,
                         double p_L, double rho_R, double u_R, double v_R, double w_R,
                         double p_R, double n_x, double n_y, double n_z, double R[5][5],
                         double L[5][5]) {
  const double gam1 = gamma - 1.0;
  double l_x = 0.0, l_y = n_z, l_z = -n_y;
  double m_x, m_y, m_z;
  double n_abs = sqrt(l_x * l_x + l_y * l_y + l_z * l_z);
  if (n_abs > 1.0e-8) {
    m_x = -n_y * n_y - n_z * n_z;
    m_y = n_x * n_y;
    m_z = n_x * n_z;
  } else {
    l_x = -n_z; l_y = 0.0; l_z = n_x;
    m_x = n_x * n_y;
    m_y = -n_x * n_x - n_z * n_z;
    m_z = n_y * n_z;
  }
  n_abs = sqrt(n_x * n_x + n_y * n_y + n_z * n_z);
  n_x /= n_abs; n_y /= n_abs; n_z /= n_abs;
  n_abs = sqrt(l_x * l_x + l_y * l_y + l_z * l_z);
  l_x /= n_abs; l_y /= n_abs; l_z /= n_abs;
  n_abs = sqrt(m_x * m_x + m_y * m_y + m_z * m_z);
  m_x /= n_abs; m_y /= n_abs; m_z /= n_abs;

  double c_L = sqrt(gamma * p_L / rho_L);
  double H_L = c_L * c_L / gam1 + 0.5 * (u_L * u_L + v_L * v_L + w_L * w_L);
  double c_R = sqrt(gamma * p_R / rho_R);
  double H_R = c_R * c_R / gam1 + 0.5 * (u_R * u_R + v_R * v_R + w_R * w_R);
  double ratio = sqrt(rho_R / rho_L);
  double uu = (u_L + ratio * u_R) / (1.0 + ratio);
  double vv = (v_L + ratio * v_R) / (1.0 + ratio);
  double ww = (w_L + ratio * w_R) / (1.0 + ratio);
  double H = (H_L + ratio * H_R) / (1.0 + ratio);
  double q2 = uu * uu + vv * vv + ww * ww;
  double c = sqrt(gam1 * (H - 0.5 * q2));
  double qn = uu * n_x + vv * n_y + ww * n_z;
  double ql = uu * l_x + vv * l_y + ww * l_z;
  double qm = uu * m_x + vv * m_y + ww * m_z;

  R[0][0] = 1.0; R[1][0] = uu - c * n_x; R[2][0] = vv - c * n_y; R[3][0] = ww - c * n_z;
  R[4][0] = H - qn * c;
  R[0][1] = 1.0; R[1][1] = uu; R[2][1] = vv; R[3][1] = ww; R[4][1] = 0.5 * q2;
  R[0][2] = 1.0; R[1][2] = uu + c * n_x; R[2][2] = vv + c * n_y; R[3][2] = ww + c * n_z;
  R[4][2] = H + qn * c;
  R[0][3] = 0.0; R[1][3] = l_x; R[2][3] = l_y; R[3][3] = l_z; R[4][3] = ql;
  R[0][4] = 0.0; R[1][4] = m_x; R[2][4] = m_y; R[3][4] = m_z; R[4][4] = qm;

  double K_2c2 = gam1 / (2.0 * c * c);
  double one_2c = 0.5 / c;
  L[0][0] = 0.5 * K_2c2 * q2 + one_2c * qn;
  L[1][0] = 1.0 - K_2c2 * q2;
  L[2][0] = 0.5 * K_2c2 * q2 - one_2c * qn;
  L[3][0] = -ql;
  L[4][0] = -qm;
  L[0][1] = -(K_2c2 * uu + one_2c * n_x);
  L[1][1] = 2.0 * K_2c2 * uu;
  L[2][1] = -(K_2c2 * uu - one_2c * n_x);
  L[3][1] = l_x;
  L[4][1] = m_x;
  L[0][2] = -(K_2c2 * vv + one_2c * n_y);
  L[1][2] = 2.0 * K_2c2 * vv;
  L[2][2] = -(K_2c2 * vv - one_2c * n_y);
  L[3][2] = l_y;
  L[4][2] = m_y;
  L[0][3] = -(K_2c2 * ww + one_2c * n_z);
  L[1][3] = 2.0 * K_2c2 * ww;
  L[2][3] = -(K_2c2 * ww - one_2c * n_z);
  L[3][3] = l_z;
  L[4][3] = m_z;
  L[0][4] = K_2c2;
  L[1][4] = -2.0 * K_2c2;
  L[2][4] = K_2c2;
  L[3][4] = 0.0;
  L[4][4] = 0.0;
}

/* weno5 (src/weno.cpp:25-56). */
static double weno5(double Um2, double Um1, double U0, double Up1, double Up2) {
  const double eps = 1.0e-6;
  double diff1 = Um2 - 2.0 * Um1 + U0;
  double diff2 = Um2 - 4.0 * Um1 + 3.0 * U0;
  double diff3 = Um1 - 2.0 * U0 + Up1;
  double diff4 = Um1 - Up1;
  double diff5 = U0 - 2.0 * Up1 + Up2;
  double diff6 = 3.0 * U0 - 4.0 * Up1 + Up2;
  double IS1 = (13.0 / 12.0) * diff1 * diff1 + 0.25 * diff2 * diff2 + eps;
  double IS2 = (13.0 / 12.0) * diff3 * diff3 + 0.25 * diff4 * diff4 + eps;
  double IS3 = (13.0 / 12.0) * diff5 * diff5 + 0.25 * diff6 * diff6 + eps;
  double w1 = 0.1 / (IS1 * IS1);
  double w2 = 0.6 / (IS2 * IS2);
  double w3 = 0.3 / (IS3 * IS3);
  double sum = w1 + w2 + w3;
  double f1 = (2.0 * Um2 - 7.0 * Um1 + 11.0 * U0) / 6.0;
  double f2 = (-Um1 + 5.0 * U0 + 2.0 * Up1) / 6.0;
  double f3 = (2.0 * U0 + 5.0 * Up1 - Up2) / 6.0;
  return (w1 * f1 + w2 * f2 + w3 * f3) / sum;
}

/* rec_weno5 (src/weno.cpp:77-152): project the 5-point stencil of conserved
 * states onto characteristic fields with L, reconstruct each with weno5, map
 * back with R and convert to primitives. */
static void rec_weno5(const double* f1, const double* f2, const double* f3, const double* f4,
                      const double* f5, double R[5][5], double L[5][5], double gam1,
                      double* rho, double* u, double* v, double* w, double* p) {
  double fs[5][5], fc[5][5];
  const double* f[5] = {f1, f2, f3, f4, f5};
  for (int c = 0; c < 5; c++)
    for (int n = 0; n < 5; n++) fs[n][c] = f[c][n];
  for (int li = 0; li < NEQ; li++)
    for (int lj = 0; lj < 5; lj++) {
      double ss = 0.0;
      for (int lk = 0; lk < NEQ; lk++) ss += L[li][lk] * fs[lk][lj];
      fc[li][lj] = ss;
    }
  for (int n = 0; n < 5; n++) fs[n][0] = weno5(fc[n][0], fc[n][1], fc[n][2], fc[n][3], fc[n][4]);
  for (int li = 0; li < NEQ; li++) {
    double ss = 0.0;
    for (int lj = 0; lj < NEQ; lj++) ss += R[li][lj] * fs[lj][0];
    fs[li][1] = ss;
  }
  *rho = fs[0][1];
  *u = fs[1][1] / *rho;
  *v = fs[2][1] / *rho;
  *w = fs[3][1] / *rho;
  *p = gam1 * (fs[4][1] - 0.5 * *rho * (*u * *u + *v * *v + *w * *w));
}

/* lf_flux (src/lf_flux.cpp:32-99). */
static void lf_flux(double gamma, double rho_R, double u_R, double v_R, double w_R, double p_R,
                    double rho_L, double u_L, double v_L, double w_L, double p_L, double nx,
                    double ny, double nz, double* flux) {
  const double gam1 = gamma - 1.0;
  double c_R = sqrt(gamma * p_R / rho_R);
  double H_R = c_R * c_R / gam1 + 0.5 * (u_R * u_R + v_R * v_R + w_R * w_R);
  double rE_R = p_R / gam1 + 0.5 * rho_R * (u_R * u_R + v_R * v_R + w_R * w_R);
  double c_L = sqrt(gamma * p_L / rho_L);
  double H_L = c_L * c_L / gam1 + 0.5 * (u_L * u_L + v_L * v_L + w_L * w_L);
  double rE_L = p_L / gam1 + 0.5 * rho_L * (u_L * u_L + v_L * v_L + w_L * w_L);
  double q_R = u_R * nx + v_R * ny + w_R * nz;
  double q_L = u_L * nx + v_L * ny + w_L * nz;
  double ws[3], ws_max;
  ws[0] = fabs(u_R) + c_R; ws_max = fabs(u_L) + c_L; if (ws_max > ws[0]) ws[0] = ws_max;
  ws[1] = fabs(v_R) + c_R; ws_max = fabs(v_L) + c_L; if (ws_max > ws[1]) ws[1] = ws_max;
  ws[2] = fabs(w_R) + c_R; ws_max = fabs(w_L) + c_L; if (ws_max > ws[2]) ws[2] = ws_max;
  ws_max = fabs(ws[0] * nx + ws[1] * ny + ws[2] * nz);
  double diss[5], fL[5], fR[5];
  diss[0] = ws_max * (rho_R - rho_L);
  diss[1] = ws_max * (rho_R * u_R - rho_L * u_L);
  diss[2] = ws_max * (rho_R * v_R - rho_L * v_L);
  diss[3] = ws_max * (rho_R * w_R - rho_L * w_L);
  diss[4] = ws_max * (rE_R - rE_L);
  fL[0] = rho_L * q_L;
  fL[1] = rho_L * q_L * u_L + p_L * nx;
  fL[2] = rho_L * q_L * v_L + p_L * ny;
  fL[3] = rho_L * q_L * w_L + p_L * nz;
  fL[4] = rho_L * q_L * H_L;
  fR[0] = rho_R * q_R;
  fR[1] = rho_R * q_R * u_R + p_R * nx;
  fR[2] = rho_R * q_R * v_R + p_R * ny;
  fR[3] = rho_R * q_R * w_R + p_R * nz;
  fR[4] = rho_R * q_R * H_R;
  for (int li = 0; li < NEQ; li++) flux[li] = 0.5 * (fL[li] + fR[li] - diss[li]);
}

/* One face of Block3d::rec_riemann_{x,y,z} (src/Block3d.cpp:566-616, 631-681,
 * 696-746): eigenvectors from the cell primitives either side, left state from
 * the stencil (-3..+1), right state from the mirrored stencil (+2..-2), LF flux. */
static void riemann_face(const oracle_block* b, const double* Q, long cL, long cR,
                         long step, double nx, double ny, double nz, double* flux) {
  double R[5][5], L[5][5];
  const double gamma = b->sp.gamma, gam1 = b->sp.gam1;
  double rho_L = b->rho[cL], u_L = b->u[cL], v_L = b->v[cL], w_L = b->w[cL], p_L = b->p[cL];
  double rho_R = b->rho[cR], u_R = b->u[cR], v_R = b->v[cR], w_R = b->w[cR], p_R = b->p[cR];
  eigenvectors(gamma, rho_L, u_L, v_L, w_L, p_L, rho_R, u_R, v_R, w_R, p_R, nx, ny, nz, R, L);
  const double* q = Q + NEQ * cR; /* cell i */
  long s = NEQ * step;
  rec_weno5(q - 3 * s, q - 2 * s, q - s, q, q + s, R, L, gam1, &rho_L, &u_L, &v_L, &w_L, &p_L);
  rec_weno5(q + 2 * s, q + s, q, q - s, q - 2 * s, R, L, gam1, &rho_R, &u_R, &v_R, &w_R, &p_R);
  lf_flux(gamma, rho_R, u_R, v_R, w_R, p_R, rho_L, u_L, v_L, w_L, p_L, nx, ny, nz, flux);
}

/* Block3d::rec_riemann_x/y/z (src/Block3d.cpp:555-748). */
void oracle_rec_riemann(oracle_block* b, const double* Q) {
  const long IM = b->IM, JM = b->JM, KM = b->KM;
  const long sy = b->IM_G, sz = b->IM_G * b->JM_G;
#pragma omp parallel for schedule(static)
  for (long k = 0; k < KM; k++)
    for (long j = 0; j < JM; j++)
      for (long i = 0; i < IM + 1; i++)
        riemann_face(b, Q, idx(b, i - 1, j, k), idx(b, i, j, k), 1, 1.0, 0.0, 0.0,
                     &b->Ep[idx_Ep(b, 0, i, j, k)]);
#pragma omp parallel for schedule(static)
  for (long k = 0; k < KM; k++)
    for (long j = 0; j < JM + 1; j++)
      for (long i = 0; i < IM; i++)
        riemann_face(b, Q, idx(b, i, j - 1, k), idx(b, i, j, k), sy, 0.0, 1.0, 0.0,
                     &b->Fp[idx_Fp(b, 0, i, j, k)]);
#pragma omp parallel for schedule(static)
  for (long k = 0; k < KM + 1; k++)
    for (long j = 0; j < JM; j++)
      for (long i = 0; i < IM; i++)
        riemann_face(b, Q, idx(b, i, j, k - 1), idx(b, i, j, k), sz, 0.0, 0.0, 1.0,
                     &b->Gp[idx_Gp(b, 0, i, j, k)]);
}

/* calc_gradient (src/calc_gradient.cpp:17-66) on the NGV ring. */
static void calc_gradient(oracle_block* b, const double* f, double* f_x, double* f_y,
                          double* f_z) {
  const long IM = b->IM, JM = b->JM, KM = b->KM;
#pragma omp parallel for schedule(static)
  for (long k = -NGV; k < KM + NGV; k++)
    for (long j = -NGV; j < JM + NGV; j++)
      for (long i = -NGV; i < IM + NGV; i++) {
        long i0 = idx_ux(b, i, j, k);
        f_x[i0] = (1.0 / 12.0) * f[idx(b, i - 2, j, k)] - 2.0 / 3.0 * f[idx(b, i - 1, j, k)] +
                  (2.0 / 3.0) * f[idx(b, i + 1, j, k)] - 1.0 / 12.0 * f[idx(b, i + 2, j, k)];
        f_y[i0] = (1.0 / 12.0) * f[idx(b, i, j - 2, k)] - 2.0 / 3.0 * f[idx(b, i, j - 1, k)] +
                  (2.0 / 3.0) * f[idx(b, i, j + 1, k)] - 1.0 / 12.0 * f[idx(b, i, j + 2, k)];
        f_z[i0] = (1.0 / 12.0) * f[idx(b, i, j, k - 2)] - 2.0 / 3.0 * f[idx(b, i, j, k - 1)] +
                  (2.0 / 3.0) * f[idx(b, i, j, k + 1)] - 1.0 / 12.0 * f[idx(b, i, j, k + 2)];
        f_x[i0] /= b->dx;
        f_y[i0] /= b->dy;
        f_z[i0] /= b->dz;
      }
}

/* Block3d::calc_viscous_terms, calc_viscous_flux and
 * calc_viscous_flux_contribution (src/Block3d.cpp:750-918). */
void oracle_viscous(oracle_block* b) {
  const cbns_params* sp = &b->sp;
  const long IM = b->IM, JM = b->JM, KM = b->KM;
  calc_gradient(b, b->u, b->u_x, b->u_y, b->u_z);
  calc_gradient(b, b->v, b->v_x, b->v_y, b->v_z);
  calc_gradient(b, b->w, b->w_x, b->w_y, b->w_z);
  calc_gradient(b, b->T, b->T_x, b->T_y, b->T_z);
  const double C_T_inf = sp->C_T_inf, Re_inv = sp->Re_inv;
  const double kappa = -sp->Pr_inv * sp->gam1_inv / sp->Mach2;
#pragma omp parallel for schedule(static)
  for (long k = -NGV; k < KM + NGV; k++)
    for (long j = -NGV; j < JM + NGV; j++)
      for (long i = -NGV; i < IM + NGV; i++) {
        long i1 = idx(b, i, j, k), i2 = idx_ux(b, i, j, k);
        double T_l = b->T[i1];
        double mu_l = (1.0 + C_T_inf) / (T_l + C_T_inf) * sqrt(T_l * T_l * T_l);
        b->mu[i1] = mu_l;
        double u_x = b->u_x[i2], u_y = b->u_y[i2], u_z = b->u_z[i2];
        double v_x = b->v_x[i2], v_y = b->v_y[i2], v_z = b->v_z[i2];
        double w_x = b->w_x[i2], w_y = b->w_y[i2], w_z = b->w_z[i2];
        mu_l *= Re_inv;
        b->tau_xx[i2] = (2.0 / 3.0) * mu_l * (2.0 * u_x - v_y - w_z);
        b->tau_yy[i2] = (2.0 / 3.0) * mu_l * (2.0 * v_y - u_x - w_z);
        b->tau_zz[i2] = (2.0 / 3.0) * mu_l * (2.0 * w_z - u_x - v_y);
        b->tau_xy[i2] = mu_l * (u_y + v_x);
        b->tau_xz[i2] = mu_l * (u_z + w_x);
        b->tau_yz[i2] = mu_l * (v_z + w_y);
        mu_l *= kappa;
        b->q_x[i2] = mu_l * b->T_x[i2];
        b->q_y[i2] = mu_l * b->T_y[i2];
        b->q_z[i2] = mu_l * b->T_z[i2];
      }
#pragma omp parallel for schedule(static)
  for (long k = -NGV; k < KM + NGV; k++)
    for (long j = -NGV; j < JM + NGV; j++)
      for (long i = -NGV; i < IM + NGV; i++) {
        long i1 = idx(b, i, j, k), i2 = idx_ux(b, i, j, k), i3 = idx_Ev(b, 0, i, j, k);
        double uu = b->u[i1], vv = b->v[i1], ww = b->w[i1];
        double txx = b->tau_xx[i2], tyy = b->tau_yy[i2], tzz = b->tau_zz[i2];
        double txy = b->tau_xy[i2], txz = b->tau_xz[i2], tyz = b->tau_yz[i2];
        b->Ev[i3] = txx; b->Ev[i3 + 1] = txy; b->Ev[i3 + 2] = txz;
        b->Ev[i3 + 3] = uu * txx + vv * txy + ww * txz - b->q_x[i2];
        b->Fv[i3] = txy; b->Fv[i3 + 1] = tyy; b->Fv[i3 + 2] = tyz;
        b->Fv[i3 + 3] = uu * txy + vv * tyy + ww * tyz - b->q_y[i2];
        b->Gv[i3] = txz; b->Gv[i3 + 1] = tyz; b->Gv[i3 + 2] = tzz;
        b->Gv[i3 + 3] = uu * txz + vv * tyz + ww * tzz - b->q_z[i2];
      }
  const double c0 = 1.0 / 12.0, c1 = -2.0 / 3.0;
#pragma omp parallel for schedule(static)
  for (long k = 0; k < KM; k++)
    for (long j = 0; j < JM; j++)
      for (long i = 0; i < IM; i++)
        for (long n = 0; n < NEQ - 1; n++) {
          double df = (c0 * b->Ev[idx_Ev(b, n, i - 2, j, k)] + c1 * b->Ev[idx_Ev(b, n, i - 1, j, k)] -
                       c1 * b->Ev[idx_Ev(b, n, i + 1, j, k)] - c0 * b->Ev[idx_Ev(b, n, i + 2, j, k)]) /
                      b->dx;
          df += (c0 * b->Fv[idx_Ev(b, n, i, j - 2, k)] + c1 * b->Fv[idx_Ev(b, n, i, j - 1, k)] -
                 c1 * b->Fv[idx_Ev(b, n, i, j + 1, k)] - c0 * b->Fv[idx_Ev(b, n, i, j + 2, k)]) /
                b->dy;
          df += (c0 * b->Gv[idx_Ev(b, n, i, j, k - 2)] + c1 * b->Gv[idx_Ev(b, n, i, j, k - 1)] -
                 c1 * b->Gv[idx_Ev(b, n, i, j, k + 1)] - c0 * b->Gv[idx_Ev(b, n, i, j, k + 2)]) /
                b->dz;
          b->dfv[idx_dfv(b, n, i, j, k)] = df;
        }
}

/* Block3d::update_rk3 (src/Block3d.cpp:920-962). */
void oracle_update_rk3(oracle_block* b, double dt, int stage) {
  const long IM = b->IM, JM = b->JM, KM = b->KM;
#pragma omp parallel for schedule(static)
  for (long k = 0; k < KM; k++)
    for (long j = 0; j < JM; j++)
      for (long i = 0; i < IM; i++)
        for (long n = 0; n < NEQ; n++) {
          double df = (b->Ep[idx_Ep(b, n, i + 1, j, k)] - b->Ep[idx_Ep(b, n, i, j, k)]) / b->dx;
          df += (b->Fp[idx_Fp(b, n, i, j + 1, k)] - b->Fp[idx_Fp(b, n, i, j, k)]) / b->dy;
          df += (b->Gp[idx_Gp(b, n, i, j, k + 1)] - b->Gp[idx_Gp(b, n, i, j, k)]) / b->dz;
          if (n > 0) df -= b->dfv[idx_dfv(b, n - 1, i, j, k)];
          long i1 = idx_Q(b, n, i, j, k);
          if (stage == 1) b->Q_p[i1] = b->Q[i1] - dt * df;
          else if (stage == 2) b->Q_p[i1] = 0.75 * b->Q[i1] + 0.25 * (b->Q_p[i1] - dt * df);
          else if (stage == 3) b->Q[i1] = (b->Q[i1] + 2.0 * (b->Q_p[i1] - dt * df)) / 3.0;
        }
}

/* One stage of src/cbns3d.cpp:203-240. */
void oracle_stage(oracle_block* b, double dt, int stage) {
  double* U = stage == 1 ? b->Q : b->Q_p;
  double* out = stage == 3 ? b->Q : b->Q_p;
  oracle_rec_riemann(b, U);
  oracle_viscous(b);
  oracle_update_rk3(b, dt, stage);
  oracle_boundary_condition(b, out);
  oracle_calc_primitive(b, out);
}

/* Start-up of src/cbns3d.cpp:149-153 after the state is set. */
void oracle_start(oracle_block* b) {
  oracle_boundary_condition(b, b->Q);
  oracle_calc_primitive(b, b->Q);
  memcpy(b->Q_p, b->Q, sizeof(double) * NEQ * b->IM_G * b->JM_G * b->KM_G);
}

/* One iteration of src/cbns3d.cpp:176-241.  Returns 1 (and does nothing) when
 * Block3d::is_finished (src/Block3d.cpp:502-513) holds, else 0. */
int oracle_step(oracle_block* b, double* dt_out, double* t_out) {
  cbns_params* sp = &b->sp;
  if (sp->t_cur + 1.0e-5 > sp->t_end) return 1;
  double dt = oracle_calc_dt(b);
  if (sp->t_end - sp->t_cur < dt) dt = sp->t_end - sp->t_cur;
  sp->t_cur += dt;
  oracle_stage(b, dt, 1);
  oracle_stage(b, dt, 2);
  oracle_stage(b, dt, 3);
  if (dt_out) *dt_out = dt;
  if (t_out) *t_out = sp->t_cur;
  return 0;
}

/* State access in the get_idx_Q layout (ghosts included). Setting Q also sets
 * mu = 1 in the interior, the value initial_condition gives it. */
void oracle_set_Q(oracle_block* b, const double* Q, double t) {
  memcpy(b->Q, Q, sizeof(double) * NEQ * b->IM_G * b->JM_G * b->KM_G);
  for (long k = 0; k < b->KM; k++)
    for (long j = 0; j < b->JM; j++)
      for (long i = 0; i < b->IM; i++) b->mu[idx(b, i, j, k)] = 1.0;
  b->sp.t_cur = t;
}
void oracle_get_Q(const oracle_block* b, double* Q) {
  memcpy(Q, b->Q, sizeof(double) * NEQ * b->IM_G * b->JM_G * b->KM_G);
}
void oracle_get_Q_p(const oracle_block* b, double* Q) {
  memcpy(Q, b->Q_p, sizeof(double) * NEQ * b->IM_G * b->JM_G * b->KM_G);
}
void oracle_get_prims(const oracle_block* b, double* rho, double* u, double* v, double* w,
                      double* p, double* T, double* mu) {
  size_t n = sizeof(double) * b->IM_G * b->JM_G * b->KM_G;
  if (rho) memcpy(rho, b->rho, n);
  if (u) memcpy(u, b->u, n);
  if (v) memcpy(v, b->v, n);
  if (w) memcpy(w, b->w, n);
  if (p) memcpy(p, b->p, n);
  if (T) memcpy(T, b->T, n);
  if (mu) memcpy(mu, b->mu, n);
}
double oracle_get_time(const oracle_block* b) { return b->sp.t_cur; }
void oracle_get_spacing(const oracle_block* b, double* d) { d[0] = b->dx; d[1] = b->dy; d[2] = b->dz; }

/* Project-defined diagnostics (no counterpart in the reference): kinetic energy
 * KE = sum(0.5*rho*|u|^2)/N and enstrophy Omega = sum(0.5*rho*|curl u|^2)/N
 * over interior cells, N = IM*JM*KM, velocities u = Q[1..3]/Q[0] as in
 * calc_primitive, derivatives by the 4th-order central difference of
 * src/calc_gradient.cpp:29-64 (the ghost layers of Q must be filled).  Sums are
 * Neumaier-compensated and run in k, j, i order on one thread. */
static inline double vel(const double* Q, long c, int n) { return Q[NEQ * c + n] / Q[NEQ * c]; }
static inline double d4(const double* Q, long c, long s, int n, double h) {
  return ((1.0 / 12.0) * vel(Q, c - 2 * s, n) - 2.0 / 3.0 * vel(Q, c - s, n) +
          (2.0 / 3.0) * vel(Q, c + s, n) - 1.0 / 12.0 * vel(Q, c + 2 * s, n)) / h;
}
static inline void kahan_add(double* s, double* comp, double x) {
  double t = *s + x;
  if (fabs(*s) >= fabs(x)) *comp += (*s - t) + x;
  else *comp += (x - t) + *s;
  *s = t;
}
void oracle_diagnostics(const double* Q, long IM, long JM, long KM, double dx, double dy,
                        double dz, double* ke, double* enst) {
  const long IM_G = IM + 2 * NG, JM_G = JM + 2 * NG;
  const long sy = IM_G, sz = IM_G * JM_G;
  double s_ke = 0.0, c_ke = 0.0, s_en = 0.0, c_en = 0.0;
  for (long k = 0; k < KM; k++)
    for (long j = 0; j < JM; j++)
      for (long i = 0; i < IM; i++) {
        long c = (NG + i) + IM_G * ((NG + j) + JM_G * (NG + k));
        double r = Q[NEQ * c];
        double u = vel(Q, c, 1), v = vel(Q, c, 2), w = vel(Q, c, 3);
        kahan_add(&s_ke, &c_ke, 0.5 * r * (u * u + v * v + w * w));
        double wx = d4(Q, c, sy, 3, dy) - d4(Q, c, sz, 2, dz);
        double wy = d4(Q, c, sz, 1, dz) - d4(Q, c, 1, 3, dx);
        double wz = d4(Q, c, 1, 2, dx) - d4(Q, c, sy, 1, dy);
        kahan_add(&s_en, &c_en, 0.5 * r * (wx * wx + wy * wy + wz * wz));
      }
  double n = (double)IM * (double)JM * (double)KM;
  *ke = (s_ke + c_ke) / n;
  *enst = (s_en + c_en) / n;
}

/* Number of OpenMP threads the loops use (1 without OpenMP). */
int oracle_num_threads(void) {
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Hooks for property tests of the restated reference functions (test use only). */
void oracle_eigenvectors(double gamma, const double* pL, const double* pR, const double* n, double* R25,
                         double* L25) {
  double R[5][5], L[5][5];
  eigenvectors(gamma, pL[0], pL[1], pL[2], pL[3], pL[4], pR[0], pR[1], pR[2], pR[3], pR[4], n[0], n[1], n[2], R, L);
  memcpy(R25, R, sizeof R);
  memcpy(L25, L, sizeof L);
}
double oracle_weno5(const double* v) { return weno5(v[0], v[1], v[2], v[3], v[4]); }
void oracle_lf_flux(double gamma, const double* pR, const double* pL, const double* n, double* flux) {
  lf_flux(gamma, pR[0], pR[1], pR[2], pR[3], pR[4], pL[0], pL[1], pL[2], pL[3], pL[4], n[0], n[1], n[2], flux);
}
