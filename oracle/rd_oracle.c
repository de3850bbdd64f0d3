/*
 * rd_oracle.c -- CPU FP64 restatement of RUMDEED's time-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see rd_oracle.h).  Each function cites the
 * Fortran routine of NanoPhysicsCenter/RUMDEED it restates; the operation
 * order of every per-term formula follows the Fortran expression so that the
 * FP64 results are comparable to the last few ulps.
 *
 * Where the reference relies on things that cannot run here (the compiler's
 * RANDOM_NUMBER stream, the third-party Cuba library), the oracle restates
 * the algorithm the GPU library implements instead, with the same Philox
 * streams, so GPU and oracle can be compared chain for chain:
 *   - supply integral: composite Gauss-Legendre over the emitter instead of
 *     Cuba's Divonne (parity with the reference N_sup is statistical);
 *   - random numbers: Philox4x32-10 keyed by (seed) with counters
 *     (chain, iteration, step, purpose).
 */
#include "rd_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- constants: src/mod_global.F90:26-45,72-73,333 ----------------------- */
static const double PI = 3.141592653589793238462643383279502884197169399375105820974944592307816406286;
static const double H_PLANCK = 6.62607015e-34;
static const double C_LIGHT = 299792458.0;
static const double MU_0 = 1.25663706212e-6;
static const double M_U = 1.66053906660e-27;
static const double M_0 = 9.1093837015e-31;
static const double Q_0 = 1.602176634e-19;
static const double LENGTH_SCALE = 1.0e-9;
static const double TIME_SCALE = 1.0e-12;

static double EPS0, H_BAR, M_N2, M_N2P, DIV_FAC_C, A_FN, B_FN, L_CONST, L2, TIP_K;
static int g_const_init = 0;

static void init_constants(void) {
  if (g_const_init) return;
  EPS0 = 1.0 / (MU_0 * (C_LIGHT * C_LIGHT));             /* mod_global.F90:31 */
  H_BAR = H_PLANCK / (2.0 * PI);                          /* :34 */
  M_N2 = 28.0134 * M_U;                                   /* :52 */
  M_N2P = M_N2 - M_0;                                     /* :53 */
  DIV_FAC_C = 1.0 / (((4.0 * PI) * EPS0) * 1.0);          /* :333 */
  A_FN = (Q_0 * Q_0) / ((16.0 * (PI * PI)) * H_BAR);      /* fe_v2:36 */
  B_FN = (-4.0 / (3.0 * H_BAR)) * sqrt((2.0 * M_0) * Q_0); /* fe_v2:39 */
  L_CONST = Q_0 / ((4.0 * PI) * EPS0);                    /* fe_v2:47 */
  L2 = LENGTH_SCALE * LENGTH_SCALE;                       /* length_scale**2 guard */
  TIP_K = (1.0 * Q_0) / ((4.0 * PI) * EPS0);              /* acc_tip_ic_force.inc:20 */
  g_const_init = 1;
}

void orc_get_constants(orc_constants* o) {
  init_constants();
  o->pi = PI; o->h = H_PLANCK; o->c = C_LIGHT; o->mu_0 = MU_0; o->epsilon_0 = EPS0;
  o->m_u = M_U; o->h_bar = H_BAR; o->m_0 = M_0; o->q_0 = Q_0; o->m_N2 = M_N2;
  o->m_N2p = M_N2P; o->length_scale = LENGTH_SCALE; o->time_scale = TIME_SCALE;
  o->div_fac_c = DIV_FAC_C; o->a_FN = A_FN; o->b_FN = B_FN; o->l_const = L_CONST;
}

/* ---- Neumaier compensated accumulator ------------------------------------ */
typedef struct { double s, c; } nsum;
static inline void nadd(nsum* a, double x) {
  double t = a->s + x;
  if (fabs(a->s) >= fabs(x)) a->c += (a->s - t) + x;
  else a->c += (x - t) + a->s;
  a->s = t;
}
static inline double nval(const nsum* a) { return a->s + a->c; }

/* ---- FN functions: src/mod_field_emission_v2.F90:515-625 ----------------- */
static double fn_l(double F, double phi) {
  double l = (L_CONST * (-1.0 * F)) / (phi * phi);   /* :523 */
  return l;
}
double orc_v_y(double F, double phi, int ic) {       /* v_y :515-530 */
  init_constants();
  if (!ic) return 1.0;
  double l = fn_l(F, phi);
  if (l > 1.0) l = 1.0;
  return (1.0 - l) + ((1.0 / 6.0) * l) * log(l);
}
double orc_t_y(double F, double phi, int ic) {       /* t_y :532-553 */
  init_constants();
  if (!ic) return 1.0;
  double l = fn_l(F, phi);
  if (l > 1.0) l = 1.0;
  return 1.0 + l * ((1.0 / 9.0) - (1.0 / 18.0) * log(l));
}
double orc_escape_prob_log(double F, double phi, int ic) {  /* :570-575 */
  init_constants();
  double s = sqrt(phi);
  return ((B_FN * ((s * s) * s)) * orc_v_y(F, phi, ic)) / (-1.0 * F);
}
double orc_elec_supply_log(double F, double phi, int ic) {  /* :589-595 */
  init_constants();
  return (2.0 * log(-1.0 * F) - 2.0 * log(orc_t_y(F, phi, ic))) - log(phi);
}
double orc_elec_supply_v2(double F, double phi, int ic, double dt) {  /* :619-625 */
  init_constants();
  double t = orc_t_y(F, phi, ic);
  return (((dt / Q_0) * A_FN) / ((t * t) * phi)) * (F * F);
}

/* ---- checkerboard work function: src/mod_work_function.F90:389-487 ------- */
double orc_work_checkerboard(const double* w, int x_num, int y_num, const double em_pos[2],
                             const double em_dim[2], double x, double y, int* sec) {
  double xs = (x - em_pos[0]) / em_dim[0];
  double ys = (y - em_pos[1]) / em_dim[1];
  double x_len = 1.0 / x_num, y_len = 1.0 / y_num;
  int x_i = (int)floor(xs / x_len) + 1;
  int y_i = (int)floor(ys / y_len) + 1;
  if (x_i > x_num) x_i = x_num; else if (x_i < 1) x_i = 1;
  if (y_i > y_num) y_i = y_num; else if (y_i < 1) y_i = 1;
  if (sec) *sec = x_num * (y_i - 1) + x_i;
  y_i = y_num - y_i + 1;                     /* reversed y in the matrix */
  return w[(y_i - 1) * x_num + (x_i - 1)];
}
/* w_theta_gaussian, src/mod_work_function.F90:214-254 (centres and widths in nm) */
double orc_work_gaussian(const double* w, int n, double x, double y) {
  double v = w[0];
  for (int i = 0; i < n; ++i) {
    const double* g = w + 1 + 5 * i;
    double A = g[0];
    double x_c = g[1] * LENGTH_SCALE, y_c = g[2] * LENGTH_SCALE;
    double std_x = g[3] * LENGTH_SCALE, std_y = g[4] * LENGTH_SCALE;
    v = v + A * exp(-1.0 * (((x - x_c) * (x - x_c)) / (2.0 * (std_x * std_x)) +
                            ((y - y_c) * (y - y_c)) / (2.0 * (std_y * std_y))));
  }
  return v;
}

/* w_theta_voronoi, :533-571: the closest site; d starts at the single-precision 9.9E10 */
double orc_work_voronoi(const double* w, int n, const double em_pos[2], const double em_dim[2],
                        double x, double y, int* sec) {
  int k = -1;
  double d = (double)9.9e10f;
  for (int i = 0; i < n; ++i) {
    double sx = em_pos[0] + w[4 * i] * em_dim[0];   /* Read_work_function :130-131 */
    double sy = em_pos[1] + w[4 * i + 1] * em_dim[1];
    double d_p = (x - sx) * (x - sx) + (y - sy) * (y - sy);
    if (d_p < d) { k = i; d = d_p; }
  }
  if (k < 0) k = 0;
  if (sec) *sec = (int)w[4 * k + 3];
  return w[4 * k + 2];
}

static double work_at(const orc_diode* s, double x, double y, int* sec) {
  double pos[2] = {s->em_pos[0], s->em_pos[1]}, dim[2] = {s->em_dim[0], s->em_dim[1]};
  if (s->work_model == 2) {
    if (sec) *sec = 1;
    return orc_work_gaussian(s->work, s->work_nx, x, y);
  }
  if (s->work_model == 4) return orc_work_voronoi(s->work, s->work_nx, pos, dim, x, y, sec);
  return orc_work_checkerboard(s->work, s->work_nx, s->work_ny, pos, dim, x, y, sec);
}

/* ---- Philox4x32-10 --------------------------------------------------------- */
void orc_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
double orc_u01_from_words(uint32_t a, uint32_t b) {
  uint64_t m = ((uint64_t)a << 21) ^ (uint64_t)(b >> 11);
  return (double)(m & ((1ull << 53) - 1)) * (1.0 / 9007199254740992.0);
}

enum { TAG_INIT = 1, TAG_GAUSS = 2, TAG_ACCEPT = 3, TAG_EMIT = 4 };

static void rng2(uint64_t seed, uint32_t a, uint32_t b, uint32_t step, uint32_t tag,
                 double* u1, double* u2) {
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t ctr[4] = {a, b, step, tag}, o[4];
  orc_philox4x32(ctr, key, o);
  *u1 = orc_u01_from_words(o[0], o[1]);
  *u2 = orc_u01_from_words(o[2], o[3]);
}

/* box_muller (Marsaglia polar form), src/mod_global.F90:578-595; the attempt
 * index of the rejection loop is part of the counter. */
static void gauss2(uint64_t seed, uint32_t chain, uint32_t it, uint32_t step, double* g1,
                   double* g2) {
  for (uint32_t k = 0; k < 64; ++k) {
    double u1, u2;
    rng2(seed, chain, it, step, TAG_GAUSS | (k << 8), &u1, &u2);
    double x1 = 2.0 * u1 - 1.0, x2 = 2.0 * u2 - 1.0;
    double w = x1 * x1 + x2 * x2;
    if (w < 1.0 && w > 0.0) {
      double f = sqrt((-2.0 * log(w)) / w);
      *g1 = x1 * f; *g2 = x2 * f;
      return;
    }
  }
  *g1 = 0.0; *g2 = 0.0;
}

/* ---- diode lifetime ------------------------------------------------------- */
orc_diode* orc_diode_new(int geometry, int cap, double V_s, double d, double time_step,
                         int image_charge, int N_ic_max) {
  init_constants();
  orc_diode* s = (orc_diode*)calloc(1, sizeof(orc_diode));
  s->geometry = geometry;
  s->cap = cap;
  s->pos = (double*)calloc((size_t)3 * cap, sizeof(double));
  s->vel = (double*)calloc((size_t)3 * cap, sizeof(double));
  s->acc = (double*)calloc((size_t)3 * cap, sizeof(double));
  s->acc_prev = (double*)calloc((size_t)3 * cap, sizeof(double));
  s->acc_prev2 = (double*)calloc((size_t)3 * cap, sizeof(double));
  s->charge = (double*)calloc(cap, sizeof(double));
  s->mass = (double*)calloc(cap, sizeof(double));
  s->species = (int*)calloc(cap, sizeof(int));
  s->mask = (int*)calloc(cap, sizeof(int));
  s->id = (int*)calloc(cap, sizeof(int));
  s->step_created = (int*)calloc(cap, sizeof(int));
  s->section = (int*)calloc(cap, sizeof(int));
  s->V_s = V_s;
  s->d = d;
  s->box_dim[0] = 0.0; s->box_dim[1] = 0.0; s->box_dim[2] = d;
  s->E_z = -1.0 * V_s / d;                     /* Set_Voltage, mod_verlet.F90:2050-2052 */
  s->time_step = time_step;
  s->time_step2 = time_step * time_step;
  s->image_charge = image_charge;
  s->N_ic_max = N_ic_max;
  s->work_nx = s->work_ny = 1;
  s->work[0] = 4.7;
  s->work_model = 1;
  s->emitter_type = 2;
  s->tip_phi = 4.7;
  s->MH_std = 0.0125;                          /* fe_v2:58 */
  s->a_rate = 1.0;
  s->mh_jumps = 200;
  s->max_chains = 1 << 30;
  s->quad_panels = 0;   /* 0: orc_supply_panels, nodes at most 5 nm apart */
  s->quad_order = 4;
  s->init_rounds_max = 10000;
  for (int i = 0; i < cap; ++i) s->mask[i] = 1;
  return s;
}

void orc_diode_free(orc_diode* s) {
  if (!s) return;
  free(s->pos); free(s->vel); free(s->acc); free(s->acc_prev); free(s->acc_prev2);
  free(s->charge); free(s->mass); free(s->species); free(s->mask); free(s->id);
  free(s->step_created); free(s->section);
  free(s);
}

void orc_set_planar_emitter(orc_diode* s, double x0, double y0, double Lx, double Ly,
                            int nx, int ny, const double* work) {
  s->em_pos[0] = x0; s->em_pos[1] = y0; s->em_dim[0] = Lx; s->em_dim[1] = Ly;
  s->work_model = 1;
  s->emitter_type = 2;
  s->work_nx = nx; s->work_ny = ny;
  for (int i = 0; i < nx * ny && i < 64 * 64; ++i) s->work[i] = work[i];
}

void orc_set_ring(orc_diode* s, double r_out, double thickness) {
  s->emitter_type = 4;
  s->ring_thick = thickness;
  s->ring_rmin = r_out - thickness;
  s->mh_serial = 1;
}

void orc_set_work_model(orc_diode* s, int model, int n, const double* params) {
  int len = model == 2 ? 1 + 5 * n : 4 * n;
  s->work_model = model;
  s->work_nx = n;
  s->work_ny = 1;
  for (int i = 0; i < len && i < 64 * 64; ++i) s->work[i] = params[i];
}

/* Init_Emission_Tip, src/mod_emission_tip.f90:81-127 */
void orc_set_tip(orc_diode* s, double d_tip, double R_base, double h_tip, double phi) {
  init_constants();
  s->geometry = ORC_TIP;
  s->d_tip = d_tip; s->R_base = R_base; s->h_tip = h_tip; s->tip_phi = phi;
  s->d = d_tip + h_tip;
  s->box_dim[2] = s->d;
  s->max_xi = h_tip / d_tip + 1.0;
  s->a_foci = sqrt(((d_tip * d_tip) * (R_base * R_base)) / ((h_tip * h_tip) + (2.0 * d_tip) * h_tip)
                   + d_tip * d_tip);
  s->eta_1 = -1.0 * d_tip / s->a_foci;
  s->theta_tip = acos(d_tip / s->a_foci);
  s->r_tip = (s->a_foci * sin(s->theta_tip)) * tan(s->theta_tip);
  s->shift_z = fabs((s->a_foci * s->eta_1) * s->max_xi);
  const double eta_2 = 0.0;
  double pre = log((((1.0 + s->eta_1) / (1.0 - s->eta_1)) * (1.0 - eta_2)) / (1.0 + eta_2));
  s->pre_fac_E_tip_unit_voltage = (2.0 * 1.0) / (s->a_foci * pre);
  s->pre_fac_E_tip = (2.0 * s->V_s) / (s->a_foci * pre);
  s->MH_std = 1.0;                             /* mod_emission_tip.f90:50 */
  s->mh_jumps = 80;
}

void orc_set_emission(orc_diode* s, int on, uint64_t seed, int mh_jumps, int max_chains,
                      int quad_panels, int quad_order) {
  s->emission = on;
  s->seed = seed;
  if (mh_jumps > 0) s->mh_jumps = mh_jumps;
  if (max_chains > 0) s->max_chains = max_chains;
  if (quad_panels > 0) s->quad_panels = quad_panels;
  if (quad_order > 0) s->quad_order = quad_order;
}

void orc_reset(orc_diode* s) {
  s->n = 0; s->nrID = 0;
  s->n_remove = s->n_remove_top = s->n_remove_bot = 0;
  s->emitted_total = s->absorbed_top_total = s->absorbed_bot_total = s->dropped_total = 0;
  s->ramo_current = 0.0;
  memset(s->life_time, 0, sizeof(s->life_time));
  for (int i = 0; i < s->cap; ++i) s->mask[i] = 1;
  s->residual = 0.0;
}

/* ---- vacuum fields ---------------------------------------------------------- */
/* field_E_Hyperboloid, src/mod_hyperboloid_tip.f90:115-154 */
static void field_E_hyperboloid(const orc_diode* s, const double p[3], double out[3]) {
  double x = p[0], y = p[1], z = p[2], a = s->a_foci, sz = s->shift_z;
  double rp = sqrt(x * x + y * y + ((z + a) - sz) * ((z + a) - sz));
  double rm = sqrt(x * x + y * y + ((z - a) - sz) * ((z - a) - sz));
  double xi = (1.0 / (2.0 * a)) * (rp + rm);
  double eta = (1.0 / (2.0 * a)) * (rp - rm);
  double phi = (fabs(x) < 1.0e-18 && fabs(y) < 1.0e-18) ? 0.0 : atan2(y, x);
  double pre = s->pre_fac_E_tip * (1.0 / (xi * xi - eta * eta));
  double fac = (fabs(xi - 1.0) < 1.0e-6) ? 0.0 : eta * sqrt((xi * xi - 1.0) / (1.0 - eta * eta));
  out[0] = ((-1.0 * pre) * fac) * cos(phi);
  out[1] = ((-1.0 * pre) * fac) * sin(phi);
  out[2] = pre * xi;
}

void orc_field_E(const orc_diode* s, const double p[3], double out[3]) {
  if (s->geometry == ORC_TIP) { field_E_hyperboloid(s, p, out); return; }
  out[0] = 0.0; out[1] = 0.0; out[2] = s->E_z;  /* field_E_planar :1983-1999 */
}

void orc_E_zunit(const orc_diode* s, const double p[3], double out[3]) {
  if (s->geometry == ORC_TIP) {                 /* E_zunit_tip, emission_tip:133-141 */
    double e[3];
    field_E_hyperboloid(s, p, e);
    for (int k = 0; k < 3; ++k) out[k] = (e[k] * s->pre_fac_E_tip_unit_voltage) / s->pre_fac_E_tip;
    return;
  }
  out[0] = 0.0; out[1] = 0.0; out[2] = -1.0 / s->d;  /* E_zunit_planar fe_v2:158-166 */
}

/* ---- image charges ----------------------------------------------------------- */
/* Force_Image_charges_v2, src/mod_verlet.F90:1924-1979 (partners of pos_2
 * evaluated at pos_1; no charge prefactor). */
void orc_force_image_planar(const orc_diode* s, const double p1[3], const double p2[3],
                            double out[3]) {
  init_constants();
  out[0] = out[1] = out[2] = 0.0;
  if (!s->image_charge) return;
  double dx = p1[0] - p2[0], dy = p1[1] - p2[1];
  double zic = -1.0 * p2[2];
  double dz = p1[2] - zic;
  double r = sqrt((dx * dx + dy * dy) + dz * dz) + L2;
  double inv = 1.0 / ((r * r) * r);
  out[0] = (-dx) * inv; out[1] = (-dy) * inv; out[2] = (-dz) * inv;
  for (int n = 1; n <= s->N_ic_max; ++n) {
    double zs[4] = {(2.0 * n) * s->d - p2[2], (-2.0 * n) * s->d - p2[2],
                    (2.0 * n) * s->d + p2[2], (-2.0 * n) * s->d + p2[2]};
    double sg[4] = {-1.0, -1.0, 1.0, 1.0};
    for (int k = 0; k < 4; ++k) {
      dz = p1[2] - zs[k];
      r = sqrt((dx * dx + dy * dy) + dz * dz) + L2;
      inv = 1.0 / ((r * r) * r);
      out[0] += (sg[k] * dx) * inv; out[1] += (sg[k] * dy) * inv; out[2] += (sg[k] * dz) * inv;
    }
  }
}

/* Sphere_IC_field, src/mod_hyperboloid_tip.f90:168-210: image of pos_1 in
 * the apex sphere, field evaluated at pos_2, including the extra
 * q_0/(4 pi eps_0) factor of the reference. */
void orc_sphere_ic_field(const orc_diode* s, const double p1[3], const double p2[3],
                         double out[3]) {
  init_constants();
  out[0] = out[1] = out[2] = 0.0;
  if (!s->image_charge) return;
  double z0 = s->h_tip - s->r_tip, R = s->r_tip;
  double xa = p1[0], ya = p1[1], za = p1[2];
  double x = p2[0], y = p2[1], z = p2[2];
  double dza = za - z0;
  double dis_a = sqrt(xa * xa + ya * ya + dza * dza);
  double zb = z0 + (R * R) / (sqrt((1.0 + (xa * xa) / (dza * dza)) + (ya * ya) / (dza * dza)) * dis_a);
  double xb = ((zb - z0) * xa) / dza;
  double yb = ((zb - z0) * ya) / dza;
  double tda = pow((x - xa) * (x - xa) + (y - ya) * (y - ya) + (z - za) * (z - za), 1.5);
  double tdb = pow((x - xb) * (x - xb) + (y - yb) * (y - yb) + (z - zb) * (z - zb), 1.5);
  out[0] = TIP_K * ((xa - x) / tda - (R * (xb - x)) / (dis_a * tdb));
  out[1] = TIP_K * ((ya - y) / tda - (R * (yb - y)) / (dis_a * tdb));
  out[2] = TIP_K * ((za - z) / tda - (R * (zb - z)) / (dis_a * tdb));
}

static void image_effect(const orc_diode* s, const double p1[3], const double p2[3],
                         double out[3]) {
  if (s->geometry == ORC_TIP) orc_sphere_ic_field(s, p1, p2, out);
  else orc_force_image_planar(s, p1, p2, out);
}

/* ---- accelerations ------------------------------------------------------------ */
/* Calculate_Acceleration_Particles_Generic, src/mod_verlet.F90:625-751 */
void orc_accel_generic(const orc_diode* s, double* acc, int comp) {
  init_constants();
  int n = s->n;
  nsum* a = (nsum*)calloc((size_t)3 * (n > 0 ? n : 1), sizeof(nsum));
  for (int i = 0; i < n; ++i) {
    if (s->species[i] == ORC_ATOM) continue;
    const double* p1 = s->pos + 3 * i;
    double im1 = 1.0 / s->mass[i], q1 = s->charge[i], qd1 = q1 * DIV_FAC_C;
    double fE[3], e[3];
    orc_field_E(s, p1, e);
    for (int k = 0; k < 3; ++k) fE[k] = q1 * e[k];
    for (int j = i + 1; j < n; ++j) {
      if (s->species[j] == ORC_ATOM) continue;
      const double* p2 = s->pos + 3 * j;
      double im2 = 1.0 / s->mass[j], pre = qd1 * s->charge[j];
      double diff[3] = {p1[0] - p2[0], p1[1] - p2[1], p1[2] - p2[2]};
      double r = sqrt((diff[0] * diff[0] + diff[1] * diff[1]) + diff[2] * diff[2]) + L2;
      double inv = 1.0 / ((r * r) * r);
      double fc[3], ic[3], icN[3];
      for (int k = 0; k < 3; ++k) fc[k] = (pre * inv) * diff[k];
      image_effect(s, p1, p2, ic);
      for (int k = 0; k < 3; ++k) ic[k] = pre * ic[k];
      icN[0] = -1.0 * ic[0]; icN[1] = -1.0 * ic[1]; icN[2] = 1.0 * ic[2];
      for (int k = 0; k < 3; ++k) {
        double vj = im2 * (icN[k] - fc[k]), vi = im1 * (fc[k] + ic[k]);
        if (comp) { nadd(&a[3 * j + k], vj); nadd(&a[3 * i + k], vi); }
        else { a[3 * j + k].s += vj; a[3 * i + k].s += vi; }
      }
    }
    for (int k = 0; k < 3; ++k) {
      double v = fE[k] * im1;
      if (comp) nadd(&a[3 * i + k], v); else a[3 * i + k].s += v;
    }
  }
  for (int i = 0; i < 3 * n; ++i) acc[i] = nval(&a[i]);
  free(a);
}

/* Calculate_Acceleration_Particles_Planar, src/mod_verlet.F90:763-884 */
void orc_accel_planar(const orc_diode* s, double* acc, int comp) {
  init_constants();
  int n = s->n, Nic = s->N_ic_max;
  double Ez = s->E_z, d = s->d;
  nsum* a = (nsum*)calloc((size_t)3 * (n > 0 ? n : 1), sizeof(nsum));
  for (int i = 0; i < n; ++i) {
    if (s->species[i] == ORC_ATOM) continue;
    double x1 = s->pos[3 * i], y1 = s->pos[3 * i + 1], z1 = s->pos[3 * i + 2];
    double q1 = s->charge[i], qd1 = q1 * DIV_FAC_C, im1 = 1.0 / s->mass[i];
    nsum ax = {0, 0}, ay = {0, 0}, az = {0, 0};
    for (int j = i + 1; j < n; ++j) {
      if (s->species[j] == ORC_ATOM) continue;
      double x2 = s->pos[3 * j], y2 = s->pos[3 * j + 1], z2 = s->pos[3 * j + 2];
      double im2 = 1.0 / s->mass[j], pre = qd1 * s->charge[j];
      double dx = x1 - x2, dy = y1 - y2, dz = z1 - z2, dxy2 = dx * dx + dy * dy;
      double r = sqrt(dxy2 + dz * dz) + L2, inv = 1.0 / ((r * r) * r);
      double fcx = (pre * inv) * dx, fcy = (pre * inv) * dy, fcz = (pre * inv) * dz;
      double icx = 0.0, icy = 0.0, icz = 0.0;
      if (s->image_charge) {   /* acc_ic_planar_series.inc with z_a = z_1, z_b = z_2 */
        double za = z1, zb = z2, zic = -1.0 * zb, dzi = za - zic;
        r = sqrt(dxy2 + dzi * dzi) + L2; inv = 1.0 / ((r * r) * r);
        icx = -dx * inv; icy = -dy * inv; icz = -dzi * inv;
        for (int m = 1; m <= Nic; ++m) {
          double zz[4] = {(2.0 * m) * d - zb, (-2.0 * m) * d - zb, (2.0 * m) * d + zb,
                          (-2.0 * m) * d + zb};
          for (int k = 0; k < 4; ++k) {
            dzi = za - zz[k];
            r = sqrt(dxy2 + dzi * dzi) + L2; inv = 1.0 / ((r * r) * r);
            if (k < 2) { icx = icx - dx * inv; icy = icy - dy * inv; icz = icz - dzi * inv; }
            else { icx = icx + dx * inv; icy = icy + dy * inv; icz = icz + dzi * inv; }
          }
        }
      }
      double vx = fcx + pre * icx, vy = fcy + pre * icy, vz = fcz + pre * icz;
      double jx = im2 * (-pre * icx - fcx), jy = im2 * (-pre * icy - fcy), jz = im2 * (pre * icz - fcz);
      if (comp) {
        nadd(&ax, vx); nadd(&ay, vy); nadd(&az, vz);
        nadd(&a[3 * j], jx); nadd(&a[3 * j + 1], jy); nadd(&a[3 * j + 2], jz);
      } else {
        ax.s += vx; ay.s += vy; az.s += vz;
        a[3 * j].s += jx; a[3 * j + 1].s += jy; a[3 * j + 2].s += jz;
      }
    }
    double vx = nval(&ax) * im1, vy = nval(&ay) * im1, vz = (nval(&az) + q1 * Ez) * im1;
    if (comp) { nadd(&a[3 * i], vx); nadd(&a[3 * i + 1], vy); nadd(&a[3 * i + 2], vz); }
    else { a[3 * i].s += vx; a[3 * i + 1].s += vy; a[3 * i + 2].s += vz; }
  }
  for (int i = 0; i < 3 * n; ++i) acc[i] = nval(&a[i]);
  free(a);
}

/* Calculate_Acceleration_Particles_ACC, src/mod_verlet.F90:1217-1429: every
 * particle gathers over all others; the image term of the pair is always
 * evaluated with the lower-indexed particle in the (a) role and mirrored in
 * x, y for the higher-indexed one. */
static void gather_row(const orc_diode* s, int i, double* out3, int comp) {
  int n = s->n;
  const double* p1 = s->pos + 3 * i;
  double q1 = s->charge[i], qd1 = q1 * DIV_FAC_C;
  nsum a[3] = {{0, 0}, {0, 0}, {0, 0}};
  for (int j = 0; j < n; ++j) {
    if (j == i) continue;
    const double* p2 = s->pos + 3 * j;
    double pre = qd1 * s->charge[j];
    double diff[3] = {p1[0] - p2[0], p1[1] - p2[1], p1[2] - p2[2]};
    double r = sqrt((diff[0] * diff[0] + diff[1] * diff[1]) + diff[2] * diff[2]) + L2;
    double inv = 1.0 / ((r * r) * r);
    double t[3];
    for (int k = 0; k < 3; ++k) t[k] = (pre * inv) * diff[k];
    if (s->image_charge) {
      double ic[3], sgn = (j > i) ? 1.0 : -1.0;
      if (j > i) image_effect(s, p1, p2, ic); else image_effect(s, p2, p1, ic);
      t[0] += pre * (sgn * ic[0]); t[1] += pre * (sgn * ic[1]); t[2] += pre * ic[2];
    }
    for (int k = 0; k < 3; ++k) { if (comp) nadd(&a[k], t[k]); else a[k].s += t[k]; }
  }
  double e[3];
  orc_field_E(s, p1, e);
  double im1 = 1.0 / s->mass[i];
  for (int k = 0; k < 3; ++k) out3[k] = (nval(&a[k]) + q1 * e[k]) * im1;
}

void orc_accel_gather(const orc_diode* s, double* acc, int comp) {
  init_constants();
  int n = s->n;
#pragma omp parallel for schedule(dynamic, 16)
  for (int i = 0; i < n; ++i) gather_row(s, i, acc + 3 * i, comp);
}

/* orc_accel_gather for the listed particles only: acc3 gets (3, nrows), row k
 * the acceleration of particle rows[k] against all others.  The rows of a
 * gather are independent, so a sample of them checks a full-size system. */
void orc_accel_rows(const orc_diode* s, int nrows, const int* rows, double* acc3, int comp) {
  init_constants();
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < nrows; ++k) gather_row(s, rows[k], acc3 + 3 * k, comp);
}

/* Calc_Field_at, src/mod_verlet.F90:1466-1529 */
void orc_field_at(const orc_diode* s, const double p[3], double out[3], int comp) {
  init_constants();
  double e[3];
  orc_field_E(s, p, e);
  nsum f[3] = {{e[0], 0}, {e[1], 0}, {e[2], 0}};
  for (int j = 0; j < s->n; ++j) {
    if (s->species[j] == ORC_ATOM) continue;
    const double* p2 = s->pos + 3 * j;
    double pre = s->charge[j] * DIV_FAC_C;
    double diff[3] = {p[0] - p2[0], p[1] - p2[1], p[2] - p2[2]};
    double r = sqrt((diff[0] * diff[0] + diff[1] * diff[1]) + diff[2] * diff[2]) + L2;
    double inv = 1.0 / ((r * r) * r);
    double ic[3];
    image_effect(s, p, p2, ic);
    for (int k = 0; k < 3; ++k) {
      double v = pre * (diff[k] * inv + ic[k]);
      if (comp) nadd(&f[k], v); else f[k].s += v;
    }
  }
  for (int k = 0; k < 3; ++k) out[k] = nval(&f[k]);
}

void orc_field_at_batch(const orc_diode* s, int M, const double* pts, double* out, int comp) {
#pragma omp parallel for schedule(dynamic, 4)
  for (int m = 0; m < M; ++m) orc_field_at(s, pts + 3 * m, out + 3 * m, comp);
}

/* ---- particle bookkeeping: src/mod_pair.F90 ------------------------------------ */
/* Add_Particle :29-159 */
int orc_add_particle(orc_diode* s, const double pos[3], const double vel[3], int species,
                     int step, int sec) {
  init_constants();
  if (s->n + 1 > s->cap) { s->dropped_total++; return -1; }
  int i = s->n;
  for (int k = 0; k < 3; ++k) {
    s->pos[3 * i + k] = pos[k];
    s->vel[3 * i + k] = vel[k];
    s->acc[3 * i + k] = s->acc_prev[3 * i + k] = s->acc_prev2[3 * i + k] = 0.0;
  }
  s->step_created[i] = step;
  s->mask[i] = 1;
  s->species[i] = species;
  s->section[i] = sec;
  s->id[i] = s->nrID;
  if (species == ORC_ELEC) { s->charge[i] = -1.0 * Q_0; s->mass[i] = 1.0 * M_0; }
  else if (species == ORC_ION) { s->charge[i] = 1.0 * Q_0; s->mass[i] = M_N2P; }
  else { s->charge[i] = 0.0; s->mass[i] = M_N2; }
  /* seed the Beeman history with the vacuum-field acceleration :133-139 */
  double e[3];
  orc_field_E(s, pos, e);
  for (int k = 0; k < 3; ++k) {
    double a = (s->charge[i] / s->mass[i]) * e[k];
    s->acc[3 * i + k] = s->acc_prev[3 * i + k] = s->acc_prev2[3 * i + k] = a;
  }
  s->n++;
  s->nrID++;
  return i;
}

/* Mark_Particles_Remove :169-339 (electron/ion top/bot cases) */
void orc_mark_remove(orc_diode* s, int i, int why) {
  if (!s->mask[i]) return;
  s->mask[i] = 0;
  s->charge[i] = 0.0;
  s->n_remove++;
  if (s->species[i] == ORC_ELEC) {
    if (why == ORC_REMOVE_TOP) s->n_remove_top++;
    else if (why == ORC_REMOVE_BOT) s->n_remove_bot++;
  }
}

/* Remove_Particles :352-562 with compact_array :1180-1223 and
 * record_lifetime :1135-1160.  Nothing is compacted (and no lifetime is
 * recorded) when every particle is removed, as in the reference. */
void orc_remove_particles(orc_diode* s, int step) {
  s->absorbed_top_total += s->n_remove_top;
  s->absorbed_bot_total += s->n_remove_bot;
  if (s->n_remove > 0 && s->n > 0) {
    int n = s->n;
    if (n - s->n_remove > 0) {
      int k = 0;
      while (k < n && s->mask[k]) ++k;      /* First_Dead_Index :570-582 */
      int j = k;
      for (int i = k; i < n; ++i) {
        if (s->mask[i]) {
          for (int c = 0; c < 3; ++c) {
            s->pos[3 * j + c] = s->pos[3 * i + c];
            s->vel[3 * j + c] = s->vel[3 * i + c];
            s->acc[3 * j + c] = s->acc[3 * i + c];
            s->acc_prev[3 * j + c] = s->acc_prev[3 * i + c];
            s->acc_prev2[3 * j + c] = s->acc_prev2[3 * i + c];
          }
          s->charge[j] = s->charge[i]; s->mass[j] = s->mass[i];
          s->species[j] = s->species[i]; s->id[j] = s->id[i];
          s->step_created[j] = s->step_created[i]; s->section[j] = s->section[i];
          ++j;
        } else {
          int lt = step - s->step_created[i];
          if (lt <= 0) lt = 1;
          if (lt > ORC_MAX_LIFE) lt = ORC_MAX_LIFE;
          int sp = s->species[i];
          if (sp >= 1 && sp <= 3) s->life_time[lt - 1][sp - 1]++;
        }
      }
    }
    s->n = n - s->n_remove;
    for (int i = 0; i < n; ++i) s->mask[i] = 1;
    s->n_remove = s->n_remove_top = s->n_remove_bot = 0;
  }
}

/* ---- integrator: src/mod_verlet.F90 ----------------------------------------- */
double orc_tip_eta(const orc_diode* s, double x, double y, double z) {  /* eta_coor :62-67 */
  double a = s->a_foci, sz = s->shift_z;
  return (1.0 / (2.0 * a)) * (sqrt(x * x + y * y + ((z + a) - sz) * ((z + a) - sz)) -
                              sqrt(x * x + y * y + ((z - a) - sz) * ((z - a) - sz)));
}

static void check_boundary(orc_diode* s, int i) {
  double z = s->pos[3 * i + 2];
  if (z < 0.0) orc_mark_remove(s, i, ORC_REMOVE_BOT);          /* Check_Boundary_Planar :325-338 */
  else if (z > s->box_dim[2]) orc_mark_remove(s, i, ORC_REMOVE_TOP);
  if (s->geometry == ORC_TIP) {                                 /* Check_Boundary_Tip :1627-1647 */
    double eta = orc_tip_eta(s, s->pos[3 * i], s->pos[3 * i + 1], z);
    if (eta < s->eta_1) orc_mark_remove(s, i, ORC_REMOVE_BOT);
  }
}

/* Update_ElecIon_Position :197-232 (Beeman) */
void orc_update_position(orc_diode* s) {
  double dt = s->time_step, dt2 = s->time_step2;
  for (int i = 0; i < s->n; ++i) {
    if (s->species[i] == ORC_ATOM) continue;
    for (int k = 0; k < 3; ++k) {
      int q = 3 * i + k;
      s->pos[q] = (s->pos[q] + s->vel[q] * dt) +
                  ((1.0 / 6.0) * (4.0 * s->acc[q] - s->acc_prev[q])) * dt2;
      s->acc_prev2[q] = s->acc_prev[q];
      s->acc_prev[q] = s->acc[q];
      s->acc[q] = 0.0;
    }
    check_boundary(s, i);
  }
}

/* ---- two-time-step integrator (two_time_step, atom_time_interval = T > 0) ----
 * Update_Species_Position :234-290: electrons every step; ions on steps
 * divisible by T with nrStep = T; atoms never (Update_Particle_Position
 * :181-194).  Electrons are taken in their pointer order, then the ions. */
static void species_position(orc_diode* s, int species, double nr) {
  double dt = s->time_step, dt2 = s->time_step2, nr2 = nr * nr;
  for (int i = 0; i < s->n; ++i) {
    if (s->species[i] != species) continue;
    for (int k = 0; k < 3; ++k) {
      int q = 3 * i + k;
      s->pos[q] = (s->pos[q] + (s->vel[q] * dt) * nr) +
                  (((1.0 / 6.0) * (4.0 * s->acc[q] - s->acc_prev[q])) * dt2) * nr2;
      s->acc_prev2[q] = s->acc_prev[q];
      s->acc_prev[q] = s->acc[q];
      s->acc[q] = 0.0;
    }
    check_boundary(s, i);
  }
}

void orc_update_position_tts(orc_diode* s, int step) {
  species_position(s, ORC_ELEC, 1.0);
  if (step % s->atom_time_interval == 0) species_position(s, ORC_ION, (double)s->atom_time_interval);
}

/* One pair of Update_Elec_Acceleration / Update_Ion_Acceleration
 * (:899-1151): particle i in the (a) role, particle j mirrored in x, y. */
static void tts_pair(const orc_diode* s, int i, int j, nsum* a, int comp) {
  const double* p1 = s->pos + 3 * i;
  const double* p2 = s->pos + 3 * j;
  double im1 = 1.0 / s->mass[i], im2 = 1.0 / s->mass[j];
  double pre = (s->charge[i] * DIV_FAC_C) * s->charge[j];
  double diff[3] = {p1[0] - p2[0], p1[1] - p2[1], p1[2] - p2[2]};
  double r = sqrt((diff[0] * diff[0] + diff[1] * diff[1]) + diff[2] * diff[2]) + L2;
  double inv = 1.0 / ((r * r) * r);
  double fc[3], ic[3] = {0, 0, 0}, icN[3];
  for (int k = 0; k < 3; ++k) fc[k] = (pre * inv) * diff[k];
  if (s->image_charge) image_effect(s, p1, p2, ic);
  for (int k = 0; k < 3; ++k) ic[k] = pre * ic[k];
  icN[0] = -1.0 * ic[0]; icN[1] = -1.0 * ic[1]; icN[2] = 1.0 * ic[2];
  for (int k = 0; k < 3; ++k) {
    double vj = icN[k] * im2 - fc[k] * im2, vi = fc[k] * im1 + ic[k] * im1;
    if (comp) { nadd(&a[3 * j + k], vj); nadd(&a[3 * i + k], vi); }
    else { a[3 * j + k].s += vj; a[3 * i + k].s += vi; }
  }
}

static void tts_field(const orc_diode* s, int i, nsum* a, int comp) {
  double e[3], im1 = 1.0 / s->mass[i];
  orc_field_E(s, s->pos + 3 * i, e);
  for (int k = 0; k < 3; ++k) {
    double v = (s->charge[i] * e[k]) * im1;
    if (comp) nadd(&a[3 * i + k], v); else a[3 * i + k].s += v;
  }
}

/* Update_Particle_Acceleration :886-897 in two-time-step mode: the electron
 * pass (every electron against the later electrons and all ions, the
 * electron in the (a) role of every electron-ion pair) on every step, the
 * ion pass (ions against later ions, plus the field) on steps divisible by
 * T; both add their sums to particles_cur_accel, which the position update
 * cleared only for the particles it moved. */
void orc_accel_tts(orc_diode* s, int step, int comp) {
  init_constants();
  int n = s->n;
  nsum* a = (nsum*)calloc((size_t)3 * (n > 0 ? n : 1), sizeof(nsum));
  for (int i = 0; i < n; ++i) {           /* Update_Elec_Acceleration */
    if (s->species[i] != ORC_ELEC) continue;
    for (int j = i + 1; j < n; ++j)
      if (s->species[j] == ORC_ELEC) tts_pair(s, i, j, a, comp);
    for (int j = 0; j < n; ++j)
      if (s->species[j] == ORC_ION) tts_pair(s, i, j, a, comp);
    tts_field(s, i, a, comp);
  }
  for (int k = 0; k < 3 * n; ++k) s->acc[k] += nval(&a[k]);
  if (step % s->atom_time_interval == 0) {  /* Update_Ion_Acceleration */
    memset(a, 0, sizeof(nsum) * 3 * (size_t)n);
    for (int i = 0; i < n; ++i) {
      if (s->species[i] != ORC_ION) continue;
      for (int j = i + 1; j < n; ++j)
        if (s->species[j] == ORC_ION) tts_pair(s, i, j, a, comp);
      tts_field(s, i, a, comp);
    }
    for (int k = 0; k < 3 * n; ++k) s->acc[k] += nval(&a[k]);
  }
  free(a);
}

/* Average_Velocities :428-447: the velocity sums of the particles the update
 * moved, over nrPart / nrElec / nrIon before removal; the mobility from the
 * electrons' mean velocity. */
static void average_velocities(orc_diode* s, const double* se, const double* si) {
  int ne = 0, ni = 0;
  for (int i = 0; i < s->n; ++i) {
    if (s->species[i] == ORC_ELEC) ne++;
    else if (s->species[i] == ORC_ION) ni++;
  }
  for (int k = 0; k < 3; ++k) {
    s->avg_part_vel[k] = s->n ? (se[k] + si[k]) / s->n : 0.0;
    s->avg_elec_vel[k] = ne ? se[k] / ne : 0.0;
    s->avg_ion_vel[k] = ni ? si[k] / ni : 0.0;
  }
  double a = sqrt(s->avg_elec_vel[0] * s->avg_elec_vel[0] + s->avg_elec_vel[1] * s->avg_elec_vel[1] +
                  s->avg_elec_vel[2] * s->avg_elec_vel[2]);
  s->avg_mob = s->E_z != 0.0 ? a / (-1.0 * s->E_z) : 0.0;
  s->n_part_vel = s->n; s->n_elec_vel = ne; s->n_ion_vel = ni;
}

/* Beeman velocity and Ramo current of one particle (the loop bodies of
 * Update_ElecIon_Velocity :449-509 and Update_Species_Velocity :511-590). */
static void velocity_one(orc_diode* s, int i, double nr, nsum* ramo, nsum* ramo_ion, double* sum,
                         double* sum_ion) {
  double dt = s->time_step;
  for (int k = 0; k < 3; ++k) {
    int q = 3 * i + k;
    s->vel[q] = s->vel[q] + (((1.0 / 6.0) * ((2.0 * s->acc[q] + 5.0 * s->acc_prev[q]) -
                                              s->acc_prev2[q])) * dt) * nr;
  }
  double ez[3];
  orc_E_zunit(s, s->pos + 3 * i, ez);
  double ezv = (s->vel[3 * i] * ez[0] + s->vel[3 * i + 1] * ez[1]) + s->vel[3 * i + 2] * ez[2];
  if (s->species[i] == ORC_ELEC) {
    nadd(ramo, s->charge[i] * ezv);
    for (int k = 0; k < 3; ++k) sum[k] += s->vel[3 * i + k];
  } else if (s->species[i] == ORC_ION) {
    nadd(ramo_ion, s->charge[i] * ezv);
    for (int k = 0; k < 3; ++k) sum_ion[k] += s->vel[3 * i + k];
  }
}

void orc_update_velocity_tts(orc_diode* s, int step) {
  nsum ramo = {0, 0}, ramo_ion = {0, 0};
  double sum[3] = {0, 0, 0}, sum_ion[3] = {0, 0, 0};
  for (int i = 0; i < s->n; ++i)
    if (s->species[i] == ORC_ELEC) velocity_one(s, i, 1.0, &ramo, &ramo_ion, sum, sum_ion);
  if (step % s->atom_time_interval == 0)
    for (int i = 0; i < s->n; ++i)
      if (s->species[i] == ORC_ION)
        velocity_one(s, i, (double)s->atom_time_interval, &ramo, &ramo_ion, sum, sum_ion);
  s->ramo_current = nval(&ramo);
  s->ramo_current_ion = nval(&ramo_ion);
  average_velocities(s, sum, sum_ion);
}

/* Update_ElecIon_Velocity :449-509 + Average_Velocities :428-447 */
void orc_update_velocity(orc_diode* s) {
  double dt = s->time_step;
  nsum ramo = {0, 0}, ramo_ion = {0, 0};
  double sum[3] = {0, 0, 0}, sum_ion[3] = {0, 0, 0};
  for (int i = 0; i < s->n; ++i) {
    if (s->species[i] == ORC_ATOM) continue;
    for (int k = 0; k < 3; ++k) {
      int q = 3 * i + k;
      s->vel[q] = s->vel[q] + ((1.0 / 6.0) * ((2.0 * s->acc[q] + 5.0 * s->acc_prev[q]) -
                                               s->acc_prev2[q])) * dt;
    }
    double ez[3];
    orc_E_zunit(s, s->pos + 3 * i, ez);
    double ezv = (s->vel[3 * i] * ez[0] + s->vel[3 * i + 1] * ez[1]) + s->vel[3 * i + 2] * ez[2];
    if (s->species[i] == ORC_ELEC) {
      nadd(&ramo, s->charge[i] * ezv);
      for (int k = 0; k < 3; ++k) sum[k] += s->vel[3 * i + k];
    } else if (s->species[i] == ORC_ION) {
      nadd(&ramo_ion, s->charge[i] * ezv);
      for (int k = 0; k < 3; ++k) sum_ion[k] += s->vel[3 * i + k];
    }
  }
  s->ramo_current = nval(&ramo);
  s->ramo_current_ion = nval(&ramo_ion);
  average_velocities(s, sum, sum_ion);
}

/* Velocity_Verlet :123-162 with the gather acceleration (the GPU semantics),
 * or the two-time-step routines when atom_time_interval > 0 */
void orc_velocity_verlet(orc_diode* s, int step) {
  if (s->atom_time_interval > 0) {
    orc_update_position_tts(s, step);
    orc_accel_tts(s, step, 1);
    orc_update_velocity_tts(s, step);
    return;
  }
  orc_update_position(s);
  orc_accel_gather(s, s->acc, 1);
  orc_update_velocity(s);
}

/* ---- tip geometry: src/mod_hyperboloid_tip.f90 ------------------------------ */
void orc_tip_xyz(const orc_diode* s, double xi, double eta, double phi, double out[3]) {
  double xy = s->a_foci * sqrt((xi * xi - 1.0) * (1.0 - eta * eta));   /* xyz_corr :25-34 */
  out[0] = xy * cos(phi);
  out[1] = xy * sin(phi);
  out[2] = (s->a_foci * xi) * eta + s->shift_z;
}

void orc_tip_surface_normal(const orc_diode* s, const double p[3], double out[3]) {
  double e1 = s->eta_1;                                                 /* :78-99 */
  double eta_fac = e1 / sqrt(1.0 - e1 * e1);
  double div_fac = -1.0 / sqrt(p[0] * p[0] + p[1] * p[1] + (s->a_foci * s->a_foci) * (1.0 - e1 * e1));
  out[0] = (eta_fac * p[0]) * div_fac;
  out[1] = (eta_fac * p[1]) * div_fac;
  out[2] = 1.0;
  double nn = sqrt(out[0] * out[0] + out[1] * out[1] + out[2] * out[2]);
  for (int k = 0; k < 3; ++k) out[k] = out[k] / nn;
}

double orc_tip_area(const orc_diode* s, double xi1, double xi2, double phi1, double phi2) {
  double e2 = s->eta_1 * s->eta_1;                                       /* Tip_Area :156-163 */
  double f1 = xi1 * sqrt(xi1 * xi1 - e2) - e2 * log(xi1 + sqrt(xi1 * xi1 - e2));
  double f2 = xi2 * sqrt(xi2 * xi2 - e2) - e2 * log(xi2 + sqrt(xi2 * xi2 - e2));
  return (((0.5 * (s->a_foci * s->a_foci)) * sqrt(1.0 - e2)) * (phi2 - phi1)) * (f2 - f1);
}

static double field_normal(const orc_diode* s, const double p[3]) {
  double f[3], nrm[3];
  orc_field_at(s, p, f, 1);
  orc_tip_surface_normal(s, p, nrm);
  return (nrm[0] * f[0] + nrm[1] * f[1]) + nrm[2] * f[2];              /* Field_normal :105-112 */
}

/* ---- planar emission ------------------------------------------------------------ */
/* Gauss-Legendre nodes on [-1, 1] by Newton iteration on P_n. */
static void gauss_legendre(int n, double* x, double* w) {
  for (int k = 0; k < n; ++k) {
    double z = cos(PI * (k + 0.75) / (n + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int m = 2; m <= n; ++m) {
        double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m;
        p0 = p1; p1 = p2;
      }
      if (n == 1) { p1 = z; p0 = 1.0; }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) break;
    }
    double p0 = 1.0, p1 = z;
    for (int m = 2; m <= n; ++m) { double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m; p0 = p1; p1 = p2; }
    dp = n * (z * p1 - p0) / (z * z - 1.0);
    x[k] = -z;
    w[k] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
  if (n == 1) { x[0] = 0.0; w[0] = 2.0; }
}

/* Supply integral N_sup = int_emitter A * Elec_Supply_V2(F_z) (Do_Surface_
 * Integration_FE, src/mod_field_emission_v2.F90:635-656 with the integrand
 * integrand_cuba_fe_v :668-745), by a composite Gauss-Legendre rule in place
 * of the third-party Cuba library. */
/* Panels per side of the supply rule when none are set: Gauss-Legendre nodes at
 * most 5 nm apart along the emitter's longer side (a ring: the longer of its
 * outer circumference and its width), 16 to 256 panels -- the GPU library's
 * default rule, stated identically. */
int orc_supply_panels(const orc_diode* s) {
  if (s->quad_panels > 0) return s->quad_panels;
  int Q = s->quad_order > 0 ? s->quad_order : 4;
  double L = s->em_dim[0] > s->em_dim[1] ? s->em_dim[0] : s->em_dim[1];
  if (s->emitter_type == 4) {
    double c = 2.0 * 3.14159265358979323846 * (s->ring_rmin + s->ring_thick);
    L = c > s->ring_thick ? c : s->ring_thick;
  }
  double r = L / (Q * 5.0e-9);
  int P = (int)ceil(r * (1.0 - 1e-12));
  return P < 16 ? 16 : (P > 256 ? 256 : P);
}

double orc_supply_integral_planar(orc_diode* s) {
  int P = orc_supply_panels(s), Q = s->quad_order;
  double gx[16], gw[16];
  gauss_legendre(Q, gx, gw);
  double A = s->em_dim[0] * s->em_dim[1];
  int npt = P * Q;
  double* val = (double*)calloc((size_t)npt * npt, sizeof(double));
  double* fz = (double*)calloc((size_t)npt * 3 * npt, sizeof(double));   /* z, then x, y */
  double* fxy = fz + (size_t)npt * npt;
#pragma omp parallel for schedule(dynamic, 8)
  for (int k = 0; k < npt * npt; ++k) {
    int iy = k / npt, ix = k % npt;
    double uy = ((iy / Q) + 0.5 * (gx[iy % Q] + 1.0)) / P;
    double wy = 0.5 * gw[iy % Q] / P;
    double ux = ((ix / Q) + 0.5 * (gx[ix % Q] + 1.0)) / P;
    double wx = 0.5 * gw[ix % Q] / P;
    double p[3] = {s->em_pos[0] + ux * s->em_dim[0], s->em_pos[1] + uy * s->em_dim[1], 0.0};
    double Ak = A;
    if (s->emitter_type == 4) {   /* integrand_cuba_fe_v EMIT_RING, :701-707 */
      double angle = ux * 2.0 * PI, radius = s->ring_rmin + uy * s->ring_thick;
      p[0] = radius * cos(angle);
      p[1] = radius * sin(angle);
      Ak = 2.0 * PI * s->ring_thick * radius;
    }
    double f[3];
    orc_field_at(s, p, f, 1);
    fz[k] = f[2];
    fxy[2 * (size_t)k] = f[0];
    fxy[2 * (size_t)k + 1] = f[1];
    if (f[2] < 0.0) {
      double phi = work_at(s, p[0], p[1], NULL);
      val[k] = (wx * wy) * (Ak * orc_elec_supply_v2(f[2], phi, s->image_charge, s->time_step));
    }
  }
  nsum tot = {0, 0}, ftot = {0, 0}, fxt = {0, 0}, fyt = {0, 0};
  for (int k = 0; k < npt * npt; ++k) {
    if (val[k] != 0.0) nadd(&tot, val[k]);
    nadd(&ftot, fz[k]);
    nadd(&fxt, fxy[2 * (size_t)k]);
    nadd(&fyt, fxy[2 * (size_t)k + 1]);
  }
  s->F_avg_z = nval(&ftot) / (double)(npt * npt);   /* F_avg, fe_v2:644-651 */
  s->F_avg_x = nval(&fxt) / (double)(npt * npt);
  s->F_avg_y = nval(&fyt) / (double)(npt * npt);
  free(val); free(fz);
  return nval(&tot);
}

/* ---- converged supply integral (checker of the quadrature rules) ---------------
 * The same integrand as orc_supply_integral_planar, integrated adaptively to a
 * converged value: every panel of the P x P rule is bisected into 2 x 2
 * children while the Q x Q Gauss-Legendre sums of parent and children differ
 * by more than the panel's share of `tol` (halved at each level), and also
 * while an electron whose height h is below half the panel width lies within
 * the panel widened by 4 h -- the field of such an electron varies on the
 * scale h, below the node spacing, where no error estimate can see it.  At
 * most max_depth levels.  This stands in for the adaptive integrator of the
 * reference (Cuba Divonne, asked for max(0.5 electron, 1e-3 N_sup),
 * src/mod_global.F90:84-92) as the value a rule must reproduce. */
typedef struct {
  const orc_diode* s;
  const double* nx; const double* ny; const double* nh; int nn;   /* electrons below the cut */
  double gx[16], gw[16];
  int Q, max_depth;
  long long evals;
} adapt_ctx;

static double supply_point(const orc_diode* s, double x, double y) {
  double p[3] = {x, y, 0.0}, f[3];
  orc_field_at(s, p, f, 1);
  if (f[2] >= 0.0) return 0.0;
  double phi = work_at(s, x, y, NULL);
  return s->em_dim[0] * s->em_dim[1] * orc_elec_supply_v2(f[2], phi, s->image_charge, s->time_step);
}

/* Q x Q Gauss-Legendre sum over [x0, x0 + hx] x [y0, y0 + hy], in units of the
 * emitter area (weights as the P x P rule's) */
static double panel_sum(adapt_ctx* c, double x0, double y0, double hx, double hy) {
  const orc_diode* s = c->s;
  double t = 0.0;
  for (int iy = 0; iy < c->Q; ++iy)
    for (int ix = 0; ix < c->Q; ++ix) {
      double x = x0 + 0.5 * (c->gx[ix] + 1.0) * hx, y = y0 + 0.5 * (c->gx[iy] + 1.0) * hy;
      t += (0.25 * c->gw[ix] * c->gw[iy]) * (hx * hy) / (s->em_dim[0] * s->em_dim[1]) * supply_point(s, x, y);
      c->evals++;
    }
  return t;
}

static int panel_has_low_electron(const adapt_ctx* c, double x0, double y0, double hx, double hy) {
  double w = hx > hy ? hx : hy;
  for (int j = 0; j < c->nn; ++j) {
    double h = c->nh[j];
    if (h >= 0.5 * w) continue;
    double m = 4.0 * h;
    if (c->nx[j] >= x0 - m && c->nx[j] <= x0 + hx + m && c->ny[j] >= y0 - m && c->ny[j] <= y0 + hy + m)
      return 1;
  }
  return 0;
}

static double adapt_panel(adapt_ctx* c, double x0, double y0, double hx, double hy, double whole,
                          double tol, int depth) {
  double hx2 = 0.5 * hx, hy2 = 0.5 * hy, q[4];
  q[0] = panel_sum(c, x0, y0, hx2, hy2);
  q[1] = panel_sum(c, x0 + hx2, y0, hx2, hy2);
  q[2] = panel_sum(c, x0, y0 + hy2, hx2, hy2);
  q[3] = panel_sum(c, x0 + hx2, y0 + hy2, hx2, hy2);
  double kids = (q[0] + q[1]) + (q[2] + q[3]);
  if (depth >= c->max_depth) return kids;
  int low = panel_has_low_electron(c, x0, y0, hx, hy);
  if (!low && fabs(kids - whole) <= tol) return kids;
  double x[4] = {x0, x0 + hx2, x0, x0 + hx2}, y[4] = {y0, y0, y0 + hy2, y0 + hy2}, t = 0.0;
  for (int k = 0; k < 4; ++k) t += adapt_panel(c, x[k], y[k], hx2, hy2, q[k], 0.5 * tol, depth + 1);
  return t;
}

double orc_supply_planar_converged(orc_diode* s, double tol, int max_depth, long long* evals) {
  init_constants();
  int P = orc_supply_panels(s), Q = s->quad_order > 0 ? s->quad_order : 4;
  int n = s->n, nn = 0;
  double* buf = (double*)malloc(sizeof(double) * 3 * (n > 0 ? n : 1));
  double *nx = buf, *ny = buf + n, *nh = buf + 2 * n;
  double wmax = (s->em_dim[0] > s->em_dim[1] ? s->em_dim[0] : s->em_dim[1]) / P;
  for (int j = 0; j < n; ++j) {
    if (s->species[j] == ORC_ATOM) continue;
    double h = s->pos[3 * j + 2];
    if (h > 0.0 && h < 0.5 * wmax) { nx[nn] = s->pos[3 * j]; ny[nn] = s->pos[3 * j + 1]; nh[nn] = h; nn++; }
  }
  double hx = s->em_dim[0] / P, hy = s->em_dim[1] / P, tot = 0.0;
  long long ev = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : tot, ev)
  for (int k = 0; k < P * P; ++k) {
    adapt_ctx c;
    c.s = s; c.nx = nx; c.ny = ny; c.nh = nh; c.nn = nn; c.Q = Q; c.max_depth = max_depth; c.evals = 0;
    gauss_legendre(Q, c.gx, c.gw);
    double x0 = s->em_pos[0] + (k % P) * hx, y0 = s->em_pos[1] + (k / P) * hy;
    double whole = panel_sum(&c, x0, y0, hx, hy);
    tot += adapt_panel(&c, x0, y0, hx, hy, whole, tol / (P * P), 0);
    ev += c.evals;
  }
  free(buf);
  if (evals) *evals = ev;
  return tot;
}

static long nint_f(double x) { return (long)(x >= 0 ? floor(x + 0.5) : -floor(-x + 0.5)); }

static void mh_std_update(double* mh, double rate, double lo, double hi) {  /* :603-612 */
  *mh = *mh * exp(0.025 * (rate - 0.35));
  if (*mh > hi) *mh = hi; else if (*mh < lo) *mh = lo;
}

/* Metropolis_Hastings_rectangle_J_batch, src/mod_field_emission_v2.F90:1284-1458,
 * with check_limits_metro_rec :1466-1516.  Chains advance in lockstep and
 * MH_std gets one update per jump iteration from the batch acceptance rate. */
void orc_mh_batch_planar(orc_diode* s, int step, int M, double* df_out, double* F_out,
                         double* pos_out, int* ok) {
  int ndim = s->mh_jumps, ndim_first = (int)nint_f(ndim * 0.25);
  double* sup = (double*)malloc(sizeof(double) * (M > 0 ? M : 1));
  double std[2] = {s->em_dim[0] * 0.10, s->em_dim[1] * 0.10};
#pragma omp parallel for schedule(dynamic, 1)
  for (int c = 0; c < M; ++c) {
    ok[c] = 0;
    for (int r = 0; r < s->init_rounds_max; ++r) {
      double u1, u2;
      rng2(s->seed, c, r, step, TAG_INIT, &u1, &u2);
      double p[3] = {u1 * s->em_dim[0] + s->em_pos[0], u2 * s->em_dim[1] + s->em_pos[1], 0.0};
      double f[3];
      orc_field_at(s, p, f, 1);
      if (f[2] < 0.0) {
        pos_out[3 * c] = p[0]; pos_out[3 * c + 1] = p[1]; pos_out[3 * c + 2] = 0.0;
        F_out[c] = f[2];
        sup[c] = orc_elec_supply_log(f[2], work_at(s, p[0], p[1], NULL), s->image_charge);
        ok[c] = 1;
        break;
      }
    }
    if (!ok[c]) {
      F_out[c] = 1.0; sup[c] = -DBL_MAX;
      pos_out[3 * c] = s->em_pos[0]; pos_out[3 * c + 1] = s->em_pos[1]; pos_out[3 * c + 2] = 0.0;
    }
  }
  int any_ok = 0;
  for (int c = 0; c < M; ++c) any_ok |= ok[c];
  for (int it = 1; it <= ndim && any_ok; ++it) {
    if (it > ndim_first) { std[0] = s->em_dim[0] * s->MH_std; std[1] = s->em_dim[1] * s->MH_std; }
    int acc = 0, rej = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : acc, rej)
    for (int c = 0; c < M; ++c) {
      if (!ok[c]) continue;
      double g1, g2;
      gauss2(s->seed, c, it, step, &g1, &g2);
      double w[3] = {g1 * std[0] + pos_out[3 * c], g2 * std[1] + pos_out[3 * c + 1], 0.0};
      for (int k = 0; k < 2; ++k) {     /* check_limits_metro_rec */
        double lo = s->em_pos[k], hi = s->em_pos[k] + s->em_dim[k];
        if (w[k] > hi) w[k] = hi - (w[k] - hi);
        else if (w[k] < lo) w[k] = (lo - w[k]) + lo;
      }
      double f[3];
      orc_field_at(s, w, f, 1);
      if (f[2] >= 0.0) { rej++; continue; }
      double sn = orc_elec_supply_log(f[2], work_at(s, w[0], w[1], NULL), s->image_charge);
      double alpha = sn - sup[c];
      int take = 0;
      if (sn >= sup[c]) take = 1;
      else {
        double u1, u2;
        rng2(s->seed, c, it, step, TAG_ACCEPT, &u1, &u2);
        take = (log(u1) <= alpha);
      }
      if (take) {
        pos_out[3 * c] = w[0]; pos_out[3 * c + 1] = w[1];
        sup[c] = sn; F_out[c] = f[2]; acc++;
      } else rej++;
    }
    if (it > ndim_first && acc + rej > 0) {
      s->a_rate = (double)acc / (double)(acc + rej);
      mh_std_update(&s->MH_std, s->a_rate, 0.00005, 0.1250);
    }
  }
  for (int c = 0; c < M; ++c)
    df_out[c] = ok[c] ? orc_escape_prob_log(F_out[c], work_at(s, pos_out[3 * c], pos_out[3 * c + 1], NULL),
                                            s->image_charge)
                      : -DBL_MAX;
  free(sup);
}

/* Metropolis_Hastings_rectangle_J, src/mod_field_emission_v2.F90:1122-1265: one
 * chain run to completion against the current particles (including the ones
 * earlier chains of the step emitted); MH_std is fixed within the chain and
 * updated once from the chain's acceptance rate over the jumps after the
 * warm-up.  Same Philox counters as the batched sampler. */
static void mh_serial_chain(orc_diode* s, int step, int c, double* df_out, double* F_out, double pos[3]) {
  int ndim = s->mh_jumps, ndim_first = (int)nint_f(ndim * 0.25);
  double std[2] = {s->em_dim[0] * 0.10, s->em_dim[1] * 0.10};
  double cur[3] = {0, 0, 0}, f[3];
  int found = 0;
  for (int r = 0; r < s->init_rounds_max; ++r) {
    double u1, u2;
    rng2(s->seed, c, r, step, TAG_INIT, &u1, &u2);
    cur[0] = u1 * s->em_dim[0] + s->em_pos[0];
    cur[1] = u2 * s->em_dim[1] + s->em_pos[1];
    orc_field_at(s, cur, f, 1);
    if (f[2] < 0.0) { found = 1; break; }
  }
  if (!found) {   /* :1161-1170 */
    *F_out = 1.0; *df_out = -DBL_MAX;
    pos[0] = s->em_pos[0]; pos[1] = s->em_pos[1]; pos[2] = 0.0;
    return;
  }
  *F_out = f[2];
  double sup_cur = orc_elec_supply_log(f[2], work_at(s, cur[0], cur[1], NULL), s->image_charge);
  int ja = 0, jr = 0;
  for (int i = 1; i <= ndim; ++i) {
    if (i > ndim_first) { std[0] = s->em_dim[0] * s->MH_std; std[1] = s->em_dim[1] * s->MH_std; }
    double g1, g2;
    gauss2(s->seed, c, i, step, &g1, &g2);
    double w[3] = {g1 * std[0] + cur[0], g2 * std[1] + cur[1], 0.0};
    for (int k = 0; k < 2; ++k) {     /* check_limits_metro_rec */
      double lo = s->em_pos[k], hi = s->em_pos[k] + s->em_dim[k];
      if (w[k] > hi) w[k] = hi - (w[k] - hi);
      else if (w[k] < lo) w[k] = (lo - w[k]) + lo;
    }
    orc_field_at(s, w, f, 1);
    if (f[2] >= 0.0) { if (i > ndim_first) jr++; continue; }
    double sn = orc_elec_supply_log(f[2], work_at(s, w[0], w[1], NULL), s->image_charge);
    double alpha = sn - sup_cur;
    int take = 0;
    if (sn >= sup_cur) take = 1;
    else {
      double u1, u2;
      rng2(s->seed, c, i, step, TAG_ACCEPT, &u1, &u2);
      take = (log(u1) <= alpha);
    }
    if (take) {
      cur[0] = w[0]; cur[1] = w[1]; sup_cur = sn; *F_out = f[2];
      if (i > ndim_first) ja++;
    } else if (i > ndim_first) jr++;
  }
  if (ja + jr > 0) {   /* :1251-1254 */
    s->a_rate = (double)ja / (double)(jr + ja);
    mh_std_update(&s->MH_std, s->a_rate, 0.00005, 0.1250);
  }
  pos[0] = cur[0]; pos[1] = cur[1]; pos[2] = 0.0;
  *df_out = orc_escape_prob_log(*F_out, work_at(s, cur[0], cur[1], NULL), s->image_charge);
}

/* Metropolis_Hastings_ring_J, :1521-1685: the chain moves in (angle, radius)
 * of the ring; proposals off the ring are rejected; log(radius) is added to
 * the target (the Jacobian).  MH_std updated once per chain. */
static void mh_ring_chain(orc_diode* s, int step, int c, double* df_out, double* F_out, double pos[3]) {
  int ndim = s->mh_jumps, ndim_first = (int)nint_f(ndim * 0.25);
  double r_min = s->ring_rmin, r_max = s->ring_rmin + s->ring_thick;
  double std[2] = {2.0 * PI * 0.10, s->ring_thick * 0.10};
  double cur[3] = {0, 0, 0}, f[3], ca = 0.0, cr = r_min;
  int found = 0;
  for (int r = 0; r < s->init_rounds_max; ++r) {
    double u1, u2;
    rng2(s->seed, c, r, step, TAG_INIT, &u1, &u2);
    ca = u1 * 2.0 * PI;
    cr = r_min + u2 * s->ring_thick;
    cur[0] = cr * cos(ca);
    cur[1] = cr * sin(ca);
    orc_field_at(s, cur, f, 1);
    if (f[2] < 0.0) { found = 1; break; }
  }
  if (!found) {
    *F_out = 1.0; *df_out = -DBL_MAX;
    pos[0] = r_min; pos[1] = 0.0; pos[2] = 0.0;
    return;
  }
  *F_out = f[2];
  double sup_cur = orc_elec_supply_log(f[2], work_at(s, cur[0], cur[1], NULL), s->image_charge) + log(cr);
  int ja = 0, jr = 0;
  for (int i = 1; i <= ndim; ++i) {
    if (i > ndim_first) { std[0] = 2.0 * PI * s->MH_std; std[1] = s->ring_thick * s->MH_std; }
    double g1, g2;
    gauss2(s->seed, c, i, step, &g1, &g2);
    double a = g1 * std[0] + ca;
    double na = a - floor(a / (2.0 * PI)) * (2.0 * PI), nr = g2 * std[1] + cr;
    if (nr < r_min || nr > r_max) { if (i > ndim_first) jr++; continue; }
    double w[3] = {nr * cos(na), nr * sin(na), 0.0};
    orc_field_at(s, w, f, 1);
    if (f[2] >= 0.0) { if (i > ndim_first) jr++; continue; }
    double sn = orc_elec_supply_log(f[2], work_at(s, w[0], w[1], NULL), s->image_charge) + log(nr);
    double alpha = sn - sup_cur;
    int take = 0;
    if (sn >= sup_cur) take = 1;
    else {
      double u1, u2;
      rng2(s->seed, c, i, step, TAG_ACCEPT, &u1, &u2);
      take = (log(u1) <= alpha);
    }
    if (take) {
      cur[0] = w[0]; cur[1] = w[1]; ca = na; cr = nr; sup_cur = sn; *F_out = f[2];
      if (i > ndim_first) ja++;
    } else if (i > ndim_first) jr++;
  }
  if (ja + jr > 0) {
    s->a_rate = (double)ja / (double)(jr + ja);
    mh_std_update(&s->MH_std, s->a_rate, 0.00005, 0.1250);
  }
  pos[0] = cur[0]; pos[1] = cur[1]; pos[2] = 0.0;
  *df_out = orc_escape_prob_log(*F_out, work_at(s, cur[0], cur[1], NULL), s->image_charge);
}

/* The serial branch of Do_Field_Emission_Planar_rectangle (:322-333, 338-383)
 * and Do_Field_Emission_Planar_ring (:399-505): each candidate's chain, its
 * emission test and its Add_Particle before the next candidate's chain. */
static int emission_planar_serial(orc_diode* s, int step, int M) {
  int emitted = 0;
  double df_sum = 0.0;
  for (int c = 0; c < M; ++c) {
    double D, F, p[3];
    if (s->emitter_type == 4) mh_ring_chain(s, step, c, &D, &F, p);
    else mh_serial_chain(s, step, c, &D, &F, p);
    if (F >= 0.0) {
      D = -DBL_MAX;
      if (s->emitter_type == 4) break;   /* Do_Field_Emission_Planar_ring exits here, :447-455 */
    }
    df_sum += exp(D);
    double u1, u2;
    rng2(s->seed, c, 0, step, TAG_EMIT, &u1, &u2);
    if (log(u1) <= D) {
      double q[3] = {p[0], p[1], 1.0 * LENGTH_SCALE}, v[3] = {0, 0, 0};
      int sec = 1;
      work_at(s, q[0], q[1], &sec);
      if (orc_add_particle(s, q, v, ORC_ELEC, step, sec) >= 0) emitted++;
    }
  }
  s->df_avg = s->N_sup > 0.0 ? df_sum / s->N_sup : 0.0;
  s->emitted_step = emitted;
  s->emitted_total += emitted;
  return emitted;
}

/* Do_Field_Emission_Planar_rectangle, src/mod_field_emission_v2.F90:261-395 */
int orc_do_emission_planar(orc_diode* s, int step) {
  double N_sup = orc_supply_integral_planar(s);
  s->N_sup = N_sup;
  long N_round = nint_f(N_sup + s->residual);
  s->residual = N_sup - (double)N_round;
  int M = N_round > 0 ? (int)N_round : 0;
  if (M > s->max_chains) M = s->max_chains;
  s->last_chains = M;
  s->emitted_step = 0;
  s->df_avg = 0.0;
  if (M == 0) return 0;
  if (s->mh_serial) return emission_planar_serial(s, step, M);
  double* df = (double*)malloc(sizeof(double) * M);
  double* F = (double*)malloc(sizeof(double) * M);
  double* P = (double*)malloc(sizeof(double) * 3 * M);
  int* ok = (int*)malloc(sizeof(int) * M);
  orc_mh_batch_planar(s, step, M, df, F, P, ok);
  int emitted = 0, failed = 0;
  double df_sum = 0.0;
  for (int c = 0; c < M; ++c) {
    double D = df[c];
    if (!ok[c]) failed++;
    if (F[c] >= 0.0) D = -DBL_MAX;
    df_sum += exp(D);   /* df_avg, :354 */
    double u1, u2;
    rng2(s->seed, c, 0, step, TAG_EMIT, &u1, &u2);
    if (log(u1) <= D) {
      double p[3] = {P[3 * c], P[3 * c + 1], 1.0 * LENGTH_SCALE}, v[3] = {0, 0, 0};
      int sec = 1;
      work_at(s, p[0], p[1], &sec);
      if (orc_add_particle(s, p, v, ORC_ELEC, step, sec) >= 0) emitted++;
    }
  }
  s->last_failed_chains = failed;
  s->df_avg = N_sup > 0.0 ? df_sum / N_sup : 0.0;   /* :385 */
  free(df); free(F); free(P); free(ok);
  s->emitted_step = emitted;
  s->emitted_total += emitted;
  return emitted;
}

/* ---- tip emission: src/mod_emission_tip.f90:417-534 (supply grid) and
 *      Metro_algo_tip_v3 :1241-1390 run as a lockstep batch ----------------- */
static double tip_supply_log_target(const orc_diode* s, double F, double xi) {
  double t = orc_t_y(F, s->tip_phi, s->image_charge);
  double sup = (((s->time_step / Q_0) * A_FN) / ((t * t) * s->tip_phi)) * (F * F);
  double v = sup > DBL_MIN ? sup : DBL_MIN;       /* Tip_fe_target_log :1213-1219 */
  return log(v) + 0.5 * log(xi * xi - s->eta_1 * s->eta_1);
}

double orc_supply_tip(orc_diode* s) {
  const int nr = 100;
  double len_phi = 2.0 * PI / nr, len_xi = (s->max_xi - 1.0) / nr;
  double* val = (double*)calloc((size_t)nr * nr, sizeof(double));
#pragma omp parallel for schedule(dynamic, 8)
  for (int k = 0; k < nr * nr; ++k) {
    int i = k / nr + 1, j = k % nr + 1;
    double xi_c = 1.0 + (i - 0.5) * len_xi, phi_c = (j - 0.5) * len_phi;
    double p[3];
    orc_tip_xyz(s, xi_c, s->eta_1, phi_c, p);
    double F = field_normal(s, p);
    if (F < 0.0) {
      double A = orc_tip_area(s, 1.0 + (i - 1.0) * len_xi, 1.0 + (i + 0.0) * len_xi,
                              (j - 1.0) * len_phi, (j + 0.0) * len_phi);
      double t = orc_t_y(F, s->tip_phi, s->image_charge);       /* Elec_Supply :1710-1718 */
      val[k] = (((A * A_FN) * (F * F)) * s->time_step) / ((Q_0 * s->tip_phi) * (t * t));
    }
  }
  nsum ns = {0, 0};
  for (int k = 0; k < nr * nr; ++k) if (val[k] != 0.0) nadd(&ns, val[k]);
  free(val);
  return nval(&ns);
}

void orc_mh_batch_tip(orc_diode* s, int step, int M, double* df_out, double* F_out,
                      double* pos_out, int* ok) {
  int ndim = s->mh_jumps, ndim_first = (int)nint_f(ndim * 0.25);
  const double lo = 0.0005, hi = 0.125;
  if (s->MH_std > hi) s->MH_std = hi; else if (s->MH_std < lo) s->MH_std = lo;
  double* sup = (double*)malloc(sizeof(double) * (M > 0 ? M : 1));
  double* xi = (double*)malloc(sizeof(double) * (M > 0 ? M : 1));
  double* ph = (double*)malloc(sizeof(double) * (M > 0 ? M : 1));
  double std[2] = {(s->max_xi - 1.0) * 0.10, (2.0 * PI) * 0.10};
#pragma omp parallel for schedule(dynamic, 1)
  for (int c = 0; c < M; ++c) {
    ok[c] = 0;
    for (int r = 0; r < s->init_rounds_max; ++r) {
      double u1, u2;
      rng2(s->seed, c, r, step, TAG_INIT, &u1, &u2);
      double x = 1.0 + (s->max_xi - 1.0) * u1, f = (2.0 * PI) * u2, p[3];
      orc_tip_xyz(s, x, s->eta_1, f, p);
      double F = field_normal(s, p);
      if (F < 0.0) {
        xi[c] = x; ph[c] = f; F_out[c] = F;
        for (int k = 0; k < 3; ++k) pos_out[3 * c + k] = p[k];
        sup[c] = tip_supply_log_target(s, F, x);
        ok[c] = 1;
        break;
      }
    }
    if (!ok[c]) {
      xi[c] = 1.0; ph[c] = 0.0; F_out[c] = 1.0; sup[c] = -DBL_MAX;
      orc_tip_xyz(s, 1.0, s->eta_1, 0.0, pos_out + 3 * c);
    }
  }
  int any_ok = 0;
  for (int c = 0; c < M; ++c) any_ok |= ok[c];
  for (int it = 1; it <= ndim && any_ok; ++it) {
    if (it > ndim_first) { std[0] = (s->max_xi - 1.0) * s->MH_std; std[1] = (2.0 * PI) * s->MH_std; }
    int acc = 0, rej = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : acc, rej)
    for (int c = 0; c < M; ++c) {
      if (!ok[c]) continue;
      double g1, g2;
      gauss2(s->seed, c, it, step, &g1, &g2);
      double nxi = xi[c] + g1 * std[0];
      double a = ph[c] + g2 * std[1], twopi = 2.0 * PI;
      double nph = a - floor(a / twopi) * twopi;     /* Fortran MODULO */
      if (nxi > s->max_xi) nxi = 2.0 * s->max_xi - nxi;
      if (nxi < 1.0) nxi = 2.0 - nxi;
      if (nxi < 1.0 || nxi > s->max_xi) { rej++; continue; }
      double p[3];
      orc_tip_xyz(s, nxi, s->eta_1, nph, p);
      double F = field_normal(s, p);
      if (F >= 0.0) { rej++; continue; }
      double sn = tip_supply_log_target(s, F, nxi);
      int take = 0;
      if (sn >= sup[c]) take = 1;
      else {
        double u1, u2;
        rng2(s->seed, c, it, step, TAG_ACCEPT, &u1, &u2);
        take = (log(u1) <= sn - sup[c]);
      }
      if (take) {
        xi[c] = nxi; ph[c] = nph; F_out[c] = F; sup[c] = sn;
        for (int k = 0; k < 3; ++k) pos_out[3 * c + k] = p[k];
        acc++;
      } else rej++;
    }
    if (it > ndim_first && acc + rej > 0) {
      s->a_rate = (double)acc / (double)(acc + rej);
      mh_std_update(&s->MH_std, s->a_rate, lo, hi);
    }
  }
  for (int c = 0; c < M; ++c) {
    if (ok[c]) {   /* Escape_Prob_Tip :1734-1758 */
      double sq = sqrt(s->tip_phi);
      df_out[c] = exp(((B_FN * ((sq * sq) * sq)) * orc_v_y(F_out[c], s->tip_phi, s->image_charge)) / fabs(F_out[c]));
    } else df_out[c] = 0.0;
  }
  free(sup); free(xi); free(ph);
}

int orc_do_emission_tip(orc_diode* s, int step) {
  double n_s = orc_supply_tip(s);
  s->N_sup = n_s;
  long n_r = nint_f(n_s);
  int M = n_r > 0 ? (int)n_r : 0;
  if (M > s->max_chains) M = s->max_chains;
  s->last_chains = M;
  s->emitted_step = 0;
  if (M == 0) return 0;
  double* df = (double*)malloc(sizeof(double) * M);
  double* F = (double*)malloc(sizeof(double) * M);
  double* P = (double*)malloc(sizeof(double) * 3 * M);
  int* ok = (int*)malloc(sizeof(int) * M);
  orc_mh_batch_tip(s, step, M, df, F, P, ok);
  int emitted = 0, failed = 0;
  for (int c = 0; c < M; ++c) {
    if (!ok[c]) failed++;
    double u1, u2;
    rng2(s->seed, c, 0, step, TAG_EMIT, &u1, &u2);
    if (F[c] < 0.0 && u1 <= df[c]) {
      double nrm[3], p[3], v[3] = {0, 0, 0};
      orc_tip_surface_normal(s, P + 3 * c, nrm);
      for (int k = 0; k < 3; ++k) p[k] = P[3 * c + k] + nrm[k] * LENGTH_SCALE;
      if (orc_add_particle(s, p, v, ORC_ELEC, step, 1) >= 0) emitted++;
    }
  }
  s->last_failed_chains = failed;
  free(df); free(F); free(P); free(ok);
  s->emitted_step = emitted;
  s->emitted_total += emitted;
  return emitted;
}

int orc_do_emission(orc_diode* s, int step) {
  if (!s->emission) { s->emitted_step = 0; return 0; }
  if (step <= s->emit_delay) {   /* emitters_delay(i) < step, fe_v2:181 */
    s->emitted_step = 0; s->N_sup = 0.0; s->last_chains = 0; s->F_avg_z = 0.0; s->df_avg = 0.0;
    s->F_avg_x = 0.0; s->F_avg_y = 0.0;
    return 0;
  }
  return s->geometry == ORC_TIP ? orc_do_emission_tip(s, step) : orc_do_emission_planar(s, step);
}

void orc_step(orc_diode* s, int step) {
  orc_do_emission(s, step);
  orc_velocity_verlet(s, step);
  orc_remove_particles(s, step);
}

/* ---- CPU baseline: OpenMP half-pair planar loop ----------------------------- */
int orc_omp_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_accel_planar_omp(int n, const double* pos, const double* charge, const double* mass,
                          double Ez, double d, int ic, int Nic, double* acc) {
  init_constants();
  int nt = orc_omp_threads();
  double* part = (double*)calloc((size_t)nt * 3 * (n > 0 ? n : 1), sizeof(double));
#pragma omp parallel
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
#else
    int tid = 0;
#endif
    double* a = part + (size_t)tid * 3 * n;
#pragma omp for schedule(dynamic, 1)
    for (int i = 0; i < n; ++i) {
      double x1 = pos[3 * i], y1 = pos[3 * i + 1], z1 = pos[3 * i + 2];
      double q1 = charge[i], qd1 = q1 * DIV_FAC_C, im1 = 1.0 / mass[i];
      double ax = 0, ay = 0, az = 0;
      for (int j = i + 1; j < n; ++j) {
        double pre = qd1 * charge[j], im2 = 1.0 / mass[j];
        double dx = x1 - pos[3 * j], dy = y1 - pos[3 * j + 1], dz = z1 - pos[3 * j + 2];
        double dxy2 = dx * dx + dy * dy;
        double r = sqrt(dxy2 + dz * dz) + L2, inv = 1.0 / ((r * r) * r);
        double fcx = (pre * inv) * dx, fcy = (pre * inv) * dy, fcz = (pre * inv) * dz;
        double icx = 0, icy = 0, icz = 0;
        if (ic) {
          double zb = pos[3 * j + 2], dzi = z1 + zb;
          r = sqrt(dxy2 + dzi * dzi) + L2; inv = 1.0 / ((r * r) * r);
          icx = -dx * inv; icy = -dy * inv; icz = -dzi * inv;
          for (int m = 1; m <= Nic; ++m) {
            double zz[4] = {(2.0 * m) * d - zb, (-2.0 * m) * d - zb, (2.0 * m) * d + zb, (-2.0 * m) * d + zb};
            for (int k = 0; k < 4; ++k) {
              dzi = z1 - zz[k];
              r = sqrt(dxy2 + dzi * dzi) + L2; inv = 1.0 / ((r * r) * r);
              double sg = k < 2 ? -1.0 : 1.0;
              icx += sg * dx * inv; icy += sg * dy * inv; icz += sg * dzi * inv;
            }
          }
        }
        ax += fcx + pre * icx; ay += fcy + pre * icy; az += fcz + pre * icz;
        a[3 * j] += im2 * (-pre * icx - fcx);
        a[3 * j + 1] += im2 * (-pre * icy - fcy);
        a[3 * j + 2] += im2 * (pre * icz - fcz);
      }
      a[3 * i] += ax * im1; a[3 * i + 1] += ay * im1; a[3 * i + 2] += (az + q1 * Ez) * im1;
    }
  }
  for (int i = 0; i < 3 * n; ++i) {
    double v = 0;
    for (int t = 0; t < nt; ++t) v += part[(size_t)t * 3 * n + i];
    acc[i] = v;
  }
  free(part);
}
