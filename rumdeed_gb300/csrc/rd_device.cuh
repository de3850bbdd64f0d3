// rd_device.cuh -- device helpers of librumdeed_gb300: physical constants,
// the Philox4x32-10 counter RNG, the Fowler-Nordheim functions, the
// checkerboard work function and the hyperboloid tip geometry.  Every
// formula cites the reference routine (NanoPhysicsCenter/RUMDEED, src/...)
// whose result it reproduces.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "rd_internal.h"
#include "rd_split.h"

// Each translation unit holds its own copy of the constants (no relocatable
// device code); rd_upload_constants_<unit>() fills it at engine creation.
static __constant__ RdConst c_k;
#define RD_DEFINE_CONSTANT_UPLOAD(unit)                                   \
  cudaError_t rd_upload_constants_##unit(const RdConst& k) {              \
    return cudaMemcpyToSymbol(c_k, &k, sizeof(RdConst));                  \
  }

#define RD_HD __host__ __device__ __forceinline__

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) ----------------------
RD_HD void philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                      uint32_t k1, uint32_t out[4]) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    c1 = (uint32_t)p1;
    c3 = (uint32_t)p0;
    c0 = n0;
    c2 = n2;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

RD_HD double u01_words(uint32_t a, uint32_t b) {
  uint64_t m = ((uint64_t)a << 21) ^ (uint64_t)(b >> 11);
  return (double)(m & ((1ull << 53) - 1)) * (1.0 / 9007199254740992.0);
}

enum { RNG_INIT = 1, RNG_GAUSS = 2, RNG_ACCEPT = 3, RNG_EMIT = 4 };

RD_HD void rng2(unsigned long long seed, uint32_t a, uint32_t b, uint32_t step, uint32_t tag,
                double* u1, double* u2) {
  uint32_t o[4];
  philox4x32(a, b, step, tag, (uint32_t)seed, (uint32_t)(seed >> 32), o);
  *u1 = u01_words(o[0], o[1]);
  *u2 = u01_words(o[2], o[3]);
}

// box_muller, Marsaglia polar form (src/mod_global.F90:578-595); the attempt
// index of the rejection loop is part of the counter.
__device__ __forceinline__ void gauss2(unsigned long long seed, uint32_t chain, uint32_t it,
                                       uint32_t step, double* g1, double* g2) {
  for (uint32_t k = 0; k < 64; ++k) {
    double u1, u2;
    rng2(seed, chain, it, step, RNG_GAUSS | (k << 8), &u1, &u2);
    double x1 = 2.0 * u1 - 1.0, x2 = 2.0 * u2 - 1.0;
    double w = x1 * x1 + x2 * x2;
    if (w < 1.0 && w > 0.0) {
      double f = sqrt((-2.0 * log(w)) / w);
      *g1 = x1 * f;
      *g2 = x2 * f;
      return;
    }
  }
  *g1 = 0.0;
  *g2 = 0.0;
}

// ---- Fowler-Nordheim functions (src/mod_field_emission_v2.F90:515-625) ------
__device__ __forceinline__ double fn_v_y(double F, double phi, int ic) {
  if (!ic) return 1.0;
  double l = (c_k.l_const * (-1.0 * F)) / (phi * phi);
  if (l > 1.0) l = 1.0;
  return (1.0 - l) + ((1.0 / 6.0) * l) * log(l);
}
__device__ __forceinline__ double fn_t_y(double F, double phi, int ic) {
  if (!ic) return 1.0;
  double l = (c_k.l_const * (-1.0 * F)) / (phi * phi);
  if (l > 1.0) l = 1.0;
  return 1.0 + l * ((1.0 / 9.0) - (1.0 / 18.0) * log(l));
}
__device__ __forceinline__ double fn_escape_log(double F, double phi, int ic) {
  double s = sqrt(phi);
  return ((c_k.b_FN * ((s * s) * s)) * fn_v_y(F, phi, ic)) / (-1.0 * F);
}
__device__ __forceinline__ double fn_supply_log(double F, double phi, int ic) {
  return (2.0 * log(-1.0 * F) - 2.0 * log(fn_t_y(F, phi, ic))) - log(phi);
}
__device__ __forceinline__ double fn_supply_v2(double F, double phi, int ic, double dt) {
  double t = fn_t_y(F, phi, ic);
  return (((dt / c_k.q0) * c_k.a_FN) / ((t * t) * phi)) * (F * F);
}

// ---- work-function models (src/mod_work_function.F90) ----------------------
// Voronoi site closest to (x, y) (w_theta_voronoi :533-571): sites stored as
// (x, y) fractions of the emitter, phi, section; converted like
// Read_work_function (:124-134).  The start distance is the reference's
// single-precision literal 9.9E10.
__device__ __forceinline__ int voronoi_site(const DiodeParams& P, const double* w, double x, double y) {
  int k = 0;
  double d = (double)9.9e10f;
  for (int i = 0; i < P.work_nx; ++i) {
    const double sx = P.em_x0 + w[4 * i] * P.em_Lx, sy = P.em_y0 + w[4 * i + 1] * P.em_Ly;
    const double dp = (x - sx) * (x - sx) + (y - sy) * (y - sy);
    if (dp < d) { k = i; d = dp; }
  }
  return k;
}

// w_theta_gaussian (:214-254): base + sum A exp(-((x-xc)^2/(2 sx^2) + (y-yc)^2/(2 sy^2))),
// centres and widths in nm.
__device__ __forceinline__ double gaussian_work(const DiodeParams& P, const double* w, double x, double y) {
  double v = w[0];
  for (int i = 0; i < P.work_nx; ++i) {
    const double* g = w + 1 + 5 * i;
    const double xc = g[1] * c_k.length_scale, yc = g[2] * c_k.length_scale;
    const double sx = g[3] * c_k.length_scale, sy = g[4] * c_k.length_scale;
    v = v + g[0] * exp(-1.0 * (((x - xc) * (x - xc)) / (2.0 * (sx * sx)) + ((y - yc) * (y - yc)) / (2.0 * (sy * sy))));
  }
  return v;
}

// The work function at (x, y) and its section (ptr_Work_fun): checkerboard
// (w_theta_checkerboard :389-487), Gaussian (section 1) or Voronoi.
__device__ __forceinline__ double work_at(const DiodeParams& P, const double* work, double x,
                                          double y, int* sec) {
  const double* w = work + P.work_off;
  if (P.work_model == 2) {
    if (sec) *sec = 1;
    return gaussian_work(P, w, x, y);
  }
  if (P.work_model == 4) {
    const int k = voronoi_site(P, w, x, y);
    if (sec) *sec = (int)w[4 * k + 3];
    return w[4 * k + 2];
  }
  double xs = (x - P.em_x0) / P.em_Lx, ys = (y - P.em_y0) / P.em_Ly;
  int nx = P.work_nx, ny = P.work_ny;
  int xi = (int)floor(xs / (1.0 / nx)) + 1, yi = (int)floor(ys / (1.0 / ny)) + 1;
  xi = xi > nx ? nx : (xi < 1 ? 1 : xi);
  yi = yi > ny ? ny : (yi < 1 ? 1 : yi);
  if (sec) *sec = nx * (yi - 1) + xi;
  yi = ny - yi + 1;
  return w[(yi - 1) * nx + (xi - 1)];
}

// ---- hyperboloid tip (src/mod_hyperboloid_tip.f90) ---------------------------
// field_E_Hyperboloid :115-154
__host__ __device__ __forceinline__ void tip_field_E(const DiodeParams& P, double x, double y, double z,
                                            double* ex, double* ey, double* ez) {
  double a = P.a_foci, sz = P.shift_z;
  double rp = sqrt(x * x + y * y + ((z + a) - sz) * ((z + a) - sz));
  double rm = sqrt(x * x + y * y + ((z - a) - sz) * ((z - a) - sz));
  double xi = (1.0 / (2.0 * a)) * (rp + rm);
  double eta = (1.0 / (2.0 * a)) * (rp - rm);
  double phi = (fabs(x) < 1.0e-18 && fabs(y) < 1.0e-18) ? 0.0 : atan2(y, x);
  double pre = P.pre_E * (1.0 / (xi * xi - eta * eta));
  double fac = (fabs(xi - 1.0) < 1.0e-6) ? 0.0 : eta * sqrt((xi * xi - 1.0) / (1.0 - eta * eta));
  *ex = ((-1.0 * pre) * fac) * cos(phi);
  *ey = ((-1.0 * pre) * fac) * sin(phi);
  *ez = pre * xi;
}
// eta_coor :62-67
__device__ __forceinline__ double tip_eta(const DiodeParams& P, double x, double y, double z) {
  double a = P.a_foci, sz = P.shift_z;
  return (1.0 / (2.0 * a)) * (sqrt(x * x + y * y + ((z + a) - sz) * ((z + a) - sz)) -
                              sqrt(x * x + y * y + ((z - a) - sz) * ((z - a) - sz)));
}
// xyz_corr :25-34
__device__ __forceinline__ void tip_xyz(const DiodeParams& P, double xi, double eta, double phi,
                                        double* x, double* y, double* z) {
  double xy = P.a_foci * sqrt((xi * xi - 1.0) * (1.0 - eta * eta));
  *x = xy * cos(phi);
  *y = xy * sin(phi);
  *z = (P.a_foci * xi) * eta + P.shift_z;
}
// surface_normal :78-99
__device__ __forceinline__ void tip_normal(const DiodeParams& P, double x, double y, double* nx,
                                           double* ny, double* nz) {
  double e1 = P.eta_1;
  double eta_fac = e1 / sqrt(1.0 - e1 * e1);
  double div_fac = -1.0 / sqrt(x * x + y * y + (P.a_foci * P.a_foci) * (1.0 - e1 * e1));
  double a = (eta_fac * x) * div_fac, b = (eta_fac * y) * div_fac, c = 1.0;
  double nn = sqrt(a * a + b * b + c * c);
  *nx = a / nn; *ny = b / nn; *nz = c / nn;
}
// Tip_Area :156-163
__device__ __forceinline__ double tip_area(const DiodeParams& P, double xi1, double xi2,
                                           double phi1, double phi2) {
  double e2 = P.eta_1 * P.eta_1;
  double f1 = xi1 * sqrt(xi1 * xi1 - e2) - e2 * log(xi1 + sqrt(xi1 * xi1 - e2));
  double f2 = xi2 * sqrt(xi2 * xi2 - e2) - e2 * log(xi2 + sqrt(xi2 * xi2 - e2));
  return (((0.5 * (P.a_foci * P.a_foci)) * sqrt(1.0 - e2)) * (phi2 - phi1)) * (f2 - f1);
}
// Image point of a charge at (xa, ya, za) in the apex sphere
// (acc_tip_image_point.inc:14-18).  Returns dis_a.
__device__ __forceinline__ double tip_image_point(const DiodeParams& P, double xa, double ya,
                                                  double za, double* xi, double* yi,
                                                  double* zi) {
  double z0 = P.h_tip - P.r_tip, R = P.r_tip;
  double dza = za - z0;
  double dis = sqrt(xa * xa + ya * ya + dza * dza);
  double zb = z0 + (R * R) / (sqrt((1.0 + (xa * xa) / (dza * dza)) + (ya * ya) / (dza * dza)) * dis);
  *xi = ((zb - z0) * xa) / dza;
  *yi = ((zb - z0) * ya) / dza;
  *zi = zb;
  return dis;
}

// Vacuum field of the geometry at a point (ptr_field_E).
__device__ __forceinline__ void vacuum_field(const DiodeParams& P, double x, double y, double z,
                                             double* ex, double* ey, double* ez) {
  if (P.geometry == RD_G_TIP) {
    tip_field_E(P, x, y, z, ex, ey, ez);
  } else {
    *ex = 0.0; *ey = 0.0; *ez = P.E_z;
  }
}

// ---- FP32 frame ---------------------------------------------------------------
// Position in nm split into a high float and the float of the remainder
// (hi = (float)v, lo = (float)(v - hi); formed from the bits, rd_split.h).
__device__ __forceinline__ void split_nm(double v_m, double origin_m, float* hi, float* lo) {
  rd_split_exact((v_m - origin_m) * 1.0e9, hi, lo);
}

// Append one record to the event log (no-op without a log).
__device__ __forceinline__ void log_event(const EventLog& L, double x, double y, double z, double vx,
                                          double vy, double vz, int diode, int kind, int section,
                                          int id, int species, int step) {
  if (!L.buf) return;
  const int k = atomicAdd(L.count, 1);
  if (k >= L.cap) return;
  rd_event& r = L.buf[k];
  r.pos[0] = x; r.pos[1] = y; r.pos[2] = z;
  r.vel[0] = vx; r.vel[1] = vy; r.vel[2] = vz;
  r.diode = diode; r.kind = kind; r.section = section; r.id = id; r.species = species; r.step = step;
}

// Knuth two-sum accumulation of a float into a (hi, lo) pair.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float v) {
  float s = hi + v;
  float bp = s - hi;
  float err = (hi - (s - bp)) + (v - bp);
  hi = s;
  lo += err;
}

// (hi, lo) += (h, l) for float pairs: the two-sum of the high parts, the low
// parts and its error added, then renormalised (fast two-sum), so that
// lo stays below an ulp of hi.  Sums of chunk partials in chunk order.
__device__ __forceinline__ void pair_add(float& hi, float& lo, float h, float l) {
  const float s = hi + h;
  const float bp = s - hi;
  const float err = (hi - (s - bp)) + (h - bp);
  const float t = (lo + l) + err;
  hi = s + t;
  lo = t - (hi - s);
}
