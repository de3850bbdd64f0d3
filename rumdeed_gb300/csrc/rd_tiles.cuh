// rd_tiles.cuh -- per-pair arithmetic of one shared-memory j-tile, shared by
// the force kernels (i = particle) and the field kernels (i = evaluation
// point, always in the upper role: the point images / is imaged as the "a"
// argument of the reference image functions).
#pragma once
#include "rd_pair.cuh"

enum { T_UPPER = 0, T_LOWER = 1, T_DIAG = 2 };

struct F32Acc {
  float hx, lx, hy, ly, hz, lz;
  __device__ void zero() { hx = lx = hy = ly = hz = lz = 0.f; }
  __device__ void add(float tx, float ty, float tz) {
    two_sum_acc(hx, lx, tx);
    two_sum_acc(hy, ly, ty);
    two_sum_acc(hz, lz, tz);
  }
};

// ---- planar, FP32 compensated ------------------------------------------------
// One j-tile against the thread's particle i.  NIC0: N_ic_max == 0 fast path.
// ELEC (tiles whose charges are all -1, the electrons' q/q0; not the
// diagonal tile): the charge is a constant, so its multiplies fold into signs.
template <int MODE, bool NIC0, bool ELEC = false>
__device__ __forceinline__ void planar_tile_f32(const float4* __restrict__ sh, const float4* __restrict__ sl,
                                                int kmax, float4 ih, float4 il, int self_k,
                                                int nic, float dnm, int ic, float& tx,
                                                float& ty, float& tz) {
  float sx = 0.f, sy = 0.f, sz = 0.f, szs = 0.f;
#pragma unroll 4
  for (int k = 0; k < kmax; ++k) {
    float4 h = sh[k], l = sl[k];
    float q = ELEC ? -1.f : h.w;
    if (MODE == T_DIAG) q = (k == self_k) ? 0.f : q;
    float dx = (ih.x - h.x) + (il.x - l.x);
    float dy = (ih.y - h.y) + (il.y - l.y);
    float dz = (ih.z - h.z) + (il.z - l.z);
    float dxy2 = fmaf(dx, dx, dy * dy);
    float r2 = fmaf(dz, dz, dxy2);
    float inv = rsqrtf(fmaxf(r2, 1e-20f));
    float s = q * (inv * inv) * inv;
    sx = fmaf(s, dx, sx);
    sy = fmaf(s, dy, sy);
    sz = fmaf(s, dz, sz);
    if (ic) {
      // n = 0 partner at -z_b: dz = z_a + z_b (symmetric in the roles)
      float zs = (ih.z + h.z) + (il.z + l.z);
      float ri = rsqrtf(fmaxf(fmaf(zs, zs, dxy2), 1e-20f));
      float si = q * (ri * ri) * ri;
      sx = fmaf(-si, dx, sx);
      sy = fmaf(-si, dy, sy);
      sz = fmaf(-si, zs, sz);
      if (!NIC0) {
        // anode distances u = d - z, exact near the anode
        float us = il.w + l.w;
        for (int n = 1; n <= nic; ++n) {
          float two_nd = 2.0f * n * dnm;
          // opposite-charge partners (symmetric in the roles)
          float z1 = (n == 1) ? -us : zs - two_nd;   // z_a + z_b - 2nd
          float z2 = zs + two_nd;                      // z_a + z_b + 2nd
          float r1 = rsqrtf(fmaxf(fmaf(z1, z1, dxy2), 1e-20f));
          float r2b = rsqrtf(fmaxf(fmaf(z2, z2, dxy2), 1e-20f));
          float s1 = q * (r1 * r1) * r1, s2 = q * (r2b * r2b) * r2b;
          sx = fmaf(-(s1 + s2), dx, sx);
          sy = fmaf(-(s1 + s2), dy, sy);
          sz = fmaf(-s1, z1, fmaf(-s2, z2, sz));
          // same-charge partners, evaluated with a = i; the z part changes
          // sign when j < i (lower-index role convention)
          float z3 = dz - two_nd, z4 = dz + two_nd;
          float r3 = rsqrtf(fmaxf(fmaf(z3, z3, dxy2), 1e-20f));
          float r4 = rsqrtf(fmaxf(fmaf(z4, z4, dxy2), 1e-20f));
          float s3 = q * (r3 * r3) * r3, s4 = q * (r4 * r4) * r4;
          sx = fmaf(s3 + s4, dx, sx);
          sy = fmaf(s3 + s4, dy, sy);
          float zsame = fmaf(s3, z3, s4 * z4);
          if (MODE == T_DIAG) zsame = (k > self_k) ? zsame : -zsame;
          szs += zsame;
        }
      }
    }
  }
  if (!NIC0) {
    if (MODE == T_LOWER) szs = -szs;
    sz += szs;
  }
  tx += sx; ty += sy; tz += sz;
}

// ---- planar, FP64 (reference arithmetic) ---------------------------------------
// One pair (i, j): Coulomb term plus, with image charges on, the planar
// series of acc_ic_planar_series.inc with i in the "a" role when upper and j
// in it otherwise (the x, y parts then change sign: force_ic_N).
__device__ __forceinline__ void planar_pair_f64(const rd_d4& pj, double x1, double y1, double z1,
                                                double qd1, bool upper, int nic, double d, int ic,
                                                double L2, double& ax, double& ay, double& az) {
  double pre = qd1 * pj.w;
  double dx = x1 - pj.x, dy = y1 - pj.y, dz = z1 - pj.z;
  double dxy2 = dx * dx + dy * dy;
  double r = sqrt(dxy2 + dz * dz) + L2;
  double inv = 1.0 / ((r * r) * r);
  ax = ax + (pre * inv) * dx;
  ay = ay + (pre * inv) * dy;
  az = az + (pre * inv) * dz;
  if (ic) {
    double za = upper ? z1 : pj.z, zb = upper ? pj.z : z1;
    // acc_ic_planar_series.inc
    double zic = -1.0 * zb, dzi = za - zic;
    r = sqrt(dxy2 + dzi * dzi) + L2;
    inv = 1.0 / ((r * r) * r);
    double icx = -dx * inv, icy = -dy * inv, icz = -dzi * inv;
    for (int n = 1; n <= nic; ++n) {
      double zz0 = (2.0 * n) * d - zb, zz1 = (-2.0 * n) * d - zb;
      double zz2 = (2.0 * n) * d + zb, zz3 = (-2.0 * n) * d + zb;
      dzi = za - zz0; r = sqrt(dxy2 + dzi * dzi) + L2; inv = 1.0 / ((r * r) * r);
      icx = icx - dx * inv; icy = icy - dy * inv; icz = icz - dzi * inv;
      dzi = za - zz1; r = sqrt(dxy2 + dzi * dzi) + L2; inv = 1.0 / ((r * r) * r);
      icx = icx - dx * inv; icy = icy - dy * inv; icz = icz - dzi * inv;
      dzi = za - zz2; r = sqrt(dxy2 + dzi * dzi) + L2; inv = 1.0 / ((r * r) * r);
      icx = icx + dx * inv; icy = icy + dy * inv; icz = icz + dzi * inv;
      dzi = za - zz3; r = sqrt(dxy2 + dzi * dzi) + L2; inv = 1.0 / ((r * r) * r);
      icx = icx + dx * inv; icy = icy + dy * inv; icz = icz + dzi * inv;
    }
    ax = ax + pre * icx;
    ay = ay + pre * icy;
    az = az + pre * icz;
  }
}

template <int MODE>
__device__ __forceinline__ void planar_tile_f64(const rd_d4* __restrict__ sj, int kmax, double x1,
                                                double y1, double z1, double qd1, int self_k,
                                                int nic, double d, int ic, double L2,
                                                double& ax, double& ay, double& az) {
  for (int k = 0; k < kmax; ++k) {
    if (MODE == T_DIAG && k == self_k) continue;
    const bool upper = (MODE == T_UPPER) || (MODE == T_DIAG && k > self_k);
    planar_pair_f64(sj[k], x1, y1, z1, qd1, upper, nic, d, ic, L2, ax, ay, az);
  }
}

// ---- hyperboloid tip -------------------------------------------------------------
// Sphere image term (acc_tip_image_point.inc + acc_tip_ic_force.inc):
// a = lower-indexed particle, b = higher-indexed,
//   IC = K [ (a - b)/|b - a|^3 - c_a (im_a - b)/|b - im_a|^3 ],  c_a = R / dis_a,
// applied to the lower particle as is and to the higher one mirrored in x, y.
// With K = q0 / (4 pi eps0) ~ 1.4e-9 this part sits far below the FP32
// resolution of the direct sum, so the FP32 tiles keep it in separate sums
// that the caller scales by K in FP64.  For particle i against the j of one
// tile (d = x_i - x_j, e = image point - position):
//   D  = sum q d / |d|^3                          (all j; compensated d)
//   U  = sum_{j > i} q e_i / |e_i|^3,   e_i = im_i - x_j   (i in the a role)
//   W  = sum_{j < i} q c_j (ex, ey, -ez)_j / |e_j|^3,  e_j = im_j - x_i
//   Lz = sum_{j < i} q dz / |d|^3
// and the field is (1 + K) D + K (W - c_i U - 2 Lz z^).  U and W use the high
// words only: their relative error (~1e-5 for the nearest charges) is ~1e-14
// of the field once scaled by K.  MODE T_UPPER: every j in the a... b role of
// a point (fields), T_LOWER: every j lower, T_DIAG: by index against self_k.
struct TipSums {
  float dx, dy, dz, ux, uy, uz, wx, wy, wz, lz;
  __device__ void zero() { dx = dy = dz = ux = uy = uz = wx = wy = wz = lz = 0.f; }
};

// ELEC (off-diagonal tiles whose charges are all -1, the electrons' q/q0):
// the charge is a constant and its multiplies fold into the sums' signs.
template <int MODE, bool ELEC = false>
__device__ __forceinline__ void tip_tile_split_f32(const float4* __restrict__ sh, const float4* __restrict__ sl,
                                                   const float4* __restrict__ sih, int kmax, float4 ih,
                                                   float4 il, float4 iih, int self_k, int ic, TipSums& t) {
  for (int k = 0; k < kmax; ++k) {
    const float4 h = sh[k], l = sl[k];
    const float q = ELEC ? -1.f : ((MODE == T_DIAG && k == self_k) ? 0.f : h.w);
    const float dx = (ih.x - h.x) + (il.x - l.x);
    const float dy = (ih.y - h.y) + (il.y - l.y);
    const float dz = (ih.z - h.z) + (il.z - l.z);
    const float inv = rsqrtf(fmaf(dz, dz, fmaf(dx, dx, fmaf(dy, dy, 1e-20f))));
    const float s = q * ((inv * inv) * inv);
    t.dx = fmaf(s, dx, t.dx);
    t.dy = fmaf(s, dy, t.dy);
    t.dz = fmaf(s, dz, t.dz);
    if (ic) {
      const bool upper = (MODE == T_UPPER) || (MODE == T_DIAG && k > self_k);
      if (upper) {
        const float ex = iih.x - h.x, ey = iih.y - h.y, ez = iih.z - h.z;
        const float re = rsqrtf(fmaf(ez, ez, fmaf(ex, ex, fmaf(ey, ey, 1e-20f))));
        const float se = q * ((re * re) * re);
        t.ux = fmaf(se, ex, t.ux);
        t.uy = fmaf(se, ey, t.uy);
        t.uz = fmaf(se, ez, t.uz);
      } else {
        const float4 jh = sih[k];
        const float ex = jh.x - ih.x, ey = jh.y - ih.y, ez = jh.z - ih.z;
        const float re = rsqrtf(fmaf(ez, ez, fmaf(ex, ex, fmaf(ey, ey, 1e-20f))));
        const float se = (q * jh.w) * ((re * re) * re);
        t.wx = fmaf(se, ex, t.wx);
        t.wy = fmaf(se, ey, t.wy);
        t.wz = fmaf(-se, ez, t.wz);
        t.lz = fmaf(s, dz, t.lz);
      }
    }
  }
}

// The FP64 finish of the split sums: (1 + K) D + K (W - c_i U - 2 Lz z^), D
// given in FP64 (compensated across tiles), c_i = R / dis_i of the point.
__device__ __forceinline__ void tip_split_finish(double Dx, double Dy, double Dz, const TipSums& t, float ci,
                                                 int ic, double K, double* fx, double* fy, double* fz) {
  if (!ic) { *fx = Dx; *fy = Dy; *fz = Dz; return; }
  const double c = (double)ci;
  *fx = (1.0 + K) * Dx + K * ((double)t.wx - c * (double)t.ux);
  *fy = (1.0 + K) * Dy + K * ((double)t.wy - c * (double)t.uy);
  *fz = (1.0 + K) * Dz + K * (((double)t.wz - c * (double)t.uz) - 2.0 * (double)t.lz);
}

// FP64 tip gather: Calculate_Acceleration_Particles_ACC tip branch (:1344-1426).
// One pair (i, j); upper: i is the lower-indexed ("a") particle.
__device__ __forceinline__ void tip_pair_f64(const rd_d4& pj, double x1, double y1, double z1,
                                             double qd1, bool upper, int ic, const DiodeParams& p,
                                             double L2, double K, double& ax, double& ay,
                                             double& az) {
  const double z0 = p.h_tip - p.r_tip, R = p.r_tip;
  double pre = qd1 * pj.w;
  double dx = x1 - pj.x, dy = y1 - pj.y, dz = z1 - pj.z;
  double r = sqrt(dx * dx + dy * dy + dz * dz) + L2;
  double inv = 1.0 / ((r * r) * r);
  ax = ax + (pre * inv) * dx;
  ay = ay + (pre * inv) * dy;
  az = az + (pre * inv) * dz;
  if (ic) {
    double xa = upper ? x1 : pj.x, ya = upper ? y1 : pj.y, za = upper ? z1 : pj.z;
    double xb = upper ? pj.x : x1, yb = upper ? pj.y : y1, zb = upper ? pj.z : z1;
    double sgn = upper ? 1.0 : -1.0;
    double dza = za - z0;
    double dis = sqrt(xa * xa + ya * ya + dza * dza);
    double zim = z0 + (R * R) / (sqrt((1.0 + (xa * xa) / (dza * dza)) + (ya * ya) / (dza * dza)) * dis);
    double xim = ((zim - z0) * xa) / dza, yim = ((zim - z0) * ya) / dza;
    double tda = pow((xb - xa) * (xb - xa) + (yb - ya) * (yb - ya) + (zb - za) * (zb - za), 1.5);
    double tdb = pow((xb - xim) * (xb - xim) + (yb - yim) * (yb - yim) + (zb - zim) * (zb - zim), 1.5);
    double icx = K * ((xa - xb) / tda - (R * (xim - xb)) / (dis * tdb));
    double icy = K * ((ya - yb) / tda - (R * (yim - yb)) / (dis * tdb));
    double icz = K * ((za - zb) / tda - (R * (zim - zb)) / (dis * tdb));
    ax = ax + pre * sgn * icx;
    ay = ay + pre * sgn * icy;
    az = az + pre * icz;
  }
}

template <int MODE>
__device__ __forceinline__ void tip_tile_f64(const rd_d4* __restrict__ sj, int kmax, double x1,
                                             double y1, double z1, double qd1, int self_k, int ic,
                                             const DiodeParams& p, double L2, double K,
                                             double& ax, double& ay, double& az) {
  for (int k = 0; k < kmax; ++k) {
    if (MODE == T_DIAG && k == self_k) continue;
    const bool upper = (MODE == T_UPPER) || (MODE == T_DIAG && k > self_k);
    tip_pair_f64(sj[k], x1, y1, z1, qd1, upper, ic, p, L2, K, ax, ay, az);
  }
}
