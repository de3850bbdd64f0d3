// rd_force.cu -- all-pairs acceleration kernels (Calculate_Acceleration_Particles).
//
// Semantics follow the gather form of the reference,
// Calculate_Acceleration_Particles_ACC (src/mod_verlet.F90:1217-1429):
//   a_i = (1/m_i) [ sum_{j != i} q_i q_j k ( d_ij/(|d_ij| + l^2)^3 + IC_ij ) + q_i E_vac(x_i) ]
// with the image term IC_ij of the pair always evaluated with the
// lower-indexed particle in the "a" role and mirrored in x and y for the
// higher-indexed one (:1303-1323, :1372-1402).
//
// Two precisions:
//  * FP64 ("plain"): the reference's arithmetic in SI units.
//  * FP32 compensated: positions as (hi, lo) float pairs in nm, rsqrt and
//    per-j-tile float accumulation, tile sums folded into (hi, lo) pairs with
//    two-sum, the final sum and all prefactors in FP64.  The image partner
//    heights are formed from sums of absolute heights (z_a + z_b, or the
//    anode distances) so terms do not cancel next to the electrodes.
//
// Tiles are aligned (i0 and j0 multiples of RD_TILE), so a j-tile is either
// entirely above the i-tile (all j > i), entirely below, or the diagonal
// tile; the role selection and the self-exclusion are per pair only on the
// diagonal tile.
#include "rd_tiles.cuh"

namespace {

// ---- planar, FP32 compensated, one image partner (N_ic_max = 0) -----------------
// Two i-particles per thread (64 threads per 128-particle tile), so one
// shared-memory load of a j-particle feeds two pairs.  Per pair: the Coulomb
// term and the n = 0 image partner at -z_j, whose height difference is
// z_i + z_j = 2 z_i - dz (2 z_i as one float: relative error 6e-8).  The
// 1e-20 nm^2 floor inside dxy^2 keeps the self pair and coincident pairs
// finite (their q or d is zero).
// ELEC (off-diagonal tiles whose charges are all -1, the electrons' q/q0):
// the charge multiplies are dropped and the sign folded into the sums.
template <bool IC, bool DIAG, bool ELEC = false>
__device__ __forceinline__ void planar_tile2_nic0(const float4* __restrict__ sh, const float4* __restrict__ sl,
                                                  int kmax, float4 ah, float4 al, float atz, float4 bh,
                                                  float4 bl, float btz, int self_a, int self_b,
                                                  float3& ta, float3& tb) {
  float ax = 0.f, ay = 0.f, az = 0.f, bx = 0.f, by = 0.f, bz = 0.f;
#pragma unroll 2
  for (int k = 0; k < kmax; ++k) {
    const float4 h = sh[k], l = sl[k];
    const float qa = ELEC ? 1.f : ((DIAG && k == self_a) ? 0.f : h.w);
    const float qb = ELEC ? 1.f : ((DIAG && k == self_b) ? 0.f : h.w);
    {
      const float dx = (ah.x - h.x) + (al.x - l.x), dy = (ah.y - h.y) + (al.y - l.y);
      const float dz = (ah.z - h.z) + (al.z - l.z);
      const float dxy2 = fmaf(dx, dx, fmaf(dy, dy, 1e-20f));
      const float inv = rsqrtf(fmaf(dz, dz, dxy2));
      const float s = qa * ((inv * inv) * inv);
      if (IC) {
        const float zs = atz - dz;
        const float ri = rsqrtf(fmaf(zs, zs, dxy2));
        const float si = qa * ((ri * ri) * ri);
        const float t = s - si;
        ax = fmaf(t, dx, ax); ay = fmaf(t, dy, ay);
        az = fmaf(s, dz, fmaf(-si, zs, az));
      } else {
        ax = fmaf(s, dx, ax); ay = fmaf(s, dy, ay); az = fmaf(s, dz, az);
      }
    }
    {
      const float dx = (bh.x - h.x) + (bl.x - l.x), dy = (bh.y - h.y) + (bl.y - l.y);
      const float dz = (bh.z - h.z) + (bl.z - l.z);
      const float dxy2 = fmaf(dx, dx, fmaf(dy, dy, 1e-20f));
      const float inv = rsqrtf(fmaf(dz, dz, dxy2));
      const float s = qb * ((inv * inv) * inv);
      if (IC) {
        const float zs = btz - dz;
        const float ri = rsqrtf(fmaf(zs, zs, dxy2));
        const float si = qb * ((ri * ri) * ri);
        const float t = s - si;
        bx = fmaf(t, dx, bx); by = fmaf(t, dy, by);
        bz = fmaf(s, dz, fmaf(-si, zs, bz));
      } else {
        bx = fmaf(s, dx, bx); by = fmaf(s, dy, by); bz = fmaf(s, dz, bz);
      }
    }
  }
  if (ELEC) { ax = -ax; ay = -ay; az = -az; bx = -bx; by = -by; bz = -bz; }
  ta.x += ax; ta.y += ay; ta.z += az;
  tb.x += bx; tb.y += by; tb.z += bz;
}

__global__ void __launch_bounds__(64)
k_force_planar_f32_nic0(const DiodeParams* __restrict__ P, Pool pool,
                        const PlanEntry* __restrict__ plan, const PlanHeader* __restrict__ ph,
                        double* __restrict__ partial, int* __restrict__ tickets, double kscale, int* __restrict__ queue) {
  __shared__ int s_item;
  __shared__ float4 sh[RD_TILE], sl[RD_TILE];
  const int total = ph->total_items, nd = ph->n_diodes;
  const int tid = threadIdx.x, nt = 64;
  for (int g = queue_first(0, total); g < total; g = queue_next(queue, &s_item, 0, total)) {
    ItemRef it = decode_item(plan, nd, g);
    const DiodeParams& p = P[it.d];
    const int off = p.off, n = plan[it.d].n_i;
    const int ia = it.i0 + tid, ib = it.i0 + nt + tid;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 ah = ia < n ? pool.pk_hi[off + ia] : z4, al = ia < n ? pool.pk_lo[off + ia] : z4;
    const float4 bh = ib < n ? pool.pk_hi[off + ib] : z4, bl = ib < n ? pool.pk_lo[off + ib] : z4;
    const float atz = 2.f * (ah.z + al.z), btz = 2.f * (bh.z + bl.z);
    const bool ic = p.image_charge != 0;
    F32Acc A, B;
    A.zero(); B.zero();
    for (int jt = it.j0; jt < it.j1; jt += RD_TILE) {
      __syncthreads();
      int elec = 1;   // every charge of the tile is an electron's
      for (int q = tid; q < RD_TILE; q += nt) {
        const int j = jt + q;
        if (j < it.j1) {
          const float4 hj = pool.pk_hi[off + j];
          sh[q] = hj; sl[q] = pool.pk_lo[off + j];
          elec &= (hj.w == -1.0f);
        }
      }
      elec = __syncthreads_and(elec);
      const int kmax = min(RD_TILE, it.j1 - jt);
      float3 ta = make_float3(0.f, 0.f, 0.f), tb = ta;
      const bool diag = (jt == it.i0);
      if (ic) {
        if (diag) planar_tile2_nic0<true, true>(sh, sl, kmax, ah, al, atz, bh, bl, btz, tid, nt + tid, ta, tb);
        else if (elec) planar_tile2_nic0<true, false, true>(sh, sl, kmax, ah, al, atz, bh, bl, btz, -1, -1, ta, tb);
        else planar_tile2_nic0<true, false>(sh, sl, kmax, ah, al, atz, bh, bl, btz, -1, -1, ta, tb);
      } else {
        if (diag) planar_tile2_nic0<false, true>(sh, sl, kmax, ah, al, atz, bh, bl, btz, tid, nt + tid, ta, tb);
        else planar_tile2_nic0<false, false>(sh, sl, kmax, ah, al, atz, bh, bl, btz, -1, -1, ta, tb);
      }
      A.add(ta.x, ta.y, ta.z);
      B.add(tb.x, tb.y, tb.z);
    }
    double f[2][3] = {{(double)A.hx + (double)A.lx, (double)A.hy + (double)A.ly, (double)A.hz + (double)A.lz},
                      {(double)B.hx + (double)B.lx, (double)B.hy + (double)B.ly, (double)B.hz + (double)B.lz}};
    if (it.nch > 1) {
      double* pp = partial + (size_t)g * 3 * RD_ITILE;
      for (int q = 0; q < 2; ++q)
        for (int c = 0; c < 3; ++c) pp[c * RD_ITILE + tid + q * nt] = f[q][c];
      if (!tile_ticket(tickets, it)) continue;
      for (int q = 0; q < 2; ++q)
        for (int c = 0; c < 3; ++c) {
          double v = 0.0;
          for (int cc = 0; cc < it.nch; ++cc)
            v += __ldcg(partial + (size_t)(it.base + cc) * 3 * RD_ITILE + c * RD_ITILE + tid + q * nt);
          f[q][c] = v;
        }
    }
    for (int q = 0; q < 2; ++q) {
      const int i = it.i0 + tid + q * nt;
      if (i >= n) continue;
      const int gi = off + i;
      const double qi = pool.q[gi], im = 1.0 / pool.m[gi];
      const double pre = (qi * kscale) * im;   // kscale = k q0 1e18 (nm -> m)
      pool.ax[gi] = pre * f[q][0];
      pool.ay[gi] = pre * f[q][1];
      pool.az[gi] = pre * f[q][2] + qi * p.E_z * im;
    }
  }
  queue_leave(queue, 0, total);
}

template <bool NIC0>
__global__ void __launch_bounds__(RD_ITILE)
k_force_planar_f32(const DiodeParams* __restrict__ P, const DiodeDyn* __restrict__ Dy, Pool pool,
                   const PlanEntry* __restrict__ plan, const PlanHeader* __restrict__ ph,
                   double* __restrict__ partial, int* __restrict__ tickets, double kscale, int* __restrict__ queue) {
  __shared__ int s_item;
  __shared__ float4 sh[RD_TILE], sl[RD_TILE];
  const int total = ph->total_items, nd = ph->n_diodes;
  const int tid = threadIdx.x;
  for (int g = queue_first(0, total); g < total; g = queue_next(queue, &s_item, 0, total)) {
    ItemRef it = decode_item(plan, nd, g);
    const DiodeParams& p = P[it.d];
    const int off = p.off, n = plan[it.d].n_i;
    const int i = it.i0 + tid;
    const bool valid = i < n;
    float4 ih = valid ? pool.pk_hi[off + i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 il = valid ? pool.pk_lo[off + i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float dnm = (float)(p.d * 1.0e9);
    const int nic = p.N_ic_max, ic = p.image_charge;
    F32Acc acc;
    acc.zero();
    for (int jt = it.j0; jt < it.j1; jt += RD_TILE) {
      __syncthreads();
      int j = jt + tid;
      int elec = 1;   // every charge of the tile is an electron's
      if (j < it.j1) {
        const float4 hj = pool.pk_hi[off + j];
        sh[tid] = hj; sl[tid] = pool.pk_lo[off + j];
        elec = (hj.w == -1.0f);
      }
      elec = __syncthreads_and(elec);
      int kmax = min(RD_TILE, it.j1 - jt);
      float tx = 0.f, ty = 0.f, tz = 0.f;
      if (jt == it.i0)
        planar_tile_f32<T_DIAG, NIC0>(sh, sl, kmax, ih, il, tid, nic, dnm, ic, tx, ty, tz);
      else if (jt > it.i0)
        elec ? planar_tile_f32<T_UPPER, NIC0, true>(sh, sl, kmax, ih, il, -1, nic, dnm, ic, tx, ty, tz)
             : planar_tile_f32<T_UPPER, NIC0>(sh, sl, kmax, ih, il, -1, nic, dnm, ic, tx, ty, tz);
      else
        elec ? planar_tile_f32<T_LOWER, NIC0, true>(sh, sl, kmax, ih, il, -1, nic, dnm, ic, tx, ty, tz)
             : planar_tile_f32<T_LOWER, NIC0>(sh, sl, kmax, ih, il, -1, nic, dnm, ic, tx, ty, tz);
      acc.add(tx, ty, tz);
    }
    double fx = (double)acc.hx + (double)acc.lx;
    double fy = (double)acc.hy + (double)acc.ly;
    double fz = (double)acc.hz + (double)acc.lz;
    if (it.nch > 1) {
      double* pp = partial + (size_t)g * 3 * RD_ITILE;
      pp[tid] = fx; pp[RD_ITILE + tid] = fy; pp[2 * RD_ITILE + tid] = fz;
      if (!tile_ticket(tickets, it)) continue;
      fx = fy = fz = 0.0;
      for (int c = 0; c < it.nch; ++c) {
        const double* q = partial + (size_t)(it.base + c) * 3 * RD_ITILE;
        fx += __ldcg(q + tid); fy += __ldcg(q + RD_ITILE + tid); fz += __ldcg(q + 2 * RD_ITILE + tid);
      }
    }
    if (valid) {
      // a_i = (q_i k e^2 1e18 / m_i) * sum + q_i E_vac / m_i   (nm -> m: 1e18)
      const int gi = off + i;
      double qi = pool.q[gi], im = 1.0 / pool.m[gi];
      double pre = (qi * kscale) * im;   // kscale = k * q0 * 1e18 (per unit q_j/q0)
      pool.ax[gi] = pre * fx;
      pool.ay[gi] = pre * fy;
      pool.az[gi] = pre * fz + qi * p.E_z * im;
    }
  }
  queue_leave(queue, 0, total);
}

__global__ void __launch_bounds__(RD_ITILE)
k_force_planar_f64(const DiodeParams* __restrict__ P, const DiodeDyn* __restrict__ Dy, Pool pool,
                   const PlanEntry* __restrict__ plan, const PlanHeader* __restrict__ ph,
                   double* __restrict__ partial, int* __restrict__ tickets, int* __restrict__ queue) {
  __shared__ int s_item;
  __shared__ rd_d4 sj[RD_TILE];
  const int total = ph->total_items, nd = ph->n_diodes;
  const int tid = threadIdx.x;
  const double L2 = c_k.L2, dfc = c_k.div_fac_c;
  for (int g = queue_first(0, total); g < total; g = queue_next(queue, &s_item, 0, total)) {
    ItemRef it = decode_item(plan, nd, g);
    const DiodeParams& p = P[it.d];
    const int off = p.off, n = plan[it.d].n_i;
    const int i = it.i0 + tid;
    const bool valid = i < n;
    double x1 = 0, y1 = 0, z1 = 0, q1 = 0;
    if (valid) { x1 = pool.x[off + i]; y1 = pool.y[off + i]; z1 = pool.z[off + i]; q1 = pool.q[off + i]; }
    const double qd1 = q1 * dfc;
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int jt = it.j0; jt < it.j1; jt += RD_TILE) {
      __syncthreads();
      int j = jt + tid;
      if (j < it.j1) sj[tid] = make_d4(pool.x[off + j], pool.y[off + j], pool.z[off + j], pool.q[off + j]);
      __syncthreads();
      int kmax = min(RD_TILE, it.j1 - jt);
      if (jt == it.i0)
        planar_tile_f64<T_DIAG>(sj, kmax, x1, y1, z1, qd1, tid, p.N_ic_max, p.d, p.image_charge, L2, ax, ay, az);
      else if (jt > it.i0)
        planar_tile_f64<T_UPPER>(sj, kmax, x1, y1, z1, qd1, -1, p.N_ic_max, p.d, p.image_charge, L2, ax, ay, az);
      else
        planar_tile_f64<T_LOWER>(sj, kmax, x1, y1, z1, qd1, -1, p.N_ic_max, p.d, p.image_charge, L2, ax, ay, az);
    }
    if (it.nch > 1) {
      double* pp = partial + (size_t)g * 3 * RD_ITILE;
      pp[tid] = ax; pp[RD_ITILE + tid] = ay; pp[2 * RD_ITILE + tid] = az;
      if (!tile_ticket(tickets, it)) continue;
      ax = ay = az = 0.0;
      for (int c = 0; c < it.nch; ++c) {
        const double* q = partial + (size_t)(it.base + c) * 3 * RD_ITILE;
        ax += __ldcg(q + tid); ay += __ldcg(q + RD_ITILE + tid); az += __ldcg(q + 2 * RD_ITILE + tid);
      }
    }
    if (valid) {
      const int gi = off + i;
      double im = 1.0 / pool.m[gi];
      pool.ax[gi] = ax * im;
      pool.ay[gi] = ay * im;
      pool.az[gi] = (az + q1 * p.E_z) * im;
    }
  }
  queue_leave(queue, 0, total);
}

__global__ void __launch_bounds__(RD_ITILE)
k_force_tip_f32(const DiodeParams* __restrict__ P, const DiodeDyn* __restrict__ Dy, Pool pool,
                const PlanEntry* __restrict__ plan, const PlanHeader* __restrict__ ph,
                double* __restrict__ partial, int* __restrict__ tickets, double kscale, int* __restrict__ queue) {
  __shared__ int s_item;
  __shared__ float4 sh[RD_TILE], sl[RD_TILE], sih[RD_TILE];
  const int total = ph->total_items, nd = ph->n_diodes;
  const int tid = threadIdx.x;
  for (int g = queue_first(0, total); g < total; g = queue_next(queue, &s_item, 0, total)) {
    ItemRef it = decode_item(plan, nd, g);
    const DiodeParams& p = P[it.d];
    const int off = p.off, n = plan[it.d].n_i;
    const int i = it.i0 + tid;
    const bool valid = i < n;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 ih = valid ? pool.pk_hi[off + i] : z4, il = valid ? pool.pk_lo[off + i] : z4;
    float4 iih = valid ? pool.ip_hi[off + i] : z4;
    F32Acc acc;          // the direct sum D, compensated across tiles
    acc.zero();
    TipSums ts;          // the K-scaled image sums U, W, Lz (tip_tile_split_f32)
    ts.zero();
    for (int jt = it.j0; jt < it.j1; jt += RD_TILE) {
      __syncthreads();
      int j = jt + tid;
      int elec = 1;   // every charge of the tile is an electron's
      if (j < it.j1) {
        const float4 hj = pool.pk_hi[off + j];
        sh[tid] = hj; sl[tid] = pool.pk_lo[off + j];
        sih[tid] = pool.ip_hi[off + j];
        elec = (hj.w == -1.0f);
      }
      elec = __syncthreads_and(elec);
      int kmax = min(RD_TILE, it.j1 - jt);
      ts.dx = ts.dy = ts.dz = 0.f;
      if (jt == it.i0)
        tip_tile_split_f32<T_DIAG>(sh, sl, sih, kmax, ih, il, iih, tid, p.image_charge, ts);
      else if (jt > it.i0)
        elec ? tip_tile_split_f32<T_UPPER, true>(sh, sl, sih, kmax, ih, il, iih, -1, p.image_charge, ts)
             : tip_tile_split_f32<T_UPPER>(sh, sl, sih, kmax, ih, il, iih, -1, p.image_charge, ts);
      else
        elec ? tip_tile_split_f32<T_LOWER, true>(sh, sl, sih, kmax, ih, il, iih, -1, p.image_charge, ts)
             : tip_tile_split_f32<T_LOWER>(sh, sl, sih, kmax, ih, il, iih, -1, p.image_charge, ts);
      acc.add(ts.dx, ts.dy, ts.dz);
    }
    double fx, fy, fz;
    tip_split_finish((double)acc.hx + (double)acc.lx, (double)acc.hy + (double)acc.ly,
                     (double)acc.hz + (double)acc.lz, ts, iih.w, p.image_charge, c_k.tip_K, &fx, &fy, &fz);
    if (it.nch > 1) {
      double* pp = partial + (size_t)g * 3 * RD_ITILE;
      pp[tid] = fx; pp[RD_ITILE + tid] = fy; pp[2 * RD_ITILE + tid] = fz;
      if (!tile_ticket(tickets, it)) continue;
      fx = fy = fz = 0.0;
      for (int c = 0; c < it.nch; ++c) {
        const double* q = partial + (size_t)(it.base + c) * 3 * RD_ITILE;
        fx += __ldcg(q + tid); fy += __ldcg(q + RD_ITILE + tid); fz += __ldcg(q + 2 * RD_ITILE + tid);
      }
    }
    if (valid) {
      const int gi = off + i;
      double qi = pool.q[gi], im = 1.0 / pool.m[gi];
      double pre = (qi * kscale) * im;
      double ex, ey, ez;
      tip_field_E(p, pool.x[gi], pool.y[gi], pool.z[gi], &ex, &ey, &ez);
      pool.ax[gi] = pre * fx + qi * ex * im;
      pool.ay[gi] = pre * fy + qi * ey * im;
      pool.az[gi] = pre * fz + qi * ez * im;
    }
  }
  queue_leave(queue, 0, total);
}

__global__ void __launch_bounds__(RD_ITILE)
k_force_tip_f64(const DiodeParams* __restrict__ P, const DiodeDyn* __restrict__ Dy, Pool pool,
                const PlanEntry* __restrict__ plan, const PlanHeader* __restrict__ ph,
                double* __restrict__ partial, int* __restrict__ tickets, int* __restrict__ queue) {
  __shared__ int s_item;
  __shared__ rd_d4 sj[RD_TILE];
  const int total = ph->total_items, nd = ph->n_diodes;
  const int tid = threadIdx.x;
  const double L2 = c_k.L2, dfc = c_k.div_fac_c, K = c_k.tip_K;
  for (int g = queue_first(0, total); g < total; g = queue_next(queue, &s_item, 0, total)) {
    ItemRef it = decode_item(plan, nd, g);
    const DiodeParams& p = P[it.d];
    const int off = p.off, n = plan[it.d].n_i;
    const int i = it.i0 + tid;
    const bool valid = i < n;
    double x1 = 0, y1 = 0, z1 = 0, q1 = 0;
    if (valid) { x1 = pool.x[off + i]; y1 = pool.y[off + i]; z1 = pool.z[off + i]; q1 = pool.q[off + i]; }
    const double qd1 = q1 * dfc;
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int jt = it.j0; jt < it.j1; jt += RD_TILE) {
      __syncthreads();
      int j = jt + tid;
      if (j < it.j1) sj[tid] = make_d4(pool.x[off + j], pool.y[off + j], pool.z[off + j], pool.q[off + j]);
      __syncthreads();
      int kmax = min(RD_TILE, it.j1 - jt);
      if (jt == it.i0)
        tip_tile_f64<T_DIAG>(sj, kmax, x1, y1, z1, qd1, tid, p.image_charge, p, L2, K, ax, ay, az);
      else if (jt > it.i0)
        tip_tile_f64<T_UPPER>(sj, kmax, x1, y1, z1, qd1, -1, p.image_charge, p, L2, K, ax, ay, az);
      else
        tip_tile_f64<T_LOWER>(sj, kmax, x1, y1, z1, qd1, -1, p.image_charge, p, L2, K, ax, ay, az);
    }
    if (it.nch > 1) {
      double* pp = partial + (size_t)g * 3 * RD_ITILE;
      pp[tid] = ax; pp[RD_ITILE + tid] = ay; pp[2 * RD_ITILE + tid] = az;
      if (!tile_ticket(tickets, it)) continue;
      ax = ay = az = 0.0;
      for (int c = 0; c < it.nch; ++c) {
        const double* q = partial + (size_t)(it.base + c) * 3 * RD_ITILE;
        ax += __ldcg(q + tid); ay += __ldcg(q + RD_ITILE + tid); az += __ldcg(q + 2 * RD_ITILE + tid);
      }
    }
    if (valid) {
      const int gi = off + i;
      double im = 1.0 / pool.m[gi];
      double ex, ey, ez;
      tip_field_E(p, x1, y1, z1, &ex, &ey, &ez);
      pool.ax[gi] = (ax + q1 * ex) * im;
      pool.ay[gi] = (ay + q1 * ey) * im;
      pool.az[gi] = (az + q1 * ez) * im;
    }
  }
  queue_leave(queue, 0, total);
}

// ---- two-time-step diodes (FP64, both geometries) ----------------------------------
// Update_Elec_Acceleration and Update_Ion_Acceleration
// (src/mod_verlet.F90:899-1151) as a gather.  Pairs run over the electron and
// ion lists only (atoms take no part); the image term of an electron-ion
// pair has the electron in the "a" role whatever the indices, a pair of the
// same species the lower index.  Electrons gather from electrons and ions on
// every step.  Ions gather the electron forces on every step and, on steps
// divisible by T, the ion-ion forces and the vacuum field: on those steps the
// position update has just cleared their acceleration, on the others the
// electron forces add to what is there, as the reference's accumulation into
// particles_cur_accel does.
__global__ void __launch_bounds__(RD_ITILE)
k_force_tts_f64(const DiodeParams* __restrict__ P, const DiodeDyn* __restrict__ Dy, Pool pool,
                const PlanEntry* __restrict__ plan, const PlanHeader* __restrict__ ph,
                double* __restrict__ partial, int* __restrict__ tickets, int* __restrict__ queue,
                const int* __restrict__ step_ptr) {
  __shared__ int s_item;
  __shared__ rd_d4 sj[RD_TILE];
  __shared__ int ssp[RD_TILE];
  const int total = ph->total_items, nd = ph->n_diodes;
  const int tid = threadIdx.x;
  const double L2 = c_k.L2, dfc = c_k.div_fac_c, K = c_k.tip_K;
  for (int g = queue_first(0, total); g < total; g = queue_next(queue, &s_item, 0, total)) {
    ItemRef it = decode_item(plan, nd, g);
    const DiodeParams& p = P[it.d];
    const int off = p.off, n = plan[it.d].n_i;
    const int i = it.i0 + tid;
    const bool valid = i < n;
    const bool ion_step = (*step_ptr - Dy[it.d].step_offset) % p.tts == 0;
    const bool tip = p.geometry == RD_G_TIP;
    double x1 = 0, y1 = 0, z1 = 0, q1 = 0;
    int si = 3;
    if (valid) {
      x1 = pool.x[off + i]; y1 = pool.y[off + i]; z1 = pool.z[off + i]; q1 = pool.q[off + i];
      si = pool.species[off + i];
    }
    const double qd1 = q1 * dfc;
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int jt = it.j0; jt < it.j1; jt += RD_TILE) {
      __syncthreads();
      int j = jt + tid;
      if (j < it.j1) {
        sj[tid] = make_d4(pool.x[off + j], pool.y[off + j], pool.z[off + j], pool.q[off + j]);
        ssp[tid] = pool.species[off + j];
      }
      __syncthreads();
      const int kmax = min(RD_TILE, it.j1 - jt);
      for (int k = 0; k < kmax; ++k) {
        const int jj = jt + k, sjk = ssp[k];
        if (jj == i) continue;
        const bool take = (si == 1 && (sjk == 1 || sjk == 2)) ||
                          (si == 2 && (sjk == 1 || (sjk == 2 && ion_step)));
        if (!take) continue;
        const bool upper = (si != sjk) ? (si == 1) : (jj > i);
        if (tip)
          tip_pair_f64(sj[k], x1, y1, z1, qd1, upper, p.image_charge, p, L2, K, ax, ay, az);
        else
          planar_pair_f64(sj[k], x1, y1, z1, qd1, upper, p.N_ic_max, p.d, p.image_charge, L2, ax, ay, az);
      }
    }
    if (it.nch > 1) {
      double* pp = partial + (size_t)g * 3 * RD_ITILE;
      pp[tid] = ax; pp[RD_ITILE + tid] = ay; pp[2 * RD_ITILE + tid] = az;
      if (!tile_ticket(tickets, it)) continue;
      ax = ay = az = 0.0;
      for (int c = 0; c < it.nch; ++c) {
        const double* q = partial + (size_t)(it.base + c) * 3 * RD_ITILE;
        ax += __ldcg(q + tid); ay += __ldcg(q + RD_ITILE + tid); az += __ldcg(q + 2 * RD_ITILE + tid);
      }
    }
    if (valid && (si == 1 || si == 2)) {
      const int gi = off + i;
      const double im = 1.0 / pool.m[gi];
      if (si == 1 || ion_step) {
        double ex = 0.0, ey = 0.0, ez = p.E_z;
        if (tip) tip_field_E(p, x1, y1, z1, &ex, &ey, &ez);
        pool.ax[gi] = (ax + q1 * ex) * im;
        pool.ay[gi] = (ay + q1 * ey) * im;
        pool.az[gi] = (az + q1 * ez) * im;
      } else {
        pool.ax[gi] += ax * im;
        pool.ay[gi] += ay * im;
        pool.az[gi] += az * im;
      }
    }
  }
  queue_leave(queue, 0, total);
}

}  // namespace

// Launch wrappers (called by the engine).
cudaError_t rd_launch_force(int prec, int geometry_mask, int nic_general, int grid,
                            cudaStream_t st, const DiodeParams* P, const DiodeDyn* Dy,
                            const Pool& pool, const PlanEntry* plan, const PlanHeader* ph,
                            double* partial, int* tickets, double kscale, int* queue) {
  // geometry_mask: bit0 planar diodes present, bit1 tip diodes present.  The
  // planar and tip kernels each skip items of the other geometry through the
  // plan (separate plans per geometry are built by the engine).
  if (prec == 0) {
    if (geometry_mask & 1)
      k_force_planar_f64<<<rd_grid(k_force_planar_f64, RD_ITILE, grid), RD_ITILE, 0, st>>>(P, Dy, pool, plan, ph, partial, tickets, queue);
    else
      k_force_tip_f64<<<rd_grid(k_force_tip_f64, RD_ITILE, grid), RD_ITILE, 0, st>>>(P, Dy, pool, plan, ph, partial, tickets, queue);
  } else {
    if (geometry_mask & 1) {
      if (nic_general)
        k_force_planar_f32<false><<<rd_grid(k_force_planar_f32<false>, RD_ITILE, grid), RD_ITILE, 0, st>>>(P, Dy, pool, plan, ph, partial, tickets, kscale, queue);
      else
        k_force_planar_f32_nic0<<<rd_grid(k_force_planar_f32_nic0, 64, grid), 64, 0, st>>>(P, pool, plan, ph, partial, tickets, kscale, queue);
    } else {
      k_force_tip_f32<<<rd_grid(k_force_tip_f32, RD_ITILE, grid), RD_ITILE, 0, st>>>(P, Dy, pool, plan, ph, partial, tickets, kscale, queue);
    }
  }
  return cudaGetLastError();
}

// Two-time-step diodes of both geometries; the plan (PM_FORCE_TTS) holds only them.
cudaError_t rd_launch_force_tts(int grid, cudaStream_t st, const DiodeParams* P, const DiodeDyn* Dy,
                                const Pool& pool, const PlanEntry* plan, const PlanHeader* ph,
                                double* partial, int* tickets, int* queue, const int* step_ptr) {
  k_force_tts_f64<<<rd_grid(k_force_tts_f64, RD_ITILE, grid), RD_ITILE, 0, st>>>(P, Dy, pool, plan, ph, partial,
                                                                                 tickets, queue, step_ptr);
  return cudaGetLastError();
}

RD_DEFINE_CONSTANT_UPLOAD(force)
