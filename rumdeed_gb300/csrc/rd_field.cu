// rd_field.cu -- field at points and the emission pipeline.
//
//  * k_field_points: E at arbitrary points (Calc_Field_at_Batch,
//    src/mod_verlet.F90:1635-1911): vacuum field plus, for every particle j,
//    q_j k [ (p - x_j)/(|p - x_j| + l^2)^3 + IC(p, x_j) ] with the image
//    function evaluated with the point in the "a" role (:1762-1793, :1822-1893).
//  * k_z0_points / k_mh_jump_planar: the z component at cathode points
//    (z = 0).  There the Coulomb term and the n = 0 image partner share the
//    same distance and their x, y parts cancel exactly, so per particle the
//    field is -2 q_j k sum_h h/(sqrt(dxy^2 + h^2) + l^2)^3 over the partner
//    heights h in {z_j, z_j +- 2nd}: half the rsqrt count of the generic form
//    with the same result.
//  * supply integral, MH chains and emission: the batched planar sampler
//    Metropolis_Hastings_rectangle_J_batch (src/mod_field_emission_v2.F90:
//    1284-1458) and the tip sampler Metro_algo_tip_v3 (src/mod_emission_tip.f90:
//    1241-1390) run as one lockstep batch per diode; the supply integral uses a
//    composite Gauss-Legendre rule (planar; the reference uses the third-party
//    Cuba library) or the reference's own 100x100 midpoint grid (tip,
//    Do_Field_Emission_Tip_OLDCODE :417-534).  Random numbers are Philox
//    streams keyed by the diode seed with counters (chain, iteration, step,
//    purpose), so every chain is reproducible and independent of scheduling.
#include <cooperative_groups.h>
#include <type_traits>

#include "rd_tiles.cuh"


namespace {

// ---- general field at points ---------------------------------------------------
__device__ __forceinline__ void point_pack(const DiodeParams& p, double x, double y, double z,
                                           float4& ih, float4& il, float4& iih, float4& iil) {
  float a, b;
  split_nm(x, p.org_x, &a, &b); ih.x = a; il.x = b;
  split_nm(y, p.org_y, &a, &b); ih.y = a; il.y = b;
  split_nm(z, 0.0, &a, &b); ih.z = a; il.z = b;
  ih.w = 1.f;
  il.w = (float)((p.d - z) * 1.0e9);
  iih = iil = make_float4(0.f, 0.f, 0.f, 0.f);
  if (p.geometry == RD_G_TIP) {
    double xi, yi, zi;
    double dis = tip_image_point(p, x, y, z, &xi, &yi, &zi);
    split_nm(xi, p.org_x, &a, &b); iih.x = a; iil.x = b;
    split_nm(yi, p.org_y, &a, &b); iih.y = a; iil.y = b;
    split_nm(zi, 0.0, &a, &b); iih.z = a; iil.z = b;
    iih.w = (float)(p.r_tip / dis);
  }
}

template <int PREC, int GEOM>
__global__ void __launch_bounds__(RD_ITILE)
k_field_points(const DiodeParams* __restrict__ P, Pool pool, const PlanEntry* __restrict__ plan,
               const PlanHeader* __restrict__ ph, PointSet pts, double* __restrict__ partial,
               int* __restrict__ tickets, double kscale) {
  __shared__ float4 sh[RD_TILE], sl[RD_TILE], sih[RD_TILE];
  __shared__ rd_d4 sj[RD_TILE];
  const int total = ph->total_items, nd = ph->n_diodes, tid = threadIdx.x;
  for (int g = blockIdx.x; g < total; g += gridDim.x) {
    ItemRef it = decode_item(plan, nd, g);
    const DiodeParams& p = P[it.d];
    const int off = p.off, m = plan[it.d].n_i, po = pts.off[it.d];
    const int i = it.i0 + tid;
    const bool valid = i < m;
    double X = valid ? pts.x[po + i] : 0.0, Y = valid ? pts.y[po + i] : 0.0;
    double Z = valid ? pts.z[po + i] : 0.5 * p.d;
    double fx, fy, fz;
    if (PREC == 1) {
      float4 ih, il, iih, iil;
      point_pack(p, X, Y, Z, ih, il, iih, iil);
      const float dnm = (float)(p.d * 1.0e9);
      F32Acc acc;
      acc.zero();
      TipSums ts;   // tip: the K-scaled image sums, kept apart (tip_tile_split_f32)
      ts.zero();
      for (int jt = it.j0; jt < it.j1; jt += RD_TILE) {
        __syncthreads();
        int j = jt + tid;
        int elec = 1;   // every charge of the tile is an electron's
        if (j < it.j1) {
          const float4 hj = pool.pk_hi[off + j];
          sh[tid] = hj; sl[tid] = pool.pk_lo[off + j];
          if (GEOM == RD_G_TIP) sih[tid] = pool.ip_hi[off + j];
          elec = (hj.w == -1.0f);
        }
        elec = __syncthreads_and(elec);
        int kmax = min(RD_TILE, it.j1 - jt);
        float tx = 0.f, ty = 0.f, tz = 0.f;
        if (GEOM == RD_G_TIP) {   // D per tile (folded into acc), U across the tiles
          ts.dx = ts.dy = ts.dz = 0.f;
          if (elec) tip_tile_split_f32<T_UPPER, true>(sh, sl, sih, kmax, ih, il, iih, -1, p.image_charge, ts);
          else tip_tile_split_f32<T_UPPER>(sh, sl, sih, kmax, ih, il, iih, -1, p.image_charge, ts);
          tx = ts.dx; ty = ts.dy; tz = ts.dz;
        } else if (p.N_ic_max == 0) {
          if (elec) planar_tile_f32<T_UPPER, true, true>(sh, sl, kmax, ih, il, -1, 0, dnm, p.image_charge, tx, ty, tz);
          else planar_tile_f32<T_UPPER, true>(sh, sl, kmax, ih, il, -1, 0, dnm, p.image_charge, tx, ty, tz);
        } else {
          if (elec) planar_tile_f32<T_UPPER, false, true>(sh, sl, kmax, ih, il, -1, p.N_ic_max, dnm, p.image_charge, tx, ty, tz);
          else planar_tile_f32<T_UPPER, false>(sh, sl, kmax, ih, il, -1, p.N_ic_max, dnm, p.image_charge, tx, ty, tz);
        }
        acc.add(tx, ty, tz);
      }
      fx = ((double)acc.hx + (double)acc.lx);
      fy = ((double)acc.hy + (double)acc.ly);
      fz = ((double)acc.hz + (double)acc.lz);
      if (GEOM == RD_G_TIP) tip_split_finish(fx, fy, fz, ts, iih.w, p.image_charge, c_k.tip_K, &fx, &fy, &fz);
      fx *= kscale; fy *= kscale; fz *= kscale;
    } else {
      const double L2 = c_k.L2, dfc = c_k.div_fac_c;
      fx = fy = fz = 0.0;
      for (int jt = it.j0; jt < it.j1; jt += RD_TILE) {
        __syncthreads();
        int j = jt + tid;
        if (j < it.j1) sj[tid] = make_d4(pool.x[off + j], pool.y[off + j], pool.z[off + j], pool.q[off + j]);
        __syncthreads();
        int kmax = min(RD_TILE, it.j1 - jt);
        if (GEOM == RD_G_TIP)
          tip_tile_f64<T_UPPER>(sj, kmax, X, Y, Z, dfc, -1, p.image_charge, p, L2, c_k.tip_K, fx, fy, fz);
        else
          planar_tile_f64<T_UPPER>(sj, kmax, X, Y, Z, dfc, -1, p.N_ic_max, p.d, p.image_charge, L2, fx, fy, fz);
      }
    }
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
      double ex, ey, ez;
      vacuum_field(p, X, Y, Z, &ex, &ey, &ez);
      pts.fx[po + i] = ex + fx;
      pts.fy[po + i] = ey + fy;
      pts.fz[po + i] = ez + fz;
    }
  }
}

// ---- work-function cell and the tabulated supply logarithm ------------------------------
// Cell of the checkerboard (as work_at) without the section number.
// The supply-table entry of (x, y): the checkerboard cell or the Voronoi
// site; -1 for the Gaussian model, whose work function has no cells.
__device__ __forceinline__ int work_cell(const DiodeParams& p, double x, double y) {
  if (p.work_model == 2) return -1;
  if (p.work_model == 4) return voronoi_site(p, p.work_data, x, y);
  if (p.work_nx == 1 && p.work_ny == 1) return 0;
  double xs = (x - p.em_x0) / p.em_Lx, ys = (y - p.em_y0) / p.em_Ly;
  int nx = p.work_nx, ny = p.work_ny;
  int xi = (int)floor(xs / (1.0 / nx)) + 1, yi = (int)floor(ys / (1.0 / ny)) + 1;
  xi = xi > nx ? nx : (xi < 1 ? 1 : xi);
  yi = yi > ny ? ny : (yi < 1 ? 1 : yi);
  yi = ny - yi + 1;
  return (yi - 1) * nx + (xi - 1);
}

// Elec_Supply_log (src/mod_field_emission_v2.F90:589-595) with t_y (:532-553)
// from a per-cell table (log phi, log(l_const/phi^2), l_const/phi^2):
// log l = log(l_const/phi^2) + log(-F), so one log of -F and one of t_y.
__device__ __forceinline__ double supply_log_tab(const DiodeParams& p, const double* __restrict__ wtab,
                                                 int cell, double F) {
  const double* t = wtab + 3 * (p.work_off + cell);
  const double LF = log(-1.0 * F);
  if (!p.image_charge) return 2.0 * LF - t[0];
  double l = t[2] * (-1.0 * F), ll = t[1] + LF;
  if (l > 1.0) { l = 1.0; ll = 0.0; }
  const double ty = 1.0 + l * ((1.0 / 9.0) - (1.0 / 18.0) * ll);
  return (2.0 * LF - 2.0 * log(ty)) - t[0];
}

// Elec_Supply_log at (x, y) for any work-function model: tabulated per cell
// or site, computed from phi(x, y) for the Gaussian model.
__device__ __forceinline__ double supply_log_xy(const DiodeParams& p, const double* __restrict__ wtab,
                                                double x, double y, double F) {
  const int cell = work_cell(p, x, y);
  if (cell < 0) return fn_supply_log(F, gaussian_work(p, p.work_data, x, y), p.image_charge);
  return supply_log_tab(p, wtab, cell, F);
}

// ---- FP32 forms of the MH arithmetic (FP32-compensated planar chains) -----------------
// The FP32 form keeps each chain as FP32 nm offsets from the emitter centre
// and draws and proposes in FP32; the field finish, the state handed to the
// emission test (x, y, F of accepted points) and the accept / reject decision
// are FP64 (mh_accept_one_f: an FP32 filter decides when it is certain, the
// FP64 targets otherwise).  FP64 is a small fraction of the FP32 rate on this
// part, and this arithmetic runs once per chain per work item.

// A uniform float in (0, 1) from 24 bits of a Philox word.
__device__ __forceinline__ float u01f(uint32_t w) {
  return ((float)(w >> 8) + 0.5f) * (1.0f / 16777216.0f);
}

__device__ __forceinline__ void rng2f(unsigned long long seed, uint32_t a, uint32_t b, uint32_t step,
                                      uint32_t tag, float* u1, float* u2) {
  uint32_t o[4];
  philox4x32(a, b, step, tag, (uint32_t)seed, (uint32_t)(seed >> 32), o);
  *u1 = u01f(o[0]);
  *u2 = u01f(o[2]);
}

// box_muller, Marsaglia polar form (src/mod_global.F90:578-595) in FP32, on
// the counters of gauss2.
__device__ __forceinline__ void gauss2f(unsigned long long seed, uint32_t chain, uint32_t it,
                                        uint32_t step, float* g1, float* g2) {
  for (uint32_t k = 0; k < 64; ++k) {
    float u1, u2;
    rng2f(seed, chain, it, step, RNG_GAUSS | (k << 8), &u1, &u2);
    const float x1 = 2.0f * u1 - 1.0f, x2 = 2.0f * u2 - 1.0f;
    const float w = x1 * x1 + x2 * x2;
    if (w < 1.0f && w > 0.0f) {
      const float m = sqrtf((-2.0f * logf(w)) / w);
      *g1 = x1 * m;
      *g2 = x2 * m;
      return;
    }
  }
  *g1 = 0.0f;
  *g2 = 0.0f;
}

// work_cell for a point given as FP32 nm offsets from the emitter centre.
__device__ __forceinline__ int work_cell_f(const DiodeParams& p, float x, float y) {
  if (p.work_nx == 1 && p.work_ny == 1) return 0;
  const float xs = (x + 0.5f * p.em_wx) / p.em_wx, ys = (y + 0.5f * p.em_wy) / p.em_wy;
  const int nx = p.work_nx, ny = p.work_ny;
  int xi = (int)floorf(xs * (float)nx) + 1, yi = (int)floorf(ys * (float)ny) + 1;
  xi = xi > nx ? nx : (xi < 1 ? 1 : xi);
  yi = yi > ny ? ny : (yi < 1 ? 1 : yi);
  yi = ny - yi + 1;
  return (yi - 1) * nx + (xi - 1);
}

// The FP32 chains compare targets by their parts.  Elec_Supply_log
// (src/mod_field_emission_v2.F90:589-595) is
//   s = 2 log(-F) - rho,   rho = 2 log t_y + log phi,
//   t_y = 1 + l (1/9 - log(l) / 18),  l = min(l_const / phi^2 (-F), 1)
// (t_y = 1 without image charges), and two targets differ by
//   d = s_n - s_c = 2 log(F_n / F_c) - (rho_n - rho_c),
// which the FP32 form evaluates without cancelling two values near 40
// (mh_accept_one_f).  A chain keeps rho and its field as floats.  2 log t_y
// lies in [0, 0.212] and is formed as 2 log1p(l (1/9 - log(l) / 18)).
__device__ __forceinline__ float rho_entry_f(const DiodeParams& p, float t0, float t2, float F) {
  if (!p.image_charge) return t0;
  const float l = t2 * (-F);
  float tau = 0.0f;                          // l below 1e-30: t_y - 1 < 4e-30
  if (l > 1.0f) tau = 1.0f / 9.0f;
  else if (l > 1.0e-30f) tau = l * ((1.0f / 9.0f) - (1.0f / 18.0f) * logf(l));
  return fmaf(2.0f, log1pf(tau), t0);
}

// Work-function cell or site of an FP32 chain's point (FP32 nm offsets from
// the emitter centre); -1 for the Gaussian model, whose phi varies within any
// cell.  It is the cell supply_log_chain_d takes.
__device__ __forceinline__ int chain_cell_f(const DiodeParams& p, float x, float y) {
  if (p.work_model == 1) return work_cell_f(p, x, y);
  return work_cell(p, p.org_x + (double)x * 1.0e-9, p.org_y + (double)y * 1.0e-9);
}

// log phi and l_const / phi^2 as floats at an FP32 chain's point of cell `cell`.
__device__ __forceinline__ void work_entry_f(const DiodeParams& p, const double* __restrict__ wtab, int cell,
                                             float x, float y, float* t0, float* t2) {
  if (cell >= 0) {
    const double* t = wtab + 3 * (p.work_off + cell);
    *t0 = (float)t[0]; *t2 = (float)t[2];
    return;
  }
  const double phi = gaussian_work(p, p.work_data, p.org_x + (double)x * 1.0e-9, p.org_y + (double)y * 1.0e-9);
  *t0 = (float)log(phi); *t2 = (float)(c_k.l_const / (phi * phi));
}

// rho of an FP32 chain's point for the field F < 0 (as a float).
__device__ __forceinline__ float rho_xy_f(const DiodeParams& p, const double* __restrict__ wtab, float x,
                                          float y, float F) {
  float t0, t2;
  work_entry_f(p, wtab, chain_cell_f(p, x, y), x, y, &t0, &t2);
  return rho_entry_f(p, t0, t2, F);
}

// ---- cathode z = 0 field, planar ----------------------------------------------------
// Sum over one j-tile of q_j sum_h h / r_h^3 (nm units) for a point at z = 0
// given as (x_hi, x_lo, y_hi, y_lo).  Uses the cathode pack: zk_hi =
// (x_hi, y_hi, z^2, q z), zk_lo = (x_lo, y_lo, z, q); z^2 >= 1e-20 so r^2 > 0.
template <bool NIC0>
__device__ __forceinline__ float z0_tile_f32(const float4* __restrict__ sh, const float4* __restrict__ sl,
                                             int kmax, float4 pp, int nic, float dnm) {
  float s0 = 0.f, s1 = 0.f;
  int k = 0;
  if (NIC0) {
#pragma unroll 4
    for (; k + 1 < kmax; k += 2) {   // two independent accumulators
      float4 h0 = sh[k], h1 = sh[k + 1];
      float2 l0 = *reinterpret_cast<const float2*>(&sl[k]);
      float2 l1 = *reinterpret_cast<const float2*>(&sl[k + 1]);
      float dx0 = (pp.x - h0.x) + (pp.y - l0.x), dy0 = (pp.z - h0.y) + (pp.w - l0.y);
      float dx1 = (pp.x - h1.x) + (pp.y - l1.x), dy1 = (pp.z - h1.y) + (pp.w - l1.y);
      float i0 = rsqrtf(fmaf(dx0, dx0, fmaf(dy0, dy0, h0.z)));
      float i1 = rsqrtf(fmaf(dx1, dx1, fmaf(dy1, dy1, h1.z)));
      s0 = fmaf(h0.w, (i0 * i0) * i0, s0);
      s1 = fmaf(h1.w, (i1 * i1) * i1, s1);
    }
  }
  for (; k < kmax; ++k) {
    float4 h = sh[k], l = sl[k];
    float dx = (pp.x - h.x) + (pp.y - l.x), dy = (pp.z - h.y) + (pp.w - l.y);
    float dxy2 = fmaf(dx, dx, dy * dy);
    float inv = rsqrtf(dxy2 + h.z);
    s0 = fmaf(h.w, (inv * inv) * inv, s0);
    if (!NIC0) {
      for (int n = 1; n <= nic; ++n) {
        float ha = l.z + 2.0f * n * dnm, hb = l.z - 2.0f * n * dnm;
        float ia = rsqrtf(fmaf(ha, ha, dxy2)), ib = rsqrtf(fmaxf(fmaf(hb, hb, dxy2), 1e-20f));
        s0 = fmaf(l.w * ha, (ia * ia) * ia, s0);
        s0 = fmaf(l.w * hb, (ib * ib) * ib, s0);
      }
    }
  }
  return s0 + s1;
}

// Tile sums for 2 NP points at z = 0 (nic = 0) in packed FP32x2 arithmetic:
// points 2i and 2i+1 in the .x and .y lanes of pair i.  The j data sit in
// shared memory duplicated and negated, s0 = (-x_hi, -x_hi, -x_lo, -x_lo),
// s1 = (-y_hi, ..), s2 = (z^2, z^2, q z, q z), so each step for a pair of
// points is one packed instruction (rsqrt stays per lane), and one set of
// shared loads feeds all 2 NP points.  The points are taken at their FP32 nm
// offsets (PX, PY: their high words; the FP32 MH chains are kept as such
// offsets), so dx = (p - x_hi) - x_lo: the first difference is exact for
// nearby pairs (Sterbenz) and the particle's low word restores its FP64
// position.
template <int NP>
__device__ __forceinline__ void z0_tile_x2(const float4* __restrict__ s0, const float4* __restrict__ s1,
                                           const float4* __restrict__ s2, int kmax, const float2* PX,
                                           const float2* PY, float* r) {
  float2 s[NP];
#pragma unroll
  for (int i = 0; i < NP; ++i) s[i] = make_float2(0.f, 0.f);
#pragma unroll 4
  for (int k = 0; k < kmax; ++k) {
    const float4 a = s0[k], b = s1[k], c = s2[k];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const float2 dx = __fadd2_rn(__fadd2_rn(PX[i], make_float2(a.x, a.y)), make_float2(a.z, a.w));
      const float2 dy = __fadd2_rn(__fadd2_rn(PY[i], make_float2(b.x, b.y)), make_float2(b.z, b.w));
      const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, make_float2(c.x, c.y)));
      float2 inv;
      inv.x = rsqrtf(r2.x);
      inv.y = rsqrtf(r2.y);
      s[i] = __ffma2_rn(make_float2(c.z, c.w), __fmul2_rn(__fmul2_rn(inv, inv), inv), s[i]);
    }
  }
#pragma unroll
  for (int i = 0; i < NP; ++i) { r[2 * i] += s[i].x; r[2 * i + 1] += s[i].y; }
}

// Partial F_z sums of the item for CPT points at z = 0 (FP32 compensated),
// given as (x_hi, x_lo, y_hi, y_lo) nm; blockDim threads load the j-tiles.
// The raw sums (nm units) are folded into (hi, lo) pairs across j-tiles with
// two-sum and returned as doubles; z0_finish turns them into V/m.
template <int CPT>
__device__ __forceinline__ void z0_item_sumN(const DiodeParams& p, const Pool& pool, const ItemRef& it,
                                             const float4* pts, float* out_hi, float* out_lo) {
  constexpr int NP = CPT / 2;
  __shared__ float4 sp[3][RD_TILE];
  float4* sh = sp[0];   // nic > 0: raw packs
  float4* sl = sp[1];
  const int off = p.off, tid = threadIdx.x, nt = blockDim.x;
  const int nic = p.image_charge ? p.N_ic_max : 0;
  const float dnm = (float)(p.d * 1.0e9);
  float hi[CPT], lo[CPT];
  float2 PX[NP], PY[NP];
#pragma unroll
  for (int i = 0; i < CPT; ++i) { hi[i] = 0.f; lo[i] = 0.f; }
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    PX[i] = make_float2(pts[2 * i].x, pts[2 * i + 1].x);
    PY[i] = make_float2(pts[2 * i].z, pts[2 * i + 1].z);
  }
  for (int jt = it.j0; jt < it.j1; jt += RD_TILE) {
    __syncthreads();
    for (int q = tid; q < RD_TILE; q += nt) {
      const int j = jt + q;
      if (j < it.j1) {
        const float4 h = pool.zk_hi[off + j], l = pool.zk_lo[off + j];
        if (nic == 0) {
          sp[0][q] = make_float4(-h.x, -h.x, -l.x, -l.x);
          sp[1][q] = make_float4(-h.y, -h.y, -l.y, -l.y);
          sp[2][q] = make_float4(h.z, h.z, h.w, h.w);
        } else {
          sh[q] = h; sl[q] = l;
        }
      }
    }
    __syncthreads();
    const int kmax = min(RD_TILE, it.j1 - jt);
    float t[CPT];
#pragma unroll
    for (int i = 0; i < CPT; ++i) t[i] = 0.f;
    if (nic == 0) {
      z0_tile_x2<NP>(sp[0], sp[1], sp[2], kmax, PX, PY, t);
    } else {
#pragma unroll
      for (int i = 0; i < CPT; ++i) t[i] = z0_tile_f32<false>(sh, sl, kmax, pts[i], nic, dnm);
    }
#pragma unroll
    for (int i = 0; i < CPT; ++i) two_sum_acc(hi[i], lo[i], t[i]);
  }
#pragma unroll
  for (int i = 0; i < CPT; ++i) { out_hi[i] = hi[i]; out_lo[i] = lo[i]; }
}

__device__ __forceinline__ double z0_tile_f64(const rd_d4* __restrict__ sj, int kmax, double px,
                                              double py, int nic, double d, double L2) {
  double s = 0.0;
  for (int k = 0; k < kmax; ++k) {
    rd_d4 pj = sj[k];
    double dx = px - pj.x, dy = py - pj.y, dxy2 = dx * dx + dy * dy;
    double r = sqrt(dxy2 + pj.z * pj.z) + L2;
    s += (pj.w * pj.z) / ((r * r) * r);
    for (int n = 1; n <= nic; ++n) {
      double h1 = pj.z + (2.0 * n) * d, h2 = pj.z - (2.0 * n) * d;
      double r1 = sqrt(dxy2 + h1 * h1) + L2, r2 = sqrt(dxy2 + h2 * h2) + L2;
      s += (pj.w * h1) / ((r1 * r1) * r1);
      s += (pj.w * h2) / ((r2 * r2) * r2);
    }
  }
  return s;
}

// A point at z = 0 in the FP32 frame of the diode: (x_hi, x_lo, y_hi, y_lo).
__device__ __forceinline__ float4 z0_point(const DiodeParams& p, double px, double py) {
  float4 r;
  split_nm(px, p.org_x, &r.x, &r.y);
  split_nm(py, p.org_y, &r.z, &r.w);
  return r;
}

// Partial F_z sum of the item for one point at z = 0, in the units that
// z0_finish turns into V/m.  Loads the j-tiles into shared memory.
template <int PREC>
__device__ __forceinline__ double z0_item_sum(const DiodeParams& p, const Pool& pool, const ItemRef& it,
                                              double px, double py, float4 pp, float4* sh,
                                              float4* sl, rd_d4* sj) {
  const int off = p.off, tid = threadIdx.x;
  const int nic = p.image_charge ? p.N_ic_max : 0;
  if (PREC == 1) {
    const float dnm = (float)(p.d * 1.0e9);
    float hi = 0.f, lo = 0.f;
    for (int jt = it.j0; jt < it.j1; jt += RD_TILE) {
      __syncthreads();
      int j = jt + tid;
      if (j < it.j1) { sh[tid] = pool.zk_hi[off + j]; sl[tid] = pool.zk_lo[off + j]; }
      __syncthreads();
      const int kmax = min(RD_TILE, it.j1 - jt);
      two_sum_acc(hi, lo, nic == 0 ? z0_tile_f32<true>(sh, sl, kmax, pp, 0, dnm)
                                   : z0_tile_f32<false>(sh, sl, kmax, pp, nic, dnm));
    }
    return (double)hi + (double)lo;
  } else {
    double s = 0.0;
    for (int jt = it.j0; jt < it.j1; jt += RD_TILE) {
      __syncthreads();
      int j = jt + tid;
      if (j < it.j1) sj[tid] = make_d4(pool.x[off + j], pool.y[off + j], pool.z[off + j], pool.q[off + j]);
      __syncthreads();
      s += z0_tile_f64(sj, min(RD_TILE, it.j1 - jt), px, py, nic, p.d, c_k.L2);
    }
    return s;
  }
}

// F_z from the summed partials.  Without image charges the x, y cancellation
// does not hold and the plain Coulomb z term is -z_j only: factor 1 not 2.
template <int PREC>
__device__ __forceinline__ double z0_finish(const DiodeParams& p, double s, double kscale) {
  double f = p.image_charge ? -2.0 : -1.0;
  if (PREC == 1) return p.E_z + f * kscale * s;
  return p.E_z + f * c_k.div_fac_c * s;
}

// Chunk partials of FP32 pair sums: a chunk of a tile with more than one
// stores its (hi, lo) pairs in the partial scratch (8 bytes per sum, as the
// FP64 partials); the tile's last chunk (tile_ticket) adds them in chunk order
// with pair_add and returns true, the others return false.  Float pairs keep
// ~44 bits, far below the FP32 tiles' own rounding, and their sum costs no
// FP64 operation.
template <int CPT>
__device__ __forceinline__ bool pair_partials(double* partial, int* tickets, const ItemRef& it, int g, int tid,
                                              int nt, float* hi, float* lo) {
  if (it.nch <= 1) return true;
  float2* pf = reinterpret_cast<float2*>(partial);
#pragma unroll
  for (int q = 0; q < CPT; ++q) pf[(size_t)g * RD_ITILE + tid + q * nt] = make_float2(hi[q], lo[q]);
  if (!tile_ticket(tickets, it)) return false;
#pragma unroll
  for (int q = 0; q < CPT; ++q) {
    float H = 0.0f, L = 0.0f;
    for (int c = 0; c < it.nch; ++c) {
      const float2 v = __ldcg(pf + (size_t)(it.base + c) * RD_ITILE + tid + q * nt);
      pair_add(H, L, v.x, v.y);
    }
    hi[q] = H; lo[q] = L;
  }
  return true;
}

// F_z at the supply quadrature points (qpp holds their FP32-frame split).
// FP32: 32 threads, four points each (the MH jump's form: one shared load feeds
// four points, and a point's sum is the same lane arithmetic in the same j
// order in any form); FP64: 128 threads, one point each.
template <int PREC>
__global__ void __launch_bounds__(PREC == 1 ? 32 : RD_ITILE, PREC == 1 ? 32 : 1)
k_z0_points(const DiodeParams* __restrict__ P, Pool pool, const PlanEntry* __restrict__ plan,
            const PlanHeader* __restrict__ ph, const double* __restrict__ qx,
            const double* __restrict__ qy, const float4* __restrict__ qpp, double* __restrict__ qF,
            double* __restrict__ partial, int* __restrict__ tickets, double kscale, int* __restrict__ queue) {
  __shared__ int s_item;
  __shared__ float4 sh[RD_TILE], sl[RD_TILE];
  __shared__ rd_d4 sj[RD_TILE];
  constexpr int CPT = PREC == 1 ? 4 : 1;
  const int nt = blockDim.x;
  const int total = ph->total_items, nd = ph->n_diodes, tid = threadIdx.x;
  for (int g = queue_first(0, total); g < total; g = queue_next(queue, &s_item, 0, total)) {
    ItemRef it = decode_item(plan, nd, g);
    const DiodeParams& p = P[it.d];
    const int m = plan[it.d].n_i, qo = p.q_off;
    double s[CPT];
    if constexpr (PREC == 1) {
      const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
      float4 pts[CPT];
#pragma unroll
      for (int q = 0; q < CPT; ++q) {
        const int i = it.i0 + tid + q * nt;
        pts[q] = i < m ? qpp[qo + i] : z4;
      }
      float hi[CPT], lo[CPT];
      z0_item_sumN<CPT>(p, pool, it, pts, hi, lo);
      if (!pair_partials<CPT>(partial, tickets, it, g, tid, nt, hi, lo)) continue;
#pragma unroll
      for (int q = 0; q < CPT; ++q) s[q] = (double)hi[q] + (double)lo[q];
    } else {
      const int i = it.i0 + tid;
      const bool valid = i < m;
      s[0] = z0_item_sum<PREC>(p, pool, it, valid ? qx[qo + i] : p.em_x0, valid ? qy[qo + i] : p.em_y0,
                               make_float4(0.f, 0.f, 0.f, 0.f), sh, sl, sj);
      if (it.nch > 1) {
        partial[(size_t)g * RD_ITILE + tid] = s[0];
        if (!tile_ticket(tickets, it)) continue;
        s[0] = 0.0;
        for (int c = 0; c < it.nch; ++c) s[0] += __ldcg(partial + (size_t)(it.base + c) * RD_ITILE + tid);
      }
    }
    for (int q = 0; q < CPT; ++q) {
      const int i = it.i0 + tid + q * nt;
      if (i < m) qF[qo + i] = z0_finish<PREC>(p, s[q], kscale);
    }
  }
  queue_leave(queue, 0, total);
}

// ---- supply integrals ------------------------------------------------------------------
__device__ __forceinline__ double block_sum(double v, double* red) {
  const int tid = threadIdx.x;
  red[tid] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (tid < s) red[tid] += red[tid + s];
    __syncthreads();
  }
  double r = red[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ long nint_d(double x) {
  return (long)(x >= 0 ? floor(x + 0.5) : -floor(-x + 0.5));
}

// N_sup = sum_k w_k A S(F_k), N_round = nint(N_sup + residual) (planar,
// Do_Field_Emission_Planar_rectangle :282-285) or nint(N_sup) (tip, :488).
// The FN supply of a point is FP64 transcendental work, so a diode's points
// are spread over RD_SUP_SPLIT blocks (contiguous ranges); each block writes
// its (supply, field) sums and k_supply_finish adds a diode's block sums in
// block order, so N_sup depends only on the diode's own points.
__device__ __forceinline__ bool supply_live(const DiodeParams& p, const DiodeDyn& y, const int* step_ptr) {
  return p.active && p.emission && *step_ptr - y.step_offset > p.emit_delay;   // emitter on (:181)
}

__global__ void __launch_bounds__(256)
k_supply_reduce(const DiodeParams* __restrict__ P, const DiodeDyn* __restrict__ Dy,
                const double* __restrict__ qx, const double* __restrict__ qy,
                const double* __restrict__ qw, const double* __restrict__ qF,
                const double* __restrict__ qfx, const double* __restrict__ qfy,
                const double* __restrict__ work, const int* __restrict__ step_ptr,
                double* __restrict__ sup_part) {
  __shared__ double red[256];
  const int d = blockIdx.x, b = blockIdx.y;
  const DiodeParams& p = P[d];
  if (!supply_live(p, Dy[d], step_ptr)) return;
  const int npt = (p.geometry == RD_G_TIP) ? 10000 : p.quad_n * p.quad_n;
  const int per = (npt + RD_SUP_SPLIT - 1) / RD_SUP_SPLIT;
  const int k0 = b * per, k1 = min(npt, k0 + per);
  // planar diodes without image charges carry all three field components (PM_SUPPLY_LAT):
  // their lateral mean goes to field.dt too
  const bool lat = p.geometry == RD_G_PLANAR && !p.image_charge;
  double acc = 0.0, fsum = 0.0, fxs = 0.0, fys = 0.0;
  for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
    double F = qF[p.q_off + k];
    fsum += F;
    if (lat) { fxs += qfx[p.q_off + k]; fys += qfy[p.q_off + k]; }
    if (p.geometry == RD_G_TIP) {   // Field_normal :105-112
      double nx, ny, nz;
      tip_normal(p, qx[p.q_off + k], qy[p.q_off + k], &nx, &ny, &nz);
      F = (nx * qfx[p.q_off + k] + ny * qfy[p.q_off + k]) + nz * F;
    }
    if (F < 0.0) {
      if (p.geometry == RD_G_TIP) {
        double t = fn_t_y(F, p.tip_phi, p.image_charge);   // Elec_Supply (tip) :1710-1718
        acc += (((qw[p.q_off + k] * c_k.a_FN) * (F * F)) * p.dt) / ((c_k.q0 * p.tip_phi) * (t * t));
      } else {
        double phi = work_at(p, work, qx[p.q_off + k], qy[p.q_off + k], nullptr);
        acc += qw[p.q_off + k] * fn_supply_v2(F, phi, p.image_charge, p.dt);
      }
    }
  }
  const double N_sup = block_sum(acc, red);
  const double F_sum = block_sum(fsum, red);
  const double Fx_sum = lat ? block_sum(fxs, red) : 0.0;   // block-uniform condition
  const double Fy_sum = lat ? block_sum(fys, red) : 0.0;
  if (threadIdx.x == 0) {
    double* o = sup_part + ((size_t)d * RD_SUP_SPLIT + b) * 4;
    o[0] = N_sup; o[1] = F_sum; o[2] = Fx_sum; o[3] = Fy_sum;
  }
}

__global__ void k_supply_finish(const DiodeParams* __restrict__ P, DiodeDyn* __restrict__ Dy, int nslots,
                                const int* __restrict__ step_ptr, const double* __restrict__ sup_part) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nslots) return;
  const DiodeParams& p = P[d];
  if (!p.active || !p.emission) return;
  DiodeDyn& y = Dy[d];
  if (!supply_live(p, y, step_ptr)) {   // the emitter is not on yet (:181)
    y.N_sup = 0.0; y.chains = y.chains_capped = y.chains_failed = 0;
    y.mh_acc = y.mh_rej = y.mh_done = 0;
    y.F_avg_z = 0.0; y.F_avg_x = 0.0; y.F_avg_y = 0.0; y.df_avg = 0.0;
    return;
  }
  const int npt = (p.geometry == RD_G_TIP) ? 10000 : p.quad_n * p.quad_n;
  double N_sup = 0.0, F_sum = 0.0, Fx_sum = 0.0, Fy_sum = 0.0;
  for (int b = 0; b < RD_SUP_SPLIT; ++b) {
    const double* o = sup_part + ((size_t)d * RD_SUP_SPLIT + b) * 4;
    N_sup += o[0]; F_sum += o[1]; Fx_sum += o[2]; Fy_sum += o[3];
  }
  y.N_sup = N_sup;
  y.F_avg_z = p.geometry == RD_G_TIP ? 0.0 : F_sum / npt;   // F_avg, :644-651 (planar)
  y.F_avg_x = p.geometry == RD_G_TIP ? 0.0 : Fx_sum / npt;
  y.F_avg_y = p.geometry == RD_G_TIP ? 0.0 : Fy_sum / npt;
  long nr;
  if (p.geometry == RD_G_TIP) {
    nr = nint_d(N_sup);
  } else {
    nr = nint_d(N_sup + y.residual);
    y.residual = N_sup - (double)nr;
  }
  long M = nr > 0 ? nr : 0;
  y.chains_capped = M > p.max_chains ? (int)(M - p.max_chains) : 0;
  y.chains = (int)(M > p.max_chains ? p.max_chains : M);
  y.chains_failed = 0;
  y.mh_acc = y.mh_rej = y.mh_done = 0;
}

// ---- MH chain initialisation: one warp per chain --------------------------------------
// Uniform proposals until the field is favourable (F < 0), at most
// init_rounds rounds (10000 in the reference, :1321-1364 and
// mod_emission_tip.f90:1292-1318).  Round 0 of every chain runs tiled in the
// jump kernels (it_idx 0); this kernel continues from round 1 for the chains
// whose first point was unfavourable.
template <int PREC>
__device__ double warp_field_planar_z0(const DiodeParams& p, const Pool& pool, int n, double px,
                                       double py, double kscale) {
  const int lane = threadIdx.x & 31, off = p.off;
  const int nic = p.image_charge ? p.N_ic_max : 0;
  double s;
  if (PREC == 1) {
    const float4 pp = z0_point(p, px, py);
    const float dnm = (float)(p.d * 1.0e9);
    float hi = 0.f, lo = 0.f;
    for (int j = lane; j < n; j += 32) {
      float4 h = pool.zk_hi[off + j], l = pool.zk_lo[off + j];
      two_sum_acc(hi, lo, nic == 0 ? z0_tile_f32<true>(&h, &l, 1, pp, 0, dnm)
                                   : z0_tile_f32<false>(&h, &l, 1, pp, nic, dnm));
    }
    s = (double)hi + (double)lo;
  } else {
    s = 0.0;
    for (int j = lane; j < n; j += 32) {
      rd_d4 pj = make_d4(pool.x[off + j], pool.y[off + j], pool.z[off + j], pool.q[off + j]);
      s += z0_tile_f64(&pj, 1, px, py, nic, p.d, c_k.L2);
    }
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return z0_finish<PREC>(p, s, kscale);
}

template <int PREC>
__device__ void warp_field_general(const DiodeParams& p, const Pool& pool, int n, double X,
                                   double Y, double Z, double kscale, double* ex, double* ey,
                                   double* ez) {
  const int lane = threadIdx.x & 31, off = p.off;
  double fx = 0, fy = 0, fz = 0;
  if (PREC == 1) {
    float4 ih, il, iih, iil;
    point_pack(p, X, Y, Z, ih, il, iih, iil);
    const float dnm = (float)(p.d * 1.0e9);
    F32Acc acc;
    acc.zero();
    TipSums ts;   // tip: the K-scaled image sums, kept apart (tip_tile_split_f32)
    ts.zero();
    for (int j = lane; j < n; j += 32) {
      float4 h = pool.pk_hi[off + j], l = pool.pk_lo[off + j];
      float tx = 0.f, ty = 0.f, tz = 0.f;
      if (p.geometry == RD_G_TIP) {
        float4 jh = pool.ip_hi[off + j];
        ts.dx = ts.dy = ts.dz = 0.f;
        tip_tile_split_f32<T_UPPER>(&h, &l, &jh, 1, ih, il, iih, -1, p.image_charge, ts);
        tx = ts.dx; ty = ts.dy; tz = ts.dz;
      } else {
        planar_tile_f32<T_UPPER, false>(&h, &l, 1, ih, il, -1, p.N_ic_max, dnm, p.image_charge, tx, ty, tz);
      }
      acc.add(tx, ty, tz);
    }
    fx = ((double)acc.hx + (double)acc.lx);
    fy = ((double)acc.hy + (double)acc.ly);
    fz = ((double)acc.hz + (double)acc.lz);
    if (p.geometry == RD_G_TIP) tip_split_finish(fx, fy, fz, ts, iih.w, p.image_charge, c_k.tip_K, &fx, &fy, &fz);
    fx *= kscale; fy *= kscale; fz *= kscale;
  } else {
    for (int j = lane; j < n; j += 32) {
      rd_d4 pj = make_d4(pool.x[off + j], pool.y[off + j], pool.z[off + j], pool.q[off + j]);
      if (p.geometry == RD_G_TIP)
        tip_tile_f64<T_UPPER>(&pj, 1, X, Y, Z, c_k.div_fac_c, -1, p.image_charge, p, c_k.L2, c_k.tip_K, fx, fy, fz);
      else
        planar_tile_f64<T_UPPER>(&pj, 1, X, Y, Z, c_k.div_fac_c, -1, p.N_ic_max, p.d, p.image_charge, c_k.L2, fx, fy, fz);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    fx += __shfl_xor_sync(0xffffffffu, fx, o);
    fy += __shfl_xor_sync(0xffffffffu, fy, o);
    fz += __shfl_xor_sync(0xffffffffu, fz, o);
  }
  double vx, vy, vz;
  vacuum_field(p, X, Y, Z, &vx, &vy, &vz);
  *ex = vx + fx; *ey = vy + fy; *ez = vz + fz;
}

__device__ __forceinline__ double tip_target_log(const DiodeParams& p, double F, double xi) {
  double t = fn_t_y(F, p.tip_phi, p.image_charge);   // Tip_fe_target_log :1213-1219
  double sup = (((p.dt / c_k.q0) * c_k.a_FN) / ((t * t) * p.tip_phi)) * (F * F);
  double v = sup > 2.2250738585072014e-308 ? sup : 2.2250738585072014e-308;
  return log(v) + 0.5 * log(xi * xi - p.eta_1 * p.eta_1);
}

template <int PREC>
__global__ void k_mh_init(const DiodeParams* __restrict__ P, DiodeDyn* __restrict__ Dy, Pool pool,
                          const PlanEntry* __restrict__ plan, const PlanHeader* __restrict__ ph,
                          ChainState cs, const int* __restrict__ ch_off, const double* __restrict__ wtab,
                          const int* __restrict__ step_ptr, double kscale) {
  const int nd = ph->n_diodes;
  const int warps_total = (gridDim.x * blockDim.x) >> 5;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  // chain prefix: plan[d].pad0 holds the first global chain index of diode d
  int total = nd > 0 ? plan[nd - 1].pad0 + plan[nd - 1].n_i : 0;
  for (int g = wid; g < total; g += warps_total) {
    int lo = 0, hi = nd - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (plan[mid].pad0 <= g) lo = mid; else hi = mid - 1; }
    const int d = lo, c = g - plan[d].pad0;
    const DiodeParams& p = P[d];
    const int n = plan[d].n_j, k = ch_off[d] + c;
    const uint32_t step = (uint32_t)(*step_ptr - Dy[d].step_offset);
    if (cs.ok[k]) continue;   // round 0 made it (k_mh_jump_planar / k_mh_jump_tip, it_idx 0)
    int ok = 0;
    double F = 1.0, sup = -1.79769313486231570e308, X = 0, Y = 0, Z = 0, xi = 1.0, ph_ = 0.0;
    for (int r = 1; r < p.init_rounds && !ok; ++r) {
      double u1, u2;
      rng2(p.seed, (uint32_t)c, (uint32_t)r, step, RNG_INIT, &u1, &u2);
      if (p.geometry == RD_G_TIP) {
        double txi = 1.0 + (p.max_xi - 1.0) * u1, tph = (2.0 * c_k.pi) * u2;
        double x, y, z, ex, ey, ez, nx, ny, nz;
        tip_xyz(p, txi, p.eta_1, tph, &x, &y, &z);
        warp_field_general<PREC>(p, pool, n, x, y, z, kscale, &ex, &ey, &ez);
        tip_normal(p, x, y, &nx, &ny, &nz);
        double Fn = (nx * ex + ny * ey) + nz * ez;
        if (Fn < 0.0) { ok = 1; F = Fn; X = x; Y = y; Z = z; xi = txi; ph_ = tph; sup = tip_target_log(p, Fn, txi); }
      } else if constexpr (PREC == 1) {   // FP32 chains: the draw of k_mh_jump_planar's round 0
        float v1, v2;
        rng2f(p.seed, (uint32_t)c, (uint32_t)r, step, RNG_INIT, &v1, &v2);
        const float fx = fminf(fmaf(v1, p.em_wx, -p.em_hx), p.em_hx);
        const float fy = fminf(fmaf(v2, p.em_wy, -p.em_hy), p.em_hy);
        const double x = p.org_x + (double)fx * 1.0e-9, y = p.org_y + (double)fy * 1.0e-9;
        const double Fz = warp_field_planar_z0<PREC>(p, pool, n, x, y, kscale);
        if (Fz < 0.0) {
          ok = 1; F = Fz; X = x; Y = y;
          if (lane == 0) {
            cs.fx[k] = fx; cs.fy[k] = fy;
            const float Ff = (float)Fz;
            cs.fsup[k] = rho_xy_f(p, wtab, fx, fy, Ff);
            cs.fF[k] = Ff;
          }
        }
      } else {
        const double x = u1 * p.em_Lx + p.em_x0, y = u2 * p.em_Ly + p.em_y0;
        const double Fz = warp_field_planar_z0<PREC>(p, pool, n, x, y, kscale);
        if (Fz < 0.0) {
          ok = 1; F = Fz; X = x; Y = y;
          sup = supply_log_xy(p, wtab, x, y, Fz);
        }
      }
    }
    if (lane == 0) {
      if (!ok) {
        F = 1.0; sup = -1.79769313486231570e308;
        if (p.geometry == RD_G_TIP) { xi = 1.0; ph_ = 0.0; tip_xyz(p, 1.0, p.eta_1, 0.0, &X, &Y, &Z); }
        else { X = p.em_x0; Y = p.em_y0; }
        atomicAdd(&Dy[d].chains_failed, 1);
      }
      cs.ok[k] = ok; cs.F[k] = F; cs.sup[k] = sup;
      if (p.geometry == RD_G_TIP) { cs.x[k] = xi; cs.y[k] = ph_; cs.tx[k] = X; cs.ty[k] = Y; cs.tz[k] = Z; }
      else {
        cs.x[k] = X; cs.y[k] = Y;
        if (ok) {   // Gaussian pair of the first jump
          if constexpr (PREC == 1) {
            float g1, g2;
            gauss2f(p.seed, (uint32_t)c, 1u, step, &g1, &g2);
            cs.fgx[k] = g1; cs.fgy[k] = g2;
          } else {
            double g1, g2;
            gauss2(p.seed, (uint32_t)c, 1u, step, &g1, &g2);
            cs.gx[k] = g1; cs.gy[k] = g2;
          }
        }
      }
    }
  }
}

// ---- MH jump iteration ---------------------------------------------------------------------
// The MH_std update of one jump iteration from its acceptance counts
// (MH_std_update :603-612, once per iteration after the warm-up jumps).
// MH_std_update (:603-612) in parts: the factor of a jump with A accepted and
// R rejected proposals (A + R > 0), and the clamped product.
__device__ __forceinline__ double mh_std_gain(int A, int R, double* rate) {
  *rate = (double)A / (double)(A + R);
  return exp(0.025 * (*rate - 0.35));
}
__device__ __forceinline__ double mh_std_clamp(const DiodeParams& p, double s) {
  if (s > p.mh_hi) s = p.mh_hi; else if (s < p.mh_lo) s = p.mh_lo;
  return s;
}
__device__ __forceinline__ void mh_std_step(const DiodeParams& p, double* mh_std, double* a_rate, int it_idx,
                                            int ndim_first, int A, int R) {
  if (it_idx > ndim_first && A + R > 0) {
    const double g = mh_std_gain(A, R, a_rate);
    *mh_std = mh_std_clamp(p, *mh_std * g);
  }
}

__device__ __forceinline__ void mh_counts_and_update(const DiodeParams& p, DiodeDyn& y, int tiles,
                                                     int it_idx, int ndim_first, int a, int r,
                                                     int* red_i) {
  // block reduce (a, r); blockDim is a power of two <= RD_ITILE
  const int tid = threadIdx.x, nt = blockDim.x;
  red_i[tid] = a; red_i[RD_ITILE + tid] = r;
  __syncthreads();
  for (int s = nt / 2; s > 0; s >>= 1) {
    if (tid < s) { red_i[tid] += red_i[tid + s]; red_i[RD_ITILE + tid] += red_i[RD_ITILE + tid + s]; }
    __syncthreads();
  }
  if (tid == 0) {
    atomicAdd(&y.mh_acc, red_i[0]);
    atomicAdd(&y.mh_rej, red_i[RD_ITILE]);
    __threadfence();
    int prev = atomicAdd(&y.mh_done, 1);
    if (prev == tiles - 1) {
      __threadfence();
      int A = atomicExch(&y.mh_acc, 0), R = atomicExch(&y.mh_rej, 0);
      y.mh_done = 0;
      mh_std_step(p, &y.MH_std, &y.a_rate, it_idx, ndim_first, A, R);
    }
  }
  __syncthreads();
}

// Accept / reject of one planar proposal (:1400-1443) and the Gaussian pair
// of the chain's next proposal.  Returns 1 for accepted, 0 for rejected.
__device__ __forceinline__ int mh_accept_one(const DiodeParams& p, ChainState& cs, const double* wtab,
                                             int c, int k, int it_idx, uint32_t step, double F,
                                             double wx, double wy) {
  int a = 0;
  if (F < 0.0) {
    const double sn = supply_log_xy(p, wtab, wx, wy, F);
    const double sc = cs.sup[k];
    bool take = sn >= sc;
    if (!take) {
      double u1, u2;
      rng2(p.seed, (uint32_t)c, (uint32_t)it_idx, step, RNG_ACCEPT, &u1, &u2);
      take = log(u1) <= sn - sc;
    }
    if (take) { cs.x[k] = wx; cs.y[k] = wy; cs.sup[k] = sn; cs.F[k] = F; a = 1; }
  }
  if (it_idx < p.mh_jumps) {
    double g1, g2;
    gauss2(p.seed, (uint32_t)c, (uint32_t)(it_idx + 1), step, &g1, &g2);
    cs.gx[k] = g1; cs.gy[k] = g2;
  }
  return a;
}

// The FP64 target Elec_Supply_log (src/mod_field_emission_v2.F90:589-595) of
// an FP32 chain's point (FP32 nm offsets from the emitter centre), with the
// work-function cell or site chosen exactly as chain_cell_f chooses it.
__device__ __forceinline__ double supply_log_chain_d(const DiodeParams& p, const double* __restrict__ wtab,
                                                     float x, float y, double F) {
  if (p.work_model == 1) return supply_log_tab(p, wtab, work_cell_f(p, x, y), F);
  const double X = p.org_x + (double)x * 1.0e-9, Y = p.org_y + (double)y * 1.0e-9;
  const int cell = work_cell(p, X, Y);
  if (cell >= 0) return supply_log_tab(p, wtab, cell, F);
  return fn_supply_log(F, gaussian_work(p, p.work_data, X, Y), p.image_charge);
}

// The FP64 form's accept test for a decision the FP32 filter leaves open
// (rare; kept out of line so that it does not cost the pair-sum loop
// registers).  o0, o1 are the Philox words of the FP64 form's uniform u
// (u01_words).
__device__ __noinline__ bool mh_take_fp64(const DiodeParams& p, const double* __restrict__ wtab, float wx,
                                          float wy, double F, float cx, float cy, double Fc, uint32_t o0,
                                          uint32_t o1) {
  const double snd = supply_log_chain_d(p, wtab, wx, wy, F);
  const double scd = supply_log_chain_d(p, wtab, cx, cy, Fc);
  return snd >= scd || log(u01_words(o0, o1)) <= snd - scd;
}

// Guard of the FP32 acceptance filter: ten times a bound on how far its
// estimates of d = s_n - s_c and of log u can lie from the FP64 form's values.
// With e = 2^-24: 2 log(F_n / F_c) from the fields rounded to floats and one
// division is within 6.2e + 2e |.| of its value; each rho within
// 1.95e + 2e |rho| (logf and log1pf within 1 ulp, the table entries rounded to
// floats, t_y - 1 <= 1/9 with |l d(t_y)/dl| <= 1/18); log u within
// 2.01e + 2e |log u| (the 53-bit u rounded to a float); three sums rounded.
// In all |error| <= 12.2e + 5e S with S = |2 log(F_n / F_c)| + |rho_n| +
// |rho_c| (+ |log u| once it is formed): 7.3e-7 + 3.0e-7 S.  The FP64 values'
// own rounding (~1e-13) does not matter at this scale.
__device__ __forceinline__ float mh_guard(float S) { return 8.0e-6f + 4.0e-6f * S; }

// The accept / reject decision of an FP32 chain (:1400-1443) as the FP64 form
// takes it: take the proposal (wx, wy; field F, Ff = (float)F; rho_n) iff
// s_n >= s_c or log u <= s_n - s_c, with the FP64 targets and the 53-bit
// uniform u of the FP64 form; the chain is at (cx, cy) with field Fc (Fcf its
// float) and rho_c.  The FP32 estimates decide whenever they lie further than
// mh_guard from the threshold, where the FP64 comparison must agree; inside
// the guard the FP64 test runs (about one decision in 10^5).  Equal fields
// and one work-function cell give equal FP64 targets, hence s_n >= s_c.
__device__ __forceinline__ bool mh_decide_f(const DiodeParams& p, const double* __restrict__ wtab, int c,
                                            int it_idx, uint32_t step, double F, float Ff, float rn, float wx,
                                            float wy, float cx, float cy, double Fc, float Fcf, float rc) {
  const float l2 = 2.0f * logf(Ff / Fcf);
  const float df = l2 - (rn - rc);
  const float S = fabsf(l2) + fabsf(rn) + fabsf(rc);
  if (isfinite(df) && df >= mh_guard(S)) return true;   // s_n > s_c in FP64 too
  if (df == 0.0f && __double_as_longlong(F) == __double_as_longlong(Fc)) {
    const int cn = chain_cell_f(p, wx, wy);
    if (cn >= 0 && cn == chain_cell_f(p, cx, cy)) return true;
  }
  uint32_t o[4];
  philox4x32((uint32_t)c, (uint32_t)it_idx, step, RNG_ACCEPT, (uint32_t)p.seed, (uint32_t)(p.seed >> 32), o);
  // u = o0 / 2^32 + (o1 >> 11) / 2^53 exactly (u01_words); the float carries two roundings
  const float lu = logf(fmaf((float)(o[1] >> 11), 1.1102230246251565e-16f, (float)o[0] * 2.3283064365386963e-10f));
  if (isfinite(df)) {
    const float g = mh_guard(S + fabsf(lu));
    if (lu <= df - g) return true;
    if (lu > df + g) return false;
  }
  return mh_take_fp64(p, wtab, wx, wy, F, cx, cy, Fc, o[0], o[1]);
}

// mh_accept_one for the FP32 chains (proposal wx, wy in FP32 nm offsets), the
// decision by mh_decide_f.  Chains store their point, rho and field as floats
// and the field in FP64 (cs.F), from which mh_take_fp64 recomputes the FP64
// target when it is needed.  The point in FP64 metres (cs.x, cs.y), which only
// the emission test reads, is formed once, at the last jump.
__device__ __forceinline__ int mh_accept_one_f(const DiodeParams& p, ChainState& cs, const double* wtab,
                                               int c, int k, int it_idx, uint32_t step, double F,
                                               float wx, float wy) {
  int a = 0;
  float cx = cs.fx[k], cy = cs.fy[k];
  if (F < 0.0) {
    const float Ff = (float)F;
    const float rn = rho_xy_f(p, wtab, wx, wy, Ff);
    if (mh_decide_f(p, wtab, c, it_idx, step, F, Ff, rn, wx, wy, cx, cy, cs.F[k], cs.fF[k], cs.fsup[k])) {
      cs.fx[k] = wx; cs.fy[k] = wy; cs.fsup[k] = rn; cs.fF[k] = Ff; cs.F[k] = F;
      cx = wx; cy = wy;
      a = 1;
    }
  }
  if (it_idx < p.mh_jumps) {
    float g1, g2;
    gauss2f(p.seed, (uint32_t)c, (uint32_t)(it_idx + 1), step, &g1, &g2);
    cs.fgx[k] = g1; cs.fgy[k] = g2;
  } else {
    cs.x[k] = p.org_x + (double)cx * 1.0e-9;
    cs.y[k] = p.org_y + (double)cy * 1.0e-9;
  }
  return a;
}

// Proposal of planar chain c (slot k) for a jump: round 0 of the uniform start
// (init, :1321-1364), the current point (dry: autotuner timing), or the stored
// Gaussian pair times the step size (sx, sy) plus the current point, reflected
// at the emitter edges (check_limits_metro_rec :1466-1516).  FP32 chains: nm
// offsets from the emitter centre, half widths hx, hy.
__device__ __forceinline__ void mh_propose_f32(const DiodeParams& p, const ChainState& cs, int k, int c, int ok,
                                               bool init, bool dry, uint32_t step, float sx, float sy, float hx,
                                               float hy, float* px, float* py) {
  float x = 0.0f, yv = 0.0f;
  if (init && ok) {
    float u1, u2;
    rng2f(p.seed, (uint32_t)c, 0u, step, RNG_INIT, &u1, &u2);
    x = fminf(fmaf(u1, p.em_wx, -hx), hx);
    yv = fminf(fmaf(u2, p.em_wy, -hy), hy);
  } else if (dry && ok) {
    x = cs.fx[k]; yv = cs.fy[k];
  } else if (ok) {
    x = fmaf(cs.fgx[k], sx, cs.fx[k]);
    yv = fmaf(cs.fgy[k], sy, cs.fy[k]);
    if (x > hx) x = hx - (x - hx); else if (x < -hx) x = -hx - (x + hx);
    if (yv > hy) yv = hy - (yv - hy); else if (yv < -hy) yv = -hy - (yv + hy);
  }
  *px = x; *py = yv;
}

__device__ __forceinline__ void mh_propose_f64(const DiodeParams& p, const ChainState& cs, int k, int c, int ok,
                                               bool init, bool dry, uint32_t step, double sx, double sy,
                                               double* px, double* py) {
  double wx = p.em_x0, wy = p.em_y0;
  if (init && ok) {
    double u1, u2;
    rng2(p.seed, (uint32_t)c, 0u, step, RNG_INIT, &u1, &u2);
    wx = u1 * p.em_Lx + p.em_x0;
    wy = u2 * p.em_Ly + p.em_y0;
  } else if (dry && ok) {
    wx = cs.x[k]; wy = cs.y[k];
  } else if (ok) {
    double x = cs.gx[k] * sx + cs.x[k], yv = cs.gy[k] * sy + cs.y[k];
    const double hx = p.em_x0 + p.em_Lx, hy = p.em_y0 + p.em_Ly;
    if (x > hx) x = hx - (x - hx); else if (x < p.em_x0) x = (p.em_x0 - x) + p.em_x0;
    if (yv > hy) yv = hy - (yv - hy); else if (yv < p.em_y0) yv = (p.em_y0 - yv) + p.em_y0;
    wx = x; wy = yv;
  }
  *px = wx; *py = wy;
}

// Round 0 of a chain's uniform start, given the field F at its first draw: a
// favourable point (F < 0) makes the chain, with its target and the Gaussian
// pair of jump 1; otherwise k_mh_init continues from round 1.
__device__ __forceinline__ void mh_start_f32(const DiodeParams& p, ChainState& cs, const double* wtab, int k, int c,
                                             uint32_t step, double F, float x, float y) {
  if (F < 0.0 && p.init_rounds > 0) {
    cs.ok[k] = 1; cs.F[k] = F;
    cs.fx[k] = x; cs.fy[k] = y;
    cs.x[k] = p.org_x + (double)x * 1.0e-9;
    cs.y[k] = p.org_y + (double)y * 1.0e-9;
    const float Ff = (float)F;
    cs.fsup[k] = rho_xy_f(p, wtab, x, y, Ff);
    cs.fF[k] = Ff;
    float g1, g2;
    gauss2f(p.seed, (uint32_t)c, 1u, step, &g1, &g2);
    cs.fgx[k] = g1; cs.fgy[k] = g2;
  } else {
    cs.ok[k] = 0;
  }
}

__device__ __forceinline__ void mh_start_f64(const DiodeParams& p, ChainState& cs, const double* wtab, int k, int c,
                                             uint32_t step, double F, double x, double y) {
  if (F < 0.0 && p.init_rounds > 0) {
    cs.ok[k] = 1; cs.F[k] = F; cs.x[k] = x; cs.y[k] = y;
    cs.sup[k] = supply_log_xy(p, wtab, x, y, F);
    double g1, g2;
    gauss2(p.seed, (uint32_t)c, 1u, step, &g1, &g2);
    cs.gx[k] = g1; cs.gy[k] = g2;
  } else {
    cs.ok[k] = 0;
  }
}

// One Metropolis-Hastings jump iteration of the planar chains (it_idx >= 1),
// or round 0 of their uniform start (it_idx == 0: every chain of the step
// evaluates its first uniform draw here, tiled like a jump; the chains that
// drew an unfavourable point continue in k_mh_init from round 1), or a dry
// pass for the autotuner (it_idx < 0: the field at every chain's current
// point, nothing written but the scratch).  The
// proposal is the stored Gaussian pair (box_muller, src/mod_global.F90:
// 578-595) times the step size of this iteration (fixed during the warm-up,
// MH_std afterwards, :1373-1378) plus the current position, reflected at the
// emitter edges (check_limits_metro_rec :1466-1516).  The CTA completing a
// tile then runs the accept / reject test of its chains (:1400-1443), draws
// their next Gaussian pairs and counts acceptances; the tile completing the
// diode updates MH_std from the iteration's acceptance rate (:1438-1443).
// FP32: 32 threads, four chains each, at most 64 registers so that 32 CTAs
// (the per-SM block limit) are resident: 32 warps instead of the 28 that
// 72 registers allowed, +1.6 % on the served step; FP64: 128 threads, one
// chain each.  LONE (FP32): 64 threads, two chains each, so that a diode's few
// tiles spread over twice the warps (the default for a single emitting planar
// diode; rd_autotune may pick it for any mix); a chain's sum is the same lane
// arithmetic in the same j order either way.
template <int PREC, int LONE>
__global__ void __launch_bounds__(PREC == 1 ? (LONE ? 64 : 32) : RD_ITILE, PREC == 1 ? (LONE ? 16 : 32) : 1)
k_mh_jump_planar(const DiodeParams* __restrict__ P, DiodeDyn* __restrict__ Dy, Pool pool,
                 const PlanEntry* __restrict__ plan, const PlanHeader* __restrict__ ph, ChainState cs,
                 const int* __restrict__ ch_off, const double* __restrict__ wtab,
                 const int* __restrict__ step_ptr, int it_idx, double* __restrict__ partial,
                 int* __restrict__ tickets, double kscale, int* __restrict__ queue, int part, int nparts) {
  __shared__ int red_i[2 * RD_ITILE];
  __shared__ int s_item;
  constexpr int CPT = PREC == 1 ? (LONE ? 2 : 4) : 1;
  const int nt = blockDim.x;
  const int total = ph->total_items, nd = ph->n_diodes, tid = threadIdx.x;
  const bool init = it_idx == 0;
  const bool dry = it_idx < 0;   // timing pass: field at the current points, nothing written
  int lo, hi;   // this launch's part of the plan (part_range)
  part_range(plan, nd, total, part, nparts, &lo, &hi);
  for (int g = queue_first(lo, hi); g < hi; g = queue_next(queue, &s_item, lo, hi)) {
    ItemRef it = decode_item(plan, nd, g);
    const DiodeParams& p = P[it.d];
    if (p.geometry != RD_G_PLANAR || it_idx > p.mh_jumps) continue;
    DiodeDyn& y = Dy[it.d];
    const int ndim_first = (p.mh_jumps + 2) / 4;   // nint(0.25 mh_jumps), :1141
    const int M = plan[it.d].n_i;
    const uint32_t step = (uint32_t)(*step_ptr - y.step_offset);
    int ok[CPT], kk[CPT];
    double wx[CPT], wy[CPT];   // FP64 chains: proposal (m)
    float fwx[CPT], fwy[CPT];  // FP32 chains: proposal (nm from the emitter centre)
    if constexpr (PREC == 1) {
      const float mhs = (float)y.MH_std;
      const float sx = (it_idx > ndim_first) ? p.em_wx * mhs : p.em_wx * 0.10f;
      const float sy = (it_idx > ndim_first) ? p.em_wy * mhs : p.em_wy * 0.10f;
      const float hx = p.em_hx, hy = p.em_hy;
      for (int q = 0; q < CPT; ++q) {
        const int c = it.i0 + tid + q * nt;
        kk[q] = ch_off[it.d] + c;
        ok[q] = (c < M) ? (init ? 1 : cs.ok[kk[q]]) : 0;
        mh_propose_f32(p, cs, kk[q], c, ok[q], init, dry, step, sx, sy, hx, hy, &fwx[q], &fwy[q]);
      }
    } else {
      const double mhs = y.MH_std;
      const double sx = (it_idx > ndim_first) ? p.em_Lx * mhs : p.em_Lx * 0.10;
      const double sy = (it_idx > ndim_first) ? p.em_Ly * mhs : p.em_Ly * 0.10;
      for (int q = 0; q < CPT; ++q) {
        const int c = it.i0 + tid + q * nt;
        kk[q] = ch_off[it.d] + c;
        ok[q] = (c < M) ? (init ? 1 : cs.ok[kk[q]]) : 0;
        mh_propose_f64(p, cs, kk[q], c, ok[q], init, dry, step, sx, sy, &wx[q], &wy[q]);
      }
    }
    double s[CPT];
    if constexpr (PREC == 1) {
      float4 pts[CPT];
#pragma unroll
      for (int q = 0; q < CPT; ++q) pts[q] = make_float4(fwx[q], 0.f, fwy[q], 0.f);
      float hi[CPT], lo[CPT];
      z0_item_sumN<CPT>(p, pool, it, pts, hi, lo);
      if (!pair_partials<CPT>(partial, tickets, it, g, tid, nt, hi, lo)) continue;
#pragma unroll
      for (int q = 0; q < CPT; ++q) s[q] = (double)hi[q] + (double)lo[q];
    } else {
      __shared__ float4 sh[RD_TILE], sl[RD_TILE];
      __shared__ rd_d4 sj[RD_TILE];
      s[0] = z0_item_sum<PREC>(p, pool, it, wx[0], wy[0], make_float4(0.f, 0.f, 0.f, 0.f), sh, sl, sj);
      if (it.nch > 1) {
        partial[(size_t)g * RD_ITILE + tid] = s[0];
        if (!tile_ticket(tickets, it)) continue;
        s[0] = 0.0;
        for (int cc = 0; cc < it.nch; ++cc) s[0] += __ldcg(partial + (size_t)(it.base + cc) * RD_ITILE + tid);
      }
    }
    // epilogue of the completed tile
    if (dry) continue;
    if (init) {   // a favourable start (F < 0) makes the chain; the others go to k_mh_init
      for (int q = 0; q < CPT; ++q) {
        if (!ok[q]) continue;
        const int c = it.i0 + tid + q * nt, k = kk[q];
        const double F = z0_finish<PREC>(p, s[q], kscale);
        if constexpr (PREC == 1) mh_start_f32(p, cs, wtab, k, c, step, F, fwx[q], fwy[q]);
        else mh_start_f64(p, cs, wtab, k, c, step, F, wx[q], wy[q]);
      }
      continue;
    }
    int a = 0, r = 0;
    for (int q = 0; q < CPT; ++q) {
      if (!ok[q]) continue;
      const int c = it.i0 + tid + q * nt;
      const double F = z0_finish<PREC>(p, s[q], kscale);
      int acc;
      if constexpr (PREC == 1) acc = mh_accept_one_f(p, cs, wtab, c, kk[q], it_idx, step, F, fwx[q], fwy[q]);
      else acc = mh_accept_one(p, cs, wtab, c, kk[q], it_idx, step, F, wx[q], wy[q]);
      a += acc;
      r += 1 - acc;
    }
    mh_counts_and_update(p, y, plan[it.d].tiles, it_idx, ndim_first, a, r, red_i);
  }
  queue_leave(queue, lo, hi);
}

// mh_decide_f for a vacuum-field chain (F_n = F_c), out of line: k_mh_vacuum
// reaches it only for a proposal into another work-function cell.
__device__ __noinline__ bool mh_decide_vac(const DiodeParams& p, const double* __restrict__ wtab, int c, int it_idx,
                                           uint32_t step, double F, float Ff, float rn, float wx, float wy, float cx,
                                           float cy, float rc) {
  return mh_decide_f(p, wtab, c, it_idx, step, F, Ff, rn, wx, wy, cx, cy, F, Ff, rc);
}

// The whole batched MH sampling of a planar diode with no particle in flight
// (rd_mh_vacuum), in one launch: one cluster of RD_VAC_CTAS CTAs per diode
// slot runs round 0 of the chains' start, the rounds k_mh_init would run, and
// every jump.  With no charges the field at every point is z0_finish(p, 0), the
// value the tiled kernels compute from their empty pair sums.  Each thread
// keeps its RD_VAC_CPT chains in registers for the whole sampling and writes
// them back at the end; the proposal, start and accept arithmetic is that of
// mh_propose_*, mh_start_* and mh_accept_one(_f) step for step (the tiled path
// keeps the same state in memory), so the chains evolve bit for bit as in
// k_mh_jump_planar + k_mh_init.  One field everywhere makes the FP64 targets of
// two points of one work-function cell equal, so such a proposal is taken
// (s_n >= s_c) without a draw, as the FP64 form takes it; a uniform work
// function makes every jump such, and k_mh_vacuum_uniform samples those
// diodes instead (this kernel leaves them).  After each jump the CTAs reduce their
// acceptance counts, exchange them through distributed shared memory across a
// cluster barrier and each apply the same MH_std update (MH_std_update
// :603-612); jumps alternate between two count buffers, so a CTA never
// overwrites counts another may still read.  Clusters of slots that are not
// such diodes leave at once (the test is uniform over a cluster).
template <int PREC>
__global__ void __cluster_dims__(RD_VAC_CTAS, 1, 1) __launch_bounds__(RD_VAC_THREADS)
k_mh_vacuum(const DiodeParams* __restrict__ P, DiodeDyn* __restrict__ Dy, ChainState cs,
            const int* __restrict__ ch_off, const double* __restrict__ wtab, const int* __restrict__ step_ptr,
            double kscale, int nslots) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  constexpr int NW = RD_VAC_THREADS / 32;
  __shared__ unsigned s_cnt[2];          // this CTA's counts of a jump: (rejected << 16) | accepted
  __shared__ unsigned s_red[NW];
  __shared__ double s_mhs;
  __shared__ float s_mhf;
  // the diode's parameters and supply-target table in shared memory for the whole
  // sampling: global data would be fetched again after every cluster barrier
  __shared__ DiodeParams sp;
  __shared__ double swt[3 * RD_VAC_WTAB];
  __shared__ float2 swf[RD_VAC_WTAB];   // (log phi, l_const / phi^2) as floats
  const int d = blockIdx.x / RD_VAC_CTAS;
  if (d >= nslots) return;
  DiodeDyn& y = Dy[d];
  if (!P[d].active || !rd_mh_vacuum(P[d], y) || y.chains <= 0) return;
  const int rank = (int)cl.block_rank(), tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  {
    const int* src = reinterpret_cast<const int*>(P + d);
    int* dst = reinterpret_cast<int*>(&sp);
    for (int k = tid; k < (int)(sizeof(DiodeParams) / sizeof(int)); k += blockDim.x) dst[k] = src[k];
  }
  __syncthreads();
  const int cells = sp.work_model == 1 ? sp.work_nx * sp.work_ny : (sp.work_model == 4 ? sp.work_nx : 0);
  const bool wsh = cells <= RD_VAC_WTAB;   // the table's values are the same wherever they are read
  if (wsh)
    for (int k = tid; k < cells; k += blockDim.x) {
      const double* t = wtab + 3 * (sp.work_off + k);
      swt[3 * k] = t[0]; swt[3 * k + 1] = t[1]; swt[3 * k + 2] = t[2];
      swf[k] = make_float2((float)t[0], (float)t[2]);
    }
  __syncthreads();
  // a uniform work function: every cell's entry the same (bit for bit)
  int differs = 0;
  if (wsh)
    for (int k = tid; k < cells; k += blockDim.x)
      for (int e = 0; e < 3; ++e)
        differs |= __double_as_longlong(swt[3 * k + e]) != __double_as_longlong(swt[e]);
  const bool uniform = __syncthreads_or(differs) == 0 && wsh && cells >= 1 && sp.mh_jumps <= RD_VAC_MAXJ;
  if (uniform) return;   // k_mh_vacuum_uniform samples it (the test is uniform over the cluster)
  if (wsh && tid == 0) sp.work_off = 0;   // entries now at swt[3 * cell]
  __syncthreads();
  if (wsh) wtab = swt;
  const DiodeParams& p = sp;
  const int M = y.chains, base = ch_off[d];
  const int G = RD_VAC_CTAS * RD_VAC_THREADS, g0 = rank * RD_VAC_THREADS + tid;
  const uint32_t step = (uint32_t)(*step_ptr - y.step_offset);
  const double F = z0_finish<PREC>(p, 0.0, kscale);
  const float Ff = (float)F;
  const bool start_ok = F < 0.0 && p.init_rounds > 0;
  const int ndim_first = (p.mh_jumps + 2) / 4;
  double mhs = y.MH_std, arate = y.a_rate;
  float mhf = (float)mhs;
  // the FP32 chains' rho at (x, y) of cell `cell`, from the staged float table
  auto rho_at = [&](int cell, float x, float yv) -> float {
    float t0, t2;
    if (wsh && cell >= 0) { const float2 e = swf[cell]; t0 = e.x; t2 = e.y; }
    else work_entry_f(p, wtab, cell, x, yv, &t0, &t2);
    return rho_entry_f(p, t0, t2, Ff);
  };
  // chain state in registers: FP32 chains (nm offsets) or FP64 chains (m)
  int ok[RD_VAC_CPT], cc[RD_VAC_CPT];
  float fx[RD_VAC_CPT], fy[RD_VAC_CPT], rc[RD_VAC_CPT], fgx[RD_VAC_CPT], fgy[RD_VAC_CPT];
  double dx[RD_VAC_CPT], dy[RD_VAC_CPT], dsup[RD_VAC_CPT], dgx[RD_VAC_CPT], dgy[RD_VAC_CPT];
  // the start: round 0; a chain that fails it fails every round (the field does not change)
  int failed = 0;
#pragma unroll
  for (int q = 0; q < RD_VAC_CPT; ++q) {
    const int c = g0 + q * G;
    ok[q] = 0; cc[q] = -1;
    fx[q] = fy[q] = rc[q] = fgx[q] = fgy[q] = 0.0f;
    dx[q] = dy[q] = dsup[q] = dgx[q] = dgy[q] = 0.0;
    if (c >= M) continue;
    if constexpr (PREC == 1) {   // mh_propose_f32 (init) + mh_start_f32
      float u1, u2;
      rng2f(p.seed, (uint32_t)c, 0u, step, RNG_INIT, &u1, &u2);
      const float x = fminf(fmaf(u1, p.em_wx, -p.em_hx), p.em_hx);
      const float yv = fminf(fmaf(u2, p.em_wy, -p.em_hy), p.em_hy);
      if (start_ok) {
        ok[q] = 1; fx[q] = x; fy[q] = yv;
        cc[q] = chain_cell_f(p, x, yv);
        rc[q] = rho_at(cc[q], x, yv);
        gauss2f(p.seed, (uint32_t)c, 1u, step, &fgx[q], &fgy[q]);
      }
    } else {                     // mh_propose_f64 (init) + mh_start_f64
      double u1, u2;
      rng2(p.seed, (uint32_t)c, 0u, step, RNG_INIT, &u1, &u2);
      const double x = u1 * p.em_Lx + p.em_x0, yv = u2 * p.em_Ly + p.em_y0;
      if (start_ok) {
        ok[q] = 1; dx[q] = x; dy[q] = yv;
        dsup[q] = supply_log_xy(p, wtab, x, yv, F);
        gauss2(p.seed, (uint32_t)c, 1u, step, &dgx[q], &dgy[q]);
      }
    }
    if (!ok[q]) failed++;
  }
  if (failed) atomicAdd(&y.chains_failed, failed);
  for (int it = 1; it <= p.mh_jumps; ++it) {
    unsigned cnt = 0;   // (rejected << 16) | accepted over this thread's chains
    if constexpr (PREC == 1) {
      const float mf = mhf;
      const float sx = (it > ndim_first) ? p.em_wx * mf : p.em_wx * 0.10f;
      const float sy = (it > ndim_first) ? p.em_wy * mf : p.em_wy * 0.10f;
      const float hx = p.em_hx, hy = p.em_hy;
#pragma unroll
      for (int q = 0; q < RD_VAC_CPT; ++q) {
        if (!ok[q]) continue;   // an ok chain has F < 0
        const int c = g0 + q * G;
        // mh_propose_f32
        float x = fmaf(fgx[q], sx, fx[q]);
        float yv = fmaf(fgy[q], sy, fy[q]);
        if (x > hx) x = hx - (x - hx); else if (x < -hx) x = -hx - (x + hx);
        if (yv > hy) yv = hy - (yv - hy); else if (yv < -hy) yv = -hy - (yv + hy);
        // mh_accept_one_f
        const int cn = chain_cell_f(p, x, yv);
        bool take = cn >= 0 && cn == cc[q];   // equal FP64 targets
        float rn = rc[q];
        if (!take) {
          rn = rho_at(cn, x, yv);
          take = mh_decide_vac(p, wtab, c, it, step, F, Ff, rn, x, yv, fx[q], fy[q], rc[q]);
        }
        if (take) { fx[q] = x; fy[q] = yv; rc[q] = rn; cc[q] = cn; cnt += 1u; }
        else cnt += 1u << 16;
        if (it < p.mh_jumps) gauss2f(p.seed, (uint32_t)c, (uint32_t)(it + 1), step, &fgx[q], &fgy[q]);
      }
    } else {
      const double sx = (it > ndim_first) ? p.em_Lx * mhs : p.em_Lx * 0.10;
      const double sy = (it > ndim_first) ? p.em_Ly * mhs : p.em_Ly * 0.10;
      const double hx = p.em_x0 + p.em_Lx, hy = p.em_y0 + p.em_Ly;
#pragma unroll
      for (int q = 0; q < RD_VAC_CPT; ++q) {
        if (!ok[q]) continue;
        const int c = g0 + q * G;
        // mh_propose_f64
        double x = dgx[q] * sx + dx[q], yv = dgy[q] * sy + dy[q];
        if (x > hx) x = hx - (x - hx); else if (x < p.em_x0) x = (p.em_x0 - x) + p.em_x0;
        if (yv > hy) yv = hy - (yv - hy); else if (yv < p.em_y0) yv = (p.em_y0 - yv) + p.em_y0;
        // mh_accept_one
        const double sn = supply_log_xy(p, wtab, x, yv, F);
        const double sc = dsup[q];
        bool take = sn >= sc;
        if (!take) {
          double u1, u2;
          rng2(p.seed, (uint32_t)c, (uint32_t)it, step, RNG_ACCEPT, &u1, &u2);
          take = log(u1) <= sn - sc;
        }
        if (take) { dx[q] = x; dy[q] = yv; dsup[q] = sn; cnt += 1u; }
        else cnt += 1u << 16;
        if (it < p.mh_jumps) gauss2(p.seed, (uint32_t)c, (uint32_t)(it + 1), step, &dgx[q], &dgy[q]);
      }
    }
    // at most RD_VAC_MAX_CHAINS = 8192 chains: each half of the packed sum stays below 2^16
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    if (lane == 0) s_red[w] = cnt;
    __syncthreads();
    const int par = it & 1;
    if (w == 0) {   // this CTA's counts
      unsigned v = __reduce_add_sync(0xffffffffu, lane < NW ? s_red[lane] : 0u);
      if (lane == 0) s_cnt[par] = v;
    }
    cl.sync();   // every CTA's counts of this jump are in place
    if (w == 0) {   // the cluster's counts: lane q reads CTA q's
      const unsigned v = __reduce_add_sync(0xffffffffu, lane < RD_VAC_CTAS ? *cl.map_shared_rank(&s_cnt[par], lane) : 0u);
      if (lane == 0) {
        mh_std_step(p, &mhs, &arate, it, ndim_first, (int)(v & 0xffffu), (int)(v >> 16));
        s_mhs = mhs; s_mhf = (float)mhs;
      }
    }
    __syncthreads();
    mhs = s_mhs; mhf = s_mhf;
  }
  // the chains back to memory, as the tiled path leaves them
#pragma unroll
  for (int q = 0; q < RD_VAC_CPT; ++q) {
    const int c = g0 + q * G;
    if (c >= M) continue;
    const int k = base + c;
    cs.ok[k] = ok[q];
    if (!ok[q]) {   // k_mh_init's record of a chain with no favourable start
      cs.F[k] = 1.0; cs.sup[k] = -1.79769313486231570e308;
      cs.x[k] = p.em_x0; cs.y[k] = p.em_y0;
      continue;
    }
    cs.F[k] = F;
    if constexpr (PREC == 1) {
      cs.fx[k] = fx[q]; cs.fy[k] = fy[q]; cs.fsup[k] = rc[q]; cs.fF[k] = Ff;
      cs.fgx[k] = fgx[q]; cs.fgy[k] = fgy[q];
      cs.x[k] = p.org_x + (double)fx[q] * 1.0e-9;
      cs.y[k] = p.org_y + (double)fy[q] * 1.0e-9;
    } else {
      cs.x[k] = dx[q]; cs.y[k] = dy[q]; cs.sup[k] = dsup[q]; cs.gx[k] = dgx[q]; cs.gy[k] = dgy[q];
    }
  }
  if (rank == 0 && tid == 0) { y.MH_std = mhs; y.a_rate = arate; }
  cl.sync();   // no CTA leaves while another may still read its counts
}

// The batched MH sampling of a vacuum-field diode (rd_mh_vacuum) whose work
// function is uniform (every cell's supply-target entry the same, bit for bit).
// One field and one target everywhere: every proposal of a started chain is
// taken (s_n >= s_c), so each jump's counts are (T, 0) for the T = M chains
// that started (none when the field is not favourable) and the MH_std schedule
// is known before the first jump.  A chain's walk then needs only its Gaussian
// pairs, whose Philox counters (chain, jump, step) make them independent: the
// RD_VU_THREADS threads of a block draw them for its RD_VU_CHAINS chains, a
// chunk of RD_VU_JCHUNK jumps at a time, into shared memory, and each chain
// walks the chunk in one lane of warp 1.  Thread 0 forms the schedule with
// mh_std_gain / mh_std_clamp meanwhile, as mh_std_step does jump by jump; once
// the clamped step size stops changing, every later jump takes it.  Blocks
// (x: group of chains, y: diode slot) spread a diode's chains over the GPU.
// The start, the draws and the step arithmetic are those of k_mh_vacuum (and
// of mh_propose_* / mh_start_* on the tiled path), in the same order, so the
// chains end bit for bit as there.  The last block of a diode to finish writes
// MH_std and a_rate (a ticket on mh_done, which is 0 between jumps), after
// every block has read the old values.
template <int PREC>
__global__ void __launch_bounds__(RD_VU_THREADS)
k_mh_vacuum_uniform(const DiodeParams* __restrict__ P, DiodeDyn* __restrict__ Dy, ChainState cs,
                    const int* __restrict__ ch_off, const double* __restrict__ wtab,
                    const int* __restrict__ step_ptr, double kscale) {
  using Real = typename std::conditional<PREC == 1, float, double>::type;
  __shared__ DiodeParams sp;
  __shared__ double s_seq[RD_VAC_MAXJ + 1];   // the step-size factor of each jump
  __shared__ float s_seqf[RD_VAC_MAXJ + 1];   // the same for the FP32 chains
  __shared__ double s_end[2];
  __shared__ Real s_g[RD_VU_JCHUNK][RD_VU_CHAINS][2];   // Gaussian pairs of a chunk of jumps
  __shared__ int s_last;
  const int d = blockIdx.y, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  DiodeDyn& y = Dy[d];
  if (!P[d].active || !rd_mh_vacuum(P[d], y) || y.chains <= 0) return;
  const int M = y.chains, c0 = blockIdx.x * RD_VU_CHAINS;
  if (c0 >= M) return;
  {
    const int* src = reinterpret_cast<const int*>(P + d);
    int* dst = reinterpret_cast<int*>(&sp);
    for (int k = tid; k < (int)(sizeof(DiodeParams) / sizeof(int)); k += blockDim.x) dst[k] = src[k];
  }
  __syncthreads();
  const DiodeParams& p = sp;
  // the test of k_mh_vacuum: every entry of the diode's table equal to the first
  const int cells = p.work_model == 1 ? p.work_nx * p.work_ny : (p.work_model == 4 ? p.work_nx : 0);
  const bool wsh = cells <= RD_VAC_WTAB;
  int differs = 0;
  if (wsh)
    for (int k = tid; k < cells; k += blockDim.x)
      for (int e = 0; e < 3; ++e)
        differs |= __double_as_longlong(wtab[3 * (p.work_off + k) + e]) !=
                   __double_as_longlong(wtab[3 * p.work_off + e]);
  if (!(__syncthreads_or(differs) == 0 && wsh && cells >= 1 && p.mh_jumps <= RD_VAC_MAXJ)) return;
  const int J = p.mh_jumps, base = ch_off[d];
  const uint32_t step = (uint32_t)(*step_ptr - y.step_offset);
  const double F = z0_finish<PREC>(p, 0.0, kscale);
  const float Ff = (float)F;
  const bool start_ok = F < 0.0 && p.init_rounds > 0;
  const int ndim_first = (J + 2) / 4;
  const int nc = min(RD_VU_CHAINS, M - c0);   // chains of this block
  if (tid == 0) {   // the schedule
    const int T = start_ok ? M : 0;
    double m = y.MH_std, ar = y.a_rate, rate = 0.0, g = 0.0;
    if (T > 0) g = mh_std_gain(T, 0, &rate);
    for (int it = 1; it <= J; ++it) {
      if (it > ndim_first && T > 0) {
        s_seq[it] = m; s_seqf[it] = (float)m;
        ar = rate;
        const double nx = mh_std_clamp(p, m * g);
        if (nx == m) {   // a fixed point: every later jump takes the same step size
          const float mf = (float)m;
          for (int k = it + 1; k <= J; ++k) { s_seq[k] = m; s_seqf[k] = mf; }
          break;
        }
        m = nx;
      } else {
        s_seq[it] = (it > ndim_first) ? m : 0.10;
        s_seqf[it] = (it > ndim_first) ? (float)m : 0.10f;
      }
    }
    s_end[0] = m; s_end[1] = ar;
  }
  // the start (round 0) of the block's chains, one per lane of warp 1
  const int c = c0 + lane;
  const bool mine = w == 1 && lane < nc;
  Real px = 0, py = 0, gx = 0, gy = 0;
  float rc = 0.0f;
  double dsup = 0.0;
  if (mine && start_ok) {
    if constexpr (PREC == 1) {   // mh_propose_f32 (init) + mh_start_f32
      float u1, u2;
      rng2f(p.seed, (uint32_t)c, 0u, step, RNG_INIT, &u1, &u2);
      px = fminf(fmaf(u1, p.em_wx, -p.em_hx), p.em_hx);
      py = fminf(fmaf(u2, p.em_wy, -p.em_hy), p.em_hy);
      rc = rho_xy_f(p, wtab, px, py, Ff);
    } else {                     // mh_propose_f64 (init) + mh_start_f64
      double u1, u2;
      rng2(p.seed, (uint32_t)c, 0u, step, RNG_INIT, &u1, &u2);
      px = u1 * p.em_Lx + p.em_x0;
      py = u2 * p.em_Ly + p.em_y0;
      dsup = supply_log_xy(p, wtab, px, py, F);
    }
    if (J == 0) {   // the start's draw is the chain's last
      if constexpr (PREC == 1) gauss2f(p.seed, (uint32_t)c, 1u, step, &gx, &gy);
      else gauss2(p.seed, (uint32_t)c, 1u, step, &gx, &gy);
    }
  }
  if (start_ok) {
    for (int j0 = 1; j0 <= J; j0 += RD_VU_JCHUNK) {
      const int nj = min(RD_VU_JCHUNK, J - j0 + 1);
      __syncthreads();   // the previous chunk's walk is done with s_g
      // the Gaussian pair of jump it is the draw with counter it (the start's for jump 1)
      for (int k = tid - (j0 == 1 ? 32 : 0); k < nj * nc; k += blockDim.x - (j0 == 1 ? 32 : 0)) {
        if (k < 0) break;   // thread 0's warp forms the schedule during the first chunk
        const int jj = k / nc, q = k - jj * nc;
        Real a, b;
        if constexpr (PREC == 1) gauss2f(p.seed, (uint32_t)(c0 + q), (uint32_t)(j0 + jj), step, &a, &b);
        else gauss2(p.seed, (uint32_t)(c0 + q), (uint32_t)(j0 + jj), step, &a, &b);
        s_g[jj][q][0] = a; s_g[jj][q][1] = b;
      }
      __syncthreads();
      if (mine) {
        for (int jj = 0; jj < nj; ++jj) {
          const int it = j0 + jj;
          gx = s_g[jj][lane][0]; gy = s_g[jj][lane][1];
          if constexpr (PREC == 1) {
            const float mf = s_seqf[it];
            const float sx = p.em_wx * mf, sy = p.em_wy * mf, hx = p.em_hx, hy = p.em_hy;
            float x = fmaf(gx, sx, px), yv = fmaf(gy, sy, py);
            if (x > hx) x = hx - (x - hx); else if (x < -hx) x = -hx - (x + hx);
            if (yv > hy) yv = hy - (yv - hy); else if (yv < -hy) yv = -hy - (yv + hy);
            px = x; py = yv;
          } else {
            const double sx = p.em_Lx * s_seq[it], sy = p.em_Ly * s_seq[it];
            const double hx = p.em_x0 + p.em_Lx, hy = p.em_y0 + p.em_Ly;
            double x = gx * sx + px, yv = gy * sy + py;
            if (x > hx) x = hx - (x - hx); else if (x < p.em_x0) x = (p.em_x0 - x) + p.em_x0;
            if (yv > hy) yv = hy - (yv - hy); else if (yv < p.em_y0) yv = (p.em_y0 - yv) + p.em_y0;
            px = x; py = yv;
          }
        }
      }
    }
  }
  __syncthreads();   // the schedule's end values
  // the chains back to memory, as k_mh_vacuum leaves them
  if (mine) {
    const int k = base + c;
    cs.ok[k] = start_ok ? 1 : 0;
    if (!start_ok) {   // k_mh_init's record of a chain with no favourable start
      cs.F[k] = 1.0; cs.sup[k] = -1.79769313486231570e308;
      cs.x[k] = p.em_x0; cs.y[k] = p.em_y0;
    } else {
      cs.F[k] = F;
      if constexpr (PREC == 1) {
        cs.fx[k] = px; cs.fy[k] = py; cs.fsup[k] = rc; cs.fF[k] = Ff;
        cs.fgx[k] = gx; cs.fgy[k] = gy;
        cs.x[k] = p.org_x + (double)px * 1.0e-9;
        cs.y[k] = p.org_y + (double)py * 1.0e-9;
      } else {
        cs.x[k] = px; cs.y[k] = py; cs.sup[k] = dsup; cs.gx[k] = gx; cs.gy[k] = gy;
      }
    }
  }
  if (tid == 0) {
    if (!start_ok) atomicAdd(&y.chains_failed, nc);
    __threadfence();
    const int nblk = (M + RD_VU_CHAINS - 1) / RD_VU_CHAINS;
    s_last = atomicAdd(&y.mh_done, 1) == nblk - 1;
    if (s_last) {   // every block of the diode has read MH_std and a_rate
      y.mh_done = 0;
      y.MH_std = s_end[0];
      y.a_rate = s_end[1];
    }
  }
}

// Field sums of one j-tile at CPT tip proposals (upper role: the point's own
// apex-sphere image, as tip_tile_split_f32<T_UPPER>); one shared load feeds all of the
// thread's points.  The tip image term of the reference carries an extra
// factor K = q0 / (4 pi eps0) (acc_tip_ic_force.inc:17-22):
//   E = sum_j q_j [ d/|d|^3 + K (d/|d|^3 - c e/|e|^3) ] = (1 + K) D - K c S,
// D = sum q d/|d|^3, S = sum q e/|e|^3, c = R / dis of the point (applied by
// the caller); the two sums are kept apart here (td, te) and combined in
// FP64 by the caller, so the K-scaled image part is not lost below the FP32
// resolution of the direct part.  (A packed FP32x2 form of this tile ran no
// faster: the FMA pipe, 75 % busy, is the limit either way.)  The proposals sit
// on the FP32 nm grid (k_mh_propose), so d = (p - x_hi) - x_lo.  S is formed
// from high words only (e = image_hi - x_hi): its relative error, ~1e-5 for
// the nearest charges, is ~1e-14 of the field once scaled by K.
// ELEC: every charge of the tile is -1 (q/q0 of an electron; the common case,
// known from the tile load): the charge multiply is dropped and the sign goes
// into the accumulating FMA, which saves one of the ~27 FP32 operations of
// each term pair.
template <int CPT, bool ELEC, bool IC>
__device__ __forceinline__ void tip_point_tiles_f32(const float4* __restrict__ sh, const float4* __restrict__ sl,
                                                    int kmax, const float4* ih, const float4* iih,
                                                    float (*td)[3], float (*te)[3]) {
  constexpr bool ic = IC;   // image charges on: a template argument, no branch in the pair loop
  float dx_[CPT], dy_[CPT], dz_[CPT], ex_[CPT], ey_[CPT], ez_[CPT];
#pragma unroll
  for (int q = 0; q < CPT; ++q) dx_[q] = dy_[q] = dz_[q] = ex_[q] = ey_[q] = ez_[q] = 0.f;
  constexpr int kUnroll = RD_TIP_UNROLL;
#pragma unroll kUnroll
  for (int k = 0; k < kmax; ++k) {
    const float4 h = sh[k], l = sl[k];
    const float qj = h.w;
#pragma unroll
    for (int q = 0; q < CPT; ++q) {
      const float dx = (ih[q].x - h.x) - l.x;
      const float dy = (ih[q].y - h.y) - l.y;
      const float dz = (ih[q].z - h.z) - l.z;
      const float inv = rsqrtf(fmaf(dz, dz, fmaf(dx, dx, fmaf(dy, dy, 1e-20f))));
      const float s = ELEC ? -((inv * inv) * inv) : qj * ((inv * inv) * inv);
      dx_[q] = fmaf(s, dx, dx_[q]);
      dy_[q] = fmaf(s, dy, dy_[q]);
      dz_[q] = fmaf(s, dz, dz_[q]);
      if (ic) {   // high words only: this sum enters scaled by K ~ 1e-9 (see above)
        const float ex = iih[q].x - h.x;
        const float ey = iih[q].y - h.y;
        const float ez = iih[q].z - h.z;
        const float re = rsqrtf(fmaf(ez, ez, fmaf(ex, ex, fmaf(ey, ey, 1e-20f))));
        const float se = ELEC ? -((re * re) * re) : qj * ((re * re) * re);
        ex_[q] = fmaf(se, ex, ex_[q]);
        ey_[q] = fmaf(se, ey, ey_[q]);
        ez_[q] = fmaf(se, ez, ez_[q]);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < CPT; ++q) {
    td[q][0] += dx_[q]; td[q][1] += dy_[q]; td[q][2] += dz_[q];
    te[q][0] += ex_[q]; te[q][1] += ey_[q]; te[q][2] += ez_[q];
  }
}

// One Metropolis-Hastings jump iteration of the tip chains (it_idx >= 1), or
// round 0 of their uniform start (it_idx == 0; the chains whose first point
// sees F >= 0 continue in k_mh_init).  The proposals come from k_mh_propose,
// already packed into the FP32 frame.  The field at the proposal (all three
// components: direct and sphere-image terms) is summed over the item's
// j-chunk; the CTA completing a tile projects the total field (plus the
// hyperboloid vacuum field) on the surface normal and runs the accept /
// reject test (Metro_algo_tip_v3, src/mod_emission_tip.f90:1351-1389).
// FP32: RD_TIP_CPT chains per thread (RD_ITILE / RD_TIP_CPT threads); FP64:
// 128 threads, one chain each.
template <int PREC>
__global__ void __launch_bounds__(RD_ITILE)
k_mh_jump_tip(const DiodeParams* __restrict__ P, DiodeDyn* __restrict__ Dy, Pool pool,
              const PlanEntry* __restrict__ plan, const PlanHeader* __restrict__ ph,
              ChainState cs, const int* __restrict__ ch_off, const int* __restrict__ step_ptr,
              int it_idx, double* __restrict__ partial, int* __restrict__ tickets, double kscale,
              int* __restrict__ queue) {
  __shared__ int s_item;
  __shared__ int red_i[2 * RD_ITILE];
  constexpr int CPT = PREC == 1 ? RD_TIP_CPT : 1;
  const int nt = blockDim.x;
  const int total = ph->total_items, nd = ph->n_diodes, tid = threadIdx.x;
  const bool init = it_idx == 0;
  for (int g = queue_first(0, total); g < total; g = queue_next(queue, &s_item, 0, total)) {
    ItemRef it = decode_item(plan, nd, g);
    const DiodeParams& p = P[it.d];
    if (p.geometry != RD_G_TIP || it_idx > p.mh_jumps) continue;
    DiodeDyn& y = Dy[it.d];
    const uint32_t step = (uint32_t)(*step_ptr - y.step_offset);
    const int M = plan[it.d].n_i;
    const int ndim_first = (int)nint_d(p.mh_jumps * 0.25);
    const int off = p.off;
    int ok[CPT], kk[CPT];
#pragma unroll
    for (int q = 0; q < CPT; ++q) {
      const int c = it.i0 + tid + q * nt;
      kk[q] = ch_off[it.d] + c;
      ok[q] = (c < M) ? (init ? 1 : cs.ok[kk[q]]) : 0;
    }
    double f3[CPT][3];
    if constexpr (PREC == 1) {
      __shared__ float4 sh[RD_TILE], sl[RD_TILE];
      float4 ih[CPT], iih[CPT];
#pragma unroll
      for (int q = 0; q < CPT; ++q) {
        if (ok[q]) {
          const int k = kk[q];
          ih[q] = cs.pph[k]; iih[q] = cs.pih[k];
        } else {   // idle lane: a point far above the tip, no image
          ih[q] = make_float4(0.f, 0.f, 1.0e4f, 1.f);
          iih[q] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
      }
      F32Acc accd[CPT];        // direct part: two-sum across tiles
      float acce[CPT][3];      // image part (scaled by K ~ 1e-9 at the end): plain float sums
#pragma unroll
      for (int q = 0; q < CPT; ++q) { accd[q].zero(); acce[q][0] = acce[q][1] = acce[q][2] = 0.f; }
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
        float td[CPT][3], te[CPT][3];
#pragma unroll
        for (int q = 0; q < CPT; ++q) td[q][0] = td[q][1] = td[q][2] = te[q][0] = te[q][1] = te[q][2] = 0.f;
        const int kmax = min(RD_TILE, it.j1 - jt);
        if (p.image_charge) {
          if (elec) tip_point_tiles_f32<CPT, true, true>(sh, sl, kmax, ih, iih, td, te);
          else tip_point_tiles_f32<CPT, false, true>(sh, sl, kmax, ih, iih, td, te);
        } else {
          if (elec) tip_point_tiles_f32<CPT, true, false>(sh, sl, kmax, ih, iih, td, te);
          else tip_point_tiles_f32<CPT, false, false>(sh, sl, kmax, ih, iih, td, te);
        }
#pragma unroll
        for (int q = 0; q < CPT; ++q) {
          accd[q].add(td[q][0], td[q][1], td[q][2]);
          acce[q][0] += te[q][0]; acce[q][1] += te[q][1]; acce[q][2] += te[q][2];
        }
      }
      const double K = c_k.tip_K, cd = p.image_charge ? (1.0 + K) * kscale : kscale, ce = K * kscale;
#pragma unroll
      for (int q = 0; q < CPT; ++q) {
        const double cq = ce * (double)iih[q].w;
        f3[q][0] = ((double)accd[q].hx + (double)accd[q].lx) * cd - (double)acce[q][0] * cq;
        f3[q][1] = ((double)accd[q].hy + (double)accd[q].ly) * cd - (double)acce[q][1] * cq;
        f3[q][2] = ((double)accd[q].hz + (double)accd[q].lz) * cd - (double)acce[q][2] * cq;
      }
    } else {
      __shared__ rd_d4 sj[RD_TILE];
      double X, Y, Z;
      if (ok[0]) { X = cs.pxx[kk[0]]; Y = cs.pyy[kk[0]]; Z = cs.pzz[kk[0]]; }
      else tip_xyz(p, 1.5, p.eta_1, 0.0, &X, &Y, &Z);
      double fx = 0, fy = 0, fz = 0;
      for (int jt = it.j0; jt < it.j1; jt += RD_TILE) {
        __syncthreads();
        int j = jt + tid;
        if (j < it.j1) sj[tid] = make_d4(pool.x[off + j], pool.y[off + j], pool.z[off + j], pool.q[off + j]);
        __syncthreads();
        tip_tile_f64<T_UPPER>(sj, min(RD_TILE, it.j1 - jt), X, Y, Z, c_k.div_fac_c, -1,
                              p.image_charge, p, c_k.L2, c_k.tip_K, fx, fy, fz);
      }
      f3[0][0] = fx; f3[0][1] = fy; f3[0][2] = fz;
    }
    if (it.nch > 1) {
      double* pp = partial + (size_t)g * 3 * RD_ITILE;
#pragma unroll
      for (int q = 0; q < CPT; ++q)
        for (int i = 0; i < 3; ++i) pp[i * RD_ITILE + tid + q * nt] = f3[q][i];
      if (!tile_ticket(tickets, it)) continue;
#pragma unroll
      for (int q = 0; q < CPT; ++q)
        for (int i = 0; i < 3; ++i) {
          double s = 0.0;
          for (int cc = 0; cc < it.nch; ++cc)
            s += __ldcg(partial + (size_t)(it.base + cc) * 3 * RD_ITILE + i * RD_ITILE + tid + q * nt);
          f3[q][i] = s;
        }
    }
    // epilogue of the completed tile: F = n . (E_vac + E_particles) at the proposal
    int a = 0, r = 0;
#pragma unroll
    for (int q = 0; q < CPT; ++q) {
      if (!ok[q]) continue;
      const int c = it.i0 + tid + q * nt, k = kk[q];
      const double X = cs.pxx[k], Y = cs.pyy[k], Z = cs.pzz[k], nxi = cs.px[k], nph = cs.py[k];
      if (init) {   // a favourable start makes the chain; the others go to k_mh_init
        double ex, ey, ez, nx, ny, nz;
        tip_field_E(p, X, Y, Z, &ex, &ey, &ez);
        ex += f3[q][0]; ey += f3[q][1]; ez += f3[q][2];
        tip_normal(p, X, Y, &nx, &ny, &nz);
        const double F = (nx * ex + ny * ey) + nz * ez;
        if (F < 0.0 && p.init_rounds > 0) {
          cs.ok[k] = 1; cs.x[k] = nxi; cs.y[k] = nph; cs.F[k] = F; cs.sup[k] = tip_target_log(p, F, nxi);
          cs.tx[k] = X; cs.ty[k] = Y; cs.tz[k] = Z;
        } else {
          cs.ok[k] = 0;
        }
        continue;
      }
      if (!cs.prop_ok[k]) { r += 1; continue; }
      double ex, ey, ez, nx, ny, nz;
      tip_field_E(p, X, Y, Z, &ex, &ey, &ez);
      ex += f3[q][0]; ey += f3[q][1]; ez += f3[q][2];
      tip_normal(p, X, Y, &nx, &ny, &nz);
      const double F = (nx * ex + ny * ey) + nz * ez;
      if (F >= 0.0) { r += 1; continue; }
      const double sn = tip_target_log(p, F, nxi), sc = cs.sup[k];
      bool take = sn >= sc;
      if (!take) {
        double u1, u2;
        rng2(p.seed, (uint32_t)c, (uint32_t)it_idx, step, RNG_ACCEPT, &u1, &u2);
        take = log(u1) <= sn - sc;
      }
      if (take) {
        cs.x[k] = nxi; cs.y[k] = nph; cs.F[k] = F; cs.sup[k] = sn;
        cs.tx[k] = X; cs.ty[k] = Y; cs.tz[k] = Z;
        a += 1;
      } else {
        r += 1;
      }
    }
    if (init) continue;
    mh_counts_and_update(p, y, plan[it.d].tiles, it_idx, ndim_first, a, r, red_i);
  }
  queue_leave(queue, 0, total);
}

// ---- tip MH proposals: one thread per chain ---------------------------------------------
// Jump it >= 1: Gaussian step in (xi, phi), phi wrapped, xi reflected once
// (Metro_algo_tip_v3, src/mod_emission_tip.f90:1334-1350); the step uses the
// fixed warm-up size for the first quarter of the jumps and MH_std
// afterwards (MH_std was updated at the end of the previous iteration).
// it = 0: round 0 of the uniform start of every chain.  The proposal is also
// packed into the FP32 frame here, once, for the field tiles of the jump.
__global__ void k_mh_propose(const DiodeParams* __restrict__ P, const DiodeDyn* __restrict__ Dy,
                             const PlanEntry* __restrict__ plan, const PlanHeader* __restrict__ ph,
                             ChainState cs, const int* __restrict__ ch_off,
                             const int* __restrict__ step_ptr, int it_idx, int f32_grid) {
  const int nd = ph->n_diodes;
  const int total = nd > 0 ? plan[nd - 1].pad0 + plan[nd - 1].n_i : 0;
  const double twopi = 2.0 * c_k.pi;
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    int lo = 0, hi = nd - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (plan[mid].pad0 <= g) lo = mid; else hi = mid - 1; }
    const int d = lo, c = g - plan[d].pad0;
    const DiodeParams& p = P[d];
    if (p.geometry != RD_G_TIP || it_idx > p.mh_jumps) continue;
    const int k = ch_off[d] + c;
    const DiodeDyn& y = Dy[d];
    const uint32_t step = (uint32_t)(*step_ptr - y.step_offset);
    double nxi, nph;
    int inside = 1;
    if (it_idx == 0) {   // round 0 of the uniform start (mod_emission_tip.f90:1292-1318)
      double u1, u2;
      rng2(p.seed, (uint32_t)c, 0u, step, RNG_INIT, &u1, &u2);
      nxi = 1.0 + (p.max_xi - 1.0) * u1;
      nph = twopi * u2;
    } else {             // Gaussian step in (xi, phi), xi reflected, phi wrapped (:1337-1365)
      if (!cs.ok[k]) continue;
      const int ndim_first = (int)nint_d(p.mh_jumps * 0.25);
      double g1, g2;
      gauss2(p.seed, (uint32_t)c, (uint32_t)it_idx, step, &g1, &g2);
      const double sxi = (it_idx > ndim_first) ? (p.max_xi - 1.0) * y.MH_std : (p.max_xi - 1.0) * 0.10;
      const double sph = (it_idx > ndim_first) ? twopi * y.MH_std : twopi * 0.10;
      nxi = cs.x[k] + g1 * sxi;
      const double a = cs.y[k] + g2 * sph;
      nph = a - floor(a / twopi) * twopi;   // Fortran MODULO
      if (nxi > p.max_xi) nxi = 2.0 * p.max_xi - nxi;
      if (nxi < 1.0) nxi = 2.0 - nxi;
      inside = !(nxi < 1.0 || nxi > p.max_xi);
    }
    double X, Y, Z;
    tip_xyz(p, inside ? nxi : 1.5, p.eta_1, nph, &X, &Y, &Z);
    if (f32_grid) {   // FP32 form: the point at its FP32 nm coordinates (at most 6e-5 nm off the surface)
      X = (double)(float)(X * 1.0e9) * 1.0e-9;
      Y = (double)(float)(Y * 1.0e9) * 1.0e-9;
      Z = (double)(float)(Z * 1.0e9) * 1.0e-9;
    }
    cs.px[k] = nxi; cs.py[k] = nph; cs.prop_ok[k] = inside;
    cs.pxx[k] = X; cs.pyy[k] = Y; cs.pzz[k] = Z;
    float4 ih, il, iih, iil;   // FP32 frame of the proposal, once per jump
    point_pack(p, X, Y, Z, ih, il, iih, iil);
    cs.pph[k] = ih; cs.pih[k] = iih;
  }
}

// ---- emission decisions and stable append ----------------------------------------------------
// One CTA per emitting diode.  Candidates are tested in chain order
// (Do_Field_Emission_Planar_rectangle :345-381; Do_Field_Emission_Tip_OLDCODE
// :504-523) and the emitted electrons are appended in that order with
// Add_Particle semantics (src/mod_pair.F90:29-159): capacity check with a
// drop count, q = -q0, m = m0, the Beeman history seeded with (q/m) E_vac.
// Accept test of every chain's final state (Escape_Prob_Planar / _Tip and the
// uniform draw), spread over RD_EMIT_SPLIT blocks per diode: the FN escape
// exponent is FP64 transcendental work.  Stores the chain's escape
// probability (cs.df, the term of df_avg) and whether it emits (cs.em);
// k_emit then appends in chain order.
__global__ void __launch_bounds__(256)
k_emit_test(const DiodeParams* __restrict__ P, const DiodeDyn* __restrict__ Dy, ChainState cs,
            const int* __restrict__ ch_off, const double* __restrict__ work, const int* __restrict__ step_ptr) {
  const int d = blockIdx.x;
  const DiodeParams& p = P[d];
  if (!p.active || !p.emission || p.mh_serial) return;   // serial diodes emit in k_mh_serial
  const DiodeDyn& y = Dy[d];
  const int step = *step_ptr - y.step_offset;
  const int M = y.chains;
  for (int c = blockIdx.y * blockDim.x + threadIdx.x; c < M; c += gridDim.y * blockDim.x) {
    const int k = ch_off[d] + c;
    double u1, u2;
    rng2(p.seed, (uint32_t)c, 0u, (uint32_t)step, RNG_EMIT, &u1, &u2);
    const int ok = cs.ok[k];
    const double F = cs.F[k];
    int e = 0;
    double df;
    if (p.geometry == RD_G_TIP) {
      double Df = 0.0;
      if (ok) {
        double sq = sqrt(p.tip_phi);   // Escape_Prob_Tip :1734-1758
        Df = exp(((c_k.b_FN * ((sq * sq) * sq)) * fn_v_y(F, p.tip_phi, p.image_charge)) / fabs(F));
      }
      df = Df;
      e = F < 0.0 && u1 <= Df;
    } else {
      const double phi = work_at(p, work, cs.x[k], cs.y[k], nullptr);
      double D = ok ? fn_escape_log(F, phi, p.image_charge) : -1.79769313486231570e308;
      if (F >= 0.0) D = -1.79769313486231570e308;
      df = exp(D);
      e = log(u1) <= D;
    }
    cs.df[k] = df;
    cs.em[k] = e;
  }
}

// Append the emitted electrons of each diode in chain order (one block per
// diode: block-wide scan of k_emit_test's flags) and average the escape
// probabilities (df_avg, :354; fixed summation order).
__global__ void __launch_bounds__(1024)
k_emit(const DiodeParams* __restrict__ P, DiodeDyn* __restrict__ Dy, Pool pool, ChainState cs,
       const int* __restrict__ ch_off, const double* __restrict__ work,
       const int* __restrict__ step_ptr, EventLog ev) {
  __shared__ int warp_tot[32];
  __shared__ int s_base;
  __shared__ double warp_df[32];
  const int d = blockIdx.x;
  const DiodeParams& p = P[d];
  if (!p.active || !p.emission || p.mh_serial) return;   // serial diodes emit in k_mh_serial
  DiodeDyn& y = Dy[d];
  double df_sum = 0.0;   // sum of the candidates' escape probabilities (df_avg, :354)
  const int step = *step_ptr - y.step_offset;
  const int M = y.chains;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  if (tid == 0) s_base = 0;
  __syncthreads();
  const int n0 = y.n, id0 = y.nrID;
  int emitted = 0, dropped = 0;
  for (int c0 = 0; c0 < M; c0 += blockDim.x) {
    const int c = c0 + tid, k = ch_off[d] + c;
    int e = 0;
    if (c < M) {
      df_sum += cs.df[k];
      e = cs.em[k];
    }
    // block-wide exclusive scan of e
    unsigned bal = __ballot_sync(0xffffffffu, e);
    int wpre = __popc(bal & ((1u << lane) - 1));
    if (lane == 0) warp_tot[w] = __popc(bal);
    __syncthreads();
    int base = 0, tot = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { if (q < w) base += warp_tot[q]; tot += warp_tot[q]; }
    const int slot = s_base + base + wpre;   // emitted so far in chain order
    if (e) {
      int i = n0 + slot;
      if (i < p.cap) {
        double X, Y, Z;
        int sec = 1;
        if (p.geometry == RD_G_TIP) {   // one length scale out along the surface normal
          double nx, ny, nz;
          tip_normal(p, cs.tx[k], cs.ty[k], &nx, &ny, &nz);
          X = cs.tx[k] + nx * c_k.length_scale;
          Y = cs.ty[k] + ny * c_k.length_scale;
          Z = cs.tz[k] + nz * c_k.length_scale;
        } else {
          X = cs.x[k]; Y = cs.y[k];
          work_at(p, work, X, Y, &sec);
          Z = 1.0 * c_k.length_scale;
        }
        int gi = p.off + i;
        double qm = (-1.0 * c_k.q0) / (1.0 * c_k.m0), ex, ey, ez;
        vacuum_field(p, X, Y, Z, &ex, &ey, &ez);
        pool.x[gi] = X; pool.y[gi] = Y; pool.z[gi] = Z;
        pool.vx[gi] = 0.0; pool.vy[gi] = 0.0; pool.vz[gi] = 0.0;
        pool.ax[gi] = pool.bx[gi] = pool.cx[gi] = qm * ex;
        pool.ay[gi] = pool.by[gi] = pool.cy[gi] = qm * ey;
        pool.az[gi] = pool.bz[gi] = pool.cz[gi] = qm * ez;
        pool.q[gi] = -1.0 * c_k.q0;
        pool.m[gi] = 1.0 * c_k.m0;
        pool.species[gi] = 1;
        pool.id[gi] = id0 + slot;
        pool.step0[gi] = step;
        pool.section[gi] = sec;
        pool.mask[gi] = 1;
        log_event(ev, X, Y, Z, 0.0, 0.0, 0.0, d, RD_EVENT_EMIT, sec, id0 + slot, 1, step);   // density_emit*.bin
      }
    }
    __syncthreads();
    if (tid == 0) s_base += tot;
    __syncthreads();
  }
  for (int o = 16; o > 0; o >>= 1) df_sum += __shfl_xor_sync(0xffffffffu, df_sum, o);
  if (lane == 0) warp_df[w] = df_sum;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += warp_df[q];
    y.df_avg = y.N_sup > 0.0 ? s / y.N_sup : 0.0;
    int tot = s_base;
    int room = p.cap - n0;
    emitted = tot < room ? tot : (room > 0 ? room : 0);
    dropped = tot - emitted;
    y.n = n0 + emitted;
    y.nrID = id0 + emitted;
    y.emitted_step = emitted;
    y.dropped_step = dropped;
    y.emitted_total += emitted;
    y.dropped_total += dropped;
  }
}

}  // namespace

// ---- serial MH sampler (mh_batch = .false.) ---------------------------------------------
// The pair sum of F_z at one cathode point over the diode's first n
// particles, summed by the whole block (every thread gets the total, before
// z0_finish).
template <int PREC>
__device__ double block_field_sum(const DiodeParams& p, const Pool& pool, int n, double px, double py,
                                  double* red) {
  const int tid = threadIdx.x, nt = blockDim.x, off = p.off;
  const int nic = p.image_charge ? p.N_ic_max : 0;
  double s;
  if (PREC == 1) {
    const float4 pp = z0_point(p, px, py);
    const float dnm = (float)(p.d * 1.0e9);
    float hi = 0.f, lo = 0.f;
    for (int j = tid; j < n; j += nt) {
      float4 h = pool.zk_hi[off + j], l = pool.zk_lo[off + j];
      two_sum_acc(hi, lo, nic == 0 ? z0_tile_f32<true>(&h, &l, 1, pp, 0, dnm)
                                   : z0_tile_f32<false>(&h, &l, 1, pp, nic, dnm));
    }
    s = (double)hi + (double)lo;
  } else {
    s = 0.0;
    for (int j = tid; j < n; j += nt) {
      rd_d4 pj = make_d4(pool.x[off + j], pool.y[off + j], pool.z[off + j], pool.q[off + j]);
      s += z0_tile_f64(&pj, 1, px, py, nic, p.d, c_k.L2);
    }
  }
  return block_sum(s, red);
}

// The serial branch of Do_Field_Emission_Planar_rectangle (:322-333, 338-383)
// with Metropolis_Hastings_rectangle_J (:1122-1265), and the ring emitter
// (Do_Field_Emission_Planar_ring :399-505 with Metropolis_Hastings_ring_J
// :1521-1685, chains in (angle, radius)): one block per serial
// diode runs its candidates' chains one after another.  Each chain starts
// from uniform draws until F_z < 0, makes mh_jumps jumps (the warm-up quarter
// with 10 % of the emitter as the step, then MH_std), updates MH_std once from
// its own acceptance rate after the warm-up, and its electron, if the escape
// test passes, is added before the next chain starts, so later chains see it.
// Same Philox counters as the batched sampler.  The whole block sums the field
// at each point (block_field_sum); thread 0 alone holds the chain and does the
// rest (draws, proposals, targets, decisions: FP64 work, which every warp
// would otherwise repeat on the part's narrow FP64 pipe) and hands the block
// the next point through shared memory.
template <int PREC>
__global__ void __launch_bounds__(256)
k_mh_serial(const DiodeParams* __restrict__ P, DiodeDyn* __restrict__ Dy, Pool pool,
            const double* __restrict__ work, const double* __restrict__ wtab,
            const int* __restrict__ step_ptr, double kscale, EventLog ev) {
  __shared__ double red[256];
  // thread 0 -> block, one slot per jump parity (a slot is rewritten only after a
  // barrier that every reader of its last value has passed)
  __shared__ double s_pt[2][2];   // the point whose field the block sums next
  __shared__ int s_sum[2];        // the block sums a field this jump (a ring proposal off the ring: no)
  __shared__ int s_found, s_add, s_stop;   // the chain started; a particle was added; the chains stop
  const int d = blockIdx.x;
  const DiodeParams& p = P[d];
  if (!p.active || !p.emission || !p.mh_serial || p.geometry != RD_G_PLANAR) return;
  DiodeDyn& y = Dy[d];
  if (y.ser_done) {   // k_mh_serial_vacuum sampled this step's chains
    __syncthreads();
    if (threadIdx.x == 0) y.ser_done = 0;
    return;
  }
  const bool t0 = threadIdx.x == 0;
  const uint32_t step = (uint32_t)(*step_ptr - y.step_offset);
  const int M = y.chains, n0 = y.n, id0 = y.nrID;
  const int ndim = p.mh_jumps, ndim_first = (ndim + 2) / 4;
  int n = n0;   // particles the field sums see (every thread)
  // thread 0's state
  int emitted = 0, dropped = 0, failed = 0;
  double mhs = y.MH_std, a_rate = y.a_rate, df_sum = 0.0;
  const bool ring = p.emitter_type == 4;
  const double twopi = 2.0 * c_k.pi, rmin = p.ring_rmin, rmax = p.ring_rmin + p.ring_thick;
  for (int c = 0; c < M; ++c) {
    double cx = p.em_x0, cy = p.em_y0, F = 1.0;
    double ca = 0.0, cr = rmin;   // ring: (angle, radius) of the chain (Metropolis_Hastings_ring_J)
    bool found = false;
    if (t0) s_found = 0;
    for (int r = 0; r < p.init_rounds; ++r) {
      if (t0) {
        double u1, u2;
        rng2(p.seed, (uint32_t)c, (uint32_t)r, step, RNG_INIT, &u1, &u2);
        if (ring) {
          ca = u1 * twopi;
          cr = rmin + u2 * p.ring_thick;
          cx = cr * cos(ca);
          cy = cr * sin(ca);
        } else {
          cx = u1 * p.em_Lx + p.em_x0;
          cy = u2 * p.em_Ly + p.em_y0;
        }
        s_pt[0][0] = cx; s_pt[0][1] = cy;
      }
      __syncthreads();
      const double sum = block_field_sum<PREC>(p, pool, n, s_pt[0][0], s_pt[0][1], red);
      if (t0) {
        F = z0_finish<PREC>(p, sum, kscale);
        found = F < 0.0;
        s_found = found;
      }
      __syncthreads();
      if (s_found) break;
    }
    __syncthreads();   // s_found final (also with no start rounds)
    double D = -1.79769313486231570e308, Fout = 1.0;
    double sup_cur = 0.0, sx = 0.0, sy = 0.0;
    int ja = 0, jr = 0;
    if (t0) {
      if (!found) {
        cx = ring ? rmin : p.em_x0;
        cy = ring ? 0.0 : p.em_y0;
        ++failed;
      } else {
        Fout = F;
        // ring: log(radius) is the Jacobian of the (angle, radius) parametrisation (:1592-1596)
        sup_cur = supply_log_xy(p, wtab, cx, cy, F) + (ring ? log(cr) : 0.0);
        sx = (ring ? twopi : p.em_Lx) * 0.10;
        sy = (ring ? p.ring_thick : p.em_Ly) * 0.10;
      }
    }
    const bool walk = s_found != 0;   // every thread: the chain found a start
    for (int i = 1; walk && i <= ndim; ++i) {
      double wx = 0.0, wy = 0.0, na = 0.0, nr = 0.0;
      if (t0) {
        if (i > ndim_first) { sx = (ring ? twopi : p.em_Lx) * mhs; sy = (ring ? p.ring_thick : p.em_Ly) * mhs; }
        double g1, g2;
        gauss2(p.seed, (uint32_t)c, (uint32_t)i, step, &g1, &g2);
        int sum_it = 1;
        if (ring) {   // angle wrapped (Fortran MODULO), radius outside the ring rejected
          const double a = g1 * sx + ca;
          na = a - floor(a / twopi) * twopi;
          nr = g2 * sy + cr;
          if (nr < rmin || nr > rmax) {
            if (i > ndim_first) ++jr;
            sum_it = 0;
          } else {
            wx = nr * cos(na);
            wy = nr * sin(na);
          }
        } else {
          wx = g1 * sx + cx;
          wy = g2 * sy + cy;
          const double hx = p.em_x0 + p.em_Lx, hy = p.em_y0 + p.em_Ly;
          if (wx > hx) wx = hx - (wx - hx); else if (wx < p.em_x0) wx = (p.em_x0 - wx) + p.em_x0;
          if (wy > hy) wy = hy - (wy - hy); else if (wy < p.em_y0) wy = (p.em_y0 - wy) + p.em_y0;
        }
        s_pt[i & 1][0] = wx; s_pt[i & 1][1] = wy;
        s_sum[i & 1] = sum_it;
      }
      __syncthreads();
      if (!s_sum[i & 1]) continue;   // block-uniform: a ring proposal off the ring, no field needed
      const double sum = block_field_sum<PREC>(p, pool, n, s_pt[i & 1][0], s_pt[i & 1][1], red);
      if (t0) {
        const double Fw = z0_finish<PREC>(p, sum, kscale);
        if (Fw >= 0.0) {
          if (i > ndim_first) ++jr;
        } else {
          const double sn = supply_log_xy(p, wtab, wx, wy, Fw) + (ring ? log(nr) : 0.0);
          bool take = sn >= sup_cur;
          if (!take) {
            double u1, u2;
            rng2(p.seed, (uint32_t)c, (uint32_t)i, step, RNG_ACCEPT, &u1, &u2);
            take = log(u1) <= sn - sup_cur;
          }
          if (take) {
            cx = wx; cy = wy; sup_cur = sn; Fout = Fw; ca = na; cr = nr;
            if (i > ndim_first) ++ja;
          } else if (i > ndim_first) {
            ++jr;
          }
        }
      }
    }
    // the chain's end: MH_std, the escape test and its electron (thread 0)
    if (t0) {
      s_add = 0;
      s_stop = 0;
      if (found) {
        if (ja + jr > 0) {   // MH_std_update once per chain (:1251-1254, :603-612)
          a_rate = (double)ja / (double)(jr + ja);
          mhs = mhs * exp(0.025 * (a_rate - 0.35));
          if (mhs > p.mh_hi) mhs = p.mh_hi; else if (mhs < p.mh_lo) mhs = p.mh_lo;
        }
        D = fn_escape_log(Fout, work_at(p, work, cx, cy, nullptr), p.image_charge);
      }
      bool stop = false;
      if (Fout >= 0.0) {
        D = -1.79769313486231570e308;
        stop = ring;   // the ring emitter's loop stops at an unfavourable chain (:447-455)
      }
      if (stop) {
        s_stop = 1;
      } else {
        df_sum += exp(D);
        double u1, u2;
        rng2(p.seed, (uint32_t)c, 0u, step, RNG_EMIT, &u1, &u2);
        if (log(u1) <= D) {
          if (n < p.cap) {   // Add_Particle (src/mod_pair.F90:29-159), visible to the next chains
            const int gi = p.off + n;
            const double X = cx, Y = cy, Z = 1.0 * c_k.length_scale;
            int sec = 1;
            work_at(p, work, X, Y, &sec);
            double ex, ey, ez;
            vacuum_field(p, X, Y, Z, &ex, &ey, &ez);
            const double qm = (-1.0 * c_k.q0) / (1.0 * c_k.m0);
            pool.x[gi] = X; pool.y[gi] = Y; pool.z[gi] = Z;
            pool.vx[gi] = 0.0; pool.vy[gi] = 0.0; pool.vz[gi] = 0.0;
            pool.ax[gi] = pool.bx[gi] = pool.cx[gi] = qm * ex;
            pool.ay[gi] = pool.by[gi] = pool.cy[gi] = qm * ey;
            pool.az[gi] = pool.bz[gi] = pool.cz[gi] = qm * ez;
            pool.q[gi] = -1.0 * c_k.q0;
            pool.m[gi] = 1.0 * c_k.m0;
            pool.species[gi] = 1;
            pool.id[gi] = id0 + emitted;
            pool.step0[gi] = (int)step;
            pool.section[gi] = sec;
            pool.mask[gi] = 1;
            float4 h, l;   // its cathode pack, for the FP32 field sums of the next chains
            split_nm(X, p.org_x, &h.x, &l.x);
            split_nm(Y, p.org_y, &h.y, &l.y);
            const float zf = (float)(Z * 1.0e9), qf = -1.0f;
            pool.zk_hi[gi] = make_float4(h.x, h.y, fmaxf(zf * zf, 1e-20f), qf * zf);
            pool.zk_lo[gi] = make_float4(l.x, l.y, zf, qf);
            log_event(ev, X, Y, Z, 0.0, 0.0, 0.0, d, RD_EVENT_EMIT, sec, id0 + emitted, 1, (int)step);
            ++emitted;
            s_add = 1;
            __threadfence_block();
          } else {
            ++dropped;
          }
        }
      }
    }
    __syncthreads();
    if (s_stop) break;
    if (s_add) ++n;
  }
  if (t0) {
    y.n = n;
    y.nrID = id0 + emitted;
    y.emitted_step = emitted;
    y.dropped_step = dropped;
    y.emitted_total += emitted;
    y.dropped_total += dropped;
    y.chains_failed = failed;
    y.MH_std = mhs;
    y.a_rate = a_rate;
    y.df_avg = y.N_sup > 0.0 ? df_sum / y.N_sup : 0.0;
  }
}

// ---- launch wrappers --------------------------------------------------------------------------
cudaError_t rd_launch_field_points(int prec, int geom, int grid, cudaStream_t st,
                                   const DiodeParams* P, const Pool& pool, const PlanEntry* plan,
                                   const PlanHeader* ph, const PointSet& pts, double* partial,
                                   int* tickets, double kscale) {
  if (prec == 1) {
    if (geom == RD_G_TIP) k_field_points<1, RD_G_TIP><<<rd_grid(k_field_points<1, RD_G_TIP>, RD_ITILE, grid), RD_ITILE, 0, st>>>(P, pool, plan, ph, pts, partial, tickets, kscale);
    else k_field_points<1, RD_G_PLANAR><<<rd_grid(k_field_points<1, RD_G_PLANAR>, RD_ITILE, grid), RD_ITILE, 0, st>>>(P, pool, plan, ph, pts, partial, tickets, kscale);
  } else {
    if (geom == RD_G_TIP) k_field_points<0, RD_G_TIP><<<rd_grid(k_field_points<0, RD_G_TIP>, RD_ITILE, grid), RD_ITILE, 0, st>>>(P, pool, plan, ph, pts, partial, tickets, kscale);
    else k_field_points<0, RD_G_PLANAR><<<rd_grid(k_field_points<0, RD_G_PLANAR>, RD_ITILE, grid), RD_ITILE, 0, st>>>(P, pool, plan, ph, pts, partial, tickets, kscale);
  }
  return cudaGetLastError();
}

// Loads the field-at-points kernels of one precision into the current context
// now (under lazy module loading they would load at their first launch).
cudaError_t rd_preload_field_points(int prec) {
  cudaFuncAttributes a;
  cudaError_t e;
  if (prec == 1) {
    if ((e = cudaFuncGetAttributes(&a, k_field_points<1, RD_G_TIP>)) != cudaSuccess) return e;
    if ((e = cudaFuncGetAttributes(&a, k_field_points<1, RD_G_PLANAR>)) != cudaSuccess) return e;
    rd_grid(k_field_points<1, RD_G_TIP>, RD_ITILE, 0);
    rd_grid(k_field_points<1, RD_G_PLANAR>, RD_ITILE, 0);
  } else {
    if ((e = cudaFuncGetAttributes(&a, k_field_points<0, RD_G_TIP>)) != cudaSuccess) return e;
    if ((e = cudaFuncGetAttributes(&a, k_field_points<0, RD_G_PLANAR>)) != cudaSuccess) return e;
    rd_grid(k_field_points<0, RD_G_TIP>, RD_ITILE, 0);
    rd_grid(k_field_points<0, RD_G_PLANAR>, RD_ITILE, 0);
  }
  return cudaSuccess;
}

cudaError_t rd_launch_z0_points(int prec, int grid, cudaStream_t st, const DiodeParams* P,
                                const Pool& pool, const PlanEntry* plan, const PlanHeader* ph,
                                const double* qx, const double* qy, const float4* qpp, double* qF,
                                double* partial, int* tickets, double kscale, int* queue) {
  if (prec == 1) k_z0_points<1><<<rd_grid(k_z0_points<1>, 32, grid), 32, 0, st>>>(P, pool, plan, ph, qx, qy, qpp, qF, partial, tickets, kscale, queue);
  else k_z0_points<0><<<rd_grid(k_z0_points<0>, RD_ITILE, grid), RD_ITILE, 0, st>>>(P, pool, plan, ph, qx, qy, qpp, qF, partial, tickets, kscale, queue);
  return cudaGetLastError();
}

cudaError_t rd_launch_supply_reduce(int nslots, cudaStream_t st, const DiodeParams* P, DiodeDyn* Dy,
                                    const double* qx, const double* qy, const double* qw,
                                    const double* qF, const double* qfx, const double* qfy,
                                    const double* work, const int* step_ptr, double* sup_part) {
  k_supply_reduce<<<dim3(nslots, RD_SUP_SPLIT), 256, 0, st>>>(P, Dy, qx, qy, qw, qF, qfx, qfy, work, step_ptr,
                                                              sup_part);
  k_supply_finish<<<(nslots + 127) / 128, 128, 0, st>>>(P, Dy, nslots, step_ptr, sup_part);
  return cudaGetLastError();
}

// Switches the step graph's conditional MH node on when the MH plan has work items.
__global__ void k_mh_cond(cudaGraphConditionalHandle h, const PlanHeader* __restrict__ ph) {
  cudaGraphSetConditional(h, ph->total_items > 0 ? 1u : 0u);
}

cudaError_t rd_launch_mh_cond(cudaStream_t st, cudaGraphConditionalHandle h, const PlanHeader* ph) {
  k_mh_cond<<<1, 1, 0, st>>>(h, ph);
  return cudaGetLastError();
}

cudaError_t rd_launch_mh_vacuum(int prec, int nslots, cudaStream_t st, const DiodeParams* P, DiodeDyn* Dy,
                                const ChainState& cs, const int* ch_off, const double* wtab, const int* step_ptr,
                                double kscale) {
  const int grid = nslots * RD_VAC_CTAS;
  const dim3 ugrid(RD_VAC_MAX_CHAINS / RD_VU_CHAINS, nslots);
  if (prec == 1) {
    k_mh_vacuum_uniform<1><<<ugrid, RD_VU_THREADS, 0, st>>>(P, Dy, cs, ch_off, wtab, step_ptr, kscale);
    k_mh_vacuum<1><<<grid, RD_VAC_THREADS, 0, st>>>(P, Dy, cs, ch_off, wtab, step_ptr, kscale, nslots);
  } else {
    k_mh_vacuum_uniform<0><<<ugrid, RD_VU_THREADS, 0, st>>>(P, Dy, cs, ch_off, wtab, step_ptr, kscale);
    k_mh_vacuum<0><<<grid, RD_VAC_THREADS, 0, st>>>(P, Dy, cs, ch_off, wtab, step_ptr, kscale, nslots);
  }
  return cudaGetLastError();
}

cudaError_t rd_launch_mh_init(int prec, int grid, cudaStream_t st, const DiodeParams* P,
                              DiodeDyn* Dy, const Pool& pool, const PlanEntry* plan,
                              const PlanHeader* ph, const ChainState& cs, const int* ch_off,
                              const double* wtab, const int* step_ptr, double kscale) {
  if (prec == 1) k_mh_init<1><<<rd_grid(k_mh_init<1>, 256, grid), 256, 0, st>>>(P, Dy, pool, plan, ph, cs, ch_off, wtab, step_ptr, kscale);
  else k_mh_init<0><<<rd_grid(k_mh_init<0>, 256, grid), 256, 0, st>>>(P, Dy, pool, plan, ph, cs, ch_off, wtab, step_ptr, kscale);
  return cudaGetLastError();
}

cudaError_t rd_launch_mh_jump(int prec, int geometry_mask, int grid, cudaStream_t st,
                              const DiodeParams* P, DiodeDyn* Dy, const Pool& pool,
                              const PlanEntry* plan, const PlanHeader* ph, const ChainState& cs,
                              const int* ch_off, const double* wtab, const int* step_ptr,
                              int it_idx, double* partial, int* tickets, double kscale, int* queue,
                              int part, int nparts, int form) {
  // part (planar jumps): 0 all items, 1..nparts one of nparts parts of the plan (part_range);
  // form (FP32): 0 32 threads x 4 chains, 1 64 threads x 2 chains (bit-identical results)
  if (geometry_mask & 1) {
    if (prec == 1 && form == 1) k_mh_jump_planar<1, 1><<<rd_grid(k_mh_jump_planar<1, 1>, 64, grid), 64, 0, st>>>(P, Dy, pool, plan, ph, cs, ch_off, wtab, step_ptr, it_idx, partial, tickets, kscale, queue, part, nparts);
    else if (prec == 1) k_mh_jump_planar<1, 0><<<rd_grid(k_mh_jump_planar<1, 0>, 32, grid), 32, 0, st>>>(P, Dy, pool, plan, ph, cs, ch_off, wtab, step_ptr, it_idx, partial, tickets, kscale, queue, part, nparts);
    else k_mh_jump_planar<0, 0><<<rd_grid(k_mh_jump_planar<0, 0>, RD_ITILE, grid), RD_ITILE, 0, st>>>(P, Dy, pool, plan, ph, cs, ch_off, wtab, step_ptr, it_idx, partial, tickets, kscale, queue, part, nparts);
  }
  if (geometry_mask & 2) {
    k_mh_propose<<<rd_grid(k_mh_propose, 256, grid), 256, 0, st>>>(P, Dy, plan, ph, cs, ch_off, step_ptr, it_idx,
                                                                   prec == 1);
    if (prec == 1) k_mh_jump_tip<1><<<rd_grid(k_mh_jump_tip<1>, RD_ITILE / RD_TIP_CPT, grid), RD_ITILE / RD_TIP_CPT, 0, st>>>(P, Dy, pool, plan, ph, cs, ch_off, step_ptr, it_idx, partial, tickets, kscale, queue + 2);
    else k_mh_jump_tip<0><<<rd_grid(k_mh_jump_tip<0>, RD_ITILE, grid), RD_ITILE, 0, st>>>(P, Dy, pool, plan, ph, cs, ch_off, step_ptr, it_idx, partial, tickets, kscale, queue + 2);
  }
  return cudaGetLastError();
}

cudaError_t rd_launch_emit(int nslots, cudaStream_t st, const DiodeParams* P, DiodeDyn* Dy,
                           const Pool& pool, const ChainState& cs, const int* ch_off,
                           const double* work, const int* step_ptr, const EventLog& ev) {
  k_emit_test<<<dim3(nslots, RD_EMIT_SPLIT), 256, 0, st>>>(P, Dy, cs, ch_off, work, step_ptr);
  k_emit<<<nslots, 1024, 0, st>>>(P, Dy, pool, cs, ch_off, work, step_ptr, ev);
  return cudaGetLastError();
}

namespace {
// The serial sampler (k_mh_serial) on a planar rectangle-emitter diode with no
// particle in flight and a uniform work function, run speculatively in parallel.
// Chains depend on each other only through the electrons earlier chains emit
// in the step and through MH_std, which each chain updates once from its own
// acceptance rate.  With no particle in flight the field at every point is the
// vacuum field, and with a uniform work function every target is the same, so
// until a chain emits every proposal is taken: each chain's acceptance rate is
// 1, MH_std after chain c is known without running it (clamped to a fixed
// point after a few chains), the start of every chain is its round-0 draw, and
// its walk needs only its Gaussian pairs.  Blocks (x: group of RD_VU_CHAINS
// chains, y: diode slot) draw the pairs of all (chain, jump) into shared memory
// and walk each chain in one lane, as k_mh_vacuum_uniform does, with the
// chain's own step size; then each chain takes its emission draw.  If no chain
// of the diode emits (escape probabilities of ~1e-13 at 4.7 eV), the last
// block to finish writes the step's results, bit for bit those k_mh_serial
// would write (the escape-probability sum, e added M times in order, by
// rd_repeat_sum), and sets ser_done, so k_mh_serial leaves the diode.  If any
// chain emits, nothing is written and k_mh_serial samples the diode from its
// first chain as usual.
template <int PREC>
__global__ void __launch_bounds__(RD_VU_THREADS)
k_mh_serial_vacuum(const DiodeParams* __restrict__ P, DiodeDyn* __restrict__ Dy, const double* __restrict__ work,
                   const double* __restrict__ wtab, const int* __restrict__ step_ptr, double kscale) {
  __shared__ DiodeParams sp;
  __shared__ double s_mhs[RD_VU_CHAINS];           // MH_std each chain of the block walks with
  __shared__ double s_end;                          // MH_std after the diode's last chain
  __shared__ double s_g[RD_VU_JCHUNK][RD_VU_CHAINS][2];
  const int d = blockIdx.y, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const DiodeParams& pg = P[d];
  if (!pg.active || !pg.emission || !pg.mh_serial || pg.geometry != RD_G_PLANAR || pg.emitter_type == 4) return;
  DiodeDyn& y = Dy[d];
  if (y.n != 0 || y.chains <= 0 || y.chains > RD_VAC_MAX_CHAINS) return;   // the grid covers this many
  const int M = y.chains, c0 = blockIdx.x * RD_VU_CHAINS;
  if (c0 >= M) return;
  {
    const int* src = reinterpret_cast<const int*>(P + d);
    int* dst = reinterpret_cast<int*>(&sp);
    for (int k = tid; k < (int)(sizeof(DiodeParams) / sizeof(int)); k += blockDim.x) dst[k] = src[k];
  }
  __syncthreads();
  const DiodeParams& p = sp;
  const int cells = p.work_model == 1 ? p.work_nx * p.work_ny : (p.work_model == 4 ? p.work_nx : 0);
  int differs = 0;
  for (int k = tid; k < cells; k += blockDim.x)
    for (int e = 0; e < 3; ++e)
      differs |= __double_as_longlong(wtab[3 * (p.work_off + k) + e]) !=
                 __double_as_longlong(wtab[3 * p.work_off + e]);
  if (!(__syncthreads_or(differs) == 0 && cells >= 1)) return;
  const int J = p.mh_jumps, ndim_first = (J + 2) / 4;
  const uint32_t step = (uint32_t)(*step_ptr - y.step_offset);
  const double F = z0_finish<PREC>(p, 0.0, kscale);   // k_mh_serial's field with no particle: z0_finish of a zero sum
  const bool found = F < 0.0 && p.init_rounds > 0;     // every chain starts at its round-0 draw, or none does
  const bool updates = found && J > ndim_first;        // each chain updates MH_std once, at rate 1
  const int nc = min(RD_VU_CHAINS, M - c0);
  if (tid == 0) {   // MH_std of chains c0 .. c0 + nc - 1, and after chain M - 1
    const double ar = (double)(J - ndim_first) / (double)(J - ndim_first);   // 1, formed as k_mh_serial forms it
    const double g = exp(0.025 * (ar - 0.35));          // k_mh_serial's factor at that rate
    double m = y.MH_std;
    bool fixed = !updates;
    for (int c = 0; c < M; ++c) {
      if (c >= c0 && c < c0 + nc) s_mhs[c - c0] = m;
      if (fixed) {   // every later chain walks with m
        for (int k = max(c + 1, c0); k < c0 + nc; ++k) s_mhs[k - c0] = m;
        break;
      }
      double nx = m * g;
      if (nx > p.mh_hi) nx = p.mh_hi; else if (nx < p.mh_lo) nx = p.mh_lo;
      fixed = nx == m;
      m = nx;
    }
    s_end = m;
  }
  const int c = c0 + lane;
  const bool mine = w == 1 && lane < nc;
  double cx = p.em_x0, cy = p.em_y0;
  if (mine && found) {
    double u1, u2;
    rng2(p.seed, (uint32_t)c, 0u, step, RNG_INIT, &u1, &u2);
    cx = u1 * p.em_Lx + p.em_x0;
    cy = u2 * p.em_Ly + p.em_y0;
  }
  if (found) {
    for (int j0 = 1; j0 <= J; j0 += RD_VU_JCHUNK) {
      const int nj = min(RD_VU_JCHUNK, J - j0 + 1);
      __syncthreads();   // the previous chunk's walk is done with s_g, s_mhs is in place
      for (int k = tid - (j0 == 1 ? 32 : 0); k < nj * nc; k += blockDim.x - (j0 == 1 ? 32 : 0)) {
        if (k < 0) break;   // thread 0's warp forms the MH_std sequence during the first chunk
        const int jj = k / nc, q = k - jj * nc;
        double a, b;
        gauss2(p.seed, (uint32_t)(c0 + q), (uint32_t)(j0 + jj), step, &a, &b);
        s_g[jj][q][0] = a; s_g[jj][q][1] = b;
      }
      __syncthreads();
      if (mine) {
        const double mhs = s_mhs[lane];
        const double hx = p.em_x0 + p.em_Lx, hy = p.em_y0 + p.em_Ly;
        for (int jj = 0; jj < nj; ++jj) {   // k_mh_serial's rectangle step; every proposal taken
          const int i = j0 + jj;
          double sx = p.em_Lx * 0.10, sy = p.em_Ly * 0.10;
          if (i > ndim_first) { sx = p.em_Lx * mhs; sy = p.em_Ly * mhs; }
          double wx = s_g[jj][lane][0] * sx + cx;
          double wy = s_g[jj][lane][1] * sy + cy;
          if (wx > hx) wx = hx - (wx - hx); else if (wx < p.em_x0) wx = (p.em_x0 - wx) + p.em_x0;
          if (wy > hy) wy = hy - (wy - hy); else if (wy < p.em_y0) wy = (p.em_y0 - wy) + p.em_y0;
          cx = wx; cy = wy;
        }
      }
    }
  }
  __syncthreads();
  // each chain's emission draw against its escape probability
  int emits = 0;
  double D = -1.79769313486231570e308;
  if (found) D = fn_escape_log(F, work_at(p, work, p.em_x0, p.em_y0, nullptr), p.image_charge);
  if (mine) {
    double Dc = found ? fn_escape_log(F, work_at(p, work, cx, cy, nullptr), p.image_charge) : D;
    double u1, u2;
    rng2(p.seed, (uint32_t)c, 0u, step, RNG_EMIT, &u1, &u2);
    emits = log(u1) <= Dc;
  }
  emits = __syncthreads_or(emits);
  if (tid == 0) {
    if (emits) atomicOr(&y.ser_emit, 1);
    __threadfence();
    const int nblk = (M + RD_VU_CHAINS - 1) / RD_VU_CHAINS;
    if (atomicAdd(&y.ser_ticket, 1) == nblk - 1) {   // every block of the diode is done
      __threadfence();
      if (atomicAdd(&y.ser_emit, 0) == 0) {   // no chain emitted: the step's results, as k_mh_serial
        y.emitted_step = 0;
        y.dropped_step = 0;
        y.chains_failed = found ? 0 : M;
        y.MH_std = s_end;
        if (updates) y.a_rate = 1.0;
        const double df_sum = found ? rd_repeat_sum(exp(D), M) : 0.0;   // exp(D) added M times, as k_mh_serial adds it
        y.df_avg = y.N_sup > 0.0 ? df_sum / y.N_sup : 0.0;
        y.ser_done = 1;
      }
      y.ser_ticket = 0;
      y.ser_emit = 0;
    }
  }
}
}  // namespace

cudaError_t rd_launch_mh_serial(int prec, int nslots, cudaStream_t st, const DiodeParams* P, DiodeDyn* Dy,
                                const Pool& pool, const double* work, const double* wtab,
                                const int* step_ptr, double kscale, const EventLog& ev) {
  const dim3 vgrid(RD_VAC_MAX_CHAINS / RD_VU_CHAINS, nslots);
  if (prec == 1) {
    k_mh_serial_vacuum<1><<<vgrid, RD_VU_THREADS, 0, st>>>(P, Dy, work, wtab, step_ptr, kscale);
    k_mh_serial<1><<<nslots, 256, 0, st>>>(P, Dy, pool, work, wtab, step_ptr, kscale, ev);
  } else {
    k_mh_serial_vacuum<0><<<vgrid, RD_VU_THREADS, 0, st>>>(P, Dy, work, wtab, step_ptr, kscale);
    k_mh_serial<0><<<nslots, 256, 0, st>>>(P, Dy, pool, work, wtab, step_ptr, kscale, ev);
  }
  return cudaGetLastError();
}

RD_DEFINE_CONSTANT_UPLOAD(field)
