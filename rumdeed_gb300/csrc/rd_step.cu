// rd_step.cu -- per-particle kernels of the time step and the work planner.
//
//  * k_plan: builds the pair-sum plan (rd_pair.cuh) on the device from the
//    particle / point / chain counts, so a captured step graph adapts to the
//    counts of every step without host involvement.
//  * k_pack: FP32 (hi, lo) position packs, anode distances and, for tips,
//    the apex-sphere image point of every particle.
//  * k_position: Beeman position update, history shift, boundary checks and
//    removal marking (Update_ElecIon_Position, src/mod_verlet.F90:197-232;
//    Check_Boundary_Planar :325-338; Check_Boundary_Tip,
//    src/mod_emission_tip.f90:1627-1647; Mark_Particles_Remove,
//    src/mod_pair.F90:169-339), fused with the pack.
//  * k_velocity + k_ramo: Beeman velocity update and the Ramo current
//    (Update_ElecIon_Velocity, src/mod_verlet.F90:449-509), reduced per diode
//    in a fixed order.
//  * k_compact_*: stable, order-preserving compaction from the first dead
//    index (Remove_Particles :352-562, compact_array :1180-1223) with the
//    life-time histogram (record_lifetime :1135-1160).
#include "rd_pair.cuh"

namespace {

// Marks particle gi removed (mask off, charge zeroed, absorption record) and
// returns its contribution to the diode's removal counters: bit 0 removed,
// bit 1 an electron, bit 2 at the anode.  The caller adds the counters up
// (warp-aggregated in k_position, where a whole crossing front is removed at
// once; directly by mark_remove).
__device__ __forceinline__ int mark_remove_flags(const DiodeParams& p, Pool& pool, int gi, int why,
                                                 const EventLog& ev, int d, int step) {
  if (!pool.mask[gi]) return 0;
  pool.mask[gi] = 0;
  pool.q[gi] = 0.0;   // a marked particle no longer acts on others (:206-207)
  if (pool.species[gi] != 1) return 1;
  // density_absorb_{top,bot}.bin record (:241-257)
  log_event(ev, pool.x[gi], pool.y[gi], pool.z[gi], pool.vx[gi], pool.vy[gi], pool.vz[gi], d,
            why == 1 ? RD_EVENT_ABSORB_TOP : RD_EVENT_ABSORB_BOT, pool.section[gi], pool.id[gi], 1, step);
  return why == 1 ? 7 : 3;
}

// Removal counters of one warp's marks (flags as mark_remove_flags returns;
// every lane of the warp calls it, all for the same diode).
__device__ __forceinline__ void count_removals_warp(DiodeDyn& y, int flags, int i) {
  const unsigned rem = __ballot_sync(0xffffffffu, flags & 1);
  if (!rem) return;
  const unsigned top = __ballot_sync(0xffffffffu, flags == 7);
  const unsigned bot = __ballot_sync(0xffffffffu, flags == 3);
  const int imin = __reduce_min_sync(0xffffffffu, (flags & 1) ? i : 0x7fffffff);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&y.n_remove, __popc(rem));
    atomicMin(&y.first_dead, imin);
    if (top) atomicAdd(&y.n_remove_top, __popc(top));
    if (bot) atomicAdd(&y.n_remove_bot, __popc(bot));
  }
}

__device__ __forceinline__ void mark_remove(const DiodeParams& p, DiodeDyn& y, Pool& pool, int i,
                                            int gi, int why, const EventLog& ev, int d, int step) {
  const int f = mark_remove_flags(p, pool, gi, why, ev, d, step);
  if (!f) return;
  atomicAdd(&y.n_remove, 1);
  atomicMin(&y.first_dead, i);
  if (f == 7) atomicAdd(&y.n_remove_top, 1);
  else if (f == 3) atomicAdd(&y.n_remove_bot, 1);
}

// FP32 packs of particle gi from its position and charge (the caller's values
// of pool.x/y/z/q at gi).
__device__ __forceinline__ void pack_vals(const DiodeParams& p, const Pool& pool, int gi, double x, double y,
                                          double z, double q) {
  float4 h, l;
  split_nm(x, p.org_x, &h.x, &l.x);
  split_nm(y, p.org_y, &h.y, &l.y);
  split_nm(z, 0.0, &h.z, &l.z);
  h.w = (float)(q * c_k.q0_inv);   // exact for charges that are multiples of q0
  l.w = (float)((p.d - z) * 1.0e9);
  pool.pk_hi[gi] = h;
  pool.pk_lo[gi] = l;
  if (p.geometry == RD_G_PLANAR) {
    const float zf = h.z, qf = h.w;   // h.z is (float)(z 1e9): the split's origin is 0
    pool.zk_hi[gi] = make_float4(h.x, h.y, fmaxf(zf * zf, 1e-20f), qf * zf);
    pool.zk_lo[gi] = make_float4(l.x, l.y, zf, qf);
  }
  if (p.geometry == RD_G_TIP) {
    double xi, yi, zi;
    double dis = tip_image_point(p, x, y, z, &xi, &yi, &zi);
    float4 a, b;
    split_nm(xi, p.org_x, &a.x, &b.x);
    split_nm(yi, p.org_y, &a.y, &b.y);
    split_nm(zi, 0.0, &a.z, &b.z);
    a.w = (float)(p.r_tip / dis);
    b.w = 0.f;
    pool.ip_hi[gi] = a;
    pool.ip_lo[gi] = b;
  }
}

__device__ __forceinline__ void pack_one(const DiodeParams& p, const Pool& pool, int gi) {
  pack_vals(p, pool, gi, pool.x[gi], pool.y[gi], pool.z[gi], pool.q[gi]);
}

// ---- planner --------------------------------------------------------------------
__device__ __forceinline__ int plan_ni(const DiodeParams& p, const DiodeDyn& y, int mode,
                                       const int* npts, int d) {
  const int nj = y.n;
  const bool std_force = p.tts == 0 || (mode & PM_ALL_DIODES);   // else k_force_tts
  switch (mode & 0xff) {
    case PM_FORCE_PLANAR: return (p.geometry == RD_G_PLANAR && std_force) ? nj : 0;
    case PM_FORCE_TIP: return (p.geometry == RD_G_TIP && std_force) ? nj : 0;
    case PM_FORCE_TTS: return p.tts > 0 ? nj : 0;
    case PM_FIELD: return npts[d];
    case PM_SUPPLY_PLANAR:
      return (p.emission && p.geometry == RD_G_PLANAR && p.image_charge) ? p.quad_n * p.quad_n : 0;
    case PM_SUPPLY_LAT:
      return (p.emission && p.geometry == RD_G_PLANAR && !p.image_charge) ? p.quad_n * p.quad_n : 0;
    case PM_SUPPLY_TIP: return (p.emission && p.geometry == RD_G_TIP) ? 10000 : 0;
    // serial diodes: k_mh_serial; diodes with no particle in flight: k_mh_vacuum
    case PM_MH: return (p.emission && !p.mh_serial && !rd_mh_vacuum(p, y)) ? y.chains : 0;
    default: return nj;
  }
}

// Tiles and j-chunking of one diode.  The chunk length depends only on the
// diode's own counts and the engine's chunk rule (at least clen_min
// particles, at most nch_max chunks per tile; RD_CLEN_MIN / RD_NCH_MAX by
// default), so the summation order -- and therefore every result --
// is the same whether a diode runs alone or among other diodes.  Chunks of
// at most ~1024 particles also bound the cost of one work item, so the last
// items of a launch end soon after the others.
__device__ __forceinline__ void plan_split(int ni, int nj, int tsize, bool pair, int grow, int clen_min,
                                           int nch_max, int* tiles, int* nch, int* clen) {
  *tiles = (ni + tsize - 1) / tsize;
  *nch = 1;
  *clen = RD_TILE;
  if (pair && *tiles > 0) {
    int c = (nj + nch_max - 1) / nch_max;
    if (c < clen_min) c = clen_min;
    c = ((c + RD_TILE - 1) / RD_TILE) * RD_TILE;
    c <<= grow;   // only if the scratch bound is ever hit (never by construction)
    *clen = c;
    *nch = nj > 0 ? (nj + c - 1) / c : 1;
  }
}

__global__ void __launch_bounds__(1024)
k_plan(const DiodeParams* __restrict__ P, const DiodeDyn* __restrict__ Dy, int nslots, int mode,
       int chunk_rule, int max_items, const int* __restrict__ npts, PlanEntry* __restrict__ plan,
       PlanHeader* __restrict__ ph) {
  __shared__ double red[1024];
  __shared__ int s_items[32], s_chains[32];
  __shared__ int s_run_items, s_run_chains;
  const int tid = threadIdx.x;
  const int tsize = (mode == PM_PART1024) ? 1024 : RD_ITILE;
  const bool pair = ((mode & 0xff) <= PM_SUPPLY_LAT);
  const int clen_min = chunk_rule & 0xffff, nch_max = chunk_rule >> 16;   // see rd_chunk_rule
  // the planar supply points are many tiles already: at most RD_SUP_NCH chunks per tile
  const int nch_eff = ((mode & 0xff) == PM_SUPPLY_PLANAR || (mode & 0xff) == PM_SUPPLY_LAT)
                          ? min(nch_max, RD_SUP_NCH) : nch_max;
  // grow the chunk length only if the items would not fit the scratch
  __shared__ int s_grow;
  if (tid == 0) s_grow = 0;
  __syncthreads();
  for (int round = 0; round < 24; ++round) {
    const int grow = s_grow;
    double cnt = 0.0;
    for (int d = tid; d < nslots; d += blockDim.x) {
      if (!P[d].active) continue;
      int tiles, nch, clen;
      plan_split(plan_ni(P[d], Dy[d], mode, npts, d), Dy[d].n, tsize, pair, grow, clen_min, nch_eff, &tiles,
                 &nch, &clen);
      cnt += (double)tiles * nch;
    }
    red[tid] = cnt;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (tid < s) red[tid] += red[tid + s];
      __syncthreads();
    }
    const bool fits = red[0] <= (double)max_items;
    __syncthreads();
    if (fits) break;
    if (tid == 0) s_grow = grow + 1;
    __syncthreads();
  }
  const int grow = s_grow;
  // pass 3: entries with a running block scan
  if (tid == 0) { s_run_items = 0; s_run_chains = 0; }
  __syncthreads();
  for (int base = 0; base < nslots; base += blockDim.x) {
    int d = base + tid;
    int items = 0, ni = 0, nj = 0, tiles = 0, nch = 1, clen = RD_TILE, chains = 0;
    if (d < nslots && P[d].active) {
      nj = Dy[d].n;
      ni = plan_ni(P[d], Dy[d], mode, npts, d);
      if (mode == PM_MH) chains = ni;
      plan_split(ni, nj, tsize, pair, grow, clen_min, nch_eff, &tiles, &nch, &clen);
      items = tiles * nch;
    }
    int lane = tid & 31, w = tid >> 5;
    int vi = items, vc = chains;
    for (int o = 1; o < 32; o <<= 1) {
      int a = __shfl_up_sync(0xffffffffu, vi, o), b = __shfl_up_sync(0xffffffffu, vc, o);
      if (lane >= o) { vi += a; vc += b; }
    }
    if (lane == 31) { s_items[w] = vi; s_chains[w] = vc; }
    __syncthreads();
    int oi = 0, oc = 0;
    for (int q = 0; q < w; ++q) { oi += s_items[q]; oc += s_chains[q]; }
    int run_i = s_run_items, run_c = s_run_chains;
    if (d < nslots) {
      PlanEntry e;
      e.item_off = run_i + oi + vi - items;
      e.tiles = tiles; e.nch = nch; e.clen = clen; e.n_i = ni; e.n_j = nj;
      e.pad0 = run_c + oc + vc - chains;
      e.tsize = tsize;
      plan[d] = e;
    }
    __syncthreads();
    if (tid == blockDim.x - 1) { s_run_items = run_i + oi + vi; s_run_chains = run_c + oc + vc; }
    __syncthreads();
  }
  if (tid == 0) {
    ph->total_items = s_run_items < max_items ? s_run_items : max_items;
    ph->n_diodes = nslots;
  }
}

// Per-particle index space over the PM_PART plan (tiles of RD_ITILE).
__device__ __forceinline__ bool part_index(const PlanEntry* plan, const PlanHeader* ph, int g,
                                           int* d, int* i) {
  ItemRef it = decode_item(plan, ph->n_diodes, g);
  *d = it.d;
  *i = it.i0 + threadIdx.x;
  return *i < plan[it.d].n_i;
}

__global__ void __launch_bounds__(RD_ITILE)
k_pack(const DiodeParams* __restrict__ P, Pool pool, const PlanEntry* __restrict__ plan,
       const PlanHeader* __restrict__ ph) {
  for (int g = blockIdx.x; g < ph->total_items; g += gridDim.x) {
    int d, i;
    if (!part_index(plan, ph, g, &d, &i)) continue;
    pack_one(P[d], pool, P[d].off + i);
  }
}

__global__ void __launch_bounds__(RD_ITILE)
k_position(const DiodeParams* __restrict__ P, DiodeDyn* __restrict__ Dy, Pool pool,
           const PlanEntry* __restrict__ plan, const PlanHeader* __restrict__ ph, EventLog ev,
           const int* __restrict__ step_ptr) {
  for (int g = blockIdx.x; g < ph->total_items; g += gridDim.x) {
    int d, i;
    const bool valid = part_index(plan, ph, g, &d, &i);   // d is the item's diode on every lane
    int rm = 0;   // this lane's removal (mark_remove_flags)
    if (valid) {
    const DiodeParams& p = P[d];
    const int gi = p.off + i;
    const int sp = pool.species[gi];
    DiodeDyn& yy = Dy[d];
    const int step = *step_ptr - yy.step_offset;
    // two-time-step diodes: ions move only on steps divisible by T, with the
    // step T*dt (Update_Species_Position, src/mod_verlet.F90:234-290); T = 1
    // takes the plain formula (the factor 1 is exact), so it stays bit-equal
    // to the standard integrator whatever the compiler contracts
    const bool slow = p.tts > 1 && sp == 2;
    if (sp != 3 && !(slow && step % p.tts != 0)) {
      const double dt = p.dt, dt2 = p.dt2;
      double ax = pool.ax[gi], ay = pool.ay[gi], az = pool.az[gi];
      double bx = pool.bx[gi], by = pool.by[gi], bz = pool.bz[gi];
      const double z_prev = pool.z[gi];
      double x, y, z;
      if (!slow) {
        x = (pool.x[gi] + pool.vx[gi] * dt) + ((1.0 / 6.0) * (4.0 * ax - bx)) * dt2;
        y = (pool.y[gi] + pool.vy[gi] * dt) + ((1.0 / 6.0) * (4.0 * ay - by)) * dt2;
        z = (z_prev + pool.vz[gi] * dt) + ((1.0 / 6.0) * (4.0 * az - bz)) * dt2;
      } else {
        const double T = (double)p.tts, T2 = T * T;
        x = (pool.x[gi] + (pool.vx[gi] * dt) * T) + (((1.0 / 6.0) * (4.0 * ax - bx)) * dt2) * T2;
        y = (pool.y[gi] + (pool.vy[gi] * dt) * T) + (((1.0 / 6.0) * (4.0 * ay - by)) * dt2) * T2;
        z = (z_prev + (pool.vz[gi] * dt) * T) + (((1.0 / 6.0) * (4.0 * az - bz)) * dt2) * T2;
      }
      pool.x[gi] = x; pool.y[gi] = y; pool.z[gi] = z;
      pool.cx[gi] = bx; pool.cy[gi] = by; pool.cz[gi] = bz;
      pool.bx[gi] = ax; pool.by[gi] = ay; pool.bz[gi] = az;
      pool.ax[gi] = 0.0; pool.ay[gi] = 0.0; pool.az[gi] = 0.0;
      for (int k = 0; k < p.planes_n; ++k) {   // Check_Planes (src/mod_verlet.F90:343-367)
        const double zp = p.planes_z[k];
        if (zp > 0.0 && z > zp && z_prev < zp)
          log_event(ev, x, y, z, pool.vx[gi], pool.vy[gi], pool.vz[gi], d, RD_EVENT_PLANE + k,
                    pool.section[gi], pool.id[gi], pool.species[gi], step);
      }
      if (z < 0.0) rm = mark_remove_flags(p, pool, gi, 2, ev, d, step);
      else if (z > p.d) rm = mark_remove_flags(p, pool, gi, 1, ev, d, step);
      if (p.geometry == RD_G_TIP && tip_eta(p, x, y, z) < p.eta_1) rm |= mark_remove_flags(p, pool, gi, 2, ev, d, step);
    }
    pack_one(p, pool, gi);
    }
    count_removals_warp(Dy[d], rm, i);
  }
}

// Item partials of the velocity pass: 10 values per 128-particle item (ramo
// e, ramo ion, electron v (3), ion v (3), electrons, ions).
constexpr int RD_VEL_NV = 10;

// Sum of 8 per-lane values over a warp by transpose reduction: three halving
// exchanges (lanes 16, 8, 4 apart) leave each lane one value summed over 8
// lanes, two butterfly steps finish it.  Lane l returns the total of value
// (l >> 2) & 7.  9 FP64 additions per lane (a butterfly per value takes 40);
// the order is fixed, so the result does not depend on scheduling.
__device__ __forceinline__ double warp_sum8(double a[8], int lane) {
  const bool u16 = lane & 16, u8 = lane & 8, u4 = lane & 4;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const double send = u16 ? a[k] : a[k + 4], keep = u16 ? a[k + 4] : a[k];
    a[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const double send = u8 ? a[k] : a[k + 2], keep = u8 ? a[k + 2] : a[k];
    a[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
  double t;
  {
    const double send = u4 ? a[0] : a[1], keep = u4 ? a[1] : a[0];
    t = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
  t += __shfl_xor_sync(0xffffffffu, t, 2);
  t += __shfl_xor_sync(0xffffffffu, t, 1);
  return t;
}

__global__ void __launch_bounds__(RD_ITILE)
k_velocity(const DiodeParams* __restrict__ P, const DiodeDyn* __restrict__ Dy, Pool pool,
           const PlanEntry* __restrict__ plan, const PlanHeader* __restrict__ ph,
           double* __restrict__ part, const int* __restrict__ step_ptr) {
  __shared__ double s_w[RD_ITILE / 32][8];
  __shared__ int s_n[RD_ITILE / 32][2];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int g = blockIdx.x; g < ph->total_items; g += gridDim.x) {   // g is block-uniform
    int d, i;
    const bool live = part_index(plan, ph, g, &d, &i);
    const DiodeParams& p = P[d];
    const int gi = p.off + i;
    const int sp = live ? pool.species[gi] : 0;
    const bool ion_step = p.tts <= 1 || (*step_ptr - Dy[d].step_offset) % p.tts == 0;
    // a: ramo e, ramo ion, electron v (3), ion v (3)
    double a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = 0.0;
    // two-time-step diodes: ions only on steps divisible by T, with the step
    // T*dt (Update_Species_Velocity, src/mod_verlet.F90:511-590); T = 1 as in
    // k_position
    const bool slow = p.tts > 1 && sp == 2;
    if (live && sp != 3 && !(slow && !ion_step)) {
      const double dt = p.dt;
      double vx, vy, vz;
      if (!slow) {
        vx = pool.vx[gi] + ((1.0 / 6.0) * ((2.0 * pool.ax[gi] + 5.0 * pool.bx[gi]) - pool.cx[gi])) * dt;
        vy = pool.vy[gi] + ((1.0 / 6.0) * ((2.0 * pool.ay[gi] + 5.0 * pool.by[gi]) - pool.cy[gi])) * dt;
        vz = pool.vz[gi] + ((1.0 / 6.0) * ((2.0 * pool.az[gi] + 5.0 * pool.bz[gi]) - pool.cz[gi])) * dt;
      } else {
        const double T = (double)p.tts;
        vx = pool.vx[gi] + (((1.0 / 6.0) * ((2.0 * pool.ax[gi] + 5.0 * pool.bx[gi]) - pool.cx[gi])) * dt) * T;
        vy = pool.vy[gi] + (((1.0 / 6.0) * ((2.0 * pool.ay[gi] + 5.0 * pool.by[gi]) - pool.cy[gi])) * dt) * T;
        vz = pool.vz[gi] + (((1.0 / 6.0) * ((2.0 * pool.az[gi] + 5.0 * pool.bz[gi]) - pool.cz[gi])) * dt) * T;
      }
      pool.vx[gi] = vx; pool.vy[gi] = vy; pool.vz[gi] = vz;
      double r;   // ramo_current(species): electrons and ions
      if (p.geometry == RD_G_TIP) {   // E_zunit_tip
        double ex, ey, ez;
        tip_field_E(p, pool.x[gi], pool.y[gi], pool.z[gi], &ex, &ey, &ez);
        const double ux = (ex * p.pre_E_unit) / p.pre_E, uy = (ey * p.pre_E_unit) / p.pre_E,
                     uz = (ez * p.pre_E_unit) / p.pre_E;
        r = pool.q[gi] * ((vx * ux + vy * uy) + vz * uz);
      } else {                        // E_zunit_planar: (0, 0, -1/d); the x, y terms are 0
        r = pool.q[gi] * (vz * p.ramo_uz);
      }
      if (sp == 2) {
        a[1] = r; a[5] = vx; a[6] = vy; a[7] = vz;
      } else {
        a[0] = r;
        if (sp == 1) { a[2] = vx; a[3] = vy; a[4] = vz; }
      }
    }
    // Average_Velocities counts the particles before removal, moved or not
    const int ne = __popc(__ballot_sync(0xffffffffu, live && sp == 1));
    const int ni = __popc(__ballot_sync(0xffffffffu, live && sp == 2));
    const double t = warp_sum8(a, lane);
    if ((lane & 3) == 0) s_w[w][lane >> 2] = t;
    if (lane == 0) { s_n[w][0] = ne; s_n[w][1] = ni; }
    __syncthreads();
    if (threadIdx.x < 8) {
      double u = s_w[0][threadIdx.x];
#pragma unroll
      for (int q = 1; q < RD_ITILE / 32; ++q) u += s_w[q][threadIdx.x];
      part[(size_t)g * RD_VEL_NV + threadIdx.x] = u;
    } else if (threadIdx.x < RD_VEL_NV) {
      int c = 0;
#pragma unroll
      for (int q = 0; q < RD_ITILE / 32; ++q) c += s_n[q][threadIdx.x - 8];
      part[(size_t)g * RD_VEL_NV + threadIdx.x] = (double)c;
    }
    __syncthreads();
  }
}

// Ramo current per species, the mean velocities of Average_Velocities
// (src/mod_verlet.F90:428-447: sums over the particles the velocity update
// moved, divided by the particle counts before removal) and the
// electron-step count, per diode: the diode's item partials (k_velocity)
// added in a fixed order.
__global__ void __launch_bounds__(256)
k_ramo(const DiodeParams* __restrict__ P, DiodeDyn* __restrict__ Dy, const PlanEntry* __restrict__ plan,
       const double* __restrict__ part) {
  __shared__ double red[RD_VEL_NV][256];
  const int d = blockIdx.x;
  const DiodeParams& p = P[d];
  if (!p.active) return;
  DiodeDyn& y = Dy[d];
  const int n = y.n;
  const int g0 = plan[d].item_off, items = plan[d].tiles;
  double v[RD_VEL_NV];
  for (int k = 0; k < RD_VEL_NV; ++k) v[k] = 0.0;
  for (int t = threadIdx.x; t < items; t += blockDim.x)
    for (int k = 0; k < RD_VEL_NV; ++k) v[k] += part[(size_t)(g0 + t) * RD_VEL_NV + k];
  for (int k = 0; k < RD_VEL_NV; ++k) red[k][threadIdx.x] = v[k];
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
      for (int k = 0; k < RD_VEL_NV; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double ne = red[8][0], ni = red[9][0];
    y.ramo_current = red[0][0];
    y.ramo_ion = red[1][0];
    for (int c = 0; c < 3; ++c) {
      const double se = red[2 + c][0], si = red[5 + c][0];
      y.avg_part_vel[c] = n > 0 ? (se + si) / n : 0.0;
      y.avg_elec_vel[c] = ne > 0.0 ? se / ne : 0.0;
      y.avg_ion_vel[c] = ni > 0.0 ? si / ni : 0.0;
    }
    const double ae = sqrt((y.avg_elec_vel[0] * y.avg_elec_vel[0] + y.avg_elec_vel[1] * y.avg_elec_vel[1]) +
                           y.avg_elec_vel[2] * y.avg_elec_vel[2]);
    y.avg_mob = p.E_z != 0.0 ? ae / (-1.0 * p.E_z) : 0.0;
    y.n_vel = n;
    y.n_elec_vel = (int)ne;
    y.n_ion_vel = (int)ni;
    y.electron_steps += n;
    y.steps_done += 1;
  }
}

// ---- compaction ------------------------------------------------------------------------
// Stable compaction in place over 256-particle units (four per 1024-particle
// tile of the PM_PART1024 plan; unit u = 4 x item + quarter):
//  * k_compact_count: survivors per unit (cnt[u]), and the units' load flags
//    cleared.
//  * k_compact_scan: per diode, the survivors of the diode's earlier units
//    (pre[u], an exclusive scan in unit order): the unit's first destination.
//  * k_compact_move: units taken in increasing order from a counter.  A unit
//    loads its moving survivors (those behind the diode's first removed
//    particle) into registers, records the life times of its removed
//    electrons and raises its load flag; then it waits until every earlier
//    unit whose particles its destinations overwrite has raised its flag,
//    and stores.  Destinations never lie behind a survivor's own index, so
//    only earlier units are overwritten; those were taken before this one and
//    are running or done, and their loads do not wait, so every wait ends.
//    Each wait is still bounded (RD_COMPACT_SPIN polls): a wait that gives up
//    counts in cq[2] (rd_run reports it) and the unit stores nothing.
// Each moved survivor is read once and written once (152 B of state each
// way) and its FP32 packs are written from the loaded values.
__global__ void __launch_bounds__(1024)
k_compact_count(const DiodeParams* __restrict__ P, const DiodeDyn* __restrict__ Dy, Pool pool,
                const PlanEntry* __restrict__ plan, const PlanHeader* __restrict__ ph,
                int* __restrict__ cnt, int* __restrict__ flag) {
  __shared__ int wsum[32];
  for (int g = blockIdx.x; g < ph->total_items; g += gridDim.x) {
    if (threadIdx.x < 4) flag[4 * g + threadIdx.x] = 0;
    ItemRef it = decode_item(plan, ph->n_diodes, g);
    const DiodeParams& p = P[it.d];
    if (Dy[it.d].n_remove == 0) continue;   // block-uniform
    const int n = plan[it.d].n_i;
    const int i = it.i0 + threadIdx.x;
    int m = (i < n) ? pool.mask[p.off + i] : 0;
    int c = __popc(__ballot_sync(0xffffffffu, m));
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x < 4) {   // unit q: warps 8q .. 8q + 7
      int t = 0;
      for (int k = 0; k < 8; ++k) t += wsum[8 * threadIdx.x + k];
      cnt[4 * g + threadIdx.x] = t;
    }
    __syncthreads();
  }
}

// One block per diode slot with removals: pre[u] = sum of cnt over the
// diode's earlier units, in chunks of 1024 units with a carry.
__global__ void __launch_bounds__(1024)
k_compact_scan(const DiodeParams* __restrict__ P, const DiodeDyn* __restrict__ Dy,
               const PlanEntry* __restrict__ plan, const int* __restrict__ cnt, int* __restrict__ pre) {
  __shared__ int wsum[32];
  const int d = blockIdx.x;
  if (!P[d].active || Dy[d].n_remove == 0) return;
  const int base = 4 * plan[d].item_off, units = 4 * plan[d].tiles;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int carry = 0;
  for (int c0 = 0; c0 < units; c0 += 1024) {
    const int u = c0 + threadIdx.x;
    const int v = u < units ? cnt[base + u] : 0;
    int x = v;   // inclusive scan in the warp
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
      int t = wsum[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      wsum[lane] = t;   // inclusive over the warps
    }
    __syncthreads();
    const int excl = carry + (w > 0 ? wsum[w - 1] : 0) + x - v;
    if (u < units) pre[base + u] = excl;
    carry += wsum[31];
    __syncthreads();
  }
}

struct MovedParticle {
  double x, y, z, vx, vy, vz, ax, ay, az, bx, by, bz, cx, cy, cz, q, m;
  int species, id, step0, section;
};

__device__ __forceinline__ void load_particle(const Pool& a, int i, MovedParticle& r) {
  r.x = a.x[i]; r.y = a.y[i]; r.z = a.z[i];
  r.vx = a.vx[i]; r.vy = a.vy[i]; r.vz = a.vz[i];
  r.ax = a.ax[i]; r.ay = a.ay[i]; r.az = a.az[i];
  r.bx = a.bx[i]; r.by = a.by[i]; r.bz = a.bz[i];
  r.cx = a.cx[i]; r.cy = a.cy[i]; r.cz = a.cz[i];
  r.q = a.q[i]; r.m = a.m[i];
  r.species = a.species[i]; r.id = a.id[i]; r.step0 = a.step0[i]; r.section = a.section[i];
}

__device__ __forceinline__ void store_particle(const Pool& b, int i, const MovedParticle& r) {
  b.x[i] = r.x; b.y[i] = r.y; b.z[i] = r.z;
  b.vx[i] = r.vx; b.vy[i] = r.vy; b.vz[i] = r.vz;
  b.ax[i] = r.ax; b.ay[i] = r.ay; b.az[i] = r.az;
  b.bx[i] = r.bx; b.by[i] = r.by; b.bz[i] = r.bz;
  b.cx[i] = r.cx; b.cy[i] = r.cy; b.cz[i] = r.cz;
  b.q[i] = r.q; b.m[i] = r.m;
  b.species[i] = r.species; b.id[i] = r.id; b.step0[i] = r.step0; b.section[i] = r.section;
}

__global__ void __launch_bounds__(256, 4)
k_compact_move(const DiodeParams* __restrict__ P, const DiodeDyn* __restrict__ Dy, Pool pool,
               const PlanEntry* __restrict__ plan, const PlanHeader* __restrict__ ph,
               const int* __restrict__ cnt, const int* __restrict__ pre, int* __restrict__ flag,
               int* __restrict__ cq, int* __restrict__ life, const int* __restrict__ step_ptr) {
  __shared__ int wsum[8], s_unit, s_ok;
  const int total = 4 * ph->total_items, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_unit = atomicAdd(&cq[0], 1);   // units in increasing order
    __syncthreads();
    const int u = s_unit;
    if (u >= total) break;
    const int g = u >> 2;
    ItemRef it = decode_item(plan, ph->n_diodes, g);
    const DiodeParams& p = P[it.d];
    const DiodeDyn& y = Dy[it.d];
    const int n = plan[it.d].n_i, i0 = it.i0 + 256 * (u & 3), tb0 = plan[it.d].item_off;
    const int fd = y.first_dead;
    if (y.n_remove == 0 || i0 >= n || i0 + 256 <= fd) {   // nothing of this unit moves or is overwritten
      if (threadIdx.x == 0) atomicExch(&flag[u], 1);
      continue;
    }
    const int before = pre[u];
    const int i = i0 + threadIdx.x;
    const int m = (i < n) ? pool.mask[p.off + i] : 0;
    const unsigned bal = __ballot_sync(0xffffffffu, m);
    if (lane == 0) wsum[w] = __popc(bal);
    __syncthreads();
    int pos = 0;
    for (int q = 0; q < w; ++q) pos += wsum[q];
    pos += __popc(bal & ((1u << lane) - 1));
    const bool moves = i < n && i >= fd && m;
    MovedParticle r;
    if (moves) load_particle(pool, p.off + i, r);
    int bin = -1;   // life-time bin of a removed electron (record_lifetime :1135-1160)
    if (i < n && i >= fd && !m && (n - y.n_remove) > 0) {   // the reference skips the all-removed case
      int lt = (*step_ptr - y.step_offset) - pool.step0[p.off + i];
      if (lt <= 0) lt = 1;
      if (lt > RD_MAX_LIFE) lt = RD_MAX_LIFE;
      if (pool.species[p.off + i] == 1) bin = lt - 1;
    }
    // one atomic per distinct bin of the warp: electrons removed together mostly share one
    const unsigned peers = __match_any_sync(0xffffffffu, bin);
    if (bin >= 0 && lane == __ffs(peers) - 1)
      atomicAdd(&life[(size_t)it.d * RD_MAX_LIFE + bin], __popc(peers));
    if (i < n) pool.mask[p.off + i] = 1;
    __threadfence();   // this thread's loads are complete before the flag is raised
    __syncthreads();
    if (threadIdx.x == 0) atomicExch(&flag[u], 1);
    // earlier units holding positions of [before, before + cnt): the destinations
    // (each below its survivor's own index, so in this unit or an earlier one)
    const int ku = cnt[u], own = (u - 4 * tb0);
    const int t_lo = before >> 8, t_hi = ku > 0 ? min(own - 1, (before + ku - 1) >> 8) : -1;
    if (w == 0) {
      int ok = 1;
      for (int t = t_lo + lane; t <= t_hi; t += 32) {
        const volatile int* f = flag + 4 * tb0 + t;
        int spins = 0;
        while (*f == 0 && spins < RD_COMPACT_SPIN) { __nanosleep(64); ++spins; }
        if (*f == 0) ok = 0;
      }
      ok = __all_sync(0xffffffffu, ok);
      if (lane == 0) {
        if (!ok) atomicAdd(&cq[2], 1);
        s_ok = ok;
      }
      __threadfence();
    }
    __syncthreads();
    if (!s_ok) continue;
    if (moves) {
      const int dst = p.off + before + pos;
      store_particle(pool, dst, r);
      pack_vals(p, pool, dst, r.x, r.y, r.z, r.q);
    }
  }
  // the last block to leave resets the unit counter for the next launch
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&cq[1], 1) == (int)gridDim.x - 1) {
      cq[0] = 0;
      cq[1] = 0;
      __threadfence();
    }
  }
}

__global__ void k_compact_finish(const DiodeParams* __restrict__ P, DiodeDyn* __restrict__ Dy, int nslots) {
  int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nslots || !P[d].active) return;
  DiodeDyn& y = Dy[d];
  y.absorbed_top_step = y.n_remove_top;
  y.absorbed_bot_step = y.n_remove_bot;
  y.absorbed_top_total += y.n_remove_top;
  y.absorbed_bot_total += y.n_remove_bot;
  if (y.n_remove > 0 && y.n > 0) y.n = y.n - y.n_remove;
  y.n_remove = y.n_remove_top = y.n_remove_bot = 0;
  y.first_dead = 0x7fffffff;
}

__global__ void k_step_set(int* step_ptr, int step) { *step_ptr = step; }
__global__ void k_step_inc(int* step_ptr) { *step_ptr += 1; }

}  // namespace

// ---- launch wrappers ------------------------------------------------------------------
cudaError_t rd_launch_plan(cudaStream_t st, const DiodeParams* P, const DiodeDyn* Dy, int nslots,
                           int mode, int chunk_rule, int max_items, const int* npts,
                           PlanEntry* plan, PlanHeader* ph) {
  k_plan<<<1, 1024, 0, st>>>(P, Dy, nslots, mode, chunk_rule, max_items, npts, plan, ph);
  return cudaGetLastError();
}
// Loads the planner and the pack kernel into the current context now (they
// would otherwise load at their first launch under lazy module loading).
cudaError_t rd_preload_plan() {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, k_plan);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_pack);
  if (e == cudaSuccess) rd_grid(k_pack, RD_ITILE, 0);
  return e;
}
cudaError_t rd_launch_pack(int grid, cudaStream_t st, const DiodeParams* P, const Pool& pool,
                           const PlanEntry* plan, const PlanHeader* ph) {
  k_pack<<<rd_grid(k_pack, RD_ITILE, grid), RD_ITILE, 0, st>>>(P, pool, plan, ph);
  return cudaGetLastError();
}
cudaError_t rd_launch_position(int grid, cudaStream_t st, const DiodeParams* P, DiodeDyn* Dy,
                               const Pool& pool, const PlanEntry* plan, const PlanHeader* ph,
                               const EventLog& ev, const int* step_ptr) {
  k_position<<<rd_grid(k_position, RD_ITILE, grid), RD_ITILE, 0, st>>>(P, Dy, pool, plan, ph, ev, step_ptr);
  return cudaGetLastError();
}
cudaError_t rd_launch_velocity(int grid, int nslots, cudaStream_t st, const DiodeParams* P,
                               DiodeDyn* Dy, const Pool& pool, const PlanEntry* plan,
                               const PlanHeader* ph, double* part, const int* step_ptr) {
  k_velocity<<<rd_grid(k_velocity, RD_ITILE, grid), RD_ITILE, 0, st>>>(P, Dy, pool, plan, ph, part, step_ptr);
  k_ramo<<<nslots, 256, 0, st>>>(P, Dy, plan, part);
  return cudaGetLastError();
}
cudaError_t rd_launch_compact(int grid, int nslots, cudaStream_t st, const DiodeParams* P,
                              DiodeDyn* Dy, const Pool& pool, const PlanEntry* plan, const PlanHeader* ph,
                              int* cnt, int* pre, int* flag, int* cq, int* life, const int* step_ptr) {
  k_compact_count<<<rd_grid(k_compact_count, 1024, grid), 1024, 0, st>>>(P, Dy, pool, plan, ph, cnt, flag);
  if (nslots > 0) k_compact_scan<<<nslots, 1024, 0, st>>>(P, Dy, plan, cnt, pre);
  k_compact_move<<<rd_grid(k_compact_move, 256, grid), 256, 0, st>>>(P, Dy, pool, plan, ph, cnt, pre, flag, cq,
                                                                     life, step_ptr);
  k_compact_finish<<<(nslots + 127) / 128, 128, 0, st>>>(P, Dy, nslots);
  return cudaGetLastError();
}
cudaError_t rd_launch_step_set(cudaStream_t st, int* step_ptr, int step) {
  k_step_set<<<1, 1, 0, st>>>(step_ptr, step);
  return cudaGetLastError();
}
cudaError_t rd_launch_step_inc(cudaStream_t st, int* step_ptr) {
  k_step_inc<<<1, 1, 0, st>>>(step_ptr);
  return cudaGetLastError();
}

namespace {
// Add_Particle (src/mod_pair.F90:29-159) for a batch, in order.
__global__ void k_add_particles(const DiodeParams* __restrict__ P, DiodeDyn* __restrict__ Dy, Pool pool,
                                int d, int cnt, const double* __restrict__ pos, const double* __restrict__ vel,
                                const int* __restrict__ species, int step, int section) {
  const DiodeParams& p = P[d];
  DiodeDyn& y = Dy[d];
  const int n0 = y.n, id0 = y.nrID;
  const int room = p.cap - n0 > 0 ? p.cap - n0 : 0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < cnt && t < room; t += gridDim.x * blockDim.x) {
    const int i = n0 + t, gi = p.off + i;
    const double X = pos[3 * t], Y = pos[3 * t + 1], Z = pos[3 * t + 2];
    const int sp = species ? species[t] : 1;
    double q, m;
    if (sp == 1) { q = -1.0 * c_k.q0; m = 1.0 * c_k.m0; }
    else if (sp == 2) { q = 1.0 * c_k.q0; m = c_k.m_N2p; }
    else { q = 0.0; m = c_k.m_N2; }
    double ex, ey, ez;
    vacuum_field(p, X, Y, Z, &ex, &ey, &ez);
    const double qm = q / m;
    pool.x[gi] = X; pool.y[gi] = Y; pool.z[gi] = Z;
    pool.vx[gi] = vel ? vel[3 * t] : 0.0; pool.vy[gi] = vel ? vel[3 * t + 1] : 0.0;
    pool.vz[gi] = vel ? vel[3 * t + 2] : 0.0;
    pool.ax[gi] = pool.bx[gi] = pool.cx[gi] = qm * ex;
    pool.ay[gi] = pool.by[gi] = pool.cy[gi] = qm * ey;
    pool.az[gi] = pool.bz[gi] = pool.cz[gi] = qm * ez;
    pool.q[gi] = q; pool.m[gi] = m;
    pool.species[gi] = sp; pool.id[gi] = id0 + t; pool.step0[gi] = step;
    pool.section[gi] = section; pool.mask[gi] = 1;
    pack_one(p, pool, gi);
  }
}

__global__ void k_add_finish(const DiodeParams* __restrict__ P, DiodeDyn* __restrict__ Dy, int d, int cnt) {
  DiodeDyn& y = Dy[d];
  const int room = P[d].cap - y.n > 0 ? P[d].cap - y.n : 0;
  const int added = cnt < room ? cnt : room;
  y.n += added;
  y.nrID += added;
  y.dropped_total += cnt - added;
}

__global__ void k_mark(const DiodeParams* __restrict__ P, DiodeDyn* __restrict__ Dy, Pool pool, int d,
                       int i, int why) {
  if (i < Dy[d].n) {
    mark_remove(P[d], Dy[d], pool, i, P[d].off + i, why, EventLog{nullptr, nullptr, 0}, d, 0);
    pack_one(P[d], pool, P[d].off + i);
  }
}
}  // namespace

cudaError_t rd_launch_add_particles(cudaStream_t st, const DiodeParams* P, DiodeDyn* Dy, const Pool& pool,
                                    int d, int cnt, const double* pos, const double* vel,
                                    const int* species, int step, int section) {
  if (cnt > 0) {
    int blocks = (cnt + 255) / 256;
    k_add_particles<<<blocks, 256, 0, st>>>(P, Dy, pool, d, cnt, pos, vel, species, step, section);
  }
  k_add_finish<<<1, 1, 0, st>>>(P, Dy, d, cnt);
  return cudaGetLastError();
}

// Supply quadrature points of one diode with their weights (area included)
// and their FP32-frame split (split_nm), one thread per point: planar nodes
// of the composite Gauss-Legendre rule (Do_Surface_Integration_FE's
// integrand, src/mod_field_emission_v2.F90:668-745, with the ring's
// (angle, radius) map and 2 pi w r area factor, :701-707), or the tip's
// 100 x 100 midpoint grid in (xi, phi) with the cell areas
// (Do_Field_Emission_Tip_OLDCODE, src/mod_emission_tip.f90:434-481; Tip_Area).
__global__ void __launch_bounds__(256)
k_quad_fill(QuadSpec q, double* __restrict__ qx, double* __restrict__ qy, double* __restrict__ qz,
            double* __restrict__ qw, float4* __restrict__ qpp) {
  const int npt = q.geometry == RD_G_TIP ? 10000 : q.quad_n * q.quad_n;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= npt) return;
  double x, y, z = 0.0, w;
  if (q.geometry == RD_G_TIP) {
    const int nr = 100, i = k / nr + 1, j = k % nr + 1;
    const double pi = c_k.pi, len_phi = 2.0 * pi / nr, len_xi = (q.max_xi - 1.0) / nr, e2 = q.eta_1 * q.eta_1;
    const double xi_c = 1.0 + (i - 0.5) * len_xi, phi_c = (j - 0.5) * len_phi;
    const double xy = q.a_foci * sqrt((xi_c * xi_c - 1.0) * (1.0 - q.eta_1 * q.eta_1));
    x = xy * cos(phi_c);
    y = xy * sin(phi_c);
    z = (q.a_foci * xi_c) * q.eta_1 + q.shift_z;
    const double xi1 = 1.0 + (i - 1.0) * len_xi, xi2 = 1.0 + (i + 0.0) * len_xi;
    const double ph1 = (j - 1.0) * len_phi, ph2 = (j + 0.0) * len_phi;
    const double f2 = xi2 * sqrt(xi2 * xi2 - e2) - e2 * log(xi2 + sqrt(xi2 * xi2 - e2));
    const double f1 = xi1 * sqrt(xi1 * xi1 - e2) - e2 * log(xi1 + sqrt(xi1 * xi1 - e2));
    w = (((0.5 * (q.a_foci * q.a_foci)) * sqrt(1.0 - e2)) * (ph2 - ph1)) * (f2 - f1);
  } else {
    const int iy = k / q.quad_n, ix = k % q.quad_n, Q = q.Q;
    const double uy = ((iy / Q) + 0.5 * (q.gx[iy % Q] + 1.0)) / q.P, wy = 0.5 * q.gw[iy % Q] / q.P;
    const double ux = ((ix / Q) + 0.5 * (q.gx[ix % Q] + 1.0)) / q.P, wx = 0.5 * q.gw[ix % Q] / q.P;
    if (q.emitter_type == 4) {
      const double angle = ux * 2.0 * c_k.pi, radius = q.ring_rmin + uy * q.ring_thick;
      x = radius * cos(angle);
      y = radius * sin(angle);
      w = (wx * wy) * (2.0 * c_k.pi * q.ring_thick * radius);
    } else {
      x = q.x0 + ux * q.Lx;
      y = q.y0 + uy * q.Ly;
      w = (wx * wy) * (q.Lx * q.Ly);
    }
  }
  const int g = q.q_off + k;
  qx[g] = x; qy[g] = y; qz[g] = z; qw[g] = w;
  const double vx = (x - q.org_x) * 1.0e9, vy = (y - q.org_y) * 1.0e9;
  const float ax = (float)vx, ay = (float)vy;
  qpp[g] = make_float4(ax, (float)(vx - (double)ax), ay, (float)(vy - (double)ay));
}

cudaError_t rd_launch_quad_fill(cudaStream_t st, const QuadSpec& q, double* qx, double* qy, double* qz,
                                double* qw, float4* qpp) {
  const int npt = q.geometry == RD_G_TIP ? 10000 : q.quad_n * q.quad_n;
  k_quad_fill<<<(npt + 255) / 256, 256, 0, st>>>(q, qx, qy, qz, qw, qpp);
  return cudaGetLastError();
}

cudaError_t rd_launch_mark(cudaStream_t st, const DiodeParams* P, DiodeDyn* Dy, const Pool& pool, int d,
                           int i, int why) {
  k_mark<<<1, 1, 0, st>>>(P, Dy, pool, d, i, why);
  return cudaGetLastError();
}

namespace {
// State invariants of every resident diode between steps, one block per
// diode; bad[d * RD_VALIDATE_KINDS + k] counts the violations of kind k:
//   0 particle count outside [0, capacity]      1 removal bookkeeping not cleared
//   2 species outside {1, 2, 3}                  3 a particle still marked for removal
//   4 non-finite position, velocity or acceleration
//   5 ids not strictly increasing (the stable compaction keeps creation order)
//   6 charge / mass not those of the species (Add_Particle)
__global__ void __launch_bounds__(256)
k_validate(const DiodeParams* __restrict__ P, const DiodeDyn* __restrict__ Dy, Pool pool, int* __restrict__ bad) {
  const int d = blockIdx.x;
  const DiodeParams& p = P[d];
  if (!p.active) return;
  const DiodeDyn& y = Dy[d];
  int* b = bad + d * RD_VALIDATE_KINDS;
  if (threadIdx.x == 0) {
    if (y.n < 0 || y.n > p.cap) atomicAdd(&b[0], 1);
    if (y.n_remove != 0 || y.n_remove_top != 0 || y.n_remove_bot != 0) atomicAdd(&b[1], 1);
  }
  const int n = min(max(y.n, 0), p.cap);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int gi = p.off + i, sp = pool.species[gi];
    if (sp < 1 || sp > 3) atomicAdd(&b[2], 1);
    if (pool.mask[gi] != 1) atomicAdd(&b[3], 1);
    const double v[9] = {pool.x[gi], pool.y[gi], pool.z[gi], pool.vx[gi], pool.vy[gi], pool.vz[gi],
                         pool.ax[gi], pool.ay[gi], pool.az[gi]};
    bool finite = true;
    for (int k = 0; k < 9; ++k) finite = finite && isfinite(v[k]);
    if (!finite) atomicAdd(&b[4], 1);
    if (i > 0 && pool.id[gi] <= pool.id[gi - 1]) atomicAdd(&b[5], 1);
    const double q = pool.q[gi], m = pool.m[gi];
    const bool ok = (sp == 1 && q == -1.0 * c_k.q0 && m == 1.0 * c_k.m0) ||
                    (sp == 2 && q == 1.0 * c_k.q0 && m == c_k.m_N2p) || (sp == 3 && q == 0.0 && m == c_k.m_N2);
    if (!ok) atomicAdd(&b[6], 1);
  }
}
}  // namespace

cudaError_t rd_launch_validate(int nslots, cudaStream_t st, const DiodeParams* P, const DiodeDyn* Dy,
                               const Pool& pool, int* bad) {
  cudaMemsetAsync(bad, 0, sizeof(int) * (size_t)nslots * RD_VALIDATE_KINDS, st);
  if (nslots > 0) k_validate<<<nslots, 256, 0, st>>>(P, Dy, pool, bad);
  return cudaGetLastError();
}

RD_DEFINE_CONSTANT_UPLOAD(step)
