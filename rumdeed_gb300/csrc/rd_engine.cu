// rd_engine.cu -- host side of librumdeed_gb300: engine and diode-slot
// management, the step pipeline and its CUDA graph, and the C ABI declared
// in include/rumdeed_gpu.h.
//
// One engine owns one GPU stream, one particle pool shared by all diode
// slots (segment table in device memory), the scratch of the pair-sum engine
// and the Metropolis-Hastings chain pool.  The whole time step -- emission
// (supply integral, MH chains, emission test and append), Beeman position
// update, all-pairs forces, velocity update and Ramo current, stable
// compaction -- is a fixed sequence of kernels whose work lists are built on
// the device, captured once as a CUDA graph and replayed every step.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <map>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/rumdeed_gpu.h"
#include "rd_pair.cuh"

// The float next to v on the side of zero.
static float f32_toward_zero(double v) {
  float f = (float)v;
  if (std::fabs((double)f) > std::fabs(v)) f = std::nextafter(f, 0.0f);
  return f;
}

// ---- kernels (other translation units) ------------------------------------------
cudaError_t rd_upload_constants_force(const RdConst&);
cudaError_t rd_upload_constants_field(const RdConst&);
cudaError_t rd_upload_constants_step(const RdConst&);
cudaError_t rd_launch_force(int prec, int geometry_mask, int nic_general, int grid, cudaStream_t st,
                            const DiodeParams* P, const DiodeDyn* Dy, const Pool& pool,
                            const PlanEntry* plan, const PlanHeader* ph, double* partial,
                            int* tickets, double kscale, int* queue);
cudaError_t rd_launch_field_points(int prec, int geom, int grid, cudaStream_t st,
                                   const DiodeParams* P, const Pool& pool, const PlanEntry* plan,
                                   const PlanHeader* ph, const PointSet& pts, double* partial,
                                   int* tickets, double kscale);
cudaError_t rd_launch_z0_points(int prec, int grid, cudaStream_t st, const DiodeParams* P,
                                const Pool& pool, const PlanEntry* plan, const PlanHeader* ph,
                                const double* qx, const double* qy, const float4* qpp, double* qF,
                                double* partial, int* tickets, double kscale, int* queue);
cudaError_t rd_launch_supply_reduce(int nslots, cudaStream_t st, const DiodeParams* P, DiodeDyn* Dy,
                                    const double* qx, const double* qy, const double* qw,
                                    const double* qF, const double* qfx, const double* qfy,
                                    const double* work, const int* step_ptr, double* sup_part);
cudaError_t rd_launch_mh_serial(int prec, int nslots, cudaStream_t st, const DiodeParams* P, DiodeDyn* Dy,
                                const Pool& pool, const double* work, const double* wtab,
                                const int* step_ptr, double kscale, const EventLog& ev);
cudaError_t rd_launch_mh_cond(cudaStream_t st, cudaGraphConditionalHandle h, const PlanHeader* ph);
cudaError_t rd_launch_mh_vacuum(int prec, int nslots, cudaStream_t st, const DiodeParams* P, DiodeDyn* Dy,
                                const ChainState& cs, const int* ch_off, const double* wtab, const int* step_ptr,
                                double kscale);
cudaError_t rd_launch_mh_init(int prec, int grid, cudaStream_t st, const DiodeParams* P,
                              DiodeDyn* Dy, const Pool& pool, const PlanEntry* plan,
                              const PlanHeader* ph, const ChainState& cs, const int* ch_off,
                              const double* wtab, const int* step_ptr, double kscale);
cudaError_t rd_launch_mh_jump(int prec, int geometry_mask, int grid, cudaStream_t st,
                              const DiodeParams* P, DiodeDyn* Dy, const Pool& pool,
                              const PlanEntry* plan, const PlanHeader* ph, const ChainState& cs,
                              const int* ch_off, const double* wtab, const int* step_ptr,
                              int it_idx, double* partial, int* tickets, double kscale, int* queue,
                              int part = 0, int nparts = 1, int form = 0);
cudaError_t rd_launch_emit(int nslots, cudaStream_t st, const DiodeParams* P, DiodeDyn* Dy,
                           const Pool& pool, const ChainState& cs, const int* ch_off,
                           const double* work, const int* step_ptr, const EventLog& ev);
cudaError_t rd_launch_plan(cudaStream_t st, const DiodeParams* P, const DiodeDyn* Dy, int nslots,
                           int mode, int chunk_rule, int max_items, const int* npts,
                           PlanEntry* plan, PlanHeader* ph);
cudaError_t rd_launch_pack(int grid, cudaStream_t st, const DiodeParams* P, const Pool& pool,
                           const PlanEntry* plan, const PlanHeader* ph);
cudaError_t rd_launch_position(int grid, cudaStream_t st, const DiodeParams* P, DiodeDyn* Dy,
                               const Pool& pool, const PlanEntry* plan, const PlanHeader* ph, const EventLog& ev, const int* step_ptr);
cudaError_t rd_launch_velocity(int grid, int nslots, cudaStream_t st, const DiodeParams* P,
                               DiodeDyn* Dy, const Pool& pool, const PlanEntry* plan,
                               const PlanHeader* ph, double* ramo, const int* step_ptr);
cudaError_t rd_launch_force_tts(int grid, cudaStream_t st, const DiodeParams* P, const DiodeDyn* Dy,
                                const Pool& pool, const PlanEntry* plan, const PlanHeader* ph,
                                double* partial, int* tickets, int* queue, const int* step_ptr);
cudaError_t rd_launch_compact(int grid, int nslots, cudaStream_t st, const DiodeParams* P,
                              DiodeDyn* Dy, const Pool& pool, const PlanEntry* plan, const PlanHeader* ph,
                              int* cnt, int* pre, int* flag, int* cq, int* life, const int* step_ptr);
cudaError_t rd_launch_step_set(cudaStream_t st, int* step_ptr, int step);
cudaError_t rd_launch_step_inc(cudaStream_t st, int* step_ptr);
cudaError_t rd_launch_add_particles(cudaStream_t st, const DiodeParams* P, DiodeDyn* Dy,
                                    const Pool& pool, int d, int cnt, const double* pos,
                                    const double* vel, const int* species, int step, int section);
cudaError_t rd_launch_quad_fill(cudaStream_t st, const QuadSpec& q, double* qx, double* qy, double* qz,
                                double* qw, float4* qpp);
cudaError_t rd_launch_mark(cudaStream_t st, const DiodeParams* P, DiodeDyn* Dy, const Pool& pool,
                           int d, int i, int why);
cudaError_t rd_launch_validate(int nslots, cudaStream_t st, const DiodeParams* P, const DiodeDyn* Dy,
                               const Pool& pool, int* bad);


// ---- errors -------------------------------------------------------------------------
static thread_local std::string g_err;
static int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
// NVTX range over a host entry point (visible in Nsight Systems; a no-op
// unless a profiler is attached).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

#define CK(call)                                                                     \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return fail(RD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));  \
  } while (0)

// ---- constants (src/mod_global.F90:26-45,333; src/mod_field_emission_v2.F90:36-47) -----
static RdConst make_constants() {
  RdConst k;
  k.pi = 3.141592653589793238462643383279502884197169399375105820974944592307816406286;
  const double h = 6.62607015e-34, c = 299792458.0, mu0 = 1.25663706212e-6;
  const double m_u = 1.66053906660e-27;
  k.q0 = 1.602176634e-19;
  k.m0 = 9.1093837015e-31;
  k.eps0 = 1.0 / (mu0 * (c * c));
  k.hbar = h / (2.0 * k.pi);
  k.div_fac_c = 1.0 / (((4.0 * k.pi) * k.eps0) * 1.0);
  k.a_FN = (k.q0 * k.q0) / ((16.0 * (k.pi * k.pi)) * k.hbar);
  k.b_FN = (-4.0 / (3.0 * k.hbar)) * std::sqrt((2.0 * k.m0) * k.q0);
  k.l_const = k.q0 / ((4.0 * k.pi) * k.eps0);
  k.length_scale = 1.0e-9;
  k.L2 = k.length_scale * k.length_scale;
  k.tip_K = (1.0 * k.q0) / ((4.0 * k.pi) * k.eps0);
  k.m_N2 = 28.0134 * m_u;
  k.m_N2p = k.m_N2 - k.m0;
  k.q0_inv = 1.0 / k.q0;
  return k;
}

// Gauss-Legendre nodes and weights on [-1, 1] (Newton iteration on P_n).
static void gauss_legendre(int n, double* x, double* w) {
  const double pi = 3.141592653589793238462643383279502884197169399375105820974944592307816406286;
  for (int k = 0; k < n; ++k) {
    double z = std::cos(pi * (k + 0.75) / (n + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int m = 2; m <= n; ++m) {
        double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m;
        p0 = p1; p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    double p0 = 1.0, p1 = z;
    for (int m = 2; m <= n; ++m) {
      double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m;
      p0 = p1; p1 = p2;
    }
    dp = n * (z * p1 - p0) / (z * z - 1.0);
    x[k] = -z;
    w[k] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
  if (n == 1) { x[0] = 0.0; w[0] = 2.0; }
}

// ---- simple first-fit range allocator -------------------------------------------------
struct RangeAlloc {
  std::vector<std::pair<long long, long long>> free_;   // (start, length), sorted
  void init(long long cap) { free_.clear(); if (cap > 0) free_.push_back({0, cap}); }
  long long alloc(long long len, long long align) {
    if (len <= 0) return 0;
    for (size_t k = 0; k < free_.size(); ++k) {
      long long s = free_[k].first, l = free_[k].second;
      long long a = (s + align - 1) / align * align;
      if (a - s + len <= l) {
        free_.erase(free_.begin() + k);
        if (a > s) insert({s, a - s});
        if (a + len < s + l) insert({a + len, s + l - a - len});
        return a;
      }
    }
    return -1;
  }
  void release(long long s, long long len) { if (len > 0) insert({s, len}); }
  void insert(std::pair<long long, long long> r) {
    auto it = std::lower_bound(free_.begin(), free_.end(), r);
    it = free_.insert(it, r);
    size_t k = it - free_.begin();
    if (k + 1 < free_.size() && free_[k].first + free_[k].second == free_[k + 1].first) {
      free_[k].second += free_[k + 1].second;
      free_.erase(free_.begin() + k + 1);
    }
    if (k > 0 && free_[k - 1].first + free_[k - 1].second == free_[k].first) {
      free_[k - 1].second += free_[k].second;
      free_.erase(free_.begin() + k);
    }
  }
};

struct SlotHost {
  bool used = false;
  DiodeParams p{};
  long long pool_off = 0, pool_len = 0;
  long long ch_off = 0, ch_len = 0;
  long long q_off = 0, q_len = 0;
  long long w_off = 0, w_len = 0;
};

struct rd_engine {
  rd_engine_config cfg{};
  int sms = 0, grid = 0;
  cudaStream_t st = nullptr;
  cudaStream_t stp[RD_MH_PARTS_MAX] = {};    // planar MH jump parts 2.. (part 1 runs on st)
  cudaEvent_t ev_fork = nullptr;             // st -> the part streams
  cudaEvent_t ev_join[RD_MH_PARTS_MAX] = {}; // each part stream -> st
  int mh_parts = 0;   // planar MH launches per jump when two or more diodes run batched chains (0: RD_MH_PARTS)
  int mh_form = -1;   // FP32 MH jump form: 0 32 threads x 4 chains, 1 64 x 2 (-1: 1 for a lone diode, else 0)
  RdConst k{};
  double kscale = 0.0;
  int max_items = 0;
  int clen_min = RD_CLEN_MIN, nch_max = RD_NCH_MAX;   // chunk rule of the pair sums
  // device memory
  DiodeParams* dP = nullptr;
  DiodeDyn* dD = nullptr;
  Pool pool{};
  double *save_ax = nullptr, *save_ay = nullptr, *save_az = nullptr;   // accelerations kept across rd_autotune
  std::vector<void*> allocs;
  double* work = nullptr;
  double* wtab = nullptr;   // per work cell: log phi, log(l_const/phi^2), l_const/phi^2
  double *qx = nullptr, *qy = nullptr, *qz = nullptr, *qw = nullptr, *qF = nullptr, *qfx = nullptr, *qfy = nullptr;
  float4* qpp = nullptr;   // planar quadrature points in the FP32 frame
  ChainState cs{};
  int *d_choff = nullptr, *d_qoff = nullptr, *d_npts = nullptr, *d_zero_off = nullptr;
  PlanEntry* plan[PM_COUNT] = {};
  PlanHeader* ph[PM_COUNT] = {};
  double* partial = nullptr;
  double* sup_part = nullptr;   // supply sums per (diode, block of its points)
  int* tickets = nullptr;
  int* item_queue = nullptr;   // dynamic item counters (queue_next / queue_leave): [0..1] planar
                               // MH (part 0 / 1), [2..3] tip MH, [4..5] force, [6..7] supply,
                               // [6 + 2p .. 7 + 2p] planar MH part p >= 2 (8 + 2 RD_MH_PARTS_MAX)
  EventLog evlog{nullptr, nullptr, 0};   // emission / absorption records (rd_events_take)
  int *ccnt = nullptr, *cpre = nullptr, *cflag = nullptr;   // compaction: per 256-particle unit survivors,
                                                            // first destinations and load flags
  int* cq = nullptr;      // compaction: [0] tile counter, [1] blocks left, [2] waits that gave up
  double* ramo = nullptr;   // velocity-pass item partials (10 per 128-particle item)
  int* life = nullptr;
  int* d_step = nullptr;
  double *fpx = nullptr, *fpy = nullptr, *fpz = nullptr, *ffx = nullptr, *ffy = nullptr, *ffz = nullptr;
  long long fcap = 0;
  double *stage_d = nullptr;
  int* stage_i = nullptr;
  double* stage_hd = nullptr;   // pinned host mirrors of stage_d / stage_i: uploads are DMA
  int* stage_hi = nullptr;      // copies from page-locked memory
  long long stage_cap = 0;
  // overlapped admission (rd_serve): uploads on stream sa from a pinned arena into a device
  // arena, slots activated on st before the next step (activate_pending)
  cudaStream_t sa = nullptr;
  cudaStream_t sbody = nullptr;     // captures the body of the step graph's conditional MH node
  cudaEvent_t ev_adm = nullptr;
  unsigned char* adm_h = nullptr;   // pinned
  unsigned char* adm_d = nullptr;
  size_t adm_cap = 0, adm_used = 0;
  DiodeParams* act_P = nullptr;     // pinned, per slot: the parameters to activate
  DiodeDyn* act_D = nullptr;        // pinned, per slot
  int *act_choff = nullptr, *act_qoff = nullptr;   // pinned, per slot
  std::vector<int> pending;         // slots written on sa, not yet active
  // host
  std::vector<SlotHost> slots;
  RangeAlloc pool_alloc, ch_alloc, q_alloc, w_alloc;
  // graph
  cudaGraphExec_t graph = nullptr;
  std::string graph_sig;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.0;
  int last_kernels = 0;
  int kernels_in_step = 0;
  // serving
  struct Req {
    rd_diode_config cfg{};
    std::vector<double> work, pos, vel;
    int steps = 0;
    rd_request_status st{};
  };
  std::map<long long, Req> reqs;
  std::deque<long long> queue;
  std::map<int, long long> running;   // slot -> request id
  long long next_id = 1;
  int gstep = 1;                       // engine step of the next serving launch
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double clock() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }

  template <class T>
  cudaError_t dalloc(T** p, size_t count) {
    cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) allocs.push_back((void*)*p);
    return e;
  }
  // Launch shapes cover every slot (inactive ones exit at once), so the
  // captured step graph stays valid while requests come and go.
  int nslots_hw() const { return cfg.max_diodes; }
};

extern "C" {
static int flush_admissions(rd_engine* e);   // defined in the C ABI block below
}

// Panels per side of the planar supply rule when the diode does not set them:
// Gauss-Legendre nodes at most RD_SUPPLY_SPACING apart along the emitter's
// longer side (for a ring, the longer of its outer circumference and its
// width), between 16 and 256 panels.  The supply integrand varies on the scale
// of the emission height (1 nm): an electron that sits there removes a disc of
// a few nm^2 from the emitting area, and a coarser rule sees it only when a
// node happens to fall inside.  Against the converged integral of
// space-charge-limited states this spacing keeps N_sup within max(0.5,
// 1e-3 N_sup) electrons, the tolerance the reference asks of its adaptive
// integrator (src/mod_global.F90:84-92); 16 panels of 4 nodes over 1 um did not.
#define RD_SUPPLY_SPACING 5.0e-9
static int supply_panels(double Lx, double Ly, int emitter_type, double ring_rmin, double ring_thick, int Q) {
  double L = std::max(Lx, Ly);
  if (emitter_type == 4) L = std::max(2.0 * 3.14159265358979323846 * (ring_rmin + ring_thick), ring_thick);
  const double r = L / (Q * RD_SUPPLY_SPACING);
  int P = (int)std::ceil(r * (1.0 - 1e-12));
  return std::min(256, std::max(16, P));
}

static int alloc_pool(rd_engine* e, Pool& P, long long cap) {
  double** dbl[] = {&P.x, &P.y, &P.z, &P.vx, &P.vy, &P.vz, &P.ax, &P.ay, &P.az,
                    &P.bx, &P.by, &P.bz, &P.cx, &P.cy, &P.cz, &P.q, &P.m};
  for (auto p : dbl) CK(e->dalloc(p, cap));
  int** in[] = {&P.species, &P.id, &P.step0, &P.section, &P.mask};
  for (auto p : in) CK(e->dalloc(p, cap));
  float4** f4[] = {&P.pk_hi, &P.pk_lo, &P.ip_hi, &P.ip_lo, &P.zk_hi, &P.zk_lo};
  for (auto p : f4) CK(e->dalloc(p, cap));
  return RD_OK;
}

// ---- pipeline pieces ----------------------------------------------------------------
static cudaError_t plan(rd_engine* e, int mode, const int* npts = nullptr) {
  e->kernels_in_step++;
  const int slot = mode & 0xff;
  return rd_launch_plan(e->st, e->dP, e->dD, e->nslots_hw(), mode, rd_chunk_rule(e->clen_min, e->nch_max),
                        e->max_items, npts, e->plan[slot], e->ph[slot]);
}

static bool valid_chunking(int clen_min, int nch_max) {
  return clen_min >= RD_TILE && clen_min <= 65536 && clen_min % RD_TILE == 0 && nch_max >= 1 &&
         nch_max <= RD_NCH_MAX;
}

struct Sig {
  bool planar = false, tip = false, emit_planar = false, emit_tip = false, nic = false;
  bool emit_lat = false;      // some emitting planar diode has no image charges (PM_SUPPLY_LAT)
  bool emit_serial = false;   // some planar diode uses the serial MH sampler
  bool tts = false;           // some diode uses the two-time-step integrator
  int jumps = 0;
  int mh_planar = 0;          // planar diodes with batched MH chains
};
static Sig signature(const rd_engine* e) {
  Sig s;
  for (auto& sl : e->slots) {
    if (!sl.used) continue;
    const DiodeParams& p = sl.p;
    if (p.geometry == RD_G_TIP) s.tip = true; else s.planar = true;
    if (p.geometry == RD_G_PLANAR && p.image_charge && p.N_ic_max > 0) s.nic = true;
    if (p.tts > 0) s.tts = true;
    if (p.emission) {
      if (p.geometry == RD_G_TIP) s.emit_tip = true; else s.emit_planar = true;
      if (p.geometry != RD_G_TIP && !p.image_charge) s.emit_lat = true;
      if (p.geometry != RD_G_TIP && p.mh_serial) s.emit_serial = true;
      if (p.geometry != RD_G_TIP && !p.mh_serial) s.mh_planar++;
      s.jumps = std::max(s.jumps, p.mh_jumps);
    }
  }
  return s;
}

// MH launch shape of the planar jumps for the resident mix: parts of the plan
// (one launch and one stream each; one diode cannot be split) and the FP32
// thread form.  Neither changes a result: each diode's chains and counters sit
// in one part, and both forms do the same lane arithmetic in the same order.
static int mh_parts_for(const rd_engine* e, const Sig& s) {
  if (s.mh_planar <= 1) return 1;
  return e->mh_parts > 0 ? e->mh_parts : RD_MH_PARTS;
}
static int mh_form_for(const rd_engine* e, const Sig& s) {
  if (e->mh_form >= 0) return e->mh_form;
  return s.mh_planar == 1 ? 1 : 0;
}

static int planar_mh_launch(rd_engine* e, const Sig& s, int it, int parts, int form, cudaStream_t main) {
  for (int q = 0; q < parts; ++q) {
    cudaStream_t sq = q == 0 ? main : e->stp[q];
    int* queue = q == 0 ? e->item_queue : e->item_queue + 6 + 2 * (q + 1);
    CK(rd_launch_mh_jump(e->cfg.precision, 1, e->grid, sq, e->dP, e->dD, e->pool, e->plan[PM_MH], e->ph[PM_MH],
                         e->cs, e->d_choff, e->wtab, e->d_step, it, e->partial, e->tickets, e->kscale, queue,
                         parts > 1 ? q + 1 : 0, parts, form));
  }
  return RD_OK;
}

static int mh_fork(rd_engine* e, int parts, cudaStream_t main) {
  if (parts <= 1) return RD_OK;
  CK(cudaEventRecord(e->ev_fork, main));
  for (int q = 1; q < parts; ++q) CK(cudaStreamWaitEvent(e->stp[q], e->ev_fork, 0));
  return RD_OK;
}
static int mh_join(rd_engine* e, int parts, cudaStream_t main) {
  for (int q = 1; q < parts; ++q) {
    CK(cudaEventRecord(e->ev_join[q], e->stp[q]));
    CK(cudaStreamWaitEvent(main, e->ev_join[q], 0));
  }
  return RD_OK;
}

// Jumps 1..jumps of the batched MH chains.  The planar jumps run as `parts`
// launches per jump, one per part of the plan (part_range), each on its own
// stream: the parts are independent (each diode's chains and counters sit in
// one), so while one stream's launch runs its last items the others' launches
// fill the idle SMs.  Results do not depend on it.
static int launch_mh_jumps(rd_engine* e, const Sig& s, cudaStream_t main) {
  const int prec = e->cfg.precision;
  const int parts = mh_parts_for(e, s), form = mh_form_for(e, s);
  int rc = mh_fork(e, parts, main);
  if (rc) return rc;
  for (int it = 1; it <= s.jumps; ++it) {
    if (s.emit_planar) {
      if ((rc = planar_mh_launch(e, s, it, parts, form, main))) return rc;
      e->kernels_in_step += parts;
    }
    if (s.emit_tip) {   // tip propose + jump
      CK(rd_launch_mh_jump(prec, 2, e->grid, main, e->dP, e->dD, e->pool, e->plan[PM_MH], e->ph[PM_MH], e->cs,
                           e->d_choff, e->wtab, e->d_step, it, e->partial, e->tickets, e->kscale, e->item_queue));
      e->kernels_in_step += 2;
    }
  }
  return mh_join(e, parts, main);
}

// The tiled MH chains of a step on stream `main`: round 0 of the start (tiled
// like a jump), k_mh_init for the rest of the start, then the jumps.
static int launch_mh_tiled(rd_engine* e, const Sig& s, cudaStream_t main) {
  const int prec = e->cfg.precision;
  const int gmask = (s.emit_planar ? 1 : 0) | (s.emit_tip ? 2 : 0);
  CK(rd_launch_mh_jump(prec, gmask, e->grid, main, e->dP, e->dD, e->pool, e->plan[PM_MH], e->ph[PM_MH],
                       e->cs, e->d_choff, e->wtab, e->d_step, 0, e->partial, e->tickets, e->kscale, e->item_queue,
                       0, 1, mh_form_for(e, s)));
  e->kernels_in_step += ((gmask & 1) ? 1 : 0) + ((gmask & 2) ? 2 : 0);
  CK(rd_launch_mh_init(prec, e->grid, main, e->dP, e->dD, e->pool, e->plan[PM_MH], e->ph[PM_MH],
                       e->cs, e->d_choff, e->wtab, e->d_step, e->kscale));
  e->kernels_in_step++;
  return launch_mh_jumps(e, s, main);
}

// Inside a stream capture, for a lone emitting planar diode: the tiled MH
// chains as the body of a conditional (IF) graph node, which a one-thread
// kernel switches on only when the MH plan has work items.  A step whose diode
// samples the vacuum field (k_mh_vacuum) -- or has no chain at all -- then
// skips the start and jump launches entirely.  The body is captured on stream
// e->sbody.
static int launch_mh_tiled_if(rd_engine* e, const Sig& s) {
  cudaStreamCaptureStatus cst;
  cudaGraph_t cap = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  CK(cudaStreamGetCaptureInfo(e->st, &cst, nullptr, &cap, nullptr, nullptr, nullptr));
  // Only a lone emitting planar diode (the one-diode deck) gains: with two or more, every
  // one would have to be empty.  Elsewhere the plain launches are kept, which also keeps
  // the step graph's kernels visible one by one to a profiler (ncu does not profile the
  // kernel nodes of a graph that holds a conditional node).
  if (cst != cudaStreamCaptureStatusActive || s.mh_planar > 1 || s.emit_tip) return launch_mh_tiled(e, s, e->st);
  cudaGraphConditionalHandle h;
  CK(cudaGraphConditionalHandleCreate(&h, cap, 0, cudaGraphCondAssignDefault));
  CK(rd_launch_mh_cond(e->st, h, e->ph[PM_MH]));
  e->kernels_in_step++;
  CK(cudaStreamGetCaptureInfo(e->st, &cst, nullptr, &cap, &deps, nullptr, &ndeps));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeIf;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, cap, deps, nullptr, ndeps, &cp));
  CK(cudaStreamUpdateCaptureDependencies(e->st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  CK(cudaStreamBeginCaptureToGraph(e->sbody, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  int rc = launch_mh_tiled(e, s, e->sbody);
  cudaGraph_t done = nullptr;
  cudaError_t ce = cudaStreamEndCapture(e->sbody, &done);
  if (rc) return rc;
  CK(ce);
  return RD_OK;
}

static int launch_emission(rd_engine* e) {
  Sig s = signature(e);
  if (!s.emit_planar && !s.emit_tip) return RD_OK;
  const int prec = e->cfg.precision;
  const int ns = e->nslots_hw();
  if (s.emit_planar) {
    CK(plan(e, PM_SUPPLY_PLANAR));
    CK(rd_launch_z0_points(prec, e->grid, e->st, e->dP, e->pool, e->plan[PM_SUPPLY_PLANAR],
                           e->ph[PM_SUPPLY_PLANAR], e->qx, e->qy, e->qpp, e->qF, e->partial, e->tickets,
                           e->kscale, e->item_queue + 6));
    e->kernels_in_step++;
  }
  if (s.emit_lat) {   // planar diodes without image charges: all three components at the points
    CK(plan(e, PM_SUPPLY_LAT));
    PointSet lp{e->qx, e->qy, e->qz, e->qfx, e->qfy, e->qF, e->d_qoff};
    CK(rd_launch_field_points(prec, RD_G_PLANAR, e->grid, e->st, e->dP, e->pool, e->plan[PM_SUPPLY_LAT],
                              e->ph[PM_SUPPLY_LAT], lp, e->partial, e->tickets, e->kscale));
    e->kernels_in_step++;
  }
  if (s.emit_tip) {
    CK(plan(e, PM_SUPPLY_TIP));
    PointSet pts{e->qx, e->qy, e->qz, e->qfx, e->qfy, e->qF, e->d_qoff};
    CK(rd_launch_field_points(prec, RD_G_TIP, e->grid, e->st, e->dP, e->pool, e->plan[PM_SUPPLY_TIP],
                              e->ph[PM_SUPPLY_TIP], pts, e->partial, e->tickets, e->kscale));
    e->kernels_in_step++;
  }
  CK(rd_launch_supply_reduce(ns, e->st, e->dP, e->dD, e->qx, e->qy, e->qw, e->qF, e->qfx, e->qfy,
                             e->work, e->d_step, e->sup_part));
  e->kernels_in_step += 2;
  CK(plan(e, PM_MH));
  if (s.emit_planar) {   // diodes with no particle in flight: all their MH sampling in one launch
    CK(rd_launch_mh_vacuum(prec, ns, e->st, e->dP, e->dD, e->cs, e->d_choff, e->wtab, e->d_step, e->kscale));
    e->kernels_in_step += 2;   // uniform work functions, and the others
  }
  int rc = launch_mh_tiled_if(e, s);
  if (rc) return rc;
  CK(rd_launch_emit(ns, e->st, e->dP, e->dD, e->pool, e->cs, e->d_choff, e->work, e->d_step, e->evlog));
  e->kernels_in_step += 2;
  if (s.emit_serial) {   // serial MH diodes: chains one after another, one block per diode
    CK(rd_launch_mh_serial(prec, ns, e->st, e->dP, e->dD, e->pool, e->work, e->wtab, e->d_step, e->kscale,
                           e->evlog));
    e->kernels_in_step += 2;   // the parallel pass for empty diodes, and the serial kernel
  }
  return RD_OK;
}

// The acceleration pass.  In a time step (step_pass) two-time-step diodes
// take k_force_tts (Update_Particle_Acceleration, src/mod_verlet.F90:886-897);
// otherwise every diode takes the plain pass (Calculate_Acceleration_Particles,
// which does not look at two_time_step), which is also idempotent for timing.
static int launch_force(rd_engine* e, bool step_pass = false) {
  Sig s = signature(e);
  const int all = step_pass ? 0 : PM_ALL_DIODES;
  if (s.planar) {
    CK(plan(e, PM_FORCE_PLANAR | all));
    CK(rd_launch_force(e->cfg.precision, 1, s.nic ? 1 : 0, e->grid, e->st, e->dP, e->dD, e->pool,
                       e->plan[PM_FORCE_PLANAR], e->ph[PM_FORCE_PLANAR], e->partial, e->tickets,
                       e->kscale, e->item_queue + 4));
    e->kernels_in_step++;
  }
  if (s.tip) {
    CK(plan(e, PM_FORCE_TIP | all));
    CK(rd_launch_force(e->cfg.precision, 2, 0, e->grid, e->st, e->dP, e->dD, e->pool,
                       e->plan[PM_FORCE_TIP], e->ph[PM_FORCE_TIP], e->partial, e->tickets,
                       e->kscale, e->item_queue + 4));
    e->kernels_in_step++;
  }
  if (step_pass && s.tts) {
    CK(plan(e, PM_FORCE_TTS));
    CK(rd_launch_force_tts(e->grid, e->st, e->dP, e->dD, e->pool, e->plan[PM_FORCE_TTS], e->ph[PM_FORCE_TTS],
                           e->partial, e->tickets, e->item_queue + 4, e->d_step));
    e->kernels_in_step++;
  }
  return RD_OK;
}

static int launch_update_position(rd_engine* e) {
  const int ns = e->nslots_hw();
  CK(plan(e, PM_PART));
  CK(rd_launch_position(e->grid, e->st, e->dP, e->dD, e->pool, e->plan[PM_PART], e->ph[PM_PART], e->evlog,
                        e->d_step));
  e->kernels_in_step++;
  int rc = launch_force(e, true);
  if (rc) return rc;
  CK(rd_launch_velocity(e->grid, ns, e->st, e->dP, e->dD, e->pool, e->plan[PM_PART], e->ph[PM_PART],
                        e->ramo, e->d_step));
  e->kernels_in_step += 2;
  return RD_OK;
}

// Waits of the in-place compaction (k_compact_move) that gave up: each is a
// tile that stored nothing, so the particle state is no longer valid.  Read
// after the engine stream has drained.
static int compaction_check(rd_engine* e) {
  int bad = 0;
  CK(cudaMemcpyAsync(&bad, e->cq + 2, sizeof(int), cudaMemcpyDeviceToHost, e->st));
  CK(cudaStreamSynchronize(e->st));
  if (bad) return fail(RD_ERR_STATE, "compaction: a wait on an earlier tile gave up; the particle state is not valid");
  return RD_OK;
}

static int launch_remove(rd_engine* e) {
  CK(plan(e, PM_PART1024));
  CK(rd_launch_compact(e->grid, e->nslots_hw(), e->st, e->dP, e->dD, e->pool, e->plan[PM_PART1024],
                       e->ph[PM_PART1024], e->ccnt, e->cpre, e->cflag, e->cq, e->life, e->d_step));
  e->kernels_in_step += 4;
  return RD_OK;
}

static int launch_step_body(rd_engine* e) {
  e->kernels_in_step = 0;
  int rc = launch_emission(e);
  if (rc) return rc;
  rc = launch_update_position(e);
  if (rc) return rc;
  rc = launch_remove(e);
  if (rc) return rc;
  CK(rd_launch_step_inc(e->st, e->d_step));
  e->kernels_in_step++;
  return RD_OK;
}

static std::string sig_string(rd_engine* e) {
  Sig s = signature(e);
  char b[128];
  snprintf(b, sizeof b, "%d%d%d%d%d%d%d%d%d:%d:%d:%d:%d:%d", s.planar, s.tip, s.emit_planar, s.emit_tip, s.nic,
           s.emit_serial, s.tts, s.mh_planar > 1 ? 2 : s.mh_planar, s.emit_lat, s.jumps, e->clen_min, e->nch_max,
           mh_parts_for(e, s), mh_form_for(e, s));
  return b;
}

static int ensure_graph(rd_engine* e) {
  std::string sig = sig_string(e);
  if (e->graph && sig == e->graph_sig) return RD_OK;
  if (e->graph) { cudaGraphExecDestroy(e->graph); e->graph = nullptr; }
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal));
  int rc = launch_step_body(e);
  cudaError_t ce = cudaStreamEndCapture(e->st, &g);
  if (rc) { if (ce == cudaSuccess) cudaGraphDestroy(g); return rc; }
  CK(ce);
  cudaError_t ie = cudaGraphInstantiate(&e->graph, g, 0);
  cudaGraphDestroy(g);
  CK(ie);
  e->graph_sig = sig;
  e->last_kernels = e->kernels_in_step;
  return RD_OK;
}

static int repack(rd_engine* e) {
  CK(plan(e, PM_PART));
  CK(rd_launch_pack(e->grid, e->st, e->dP, e->pool, e->plan[PM_PART], e->ph[PM_PART]));
  return RD_OK;
}

static int stage(rd_engine* e, long long doubles, long long ints) {
  long long need = std::max(doubles, ints);
  if (need <= e->stage_cap) return RD_OK;
  CK(cudaStreamSynchronize(e->st));
  if (e->stage_d) cudaFree(e->stage_d);
  if (e->stage_i) cudaFree(e->stage_i);
  if (e->stage_hd) cudaFreeHost(e->stage_hd);
  if (e->stage_hi) cudaFreeHost(e->stage_hi);
  e->stage_d = nullptr; e->stage_i = nullptr; e->stage_hd = nullptr; e->stage_hi = nullptr;
  e->stage_cap = 0;
  long long cap = std::max<long long>(need, 1 << 16);
  CK(cudaMalloc(&e->stage_d, cap * sizeof(double)));
  CK(cudaMalloc(&e->stage_i, cap * sizeof(int)));
  CK(cudaHostAlloc(&e->stage_hd, cap * sizeof(double), cudaHostAllocDefault));
  CK(cudaHostAlloc(&e->stage_hi, cap * sizeof(int), cudaHostAllocDefault));
  e->stage_cap = cap;
  return RD_OK;
}

static bool valid_diode(rd_engine* e, int d) {
  return e && d >= 0 && d < (int)e->slots.size() && e->slots[d].used;
}

// ---- helpers for rd_noalloc.cu (C++ linkage, not part of the C ABI) -----------------
int rd_set_error(int code, const char* msg) { return fail(code, msg); }
int rd_noalloc_prepare(int device, int prec);   // rd_noalloc.cu

int rd_engine_view(rd_engine* e, int diode, const DiodeParams** P, const DiodeDyn** Dy, Pool* pool,
                   int* geometry, int* precision, int* grid, double* kscale, cudaStream_t* st,
                   int* device) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  if (!valid_diode(e, diode)) return fail(RD_ERR_NOTFOUND, "unknown diode");
  *P = e->dP + diode;
  *Dy = e->dD + diode;
  *pool = e->pool;
  *geometry = e->slots[diode].p.geometry;
  *precision = e->cfg.precision;
  *grid = e->grid;
  *kscale = e->kscale;
  *st = e->st;
  *device = e->cfg.device;
  return RD_OK;
}

int rd_engine_repack(rd_engine* e) { return repack(e); }
int rd_engine_chunk_rule(rd_engine* e) { return rd_chunk_rule(e->clen_min, e->nch_max); }

// ---- C ABI ----------------------------------------------------------------------------
extern "C" {

const char* rd_last_error(void) { return g_err.c_str(); }
int rd_version(void) { return 10000; }

int rd_engine_create(const rd_engine_config* cfg, rd_engine** out) {
  if (!cfg || !out) return fail(RD_ERR_INVALID, "null argument");
  if (cfg->max_diodes <= 0 || cfg->particle_capacity <= 0)
    return fail(RD_ERR_INVALID, "max_diodes and particle_capacity must be positive");
  if (cfg->precision != RD_PREC_FP64 && cfg->precision != RD_PREC_FP32C)
    return fail(RD_ERR_INVALID, "unknown precision");
  if (!valid_chunking(cfg->chunk_min > 0 ? cfg->chunk_min : RD_CLEN_MIN,
                      cfg->chunk_count_max > 0 ? cfg->chunk_count_max : RD_NCH_MAX))
    return fail(RD_ERR_INVALID, "chunk_min must be a multiple of 128 in [128, 65536], chunk_count_max in [1, 32]");
  rd_engine* e = new rd_engine();
  e->cfg = *cfg;
  int rc = RD_OK;
  auto bail = [&](int code) { rd_engine_destroy(e); return code; };
  cudaError_t ce = cudaSetDevice(cfg->device);
  if (ce != cudaSuccess) return bail(fail(RD_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(ce)));
  cudaDeviceProp prop;
  ce = cudaGetDeviceProperties(&prop, cfg->device);
  if (ce != cudaSuccess) return bail(fail(RD_ERR_CUDA, cudaGetErrorString(ce)));
  e->sms = prop.multiProcessorCount;
  e->grid = cfg->grid_blocks > 0 ? cfg->grid_blocks : 0;   // 0: occupancy-based per kernel
  e->clen_min = cfg->chunk_min > 0 ? cfg->chunk_min : RD_CLEN_MIN;
  e->nch_max = cfg->chunk_count_max > 0 ? cfg->chunk_count_max : RD_NCH_MAX;
  if ((ce = cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking)) != cudaSuccess ||
      (ce = cudaEventCreateWithFlags(&e->ev_fork, cudaEventDisableTiming)) != cudaSuccess)
    return bail(fail(RD_ERR_CUDA, cudaGetErrorString(ce)));
  for (int q = 1; q < RD_MH_PARTS_MAX; ++q)
    if ((ce = cudaStreamCreateWithFlags(&e->stp[q], cudaStreamNonBlocking)) != cudaSuccess ||
        (ce = cudaEventCreateWithFlags(&e->ev_join[q], cudaEventDisableTiming)) != cudaSuccess)
      return bail(fail(RD_ERR_CUDA, cudaGetErrorString(ce)));
  cudaEventCreate(&e->ev0);
  cudaEventCreate(&e->ev1);
  if ((ce = cudaStreamCreateWithFlags(&e->sa, cudaStreamNonBlocking)) != cudaSuccess ||
      (ce = cudaStreamCreateWithFlags(&e->sbody, cudaStreamNonBlocking)) != cudaSuccess ||
      (ce = cudaEventCreateWithFlags(&e->ev_adm, cudaEventDisableTiming)) != cudaSuccess ||
      (ce = cudaHostAlloc((void**)&e->act_P, sizeof(DiodeParams) * cfg->max_diodes, cudaHostAllocDefault)) != cudaSuccess ||
      (ce = cudaHostAlloc((void**)&e->act_D, sizeof(DiodeDyn) * cfg->max_diodes, cudaHostAllocDefault)) != cudaSuccess ||
      (ce = cudaHostAlloc((void**)&e->act_choff, sizeof(int) * cfg->max_diodes, cudaHostAllocDefault)) != cudaSuccess ||
      (ce = cudaHostAlloc((void**)&e->act_qoff, sizeof(int) * cfg->max_diodes, cudaHostAllocDefault)) != cudaSuccess)
    return bail(fail(RD_ERR_CUDA, cudaGetErrorString(ce)));
  e->k = make_constants();
  e->kscale = e->k.div_fac_c * e->k.q0 * 1.0e18;
  if (rd_upload_constants_force(e->k) != cudaSuccess || rd_upload_constants_field(e->k) != cudaSuccess ||
      rd_upload_constants_step(e->k) != cudaSuccess)
    return bail(fail(RD_ERR_CUDA, "constant upload failed"));
  const long long cap = cfg->particle_capacity;
  const int S = cfg->max_diodes;
  const long long chcap = std::max<long long>(cfg->chain_capacity, 1);
  const long long qcap = std::max<long long>(cfg->quad_capacity, 1);
  // scratch bound: at most RD_NCH_MAX chunks per tile (RD_SUP_NCH for the
  // planar supply points) and at most capacity/128 + slots tiles in any pair sum
  e->max_items = (int)std::min<long long>(
      1 << 26, std::max((long long)RD_NCH_MAX * (std::max(cap, chcap) / RD_ITILE + 4LL * S),
                        (long long)RD_SUP_NCH * (qcap / RD_ITILE + 4LL * S)) + 65536);
  // compaction units: four per 1024-particle tile, at most capacity/1024 + slots tiles
  const size_t cunits = 4 * ((size_t)cap / 1024 + (size_t)S + 1);
  if ((rc = alloc_pool(e, e->pool, cap))) return bail(rc);
  if (e->dalloc(&e->save_ax, cap) || e->dalloc(&e->save_ay, cap) || e->dalloc(&e->save_az, cap))
    return bail(fail(RD_ERR_NOMEM, "device allocation failed"));
  if (e->dalloc(&e->dP, S) || e->dalloc(&e->dD, S) || e->dalloc(&e->work, (size_t)S * 4 + 4096) || e->dalloc(&e->wtab, 3 * ((size_t)S * 4 + 4096)) ||
      e->dalloc(&e->qx, qcap) || e->dalloc(&e->qy, qcap) || e->dalloc(&e->qz, qcap) ||
      e->dalloc(&e->qw, qcap) || e->dalloc(&e->qF, qcap) || e->dalloc(&e->qfx, qcap) ||
      e->dalloc(&e->qfy, qcap) || e->dalloc(&e->qpp, qcap) || e->dalloc(&e->cs.gx, chcap) || e->dalloc(&e->cs.gy, chcap) ||
      e->dalloc(&e->cs.fx, chcap) || e->dalloc(&e->cs.fy, chcap) || e->dalloc(&e->cs.fsup, chcap) ||
      e->dalloc(&e->cs.fF, chcap) ||
      e->dalloc(&e->cs.fgx, chcap) || e->dalloc(&e->cs.fgy, chcap) ||
      e->dalloc(&e->cs.pph, chcap) || e->dalloc(&e->cs.pih, chcap) ||
      e->dalloc(&e->d_choff, S) || e->dalloc(&e->d_qoff, S) ||
      e->dalloc(&e->d_npts, S) || e->dalloc(&e->d_zero_off, S) ||
      e->dalloc(&e->partial, (size_t)e->max_items * 3 * RD_ITILE) ||
      e->dalloc(&e->tickets, e->max_items) ||
      e->dalloc(&e->ccnt, cunits) || e->dalloc(&e->cpre, cunits) || e->dalloc(&e->cflag, cunits) ||
      e->dalloc(&e->cq, 4) ||
      e->dalloc(&e->sup_part, (size_t)S * RD_SUP_SPLIT * 4) ||
      e->dalloc(&e->item_queue, 8 + 2 * RD_MH_PARTS_MAX) ||
      (cfg->event_capacity > 0 && (e->dalloc(&e->evlog.buf, (size_t)cfg->event_capacity) ||
                                   e->dalloc(&e->evlog.count, 1))) ||
      e->dalloc(&e->ramo, ((size_t)cap / RD_ITILE + S + 1) * 10) || e->dalloc(&e->life, (size_t)S * RD_MAX_LIFE) ||
      e->dalloc(&e->d_step, 1))
    return bail(fail(RD_ERR_NOMEM, "device allocation failed"));
  double** chd[] = {&e->cs.x, &e->cs.y, &e->cs.F, &e->cs.sup, &e->cs.df, &e->cs.px, &e->cs.py,
                    &e->cs.pF, &e->cs.tx, &e->cs.ty, &e->cs.tz, &e->cs.pxx, &e->cs.pyy, &e->cs.pzz};
  for (auto p : chd) if (e->dalloc(p, chcap)) return bail(fail(RD_ERR_NOMEM, "chain pool allocation failed"));
  if (e->dalloc(&e->cs.ok, chcap) || e->dalloc(&e->cs.prop_ok, chcap) || e->dalloc(&e->cs.em, chcap))
    return bail(fail(RD_ERR_NOMEM, "chain pool allocation failed"));
  for (int m = 0; m < PM_COUNT; ++m)
    if (e->dalloc(&e->plan[m], S) || e->dalloc(&e->ph[m], 1))
      return bail(fail(RD_ERR_NOMEM, "plan allocation failed"));
  cudaMemsetAsync(e->dP, 0, sizeof(DiodeParams) * S, e->st);
  cudaMemsetAsync(e->dD, 0, sizeof(DiodeDyn) * S, e->st);
  cudaMemsetAsync(e->tickets, 0, sizeof(int) * e->max_items, e->st);
  cudaMemsetAsync(e->cq, 0, sizeof(int) * 4, e->st);
  cudaMemsetAsync(e->item_queue, 0, sizeof(int) * (8 + 2 * RD_MH_PARTS_MAX), e->st);
  if (e->evlog.count) cudaMemsetAsync(e->evlog.count, 0, sizeof(int), e->st);
  e->evlog.cap = cfg->event_capacity > 0 ? cfg->event_capacity : 0;
  cudaMemsetAsync(e->life, 0, sizeof(int) * (size_t)S * RD_MAX_LIFE, e->st);
  cudaMemsetAsync(e->d_npts, 0, sizeof(int) * S, e->st);
  cudaMemsetAsync(e->d_zero_off, 0, sizeof(int) * S, e->st);
  cudaMemsetAsync(e->d_step, 0, sizeof(int), e->st);
  cudaMemsetAsync(e->pool.mask, 0, sizeof(int) * cap, e->st);
  if ((ce = cudaStreamSynchronize(e->st)) != cudaSuccess) return bail(fail(RD_ERR_CUDA, cudaGetErrorString(ce)));
  e->slots.resize(S);
  e->pool_alloc.init(cap);
  e->ch_alloc.init(chcap);
  e->q_alloc.init(qcap);
  e->w_alloc.init((long long)S * 4 + 4096);
  // load rd_field_at_noalloc's module and kernels now, so that its calls commit no memory
  if ((rc = rd_noalloc_prepare(cfg->device, cfg->precision))) return bail(rc);
  *out = e;
  return RD_OK;
}

int rd_engine_destroy(rd_engine* e) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  if (!e) return RD_OK;
  if (e->st) cudaStreamSynchronize(e->st);
  if (e->graph) cudaGraphExecDestroy(e->graph);
  for (void* p : e->allocs) cudaFree(p);
  if (e->stage_d) cudaFree(e->stage_d);
  if (e->stage_i) cudaFree(e->stage_i);
  if (e->stage_hd) cudaFreeHost(e->stage_hd);
  if (e->stage_hi) cudaFreeHost(e->stage_hi);
  if (e->fpx) { cudaFree(e->fpx); cudaFree(e->fpy); cudaFree(e->fpz); cudaFree(e->ffx); cudaFree(e->ffy); cudaFree(e->ffz); }
  if (e->ev0) cudaEventDestroy(e->ev0);
  if (e->ev1) cudaEventDestroy(e->ev1);
  if (e->sa) { cudaStreamSynchronize(e->sa); cudaStreamDestroy(e->sa); }
  if (e->sbody) cudaStreamDestroy(e->sbody);
  if (e->ev_adm) cudaEventDestroy(e->ev_adm);
  if (e->adm_h) cudaFreeHost(e->adm_h);
  if (e->adm_d) cudaFree(e->adm_d);
  if (e->act_P) cudaFreeHost(e->act_P);
  if (e->act_D) cudaFreeHost(e->act_D);
  if (e->act_choff) cudaFreeHost(e->act_choff);
  if (e->act_qoff) cudaFreeHost(e->act_qoff);
  if (e->ev_fork) cudaEventDestroy(e->ev_fork);
  for (int q = 1; q < RD_MH_PARTS_MAX; ++q) {
    if (e->ev_join[q]) cudaEventDestroy(e->ev_join[q]);
    if (e->stp[q]) cudaStreamDestroy(e->stp[q]);
  }
  if (e->st) cudaStreamDestroy(e->st);
  delete e;
  return RD_OK;
}

int rd_sync(rd_engine* e) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  if (!e) return fail(RD_ERR_INVALID, "null engine");
  CK(cudaStreamSynchronize(e->st));
  return RD_OK;
}

// Admission arena: host bytes staged in pinned memory for an upload on sa.
// The previous batch's copies are waited for before the arena is reused.
static cudaError_t adm_grow(rd_engine* e, size_t need) {
  cudaError_t ce = cudaStreamSynchronize(e->sa);
  if (ce != cudaSuccess) return ce;
  if (need <= e->adm_cap) return cudaSuccess;
  if (e->adm_h) cudaFreeHost(e->adm_h);
  if (e->adm_d) cudaFree(e->adm_d);
  e->adm_h = nullptr; e->adm_d = nullptr; e->adm_cap = 0; e->adm_used = 0;
  const size_t cap = std::max<size_t>(need, 2 * (size_t)(1 << 20));
  if ((ce = cudaHostAlloc((void**)&e->adm_h, cap, cudaHostAllocDefault)) != cudaSuccess) return ce;
  if ((ce = cudaMalloc((void**)&e->adm_d, cap)) != cudaSuccess) return ce;
  e->adm_cap = cap;
  return cudaSuccess;
}

// Room for `bytes` in the admission arena: offset of the region (host and device alike).
static cudaError_t adm_take(rd_engine* e, size_t bytes, size_t* off) {
  const size_t len = (bytes + 255) & ~(size_t)255;
  if (e->adm_used + len > e->adm_cap) {
    cudaError_t ce = adm_grow(e, std::max(e->adm_cap * 2, e->adm_used + len));
    if (ce != cudaSuccess) return ce;
    // adm_grow waited for every copy from the arena: what was taken is free again unless kept
  }
  *off = e->adm_used;
  e->adm_used += len;
  return cudaSuccess;
}

// Host -> device copy on stream us: staged through the pinned admission arena
// when `deferred` (nothing waits, the source may go away at once), directly
// from the (pageable) source otherwise (the caller synchronises us).
static cudaError_t upload(rd_engine* e, void* dst, const void* src, size_t bytes, cudaStream_t us, bool deferred) {
  if (bytes == 0) return cudaSuccess;
  if (!deferred) return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, us);
  size_t off = 0;
  cudaError_t ce = adm_take(e, bytes, &off);
  if (ce != cudaSuccess) return ce;
  std::memcpy(e->adm_h + off, src, bytes);
  return cudaMemcpyAsync(dst, e->adm_h + off, bytes, cudaMemcpyHostToDevice, us);
}

// Makes the slots admitted on sa active on the engine stream: the stream waits
// for sa's uploads, then each slot's parameters (active) are copied in.  The
// next step on the engine stream includes them.
static int activate_pending(rd_engine* e) {
  if (e->pending.empty()) return RD_OK;
  CK(cudaEventRecord(e->ev_adm, e->sa));
  CK(cudaStreamWaitEvent(e->st, e->ev_adm, 0));
  for (int s : e->pending)
    CK(cudaMemcpyAsync(e->dP + s, &e->act_P[s], sizeof(DiodeParams), cudaMemcpyHostToDevice, e->st));
  e->pending.clear();
  return RD_OK;
}

// Completes any admission still in flight (entry points that touch device state call it).
static int flush_admissions(rd_engine* e) {
  if (e->pending.empty()) return RD_OK;
  int rc = activate_pending(e);
  if (rc) return rc;
  CK(cudaStreamSynchronize(e->st));
  return RD_OK;
}

// rd_diode_add on stream `us`.  deferred: the slot is written inactive and
// its parameters are kept for activate_pending(), which makes it active on the
// engine stream before the next step; nothing here waits for the GPU, so the
// uploads overlap a step running on the engine stream (which skips inactive
// slots).  Otherwise the slot is active when the call returns.
static int diode_add_impl(rd_engine* e, const rd_diode_config* c, int* diode, cudaStream_t us, bool deferred,
                          int step_offset = 0) {
  if (!e || !c || !diode) return fail(RD_ERR_INVALID, "null argument");
  if (c->geometry != RD_GEOM_PLANAR && c->geometry != RD_GEOM_TIP) return fail(RD_ERR_INVALID, "unknown geometry");
  if (c->capacity <= 0 || c->time_step <= 0.0) return fail(RD_ERR_INVALID, "capacity and time_step must be positive");
  if (c->N_ic_max < 0 || c->N_ic_max > 64) return fail(RD_ERR_INVALID, "N_ic_max out of range");
  int s = -1;
  for (size_t k = 0; k < e->slots.size(); ++k) if (!e->slots[k].used) { s = (int)k; break; }
  if (s < 0) return fail(RD_ERR_CAPACITY, "no free diode slot");
  DiodeParams p{};
  p.active = 1;
  p.geometry = c->geometry;
  p.cap = c->capacity;
  p.image_charge = c->image_charge ? 1 : 0;
  p.N_ic_max = c->N_ic_max;
  p.emission = c->emission ? 1 : 0;
  p.V = c->V_s;
  p.dt = c->time_step;
  p.dt2 = c->time_step * c->time_step;
  p.seed = c->seed;
  p.emit_delay = c->emitter_delay > 0 ? c->emitter_delay : 0;
  p.mh_serial = c->mh_serial ? 1 : 0;
  p.emitter_type = 2;
  if (c->planes_N < 0 || c->planes_N > 10) return fail(RD_ERR_INVALID, "planes_N must be in [0, 10]");
  p.planes_n = c->planes_N;
  for (int k = 0; k < p.planes_n; ++k) p.planes_z[k] = c->planes_z[k];
  if (c->atom_time_interval < 0) return fail(RD_ERR_INVALID, "atom_time_interval must be >= 0");
  p.tts = c->atom_time_interval;
  p.init_rounds = c->init_rounds > 0 ? c->init_rounds : 10000;
  p.work_nx = p.work_ny = 1;
  p.work_model = 1;
  if (c->geometry == RD_GEOM_PLANAR) {
    if (c->gap <= 0.0) return fail(RD_ERR_INVALID, "gap must be positive");
    p.d = c->gap;
    p.E_z = -1.0 * c->V_s / p.d;                   // Set_Voltage :2050-2052
    p.em_x0 = c->emitter_pos[0]; p.em_y0 = c->emitter_pos[1];
    p.em_Lx = c->emitter_dim[0]; p.em_Ly = c->emitter_dim[1];
    if (p.emission && (p.em_Lx <= 0.0 || p.em_Ly <= 0.0)) return fail(RD_ERR_INVALID, "emitter_dim must be positive");
    p.org_x = p.em_x0 + 0.5 * p.em_Lx;
    p.org_y = p.em_y0 + 0.5 * p.em_Ly;
    p.emitter_type = c->emitter_type > 0 ? c->emitter_type : 2;
    if (p.emitter_type != 1 && p.emitter_type != 2 && p.emitter_type != 4)
      return fail(RD_ERR_INVALID, "emitter_type must be 1 (circle), 2 (rectangle) or 4 (ring)");
    if (p.emitter_type == 4) {   // emitters_ring (src/main.F90:363-371), centred on the axis
      p.ring_thick = c->emitter_thickness > 0.0
                         ? c->emitter_thickness
                         : std::sqrt((e->k.q0 * p.d) / (e->k.pi * e->k.eps0 * c->V_s));
      p.ring_rmin = p.em_Lx - p.ring_thick;
      if (p.ring_thick <= 0.0 || p.ring_rmin < 0.0)
        return fail(RD_ERR_INVALID, "ring emitter: emitter_dim[0] (outer radius) must exceed its thickness");
      p.org_x = 0.0;
      p.org_y = 0.0;
      p.mh_serial = 1;
    }
    p.em_hx = f32_toward_zero(0.5 * p.em_Lx * 1.0e9);
    p.em_hy = f32_toward_zero(0.5 * p.em_Ly * 1.0e9);
    p.em_wx = (float)(p.em_Lx * 1.0e9);
    p.em_wy = (float)(p.em_Ly * 1.0e9);
    p.mh_jumps = c->mh_jumps > 0 ? c->mh_jumps : 200;   // MH_ndim, fe_v2:70
    p.mh_lo = 0.00005; p.mh_hi = 0.1250;                 // fe_v2:75-76
    p.work_model = c->work_model > 0 ? c->work_model : 1;
    if (p.work_model != 1 && p.work_model != 2 && p.work_model != 4)
      return fail(RD_ERR_INVALID, "work_model must be 1 (checkerboard), 2 (Gaussian) or 4 (Voronoi)");
    if (p.work_model == 1) {
      if (c->work_nx > 0 && c->work_ny > 0 && c->work) { p.work_nx = c->work_nx; p.work_ny = c->work_ny; }
    } else {
      if (!c->work || c->work_nx < (p.work_model == 4 ? 1 : 0))
        return fail(RD_ERR_INVALID, "the Gaussian / Voronoi work function needs its parameters (work, work_nx)");
      p.work_nx = c->work_nx;
      p.work_ny = 1;
    }
  } else {
    // Init_Emission_Tip, src/mod_emission_tip.f90:81-127
    double dt_ = c->tip_dim[0], Rb = c->tip_dim[1], ht = c->tip_dim[2];
    if (dt_ <= 0.0 || Rb <= 0.0 || ht <= 0.0) return fail(RD_ERR_INVALID, "tip_dim must be positive");
    p.d = dt_ + ht;
    p.h_tip = ht;
    p.max_xi = ht / dt_ + 1.0;
    p.a_foci = std::sqrt(((dt_ * dt_) * (Rb * Rb)) / ((ht * ht) + (2.0 * dt_) * ht) + dt_ * dt_);
    p.eta_1 = -1.0 * dt_ / p.a_foci;
    double theta = std::acos(dt_ / p.a_foci);
    p.r_tip = (p.a_foci * std::sin(theta)) * std::tan(theta);
    p.shift_z = std::fabs((p.a_foci * p.eta_1) * p.max_xi);
    double pre = std::log((((1.0 + p.eta_1) / (1.0 - p.eta_1)) * (1.0 - 0.0)) / (1.0 + 0.0));
    p.pre_E_unit = (2.0 * 1.0) / (p.a_foci * pre);
    p.pre_E = (2.0 * c->V_s) / (p.a_foci * pre);
    p.tip_phi = c->tip_work_function > 0.0 ? c->tip_work_function : 4.7;
    p.org_x = 0.0; p.org_y = 0.0;
    p.mh_jumps = c->mh_jumps > 0 ? c->mh_jumps : 80;     // ndim, emission_tip:506
    p.mh_lo = 0.0005; p.mh_hi = 0.125;                   // emission_tip:62-63
  }
  p.ramo_uz = -1.0 / p.d;   // E_zunit_planar, once per diode
  SlotHost sl;
  sl.pool_len = p.cap;
  sl.pool_off = e->pool_alloc.alloc(sl.pool_len, 32);
  if (sl.pool_off < 0) return fail(RD_ERR_CAPACITY, "particle pool full");
  p.off = (int)sl.pool_off;
  auto undo = [&]() {
    e->pool_alloc.release(sl.pool_off, sl.pool_len);
    if (sl.ch_len) e->ch_alloc.release(sl.ch_off, sl.ch_len);
    if (sl.q_len) e->q_alloc.release(sl.q_off, sl.q_len);
    if (sl.w_len) e->w_alloc.release(sl.w_off, sl.w_len);
  };
  // work function table: checkerboard values, Gaussian parameters or Voronoi sites
  sl.w_len = (long long)p.work_nx * p.work_ny;
  if (p.work_model == 2) sl.w_len = 1 + 5LL * p.work_nx;
  if (p.work_model == 4) sl.w_len = 4LL * p.work_nx;
  sl.w_off = e->w_alloc.alloc(sl.w_len, 1);
  if (sl.w_off < 0) { sl.w_len = 0; undo(); return fail(RD_ERR_CAPACITY, "work-function table full"); }
  p.work_off = (int)sl.w_off;
  p.work_data = e->work + sl.w_off;
  std::vector<double> wv(sl.w_len, 4.7);
  if (c->geometry == RD_GEOM_PLANAR && c->work && (p.work_model != 1 || (c->work_nx > 0 && c->work_ny > 0)))
    for (long long k2 = 0; k2 < sl.w_len; ++k2) wv[k2] = c->work[k2];
  if (p.emission) {
    p.max_chains = c->max_chains > 0 ? c->max_chains : p.cap;
    sl.ch_len = p.max_chains;
    sl.ch_off = e->ch_alloc.alloc(sl.ch_len, 32);
    if (sl.ch_off < 0) { sl.ch_len = 0; undo(); return fail(RD_ERR_CAPACITY, "MH chain pool full"); }
    int npt;
    int P_ = 0, Q = 4;
    if (c->geometry == RD_GEOM_PLANAR) {
      Q = c->quad_order > 0 ? c->quad_order : 4;
      if (Q > 16) { undo(); return fail(RD_ERR_INVALID, "quad_order must be <= 16"); }
      P_ = c->quad_panels > 0 ? c->quad_panels : supply_panels(p.em_Lx, p.em_Ly, p.emitter_type, p.ring_rmin, p.ring_thick, Q);
      if ((long long)P_ * Q > 4096) { undo(); return fail(RD_ERR_INVALID, "quad_panels x quad_order must be <= 4096"); }
      p.quad_n = P_ * Q;
      npt = p.quad_n * p.quad_n;
    } else {
      npt = 10000;
    }
    sl.q_len = npt;
    sl.q_off = e->q_alloc.alloc(sl.q_len, 32);
    if (sl.q_off < 0) { sl.q_len = 0; undo(); return fail(RD_ERR_CAPACITY, "quadrature table full"); }
    p.q_off = (int)sl.q_off;
    // the grid is filled on the device: nothing but this description crosses the bus
    QuadSpec qs{};
    qs.geometry = p.geometry; qs.emitter_type = p.emitter_type; qs.P = P_; qs.Q = Q;
    qs.quad_n = p.quad_n; qs.q_off = (int)sl.q_off;
    qs.x0 = p.em_x0; qs.y0 = p.em_y0; qs.Lx = p.em_Lx; qs.Ly = p.em_Ly;
    qs.ring_rmin = p.ring_rmin; qs.ring_thick = p.ring_thick; qs.org_x = p.org_x; qs.org_y = p.org_y;
    qs.a_foci = p.a_foci; qs.eta_1 = p.eta_1; qs.max_xi = p.max_xi; qs.shift_z = p.shift_z;
    if (c->geometry == RD_GEOM_PLANAR) gauss_legendre(Q, qs.gx, qs.gw);
    CK(rd_launch_quad_fill(us, qs, e->qx, e->qy, e->qz, e->qw, e->qpp));
  }
  CK(upload(e, e->work + sl.w_off, wv.data(), sl.w_len * sizeof(double), us, deferred));
  // supply-target table per checkerboard cell or Voronoi site (the Gaussian model has none)
  std::vector<double> wt(3 * sl.w_len, 0.0);
  const long long cells = p.work_model == 1 ? sl.w_len : (p.work_model == 4 ? p.work_nx : 0);
  for (long long k2 = 0; k2 < cells; ++k2) {
    const double phi = p.work_model == 4 ? wv[4 * k2 + 2] : wv[k2];
    wt[3 * k2] = std::log(phi);
    wt[3 * k2 + 1] = std::log(e->k.l_const / (phi * phi));
    wt[3 * k2 + 2] = e->k.l_const / (phi * phi);
  }
  CK(upload(e, e->wtab + 3 * sl.w_off, wt.data(), wt.size() * sizeof(double), us, deferred));
  DiodeDyn y{};
  y.MH_std = (c->geometry == RD_GEOM_TIP) ? 0.125 : 0.0125;   // fe_v2:58; tip 1.0 clamped to 0.125
  y.a_rate = (c->geometry == RD_GEOM_TIP) ? 0.5 : 1.0;
  y.first_dead = 0x7fffffff;
  y.step_offset = step_offset;
  DiodeParams pw = p;
  if (deferred) pw.active = 0;   // activate_pending() sets it before the next step
  e->act_P[s] = p;               // pinned: the source of the activation copy
  e->act_P[s].active = 1;
  e->act_D[s] = y;
  e->act_choff[s] = (int)sl.ch_off;
  e->act_qoff[s] = (int)sl.q_off;
  CK(upload(e, e->dP + s, &pw, sizeof p, us, deferred));
  CK(cudaMemcpyAsync(e->dD + s, &e->act_D[s], sizeof y, cudaMemcpyHostToDevice, us));
  CK(cudaMemcpyAsync(e->d_choff + s, &e->act_choff[s], sizeof(int), cudaMemcpyHostToDevice, us));
  CK(cudaMemcpyAsync(e->d_qoff + s, &e->act_qoff[s], sizeof(int), cudaMemcpyHostToDevice, us));
  CK(cudaMemsetAsync(e->life + (size_t)s * RD_MAX_LIFE, 0, sizeof(int) * RD_MAX_LIFE, us));
  CK(cudaMemsetAsync(e->pool.mask + p.off, 0, sizeof(int) * p.cap, us));
  if (deferred) e->pending.push_back(s);
  else CK(cudaStreamSynchronize(us));
  sl.used = true;
  sl.p = p;
  e->slots[s] = sl;
  *diode = s;
  return RD_OK;
}

int rd_diode_add(rd_engine* e, const rd_diode_config* c, int* diode) {
  if (!e) return fail(RD_ERR_INVALID, "null argument");
  int rc = flush_admissions(e);
  if (rc) return rc;
  return diode_add_impl(e, c, diode, e->st, false);
}

int rd_diode_remove(rd_engine* e, int d) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  if (!valid_diode(e, d)) return fail(RD_ERR_NOTFOUND, "unknown diode");
  SlotHost& sl = e->slots[d];
  DiodeParams p{};
  DiodeDyn y{};
  CK(cudaMemcpyAsync(e->dP + d, &p, sizeof p, cudaMemcpyHostToDevice, e->st));
  CK(cudaMemcpyAsync(e->dD + d, &y, sizeof y, cudaMemcpyHostToDevice, e->st));
  CK(cudaStreamSynchronize(e->st));
  e->pool_alloc.release(sl.pool_off, sl.pool_len);
  if (sl.ch_len) e->ch_alloc.release(sl.ch_off, sl.ch_len);
  if (sl.q_len) e->q_alloc.release(sl.q_off, sl.q_len);
  if (sl.w_len) e->w_alloc.release(sl.w_off, sl.w_len);
  sl = SlotHost();
  return RD_OK;
}

int rd_diode_count(rd_engine* e, int* active) {
  if (!e || !active) return fail(RD_ERR_INVALID, "null argument");
  int n = 0;
  for (auto& s : e->slots) n += s.used ? 1 : 0;
  *active = n;
  return RD_OK;
}

// Add_Particle for a slot being admitted (deferred, on sa): positions and
// velocities staged through the admission arena, k_add_particles on sa.
static int add_particles_deferred(rd_engine* e, int d, int n, const double* pos, const double* vel, int step,
                                  int section) {
  size_t off = 0;
  if (n > 0) {
    const size_t bytes = (vel ? 6 : 3) * sizeof(double) * (size_t)n;
    CK(adm_take(e, bytes, &off));
    std::memcpy(e->adm_h + off, pos, 3 * sizeof(double) * n);
    if (vel) std::memcpy(e->adm_h + off + 3 * sizeof(double) * n, vel, 3 * sizeof(double) * n);
    CK(cudaMemcpyAsync(e->adm_d + off, e->adm_h + off, bytes, cudaMemcpyHostToDevice, e->sa));
  }
  const double* dpos = (const double*)(e->adm_d + off);
  CK(rd_launch_add_particles(e->sa, e->dP, e->dD, e->pool, d, n, dpos, vel ? dpos + 3LL * n : nullptr, nullptr,
                             step, section));
  return RD_OK;
}

int rd_add_particles(rd_engine* e, int d, int n, const double* pos, const double* vel,
                     const int* species, int step, int section) {
  if (e) { int rc0 = flush_admissions(e); if (rc0) return rc0; }
  if (!valid_diode(e, d)) return fail(RD_ERR_NOTFOUND, "unknown diode");
  if (n < 0 || (n > 0 && !pos)) return fail(RD_ERR_INVALID, "bad particle arrays");
  int rc = stage(e, 6LL * n, n);
  if (rc) return rc;
  if (n > 0) {
    // the previous upload from the pinned stage has completed (every call ends with a
    // stream synchronize), so the stage can be refilled
    std::memcpy(e->stage_hd, pos, 3 * sizeof(double) * n);
    if (vel) std::memcpy(e->stage_hd + 3LL * n, vel, 3 * sizeof(double) * n);
    CK(cudaMemcpyAsync(e->stage_d, e->stage_hd, (vel ? 6 : 3) * sizeof(double) * n, cudaMemcpyHostToDevice, e->st));
    if (species) {
      std::memcpy(e->stage_hi, species, sizeof(int) * n);
      CK(cudaMemcpyAsync(e->stage_i, e->stage_hi, sizeof(int) * n, cudaMemcpyHostToDevice, e->st));
    }
  }
  CK(rd_launch_add_particles(e->st, e->dP, e->dD, e->pool, d, n, e->stage_d, vel ? e->stage_d + 3LL * n : nullptr,
                             species ? e->stage_i : nullptr, step, section));
  CK(cudaStreamSynchronize(e->st));
  return RD_OK;
}

static int read_dyn(rd_engine* e, int d, DiodeDyn* y) {
  CK(cudaMemcpyAsync(y, e->dD + d, sizeof(DiodeDyn), cudaMemcpyDeviceToHost, e->st));
  CK(cudaStreamSynchronize(e->st));
  return RD_OK;
}

int rd_get_particles(rd_engine* e, int d, int cap, double* pos, double* vel, double* acc,
                     double* charge, int* id, int* section, int* n_out) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  if (!valid_diode(e, d)) return fail(RD_ERR_NOTFOUND, "unknown diode");
  DiodeDyn y;
  int rc = read_dyn(e, d, &y);
  if (rc) return rc;
  if (n_out) *n_out = y.n;
  int n = std::min(y.n, cap);
  if (n <= 0) return RD_OK;
  const int off = e->slots[d].p.off;
  std::vector<double> buf(n);
  auto get3 = [&](double* dst, double* a, double* b, double* c2) -> int {
    double* src[3] = {a, b, c2};
    for (int k2 = 0; k2 < 3; ++k2) {
      CK(cudaMemcpy(buf.data(), src[k2] + off, sizeof(double) * n, cudaMemcpyDeviceToHost));
      for (int i = 0; i < n; ++i) dst[3 * i + k2] = buf[i];
    }
    return RD_OK;
  };
  if (pos && (rc = get3(pos, e->pool.x, e->pool.y, e->pool.z))) return rc;
  if (vel && (rc = get3(vel, e->pool.vx, e->pool.vy, e->pool.vz))) return rc;
  if (acc && (rc = get3(acc, e->pool.ax, e->pool.ay, e->pool.az))) return rc;
  if (charge) CK(cudaMemcpy(charge, e->pool.q + off, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (id) CK(cudaMemcpy(id, e->pool.id + off, sizeof(int) * n, cudaMemcpyDeviceToHost));
  if (section) CK(cudaMemcpy(section, e->pool.section + off, sizeof(int) * n, cudaMemcpyDeviceToHost));
  return RD_OK;
}

int rd_set_particles(rd_engine* e, int d, int n, const double* pos, const double* vel,
                     const double* acc, const double* accp, const double* accp2) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  if (!valid_diode(e, d)) return fail(RD_ERR_NOTFOUND, "unknown diode");
  DiodeDyn y;
  int rc = read_dyn(e, d, &y);
  if (rc) return rc;
  if (n < 0 || n > y.n) return fail(RD_ERR_INVALID, "n exceeds the particles in flight");
  const int off = e->slots[d].p.off;
  std::vector<double> buf(std::max(n, 1));
  auto put3 = [&](const double* srcv, double* a, double* b, double* c2) -> int {
    double* dst[3] = {a, b, c2};
    for (int k2 = 0; k2 < 3; ++k2) {
      for (int i = 0; i < n; ++i) buf[i] = srcv[3 * i + k2];
      CK(cudaMemcpy(dst[k2] + off, buf.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    }
    return RD_OK;
  };
  if (n > 0) {
    if (pos && (rc = put3(pos, e->pool.x, e->pool.y, e->pool.z))) return rc;
    if (vel && (rc = put3(vel, e->pool.vx, e->pool.vy, e->pool.vz))) return rc;
    if (acc && (rc = put3(acc, e->pool.ax, e->pool.ay, e->pool.az))) return rc;
    if (accp && (rc = put3(accp, e->pool.bx, e->pool.by, e->pool.bz))) return rc;
    if (accp2 && (rc = put3(accp2, e->pool.cx, e->pool.cy, e->pool.cz))) return rc;
  }
  if ((rc = repack(e))) return rc;
  CK(cudaStreamSynchronize(e->st));
  return RD_OK;
}

int rd_accel(rd_engine* e, int d, double* acc3n) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  NvtxRange nvtx_range("rd_accel");
  if (!valid_diode(e, d)) return fail(RD_ERR_NOTFOUND, "unknown diode");
  int rc = repack(e);
  if (rc) return rc;
  if ((rc = launch_force(e))) return rc;
  CK(cudaStreamSynchronize(e->st));
  if (acc3n) return rd_get_particles(e, d, 1 << 30, nullptr, nullptr, acc3n, nullptr, nullptr, nullptr, nullptr);
  return RD_OK;
}

static int field_at_batch(rd_engine* e, int d, int M, const double* pos, double* field);

int rd_field_at(rd_engine* e, int d, int M, const double* pos, double* field) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  NvtxRange nvtx_range("rd_field_at");
  if (!valid_diode(e, d)) return fail(RD_ERR_NOTFOUND, "unknown diode");
  if (M < 0 || (M > 0 && (!pos || !field))) return fail(RD_ERR_INVALID, "bad point arrays");
  const int chunk = (e->max_items / 2) * RD_ITILE;
  for (int m0 = 0; m0 < M; m0 += chunk) {
    int rc = field_at_batch(e, d, std::min(chunk, M - m0), pos + 3LL * m0, field + 3LL * m0);
    if (rc) return rc;
  }
  return RD_OK;
}

static int field_at_batch(rd_engine* e, int d, int M, const double* pos, double* field) {
  if (M == 0) return RD_OK;
  if (M > e->fcap) {
    if (e->fpx) { cudaFree(e->fpx); cudaFree(e->fpy); cudaFree(e->fpz); cudaFree(e->ffx); cudaFree(e->ffy); cudaFree(e->ffz); }
    long long cap = std::max<long long>(M, 4096);
    double** bufs[] = {&e->fpx, &e->fpy, &e->fpz, &e->ffx, &e->ffy, &e->ffz};
    for (auto b : bufs) CK(cudaMalloc(b, cap * sizeof(double)));
    e->fcap = cap;
  }
  std::vector<double> h(M);
  double* dsts[3] = {e->fpx, e->fpy, e->fpz};
  for (int k2 = 0; k2 < 3; ++k2) {
    for (int i = 0; i < M; ++i) h[i] = pos[3 * i + k2];
    CK(cudaMemcpyAsync(dsts[k2], h.data(), sizeof(double) * M, cudaMemcpyHostToDevice, e->st));
    CK(cudaStreamSynchronize(e->st));
  }
  std::vector<int> np(e->slots.size(), 0);
  np[d] = M;
  CK(cudaMemcpyAsync(e->d_npts, np.data(), sizeof(int) * np.size(), cudaMemcpyHostToDevice, e->st));
  int rc = repack(e);
  if (rc) return rc;
  CK(plan(e, PM_FIELD, e->d_npts));
  PointSet pts{e->fpx, e->fpy, e->fpz, e->ffx, e->ffy, e->ffz, e->d_zero_off};
  CK(rd_launch_field_points(e->cfg.precision, e->slots[d].p.geometry, e->grid, e->st, e->dP, e->pool,
                            e->plan[PM_FIELD], e->ph[PM_FIELD], pts, e->partial, e->tickets, e->kscale));
  double* srcs[3] = {e->ffx, e->ffy, e->ffz};
  for (int k2 = 0; k2 < 3; ++k2) {
    CK(cudaMemcpyAsync(h.data(), srcs[k2], sizeof(double) * M, cudaMemcpyDeviceToHost, e->st));
    CK(cudaStreamSynchronize(e->st));
    for (int i = 0; i < M; ++i) field[3 * i + k2] = h[i];
  }
  return RD_OK;
}

int rd_time_accel(rd_engine* e, int reps, double* ms_per_eval) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  if (!e || !ms_per_eval || reps <= 0) return fail(RD_ERR_INVALID, "bad argument");
  int rc = repack(e);
  if (rc) return rc;
  if ((rc = launch_force(e))) return rc;   // warm-up
  CK(cudaEventRecord(e->ev0, e->st));
  for (int r = 0; r < reps; ++r)
    if ((rc = launch_force(e))) return rc;
  CK(cudaEventRecord(e->ev1, e->st));
  CK(cudaEventSynchronize(e->ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
  *ms_per_eval = ms / reps;
  return RD_OK;
}

int rd_time_verlet(rd_engine* e, int reps, double* position_ms, double* velocity_ms) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  NvtxRange nvtx_range("rd_time_verlet");
  if (!e || !position_ms || !velocity_ms || reps <= 0) return fail(RD_ERR_INVALID, "bad argument");
  const int ns = e->nslots_hw();
  CK(plan(e, PM_PART));
  CK(rd_launch_position(e->grid, e->st, e->dP, e->dD, e->pool, e->plan[PM_PART], e->ph[PM_PART], e->evlog,
                        e->d_step));   // warm-up
  CK(rd_launch_velocity(e->grid, ns, e->st, e->dP, e->dD, e->pool, e->plan[PM_PART], e->ph[PM_PART], e->ramo,
                        e->d_step));
  float ms = 0.f;
  CK(cudaEventRecord(e->ev0, e->st));
  for (int r = 0; r < reps; ++r)
    CK(rd_launch_position(e->grid, e->st, e->dP, e->dD, e->pool, e->plan[PM_PART], e->ph[PM_PART], e->evlog,
                          e->d_step));
  CK(cudaEventRecord(e->ev1, e->st));
  CK(cudaEventSynchronize(e->ev1));
  CK(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
  *position_ms = ms / reps;
  CK(cudaEventRecord(e->ev0, e->st));
  for (int r = 0; r < reps; ++r)
    CK(rd_launch_velocity(e->grid, ns, e->st, e->dP, e->dD, e->pool, e->plan[PM_PART], e->ph[PM_PART], e->ramo,
                          e->d_step));
  CK(cudaEventRecord(e->ev1, e->st));
  CK(cudaEventSynchronize(e->ev1));
  CK(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
  *velocity_ms = ms / reps;
  return RD_OK;
}

int rd_time_remove(rd_engine* e, double* position_ms, double* remove_ms, long long* moved, long long* removed) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  NvtxRange nvtx_range("rd_time_remove");
  if (!e || !position_ms || !remove_ms || !moved || !removed) return fail(RD_ERR_INVALID, "bad argument");
  const int S = e->cfg.max_diodes;
  float ms = 0.f;
  CK(plan(e, PM_PART));
  CK(cudaEventRecord(e->ev0, e->st));
  CK(rd_launch_position(e->grid, e->st, e->dP, e->dD, e->pool, e->plan[PM_PART], e->ph[PM_PART], e->evlog,
                        e->d_step));
  CK(cudaEventRecord(e->ev1, e->st));
  CK(cudaEventSynchronize(e->ev1));
  CK(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
  *position_ms = ms;
  // survivors behind the first removed particle are the ones compaction moves
  std::vector<DiodeDyn> dyn(S);
  CK(cudaMemcpy(dyn.data(), e->dD, sizeof(DiodeDyn) * S, cudaMemcpyDeviceToHost));
  *moved = 0;
  *removed = 0;
  for (int d = 0; d < S; ++d) {
    if (!e->slots[d].used || dyn[d].n_remove == 0) continue;
    *moved += (long long)dyn[d].n - dyn[d].first_dead - dyn[d].n_remove;
    *removed += dyn[d].n_remove;
  }
  CK(plan(e, PM_PART1024));
  CK(cudaEventRecord(e->ev0, e->st));
  CK(rd_launch_compact(e->grid, e->nslots_hw(), e->st, e->dP, e->dD, e->pool, e->plan[PM_PART1024],
                       e->ph[PM_PART1024], e->ccnt, e->cpre, e->cflag, e->cq, e->life, e->d_step));
  CK(cudaEventRecord(e->ev1, e->st));
  CK(cudaEventSynchronize(e->ev1));
  CK(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
  *remove_ms = ms;
  return compaction_check(e);
}

int rd_time_field_at(rd_engine* e, int d, int M, const double* pos, int reps, double* ms_per_eval) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  if (!valid_diode(e, d)) return fail(RD_ERR_NOTFOUND, "unknown diode");
  if (M <= 0 || !pos || !ms_per_eval || reps <= 0) return fail(RD_ERR_INVALID, "bad argument");
  if (M > (e->max_items / 2) * RD_ITILE) return fail(RD_ERR_CAPACITY, "too many points for one evaluation");
  std::vector<double> field(3LL * M);
  int rc = field_at_batch(e, d, M, pos, field.data());   // uploads the points; warm-up
  if (rc) return rc;
  PointSet pts{e->fpx, e->fpy, e->fpz, e->ffx, e->ffy, e->ffz, e->d_zero_off};
  CK(cudaEventRecord(e->ev0, e->st));
  for (int r = 0; r < reps; ++r) {
    CK(plan(e, PM_FIELD, e->d_npts));
    CK(rd_launch_field_points(e->cfg.precision, e->slots[d].p.geometry, e->grid, e->st, e->dP, e->pool,
                              e->plan[PM_FIELD], e->ph[PM_FIELD], pts, e->partial, e->tickets, e->kscale));
  }
  CK(cudaEventRecord(e->ev1, e->st));
  CK(cudaEventSynchronize(e->ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
  *ms_per_eval = ms / reps;
  return RD_OK;
}

// ---- event log -------------------------------------------------------------------------
int rd_events_take(rd_engine* e, int cap, rd_event* out, int* n_out, long long* n_lost) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  if (!e || !n_out || !n_lost || cap < 0 || (cap > 0 && !out)) return fail(RD_ERR_INVALID, "bad argument");
  *n_out = 0;
  *n_lost = 0;
  if (!e->evlog.buf) return fail(RD_ERR_STATE, "the engine has no event log (event_capacity = 0)");
  int count = 0;
  CK(cudaMemcpyAsync(&count, e->evlog.count, sizeof(int), cudaMemcpyDeviceToHost, e->st));
  CK(cudaStreamSynchronize(e->st));
  const int n = std::min(count, e->evlog.cap);
  std::vector<rd_event> recs((size_t)n);
  if (n > 0) CK(cudaMemcpyAsync(recs.data(), e->evlog.buf, sizeof(rd_event) * n, cudaMemcpyDeviceToHost, e->st));
  CK(cudaMemsetAsync(e->evlog.count, 0, sizeof(int), e->st));
  CK(cudaStreamSynchronize(e->st));
  std::sort(recs.begin(), recs.end(), [](const rd_event& a, const rd_event& b) {
    if (a.diode != b.diode) return a.diode < b.diode;
    if (a.kind != b.kind) return a.kind < b.kind;
    return a.id < b.id;
  });
  const int m = std::min(n, cap);
  std::copy(recs.begin(), recs.begin() + m, out);
  *n_out = m;
  *n_lost = (long long)(count - n) + (n - m);
  return RD_OK;
}

// ---- autotuner ------------------------------------------------------------------------
// Device time of the pair-sum passes of one step under the current chunking:
// the force pass and, if planar diodes emit, a dry MH jump pass (field at
// every chain's current point; nothing written but scratch), each averaged
// over `reps` launches after one warm-up.
static int time_pair_passes(rd_engine* e, int reps, double* force_ms, double* mh_ms) {
  Sig s = signature(e);
  float ms = 0.f;
  int rc = launch_force(e);
  if (rc) return rc;
  CK(cudaEventRecord(e->ev0, e->st));
  for (int r = 0; r < reps; ++r)
    if ((rc = launch_force(e))) return rc;
  CK(cudaEventRecord(e->ev1, e->st));
  CK(cudaEventSynchronize(e->ev1));
  CK(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
  *force_ms = ms / reps;
  *mh_ms = 0.0;
  if (s.emit_planar) {
    // dry jumps back to back on the part streams, forked and joined once, as a step runs its
    // jumps: successive launches of a stream overlap the other streams' tails
    const int parts = mh_parts_for(e, s), form = mh_form_for(e, s);
    CK(plan(e, PM_MH));
    if ((rc = mh_fork(e, parts, e->st)) || (rc = planar_mh_launch(e, s, -1, parts, form, e->st)) ||
        (rc = mh_join(e, parts, e->st)))
      return rc;
    CK(cudaEventRecord(e->ev0, e->st));
    if ((rc = mh_fork(e, parts, e->st))) return rc;
    for (int r = 0; r < reps; ++r)
      if ((rc = planar_mh_launch(e, s, -1, parts, form, e->st))) return rc;
    if ((rc = mh_join(e, parts, e->st))) return rc;
    CK(cudaEventRecord(e->ev1, e->st));
    CK(cudaEventSynchronize(e->ev1));
    CK(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
    *mh_ms = ms / reps;
  }
  return RD_OK;
}

int rd_autotune(rd_engine* e, rd_tune_result* out) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  NvtxRange nvtx_range("rd_autotune");
  if (!e || !out) return fail(RD_ERR_INVALID, "null argument");
  *out = rd_tune_result{};
  out->chunk_min = e->clen_min;
  out->chunk_count_max = e->nch_max;
  if (e->nslots_hw() == 0) return RD_OK;
  int rc = repack(e);
  if (rc) return rc;
  // the force passes overwrite the current accelerations: keep them in the compaction pool
  const size_t bytes = sizeof(double) * (size_t)e->cfg.particle_capacity;
  CK(cudaMemcpyAsync(e->save_ax, e->pool.ax, bytes, cudaMemcpyDeviceToDevice, e->st));
  CK(cudaMemcpyAsync(e->save_ay, e->pool.ay, bytes, cudaMemcpyDeviceToDevice, e->st));
  CK(cudaMemcpyAsync(e->save_az, e->pool.az, bytes, cudaMemcpyDeviceToDevice, e->st));
  const int jumps = std::max(signature(e).jumps, 1);
  const int saved_min = e->clen_min, saved_max = e->nch_max;
  const int user_parts = e->mh_parts, user_form = e->mh_form;
  e->mh_parts = 0;    // the chunking is searched at the default launch shape
  e->mh_form = -1;
  double best = 1e300, at_default = 0.0, best_fms = 0.0;
  int best_min = saved_min, best_max = saved_max;
  const int mins[] = {128, 256, 512, 1024, 2048};   // short chunks: more items for small systems
  const int maxs[] = {8, 16, 32};
  for (int a : mins)
    for (int b : maxs) {
      e->clen_min = a;
      e->nch_max = b;
      double fms = 0.0, mms = 0.0;
      if ((rc = time_pair_passes(e, 2, &fms, &mms))) {
        e->clen_min = saved_min; e->nch_max = saved_max; e->mh_parts = user_parts; e->mh_form = user_form;
        return rc;
      }
      const double est = fms + jumps * mms;
      if (a == RD_CLEN_MIN && b == RD_NCH_MAX) at_default = est;
      if (est < best) { best = est; best_min = a; best_max = b; best_fms = fms; }
      out->candidates++;
    }
  e->clen_min = best_min;
  e->nch_max = best_max;
  // the MH launch shape under the chosen chunking: plan parts (with two or more
  // diodes running batched chains) and the FP32 thread form; both bit-identical
  const Sig sg = signature(e);
  const int saved_parts = user_parts, saved_form = user_form;
  int best_parts = mh_parts_for(e, sg), best_form = mh_form_for(e, sg);
  double best_mh_ms = 1e300;
  if (sg.emit_planar) {
    double& best_mh = best_mh_ms;
    const int max_parts = sg.mh_planar > 1 ? RD_MH_PARTS_MAX : 1;
    const int max_form = e->cfg.precision == RD_PREC_FP32C ? 1 : 0;
    for (int parts = 1; parts <= max_parts; ++parts)
      for (int form = 0; form <= max_form; ++form) {
        e->mh_parts = parts;
        e->mh_form = form;
        double fms = 0.0, mms = 0.0;
        if ((rc = time_pair_passes(e, 6, &fms, &mms))) { e->mh_parts = saved_parts; e->mh_form = saved_form; return rc; }
        if (mms < best_mh) { best_mh = mms; best_parts = parts; best_form = form; }
        out->candidates++;
      }
  }
  e->mh_parts = best_parts;
  e->mh_form = best_form;
  if (sg.emit_planar) best = std::min(best, best_fms + jumps * best_mh_ms);
  CK(cudaMemcpyAsync(e->pool.ax, e->save_ax, bytes, cudaMemcpyDeviceToDevice, e->st));
  CK(cudaMemcpyAsync(e->pool.ay, e->save_ay, bytes, cudaMemcpyDeviceToDevice, e->st));
  CK(cudaMemcpyAsync(e->pool.az, e->save_az, bytes, cudaMemcpyDeviceToDevice, e->st));
  CK(cudaStreamSynchronize(e->st));
  out->chunk_min = best_min;
  out->chunk_count_max = best_max;
  out->mh_parts = best_parts;
  out->mh_form = best_form;
  out->ms_default = at_default;
  out->ms_chosen = best;
  return RD_OK;   // the step graph is rebuilt at the next step (its signature holds the choices)
}

int rd_supply_points(const rd_diode_config* c, long long* npts) {
  if (!c || !npts) return fail(RD_ERR_INVALID, "null argument");
  *npts = 0;
  if (!c->emission) return RD_OK;
  if (c->geometry == RD_GEOM_TIP) { *npts = 10000; return RD_OK; }
  if (c->geometry != RD_GEOM_PLANAR) return fail(RD_ERR_INVALID, "unknown geometry");
  const int Q = c->quad_order > 0 ? c->quad_order : 4;
  int P = c->quad_panels;
  if (P <= 0) {
    const RdConst k = make_constants();
    const int type = c->emitter_type > 0 ? c->emitter_type : 2;
    double thick = 0.0, rmin = 0.0;
    if (type == 4) {
      thick = c->emitter_thickness > 0.0 ? c->emitter_thickness
                                         : std::sqrt((k.q0 * c->gap) / (k.pi * k.eps0 * c->V_s));
      rmin = c->emitter_dim[0] - thick;
    }
    P = supply_panels(c->emitter_dim[0], c->emitter_dim[1], type, rmin, thick, Q);
  }
  *npts = (long long)(P * Q) * (P * Q);
  return RD_OK;
}

int rd_set_mh_launch(rd_engine* e, int parts, int form) {
  if (!e) return fail(RD_ERR_INVALID, "null engine");
  if (parts < 0 || parts > RD_MH_PARTS_MAX) return fail(RD_ERR_INVALID, "parts must be in [0, 4] (0: default)");
  if (form < -1 || form > 1) return fail(RD_ERR_INVALID, "form must be -1 (default), 0 or 1");
  e->mh_parts = parts;
  e->mh_form = form;
  return RD_OK;
}

int rd_get_mh_launch(rd_engine* e, int* parts, int* form) {
  if (!e || !parts || !form) return fail(RD_ERR_INVALID, "null argument");
  const Sig s = signature(e);
  *parts = mh_parts_for(e, s);
  *form = mh_form_for(e, s);
  return RD_OK;
}

int rd_set_chunking(rd_engine* e, int chunk_min, int chunk_count_max) {
  if (!e) return fail(RD_ERR_INVALID, "null engine");
  const int a = chunk_min > 0 ? chunk_min : RD_CLEN_MIN, b = chunk_count_max > 0 ? chunk_count_max : RD_NCH_MAX;
  if (!valid_chunking(a, b))
    return fail(RD_ERR_INVALID, "chunk_min must be a multiple of 128 in [128, 65536], chunk_count_max in [1, 32]");
  e->clen_min = a;
  e->nch_max = b;
  return RD_OK;
}

int rd_get_chunking(rd_engine* e, int* chunk_min, int* chunk_count_max) {
  if (!e || !chunk_min || !chunk_count_max) return fail(RD_ERR_INVALID, "null argument");
  *chunk_min = e->clen_min;
  *chunk_count_max = e->nch_max;
  return RD_OK;
}

int rd_mark_remove(rd_engine* e, int d, int i, int why) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  if (!valid_diode(e, d)) return fail(RD_ERR_NOTFOUND, "unknown diode");
  if (why != RD_REMOVE_TOP && why != RD_REMOVE_BOT) return fail(RD_ERR_INVALID, "unknown removal flag");
  CK(rd_launch_mark(e->st, e->dP, e->dD, e->pool, d, i, why));
  CK(cudaStreamSynchronize(e->st));
  return RD_OK;
}

int rd_do_emission(rd_engine* e, int step) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  NvtxRange nvtx_range("rd_do_emission");
  if (!e) return fail(RD_ERR_INVALID, "null engine");
  CK(rd_launch_step_set(e->st, e->d_step, step));
  int rc = launch_emission(e);
  if (rc) return rc;
  CK(cudaStreamSynchronize(e->st));
  return RD_OK;
}

int rd_update_position(rd_engine* e, int step) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  NvtxRange nvtx_range("rd_update_position");
  if (!e) return fail(RD_ERR_INVALID, "null engine");
  CK(rd_launch_step_set(e->st, e->d_step, step));
  int rc = launch_update_position(e);
  if (rc) return rc;
  CK(cudaStreamSynchronize(e->st));
  return RD_OK;
}

int rd_remove_particles(rd_engine* e, int step) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  NvtxRange nvtx_range("rd_remove_particles");
  if (!e) return fail(RD_ERR_INVALID, "null engine");
  CK(rd_launch_step_set(e->st, e->d_step, step));
  int rc = launch_remove(e);
  if (rc) return rc;
  CK(cudaStreamSynchronize(e->st));
  return compaction_check(e);
}

int rd_run(rd_engine* e, int first_step, int nsteps) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  NvtxRange nvtx_range("rd_run");
  if (!e) return fail(RD_ERR_INVALID, "null engine");
  if (nsteps < 0) return fail(RD_ERR_INVALID, "nsteps < 0");
  int rc = ensure_graph(e);
  if (rc) return rc;
  CK(rd_launch_step_set(e->st, e->d_step, first_step));
  CK(cudaEventRecord(e->ev0, e->st));
  for (int s = 0; s < nsteps; ++s) CK(cudaGraphLaunch(e->graph, e->st));
  CK(cudaEventRecord(e->ev1, e->st));
  CK(cudaStreamSynchronize(e->st));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
  e->last_ms = ms;
  return compaction_check(e);
}

int rd_step(rd_engine* e, int step) { return rd_run(e, step, 1); }

static void fill_counters(const DiodeDyn& y, rd_counters* o) {
  o->n = y.n;
  o->emitted_step = y.emitted_step; o->dropped_step = y.dropped_step;
  o->absorbed_top_step = y.absorbed_top_step; o->absorbed_bot_step = y.absorbed_bot_step;
  o->chains = y.chains; o->chains_failed = y.chains_failed; o->chains_capped = y.chains_capped;
  o->emitted_total = y.emitted_total; o->dropped_total = y.dropped_total;
  o->absorbed_top_total = y.absorbed_top_total; o->absorbed_bot_total = y.absorbed_bot_total;
  o->electron_steps = y.electron_steps; o->steps_done = y.steps_done;
  o->ramo_current = y.ramo_current; o->N_sup = y.N_sup; o->MH_std = y.MH_std;
  o->a_rate = y.a_rate; o->residual = y.residual;
  // with image charges the lateral components cancel at the cathode exactly (0)
  o->F_avg[0] = y.F_avg_x; o->F_avg[1] = y.F_avg_y; o->F_avg[2] = y.F_avg_z;
  o->df_avg = y.df_avg;
  o->ramo_current_ion = y.ramo_ion;
  for (int c = 0; c < 3; ++c) {
    o->avg_part_vel[c] = y.avg_part_vel[c];
    o->avg_elec_vel[c] = y.avg_elec_vel[c];
    o->avg_ion_vel[c] = y.avg_ion_vel[c];
  }
  o->avg_mob = y.avg_mob;
  o->n_part_vel = y.n_vel;
  o->n_elec_vel = y.n_elec_vel;
  o->n_ion_vel = y.n_ion_vel;
}

int rd_counters_get(rd_engine* e, int d, rd_counters* o) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  if (!valid_diode(e, d)) return fail(RD_ERR_NOTFOUND, "unknown diode");
  if (!o) return fail(RD_ERR_INVALID, "null argument");
  DiodeDyn y;
  int rc = read_dyn(e, d, &y);
  if (rc) return rc;
  fill_counters(y, o);
  return RD_OK;
}

int rd_validate(rd_engine* e, int counts[RD_VALIDATE_KINDS], long long* total) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  NvtxRange nvtx_range("rd_validate");
  if (!e || !counts) return fail(RD_ERR_INVALID, "null argument");
  const int S = e->nslots_hw();
  std::vector<int> bad((size_t)std::max(S, 1) * RD_VALIDATE_KINDS, 0);
  int* dbad = nullptr;
  CK(cudaMalloc(&dbad, sizeof(int) * bad.size()));
  cudaError_t ce = rd_launch_validate(S, e->st, e->dP, e->dD, e->pool, dbad);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(bad.data(), dbad, sizeof(int) * bad.size(), cudaMemcpyDeviceToHost, e->st);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->st);
  cudaFree(dbad);
  CK(ce);
  long long sum = 0;
  for (int k = 0; k < RD_VALIDATE_KINDS; ++k) {
    counts[k] = 0;
    for (int d = 0; d < S; ++d) counts[k] += bad[(size_t)d * RD_VALIDATE_KINDS + k];
    sum += counts[k];
  }
  if (total) *total = sum;
  return RD_OK;
}

// ---- diode checkpoints ----------------------------------------------------------------
namespace {
struct StateHeader {
  char magic[8];      // "RDSTATE1"
  int version;        // 1
  int n;              // particles saved
  int dyn_bytes;      // sizeof(DiodeDyn) of the writer
  int life_len;       // RD_MAX_LIFE
  int capacity;       // the slot's capacity when saved
  int pad;
};
constexpr int kStateDoubles = 17;   // x y z vx vy vz, a, a_prev, a_prev2 (9), q, m
constexpr int kStateInts = 5;       // species id step0 section mask

double* state_dbl(Pool& p, int k) {
  double* a[kStateDoubles] = {p.x, p.y, p.z, p.vx, p.vy, p.vz, p.ax, p.ay, p.az,
                              p.bx, p.by, p.bz, p.cx, p.cy, p.cz, p.q, p.m};
  return a[k];
}
int* state_int(Pool& p, int k) {
  int* a[kStateInts] = {p.species, p.id, p.step0, p.section, p.mask};
  return a[k];
}
long long state_bytes(int n) {
  return (long long)sizeof(StateHeader) + (long long)sizeof(DiodeDyn) +
         (long long)n * (kStateDoubles * (long long)sizeof(double) + kStateInts * (long long)sizeof(int)) +
         (long long)RD_MAX_LIFE * (long long)sizeof(int);
}
}  // namespace

int rd_diode_state_size(rd_engine* e, int d, long long* bytes) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  if (!valid_diode(e, d)) return fail(RD_ERR_NOTFOUND, "unknown diode");
  if (!bytes) return fail(RD_ERR_INVALID, "null argument");
  DiodeDyn y;
  int rc = read_dyn(e, d, &y);
  if (rc) return rc;
  *bytes = state_bytes(y.n);
  return RD_OK;
}

int rd_diode_save(rd_engine* e, int d, void* buf, long long cap, long long* written) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  NvtxRange nvtx_range("rd_diode_save");
  if (!valid_diode(e, d)) return fail(RD_ERR_NOTFOUND, "unknown diode");
  if (!buf) return fail(RD_ERR_INVALID, "null buffer");
  DiodeDyn y;
  int rc = read_dyn(e, d, &y);
  if (rc) return rc;
  const long long need = state_bytes(y.n);
  if (cap < need) return fail(RD_ERR_INVALID, "buffer smaller than rd_diode_state_size");
  char* out = static_cast<char*>(buf);
  StateHeader h{};
  std::memcpy(h.magic, "RDSTATE1", 8);
  h.version = 1;
  h.n = y.n;
  h.dyn_bytes = (int)sizeof(DiodeDyn);
  h.life_len = RD_MAX_LIFE;
  h.capacity = e->slots[d].p.cap;
  std::memcpy(out, &h, sizeof h);
  out += sizeof h;
  std::memcpy(out, &y, sizeof y);
  out += sizeof y;
  const int off = e->slots[d].p.off;
  for (int k = 0; k < kStateDoubles; ++k, out += sizeof(double) * (size_t)y.n)
    if (y.n) CK(cudaMemcpy(out, state_dbl(e->pool, k) + off, sizeof(double) * (size_t)y.n, cudaMemcpyDeviceToHost));
  for (int k = 0; k < kStateInts; ++k, out += sizeof(int) * (size_t)y.n)
    if (y.n) CK(cudaMemcpy(out, state_int(e->pool, k) + off, sizeof(int) * (size_t)y.n, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(out, e->life + (size_t)d * RD_MAX_LIFE, sizeof(int) * RD_MAX_LIFE, cudaMemcpyDeviceToHost));
  if (written) *written = need;
  return RD_OK;
}

int rd_diode_load(rd_engine* e, int d, const void* buf, long long size) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  NvtxRange nvtx_range("rd_diode_load");
  if (!valid_diode(e, d)) return fail(RD_ERR_NOTFOUND, "unknown diode");
  if (!buf || size < (long long)sizeof(StateHeader)) return fail(RD_ERR_INVALID, "not a diode state");
  const char* in = static_cast<const char*>(buf);
  StateHeader h;
  std::memcpy(&h, in, sizeof h);
  if (std::memcmp(h.magic, "RDSTATE1", 8) != 0 || h.version != 1 || h.dyn_bytes != (int)sizeof(DiodeDyn) ||
      h.life_len != RD_MAX_LIFE || h.n < 0)
    return fail(RD_ERR_INVALID, "not a diode state of this library version");
  if (size < state_bytes(h.n)) return fail(RD_ERR_INVALID, "diode state truncated");
  const DiodeParams& p = e->slots[d].p;
  if (h.n > p.cap) return fail(RD_ERR_CAPACITY, "saved particles exceed the slot's capacity");
  CK(cudaStreamSynchronize(e->st));
  in += sizeof h;
  DiodeDyn y;
  std::memcpy(&y, in, sizeof y);
  in += sizeof y;
  const int off = p.off;
  for (int k = 0; k < kStateDoubles; ++k, in += sizeof(double) * (size_t)h.n)
    if (h.n) CK(cudaMemcpy(state_dbl(e->pool, k) + off, in, sizeof(double) * (size_t)h.n, cudaMemcpyHostToDevice));
  for (int k = 0; k < kStateInts; ++k, in += sizeof(int) * (size_t)h.n)
    if (h.n) CK(cudaMemcpy(state_int(e->pool, k) + off, in, sizeof(int) * (size_t)h.n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(e->life + (size_t)d * RD_MAX_LIFE, in, sizeof(int) * RD_MAX_LIFE, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(e->dD + d, &y, sizeof y, cudaMemcpyHostToDevice));
  int rc = repack(e);   // the FP32 packs (and tip image points) of the loaded particles
  if (rc) return rc;
  CK(cudaStreamSynchronize(e->st));
  return RD_OK;
}

int rd_life_time(rd_engine* e, int d, int* hist) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  if (!valid_diode(e, d)) return fail(RD_ERR_NOTFOUND, "unknown diode");
  if (!hist) return fail(RD_ERR_INVALID, "null argument");
  CK(cudaMemcpy(hist, e->life + (size_t)d * RD_MAX_LIFE, sizeof(int) * RD_MAX_LIFE, cudaMemcpyDeviceToHost));
  return RD_OK;
}

int rd_last_run_stats(rd_engine* e, double* ms, int* kps) {
  if (!e) return fail(RD_ERR_INVALID, "null engine");
  if (ms) *ms = e->last_ms;
  if (kps) *kps = e->last_kernels;
  return RD_OK;
}


int rd_profile_step(rd_engine* e, int step, rd_phase_times* out) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  NvtxRange nvtx_range("rd_profile_step");
  if (!e || !out) return fail(RD_ERR_INVALID, "null argument");
  *out = rd_phase_times{};
  const int S = e->cfg.max_diodes;
  cudaEvent_t ev[9];
  for (auto& v : ev) CK(cudaEventCreate(&v));
  struct Guard { cudaEvent_t* v; ~Guard() { for (int k = 0; k < 9; ++k) cudaEventDestroy(v[k]); } } guard{ev};
  Sig s = signature(e);
  const int prec = e->cfg.precision;
  std::vector<DiodeDyn> dyn(S);
  CK(rd_launch_step_set(e->st, e->d_step, step));
  CK(cudaEventRecord(ev[0], e->st));
  if (s.emit_planar || s.emit_tip) {
    // supply integral
    if (s.emit_planar) {
      CK(plan(e, PM_SUPPLY_PLANAR));
      CK(rd_launch_z0_points(prec, e->grid, e->st, e->dP, e->pool, e->plan[PM_SUPPLY_PLANAR],
                             e->ph[PM_SUPPLY_PLANAR], e->qx, e->qy, e->qpp, e->qF, e->partial, e->tickets, e->kscale, e->item_queue + 6));
    }
    if (s.emit_lat) {
      CK(plan(e, PM_SUPPLY_LAT));
      PointSet lp{e->qx, e->qy, e->qz, e->qfx, e->qfy, e->qF, e->d_qoff};
      CK(rd_launch_field_points(prec, RD_G_PLANAR, e->grid, e->st, e->dP, e->pool, e->plan[PM_SUPPLY_LAT],
                                e->ph[PM_SUPPLY_LAT], lp, e->partial, e->tickets, e->kscale));
    }
    if (s.emit_tip) {
      CK(plan(e, PM_SUPPLY_TIP));
      PointSet pts{e->qx, e->qy, e->qz, e->qfx, e->qfy, e->qF, e->d_qoff};
      CK(rd_launch_field_points(prec, RD_G_TIP, e->grid, e->st, e->dP, e->pool, e->plan[PM_SUPPLY_TIP],
                                e->ph[PM_SUPPLY_TIP], pts, e->partial, e->tickets, e->kscale));
    }
    CK(rd_launch_supply_reduce(S, e->st, e->dP, e->dD, e->qx, e->qy, e->qw, e->qF, e->qfx, e->qfy, e->work,
                               e->d_step, e->sup_part));
    CK(cudaEventRecord(ev[1], e->st));
    CK(cudaMemcpyAsync(dyn.data(), e->dD, sizeof(DiodeDyn) * S, cudaMemcpyDeviceToHost, e->st));
    CK(cudaStreamSynchronize(e->st));
    for (int d = 0; d < S; ++d) {
      const SlotHost& sl = e->slots[d];
      if (!sl.used || !sl.p.emission) continue;
      long long npt = sl.p.geometry == RD_G_TIP ? 10000 : (long long)sl.p.quad_n * sl.p.quad_n;
      out->supply_pair_evals += npt * dyn[d].n;
      out->mh_pair_evals += (long long)dyn[d].chains * dyn[d].n * sl.p.mh_jumps;
    }
    CK(plan(e, PM_MH));
    if (s.emit_planar)
      CK(rd_launch_mh_vacuum(prec, S, e->st, e->dP, e->dD, e->cs, e->d_choff, e->wtab, e->d_step, e->kscale));
    const int gmask = (s.emit_planar ? 1 : 0) | (s.emit_tip ? 2 : 0);
    CK(rd_launch_mh_jump(prec, gmask, e->grid, e->st, e->dP, e->dD, e->pool, e->plan[PM_MH], e->ph[PM_MH],
                         e->cs, e->d_choff, e->wtab, e->d_step, 0, e->partial, e->tickets, e->kscale, e->item_queue,
                         0, 1, mh_form_for(e, s)));
    CK(rd_launch_mh_init(prec, e->grid, e->st, e->dP, e->dD, e->pool, e->plan[PM_MH], e->ph[PM_MH],
                         e->cs, e->d_choff, e->wtab, e->d_step, e->kscale));
    CK(cudaEventRecord(ev[2], e->st));
    int rcj = launch_mh_jumps(e, s, e->st);
    if (rcj) return rcj;
    out->mh_jump_launches = s.jumps;
    CK(cudaEventRecord(ev[3], e->st));
    CK(rd_launch_emit(S, e->st, e->dP, e->dD, e->pool, e->cs, e->d_choff, e->work, e->d_step, e->evlog));
    if (s.emit_serial)
      CK(rd_launch_mh_serial(prec, S, e->st, e->dP, e->dD, e->pool, e->work, e->wtab, e->d_step, e->kscale,
                             e->evlog));
  } else {
    CK(cudaEventRecord(ev[1], e->st));
    CK(cudaEventRecord(ev[2], e->st));
    CK(cudaEventRecord(ev[3], e->st));
  }
  CK(cudaEventRecord(ev[4], e->st));
  CK(plan(e, PM_PART));
  CK(rd_launch_position(e->grid, e->st, e->dP, e->dD, e->pool, e->plan[PM_PART], e->ph[PM_PART], e->evlog,
                        e->d_step));
  CK(cudaEventRecord(ev[5], e->st));
  int rc = launch_force(e, true);
  if (rc) return rc;
  CK(cudaEventRecord(ev[6], e->st));
  CK(rd_launch_velocity(e->grid, S, e->st, e->dP, e->dD, e->pool, e->plan[PM_PART], e->ph[PM_PART], e->ramo,
                        e->d_step));
  CK(cudaEventRecord(ev[7], e->st));
  CK(cudaMemcpyAsync(dyn.data(), e->dD, sizeof(DiodeDyn) * S, cudaMemcpyDeviceToHost, e->st));
  rc = launch_remove(e);
  if (rc) return rc;
  CK(rd_launch_step_inc(e->st, e->d_step));
  CK(cudaEventRecord(ev[8], e->st));
  CK(cudaStreamSynchronize(e->st));
  for (int d = 0; d < S; ++d)
    if (e->slots[d].used) out->force_pairs += (long long)dyn[d].n * (dyn[d].n > 0 ? dyn[d].n - 1 : 0);
  float t[8];
  for (int k = 0; k < 8; ++k) CK(cudaEventElapsedTime(&t[k], ev[k], ev[k + 1]));
  out->supply_ms = t[0]; out->mh_init_ms = t[1]; out->mh_jumps_ms = t[2]; out->emit_ms = t[3];
  out->position_ms = t[4]; out->force_ms = t[5]; out->velocity_ms = t[6]; out->compact_ms = t[7];
  float tot;
  CK(cudaEventElapsedTime(&tot, ev[0], ev[8]));
  out->total_ms = tot;
  return compaction_check(e);
}

// ---- serving --------------------------------------------------------------------------
int rd_clock(rd_engine* e, double* seconds) {
  if (!e || !seconds) return fail(RD_ERR_INVALID, "null argument");
  *seconds = e->clock();
  return RD_OK;
}

int rd_submit(rd_engine* e, const rd_request* req, long long* id) {
  if (!e || !req || !id) return fail(RD_ERR_INVALID, "null argument");
  if (req->steps <= 0 || req->n_init < 0 || (req->n_init > 0 && !req->pos3n))
    return fail(RD_ERR_INVALID, "bad request");
  if (req->n_init > req->diode.capacity) return fail(RD_ERR_INVALID, "n_init exceeds capacity");
  rd_engine::Req r;
  r.cfg = req->diode;
  if (req->diode.work && req->diode.work_nx > 0 && req->diode.work_ny > 0) {
    r.work.assign(req->diode.work, req->diode.work + (size_t)req->diode.work_nx * req->diode.work_ny);
  }
  r.cfg.work = nullptr;
  if (req->n_init > 0) {
    r.pos.assign(req->pos3n, req->pos3n + 3LL * req->n_init);
    if (req->vel3n) r.vel.assign(req->vel3n, req->vel3n + 3LL * req->n_init);
  }
  r.steps = req->steps;
  r.st.state = RD_REQ_QUEUED;
  r.st.diode = -1;
  r.st.steps = req->steps;
  r.st.submit_s = e->clock();
  r.st.admit_s = r.st.done_s = -1.0;
  long long k = e->next_id++;
  e->reqs[k] = std::move(r);
  e->queue.push_back(k);
  *id = k;
  return RD_OK;
}

int rd_poll(rd_engine* e, long long id, rd_request_status* out) {
  if (!e || !out) return fail(RD_ERR_INVALID, "null argument");
  auto it = e->reqs.find(id);
  if (it == e->reqs.end()) return fail(RD_ERR_NOTFOUND, "unknown request");
  *out = it->second.st;
  return RD_OK;
}

int rd_cancel(rd_engine* e, long long id) {
  if (e) { const int rcf = flush_admissions(e); if (rcf) return rcf; }
  if (!e) return fail(RD_ERR_INVALID, "null engine");
  auto it = e->reqs.find(id);
  if (it == e->reqs.end()) return fail(RD_ERR_NOTFOUND, "unknown request");
  rd_engine::Req& r = it->second;
  if (r.st.state == RD_REQ_QUEUED) {
    e->queue.erase(std::remove(e->queue.begin(), e->queue.end(), id), e->queue.end());
  } else if (r.st.state == RD_REQ_RUNNING) {
    int rc = rd_diode_remove(e, r.st.diode);
    if (rc) return rc;
    e->running.erase(r.st.diode);
    r.st.diode = -1;
  } else {
    return RD_OK;
  }
  r.st.state = RD_REQ_CANCELLED;
  r.st.done_s = e->clock();
  return RD_OK;
}

// Admits queued requests into free slots, FIFO, head of line waiting for
// capacity.  Everything is issued on the admission stream sa and nothing waits
// for the GPU: the slots become active at the next activate_pending(), so when
// a step is running on the engine stream the uploads overlap it.  first_step:
// the engine step at which the admitted diodes run their step 1.
static int serve_admit(rd_engine* e, rd_serve_stats* st, int first_step) {
  if (e->queue.empty()) return RD_OK;
  bool any_free = false;
  for (auto& sl : e->slots) if (!sl.used) { any_free = true; break; }
  if (!any_free) return RD_OK;
  // the previous batch's copies from the arena were waited for by the engine stream
  // (activate_pending) and that stream was synchronised since: the arena is free
  CK(cudaStreamSynchronize(e->sa));
  e->adm_used = 0;
  while (!e->queue.empty()) {
    long long id = e->queue.front();
    rd_engine::Req& r = e->reqs[id];
    rd_diode_config cfg = r.cfg;
    if (!r.work.empty()) cfg.work = r.work.data();
    int slot = -1;
    int rc = diode_add_impl(e, &cfg, &slot, e->sa, true, first_step - 1);
    if (rc == RD_ERR_CAPACITY) return RD_OK;   // head of line waits for capacity
    if (rc) {                                  // invalid request: drop it
      r.st.state = RD_REQ_CANCELLED;
      r.st.done_s = e->clock();
      e->queue.pop_front();
      continue;
    }
    // the slot exists on the host now; its device slot stays inactive until activation
    e->slots[slot].used = true;
    const int n = (int)(r.pos.size() / 3);
    if (n > 0 || true) {
      rc = add_particles_deferred(e, slot, n, r.pos.data(), r.vel.empty() ? nullptr : r.vel.data(), 0, 1);
      if (rc) return rc;
      st->h2d_bytes += (long long)(r.pos.size() + r.vel.size()) * sizeof(double);
    }
    r.st.state = RD_REQ_RUNNING;
    r.st.diode = slot;
    r.st.admit_s = e->clock();
    e->running[slot] = id;
    e->queue.pop_front();
    st->admitted++;
    std::vector<double>().swap(r.pos);
    std::vector<double>().swap(r.vel);
  }
  return RD_OK;
}

int rd_serve(rd_engine* e, int iterations, rd_serve_stats* out) {
  NvtxRange nvtx_range("rd_serve");
  if (!e || !out) return fail(RD_ERR_INVALID, "null argument");
  *out = rd_serve_stats{};
  const double w0 = e->clock();
  const int S = e->cfg.max_diodes;
  std::vector<DiodeDyn> dyn(S);
  std::vector<double> times;
  for (int it = 0; it < iterations; ++it) {
    int rc;
    // with nothing running, admit now; otherwise the requests admitted while the
    // previous step ran (overlapped with it) become active here
    if (e->running.empty() && (rc = serve_admit(e, out, e->gstep))) return rc;
    if ((rc = activate_pending(e))) return rc;
    if (e->running.empty()) break;
    if ((rc = ensure_graph(e))) return rc;
    CK(rd_launch_step_set(e->st, e->d_step, e->gstep));
    CK(cudaEventRecord(e->ev0, e->st));
    CK(cudaGraphLaunch(e->graph, e->st));
    CK(cudaEventRecord(e->ev1, e->st));
    CK(cudaMemcpyAsync(dyn.data(), e->dD, sizeof(DiodeDyn) * S, cudaMemcpyDeviceToHost, e->st));
    // while the step runs: admit queued requests into the slots free now, for the next step
    std::vector<char> was_pending(S, 0);
    if ((rc = serve_admit(e, out, e->gstep + 1))) return rc;
    for (int sidx : e->pending) was_pending[sidx] = 1;
    CK(cudaStreamSynchronize(e->st));
    if ((rc = compaction_check(e))) return rc;
    out->d2h_bytes += (long long)sizeof(DiodeDyn) * S;
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e->ev0, e->ev1));
    times.push_back(ms);
    out->device_ms += ms;
    out->iterations++;
    e->gstep++;
    std::vector<int> done;
    for (auto& kv : e->running) {
      if (was_pending[kv.first]) continue;   // admitted during this step: not active yet
      const DiodeDyn& y = dyn[kv.first];
      rd_engine::Req& r = e->reqs[kv.second];
      out->electron_steps += y.electron_steps - r.st.counters.electron_steps;
      fill_counters(y, &r.st.counters);
      if (y.steps_done >= r.steps) done.push_back(kv.first);
    }
    for (int slot : done) {
      rd_engine::Req& r = e->reqs[e->running[slot]];
      if ((rc = rd_diode_remove(e, slot))) return rc;
      r.st.state = RD_REQ_DONE;
      r.st.diode = -1;
      r.st.done_s = e->clock();
      e->running.erase(slot);
      out->retired++;
    }
  }
  out->running = (int)e->running.size();
  out->queued = (int)e->queue.size();
  out->wall_ms = (e->clock() - w0) * 1e3;
  if (!times.empty()) {
    std::vector<double> s(times);
    std::sort(s.begin(), s.end());
    auto pct = [&](double q) {
      double pos = q * (s.size() - 1);
      size_t lo = (size_t)pos, hi = std::min(lo + 1, s.size() - 1);
      return s[lo] + (s[hi] - s[lo]) * (pos - lo);
    };
    out->step_ms_p50 = pct(0.50);
    out->step_ms_p99 = pct(0.99);
    out->step_ms_max = s.back();
  }
  return RD_OK;
}

}  // extern "C"
