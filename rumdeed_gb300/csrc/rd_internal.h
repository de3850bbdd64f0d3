// rd_internal.h -- data model shared by the host engine and the sm_103a
// kernels of librumdeed_gb300.
//
// Layout in HBM.  All diodes of an engine share one particle pool; diode d
// owns the slots [off_d, off_d + cap_d) of every pool array (off_d is a
// multiple of 32).  The pool is struct-of-arrays so that every kernel reads
// each field with coalesced loads:
//   FP64 state  : pos x/y/z, vel x/y/z, acc (cur, prev, prev2) x/y/z, charge, mass
//   int state   : species, id, step created, section, mask
//   FP32 packs  : pk_hi = (x, y, z, q/q0) and pk_lo = (x, y, z, 0) as the high
//                 and low float parts of the position in nm (x, y relative to
//                 the diode's lateral origin, z absolute from the cathode);
//                 tip diodes add the sphere image point of each particle in
//                 the same hi/lo form (ip_hi, ip_lo).
// The segment table (DiodeParams, static per admission; DiodeDyn, dynamic
// counters) lives in device memory, so a captured step graph stays valid
// while requests are admitted and retired.
#pragma once
#include "../../include/rumdeed_gpu.h"
#include <stdint.h>

#define RD_TILE 128           // particles per shared-memory j-tile
#define RD_ITILE 128          // i-particles (or points) per work item
#ifndef RD_TIP_CPT
#define RD_TIP_CPT 2          // tip MH chains per thread (FP32 form; even)
#endif
#ifndef RD_TIP_UNROLL
#define RD_TIP_UNROLL 4       // j-loop unroll of the FP32 tip MH tile
#endif
#define RD_MH_PARTS 2         // planar MH jump launches per jump, one stream each (default)
#define RD_MH_PARTS_MAX 4     // at most this many (rd_autotune / rd_set_mh_launch choose)
#define RD_SUP_SPLIT 64       // blocks per diode in the supply reduction
#define RD_SUP_NCH 4          // at most this many j-chunks per tile of planar supply points
#define RD_EMIT_SPLIT 8       // blocks per diode in the emission accept test
// j-chunking of pair sums: at least RD_CLEN_MIN particles per chunk, at most
// RD_NCH_MAX chunks per i-tile
#define RD_CLEN_MIN 1024
#define RD_NCH_MAX 32
// the planner's chunk rule argument: clen_min | nch_max << 16
inline int rd_chunk_rule(int clen_min, int nch_max) { return clen_min | (nch_max << 16); }
#define RD_MAX_LIFE 1000
#define RD_COMPACT_SPIN (1 << 22)   // polls (64 ns sleeps) of a compaction tile waiting on an earlier one
#define RD_MAX_WORK 4096      // max checkerboard cells per diode (64x64)

enum { RD_G_PLANAR = 1, RD_G_TIP = 2 };

// 32-byte aligned quadruple of doubles (one particle of an FP64 j-tile).
struct __align__(32) rd_d4 { double x, y, z, w; };
#ifdef __CUDACC__
__host__ __device__ inline rd_d4 make_d4(double x, double y, double z, double w) {
  rd_d4 r; r.x = x; r.y = y; r.z = z; r.w = w; return r;
}
#endif

struct RdConst {
  double pi, q0, m0, eps0, hbar, div_fac_c, a_FN, b_FN, l_const, L2, tip_K, m_N2, m_N2p;
  double length_scale;
  double q0_inv;   // 1 / q0, for the FP32 charge packs
};

// Static parameters of one diode slot.
struct DiodeParams {
  int active;            // 1 while the slot holds a simulation
  int geometry;          // RD_G_PLANAR / RD_G_TIP
  int cap, off;          // capacity and pool offset
  int image_charge, N_ic_max;
  int emission;          // 0 off, 1 field emission
  int mh_jumps, max_chains, init_rounds;
  int quad_n;            // supply quadrature points per dimension (planar)
  int q_off;             // offset of this diode's quadrature points in the quad table
  int work_nx, work_ny, work_off;
  int work_model;        // 1 checkerboard, 2 Gaussian, 4 Voronoi (Read_work_function types)
  const double* work_data;   // this diode's work-function parameters (device)
  unsigned long long seed;
  double V, d, E_z, dt, dt2;
  double em_x0, em_y0, em_Lx, em_Ly;
  double org_x, org_y;   // lateral origin of the FP32 frame (m)
  // hyperboloid tip (mod_hyperboloid_tip)
  double a_foci, eta_1, max_xi, shift_z, r_tip, h_tip, pre_E, pre_E_unit, tip_phi;
  double mh_lo, mh_hi;   // MH_std clamps
  // FP32 frame of the planar emitter (nm, relative to its centre): half widths
  // rounded toward zero (chains stay inside) and full widths
  float em_hx, em_hy, em_wx, em_wy;
  int emit_delay;        // the emitter emits from step emit_delay + 1 on
  int mh_serial;         // 1: serial MH sampler (k_mh_serial)
  int emitter_type;      // 2 rectangle (1 circle is sampled as its box), 4 ring
  double ring_rmin, ring_thick;   // ring emitter: inner radius and width (m)
  int planes_n;          // measurement planes (Check_Planes)
  double planes_z[10];
  int tts;               // two-time-step interval T (atom_time_interval); 0 off
  double ramo_uz;        // -1 / d: z of the planar unit field E_zunit_planar
};

// Planner modes (k_plan): which i-set of each diode a pair-sum plan covers.
// Modes up to PM_SUPPLY_LAT are pair sums (tiles x j-chunks), the two PM_PART
// modes per-particle index spaces.  PM_SUPPLY_PLANAR: the supply points of
// planar diodes with image charges (F_z only: the lateral components cancel
// at the cathode); PM_SUPPLY_LAT: those of planar diodes without (all three
// components, for the mean field of field.dt).  PM_ALL_DIODES added to PM_FORCE_PLANAR or
// PM_FORCE_TIP also covers the two-time-step diodes (the plain
// Calculate_Acceleration_Particles pass, which ignores two_time_step).
enum { PM_FORCE_PLANAR = 0, PM_FORCE_TIP = 1, PM_FIELD = 2, PM_SUPPLY_PLANAR = 3,
       PM_SUPPLY_TIP = 4, PM_MH = 5, PM_FORCE_TTS = 6, PM_SUPPLY_LAT = 7, PM_PART = 8, PM_PART1024 = 9,
       PM_COUNT = 10, PM_ALL_DIODES = 0x100 };

// Supply quadrature grid of one diode, filled on the device (k_quad_fill):
// planar, quad_n x quad_n Gauss-Legendre nodes (P panels of Q nodes per side)
// over the emitter rectangle, or over (angle, radius) of a ring; tip, the
// 100 x 100 midpoint grid in (xi, phi).
struct QuadSpec {
  int geometry, emitter_type, P, Q, quad_n, q_off;
  double x0, y0, Lx, Ly, ring_rmin, ring_thick, org_x, org_y;
  double a_foci, eta_1, max_xi, shift_z;
  double gx[16], gw[16];
};

// Dynamic per-diode state (device resident, updated by kernels).
struct DiodeDyn {
  int n;                 // particles in flight
  int nrID;
  int n_remove, n_remove_top, n_remove_bot;
  int first_dead;
  int emitted_step, dropped_step;
  int chains, chains_failed, chains_capped;
  int mh_acc, mh_rej, mh_done;   // per-jump counters (reset by the last arriver)
  int ser_ticket, ser_emit, ser_done;   // serial sampler, speculative vacuum pass (k_mh_serial_vacuum)
  int sup_done;
  int absorbed_top_step, absorbed_bot_step;
  int step_offset;       // this diode's step = engine step - step_offset
  long long emitted_total, absorbed_top_total, absorbed_bot_total, dropped_total;
  long long electron_steps;      // sum over steps of particles in flight
  long long steps_done;
  double ramo_current, ramo_ion;   // ramo_current(species_elec), ramo_current(species_ion)
  double MH_std, a_rate, residual, N_sup;
  double F_avg_z, df_avg;   // field.dt quantities of the last emission
  double F_avg_x, F_avg_y;  // lateral mean field (planar diodes without image charges; 0 otherwise)
  double avg_part_vel[3], avg_elec_vel[3], avg_ion_vel[3], avg_mob;   // Average_Velocities
  int n_vel, n_elec_vel, n_ion_vel;   // particle counts at the velocity update (before removal)
};

// A planar diode whose batched MH chains sample the vacuum field: no particle
// in flight when its chains start, so the field at every cathode point is the
// vacuum field and no pair sum is needed.  k_mh_vacuum runs the start and all
// jumps of such a diode's chains in one launch (one cluster of RD_VAC_CTAS
// CTAs); the tiled jump kernels skip it (planner mode PM_MH).
#define RD_VAC_CTAS 8
#define RD_VAC_THREADS 512
#define RD_VAC_CPT 2          // chains per thread, kept in registers
#define RD_VAC_MAX_CHAINS (RD_VAC_CTAS * RD_VAC_THREADS * RD_VAC_CPT)
#define RD_VAC_WTAB 512       // supply-target table entries staged in shared memory
#define RD_VAC_MAXJ 1024      // jumps whose step-size schedule a uniform work function precomputes
#define RD_VU_CHAINS 32       // chains per block of k_mh_vacuum_uniform (one lane each)
#define RD_VU_THREADS 128     // its threads (all draw the Gaussian pairs)
#define RD_VU_JCHUNK 64       // jumps whose Gaussian pairs a block holds at once
#ifdef __CUDACC__
__host__ __device__ inline bool rd_mh_vacuum(const DiodeParams& p, const DiodeDyn& y) {
  return p.geometry == RD_G_PLANAR && p.emission && !p.mh_serial && y.n == 0 && y.chains <= RD_VAC_MAX_CHAINS;
}
#endif

// Particle pool (device pointers).
struct Pool {
  double *x, *y, *z, *vx, *vy, *vz;
  double *ax, *ay, *az, *bx, *by, *bz, *cx, *cy, *cz;   // acc cur / prev / prev2
  double *q, *m;
  int *species, *id, *step0, *section, *mask;
  float4 *pk_hi, *pk_lo, *ip_hi, *ip_lo;
  // cathode-field pack (planar): zk_hi = (x_hi, y_hi, max(z^2, tiny), q z),
  // zk_lo = (x_lo, y_lo, z, q), nm, z as one float (relative precision 6e-8)
  float4 *zk_hi, *zk_lo;
};

// Device event log (rd_events_take): rd_event records appended by atomic
// index; records past `cap` are only counted.
struct EventLog {
  rd_event* buf;   // null: no log
  int* count;
  int cap;
};

// One unit of a pair-sum: i-tile (or point block) x j-chunk of one diode.
struct WorkItem {
  int diode;
  int i0;        // first i (particle or point) of the tile
  int j0, j1;    // particle range of the chunk
  int tile;      // index of the tile among the diode's tiles (partials)
  int chunk, nchunks;
  int slot;      // global tile slot for partial / counter storage
};

// MH chain state (per diode, chains at [choff_d, choff_d + max_chains)).
struct ChainState {
  double *x, *y;         // planar: position; tip: xi, phi
  double *F, *sup, *df;  // field (z or normal), log target, escape (log for planar)
  double *px, *py;       // proposal
  double *pF;            // proposal field
  int *ok;
  double *tx, *ty, *tz;  // tip: cartesian position of the current state
  double *pxx, *pyy, *pzz;  // tip: cartesian position of the proposal
  int *prop_ok;          // proposal inside the domain
  int *em;               // emits this step (k_emit_test)
  double *gx, *gy;       // planar: Gaussian pair of the next proposal
  // FP32-compensated planar chains: position as FP32 nm offsets from the
  // emitter centre (the chain lives on that grid), the target's rho and the
  // field as floats (mh_decide_f), Gaussian pair
  float *fx, *fy, *fsup, *fF, *fgx, *fgy;
  // FP32-compensated tip chains: the proposal packed once per jump for the
  // field tiles (the point on the FP32 nm grid and the high words of its
  // apex-sphere image)
  float4 *pph, *pih;
};
