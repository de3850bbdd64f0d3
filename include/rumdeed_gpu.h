/*
 * rumdeed_gpu.h -- C ABI of librumdeed_gb300, the GB300 (sm_103a)
 * implementation of RUMDEED's time-step hot path.
 *
 * The reference (NanoPhysicsCenter/RUMDEED, Fortran 2008) exposes this path
 * as Fortran module procedures that share state through module globals.  Each
 * entry point below replaces one of them, and a Fortran iso_c_binding
 * interface module binds them under the old procedure names.
 *
 * Conventions
 *  - Every function returns an int status: RD_OK (0) or a negative RD_ERR_*.
 *    rd_last_error() returns a message for the last failure of the calling
 *    thread.  No function aborts the process.
 *  - Handles are opaque; device state is owned by the library.  Host pointers
 *    are borrowed for the duration of the call only.
 *  - Vectors use the reference layout: (3, N) column-major, i.e. x, y, z of a
 *    particle (or point) are consecutive.  Units are SI (m, m/s, m/s^2, C, s).
 *  - Calls on one engine are not thread-safe; use one host thread per engine
 *    (the reference calls in from one thread as well).
 *  - Indices are 0-based (the reference's are 1-based).
 */
#ifndef RUMDEED_GPU_H
#define RUMDEED_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  RD_OK = 0,
  RD_ERR_INVALID = -1,   /* bad argument */
  RD_ERR_CUDA = -2,      /* CUDA runtime error (message in rd_last_error) */
  RD_ERR_NOMEM = -3,     /* device allocation failed */
  RD_ERR_CAPACITY = -4,  /* no diode slot / pool range / chain range free */
  RD_ERR_STATE = -5,     /* call not valid in the current state */
  RD_ERR_NOTFOUND = -6   /* unknown diode */
};

enum { RD_GEOM_PLANAR = 1, RD_GEOM_TIP = 2 };
enum { RD_PREC_FP64 = 0, RD_PREC_FP32C = 1 };
enum { RD_SPECIES_ELEC = 1, RD_SPECIES_ION = 2, RD_SPECIES_ATOM = 3 };
enum { RD_REMOVE_TOP = 1, RD_REMOVE_BOT = 2 };

typedef struct rd_engine rd_engine;

/* Engine: one GPU, a pool of diode slots sharing one particle pool. */
typedef struct {
  int device;                   /* CUDA device ordinal */
  int precision;                /* RD_PREC_FP64 (plain) or RD_PREC_FP32C (compensated) */
  int max_diodes;               /* diode slots */
  long long particle_capacity;  /* particle pool size (sum of diode capacities) */
  long long chain_capacity;     /* MH chain pool size (sum of per-diode chain caps) */
  long long quad_capacity;      /* supply quadrature points over all diodes */
  int chunk_min;                /* j-chunk length floor of the pair sums, particles, a
                                   multiple of 128 (0 = 1024); see rd_autotune */
  int grid_blocks;              /* persistent grid size (0 = per kernel: resident blocks per
                                   SM at its occupancy x SM count) */
  int chunk_count_max;          /* at most this many j-chunks per i-tile, 1..32 (0 = 32) */
  int event_capacity;           /* records the event log holds between two rd_events_take
                                   calls (0 = no event log); see rd_events_take */
} rd_engine_config;

/* One diode (the namelist /input/ of one run, src/mod_global.F90:426-439). */
typedef struct {
  int geometry;            /* RD_GEOM_PLANAR or RD_GEOM_TIP */
  double V_s;              /* voltage over the gap (V) */
  double gap;              /* planar gap d = box_dim(3) (m); tips use d_tip + h_tip */
  double time_step;        /* s */
  int image_charge;        /* 0/1 */
  int N_ic_max;            /* image partners: 1 + 4*N_ic_max */
  int capacity;            /* MAX_PARTICLES of this diode */
  double emitter_pos[2];   /* planar emitter lower-left corner (m) */
  double emitter_dim[2];   /* planar emitter size (m) */
  int work_nx, work_ny;    /* checkerboard work function grid (1 x 1 = uniform); see work_model */
  const double* work;      /* work_ny x work_nx values in eV, row 0 = top row; see work_model */
  double tip_dim[3];       /* tip (d_tip, R_base, h_tip) in m */
  double tip_work_function;/* eV (the reference hard-codes 4.7) */
  int emission;            /* 0: no emission; 1: Fowler-Nordheim field emission */
  int mh_jumps;            /* 0: reference default (200 planar, 80 tip) */
  int max_chains;          /* MH chains per step at most (0: capacity) */
  int quad_panels;         /* planar supply rule: panels per side (0: enough panels for nodes at
                              most 5 nm apart along the longer emitter side, 16 to 256; see
                              rd_supply_points) */
  int quad_order;          /* planar supply rule: Gauss-Legendre order (0: 4) */
  int init_rounds;         /* MH start-position rounds (0: 10000 as the reference) */
  unsigned long long seed; /* Philox key of this diode */
  int work_model;          /* planar work-function model (Read_work_function's types,
                              src/mod_work_function.F90:53-152): 0 or 1 checkerboard
                              (work = work_ny x work_nx values, eV); 2 Gaussian (work =
                              base eV, then A eV, x_c, y_c, std_x, std_y nm per Gaussian;
                              work_nx = the number of Gaussians); 4 Voronoi (work = x, y
                              as fractions of the emitter, phi eV, section per site;
                              work_nx = the number of sites) */
  int emitter_delay;       /* the emitter emits from step emitter_delay + 1 on
                              (EMITTERS_DELAY, src/mod_field_emission_v2.F90:181) */
  int planes_N;            /* measurement planes, at most 10 (planes_N, planes_z of the
                              namelist); particles crossing one upwards are logged */
  double planes_z[10];     /* plane heights (m); <= 0: plane unused */
  int mh_serial;           /* planar MH sampler: 0 batched (chains in lockstep, mh_batch =
                              .true.), 1 serial (mh_batch = .false., the reference's default:
                              each chain runs to completion, sees the electrons earlier
                              chains of the step emitted and updates MH_std once) */
  int emitter_type;        /* planar emitter shape (EMITTERS_TYPE, src/mod_global.F90:265-268):
                              0 or 2 rectangle, 1 circle (sampled over its bounding box, as the
                              reference does), 4 ring centred on the axis: outer radius
                              emitter_dim[0], radial width emitter_thickness; a ring always
                              uses the serial sampler (Metropolis_Hastings_ring_J) */
  double emitter_thickness;/* ring width (m); 0: sqrt(q0 d / (pi eps0 V)) as the reference
                              (src/main.F90:363-371) */
  int atom_time_interval;  /* two-time-step integrator (atom_time_interval of the namelist,
                              src/main.F90:391-395): 0 off; T > 0: electrons move every step,
                              ions only on steps divisible by T with the step T*time_step, and
                              the ions' acceleration gathers the electron forces of every step
                              in between (src/mod_verlet.F90:183-194,234-290,403-416,511-590,
                              886-1151) */
} rd_diode_config;

typedef struct {
  int n;                   /* particles in flight */
  int emitted_step, dropped_step, absorbed_top_step, absorbed_bot_step;
  int chains, chains_failed, chains_capped;
  long long emitted_total, dropped_total, absorbed_top_total, absorbed_bot_total;
  long long electron_steps, steps_done;
  double ramo_current;     /* ramo_current(species_elec) of the last step (A) */
  double N_sup, MH_std, a_rate, residual;
  double F_avg[3];         /* mean cathode field over the supply evaluation points
                              (field.dt, src/mod_field_emission_v2.F90:644-651) */
  double df_avg;           /* sum of the candidates' escape probabilities / N_sup (:354,385) */
  double ramo_current_ion; /* ramo_current(species_ion) of the last step (A) */
  double avg_part_vel[3], avg_elec_vel[3], avg_ion_vel[3];   /* Average_Velocities of the last
                              step (src/mod_verlet.F90:428-447): velocity sums of the particles the
                              step moved over the counts below (m/s) */
  double avg_mob;          /* |avg_elec_vel| / (-E_z) (m^2/(V s)) */
  int n_part_vel, n_elec_vel, n_ion_vel;   /* nrPart, nrElec, nrIon at the velocity update, before
                              removal (the counts Write_Ramo_Current writes) */
} rd_counters;

const char* rd_last_error(void);
int rd_version(void);

/* Engine lifetime (Init / Particles_To_Device residency, src/main.F90:416-741,
 * src/mod_verlet.F90:71-111: state is resident for the engine's lifetime). */
int rd_engine_create(const rd_engine_config* cfg, rd_engine** out);
int rd_engine_destroy(rd_engine* e);
int rd_sync(rd_engine* e);

/* Diode slots.  rd_diode_add performs Init_Field_Emission_v2
 * (src/mod_field_emission_v2.F90:113-135) or Init_Emission_Tip
 * (src/mod_emission_tip.f90:81-127) for the new slot. */
int rd_diode_add(rd_engine* e, const rd_diode_config* cfg, int* diode);
int rd_diode_remove(rd_engine* e, int diode);
int rd_diode_count(rd_engine* e, int* active);

/* Add_Particle (src/mod_pair.F90:29-159) for n particles in order: appended
 * at the end, charge/mass by species, Beeman history seeded with
 * (q/m) E_vac(x); particles beyond the capacity are counted as dropped. */
int rd_add_particles(rd_engine* e, int diode, int n, const double* pos3n, const double* vel3n,
                     const int* species, int step, int section);

/* Full state snapshot out (any pointer may be NULL); n_out gets the count.
 * Arrays must hold `cap` particles. */
int rd_get_particles(rd_engine* e, int diode, int cap, double* pos3n, double* vel3n,
                     double* acc3n, double* charge, int* id, int* section, int* n_out);

/* Overwrite positions / velocities / the three acceleration histories of the
 * first n particles (snapshot in; any pointer may be NULL). */
int rd_set_particles(rd_engine* e, int diode, int n, const double* pos3n, const double* vel3n,
                     const double* acc3n, const double* acc_prev3n, const double* acc_prev23n);

/* Calculate_Acceleration_Particles (src/mod_verlet.F90:597-620): sets the
 * current acceleration of every particle of every diode from the current
 * positions; copies diode `diode`'s (3, n) result to acc3n if not NULL. */
int rd_accel(rd_engine* e, int diode, double* acc3n);

/* Calc_Field_at_Batch (src/mod_verlet.F90:1635-1911): field (V/m) at M
 * points of one diode. */
int rd_field_at(rd_engine* e, int diode, int M, const double* pos3m, double* field3m);

/* Supply quadrature points a diode of this configuration takes in the
 * engine's quadrature table (rd_engine_config.quad_capacity): (panels x
 * order)^2 for a planar emitter, 10000 for a tip, 0 without emission.  The
 * supply integral (Do_Surface_Integration_FE, src/mod_field_emission_v2.F90:
 * 635-656) is a composite Gauss-Legendre rule here in place of the reference's
 * adaptive Cuba integrator. */
int rd_supply_points(const rd_diode_config* c, long long* npts);

/* Mark_Particles_Remove (src/mod_pair.F90:169-339), for tests and drivers. */
int rd_mark_remove(rd_engine* e, int diode, int index, int why);

/* The main-loop phases for all diodes (src/main.F90:175-219):
 *   rd_do_emission     ptr_Do_Emission (Do_Field_Emission / Do_Emission_Tip)
 *   rd_update_position Update_Position (Velocity_Verlet, mod_verlet.F90:123-162)
 *   rd_remove_particles Remove_Particles (mod_pair.F90:352-562)
 *   rd_step            the three in order, as one captured CUDA graph
 *   rd_run             nsteps consecutive rd_step calls, steps first..first+nsteps-1
 * The compaction works in place: each 1024-particle tile waits, with a bounded
 * number of polls, until the earlier tiles it overwrites have read their
 * particles.  Those waits always end in a working run; if one ever gave up,
 * rd_remove_particles, rd_run, rd_serve, rd_profile_step and rd_time_remove
 * return RD_ERR_STATE, and the particle state is no longer valid. */
int rd_do_emission(rd_engine* e, int step);
int rd_update_position(rd_engine* e, int step);
int rd_remove_particles(rd_engine* e, int step);
int rd_step(rd_engine* e, int step);
int rd_run(rd_engine* e, int first_step, int nsteps);

int rd_counters_get(rd_engine* e, int diode, rd_counters* out);
/* Life-time histogram of removed electrons: hist[k] = electrons that lived
 * k+1 steps (record_lifetime, src/mod_pair.F90:1135-1160), 1000 entries. */
int rd_life_time(rd_engine* e, int diode, int* hist1000);

/* Checkpoint of one diode between steps: its counters and emission state
 * (MH_std, residual, ids), every particle (positions, velocities, the three
 * acceleration histories, charge, mass, species, id, creation step, section)
 * and its life-time histogram.  rd_diode_state_size gives the bytes;
 * rd_diode_save writes them to a caller buffer; rd_diode_load puts them into a
 * diode slot added with the same rd_diode_config (here or in another engine),
 * after which stepping on from the saved step gives the same results as the
 * run that was saved.  The reference has no restart file; this serves
 * eviction and re-admission of long requests and resuming runs. */
/* State invariants of every resident diode, checked on the device between
 * steps (a sanitizer-like self check; the counts do not stop anything):
 * counts[k] = violations of kind k summed over the diodes, k = 0 particle count
 * outside [0, capacity], 1 removal bookkeeping not cleared, 2 unknown
 * species, 3 particle still marked for removal, 4 non-finite position /
 * velocity / acceleration, 5 ids not strictly increasing within a diode,
 * 6 charge or mass not those of the species.  *total = their sum. */
enum { RD_VALIDATE_KINDS = 7 };
int rd_validate(rd_engine* e, int counts[7], long long* total);

int rd_diode_state_size(rd_engine* e, int diode, long long* bytes);
int rd_diode_save(rd_engine* e, int diode, void* buf, long long cap, long long* written);
int rd_diode_load(rd_engine* e, int diode, const void* buf, long long size);

/* Timing of the last rd_run: device milliseconds (CUDA events on the engine
 * stream) and launches of library kernels per step. */
int rd_last_run_stats(rd_engine* e, double* ms, int* kernels_per_step);

/* ---- field at points without allocation -----------------------------------
 * No counterpart in the reference.  The same field evaluation as rd_field_at,
 * for callers that cannot allocate device memory at the time of the call:
 * host codes whose device memory belongs to another runtime (an OpenACC
 * driver passing acc_deviceptr of its own buffers), processes with a fixed
 * device-memory budget, latency-critical loops.  The points and the result
 * are caller-owned DEVICE buffers, (3, M) doubles each; all working memory
 * of the call is a static 16 MiB device array inside the library, held by
 * every GPU that loads it until the process exits.  M may be at most 65536
 * (RD_ERR_INVALID otherwise).  rd_engine_create does the set-up: it loads the
 * module that holds the array and the kernels the call launches, and resolves
 * the array's device address on the engine's device, so no call commits
 * device memory, even under lazy module loading.  The call runs on the
 * engine's own stream, which is not ordered after the caller's streams: the
 * points must be completely written (device- or stream-synchronised) before
 * the call.  All calls share the array: calls that overlap on the GPU race,
 * so issue them one after another.  Returns after the result is written
 * (synchronises the engine stream). */
int rd_field_at_noalloc(rd_engine* e, int diode, int M, const double* pos3m_dev,
                        double* field3m_dev);

/* ---- tracing: per-phase device times of one step --------------------------
 * The reference has only wall-clock stamps at start and end of the run
 * (src/main.F90:51,267).  rd_profile_step runs one main-loop iteration
 * uncaptured with CUDA events between the phases and reports their device
 * times and work. */
typedef struct {
  double supply_ms, mh_init_ms, mh_jumps_ms, emit_ms;
  double position_ms, force_ms, velocity_ms, compact_ms, total_ms;
  int mh_jump_launches;
  long long mh_pair_evals;   /* sum over jump launches of chains x particles */
  long long force_pairs;     /* sum over diodes of n (n - 1) */
  long long supply_pair_evals;
} rd_phase_times;
int rd_profile_step(rd_engine* e, int step, rd_phase_times* out);

/* ---- kernel timing (measurement only; no counterpart in the reference) ----
 * rd_time_accel: device time of one all-pair force evaluation of every
 * resident diode (work plan + pair kernel, as inside a step), averaged over
 * `reps` back-to-back evaluations timed with CUDA events on the engine
 * stream.  rd_time_field_at: the same for the field at M points of one diode
 * (points uploaded once, before the timed region; plan + field kernel per
 * evaluation).  Both leave the particle state unchanged. */
int rd_time_accel(rd_engine* e, int reps, double* ms_per_eval);
int rd_time_field_at(rd_engine* e, int diode, int M, const double* pos3m, int reps,
                     double* ms_per_eval);
/* rd_time_verlet: device time of one Beeman position pass (k_position, with
 * the boundary checks and FP32 packs) and of one velocity pass (k_velocity +
 * the Ramo reduction) over every resident particle, averaged over `reps`
 * passes each.  Unlike the two timers above it advances the particle state
 * (positions, velocities, histories): a measurement of the HBM-bound kernels
 * on a snapshot that is thrown away. */
int rd_time_verlet(rd_engine* e, int reps, double* position_ms, double* velocity_ms);
/* rd_time_remove: device time of one Beeman position pass (which marks the
 * particles that crossed an electrode, Check_Boundary_Planar ->
 * Mark_Particles_Remove) and of the removal that follows it (the stable
 * compaction of Remove_Particles, src/mod_pair.F90:352-562, with its life-time
 * record), one launch each, CUDA events on the engine stream.  moved gets the
 * survivors the compaction moved (those behind a diode's first removed
 * particle), removed the particles removed.  Advances the state like the two
 * phases of a step, without the force and velocity passes. */
int rd_time_remove(rd_engine* e, double* position_ms, double* remove_ms, long long* moved, long long* removed);

/* ---- event log: emission and absorption records ------------------------------
 * The reference writes one record per emitted particle (density_emit.bin and
 * density_emit_elec.bin, src/mod_pair.F90:89-123, at Add_Particle) and one per
 * electron absorbed at the anode or the cathode (density_absorb_top.bin /
 * density_absorb_bot.bin, :241-257, at Mark_Particles_Remove) as the events
 * happen.  With rd_engine_config.event_capacity > 0 the step kernels append
 * the same data to a device log: position (m) and velocity (m/s) at the event
 * (emission: the placement point, velocity 0; absorption: after the position
 * update that crossed the electrode), diode, kind, section, particle id,
 * species and the diode's step.  rd_events_take copies the records logged
 * since the last take into `out` (at most `cap`), ordered by diode, kind and
 * id, empties the log and reports records that did not fit (the log's or the
 * caller's capacity) in n_lost. */
enum { RD_EVENT_EMIT = 1, RD_EVENT_ABSORB_TOP = 2, RD_EVENT_ABSORB_BOT = 3,
       RD_EVENT_PLANE = 16 /* + plane index k: crossed plane k upwards (planes-(k+1).bin,
                              Check_Planes, src/mod_verlet.F90:343-367) */ };
typedef struct {
  double pos[3], vel[3];
  int diode, kind, section, id, species, step;
} rd_event;
int rd_events_take(rd_engine* e, int cap, rd_event* out, int* n_out, long long* n_lost);

/* ---- autotuner (no counterpart in the reference) ----------------------------
 * Every pair sum (forces, cathode fields, MH jumps) cuts an i-tile's j range
 * into chunks of max(chunk_min, ceil(n / chunk_count_max)) particles (rounded
 * up to 128): longer chunks mean fewer partial sums, shorter ones a shorter
 * tail at the end of a launch.  The chunking depends only on a diode's own
 * counts and these two numbers, so a diode's results are the same alone and
 * in any mix under the same chunking; different chunkings differ in the last
 * FP32 bits.  rd_autotune times every candidate chunking on the diodes
 * resident now -- the force pass and a dry MH pass (the field at every
 * chain's current point, nothing written) weighted by the jump count --
 * keeps the fastest, then times the MH launch shapes (rd_set_mh_launch) under
 * it, rebuilds the step graph and leaves the particle state as it was.
 * rd_set_chunking sets one directly (0 = default).  The i-tile width (128
 * particles, points or chains per work item) is fixed. */
typedef struct {
  int chunk_min, chunk_count_max;   /* the chosen chunking */
  double ms_default, ms_chosen;     /* estimated step pair-sum time under the default / chosen */
  int candidates;
  int mh_parts, mh_form;            /* the chosen MH launch shape (rd_set_mh_launch) */
} rd_tune_result;
int rd_autotune(rd_engine* e, rd_tune_result* out);
int rd_set_chunking(rd_engine* e, int chunk_min, int chunk_count_max);
int rd_get_chunking(rd_engine* e, int* chunk_min, int* chunk_count_max);
/* Launch shape of the planar MH jumps, which changes no result: `parts`
 * launches per jump on as many streams, each over a part of the work plan cut
 * at diode boundaries (1..4; 0 = 2, used only when two or more diodes run
 * batched chains), and the FP32 thread form (0: 32 threads x 4 chains per
 * 128-chain tile, 1: 64 threads x 2 chains; -1 = form 1 for a single emitting
 * planar diode, else form 0).  rd_autotune searches both after the chunking;
 * rd_get_mh_launch reports what the next step uses. */
int rd_set_mh_launch(rd_engine* e, int parts, int form);
int rd_get_mh_launch(rd_engine* e, int* parts, int* form);

/* ---- serving: continuous batching of diode simulations ---------------------
 * The reference runs one simulation per process.  Requests queue in FIFO
 * order; rd_serve admits the queue head whenever a diode slot, a particle-pool
 * range of its capacity (its peak electron count, i.e. HBM) and a chain range
 * are free, advances every admitted simulation by one time step per
 * iteration (one graph launch), and retires simulations that completed their
 * step count, freeing their slot for the next request.  Each simulation
 * counts its own steps from 1, so its result does not depend on what else
 * is resident. */
typedef struct {
  rd_diode_config diode;
  int steps;               /* time steps to simulate */
  int n_init;              /* initial electrons (copied at submit) */
  const double* pos3n;     /* (3, n_init) positions */
  const double* vel3n;     /* (3, n_init) velocities or NULL */
} rd_request;

enum { RD_REQ_QUEUED = 0, RD_REQ_RUNNING = 1, RD_REQ_DONE = 2, RD_REQ_CANCELLED = 3 };

typedef struct {
  int state;
  int diode;               /* slot while running, -1 otherwise */
  int steps;
  double submit_s, admit_s, done_s;   /* engine clock, seconds */
  rd_counters counters;    /* latest counters (final once done) */
} rd_request_status;

typedef struct {
  int iterations;          /* serving iterations run by the call */
  int admitted, retired, running, queued;
  double device_ms;        /* sum of per-iteration device times */
  double wall_ms;          /* host wall time of the call */
  long long electron_steps;/* electrons in flight summed over diodes and iterations */
  double step_ms_p50, step_ms_p99, step_ms_max;   /* per-iteration device time */
  long long h2d_bytes, d2h_bytes;
} rd_serve_stats;

int rd_submit(rd_engine* e, const rd_request* req, long long* id);
int rd_poll(rd_engine* e, long long id, rd_request_status* out);
int rd_cancel(rd_engine* e, long long id);
int rd_serve(rd_engine* e, int iterations, rd_serve_stats* out);
int rd_clock(rd_engine* e, double* seconds);

#ifdef __cplusplus
}
#endif
#endif
