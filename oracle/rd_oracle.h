/*
 * rd_oracle.h -- CPU FP64 restatement of RUMDEED's time-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU
 * library: only tests/, __graft_entry__.smoke() and the cpu_baseline /
 * --impl reference legs of bench.py may load it.  The product path never
 * links or calls it.
 *
 * Every routine restates one reference routine (Fortran, NanoPhysicsCenter/
 * RUMDEED, src/...) and cites it.  Arrays follow the reference layout:
 * particle vectors are (3, N) column-major, i.e. x,y,z interleaved per
 * particle, in SI units (m, m/s, m/s^2, C, kg).
 *
 * Parity pin: the restatement is checked against every golden value and
 * known-answer test of src/mod_tests.F90 (tests/test_oracle_golden.py).
 * The Fortran reference itself cannot be compiled here (no Fortran
 * compiler, and the third-party Cuba 4.2.2 library it links is not
 * vendored), so those golden values are the pin.
 */
#ifndef RD_ORACLE_H
#define RD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- constants, src/mod_global.F90:26-45,72-73,333 and
 *      src/mod_field_emission_v2.F90:36-47 ---------------------------------- */
typedef struct {
  double pi, h, c, mu_0, epsilon_0, m_u, h_bar, m_0, q_0, m_N2, m_N2p;
  double length_scale, time_scale, div_fac_c;
  double a_FN, b_FN, l_const;
} orc_constants;
void orc_get_constants(orc_constants* out);

enum { ORC_PLANAR = 1, ORC_TIP = 2 };
enum { ORC_ELEC = 1, ORC_ION = 2, ORC_ATOM = 3 };
enum { ORC_REMOVE_TOP = 1, ORC_REMOVE_BOT = 2 };
#define ORC_MAX_LIFE 1000

/* ---- FN functions (planar, src/mod_field_emission_v2.F90:515-625) ------- */
double orc_v_y(double F, double phi, int image_charge);
double orc_t_y(double F, double phi, int image_charge);
double orc_escape_prob_log(double F, double phi, int image_charge);
double orc_elec_supply_log(double F, double phi, int image_charge);
double orc_elec_supply_v2(double F, double phi, int image_charge, double time_step);

/* ---- work function checkerboard (src/mod_work_function.F90:389-487) ---- */
double orc_work_checkerboard(const double* w_arr, int x_num, int y_num,
                             const double em_pos[2], const double em_dim[2],
                             double x, double y, int* sec);

/* ---- Philox4x32-10 counter RNG (Salmon et al., SC'11) shared bit-for-bit
 *      with the GPU library so MH chains can be compared exactly ------------ */
void orc_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double orc_u01_from_words(uint32_t a, uint32_t b);

/* ---- the diode (one emitter, one geometry) ------------------------------- */
typedef struct {
  int geometry;             /* ORC_PLANAR / ORC_TIP */
  double V_s, d, E_z;       /* volts, gap (m), vacuum field (V/m) */
  double box_dim[3];
  double time_step, time_step2;
  int image_charge, N_ic_max;
  /* planar emitter (src/mod_global.F90:215-220) */
  double em_pos[2], em_dim[2];
  int work_nx, work_ny;
  double work[64 * 64];     /* row 0 = top row, like w_theta_arr(1,:) */
  /* tip parameters (src/mod_hyperboloid_tip.f90:11-21) */
  double d_tip, R_base, h_tip;
  double a_foci, theta_tip, r_tip, eta_1, max_xi, shift_z;
  double pre_fac_E_tip, pre_fac_E_tip_unit_voltage;
  double tip_phi;           /* tip work function, eV */
  /* particles, (3, cap) layout */
  int cap, n, nrID;
  double *pos, *vel, *acc, *acc_prev, *acc_prev2;
  double *charge, *mass;
  int *species, *mask, *id, *step_created, *section;
  /* per-step bookkeeping */
  int n_remove, n_remove_top, n_remove_bot;
  long long emitted_total, absorbed_top_total, absorbed_bot_total, dropped_total;
  int emitted_step;
  double ramo_current;      /* ramo_current(species_elec) of the last step */
  double avg_elec_vel[3];
  long long life_time[ORC_MAX_LIFE][3];
  /* emission state (src/mod_field_emission_v2.F90:57-58; per emitter residual) */
  int emission;             /* 0 off, 1 field emission */
  double MH_std, a_rate, residual, N_sup;
  uint64_t seed;
  int mh_jumps, max_chains, quad_panels, quad_order;
  int init_rounds_max;      /* 10000 in the reference */
  int last_chains, last_failed_chains;
  /* work-function model (Read_work_function types): 1 checkerboard (work =
   * matrix), 2 Gaussian (work = base, then A, x_c, y_c, std_x, std_y per
   * Gaussian, work_nx of them), 4 Voronoi (work = x, y fractions of the
   * emitter, phi, section per site, work_nx of them) */
  int work_model;
  int emit_delay;           /* emitters_delay: emission from step emit_delay + 1 on */
  int mh_serial;            /* 1: mh_batch = .false. (chains one after another) */
  int emitter_type;         /* 2 rectangle, 4 ring (centred on the axis) */
  double ring_rmin, ring_thick;
  double F_avg_z, df_avg;   /* field.dt: mean cathode F_z of the supply points, sum exp(D) / N_sup */
  /* two-time-step integrator (atom_time_interval, src/main.F90:391-395): 0 off */
  int atom_time_interval;
  double ramo_current_ion;  /* ramo_current(species_ion) of the last step */
  /* Average_Velocities (src/mod_verlet.F90:428-447) of the last velocity update and the
   * particle counts it divides by (before removal); avg_elec_vel is above */
  double avg_part_vel[3], avg_ion_vel[3], avg_mob;
  int n_part_vel, n_elec_vel, n_ion_vel;
  double F_avg_x, F_avg_y;  /* field.dt: mean lateral field of the supply points (0 with image charges) */
} orc_diode;

/* Create / destroy.  Geometry parameters follow Init_Field_Emission_v2
 * (src/mod_field_emission_v2.F90:113-135) and Init_Emission_Tip
 * (src/mod_emission_tip.f90:81-127). */
orc_diode* orc_diode_new(int geometry, int cap, double V_s, double d,
                         double time_step, int image_charge, int N_ic_max);
void orc_diode_free(orc_diode* s);
void orc_set_planar_emitter(orc_diode* s, double x0, double y0, double Lx, double Ly,
                            int work_nx, int work_ny, const double* work);
void orc_set_tip(orc_diode* s, double d_tip, double R_base, double h_tip, double phi);
/* A Gaussian (model 2) or Voronoi (model 4) work function on the planar emitter;
 * n Gaussians / sites, parameters laid out as in orc_diode.work. */
void orc_set_work_model(orc_diode* s, int model, int n, const double* params);
/* A ring emitter (EMIT_RING): outer radius r_out, radial width thickness
 * (emitters_ring, src/main.F90:363-371); sampled serially
 * (Metropolis_Hastings_ring_J).  Call after orc_set_planar_emitter. */
void orc_set_ring(orc_diode* s, double r_out, double thickness);
/* w_theta_gaussian (src/mod_work_function.F90:214-254) and w_theta_voronoi
 * (:533-571; sites as fractions of the emitter, converted as in
 * Read_work_function :124-134). */
double orc_work_gaussian(const double* w, int n, double x, double y);
double orc_work_voronoi(const double* w, int n, const double em_pos[2], const double em_dim[2],
                        double x, double y, int* sec);
void orc_set_emission(orc_diode* s, int on, uint64_t seed, int mh_jumps, int max_chains,
                      int quad_panels, int quad_order);
void orc_reset(orc_diode* s);  /* Setup_Test_System, src/mod_tests.F90:324-403 */

/* Particle bookkeeping (src/mod_pair.F90) */
int orc_add_particle(orc_diode* s, const double pos[3], const double vel[3], int species,
                     int step, int sec);
void orc_mark_remove(orc_diode* s, int i, int why);
void orc_remove_particles(orc_diode* s, int step);

/* Vacuum fields */
void orc_field_E(const orc_diode* s, const double p[3], double out[3]);
void orc_E_zunit(const orc_diode* s, const double p[3], double out[3]);

/* Image-charge kernels */
void orc_force_image_planar(const orc_diode* s, const double p1[3], const double p2[3],
                            double out[3]);
void orc_sphere_ic_field(const orc_diode* s, const double p1[3], const double p2[3],
                         double out[3]);

/* Accelerations: three restatements of the same physics.
 *  generic : half-pair loop through the geometry functions (:625-751)
 *  planar  : half-pair loop with the planar series inlined (:763-884)
 *  gather  : per-particle gather with the index-order image roles (:1217-1429)
 * All add the vacuum field term; they write acc (3, n), overwriting it.
 * compensated != 0 sums with Neumaier compensation per component. */
void orc_accel_generic(const orc_diode* s, double* acc, int compensated);
void orc_accel_planar(const orc_diode* s, double* acc, int compensated);
void orc_accel_gather(const orc_diode* s, double* acc, int compensated);
/* The gather for the listed particles only: acc3 (3, nrows), row k = particle rows[k]. */
void orc_accel_rows(const orc_diode* s, int nrows, const int* rows, double* acc3, int compensated);

/* Field at points (Calc_Field_at, :1466-1529; batch semantics :1635-1911) */
void orc_field_at(const orc_diode* s, const double p[3], double out[3], int compensated);
void orc_field_at_batch(const orc_diode* s, int M, const double* pts, double* out,
                        int compensated);

/* Integrator pieces (src/mod_verlet.F90) */
void orc_update_position(orc_diode* s);  /* Update_ElecIon_Position :197-232 */
void orc_update_velocity(orc_diode* s);  /* Update_ElecIon_Velocity :449-509 + :428-447 */
void orc_velocity_verlet(orc_diode* s, int step);  /* :123-162 (accel via gather) */
/* Two-time-step routines (atom_time_interval > 0): Update_Species_Position
 * :234-290, Update_Elec_Acceleration + Update_Ion_Acceleration :886-1151 (adds
 * to acc), Update_Species_Velocity :511-590. */
void orc_update_position_tts(orc_diode* s, int step);
void orc_accel_tts(orc_diode* s, int step, int compensated);
void orc_update_velocity_tts(orc_diode* s, int step);

/* Emission (device algorithm restated with the shared Philox streams) */
double orc_supply_integral_planar(orc_diode* s);
/* Panels per side of the planar supply rule: quad_panels, or when 0 the
 * resolution rule (nodes at most 5 nm apart, 16 to 256 panels). */
int orc_supply_panels(const orc_diode* s);
/* The same supply integral integrated adaptively to convergence (rectangle
 * emitter): panels of the quad_panels x quad_order rule bisected while their
 * Gauss-Legendre sums change by more than their share of tol (electrons) or
 * while an electron lower than half a panel width sits over them; at most
 * max_depth levels.  evals gets the integrand evaluations. */
double orc_supply_planar_converged(orc_diode* s, double tol, int max_depth, long long* evals);
void orc_mh_batch_planar(orc_diode* s, int step, int M, double* df_out, double* F_out,
                         double* pos_out, int* ok_out);
int orc_do_emission_planar(orc_diode* s, int step);
double orc_supply_tip(orc_diode* s);
void orc_mh_batch_tip(orc_diode* s, int step, int M, double* df_out, double* F_out,
                      double* pos_out, int* ok_out);
int orc_do_emission_tip(orc_diode* s, int step);
int orc_do_emission(orc_diode* s, int step);

/* One main-loop iteration (src/main.F90:175-219): emit, Update_Position,
 * Remove_Particles. */
void orc_step(orc_diode* s, int step);

/* Tip geometry helpers (src/mod_hyperboloid_tip.f90:25-163) */
void orc_tip_xyz(const orc_diode* s, double xi, double eta, double phi, double out[3]);
double orc_tip_eta(const orc_diode* s, double x, double y, double z);
void orc_tip_surface_normal(const orc_diode* s, const double p[3], double out[3]);
double orc_tip_area(const orc_diode* s, double xi1, double xi2, double phi1, double phi2);

/* CPU baseline: OpenMP restatement of the reference CPU pair loop
 * (Calculate_Acceleration_Particles_Planar, src/mod_verlet.F90:763-884),
 * parallel over i with per-thread accumulation arrays. */
void orc_accel_planar_omp(int n, const double* pos, const double* charge, const double* mass,
                          double E_z, double d, int image_charge, int N_ic_max, double* acc);
int orc_omp_threads(void);

#ifdef __cplusplus
}
#endif
#endif
