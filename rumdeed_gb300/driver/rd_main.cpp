// rd_main -- native main-loop driver over the C ABI of librumdeed_gb300.
//
// It runs a RUMDEED input deck the way the reference's main program does
// (src/main.F90:175-219): read the /input/ namelist from the file `input`
// (src/mod_global.F90:426-439, src/main.F90:298-411) and, for planar field
// emission, the checkerboard work function from `work`
// (src/mod_work_function.F90:53-152); then for step = 1..STEPS do emission,
// Update_Position and Remove_Particles (one rd_step call) and write the
// per-step records to out/emitted.dt (src/mod_field_emission_v2.F90:202-204),
// out/absorbed{,_top,_bot}.dt (src/mod_pair.F90:789-804) and
// out/ramo_current.dt (src/mod_pair.F90:811-835) with the reference's Fortran
// edit descriptors, and the per-event binary files out/density_emit.bin,
// out/density_emit_elec.bin (src/mod_pair.F90:89-123),
// out/density_absorb_{top,bot}.bin (:241-257) and out/planes-<k>.bin
// (Check_Planes, src/mod_verlet.F90:343-367) from the engine's event log,
// out/field.dt (src/mod_field_emission_v2.F90:389-390), out/volt.dt
// (Set_Voltage, src/mod_verlet.F90:2050-2057) and, once, out/init.bin and
// out/init.dt (Write_Initial_Variables, src/main.F90:852-932).
//
// Supported decks: EMISSION_MODE = 10 (planar field emission, one emitter,
// EMITTERS_TYPE 1, 2 or 4) and EMISSION_MODE = 3 (hyperboloid tip);
// ATOM_TIME_INTERVAL > 0 selects the two-time-step integrator.  Extra, optional namelist /gb300/ in the same file: MAX_PARTICLES
// (default 20000), SEED, PRECISION (0 = FP64, 1 = FP32 compensated), MH_JUMPS,
// TIP_WORK_FUNCTION (eV, default 4.7 as the reference hard-codes), MH_SERIAL,
// MAX_CHAINS (MH chains per step at most, default 2^20: in effect every
// candidate runs, as in the reference).  The MH sampler is the reference's:
// serial unless /input/ sets MH_BATCH = .True.; MH_SERIAL = 0 or 1 overrides
// it; a ring emitter (EMITTERS_TYPE 4) is always serial.
//
//   rd_main [run directory]
#include <cctype>
#include <cmath>
#include <csignal>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <map>
#include <string>
#include <sys/stat.h>
#include <unistd.h>
#include <vector>

#include "../../include/rumdeed_gpu.h"

namespace {

// ---- namelist reader ---------------------------------------------------------------------
// Reads `&name key = v1, v2, ... /` groups: keys are upper-cased with their
// subscripts removed, values are split on commas/whitespace, `!` starts a
// comment, Fortran logicals and d-exponents are accepted.
using Group = std::map<std::string, std::vector<std::string>>;

std::map<std::string, Group> read_namelists(const char* path) {
  std::map<std::string, Group> out;
  FILE* f = std::fopen(path, "r");
  if (!f) return out;
  std::string text;
  char buf[4096];
  while (std::fgets(buf, sizeof buf, f)) {
    std::string l(buf);
    bool in_str = false;
    for (size_t i = 0; i < l.size(); ++i) {
      if (l[i] == '\'' || l[i] == '"') in_str = !in_str;
      if (l[i] == '!' && !in_str) { l.resize(i); break; }
    }
    text += l + " ";
  }
  std::fclose(f);
  size_t pos = 0;
  while ((pos = text.find('&', pos)) != std::string::npos) {
    size_t e = text.find_first_of(" \t\r\n", pos);
    if (e == std::string::npos) break;
    std::string name = text.substr(pos + 1, e - pos - 1);
    for (auto& c : name) c = (char)std::toupper((unsigned char)c);
    size_t end = text.find('/', e);
    if (end == std::string::npos) end = text.size();
    // tokens: split on commas and blanks outside parentheses; '=' is a token
    std::vector<std::string> tok;
    std::string cur;
    int depth = 0;
    for (size_t i = e; i < end; ++i) {
      const char c = text[i];
      if (c == '(') ++depth;
      if (c == ')') --depth;
      if (depth == 0 && (c == ',' || std::isspace((unsigned char)c) || c == '=')) {
        if (!cur.empty()) { tok.push_back(cur); cur.clear(); }
        if (c == '=') tok.push_back("=");
      } else {
        cur += c;
      }
    }
    if (!cur.empty()) tok.push_back(cur);
    Group g;
    std::string key;
    for (size_t i = 0; i < tok.size(); ++i) {
      if (i + 1 < tok.size() && tok[i + 1] == "=") {
        key.clear();
        for (char c : tok[i].substr(0, tok[i].find('('))) key += (char)std::toupper((unsigned char)c);
        g[key].clear();
        ++i;
      } else if (!key.empty()) {
        const size_t star = tok[i].find('*');   // repeat count r*v
        if (star != std::string::npos && star > 0) {
          const int r = std::atoi(tok[i].substr(0, star).c_str());
          for (int k = 0; k < r; ++k) g[key].push_back(tok[i].substr(star + 1));
        } else {
          g[key].push_back(tok[i]);
        }
      }
    }
    out[name] = g;
    pos = end;
  }
  return out;
}

double to_double(std::string s) {
  for (auto& c : s) if (c == 'd' || c == 'D') c = 'e';
  return std::strtod(s.c_str(), nullptr);
}

bool to_logical(std::string s) {
  for (auto& c : s) c = (char)std::toupper((unsigned char)c);
  return s.find('T') != std::string::npos;
}

double get(const Group& g, const char* k, size_t i, double dflt) {
  auto it = g.find(k);
  if (it == g.end() || it->second.size() <= i) return dflt;
  return to_double(it->second[i]);
}

// ---- Fortran edit descriptors ----------------------------------------------------------
// Ew.d: 0.ddddddE+ee right-justified in w characters.
std::string fmt_E(double v, int w, int d) {
  char m[64];
  if (v == 0.0) {
    std::snprintf(m, sizeof m, "0.%0*dE+00", d, 0);
  } else {
    int ex = (int)std::floor(std::log10(std::fabs(v))) + 1;
    double mant = std::fabs(v) / std::pow(10.0, ex);
    double scale = std::pow(10.0, d);
    double r = std::nearbyint(mant * scale);
    if (r >= scale) { r /= 10.0; ex += 1; }
    if (r < scale / 10.0) { r *= 10.0; ex -= 1; }
    std::snprintf(m, sizeof m, "%s0.%0*.0fE%c%02d", v < 0 ? "-" : "", d, r, ex < 0 ? '-' : '+', std::abs(ex));
  }
  std::string s(m);
  return std::string(s.size() < (size_t)w ? w - s.size() : 0, ' ') + s;
}

// ESw.d: d.ddddE+ee right-justified in w characters.
std::string fmt_ES(double v, int w, int d) {
  char m[64];
  std::snprintf(m, sizeof m, "%*.*E", w, d, v);
  return std::string(m);
}

std::string fmt_I(long long v, int w) {
  char m[64];
  std::snprintf(m, sizeof m, "%*lld", w, v);
  return std::string(m);
}

// SIGINT (ctrl+c) and SIGUSR1 (sent by Slurm before the time limit) stop the
// main loop cleanly after the current step, as Signal_Handler does
// (src/main.F90:214-217,289-294,531-535).
volatile std::sig_atomic_t g_stop = 0;
extern "C" void on_stop_signal(int) { g_stop = 1; }

int check(int rc, const char* what) {
  if (rc != RD_OK) {
    std::fprintf(stderr, "rd_main: %s failed (%d): %s\n", what, rc, rd_last_error());
    std::exit(2);
  }
  return rc;
}

}  // namespace

int main(int argc, char** argv) {
  bool print_only = false;
  const char* dir = nullptr;
  for (int a = 1; a < argc; ++a) {
    if (!std::strcmp(argv[a], "--print-config")) print_only = true;
    else dir = argv[a];
  }
  if (dir && chdir(dir) != 0) {
    std::fprintf(stderr, "rd_main: cannot enter %s\n", dir);
    return 2;
  }
  auto nl = read_namelists("input");
  if (!nl.count("INPUT")) {
    std::fprintf(stderr, "rd_main: ERROR UNABLE TO OPEN file input (or no &input group)\n");
    return 2;
  }
  const Group& in = nl["INPUT"];
  const Group gb = nl.count("GB300") ? nl["GB300"] : Group();
  const double length_scale = 1.0e-9, time_scale = 1.0e-12;
  const double V_s = get(in, "V_S", 0, 0.0);
  const double d = get(in, "BOX_DIM", 2, 0.0) * length_scale;
  const double dt = get(in, "TIME_STEP", 0, 0.0) * time_scale;
  const int steps = (int)get(in, "STEPS", 0, 0.0);
  const int mode = (int)get(in, "EMISSION_MODE", 0, 10.0);
  const int n_ic = (int)get(in, "N_IC_MAX", 0, 0.0);
  const bool image = in.count("IMAGE_CHARGE") ? to_logical(in.at("IMAGE_CHARGE")[0]) : true;
  if (steps <= 0) { std::fprintf(stderr, "ERROR: steps <= 0\n"); return 2; }
  if (mode != 10 && mode != 3) {
    std::fprintf(stderr, "rd_main: EMISSION_MODE %d is not on this path (10: planar FE, 3: tip)\n", mode);
    return 2;
  }
  if ((int)get(in, "NREMIT", 0, 1.0) != 1) {
    std::fprintf(stderr, "rd_main: one emitter per run on this path (NREMIT = 1)\n");
    return 2;
  }

  rd_diode_config dc;
  std::memset(&dc, 0, sizeof dc);
  dc.V_s = V_s;
  dc.time_step = dt;
  dc.image_charge = image ? 1 : 0;
  dc.N_ic_max = n_ic;
  dc.capacity = (int)get(gb, "MAX_PARTICLES", 0, 20000.0);
  // every one of the step's N_round candidates runs a chain, and Add_Particle drops what does
  // not fit (src/mod_field_emission_v2.F90:283-330, src/mod_pair.F90:37-44); /gb300/ MAX_CHAINS
  // caps them (the chain pool is sized to it)
  dc.max_chains = (int)get(gb, "MAX_CHAINS", 0, (double)(1 << 20));
  if (dc.max_chains < 1) { std::fprintf(stderr, "rd_main: MAX_CHAINS must be positive\n"); return 2; }
  dc.emission = 1;
  dc.mh_jumps = (int)get(gb, "MH_JUMPS", 0, 0.0);
  dc.seed = (unsigned long long)get(gb, "SEED", 0, 20261203.0);
  dc.emitter_delay = (int)get(in, "EMITTERS_DELAY", 0, 0.0);
  dc.atom_time_interval = (int)get(in, "ATOM_TIME_INTERVAL", 0, 0.0);   // two_time_step when > 0
  if (dc.atom_time_interval < 0) { std::fprintf(stderr, "rd_main: atom_time_interval must be >= 0\n"); return 2; }
  dc.planes_N = (int)get(in, "PLANES_N", 0, 0.0);
  if (dc.planes_N < 0 || dc.planes_N > 10) { std::fprintf(stderr, "rd_main: planes_N must be in [0, 10]\n"); return 2; }
  for (int k = 0; k < dc.planes_N; ++k) dc.planes_z[k] = get(in, "PLANES_Z", k, -1.0) * length_scale;
  std::vector<double> work;
  if (mode == 10) {
    dc.geometry = RD_GEOM_PLANAR;
    dc.gap = d;
    dc.emitter_dim[0] = get(in, "EMITTERS_DIM", 0, 0.0) * length_scale;
    dc.emitter_dim[1] = get(in, "EMITTERS_DIM", 1, 0.0) * length_scale;
    dc.emitter_pos[0] = get(in, "EMITTERS_POS", 0, 0.0) * length_scale;
    dc.emitter_pos[1] = get(in, "EMITTERS_POS", 1, 0.0) * length_scale;
    dc.emitter_type = (int)get(in, "EMITTERS_TYPE", 0, 2.0);
    dc.emitter_thickness = get(in, "EMITTERS_DIM", 2, 0.0) * length_scale;   // ring width (0: from V, d)
    // the reference's default sampler is serial: mh_batch = .false. unless the deck sets
    // MH_BATCH = .true. (src/mod_global.F90:316-328); /gb300/ MH_SERIAL overrides either way
    dc.mh_serial = in.count("MH_BATCH") ? !to_logical(in.at("MH_BATCH")[0]) : 1;
    if (gb.count("MH_SERIAL")) dc.mh_serial = get(gb, "MH_SERIAL", 0, 1.0) != 0.0;
    // Read_work_function (src/mod_work_function.F90:53-152): 1 checkerboard
    // (y_num x_num, then the matrix), 2 Gaussian (base, count, then A x y sx sy
    // per line), 4 Voronoi (count, then x y phi section per line)
    FILE* wf = std::fopen("work", "r");
    if (!wf) { std::fprintf(stderr, "RUMDEED: Failed to open file work. ABORTING\n"); return 2; }
    auto next = [&](double* v) {
      char tok[64];
      if (std::fscanf(wf, "%63s", tok) != 1) return false;
      *v = to_double(tok);
      return true;
    };
    double t = 0.0, a = 0.0, b = 0.0;
    if (!next(&t)) { std::fprintf(stderr, "rd_main: empty work file\n"); return 2; }
    const int type = (int)t;
    int nx = 1, ny = 1, nvals = 0;
    if (type == 1) {
      if (!next(&a) || !next(&b)) { std::fprintf(stderr, "rd_main: short work file\n"); return 2; }
      ny = (int)a; nx = (int)b; nvals = nx * ny;
    } else if (type == 2) {
      if (!next(&a) || !next(&b)) { std::fprintf(stderr, "rd_main: short work file\n"); return 2; }
      work.push_back(a);   // base
      nx = (int)b; nvals = 5 * nx;
    } else if (type == 4) {
      if (!next(&a)) { std::fprintf(stderr, "rd_main: short work file\n"); return 2; }
      nx = (int)a; nvals = 4 * nx;
    } else {
      std::fprintf(stderr, "rd_main: work function type %d is not on this path (1, 2 or 4)\n", type);
      return 2;
    }
    if (nx < 1 || ny < 1) { std::fprintf(stderr, "rd_main: bad work file sizes\n"); return 2; }
    for (int k = 0; k < nvals; ++k) {
      double v;
      if (!next(&v)) { std::fprintf(stderr, "rd_main: short work file\n"); return 2; }
      work.push_back(v);
    }
    std::fclose(wf);
    dc.work_model = type;
    dc.work_nx = nx; dc.work_ny = ny; dc.work = work.data();   // checkerboard row 0 = first row of the file
  } else {
    dc.geometry = RD_GEOM_TIP;
    dc.tip_dim[0] = get(in, "EMITTERS_DIM", 0, 0.0) * length_scale;
    dc.tip_dim[1] = get(in, "EMITTERS_DIM", 1, 0.0) * length_scale;
    dc.tip_dim[2] = get(in, "EMITTERS_DIM", 2, 0.0) * length_scale;
    dc.gap = dc.tip_dim[0] + dc.tip_dim[2];
    dc.tip_work_function = get(gb, "TIP_WORK_FUNCTION", 0, 4.7);
  }

  if (print_only) {   // the deck as read, one "key value" line each, then stop
    std::printf("geometry %d\nV_s %.17g\ngap %.17g\ntime_step %.17g\nsteps %d\nimage_charge %d\n"
                "N_ic_max %d\ncapacity %d\nseed %llu\nemitter_pos %.17g %.17g\nemitter_dim %.17g %.17g\n"
                "work %d x %d\nwork_model %d\ntip_dim %.17g %.17g %.17g\nE14.6 %s\nES12.4 %s\n"
                "emitter_delay %d\nplanes %d\nemitter_type %d\nmh_serial %d\natom_time_interval %d\n"
                "max_chains %d\n",
                dc.geometry, dc.V_s, dc.gap, dc.time_step, steps, dc.image_charge, dc.N_ic_max,
                dc.capacity, dc.seed, dc.emitter_pos[0], dc.emitter_pos[1], dc.emitter_dim[0],
                dc.emitter_dim[1], dc.work_ny, dc.work_nx, dc.work_model, dc.tip_dim[0], dc.tip_dim[1], dc.tip_dim[2],
                fmt_E(dt / time_scale, 14, 6).c_str(), fmt_ES(dt / time_scale, 12, 4).c_str(), dc.emitter_delay,
                dc.planes_N, dc.emitter_type, dc.mh_serial, dc.atom_time_interval, dc.max_chains);
    for (int k = 0; k < dc.planes_N; ++k) std::printf("plane_z %.17g\n", dc.planes_z[k]);
    for (double w : work) std::printf("work_value %.17g\n", w);
    return 0;
  }

  rd_engine_config ec;
  std::memset(&ec, 0, sizeof ec);
  ec.precision = (int)get(gb, "PRECISION", 0, 0.0);
  ec.max_diodes = 1;
  ec.particle_capacity = dc.capacity + 64;
  ec.chain_capacity = (long long)dc.max_chains + 64;
  long long supply_pts = 0;
  check(rd_supply_points(&dc, &supply_pts), "rd_supply_points");
  ec.quad_capacity = supply_pts + 64;
  ec.event_capacity = 4 * dc.capacity + 1024;   // emission and absorption records of one step
  rd_engine* e = nullptr;
  check(rd_engine_create(&ec, &e), "rd_engine_create");
  int diode = -1;
  check(rd_diode_add(e, &dc, &diode), "rd_diode_add");

  mkdir("out", 0755);
  {
    // Write_Initial_Variables (src/main.F90:852-932): out/init.bin, 7 float64 then 4 int32, which
    // the reference's readers use for the scales and the ramo_current.bin dimensions, and the
    // text summary out/init.dt
    const double scales[7] = {1.0, 1.0, 1.0, length_scale, time_scale, length_scale / time_scale, 1.0};
    const int dims[4] = {dc.capacity, 1, 96 * 96, 1000};   // MAX_PARTICLES, _EMITTERS, _SECTIONS, _LIFE_TIME
    FILE* fb = std::fopen("out/init.bin", "wb");
    FILE* ft = std::fopen("out/init.dt", "w");
    if (!fb || !ft) { std::fprintf(stderr, "rd_main: cannot write under out/\n"); return 2; }
    std::fwrite(scales, sizeof(double), 7, fb);
    std::fwrite(dims, sizeof(int), 4, fb);
    std::fclose(fb);
    auto rel = [&](const char* name, double v, const char* what) {
      std::fprintf(ft, "%s  %s  %s\n", name, fmt_ES(v, 16, 6).c_str(), what);
    };
    auto integer = [&](const char* name, long long v, const char* what) {
      std::fprintf(ft, "%s        %s      %s\n", name, fmt_I(v, 8).c_str(), what);
    };
    const char* rule = " ---------------------------------------------------------";
    std::fprintf(ft, " Vacuum Electronics Molecular Dynamics\n Values used for constans and variables\n\n");
    std::fprintf(ft, "%s\nVacuum\n", rule);
    rel("epsilon_r  = ", 1.0, "Relative permittivity");
    rel("m_eeff     = ", 1.0, "Effective mass for electrons");
    rel("m_ieff     = ", 1.0, "Effective mass for ions");
    std::fprintf(ft, "%s\n\n\n%s\n", rule, rule);
    rel("length_scale    = ", length_scale, "The length scale used for output (m)");
    rel("time_scale      = ", time_scale, "The time scale used for output (s)");
    rel("vel_scale       = ", length_scale / time_scale, "The velocity scale used for output (m/s)");
    rel("cur_scale       = ", 1.0, "The current scale used for output (A)");
    rel("time_step       = ", dt, "Size of the time_step used in the Verlet integration (s)");
    integer("steps           = ", steps, "Number of time steps in the Verlet integration");
    std::fprintf(ft, "%s\n\n\n%s\n", rule, rule);
    integer("MAX_PARTICLES       = ", dc.capacity, "Maximum number of electrons in the system");
    std::fprintf(ft, "my_seed             =         %12llu\n", dc.seed);
    std::fprintf(ft, "%s\n\n\n%s\n", rule, rule);
    rel("V_s           = ", V_s, "The Voltage from the source");
    rel("box_dim_x     = ", 0.0, "System x-length");
    rel("box_dim_y     = ", 0.0, "System y-length");
    rel("box_dim_z     = ", mode == 10 ? d : dc.gap, "System z-length");
    rel("d             = ", mode == 10 ? d : dc.gap, "Gap spacing in the system");
    rel("E_z           = ", -V_s / (mode == 10 ? d : dc.gap), "Y-component of the electric field in the system");
    std::fprintf(ft, "%s\n%s\n", rule, rule);
    integer("NrEmit        = ", 1, "Number of emitters");
    integer("EMISSION_MODE = ", mode, "The emission mechanism");
    std::fprintf(ft, "%s\n GIT VERSION\n", rule);
    std::fclose(ft);
  }
  FILE* f_emit = std::fopen("out/emitted.dt", "w");
  FILE* f_abs = std::fopen("out/absorbed.dt", "w");
  FILE* f_top = std::fopen("out/absorbed_top.dt", "w");
  FILE* f_bot = std::fopen("out/absorbed_bot.dt", "w");
  FILE* f_ramo = std::fopen("out/ramo_current.dt", "w");
  // binary event files (Fortran stream access: raw values, no record markers)
  FILE* b_emit = std::fopen("out/density_emit.bin", "wb");
  FILE* b_emit_elec = std::fopen("out/density_emit_elec.bin", "wb");
  FILE* b_abs_top = std::fopen("out/density_absorb_top.bin", "wb");
  FILE* b_abs_bot = std::fopen("out/density_absorb_bot.bin", "wb");
  FILE* f_field = std::fopen("out/field.dt", "w");
  FILE* f_volt = std::fopen("out/volt.dt", "w");
  // per-species emission files (src/main.F90:681-700): ions and atoms only appear here when the
  // library holds them; the collision files stay empty (collisions are outside this path)
  FILE* b_emit_ion = std::fopen("out/density_emit_ion.bin", "wb");
  FILE* b_emit_atom = std::fopen("out/density_emit_atom.bin", "wb");
  // the files the reference opens on every run but writes only in modes outside this path
  // (collisions, Laplace solvers, photo emission, MH tracing) are created empty, as there
  for (const char* empty : {"out/density_ion.bin", "out/density_absorb_recom.bin", "out/absorbed_recom.dt",
                            "out/ionization_data.bin", "out/recombination_data.bin", "out/collisions.dt",
                            "out/laplace_average_field.dt", "out/laplace_grid.dt", "out/gauss.dt", "out/mh.bin"}) {
    FILE* f = std::fopen(empty, "wb");
    if (f) std::fclose(f);
  }
  // integration.dt (Do_Surface_Integration_FE, src/mod_field_emission_v2.F90:653-655): the
  // reference logs Cuba's regions, evaluations, fail flag, integral, error and probability;
  // here the supply rule is a fixed composite Gauss-Legendre rule, so the line gives its panels,
  // nodes, 0 and N_sup (no error estimate: 0)
  FILE* f_integ = std::fopen("out/integration.dt", "w");
  const int q_order = dc.quad_order > 0 ? dc.quad_order : 4;   // the rule of rd_supply_points
  const int q_panels = (int)std::lround(std::sqrt((double)supply_pts)) / q_order;
  // optional files of the namelist's WRITE_POSITION_FILE / WRITE_RAMO_SEC (default off)
  const bool write_pos = in.count("WRITE_POSITION_FILE") && to_logical(in.at("WRITE_POSITION_FILE")[0]);
  const bool write_ramo_sec = in.count("WRITE_RAMO_SEC") && to_logical(in.at("WRITE_RAMO_SEC")[0]);
  if (write_ramo_sec && mode != 10) {
    std::fprintf(stderr, "rd_main: WRITE_RAMO_SEC is supported for planar decks only\n");
    return 2;
  }
  // both files are created on every run (empty unless asked for), as the reference does
  FILE* b_pos = std::fopen("out/position.bin", "wb");
  FILE* b_ramo_sec = std::fopen("out/ramo_current.bin", "wb");
  if (b_pos && !write_pos) { std::fclose(b_pos); b_pos = nullptr; }
  if (b_ramo_sec && !write_ramo_sec) { std::fclose(b_ramo_sec); b_ramo_sec = nullptr; }
  if ((write_pos && !b_pos) || (write_ramo_sec && !b_ramo_sec)) {
    std::fprintf(stderr, "rd_main: cannot write under out/\n");
    return 2;
  }
  const int max_sections = 96 * 96;   // MAX_SECTIONS x MAX_EMITTERS (= 1), src/mod_global.F90:99-100
  std::vector<double> ramo_sec(write_ramo_sec ? max_sections : 0);
  std::vector<double> pbuf, qbuf;
  std::vector<int> idbuf, secbuf;
  if (b_pos) {   // Write_Position, src/mod_pair.F90:841-867: header steps, N_steps (= 1)
    const int hdr[2] = {steps, 1};
    std::fwrite(hdr, sizeof(int), 2, b_pos);
  }
  FILE* b_planes[10] = {};
  for (int k = 0; k < dc.planes_N; ++k)
    if (dc.planes_z[k] > 0.0) {   // out/planes-<k>.bin, src/main.F90:727-738
      char name[64];
      std::snprintf(name, sizeof name, "out/planes-%d.bin", k + 1);
      b_planes[k] = std::fopen(name, "wb");
      if (!b_planes[k]) { std::fprintf(stderr, "rd_main: cannot write %s\n", name); return 2; }
    }
  if (!f_emit || !f_abs || !f_top || !f_bot || !f_ramo || !b_emit || !b_emit_elec || !b_abs_top || !b_abs_bot ||
      !f_field || !f_volt || !b_emit_ion || !b_emit_atom || !f_integ) {
    std::fprintf(stderr, "rd_main: cannot write under out/\n");
    return 2;
  }
  std::printf("RUMDEED: Starting main loop\n Doing %d time steps of size %12.4E ps\n", steps, dt / time_scale);
  std::vector<double> vel;
  std::vector<rd_event> events((size_t)ec.event_capacity);
  long long lost_total = 0;
  int progress = 1;
  std::signal(SIGINT, on_stop_signal);
  std::signal(SIGUSR1, on_stop_signal);
  for (int step = 1; step <= steps; ++step) {
    if (!b_pos) {
      check(rd_step(e, step), "rd_step");
    } else {
      // the main loop's order (src/main.F90:186-198): emission, Update_Position, Write_Position
      // (particles marked for removal still in the arrays), Remove_Particles
      check(rd_do_emission(e, step), "rd_do_emission");
      check(rd_update_position(e, step), "rd_update_position");
      rd_counters c0;
      check(rd_counters_get(e, diode, &c0), "rd_counters_get");
      const int np = c0.n;
      pbuf.resize(3 * (size_t)std::max(np, 1));
      idbuf.resize((size_t)std::max(np, 1));
      secbuf.resize((size_t)std::max(np, 1));
      int got = 0;
      check(rd_get_particles(e, diode, np, pbuf.data(), nullptr, nullptr, nullptr, idbuf.data(), secbuf.data(),
                             &got), "rd_get_particles");
      const int rec[2] = {step, got};
      std::fwrite(rec, sizeof(int), 2, b_pos);
      for (int i = 0; i < got; ++i) {   // x, y, z (m), emitter, section, id
        const int i3[3] = {1, secbuf[i], idbuf[i]};
        std::fwrite(&pbuf[3 * (size_t)i], sizeof(double), 3, b_pos);
        std::fwrite(i3, sizeof(int), 3, b_pos);
      }
      check(rd_remove_particles(e, step), "rd_remove_particles");
    }
    // volt.dt (Set_Voltage, src/mod_verlet.F90:2050-2057): "(ES12.4, tr2, i8, tr2, ES18.8)" with
    // four items, so format reversion puts V_rf (0) on a record of its own
    {
      const double t = dt * step / time_scale;
      std::fprintf(f_volt, "%s  %s  %s\n%s\n", fmt_ES(t, 12, 4).c_str(), fmt_I(step, 8).c_str(),
                   fmt_ES(V_s, 18, 8).c_str(), fmt_ES(0.0, 12, 4).c_str());
    }
    // event records of the step, in the reference's binary layouts:
    //   density_emit.bin       pos/length_scale (3 f64), emitter, section, id, species (4 i32)
    //   density_emit_elec.bin  pos/length_scale (3 f64), emitter, id (2 i32)
    //   density_absorb_top.bin x, y /length_scale (2 f64), v (3 f64, m/s), emitter, section, id (3 i32)
    //   density_absorb_bot.bin x, y /length_scale (2 f64), emitter, section, id (3 i32)
    int nev = 0;
    long long lost = 0;
    check(rd_events_take(e, (int)events.size(), events.data(), &nev, &lost), "rd_events_take");
    lost_total += lost;
    for (int k = 0; k < nev; ++k) {
      const rd_event& r = events[k];
      const double p3[3] = {r.pos[0] / length_scale, r.pos[1] / length_scale, r.pos[2] / length_scale};
      const int emitter = 1;
      if (r.kind == RD_EVENT_EMIT) {
        const int i4[4] = {emitter, r.section, r.id, r.species};
        std::fwrite(p3, sizeof(double), 3, b_emit);
        std::fwrite(i4, sizeof(int), 4, b_emit);
        const int i2[2] = {emitter, r.id};
        FILE* bs = r.species == RD_SPECIES_ION ? b_emit_ion : r.species == RD_SPECIES_ATOM ? b_emit_atom : b_emit_elec;
        std::fwrite(p3, sizeof(double), 3, bs);
        std::fwrite(i2, sizeof(int), 2, bs);
      } else {
        // absorb_top and planes: x, y, v, emitter, section, id; absorb_bot: x, y, emitter, section, id
        const int i3[3] = {emitter, r.section, r.id};
        FILE* bf = nullptr;
        if (r.kind == RD_EVENT_ABSORB_TOP) bf = b_abs_top;
        else if (r.kind == RD_EVENT_ABSORB_BOT) bf = b_abs_bot;
        else if (r.kind >= RD_EVENT_PLANE && r.kind < RD_EVENT_PLANE + 10) bf = b_planes[r.kind - RD_EVENT_PLANE];
        if (!bf) continue;
        std::fwrite(p3, sizeof(double), 2, bf);
        if (r.kind != RD_EVENT_ABSORB_BOT) std::fwrite(r.vel, sizeof(double), 3, bf);
        std::fwrite(i3, sizeof(int), 3, bf);
      }
    }
    rd_counters c;
    check(rd_counters_get(e, diode, &c), "rd_counters_get");
    const double cur_time = dt * step / time_scale;
    // emitted.dt: "(E14.6, *(tr8, i6))" time, step, emitted, electrons in flight, per emitter
    std::string s = fmt_E(cur_time, 14, 6);
    for (long long v : {(long long)step, (long long)c.emitted_step, (long long)c.n + c.absorbed_top_step +
                        c.absorbed_bot_step, (long long)c.emitted_step})
      s += std::string(8, ' ') + fmt_I(v, 6);
    std::fprintf(f_emit, "%s\n", s.c_str());
    // absorbed*.dt: "(ES12.4, *(tr2, i8))" time, step, particles, electrons, ions (+ per emitter)
    auto absorbed = [&](FILE* f, long long n, bool per_emitter) {
      std::string t = fmt_ES(cur_time, 12, 4);
      std::vector<long long> cols = {step, n, n, 0};
      if (per_emitter) cols.push_back(n);
      for (long long v : cols) t += "  " + fmt_I(v, 8);
      std::fprintf(f, "%s\n", t.c_str());
    };
    // field.dt: "(i8, tr2, E16.8, tr2, ...)" step, F_avg(1:3), N_sup, df_avg, a_rate, MH_std
    // (written by the emission, src/mod_field_emission_v2.F90:389-390)
    if (mode == 10 && step > dc.emitter_delay) {
      std::string fl = fmt_I(step, 8);
      for (double v : {c.F_avg[0], c.F_avg[1], c.F_avg[2], c.N_sup, c.df_avg, c.a_rate, c.MH_std})
        fl += "  " + fmt_E(v, 16, 8);
      std::fprintf(f_field, "%s\n", fl.c_str());
      const long long nodes = (long long)q_panels * q_order;
      std::fprintf(f_integ, "%s  %s  %s  %s  %s  %s  %s\n", fmt_I(1, 3).c_str(),
                   fmt_I((long long)q_panels * q_panels, 8).c_str(), fmt_I(nodes * nodes, 8).c_str(),
                   fmt_I(0, 4).c_str(), fmt_ES(c.N_sup, 12, 4).c_str(), fmt_ES(0.0, 12, 4).c_str(),
                   fmt_ES(0.0, 12, 4).c_str());
    }
    absorbed(f_abs, c.absorbed_top_step + c.absorbed_bot_step, false);
    absorbed(f_top, c.absorbed_top_step, true);
    absorbed(f_bot, c.absorbed_bot_step, false);
    // ramo_current.dt (Write_Ramo_Current, src/mod_pair.F90:812-835): time, step, total current
    // (sum over species), V, nrPart, nrElec, nrIon and the mean speeds and mobility of
    // Average_Velocities, all as the velocity update left them (before removal), then the
    // current per species (electron, ion, atom)
    auto norm3 = [](const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); };
    const double ramo_total = c.ramo_current + c.ramo_current_ion;
    std::string r = fmt_ES(cur_time, 12, 4) + "  " + fmt_I(step, 8) + "  " + fmt_ES(ramo_total, 12, 4) +
                    "  " + fmt_ES(V_s, 12, 4) + "  " + fmt_I(c.n_part_vel, 6) + "  " + fmt_I(c.n_elec_vel, 6) +
                    "  " + fmt_I(c.n_ion_vel, 6) + "  " + fmt_ES(c.avg_mob, 12, 4) + "  " +
                    fmt_ES(norm3(c.avg_part_vel), 12, 4) + "  " + fmt_ES(norm3(c.avg_elec_vel), 12, 4) + "  " +
                    fmt_ES(norm3(c.avg_ion_vel), 12, 4) + "  " + fmt_ES(c.ramo_current, 12, 4) + "  " +
                    fmt_ES(c.ramo_current_ion, 12, 4) + "  " + fmt_ES(0.0, 12, 4);
    std::fprintf(f_ramo, "%s\n", r.c_str());
    if (b_ramo_sec) {
      // ramo_current.bin (Write_Ramo_Current, src/mod_pair.F90:822-826): ramo_current_emit(section,
      // emitter) of the step, MAX_SECTIONS x MAX_EMITTERS doubles.  Per particle q v . E_zunit with
      // the velocities of the step; the particles removed in the step carry q = 0 there
      // (Mark_Particles_Remove), so the survivors give the whole sum.
      std::fill(ramo_sec.begin(), ramo_sec.end(), 0.0);
      const int n = c.n;
      vel.resize(3 * (size_t)std::max(n, 1));
      qbuf.resize((size_t)std::max(n, 1));
      secbuf.resize((size_t)std::max(n, 1));
      int got = 0;
      check(rd_get_particles(e, diode, n, nullptr, vel.data(), nullptr, qbuf.data(), nullptr, secbuf.data(), &got),
            "rd_get_particles");
      for (int i = 0; i < got; ++i) {
        const int sec = secbuf[i];
        if (sec >= 1 && sec <= max_sections) ramo_sec[sec - 1] += qbuf[i] * (vel[3 * (size_t)i + 2] * (-1.0 / d));
      }
      std::fwrite(ramo_sec.data(), sizeof(double), ramo_sec.size(), b_ramo_sec);
    }
    if (step * 10 >= progress * steps) {
      std::printf("RUMDEED: %3d %%  electrons %d, emitted %lld, absorbed %lld\n", progress * 10, c.n,
                  c.emitted_total, c.absorbed_top_total + c.absorbed_bot_total);
      std::fflush(stdout);
      ++progress;
    }
    if (g_stop) {
      std::printf("RUMDEED: Got signal SIGINT stopping main loop.\n");
      break;
    }
  }
  for (FILE* f : {f_emit, f_abs, f_top, f_bot, f_ramo, b_emit, b_emit_elec, b_abs_top, b_abs_bot, f_field, f_volt,
                  b_emit_ion, b_emit_atom, f_integ})
    std::fclose(f);
  for (FILE* f : b_planes) if (f) std::fclose(f);
  if (b_pos) std::fclose(b_pos);
  if (b_ramo_sec) std::fclose(b_ramo_sec);
  rd_engine_destroy(e);
  if (lost_total) std::printf("RUMDEED: %lld event records did not fit the event log\n", lost_total);
  std::printf("RUMDEED: Main loop finished\n");
  return 0;
}
