"""ctypes binding of the CPU FP64 oracle (oracle/rd_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / --impl reference legs of bench.py, never by the product path
(rumdeed_gb300).  Builds oracle/_build/liborc.so with `make` on first use.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liborc.so")

PLANAR, TIP = 1, 2
ELEC, ION, ATOM = 1, 2, 3
REMOVE_TOP, REMOVE_BOT = 1, 2
MAX_LIFE = 1000

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Constants(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "pi", "h", "c", "mu_0", "epsilon_0", "m_u", "h_bar", "m_0", "q_0", "m_N2", "m_N2p",
        "length_scale", "time_scale", "div_fac_c", "a_FN", "b_FN", "l_const")]


class Diode(C.Structure):
    _fields_ = [
        ("geometry", C.c_int),
        ("V_s", C.c_double), ("d", C.c_double), ("E_z", C.c_double),
        ("box_dim", C.c_double * 3),
        ("time_step", C.c_double), ("time_step2", C.c_double),
        ("image_charge", C.c_int), ("N_ic_max", C.c_int),
        ("em_pos", C.c_double * 2), ("em_dim", C.c_double * 2),
        ("work_nx", C.c_int), ("work_ny", C.c_int),
        ("work", C.c_double * (64 * 64)),
        ("d_tip", C.c_double), ("R_base", C.c_double), ("h_tip", C.c_double),
        ("a_foci", C.c_double), ("theta_tip", C.c_double), ("r_tip", C.c_double),
        ("eta_1", C.c_double), ("max_xi", C.c_double), ("shift_z", C.c_double),
        ("pre_fac_E_tip", C.c_double), ("pre_fac_E_tip_unit_voltage", C.c_double),
        ("tip_phi", C.c_double),
        ("cap", C.c_int), ("n", C.c_int), ("nrID", C.c_int),
        ("pos", _dp), ("vel", _dp), ("acc", _dp), ("acc_prev", _dp), ("acc_prev2", _dp),
        ("charge", _dp), ("mass", _dp),
        ("species", _ip), ("mask", _ip), ("id", _ip), ("step_created", _ip), ("section", _ip),
        ("n_remove", C.c_int), ("n_remove_top", C.c_int), ("n_remove_bot", C.c_int),
        ("emitted_total", C.c_longlong), ("absorbed_top_total", C.c_longlong),
        ("absorbed_bot_total", C.c_longlong), ("dropped_total", C.c_longlong),
        ("emitted_step", C.c_int),
        ("ramo_current", C.c_double),
        ("avg_elec_vel", C.c_double * 3),
        ("life_time", (C.c_longlong * 3) * MAX_LIFE),
        ("emission", C.c_int),
        ("MH_std", C.c_double), ("a_rate", C.c_double), ("residual", C.c_double),
        ("N_sup", C.c_double),
        ("seed", C.c_uint64),
        ("mh_jumps", C.c_int), ("max_chains", C.c_int), ("quad_panels", C.c_int),
        ("quad_order", C.c_int),
        ("init_rounds_max", C.c_int),
        ("last_chains", C.c_int), ("last_failed_chains", C.c_int),
        ("work_model", C.c_int),
        ("emit_delay", C.c_int), ("mh_serial", C.c_int),
        ("emitter_type", C.c_int), ("ring_rmin", C.c_double), ("ring_thick", C.c_double),
        ("F_avg_z", C.c_double), ("df_avg", C.c_double),
        ("atom_time_interval", C.c_int), ("ramo_current_ion", C.c_double),
        ("avg_part_vel", C.c_double * 3), ("avg_ion_vel", C.c_double * 3), ("avg_mob", C.c_double),
        ("n_part_vel", C.c_int), ("n_elec_vel", C.c_int), ("n_ion_vel", C.c_int),
        ("F_avg_x", C.c_double), ("F_avg_y", C.c_double),
    ]


_lib = None


def build(force=False):
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "rd_oracle.c")):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        D = C.POINTER(Diode)
        sig = {
            "orc_get_constants": (None, [C.POINTER(Constants)]),
            "orc_v_y": (C.c_double, [C.c_double, C.c_double, C.c_int]),
            "orc_t_y": (C.c_double, [C.c_double, C.c_double, C.c_int]),
            "orc_escape_prob_log": (C.c_double, [C.c_double, C.c_double, C.c_int]),
            "orc_elec_supply_log": (C.c_double, [C.c_double, C.c_double, C.c_int]),
            "orc_elec_supply_v2": (C.c_double, [C.c_double, C.c_double, C.c_int, C.c_double]),
            "orc_work_checkerboard": (C.c_double, [_dp, C.c_int, C.c_int, _dp, _dp, C.c_double,
                                                   C.c_double, _ip]),
            "orc_philox4x32": (None, [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                      C.POINTER(C.c_uint32)]),
            "orc_u01_from_words": (C.c_double, [C.c_uint32, C.c_uint32]),
            "orc_diode_new": (D, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                  C.c_int, C.c_int]),
            "orc_diode_free": (None, [D]),
            "orc_set_planar_emitter": (None, [D, C.c_double, C.c_double, C.c_double, C.c_double,
                                              C.c_int, C.c_int, _dp]),
            "orc_set_tip": (None, [D, C.c_double, C.c_double, C.c_double, C.c_double]),
            "orc_set_work_model": (None, [D, C.c_int, C.c_int, _dp]),
            "orc_set_ring": (None, [D, C.c_double, C.c_double]),
            "orc_work_gaussian": (C.c_double, [_dp, C.c_int, C.c_double, C.c_double]),
            "orc_work_voronoi": (C.c_double, [_dp, C.c_int, _dp, _dp, C.c_double, C.c_double, _ip]),
            "orc_set_emission": (None, [D, C.c_int, C.c_uint64, C.c_int, C.c_int, C.c_int,
                                        C.c_int]),
            "orc_reset": (None, [D]),
            "orc_add_particle": (C.c_int, [D, _dp, _dp, C.c_int, C.c_int, C.c_int]),
            "orc_mark_remove": (None, [D, C.c_int, C.c_int]),
            "orc_remove_particles": (None, [D, C.c_int]),
            "orc_field_E": (None, [D, _dp, _dp]),
            "orc_E_zunit": (None, [D, _dp, _dp]),
            "orc_force_image_planar": (None, [D, _dp, _dp, _dp]),
            "orc_sphere_ic_field": (None, [D, _dp, _dp, _dp]),
            "orc_accel_generic": (None, [D, _dp, C.c_int]),
            "orc_accel_planar": (None, [D, _dp, C.c_int]),
            "orc_accel_gather": (None, [D, _dp, C.c_int]),
            "orc_accel_rows": (None, [D, C.c_int, _ip, _dp, C.c_int]),
            "orc_field_at": (None, [D, _dp, _dp, C.c_int]),
            "orc_field_at_batch": (None, [D, C.c_int, _dp, _dp, C.c_int]),
            "orc_update_position": (None, [D]),
            "orc_update_velocity": (None, [D]),
            "orc_velocity_verlet": (None, [D, C.c_int]),
            "orc_update_position_tts": (None, [D, C.c_int]),
            "orc_accel_tts": (None, [D, C.c_int, C.c_int]),
            "orc_update_velocity_tts": (None, [D, C.c_int]),
            "orc_supply_integral_planar": (C.c_double, [D]),
            "orc_supply_panels": (C.c_int, [D]),
            "orc_supply_planar_converged": (C.c_double, [D, C.c_double, C.c_int, C.POINTER(C.c_longlong)]),
            "orc_mh_batch_planar": (None, [D, C.c_int, C.c_int, _dp, _dp, _dp, _ip]),
            "orc_do_emission_planar": (C.c_int, [D, C.c_int]),
            "orc_supply_tip": (C.c_double, [D]),
            "orc_mh_batch_tip": (None, [D, C.c_int, C.c_int, _dp, _dp, _dp, _ip]),
            "orc_do_emission_tip": (C.c_int, [D, C.c_int]),
            "orc_do_emission": (C.c_int, [D, C.c_int]),
            "orc_step": (None, [D, C.c_int]),
            "orc_tip_xyz": (None, [D, C.c_double, C.c_double, C.c_double, _dp]),
            "orc_tip_eta": (C.c_double, [D, C.c_double, C.c_double, C.c_double]),
            "orc_tip_surface_normal": (None, [D, _dp, _dp]),
            "orc_tip_area": (C.c_double, [D, C.c_double, C.c_double, C.c_double, C.c_double]),
            "orc_accel_planar_omp": (None, [C.c_int, _dp, _dp, _dp, C.c_double, C.c_double,
                                            C.c_int, C.c_int, _dp]),
            "orc_omp_threads": (C.c_int, []),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def ptr(a):
    return a.ctypes.data_as(_dp)


def constants():
    c = Constants()
    lib().orc_get_constants(C.byref(c))
    return {k: getattr(c, k) for k, _ in Constants._fields_}


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32(c, k, o)
    return list(o)


class OracleDiode:
    """One diode of the oracle (Fortran module globals of one run)."""

    def __init__(self, geometry=PLANAR, cap=1024, V_s=2.0e3, d=1000e-9, time_step=0.25e-15,
                 image_charge=True, N_ic_max=0):
        self.L = lib()
        self.p = self.L.orc_diode_new(geometry, cap, V_s, d, time_step, int(image_charge),
                                      N_ic_max)
        self.s = self.p.contents

    def __del__(self):
        try:
            self.L.orc_diode_free(self.p)
        except Exception:
            pass

    # configuration -----------------------------------------------------------
    def set_planar_emitter(self, x0, y0, Lx, Ly, work=None):
        w = np.array([[4.7]] if work is None else work, dtype=np.float64)
        ny, nx = w.shape
        self.L.orc_set_planar_emitter(self.p, x0, y0, Lx, Ly, nx, ny, ptr(np.ascontiguousarray(w)))

    def set_work_model(self, model, params):
        """Gaussian (2) or Voronoi (4) work function (flat parameter list)."""
        w = np.ascontiguousarray(params, dtype=np.float64).ravel()
        n = (w.size - 1) // 5 if model == 2 else w.size // 4
        self.L.orc_set_work_model(self.p, model, n, ptr(w))

    def set_ring(self, r_out, thickness):
        self.L.orc_set_ring(self.p, r_out, thickness)

    def set_tip(self, d_tip, R_base, h_tip, phi=4.7):
        self.L.orc_set_tip(self.p, d_tip, R_base, h_tip, phi)

    def set_emission(self, on=True, seed=1, mh_jumps=0, max_chains=0, quad_panels=0,
                     quad_order=0):
        self.L.orc_set_emission(self.p, int(on), seed, mh_jumps, max_chains, quad_panels,
                                quad_order)

    # particles ---------------------------------------------------------------
    def add(self, pos, vel=(0.0, 0.0, 0.0), species=ELEC, step=1, sec=1):
        p = np.asarray(pos, dtype=np.float64)
        v = np.asarray(vel, dtype=np.float64)
        return self.L.orc_add_particle(self.p, ptr(p), ptr(v), species, step, sec)

    @property
    def n(self):
        return self.s.n

    def arr(self, name, comps=3):
        n = self.s.n
        base = getattr(self.s, name)
        if comps == 1:
            return np.ctypeslib.as_array(base, shape=(max(self.s.cap, 1),))[:n].copy()
        return np.ctypeslib.as_array(base, shape=(max(self.s.cap, 1) * 3,))[:3 * n].reshape(n, 3).copy()

    def iarr(self, name):
        return np.ctypeslib.as_array(getattr(self.s, name), shape=(max(self.s.cap, 1),))[:self.s.n].copy()

    def set_arr(self, name, values):
        v = np.ascontiguousarray(values, dtype=np.float64).ravel()
        base = getattr(self.s, name)
        dst = np.ctypeslib.as_array(base, shape=(max(self.s.cap, 1) * 3,))
        dst[:v.size] = v

    # physics -----------------------------------------------------------------
    def accel(self, kind="gather", compensated=True):
        out = np.zeros(3 * max(self.s.n, 1))
        getattr(self.L, "orc_accel_" + kind)(self.p, ptr(out), int(compensated))
        return out[:3 * self.s.n].reshape(-1, 3)

    def accel_rows(self, rows, compensated=True):
        """The gather acceleration of the particles `rows` only, (len(rows), 3)."""
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        out = np.zeros(3 * max(len(rows), 1))
        self.L.orc_accel_rows(self.p, len(rows), rows.ctypes.data_as(_ip), ptr(out), int(compensated))
        return out[:3 * len(rows)].reshape(-1, 3)

    def add_many(self, pos, species=ELEC, step=1, sec=1):
        """Add_Particle for every row of pos (velocity 0), in order."""
        for p in np.ascontiguousarray(pos, dtype=np.float64):
            self.L.orc_add_particle(self.p, ptr(p), ptr(np.zeros(3)), species, step, sec)

    def field_at(self, pts, compensated=True):
        pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        out = np.zeros_like(pts)
        self.L.orc_field_at_batch(self.p, pts.shape[0], ptr(pts), ptr(out), int(compensated))
        return out

    def mark(self, i, why):
        self.L.orc_mark_remove(self.p, i, why)

    def remove(self, step):
        self.L.orc_remove_particles(self.p, step)

    def update_position(self):
        self.L.orc_update_position(self.p)

    def update_velocity(self):
        self.L.orc_update_velocity(self.p)

    def set_tts(self, interval):
        """Two-time-step integrator with atom_time_interval = interval (0 = off)."""
        self.s.atom_time_interval = int(interval)

    def verlet(self, step):
        self.L.orc_velocity_verlet(self.p, step)

    def emission(self, step):
        return self.L.orc_do_emission(self.p, step)

    def step(self, step):
        self.L.orc_step(self.p, step)

    def supply(self):
        if self.s.geometry == TIP:
            return self.L.orc_supply_tip(self.p)
        return self.L.orc_supply_integral_planar(self.p)

    def supply_converged(self, tol=0.01, max_depth=12):
        """The planar supply integral integrated adaptively to convergence:
        (N_sup, integrand evaluations)."""
        ev = C.c_longlong()
        v = self.L.orc_supply_planar_converged(self.p, tol, max_depth, C.byref(ev))
        return v, ev.value

    def mh_batch(self, step, M):
        df = np.zeros(max(M, 1)); F = np.zeros(max(M, 1)); P = np.zeros(3 * max(M, 1))
        ok = np.zeros(max(M, 1), dtype=np.int32)
        f = self.L.orc_mh_batch_tip if self.s.geometry == TIP else self.L.orc_mh_batch_planar
        f(self.p, step, M, ptr(df), ptr(F), ptr(P), ok.ctypes.data_as(_ip))
        return df[:M], F[:M], P[:3 * M].reshape(-1, 3), ok[:M]

    def life_time(self):
        return np.array([[self.s.life_time[i][k] for k in range(3)] for i in range(MAX_LIFE)])


def accel_planar_omp(pos, charge, mass, E_z, d, image_charge=True, N_ic_max=0):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    n = pos.shape[0]
    out = np.zeros(3 * max(n, 1))
    lib().orc_accel_planar_omp(n, ptr(pos), ptr(np.ascontiguousarray(charge, dtype=np.float64)),
                               ptr(np.ascontiguousarray(mass, dtype=np.float64)), E_z, d,
                               int(image_charge), N_ic_max, ptr(out))
    return out[:3 * n].reshape(n, 3)
