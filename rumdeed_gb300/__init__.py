"""rumdeed_gb300 -- GB300 (sm_103a) implementation of RUMDEED's time-step hot path.

Python host mirror of the reference's Fortran module interfaces for this path,
calling librumdeed_gb300.so through its C ABI (include/rumdeed_gpu.h):

    reference (NanoPhysicsCenter/RUMDEED)          here
    ---------------------------------------------  --------------------------------
    Add_Particle            mod_pair.F90:29         Diode.add_particle(s)
    Mark_Particles_Remove   mod_pair.F90:169        Diode.mark_particles_remove
    Remove_Particles        mod_pair.F90:352        Engine.remove_particles
    Update_Position         mod_verlet.F90:115      Engine.update_position
    Calculate_Acceleration_Particles  :597          Engine/Diode.calculate_acceleration_particles
    Calc_Field_at_Batch     mod_verlet.F90:1635     Diode.calc_field_at_batch
    ptr_Do_Emission / Do_Field_Emission fe_v2:170   Engine.do_emission
    main loop               main.F90:175-219        Engine.step / Engine.run

There is no CPU fallback: importing works anywhere, but creating an Engine
raises if the CUDA library is missing or no GPU is present.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "librumdeed_gb300.so")

RD_OK = 0
GEOM_PLANAR, GEOM_TIP = 1, 2
PREC_FP64, PREC_FP32C = 0, 1
ELEC, ION, ATOM = 1, 2, 3
REMOVE_TOP, REMOVE_BOT = 1, 2

# Physical constants (src/mod_global.F90:26-45).
q_0 = 1.602176634e-19
m_0 = 9.1093837015e-31
length_scale = 1.0e-9
time_scale = 1.0e-12


class RumdeedError(RuntimeError):
    pass


class EngineConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("precision", C.c_int), ("max_diodes", C.c_int),
                ("particle_capacity", C.c_longlong), ("chain_capacity", C.c_longlong),
                ("quad_capacity", C.c_longlong), ("chunk_min", C.c_int),
                ("grid_blocks", C.c_int), ("chunk_count_max", C.c_int), ("event_capacity", C.c_int)]


class Event(C.Structure):
    _fields_ = [("pos", C.c_double * 3), ("vel", C.c_double * 3), ("diode", C.c_int), ("kind", C.c_int),
                ("section", C.c_int), ("id", C.c_int), ("species", C.c_int), ("step", C.c_int)]


EVENT_EMIT, EVENT_ABSORB_TOP, EVENT_ABSORB_BOT, EVENT_PLANE = 1, 2, 3, 16


class DiodeConfig(C.Structure):
    _fields_ = [("geometry", C.c_int), ("V_s", C.c_double), ("gap", C.c_double),
                ("time_step", C.c_double), ("image_charge", C.c_int), ("N_ic_max", C.c_int),
                ("capacity", C.c_int), ("emitter_pos", C.c_double * 2),
                ("emitter_dim", C.c_double * 2), ("work_nx", C.c_int), ("work_ny", C.c_int),
                ("work", C.POINTER(C.c_double)), ("tip_dim", C.c_double * 3),
                ("tip_work_function", C.c_double), ("emission", C.c_int), ("mh_jumps", C.c_int),
                ("max_chains", C.c_int), ("quad_panels", C.c_int), ("quad_order", C.c_int),
                ("init_rounds", C.c_int), ("seed", C.c_ulonglong), ("work_model", C.c_int),
                ("emitter_delay", C.c_int), ("planes_N", C.c_int), ("planes_z", C.c_double * 10),
                ("mh_serial", C.c_int), ("emitter_type", C.c_int), ("emitter_thickness", C.c_double),
                ("atom_time_interval", C.c_int)]


class Counters(C.Structure):
    _fields_ = [("n", C.c_int), ("emitted_step", C.c_int), ("dropped_step", C.c_int),
                ("absorbed_top_step", C.c_int), ("absorbed_bot_step", C.c_int),
                ("chains", C.c_int), ("chains_failed", C.c_int), ("chains_capped", C.c_int),
                ("emitted_total", C.c_longlong), ("dropped_total", C.c_longlong),
                ("absorbed_top_total", C.c_longlong), ("absorbed_bot_total", C.c_longlong),
                ("electron_steps", C.c_longlong), ("steps_done", C.c_longlong),
                ("ramo_current", C.c_double), ("N_sup", C.c_double), ("MH_std", C.c_double),
                ("a_rate", C.c_double), ("residual", C.c_double), ("F_avg", C.c_double * 3),
                ("df_avg", C.c_double), ("ramo_current_ion", C.c_double),
                ("avg_part_vel", C.c_double * 3), ("avg_elec_vel", C.c_double * 3),
                ("avg_ion_vel", C.c_double * 3), ("avg_mob", C.c_double),
                ("n_part_vel", C.c_int), ("n_elec_vel", C.c_int), ("n_ion_vel", C.c_int)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        for k in ("F_avg", "avg_part_vel", "avg_elec_vel", "avg_ion_vel"):
            d[k] = tuple(getattr(self, k))
        return d


class PhaseTimes(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("supply_ms", "mh_init_ms", "mh_jumps_ms", "emit_ms",
                                          "position_ms", "force_ms", "velocity_ms", "compact_ms",
                                          "total_ms")] + \
               [("mh_jump_launches", C.c_int), ("mh_pair_evals", C.c_longlong),
                ("force_pairs", C.c_longlong), ("supply_pair_evals", C.c_longlong)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Request(C.Structure):
    _fields_ = [("diode", DiodeConfig), ("steps", C.c_int), ("n_init", C.c_int),
                ("pos3n", C.POINTER(C.c_double)), ("vel3n", C.POINTER(C.c_double))]


class RequestStatus(C.Structure):
    _fields_ = [("state", C.c_int), ("diode", C.c_int), ("steps", C.c_int),
                ("submit_s", C.c_double), ("admit_s", C.c_double), ("done_s", C.c_double),
                ("counters", Counters)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "counters"}
        d["counters"] = self.counters.as_dict()
        return d


class ServeStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("admitted", C.c_int), ("retired", C.c_int),
                ("running", C.c_int), ("queued", C.c_int), ("device_ms", C.c_double),
                ("wall_ms", C.c_double), ("electron_steps", C.c_longlong),
                ("step_ms_p50", C.c_double), ("step_ms_p99", C.c_double),
                ("step_ms_max", C.c_double), ("h2d_bytes", C.c_longlong),
                ("d2h_bytes", C.c_longlong)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class TuneResult(C.Structure):
    _fields_ = [("chunk_min", C.c_int), ("chunk_count_max", C.c_int), ("ms_default", C.c_double),
                ("ms_chosen", C.c_double), ("candidates", C.c_int), ("mh_parts", C.c_int), ("mh_form", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_CANCELLED = 0, 1, 2, 3


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lib = None

# Every entry point of include/rumdeed_gpu.h with its ctypes signature.
SIGNATURES = {
    "rd_last_error": (C.c_char_p, []),
    "rd_version": (C.c_int, []),
    "rd_engine_create": (C.c_int, [C.POINTER(EngineConfig), C.POINTER(C.c_void_p)]),
    "rd_engine_destroy": (C.c_int, [C.c_void_p]),
    "rd_sync": (C.c_int, [C.c_void_p]),
    "rd_diode_add": (C.c_int, [C.c_void_p, C.POINTER(DiodeConfig), _ip]),
    "rd_diode_remove": (C.c_int, [C.c_void_p, C.c_int]),
    "rd_diode_count": (C.c_int, [C.c_void_p, _ip]),
    "rd_add_particles": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _ip, C.c_int, C.c_int]),
    "rd_get_particles": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _ip, _ip, _ip]),
    "rd_set_particles": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp]),
    "rd_accel": (C.c_int, [C.c_void_p, C.c_int, _dp]),
    "rd_field_at": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _dp]),
    "rd_mark_remove": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "rd_do_emission": (C.c_int, [C.c_void_p, C.c_int]),
    "rd_update_position": (C.c_int, [C.c_void_p, C.c_int]),
    "rd_remove_particles": (C.c_int, [C.c_void_p, C.c_int]),
    "rd_step": (C.c_int, [C.c_void_p, C.c_int]),
    "rd_run": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "rd_counters_get": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(Counters)]),
    "rd_life_time": (C.c_int, [C.c_void_p, C.c_int, _ip]),
    "rd_last_run_stats": (C.c_int, [C.c_void_p, _dp, _ip]),
    "rd_profile_step": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(PhaseTimes)]),
    "rd_submit": (C.c_int, [C.c_void_p, C.POINTER(Request), C.POINTER(C.c_longlong)]),
    "rd_poll": (C.c_int, [C.c_void_p, C.c_longlong, C.POINTER(RequestStatus)]),
    "rd_cancel": (C.c_int, [C.c_void_p, C.c_longlong]),
    "rd_serve": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(ServeStats)]),
    "rd_clock": (C.c_int, [C.c_void_p, _dp]),
    "rd_field_at_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    "rd_time_accel": (C.c_int, [C.c_void_p, C.c_int, _dp]),
    "rd_time_verlet": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp]),
    "rd_time_field_at": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, C.c_int, _dp]),
    "rd_autotune": (C.c_int, [C.c_void_p, C.POINTER(TuneResult)]),
    "rd_events_take": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(Event), _ip, C.POINTER(C.c_longlong)]),
    "rd_set_chunking": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "rd_get_chunking": (C.c_int, [C.c_void_p, _ip, _ip]),
    "rd_set_mh_launch": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "rd_time_remove": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                 C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "rd_supply_points": (C.c_int, [C.POINTER(DiodeConfig), C.POINTER(C.c_longlong)]),
    "rd_get_mh_launch": (C.c_int, [C.c_void_p, _ip, _ip]),
    "rd_validate": (C.c_int, [C.c_void_p, _ip, C.POINTER(C.c_longlong)]),
    "rd_diode_state_size": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_longlong)]),
    "rd_diode_save": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong)]),
    "rd_diode_load": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_longlong]),
}


def build(force=False):
    """Compile librumdeed_gb300.so (nvcc, sm_103a) if it is missing or stale."""
    from . import builder
    return builder.build(force=force)


def lib():
    """Load librumdeed_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RumdeedError("librumdeed_gb300.so is not built (run rumdeed_gb300.build())")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc):
    if rc != RD_OK:
        msg = lib().rd_last_error().decode(errors="replace")
        raise RumdeedError("rumdeed_gb300 error %d: %s" % (rc, msg))


def _p(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _vec3(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1, 3)
    if n is not None and a.shape[0] != n:
        raise ValueError("expected %d rows" % n)
    return a


class Engine:
    """One GPU, a pool of diode slots advanced together (segment table)."""

    def __init__(self, precision=PREC_FP32C, max_diodes=16, particle_capacity=1 << 20,
                 chain_capacity=1 << 16, quad_capacity=1 << 16, device=0, chunk_min=0,
                 grid_blocks=0, chunk_count_max=0, event_capacity=0):
        self.L = lib()
        cfg = EngineConfig(device, precision, max_diodes, particle_capacity, chain_capacity,
                           quad_capacity, chunk_min, grid_blocks, chunk_count_max, event_capacity)
        h = C.c_void_p()
        _check(self.L.rd_engine_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self.precision = precision
        self.diodes = {}

    def close(self):
        if getattr(self, "h", None):
            self.L.rd_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # diode slots ---------------------------------------------------------------
    def add_diode(self, **kw):
        cfg, keep = diode_config(**kw)
        d = C.c_int()
        _check(self.L.rd_diode_add(self.h, C.byref(cfg), C.byref(d)))
        del keep
        dio = Diode(self, d.value)
        self.diodes[d.value] = dio
        return dio

    def remove_diode(self, diode):
        idx = diode.index if isinstance(diode, Diode) else int(diode)
        _check(self.L.rd_diode_remove(self.h, idx))
        self.diodes.pop(idx, None)

    # tracing -------------------------------------------------------------------
    def profile_step(self, step):
        """One main-loop iteration with CUDA-event timers between the phases."""
        t = PhaseTimes()
        _check(self.L.rd_profile_step(self.h, step, C.byref(t)))
        return t.as_dict()

    # serving -------------------------------------------------------------------
    def submit(self, steps, pos=None, vel=None, **diode_kw):
        cfg, keep = diode_config(**diode_kw)
        req = Request()
        req.diode = cfg
        req.steps = steps
        p = None if pos is None else _vec3(pos)
        v = None if vel is None else _vec3(vel)
        req.n_init = 0 if p is None else p.shape[0]
        req.pos3n = _p(p)
        req.vel3n = _p(v)
        i = C.c_longlong()
        _check(self.L.rd_submit(self.h, C.byref(req), C.byref(i)))
        del keep
        return i.value

    def poll(self, rid):
        st = RequestStatus()
        _check(self.L.rd_poll(self.h, rid, C.byref(st)))
        return st.as_dict()

    def cancel(self, rid):
        _check(self.L.rd_cancel(self.h, rid))

    def serve(self, iterations=1):
        st = ServeStats()
        _check(self.L.rd_serve(self.h, iterations, C.byref(st)))
        return st.as_dict()

    # event log -----------------------------------------------------------------
    def events_take(self, cap=1 << 20):
        """Emission / absorption records logged since the last take
        (rd_events_take): a list of dicts and the number of lost records."""
        buf = (Event * max(cap, 1))()
        n = C.c_int()
        lost = C.c_longlong()
        _check(self.L.rd_events_take(self.h, cap, buf, C.byref(n), C.byref(lost)))
        out = [{"pos": tuple(r.pos), "vel": tuple(r.vel), "diode": r.diode, "kind": r.kind,
                "section": r.section, "id": r.id, "species": r.species, "step": r.step}
               for r in buf[:n.value]]
        return out, lost.value

    # autotuner -----------------------------------------------------------------
    def autotune(self):
        """Pick the pair-sum chunking for the resident diodes (rd_autotune)."""
        t = TuneResult()
        _check(self.L.rd_autotune(self.h, C.byref(t)))
        return t.as_dict()

    def set_chunking(self, chunk_min=0, chunk_count_max=0):
        _check(self.L.rd_set_chunking(self.h, chunk_min, chunk_count_max))

    def get_chunking(self):
        a, b = C.c_int(), C.c_int()
        _check(self.L.rd_get_chunking(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_mh_launch(self, parts=0, form=-1):
        """Planar MH launch shape (rd_set_mh_launch): plan parts and FP32 thread form."""
        _check(self.L.rd_set_mh_launch(self.h, parts, form))

    def get_mh_launch(self):
        a, b = C.c_int(), C.c_int()
        _check(self.L.rd_get_mh_launch(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def time_verlet(self, reps=5):
        """Device ms of one position pass and of one velocity pass (rd_time_verlet;
        advances the state)."""
        a, b = C.c_double(), C.c_double()
        _check(self.L.rd_time_verlet(self.h, reps, C.byref(a), C.byref(b)))
        return a.value, b.value

    def time_remove(self):
        """One position pass and the removal after it (rd_time_remove): (position ms,
        removal ms, survivors moved, particles removed)."""
        a, b = C.c_double(), C.c_double()
        m, r = C.c_longlong(), C.c_longlong()
        _check(self.L.rd_time_remove(self.h, C.byref(a), C.byref(b), C.byref(m), C.byref(r)))
        return a.value, b.value, m.value, r.value

    def time_accel(self, reps=3):
        """Device milliseconds of one force evaluation of all resident diodes."""
        ms = C.c_double()
        _check(self.L.rd_time_accel(self.h, reps, C.byref(ms)))
        return ms.value

    def clock(self):
        t = C.c_double()
        _check(self.L.rd_clock(self.h, C.byref(t)))
        return t.value


    # main-loop phases (all diodes) ----------------------------------------------
    def do_emission(self, step):
        _check(self.L.rd_do_emission(self.h, step))

    def update_position(self, step):
        _check(self.L.rd_update_position(self.h, step))

    def remove_particles(self, step):
        _check(self.L.rd_remove_particles(self.h, step))

    def calculate_acceleration_particles(self):
        _check(self.L.rd_accel(self.h, next(iter(self.diodes)) if self.diodes else 0, None))

    def step(self, step):
        _check(self.L.rd_step(self.h, step))

    def run(self, first_step, nsteps):
        _check(self.L.rd_run(self.h, first_step, nsteps))

    def sync(self):
        _check(self.L.rd_sync(self.h))

    VALIDATE_KINDS = ("count_outside_capacity", "removal_not_cleared", "unknown_species", "still_marked",
                      "non_finite_state", "ids_not_increasing", "charge_mass_mismatch")

    def validate(self):
        """Device-side state invariants of every resident diode (rd_validate):
        violation counts by kind; all zero for a healthy engine."""
        counts = (C.c_int * 7)()
        total = C.c_longlong()
        _check(self.L.rd_validate(self.h, counts, C.byref(total)))
        return dict(zip(self.VALIDATE_KINDS, list(counts)))

    def last_run_stats(self):
        ms = C.c_double()
        k = C.c_int()
        _check(self.L.rd_last_run_stats(self.h, C.byref(ms), C.byref(k)))
        return ms.value, k.value


def diode_config(geometry=GEOM_PLANAR, V_s=2.0e3, gap=1000e-9, time_step=0.25e-15,
             image_charge=True, N_ic_max=0, capacity=4096, emitter_pos=(0.0, 0.0),
             emitter_dim=(0.0, 0.0), work=None, tip_dim=(0.0, 0.0, 0.0),
             tip_work_function=4.7, emission=False, mh_jumps=0, max_chains=0,
             quad_panels=0, quad_order=0, init_rounds=0, seed=1, work_model=0, emitter_delay=0,
             planes_z=(), mh_serial=False, emitter_type=0, emitter_thickness=0.0,
             atom_time_interval=0):
    """rd_diode_config from keyword arguments (the /input/ namelist of one run).
    `work`: the checkerboard matrix (work_model 0/1); for work_model 2
    (Gaussian) the flat list base, then (A, x_c, y_c, std_x, std_y) per
    Gaussian; for work_model 4 (Voronoi) the flat list (x, y, phi, section)
    per site, x, y as fractions of the emitter.  `atom_time_interval` > 0
    selects the two-time-step integrator (ions move every that many steps)."""
    cfg = DiodeConfig()
    cfg.geometry = geometry
    cfg.V_s = V_s
    cfg.gap = gap
    cfg.time_step = time_step
    cfg.image_charge = int(bool(image_charge))
    cfg.N_ic_max = N_ic_max
    cfg.capacity = capacity
    cfg.emitter_pos[:] = list(emitter_pos)
    cfg.emitter_dim[:] = list(emitter_dim)
    keep = None
    cfg.work_model = work_model
    cfg.emitter_delay = emitter_delay
    cfg.mh_serial = int(bool(mh_serial))
    cfg.emitter_type = emitter_type
    cfg.emitter_thickness = emitter_thickness
    cfg.atom_time_interval = int(atom_time_interval)
    cfg.planes_N = len(planes_z)
    for k, z in enumerate(planes_z):
        cfg.planes_z[k] = z
    if work is not None:
        if work_model in (2, 4):
            keep = np.ascontiguousarray(work, dtype=np.float64).ravel()
            cfg.work_nx = (keep.size - 1) // 5 if work_model == 2 else keep.size // 4
            cfg.work_ny = 1
        else:
            keep = np.ascontiguousarray(work, dtype=np.float64)
            cfg.work_ny, cfg.work_nx = keep.shape
        cfg.work = keep.ctypes.data_as(_dp)
    cfg.tip_dim[:] = list(tip_dim)
    cfg.tip_work_function = tip_work_function
    cfg.emission = int(bool(emission))
    cfg.mh_jumps = mh_jumps
    cfg.max_chains = max_chains
    cfg.quad_panels = quad_panels
    cfg.quad_order = quad_order
    cfg.init_rounds = init_rounds
    cfg.seed = seed
    return cfg, keep


def supply_points(**kw):
    """rd_supply_points: quadrature points a diode of this configuration takes."""
    cfg, keep = diode_config(**kw)
    n = C.c_longlong()
    _check(lib().rd_supply_points(C.byref(cfg), C.byref(n)))
    del keep
    return n.value


class Diode:
    """One diode slot of an Engine (the module globals of one reference run)."""

    def __init__(self, engine, index):
        self.e = engine
        self.index = index

    @property
    def L(self):
        return self.e.L

    def add_particles(self, pos, vel=None, species=None, step=1, section=1):
        pos = _vec3(pos)
        n = pos.shape[0]
        vel = None if vel is None else _vec3(vel, n)
        sp = None if species is None else np.ascontiguousarray(np.broadcast_to(species, (n,)), dtype=np.int32)
        _check(self.L.rd_add_particles(self.e.h, self.index, n, _p(pos), _p(vel),
                                       None if sp is None else sp.ctypes.data_as(_ip), step, section))

    def add_particle(self, pos, vel=(0.0, 0.0, 0.0), species=ELEC, step=1, section=1):
        self.add_particles([pos], [vel], [species], step, section)

    def counters(self):
        c = Counters()
        _check(self.L.rd_counters_get(self.e.h, self.index, C.byref(c)))
        return c.as_dict()

    @property
    def n(self):
        return self.counters()["n"]

    def particles(self):
        n = self.n
        cap = max(n, 1)
        pos = np.zeros((cap, 3)); vel = np.zeros((cap, 3)); acc = np.zeros((cap, 3))
        q = np.zeros(cap); ids = np.zeros(cap, dtype=np.int32); sec = np.zeros(cap, dtype=np.int32)
        nout = C.c_int()
        _check(self.L.rd_get_particles(self.e.h, self.index, cap, _p(pos), _p(vel), _p(acc), _p(q),
                                       ids.ctypes.data_as(_ip), sec.ctypes.data_as(_ip), C.byref(nout)))
        return {"pos": pos[:n], "vel": vel[:n], "acc": acc[:n], "charge": q[:n], "id": ids[:n],
                "section": sec[:n]}

    def set_particles(self, pos=None, vel=None, acc=None, acc_prev=None, acc_prev2=None):
        arrs = [None if a is None else _vec3(a) for a in (pos, vel, acc, acc_prev, acc_prev2)]
        n = next(a.shape[0] for a in arrs if a is not None)
        _check(self.L.rd_set_particles(self.e.h, self.index, n, *[_p(a) for a in arrs]))

    def calculate_acceleration_particles(self):
        n = self.n
        out = np.zeros((max(n, 1), 3))
        _check(self.L.rd_accel(self.e.h, self.index, _p(out)))
        return out[:n]

    def calc_field_at_batch(self, pts):
        pts = _vec3(pts)
        out = np.zeros_like(pts)
        _check(self.L.rd_field_at(self.e.h, self.index, pts.shape[0], _p(pts), _p(out)))
        return out

    def time_field_at(self, pts, reps=3):
        """Device milliseconds of one field evaluation at the points."""
        pts = _vec3(pts)
        ms = C.c_double()
        _check(self.L.rd_time_field_at(self.e.h, self.index, pts.shape[0], _p(pts), reps, C.byref(ms)))
        return ms.value

    def calc_field_at_batch_noalloc(self, pos_dev_ptr, field_dev_ptr, M):
        """rd_field_at_noalloc: points and result are caller-owned device
        buffers ((3, M) doubles); the call allocates nothing."""
        _check(self.L.rd_field_at_noalloc(self.e.h, self.index, M, C.c_void_p(pos_dev_ptr),
                                          C.c_void_p(field_dev_ptr)))

    def mark_particles_remove(self, i, why):
        _check(self.L.rd_mark_remove(self.e.h, self.index, i, why))

    def save_state(self):
        """Checkpoint of the diode between steps (rd_diode_save), as bytes."""
        size = C.c_longlong()
        _check(self.L.rd_diode_state_size(self.e.h, self.index, C.byref(size)))
        buf = C.create_string_buffer(size.value)
        written = C.c_longlong()
        _check(self.L.rd_diode_save(self.e.h, self.index, buf, size.value, C.byref(written)))
        return buf.raw[:written.value]

    def load_state(self, state):
        """Put a checkpoint into this diode (rd_diode_load); the diode must have
        been added with the configuration of the saved one."""
        _check(self.L.rd_diode_load(self.e.h, self.index, state, len(state)))

    def life_time(self):
        h = np.zeros(1000, dtype=np.int32)
        _check(self.L.rd_life_time(self.e.h, self.index, h.ctypes.data_as(_ip)))
        return h
