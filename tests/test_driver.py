"""rd_main, the native main-loop driver (src/main.F90:175-219) over the C ABI:
it reads a RUMDEED input deck (namelist /input/ plus the `work` file) and
writes the reference's per-step text records.  On CPU: the deck is read as the
reference reads it; on the GPU: the records agree, step for step, with the
same run driven through the Python binding."""
import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "rumdeed_gb300", "_lib", "rd_main")

# The record layouts and ramo_current.dt columns of the reference's own output
# reader (scripts/python_package/rumdeed_io.py), extracted into the golden
# fixture: that module needs pandas, which is not installed, so its readers are
# restated below on its own dtypes.
with open(os.path.join(ROOT, "tests", "golden", "reference_golden.json")) as _f:
    LAYOUT = json.load(_f)["reader_layouts"]


def reader_dtype(name):
    return np.dtype([(f, t) for f, t in LAYOUT[name]])


def read_records(path, name):
    """rumdeed_io._read_records: fixed-size records, an empty file gives none."""
    dt = reader_dtype(name)
    if os.path.getsize(path) == 0:
        return np.empty(0, dtype=dt)
    return np.array(np.memmap(path, dtype=dt, mode="r", order="F"))


def read_ramo_current(path):
    """rumdeed_io.read_ramo_current: whitespace-separated columns named RAMO_COLUMNS."""
    a = np.loadtxt(path, ndmin=2)
    assert a.shape[1] == len(LAYOUT["RAMO_COLUMNS"])
    return {name: a[:, k] for k, name in enumerate(LAYOUT["RAMO_COLUMNS"])}

DECK = """&INPUT
  V_S = 2.0d3,                        ! volts over the gap
  BOX_DIM = 0.0d0, 0.0d0, 1000.0d0,   ! nm; the last is the gap
  TIME_STEP = 2.5d-4,                 ! ps
  STEPS = 12,
  EMISSION_MODE = 10,
  NREMIT = 1,
  IMAGE_CHARGE = .True.,
  N_IC_MAX = 0,
  COLLISION_MODE = 0, T_temp = 293.15d0,
  EMITTERS_DIM(1:3, 1) = 1000.0d0, 1000.0d0, 0.0d0,
  EMITTERS_POS(1:3, 1) = -500.0d0, -500.0d0, 0.0d0,
  EMITTERS_TYPE(1) = 2,
  EMITTERS_DELAY(1) = 2,
  PLANES_N = 2,
  PLANES_Z = 200.0d0, 600.0d0,
/
&GB300
  MAX_PARTICLES = 3000, SEED = 11, MH_JUMPS = 40
/
"""
WORK = "1\n2 2\n2.0 2.2\n2.4 2.6\n"


@pytest.fixture(scope="module")
def driver():
    import rumdeed_gb300 as rg
    rg.build()
    from rumdeed_gb300 import builder
    return builder.build_driver()


def _deck(tmp_path):
    (tmp_path / "input").write_text(DECK)
    (tmp_path / "work").write_text(WORK)
    return tmp_path


def test_deck_is_read_like_the_reference(driver, tmp_path):
    out = subprocess.run([driver, "--print-config", str(_deck(tmp_path))], capture_output=True, text=True,
                         check=True).stdout
    kv = {}
    for line in out.splitlines():
        k, _, v = line.partition(" ")
        kv.setdefault(k, []).append(v)
    assert kv["geometry"] == ["1"]
    assert float(kv["V_s"][0]) == 2000.0
    assert float(kv["gap"][0]) == 1000.0 * 1.0e-9           # box_dim * length_scale
    assert float(kv["time_step"][0]) == 2.5e-4 * 1.0e-12     # time_step * time_scale
    assert kv["steps"] == ["12"] and kv["image_charge"] == ["1"] and kv["N_ic_max"] == ["0"]
    assert kv["capacity"] == ["3000"] and kv["seed"] == ["11"]
    assert [float(x) for x in kv["emitter_pos"][0].split()] == [-500.0 * 1.0e-9] * 2
    assert [float(x) for x in kv["emitter_dim"][0].split()] == [1000.0 * 1.0e-9] * 2
    assert kv["work"] == ["2 x 2"]
    assert kv["emitter_delay"] == ["2"] and kv["planes"] == ["2"]
    assert [float(z) for z in kv["plane_z"]] == [200.0 * 1.0e-9, 600.0 * 1.0e-9]
    assert [float(x) for x in kv["work_value"]] == [2.0, 2.2, 2.4, 2.6]
    # Fortran edit descriptors: E14.6 and ES12.4
    assert kv["E14.6"] == ["  0.250000E-03"]
    assert kv["ES12.4"] == ["  2.5000E-04"]
    # no MH_BATCH in the deck: the reference's serial sampler (mh_batch = .false.,
    # src/mod_global.F90:316-328), and no cap on the chains below the driver's 2^20 bound
    assert kv["mh_serial"] == ["1"] and kv["max_chains"] == [str(1 << 20)]


def test_sampler_keys(driver, tmp_path):
    """MH_BATCH = .True. selects the batched sampler; /gb300/ MH_SERIAL and
    MAX_CHAINS override the defaults."""
    def cfg(deck):
        (tmp_path / "input").write_text(deck)
        (tmp_path / "work").write_text(WORK)
        out = subprocess.run([driver, "--print-config", str(tmp_path)], capture_output=True, text=True,
                             check=True).stdout
        return dict(l.split(" ", 1) for l in out.splitlines())
    assert cfg(DECK.replace("  PLANES_N = 2,", "  MH_BATCH = .True.,\n  PLANES_N = 2,"))["mh_serial"] == "0"
    assert cfg(DECK.replace("  PLANES_N = 2,", "  MH_BATCH = .False.,\n  PLANES_N = 2,"))["mh_serial"] == "1"
    c = cfg(DECK.replace("MH_JUMPS = 40", "MH_JUMPS = 40, MH_SERIAL = 0, MAX_CHAINS = 5000"))
    assert c["mh_serial"] == "0" and c["max_chains"] == "5000"


def test_gaussian_and_voronoi_work_files_are_read(driver, tmp_path):
    (tmp_path / "input").write_text(DECK)
    (tmp_path / "work").write_text("2\n4.5\n2\n-0.5 10 -20 30 40\n0.25 0 0 5 5\n")
    out = subprocess.run([driver, "--print-config", str(tmp_path)], capture_output=True, text=True,
                         check=True).stdout
    vals = [float(l.split()[1]) for l in out.splitlines() if l.startswith("work_value")]
    assert "work_model 2" in out and "work 1 x 2" in out
    assert vals == [4.5, -0.5, 10, -20, 30, 40, 0.25, 0, 0, 5, 5]
    (tmp_path / "work").write_text("4\n2\n0.25 0.5 2.0 1\n0.75 0.5 3.0 2\n")
    out = subprocess.run([driver, "--print-config", str(tmp_path)], capture_output=True, text=True,
                         check=True).stdout
    vals = [float(l.split()[1]) for l in out.splitlines() if l.startswith("work_value")]
    assert "work_model 4" in out and vals == [0.25, 0.5, 2.0, 1, 0.75, 0.5, 3.0, 2]


def test_deck_outside_the_path_is_refused(driver, tmp_path):
    (tmp_path / "input").write_text(DECK.replace("EMISSION_MODE = 10", "EMISSION_MODE = 1"))
    (tmp_path / "work").write_text(WORK)
    r = subprocess.run([driver, "--print-config", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode != 0 and "EMISSION_MODE" in r.stderr


@pytest.mark.gpu
def test_driver_run_matches_python_binding(driver, tmp_path, rg):
    deck = _deck(tmp_path)
    r = subprocess.run([driver, str(deck)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    emitted = np.loadtxt(deck / "out" / "emitted.dt")
    top = np.loadtxt(deck / "out" / "absorbed_top.dt")
    bot = np.loadtxt(deck / "out" / "absorbed_bot.dt")
    assert emitted.shape == (12, 5) and top.shape == (12, 6) and bot.shape == (12, 5)
    # the deck sets no MH_BATCH and no MAX_CHAINS: the reference's serial sampler, every
    # candidate runs a chain (the driver's chain bound is 2^20)
    eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=1, particle_capacity=3000 + 64,
                    chain_capacity=(1 << 20) + 64, quad_capacity=65536)
    d = eng.add_diode(V_s=2.0e3, gap=1000 * 1.0e-9, time_step=2.5e-4 * 1.0e-12, image_charge=True,
                      N_ic_max=0, capacity=3000, emitter_pos=(-500.0 * 1.0e-9, -500.0 * 1.0e-9),
                      emitter_dim=(1000.0 * 1.0e-9, 1000.0 * 1.0e-9), work=[[2.0, 2.2], [2.4, 2.6]], emission=True,
                      mh_jumps=40, seed=11, emitter_delay=2, planes_z=(200.0 * 1.0e-9, 600.0 * 1.0e-9),
                      mh_serial=1, max_chains=1 << 20)
    for step in range(1, 13):
        eng.step(step)
        c = d.counters()
        row = emitted[step - 1]
        assert row[1] == step
        assert row[2] == c["emitted_step"]
        assert row[3] == c["n"] + c["absorbed_top_step"] + c["absorbed_bot_step"]
        assert top[step - 1][2] == c["absorbed_top_step"] and bot[step - 1][2] == c["absorbed_bot_step"]
    assert emitted[:, 2].sum() > 0          # the deck emits
    eng.close()
    # binary event files (Fortran stream layouts), read with the reference reader's record layouts
    out = deck / "out"
    sizes = {k: reader_dtype(k).itemsize for k in ("DENSITY_EMIT_DTYPE", "DENSITY_EMIT_SPECIES_DTYPE",
                                                   "DENSITY_ABSORB_TOP_DTYPE", "DENSITY_ABSORB_BOT_DTYPE")}
    assert list(sizes.values()) == [40, 32, 52, 28]
    de = read_records(out / "density_emit.bin", "DENSITY_EMIT_DTYPE")
    dl = read_records(out / "density_emit_elec.bin", "DENSITY_EMIT_SPECIES_DTYPE")
    dt = read_records(out / "density_absorb_top.bin", "DENSITY_ABSORB_TOP_DTYPE")
    db = read_records(out / "density_absorb_bot.bin", "DENSITY_ABSORB_BOT_DTYPE")
    assert len(de) == len(dl) == emitted[:, 2].sum()
    assert len(dt) == top[:, 2].sum() and len(db) == bot[:, 2].sum()
    np.testing.assert_allclose(de["z"], 1.0, rtol=1e-12)                     # placed 1 nm above the cathode
    assert np.all(np.abs(de["x"]) <= 500.0 + 1e-9) and np.all(np.abs(de["y"]) <= 500.0 + 1e-9)   # on the emitter
    assert np.all(de["species"] == 1) and np.all(de["emit"] == 1) and np.all(np.diff(de["id"]) > 0)
    for k in ("x", "y", "z", "emit", "id"):
        np.testing.assert_array_equal(de[k], dl[k])
    assert np.all(dt["vz"] > 0.0) if len(dt) else True                      # anode hits move up
    # field.dt: one line per step the emitter is on, F_avg_z < 0, N_sup as in the counters
    fd = np.loadtxt(out / "field.dt")
    assert fd.shape == (12 - 2, 8) and np.all(fd[:, 0] == np.arange(3, 13)) and np.all(fd[:, 3] < 0)
    # integration.dt: emitter, regions (50 x 50 panels: nodes 5 nm apart over 1000 nm), nodes
    # (200 x 200), fail 0, N_sup, 0, 0
    ig = np.loadtxt(out / "integration.dt")
    assert ig.shape == (10, 7) and np.all(ig[:, :4] == [1, 2500, 40000, 0])
    np.testing.assert_allclose(ig[:, 4], fd[:, 4], rtol=1e-4)
    # the files the reference creates on every run exist (empty outside their modes)
    for name in ("density_emit_ion.bin", "density_emit_atom.bin", "density_ion.bin", "absorbed_recom.dt",
                 "mh.bin", "position.bin", "ramo_current.bin", "init.bin", "init.dt", "volt.dt"):
        assert (out / name).exists(), name
    assert emitted[0, 2] == emitted[1, 2] == 0 and emitted[2:, 2].sum() > 0  # EMITTERS_DELAY = 2
    # planes-1.bin / planes-2.bin: 52-byte records of upward crossings of 200 nm / 600 nm
    p1 = read_records(out / "planes-1.bin", "PLANES_DTYPE")
    p2 = read_records(out / "planes-2.bin", "PLANES_DTYPE")
    assert len(p1) >= len(p2) and np.all(p1["vz"] > 0) if len(p1) else True
    # ramo_current.dt: nrPart / nrElec / nrIon at the velocity update (before removal) equal the
    # electrons in flight that emitted.dt records after the emission of the step
    ramo = read_ramo_current(out / "ramo_current.dt")
    assert len(ramo["step"]) == 12 and np.all(ramo["step"] == np.arange(1, 13))
    np.testing.assert_array_equal(ramo["nrPart"], emitted[:, 3])
    np.testing.assert_array_equal(ramo["nrElec"], emitted[:, 3])
    assert np.all(ramo["nrIon"] == 0) and np.all(ramo["avg_mob"] >= 0)
    # volt.dt: "(ES12.4, tr2, i8, tr2, ES18.8)" with 4 items: time, step, V_d, then V_rf alone on
    # the next record by format reversion (Set_Voltage, src/mod_verlet.F90:2050-2057)
    vl = (out / "volt.dt").read_text().splitlines()
    assert len(vl) == 2 * 12
    assert vl[0] == "  2.5000E-04         1      2.00000000E+03" and vl[1] == "  0.0000E+00"
    assert vl[22].split()[1] == "12"


@pytest.mark.gpu
def test_optional_position_and_section_current_files(driver, tmp_path, rg):
    """WRITE_POSITION_FILE and WRITE_RAMO_SEC: out/position.bin (Write_Position,
    src/mod_pair.F90:841-867, positions after Update_Position with the removed
    particles still in place) and out/ramo_current.bin (ramo_current_emit per
    section, 96 x 96 x 1 doubles a step).  The phase-by-phase stepping these
    files need gives the same records as the graph-captured step."""
    plain = tmp_path / "plain"
    plain.mkdir()
    _deck(plain)
    r = subprocess.run([driver, str(plain)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    opt = tmp_path / "opt"
    opt.mkdir()
    (opt / "input").write_text(DECK.replace("  PLANES_N = 2,", "  WRITE_POSITION_FILE = .True.,\n"
                                            "  WRITE_RAMO_SEC = .True.,\n  PLANES_N = 2,"))
    (opt / "work").write_text(WORK)
    r = subprocess.run([driver, str(opt)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    for name in ("emitted.dt", "absorbed_top.dt", "absorbed_bot.dt", "field.dt"):
        assert (opt / "out" / name).read_text() == (plain / "out" / name).read_text(), name
    emitted = np.loadtxt(opt / "out" / "emitted.dt")
    top = np.loadtxt(opt / "out" / "absorbed_top.dt")
    bot = np.loadtxt(opt / "out" / "absorbed_bot.dt")
    raw = (opt / "out" / "position.bin").read_bytes()
    head = np.frombuffer(raw[:8], dtype="<i4")
    assert list(head) == [12, 1]
    rec = reader_dtype("POSITION_PARTICLE_DTYPE")   # rumdeed_io.read_position_step's records
    off = 8
    for step in range(1, 13):
        st, n = np.frombuffer(raw[off:off + 8], dtype="<i4")
        off += 8
        assert st == step
        # in flight after the position update = emitted so far - absorbed in earlier steps
        absorbed_before = top[:step - 1, 2].sum() + bot[:step - 1, 2].sum()
        assert n == emitted[:step, 2].sum() - absorbed_before
        parts = np.frombuffer(raw[off:off + n * rec.itemsize], dtype=rec)
        off += n * rec.itemsize
        assert np.all(parts["emit"] == 1) and np.all(np.diff(parts["id"]) > 0)
        assert np.all(parts["sec"] >= 1) and np.all(parts["sec"] <= 4)   # the 2 x 2 work grid
    assert off == len(raw)
    # init.bin (Write_Initial_Variables): 7 float64 then 4 int32; the reference's readers take the
    # ramo_current.bin dimensions from it
    init = np.fromfile(opt / "out" / "init.bin", dtype=reader_dtype("INIT_DTYPE"), count=1)   # read_init
    assert len(init) == 1 and (opt / "out" / "init.bin").stat().st_size == 72
    np.testing.assert_allclose([init[k][0] for k in ("epsilon_r", "m_eeff", "m_ieff", "length_scale", "time_scale",
                                                     "vel_scale", "cur_scale")], [1, 1, 1, 1e-9, 1e-12, 1e3, 1])
    assert (init["MAX_PARTICLES"][0], init["MAX_EMITTERS"][0], init["MAX_SECTIONS"][0]) == (3000, 1, 96 * 96)
    assert (opt / "out" / "ramo_current.bin").stat().st_size == 96 * 96 * 1 * 12 * 8
    rs = np.fromfile(opt / "out" / "ramo_current.bin", dtype="<f8").reshape(12, 96 * 96)
    ramo = read_ramo_current(opt / "out" / "ramo_current.dt")
    np.testing.assert_allclose(rs.sum(axis=1), ramo["ramo_elec"], rtol=1e-4, atol=1e-30)   # ES12.4 text
    assert np.all(rs[:, 4:] == 0.0) and np.abs(rs).sum() > 0


@pytest.mark.gpu
def test_stop_signal_ends_the_run_cleanly(driver, tmp_path):
    """SIGUSR1 (Slurm's warning) or SIGINT stops the main loop after the
    current step, as the reference's Signal_Handler does: exit status 0, the
    stop message, whole records for the steps that ran."""
    import signal
    import time
    (tmp_path / "input").write_text(DECK.replace("STEPS = 12", "STEPS = 200000"))
    (tmp_path / "work").write_text(WORK)
    p = subprocess.Popen([driver, str(tmp_path)], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    emitted = tmp_path / "out" / "emitted.dt"
    t0 = time.time()
    while time.time() - t0 < 120 and not (emitted.exists() and emitted.stat().st_size > 0):
        time.sleep(0.2)
    p.send_signal(signal.SIGUSR1)
    out, err = p.communicate(timeout=120)
    assert p.returncode == 0, err
    assert "Got signal SIGINT stopping main loop." in out
    rows = np.loadtxt(emitted, ndmin=2)
    assert 0 < len(rows) < 200000 and rows.shape[1] == 5
    assert np.all(rows[:, 1] == np.arange(1, len(rows) + 1))


@pytest.mark.gpu
def test_event_log_counts_and_loss(rg):
    eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=1, particle_capacity=3000 + 64,
                    chain_capacity=3000 + 64, quad_capacity=65536, event_capacity=8)
    d = eng.add_diode(V_s=2.0e3, gap=1000 * 1.0e-9, time_step=2.5e-4 * 1.0e-12, image_charge=True,
                      N_ic_max=0, capacity=3000, emitter_pos=(-500.0 * 1.0e-9, -500.0 * 1.0e-9),
                      emitter_dim=(1000.0 * 1.0e-9, 1000.0 * 1.0e-9), work=[[2.0, 2.2], [2.4, 2.6]],
                      emission=True, mh_jumps=40, seed=11)
    eng.step(1)
    ev, lost = eng.events_take()
    c = d.counters()
    assert c["emitted_step"] > 8
    assert len(ev) == 8 and lost == c["emitted_step"] - 8                 # the log holds 8
    assert all(r["kind"] == rg.EVENT_EMIT and r["step"] == 1 for r in ev)
    assert [r["id"] for r in ev] == sorted(r["id"] for r in ev)
    ev2, lost2 = eng.events_take()                                           # emptied by the take
    assert ev2 == [] and lost2 == 0
    eng.close()
