"""GPU parity tests: librumdeed_gb300 (through its C ABI) against the CPU oracle.

Tolerances (per particle / point, norm-relative, as src/mod_tests.F90:1665-1669):
  FP64 plain form          <= 1e-12
  FP32 compensated form    <= 1e-5  (the stated force tolerance of the FP32 form)
Integer and index results (counts, ids, order, emitted sets) must be equal.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NM = 1e-9
TOL64, TOL32 = 1e-12, 1e-5


def nrel(a, b):
    a = np.asarray(a); b = np.asarray(b)
    return np.max(np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300))


def uniform_particles(rng, n, half=500 * NM, d=1000 * NM):
    return np.column_stack([rng.uniform(-half, half, n), rng.uniform(-half, half, n),
                            rng.uniform(1 * NM, d - 1 * NM, n)])


def both(rg, orc, prec, n=300, ic=True, nic=0, seed=1, ions=False, V=2e3, d=1000 * NM):
    rng = np.random.default_rng(seed)
    pos = uniform_particles(rng, n, d=d)
    sp = np.where(np.arange(n) % 5 == 4, 2, 1) if ions else np.ones(n, dtype=int)
    eng = rg.Engine(precision=prec, max_diodes=4, particle_capacity=max(4 * n, 4096))
    dio = eng.add_diode(V_s=V, gap=d, capacity=max(2 * n, 1024), image_charge=ic, N_ic_max=nic)
    dio.add_particles(pos, species=sp)
    o = orc.OracleDiode(cap=max(2 * n, 1024), V_s=V, d=d, image_charge=ic, N_ic_max=nic)
    for p, s in zip(pos, sp):
        o.add(p, species=int(s))
    return eng, dio, o, pos


@pytest.mark.parametrize("ic,nic,ions", [(True, 0, False), (True, 2, True), (False, 0, True), (True, 7, False)])
def test_accel_fp64_matches_oracle(rg, orc, ic, nic, ions):
    eng, dio, o, _ = both(rg, orc, rg.PREC_FP64, n=333, ic=ic, nic=nic, ions=ions)
    acc = dio.calculate_acceleration_particles()
    assert nrel(acc, o.accel("gather", True)) <= TOL64
    # and the reference CPU pair loop gives the same up to rounding
    assert nrel(acc, o.accel("planar", True)) <= TOL64
    eng.close()


@pytest.mark.parametrize("n,nic", [(1000, 0), (2048, 7), (700, 1)])
def test_accel_fp32c_within_tolerance(rg, orc, n, nic):
    eng, dio, o, _ = both(rg, orc, rg.PREC_FP32C, n=n, nic=nic)
    acc = dio.calculate_acceleration_particles()
    ref = o.accel("gather", True)
    assert nrel(acc, ref) <= TOL32
    # also on the pair part alone (vacuum-field term removed)
    k = orc.constants()
    vac = np.array([0.0, 0.0, -k["q_0"] / k["m_0"] * (-2e3 / (1000 * NM))])
    assert nrel(acc - vac, ref - vac) <= 1e-4
    eng.close()


def test_field_at_parity(rg, orc):
    rng = np.random.default_rng(3)
    pts = np.vstack([uniform_particles(rng, 100),
                     np.column_stack([rng.uniform(-500 * NM, 500 * NM, 100),
                                      rng.uniform(-500 * NM, 500 * NM, 100), np.zeros(100)])])
    for prec, tol in ((rg.PREC_FP64, TOL64), (rg.PREC_FP32C, TOL32)):
        for nic in (0, 3):
            eng, dio, o, _ = both(rg, orc, prec, n=500, nic=nic, seed=4)
            f = dio.calc_field_at_batch(pts)
            assert nrel(f, o.field_at(pts)) <= tol, (prec, nic)
            eng.close()


def test_golden_probe_on_gpu(rg, orc):
    """Test_Acceleration_Without_Image_Charge field golden value through the GPU."""
    for prec in (rg.PREC_FP64, rg.PREC_FP32C):
        eng = rg.Engine(precision=prec, max_diodes=2, particle_capacity=4096)
        d = eng.add_diode(V_s=2.0, gap=100 * NM, capacity=64, image_charge=False)
        R = np.array([[3.0, -10.0, 2.0], [-9.0, 26.0, 80.0], [6.0, -24.0, 56.53]]) * NM
        d.add_particles(R, species=[1, 1, 2])
        probe = np.array([[np.float32(-4.55), np.float32(-2.34), np.float32(96.44)]], dtype=np.float64) * NM
        E = d.calc_field_at_batch(probe)[0]
        gold = np.array([-314559.29097098, 1423979.07058996, -20246038.87978313])
        assert np.all(np.abs(E - gold) / np.abs(gold) < 0.02)
        eng.close()


def test_tip_accel_and_field(rg, orc):
    rng = np.random.default_rng(11)
    tip = (900 * NM, 100 * NM, 100 * NM)
    n = 257
    # particles above the tip surface
    pos = np.column_stack([rng.uniform(-300 * NM, 300 * NM, n), rng.uniform(-300 * NM, 300 * NM, n),
                           rng.uniform(105 * NM, 990 * NM, n)])
    pts = np.array([[0.0, 0.0, 102.0], [30.0, -10.0, 130.0], [-50.0, 40.0, 300.0], [15.0, 8.0, 500.0]]) * NM
    o = orc.OracleDiode(orc.TIP, cap=1024, V_s=2e3, d=1000 * NM, image_charge=True)
    o.set_tip(*tip, 4.7)
    for p in pos:
        o.add(p)
    ref = o.accel("gather", True)
    fref = o.field_at(pts)
    for prec, tol in ((rg.PREC_FP64, TOL64), (rg.PREC_FP32C, TOL32)):
        eng = rg.Engine(precision=prec, max_diodes=2, particle_capacity=4096)
        d = eng.add_diode(geometry=rg.GEOM_TIP, V_s=2e3, capacity=1024, tip_dim=tip)
        d.add_particles(pos)
        assert nrel(d.calculate_acceleration_particles(), ref) <= tol
        assert nrel(d.calc_field_at_batch(pts), fref) <= tol
        eng.close()


def test_beeman_kinematics_gpu(rg, orc):
    """Test_Beeman_Kinematics (src/mod_tests.F90:1403-1452) through rd_update_position."""
    k = orc.constants()
    d, V, dt, vx0 = 1000 * NM, 2.0e3, 0.25e-15, 1.0e3
    for prec in (rg.PREC_FP64, rg.PREC_FP32C):
        eng = rg.Engine(precision=prec, max_diodes=2, particle_capacity=4096)
        dio = eng.add_diode(V_s=V, gap=d, time_step=dt, image_charge=False, capacity=16)
        dio.add_particle([0.0, 0.0, 500 * NM], vel=[vx0, 0.0, 0.0])
        for i in range(1, 4):
            eng.update_position(i)
        p = dio.particles()
        az = k["q_0"] * V / (k["m_0"] * d)
        assert p["pos"][0, 2] - 500 * NM == pytest.approx(4.5 * az * dt ** 2, rel=1e-12)
        assert p["vel"][0, 2] == pytest.approx(3 * az * dt, rel=1e-12)
        assert p["pos"][0, 0] == pytest.approx(3 * vx0 * dt, rel=1e-12)
        assert dio.counters()["ramo_current"] == pytest.approx(k["q_0"] * 3 * az * dt / d, rel=1e-12)
        eng.close()


def test_transit_time_gpu(rg, orc):
    """Test_Transit_Time (src/mod_tests.F90:912-977) with rd_update_position + rd_remove_particles."""
    k = orc.constants()
    d, V, dt, z0 = 1000 * NM, 2.0e3, 0.25e-15, 1.0 * NM
    steps_exp = int(np.ceil(np.sqrt(2 * d * (d - z0) * k["m_0"] / (k["q_0"] * V)) / dt))
    eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=2, particle_capacity=4096)
    dio = eng.add_diode(V_s=V, gap=d, time_step=dt, capacity=16)
    dio.add_particle([0.0, 0.0, z0])
    o = orc.OracleDiode(cap=16, V_s=V, d=d, time_step=dt)
    o.add([0.0, 0.0, z0])
    res = None
    for i in range(1, steps_exp + 100):
        eng.update_position(i)
        eng.remove_particles(i)
        o.verlet(i); o.remove(i)
        if res is None and dio.n == 0:
            res = i
            break
    assert res is not None and abs(res - steps_exp) < 0.01 * steps_exp
    assert o.n == 0       # oracle absorbed on the same step
    c = dio.counters()
    assert c["absorbed_top_total"] == 1
    assert dio.life_time()[res - 1 - 1] == 1 or dio.life_time().sum() == 0
    eng.close()


def test_removal_compaction_gpu(rg, orc):
    """Test_Particle_Removal (src/mod_tests.F90:1193-1289) semantics on the device."""
    eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=2, particle_capacity=8192)
    dio = eng.add_diode(V_s=2.0, gap=100 * NM, capacity=3000, image_charge=False)
    n = 2500
    R = np.column_stack([np.arange(1, n + 1) * 0.01 * NM, -np.arange(1, n + 1) * 0.02 * NM,
                         np.linspace(1, 99, n) * NM])
    V = np.column_stack([np.arange(1, n + 1) * 100.0, -np.arange(1, n + 1) * 50.0, np.arange(1, n + 1) * 25.0])
    dio.add_particles(R, V, species=np.where(np.arange(n) % 7 == 3, 2, 1), step=1)
    rng = np.random.default_rng(2)
    dead = np.sort(rng.choice(n, 321, replace=False))
    for i in dead:
        dio.mark_particles_remove(int(i), rg.REMOVE_TOP)
    dio.mark_particles_remove(int(dead[0]), rg.REMOVE_TOP)     # double mark is a no-op
    eng.remove_particles(11)
    keep = np.setdiff1d(np.arange(n), dead)
    p = dio.particles()
    assert dio.n == n - len(dead)
    np.testing.assert_array_equal(p["pos"], R[keep])
    np.testing.assert_array_equal(p["vel"], V[keep])
    np.testing.assert_array_equal(p["id"], keep)
    n_elec_dead = int(np.sum((dead % 7) != 3))
    assert dio.life_time()[9] == n_elec_dead
    c = dio.counters()
    assert c["absorbed_top_total"] == n_elec_dead
    eng.close()


def test_inplace_compaction_many_tiles(rg):
    """The in-place compaction over many 1024-particle tiles: a diode losing three
    in four (survivors written over many earlier tiles, whose loads each tile waits
    for), one with 1 % scattered removals (Util/bench_compact.f90's scenario), one
    with none and one losing all, compacted twice in a row (the tile counter and the
    load flags reset between launches).  Survivors keep creation order with their
    state, as compact_array does (src/mod_pair.F90:1180-1223)."""
    eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=4, particle_capacity=100000)
    rng = np.random.default_rng(31)
    sizes = [24000, 30000, 5000, 6000]
    dios, data, alive = [], [], []
    for n in sizes:
        d = eng.add_diode(V_s=2.0e3, gap=1000 * NM, capacity=n, image_charge=False)
        R = np.column_stack([rng.uniform(-500, 500, n), rng.uniform(-500, 500, n), rng.uniform(1, 999, n)]) * NM
        V = rng.normal(0.0, 1.0e5, (n, 3))
        d.add_particles(R, V, species=np.where(np.arange(n) % 5 == 2, 2, 1), step=1)
        dios.append(d)
        data.append((R, V))
        alive.append(np.arange(n))
    for rnd in range(2):
        dead = [alive[0][(np.arange(len(alive[0])) % 4) != 0],
                np.sort(rng.choice(alive[1], len(alive[1]) // 100, replace=False)),
                np.array([], dtype=int),
                alive[3] if rnd == 0 else np.array([], dtype=int)]
        for d, k, dd in zip(dios, alive, dead):
            pos_of = {int(v): j for j, v in enumerate(k)}
            for i in dd:
                d.mark_particles_remove(pos_of[int(i)], rg.REMOVE_TOP)
        eng.remove_particles(5 + rnd)
        alive = [np.setdiff1d(k, dd) for k, dd in zip(alive, dead)]
        for d, k, (R, V) in zip(dios, alive, data):
            assert d.n == len(k)
            p = d.particles()
            np.testing.assert_array_equal(p["id"][:len(k)], k)
            np.testing.assert_array_equal(p["pos"][:len(k)], R[k])
            np.testing.assert_array_equal(p["vel"][:len(k)], V[k])
        assert sum(eng.validate().values()) == 0
    for d, n, k in zip(dios, sizes, alive):
        removed = np.setdiff1d(np.arange(n), k)
        n_elec = int(np.sum((removed % 5) != 2))
        # the reference records no life times when a diode loses every particle
        expect = 0 if d is dios[3] else n_elec
        assert int(d.life_time().sum()) == expect
        assert d.counters()["absorbed_top_total"] == n_elec
    eng.close()


def _emission_pair(rg, orc, prec, seed=77, n0=150, work=2.0, jumps=40, chains=300):
    rng = np.random.default_rng(seed)
    d, V = 500 * NM, 1.0e3
    pos = np.column_stack([rng.uniform(-60 * NM, 60 * NM, n0), rng.uniform(-60 * NM, 60 * NM, n0),
                           rng.uniform(2 * NM, 490 * NM, n0)])
    eng = rg.Engine(precision=prec, max_diodes=2, particle_capacity=8192, chain_capacity=4096)
    dio = eng.add_diode(V_s=V, gap=d, capacity=4096, emitter_pos=(-50 * NM, -50 * NM),
                        emitter_dim=(100 * NM, 100 * NM), work=[[work]], emission=True,
                        mh_jumps=jumps, max_chains=chains, quad_panels=8, quad_order=4, seed=seed)
    dio.add_particles(pos)
    o = orc.OracleDiode(cap=4096, V_s=V, d=d)
    o.set_planar_emitter(-50 * NM, -50 * NM, 100 * NM, 100 * NM, [[work]])
    o.set_emission(True, seed=seed, mh_jumps=jumps, max_chains=chains, quad_panels=8, quad_order=4)
    for p in pos:
        o.add(p)
    return eng, dio, o


def test_emission_fp64_matches_oracle_chain_for_chain(rg, orc):
    """Supply integral, MH chains (shared Philox streams) and the emission
    test: the FP64 GPU form reproduces the oracle's emitted electrons."""
    eng, dio, o = _emission_pair(rg, orc, rg.PREC_FP64)
    n_before = dio.n
    eng.do_emission(1)
    o.emission(1)
    c = dio.counters()
    assert c["N_sup"] == pytest.approx(o.s.N_sup, rel=1e-12)
    assert c["chains"] == o.s.last_chains
    assert c["MH_std"] == pytest.approx(o.s.MH_std, rel=1e-12)
    assert c["emitted_step"] == o.s.emitted_step > 0
    assert c["F_avg"][2] == pytest.approx(o.s.F_avg_z, rel=1e-12) and c["F_avg"][2] < 0   # field.dt
    assert c["df_avg"] == pytest.approx(o.s.df_avg, rel=1e-10)
    p = dio.particles()
    assert dio.n == o.n
    new = slice(n_before, dio.n)
    assert np.max(np.abs(p["pos"][new] - o.arr("pos")[new])) < 1e-12 * 100 * NM
    np.testing.assert_array_equal(p["id"], o.iarr("id"))
    eng.close()


def test_full_steps_fp64_trajectory(rg, orc):
    """Five main-loop iterations (emission, Beeman, forces, removal) agree."""
    eng, dio, o = _emission_pair(rg, orc, rg.PREC_FP64, seed=5, jumps=20)
    for i in range(1, 6):
        eng.step(i)
        o.step(i)
        assert dio.n == o.n, i
    p = dio.particles()
    assert np.max(np.abs(p["pos"] - o.arr("pos"))) < 1e-9 * NM
    assert nrel(p["vel"] + 1e-3, o.arr("vel") + 1e-3) < 1e-8
    c = dio.counters()
    assert c["emitted_total"] == o.s.emitted_total
    assert c["ramo_current"] == pytest.approx(o.s.ramo_current, rel=1e-9)
    _check_average_velocities(c, o)
    eng.close()


def _check_average_velocities(c, o):
    """Average_Velocities (src/mod_verlet.F90:428-447) of the last step against the oracle."""
    assert (c["n_part_vel"], c["n_elec_vel"], c["n_ion_vel"]) == (o.s.n_part_vel, o.s.n_elec_vel, o.s.n_ion_vel)
    for key in ("avg_part_vel", "avg_elec_vel", "avg_ion_vel"):
        np.testing.assert_allclose(c[key], list(getattr(o.s, key)), rtol=1e-8, atol=1e-6, err_msg=key)
    assert c["avg_mob"] == pytest.approx(o.s.avg_mob, rel=1e-8, abs=1e-18)


def test_emission_fp32c_statistics(rg, orc):
    """The FP32 compensated form emits the same electrons as the FP64 oracle
    unless a decision sits within the FP32 field error of its threshold."""
    eng, dio, o = _emission_pair(rg, orc, rg.PREC_FP32C, seed=9)
    eng.do_emission(1)
    o.emission(1)
    c = dio.counters()
    assert c["N_sup"] == pytest.approx(o.s.N_sup, rel=1e-5)
    assert abs(c["emitted_step"] - o.s.emitted_step) <= max(2, 0.05 * o.s.emitted_step)
    eng.close()


def test_tip_emission_fp32c_statistics(rg, orc):
    """Tip emission in the FP32 compensated form (packed FP32x2 field tiles of
    the tip MH jump) against the FP64 oracle: the same supply integral and
    chain count, and emitted counts that differ only where an accept or
    escape decision sits within the FP32 field error of its threshold."""
    tip = (900 * NM, 100 * NM, 100 * NM)
    rng = np.random.default_rng(17)
    n = 3000
    pos = np.column_stack([rng.uniform(-300 * NM, 300 * NM, n), rng.uniform(-300 * NM, 300 * NM, n),
                           rng.uniform(110 * NM, 990 * NM, n)])
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=2, particle_capacity=16384, chain_capacity=16384,
                    quad_capacity=20000)
    d = eng.add_diode(geometry=rg.GEOM_TIP, V_s=800.0, time_step=0.25e-15, capacity=8192, tip_dim=tip,
                      tip_work_function=3.0, emission=True, mh_jumps=40, max_chains=2000, seed=5)
    d.add_particles(pos, step=0)
    o = orc.OracleDiode(orc.TIP, cap=8192, V_s=800.0, d=1000 * NM)
    o.set_tip(*tip, 3.0)
    o.set_emission(True, seed=5, mh_jumps=40, max_chains=2000)
    for p in pos:
        o.add(p, step=0)
    eng.do_emission(1)
    o.emission(1)
    c = d.counters()
    assert c["N_sup"] == pytest.approx(o.s.N_sup, rel=1e-5)
    assert c["chains"] == o.s.last_chains
    assert o.s.emitted_step > 100   # 280 of 744 chains with these numbers
    assert abs(c["emitted_step"] - o.s.emitted_step) <= max(2, 0.05 * o.s.emitted_step)
    eng.close()


def test_tip_emission_fp64(rg, orc):
    tip = (900 * NM, 100 * NM, 100 * NM)
    eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=2, particle_capacity=8192, chain_capacity=8192,
                    quad_capacity=20000)
    d = eng.add_diode(geometry=rg.GEOM_TIP, V_s=800.0, time_step=0.25e-15, capacity=4096, tip_dim=tip,
                      emission=True, mh_jumps=20, max_chains=500, seed=3)
    o = orc.OracleDiode(orc.TIP, cap=4096, V_s=800.0, d=1000 * NM)
    o.set_tip(*tip, 4.7)
    o.set_emission(True, seed=3, mh_jumps=20, max_chains=500)
    for i in range(1, 3):
        eng.step(i)
        o.step(i)
        c = d.counters()
        assert c["N_sup"] == pytest.approx(o.s.N_sup, rel=1e-10)
        assert c["emitted_step"] == o.s.emitted_step
        assert d.n == o.n
    p = d.particles()
    if d.n:
        assert np.max(np.abs(p["pos"] - o.arr("pos"))) < 1e-6 * NM
    eng.close()


def test_batch_equals_alone(rg, orc):
    """A diode advanced alone and inside a mix of diodes gives bit-identical
    results: the work split of a diode depends only on its own counts."""
    rng = np.random.default_rng(21)
    cfgs = [dict(V_s=rng.uniform(500, 5000), gap=rng.uniform(200, 2000) * NM, capacity=int(c))
            for c in (300, 1500, 700)]
    pos = [uniform_particles(rng, c["capacity"] // 2, d=c["gap"]) for c in cfgs]
    for prec in (rg.PREC_FP32C, rg.PREC_FP64):
        solo = rg.Engine(precision=prec, max_diodes=2, particle_capacity=8192)
        a = solo.add_diode(**cfgs[1]); a.add_particles(pos[1])
        solo.run(1, 5)
        mix = rg.Engine(precision=prec, max_diodes=8, particle_capacity=16384)
        ds = [mix.add_diode(**c) for c in cfgs]
        for dd, p in zip(ds, pos):
            dd.add_particles(p)
        mix.run(1, 5)
        pa, pb = a.particles(), ds[1].particles()
        assert a.n == ds[1].n
        np.testing.assert_array_equal(pa["pos"], pb["pos"])
        np.testing.assert_array_equal(pa["vel"], pb["vel"])
        solo.close(); mix.close()


WORK_MODELS = {
    # Gaussian: base 2.3 eV, a 0.6 eV dip and a 0.3 eV bump (nm)
    2: [2.2, -0.6, -20.0, 10.0, 25.0, 15.0, 0.3, 30.0, -25.0, 10.0, 20.0],
    # Voronoi: four sites (fractions of the emitter), phi, section
    4: [0.2, 0.2, 1.6, 1.0, 0.8, 0.3, 1.7, 2.0, 0.4, 0.8, 1.65, 3.0, 0.7, 0.7, 2.4, 4.0],
}


@pytest.mark.parametrize("model", [2, 4])
def test_emission_work_models_fp64_match_oracle(rg, orc, model):
    """Gaussian and Voronoi work functions (mod_work_function.F90:214-254,
    :533-571): supply integral, MH chains and emission of the FP64 GPU form
    match the oracle electron for electron, sections included."""
    rng = np.random.default_rng(21)
    d, V, n0 = 500 * NM, 1.0e3, 120
    pos = np.column_stack([rng.uniform(-60 * NM, 60 * NM, n0), rng.uniform(-60 * NM, 60 * NM, n0),
                           rng.uniform(2 * NM, 490 * NM, n0)])
    kw = dict(V_s=V, gap=d, capacity=4096, emitter_pos=(-50 * NM, -50 * NM), emitter_dim=(100 * NM, 100 * NM),
              work=WORK_MODELS[model], work_model=model, emission=True, mh_jumps=40, max_chains=300,
              quad_panels=8, quad_order=4, seed=5)
    eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=2, particle_capacity=8192, chain_capacity=4096)
    dio = eng.add_diode(**kw)
    dio.add_particles(pos)
    o = orc.OracleDiode(cap=4096, V_s=V, d=d)
    o.set_planar_emitter(-50 * NM, -50 * NM, 100 * NM, 100 * NM)
    o.set_work_model(model, WORK_MODELS[model])
    o.set_emission(True, seed=5, mh_jumps=40, max_chains=300, quad_panels=8, quad_order=4)
    for p in pos:
        o.add(p)
    n_before = dio.n
    eng.do_emission(1)
    o.emission(1)
    c = dio.counters()
    assert c["N_sup"] == pytest.approx(o.s.N_sup, rel=1e-12)
    assert c["emitted_step"] == o.s.emitted_step > 0
    p = dio.particles()
    new = slice(n_before, dio.n)
    assert np.max(np.abs(p["pos"][new] - o.arr("pos")[new])) < 1e-12 * 100 * NM
    np.testing.assert_array_equal(p["section"], o.iarr("section"))
    if model == 4:
        assert len(set(p["section"][new])) > 1      # several Voronoi cells emit
    eng.close()
    # the FP32-compensated form on the same deck: same supply, statistically the same emission
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=2, particle_capacity=8192, chain_capacity=4096)
    dio = eng.add_diode(**kw)
    dio.add_particles(pos)
    eng.do_emission(1)
    c32 = dio.counters()
    assert c32["N_sup"] == pytest.approx(o.s.N_sup, rel=1e-5)
    assert abs(c32["emitted_step"] - o.s.emitted_step) <= 4 * np.sqrt(o.s.emitted_step) + 2
    eng.close()


def test_emitter_delay_matches_oracle(rg, orc):
    """EMITTERS_DELAY: the emitter emits from step delay + 1 on (fe_v2:181)."""
    o = orc.OracleDiode(cap=4096, V_s=1.0e3, d=500 * NM)
    o.set_planar_emitter(-50 * NM, -50 * NM, 100 * NM, 100 * NM, [[2.0]])
    o.set_emission(True, seed=77, mh_jumps=40, max_chains=300, quad_panels=8, quad_order=4)
    eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=2, particle_capacity=8192, chain_capacity=4096)
    dio = eng.add_diode(V_s=1.0e3, gap=500 * NM, capacity=4096, emitter_pos=(-50 * NM, -50 * NM),
                        emitter_dim=(100 * NM, 100 * NM), work=[[2.0]], emission=True, mh_jumps=40,
                        max_chains=300, quad_panels=8, quad_order=4, seed=77, emitter_delay=2)
    o.s.emit_delay = 2
    emitted = []
    for step in range(1, 5):
        eng.step(step)
        o.step(step)
        c = dio.counters()
        assert c["emitted_step"] == o.s.emitted_step
        emitted.append(c["emitted_step"])
    assert emitted[0] == emitted[1] == 0 and emitted[2] > 0
    eng.close()


def test_planes_log_upward_crossings(rg):
    """Check_Planes (src/mod_verlet.F90:343-367): a particle whose z passes a
    plane upwards during the position update is logged once for that plane."""
    rng = np.random.default_rng(8)
    n = 400
    pos = np.column_stack([rng.uniform(-50 * NM, 50 * NM, n), rng.uniform(-50 * NM, 50 * NM, n),
                           rng.uniform(5 * NM, 480 * NM, n)])
    vel = np.column_stack([np.zeros(n), np.zeros(n), rng.uniform(-2e5, 6e6, n)])
    planes = (100 * NM, 250 * NM, 0.0)
    eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=1, particle_capacity=1024, chain_capacity=256,
                    event_capacity=4096)
    d = eng.add_diode(V_s=1.0e3, gap=500 * NM, capacity=1000, time_step=2e-15, planes_z=planes)
    d.add_particles(pos, vel=vel)
    for step in range(1, 4):
        before = d.particles()
        zb = dict(zip(before["id"], before["pos"][:, 2]))
        eng.update_position(step)
        after = d.particles()        # marked particles are still present until removal
        za = dict(zip(after["id"], after["pos"][:, 2]))
        eng.remove_particles(step)
        ev, lost = eng.events_take()
        assert lost == 0
        for k, zp in enumerate(planes):
            got = sorted(r["id"] for r in ev if r["kind"] == rg.EVENT_PLANE + k)
            want = sorted(i for i in za if zp > 0 and zb[i] < zp < za[i])
            assert got == want
        assert any(r["kind"] >= rg.EVENT_PLANE for r in ev) or step > 1
    eng.close()


def test_serial_mh_fp64_matches_oracle(rg, orc):
    """mh_batch = .false. (the reference's default): each chain runs to
    completion, sees the electrons earlier chains emitted in the same step and
    updates MH_std once (src/mod_field_emission_v2.F90:322-333, 1122-1265).
    The FP64 GPU form reproduces the oracle's serial sampler electron for
    electron over two steps."""
    rng = np.random.default_rng(31)
    d, V, n0 = 500 * NM, 1.0e3, 150
    pos = np.column_stack([rng.uniform(-60 * NM, 60 * NM, n0), rng.uniform(-60 * NM, 60 * NM, n0),
                           rng.uniform(2 * NM, 490 * NM, n0)])
    eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=2, particle_capacity=8192, chain_capacity=4096)
    dio = eng.add_diode(V_s=V, gap=d, capacity=4096, emitter_pos=(-50 * NM, -50 * NM),
                        emitter_dim=(100 * NM, 100 * NM), work=[[2.0]], emission=True, mh_jumps=40,
                        max_chains=300, quad_panels=8, quad_order=4, seed=31, mh_serial=True)
    dio.add_particles(pos)
    o = orc.OracleDiode(cap=4096, V_s=V, d=d)
    o.set_planar_emitter(-50 * NM, -50 * NM, 100 * NM, 100 * NM, [[2.0]])
    o.set_emission(True, seed=31, mh_jumps=40, max_chains=300, quad_panels=8, quad_order=4)
    o.s.mh_serial = 1
    for p in pos:
        o.add(p)
    for step in (1, 2):
        eng.do_emission(step)
        o.emission(step)
        c = dio.counters()
        assert c["N_sup"] == pytest.approx(o.s.N_sup, rel=1e-12)
        assert c["emitted_step"] == o.s.emitted_step > 0
        assert c["MH_std"] == pytest.approx(o.s.MH_std, rel=1e-12)
        assert c["df_avg"] == pytest.approx(o.s.df_avg, rel=1e-10)
        assert dio.n == o.n
        p = dio.particles()
        assert np.max(np.abs(p["pos"] - o.arr("pos")[:dio.n])) < 1e-12 * 100 * NM
        np.testing.assert_array_equal(p["id"], o.iarr("id"))
    eng.close()
    # the FP32-compensated serial form: same supply, statistically the same emission
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=2, particle_capacity=8192, chain_capacity=4096)
    dio = eng.add_diode(V_s=V, gap=d, capacity=4096, emitter_pos=(-50 * NM, -50 * NM),
                        emitter_dim=(100 * NM, 100 * NM), work=[[2.0]], emission=True, mh_jumps=40,
                        max_chains=300, quad_panels=8, quad_order=4, seed=31, mh_serial=True)
    dio.add_particles(pos)
    eng.do_emission(1)
    c32 = dio.counters()
    assert c32["emitted_step"] > 0 and c32["MH_std"] != 0.0125
    eng.close()


def test_ring_emitter_fp64_matches_oracle(rg, orc):
    """Ring emitter (EMIT_RING): supply integral over (angle, radius) with the
    2 pi w r area factor (fe_v2:701-707) and the serial ring sampler
    (Metropolis_Hastings_ring_J :1521-1685, log r Jacobian, off-ring
    proposals rejected): the FP64 GPU form matches the oracle electron for
    electron."""
    rng = np.random.default_rng(41)
    d, V, n0 = 500 * NM, 1.0e3, 100
    r_out, w = 60 * NM, 20 * NM
    pos = np.column_stack([rng.uniform(-70 * NM, 70 * NM, n0), rng.uniform(-70 * NM, 70 * NM, n0),
                           rng.uniform(2 * NM, 490 * NM, n0)])
    eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=2, particle_capacity=8192, chain_capacity=4096)
    dio = eng.add_diode(V_s=V, gap=d, capacity=4096, emitter_pos=(-r_out, -r_out),
                        emitter_dim=(r_out, r_out), work=[[1.8]], emission=True, mh_jumps=40,
                        max_chains=300, quad_panels=8, quad_order=4, seed=41, emitter_type=4,
                        emitter_thickness=w)
    dio.add_particles(pos)
    o = orc.OracleDiode(cap=4096, V_s=V, d=d)
    o.set_planar_emitter(-r_out, -r_out, r_out, r_out, [[1.8]])
    o.set_ring(r_out, w)
    o.set_emission(True, seed=41, mh_jumps=40, max_chains=300, quad_panels=8, quad_order=4)
    for p in pos:
        o.add(p)
    for step in (1, 2):
        eng.do_emission(step)
        o.emission(step)
        c = dio.counters()
        assert c["N_sup"] == pytest.approx(o.s.N_sup, rel=1e-12)
        assert c["emitted_step"] == o.s.emitted_step
        assert c["MH_std"] == pytest.approx(o.s.MH_std, rel=1e-12)
        p = dio.particles()
        assert dio.n == o.n
        np.testing.assert_allclose(p["pos"], o.arr("pos")[:dio.n], rtol=0, atol=1e-12 * 100 * NM)
    new = dio.particles()["pos"][n0:]
    assert len(new) > 0
    r = np.hypot(new[:, 0], new[:, 1])
    assert np.all(r >= r_out - w - 1e-15) and np.all(r <= r_out + 1e-15)   # emitted on the ring
    eng.close()


def _tts_pair(rg, orc, geometry, T, n=300, nic=1, seed=21):
    """A diode under the two-time-step integrator on the GPU and in the
    oracle: electrons with every fourth particle an ion (the first one too,
    so electron-ion pairs take both index orders)."""
    rng = np.random.default_rng(seed)
    tip = (900 * NM, 100 * NM, 100 * NM)
    if geometry == "tip":
        pos = np.column_stack([rng.uniform(-300 * NM, 300 * NM, n), rng.uniform(-300 * NM, 300 * NM, n),
                               rng.uniform(105 * NM, 990 * NM, n)])
    else:
        pos = uniform_particles(rng, n)
    vel = rng.normal(0.0, 2e4, (n, 3))
    sp = np.where(np.arange(n) % 4 == 0, 2, 1)
    eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=2, particle_capacity=4096)
    kw = dict(V_s=2e3, capacity=1024, image_charge=True, atom_time_interval=T)
    if geometry == "tip":
        dio = eng.add_diode(geometry=rg.GEOM_TIP, tip_dim=tip, **kw)
        o = orc.OracleDiode(orc.TIP, cap=1024, V_s=2e3, d=1000 * NM, image_charge=True)
        o.set_tip(*tip, 4.7)
    else:
        dio = eng.add_diode(gap=1000 * NM, N_ic_max=nic, **kw)
        o = orc.OracleDiode(cap=1024, V_s=2e3, d=1000 * NM, image_charge=True, N_ic_max=nic)
    dio.add_particles(pos, vel=vel, species=sp)
    for p, v, s in zip(pos, vel, sp):
        o.add(p, vel=v, species=int(s))
    o.set_tts(T)
    return eng, dio, o, sp


@pytest.mark.parametrize("geometry", ["planar", "tip"])
def test_two_time_step_fp64_matches_oracle(rg, orc, geometry):
    """atom_time_interval = 3 (Update_Species_Position / _Velocity,
    Update_Elec_Acceleration / Update_Ion_Acceleration): electrons every
    step, ions on steps 3 and 6 with the step 3 dt, ion accelerations
    gathering electron forces in between; trajectories, accelerations and
    both Ramo currents agree with the oracle at every step."""
    eng, dio, o, sp = _tts_pair(rg, orc, geometry, 3)
    ion = sp == 2
    for step in range(1, 8):
        eng.update_position(step)
        o.verlet(step)
        p = dio.particles()
        assert np.max(np.abs(p["pos"] - o.arr("pos"))) < 1e-9 * NM, step
        assert nrel(p["vel"], o.arr("vel")) < 1e-11, step
        assert nrel(p["acc"], o.arr("acc")) < 1e-11, step
        c = dio.counters()
        assert c["ramo_current"] == pytest.approx(o.s.ramo_current, rel=1e-11)
        assert c["ramo_current_ion"] == pytest.approx(o.s.ramo_current_ion, rel=1e-11, abs=1e-30)
        assert (c["ramo_current_ion"] != 0.0) == (step % 3 == 0), step
    # the ions moved on steps 3 and 6 only
    eng.close()


def test_two_time_step_interval_one_equals_standard(rg, orc):
    """Test_TTS_Equivalence (src/mod_tests.F90:1455-1545) on the GPU: with
    atom_time_interval = 1 and the ions after the electrons, a two-time-step
    diode and a standard diode of the same engine step bit for bit alike; the
    plain acceleration pass (rd_accel) ignores the interval."""
    rng = np.random.default_rng(8)
    n = 257
    pos = uniform_particles(rng, n)
    vel = rng.normal(0.0, 2e4, (n, 3))
    sp = np.where(np.arange(n) >= n - 40, 2, 1)
    eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=4, particle_capacity=4096)
    a = eng.add_diode(V_s=2e3, gap=1000 * NM, capacity=1024, N_ic_max=2)
    b = eng.add_diode(V_s=2e3, gap=1000 * NM, capacity=1024, N_ic_max=2, atom_time_interval=1)
    for dio in (a, b):
        dio.add_particles(pos, vel=vel, species=sp)
    o = orc.OracleDiode(cap=1024, V_s=2e3, d=1000 * NM, image_charge=True, N_ic_max=2)
    for p, v, s in zip(pos, vel, sp):
        o.add(p, vel=v, species=int(s))
    assert nrel(b.calculate_acceleration_particles(), o.accel("gather", True)) <= TOL64
    for step in range(1, 4):
        eng.update_position(step)
    pa, pb = a.particles(), b.particles()
    for k in ("pos", "vel", "acc"):
        assert np.array_equal(pa[k], pb[k]), k
    ca, cb = a.counters(), b.counters()
    assert ca["ramo_current"] == cb["ramo_current"]
    assert ca["ramo_current_ion"] == cb["ramo_current_ion"] != 0.0
    eng.close()


def test_two_time_step_full_steps_with_emission_fp64(rg, orc):
    """Main-loop iterations (emission, Beeman, forces, removal and
    compaction) of a two-time-step diode with ions among the electrons
    (atom_time_interval = 2): the FP64 GPU form follows the oracle step for
    step, including the electrons emitted into the mix."""
    eng0, _, o = _emission_pair(rg, orc, rg.PREC_FP64, seed=31, n0=0)   # the oracle side only
    eng0.close()
    eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=2, particle_capacity=8192, chain_capacity=4096)
    dio = eng.add_diode(V_s=1.0e3, gap=500 * NM, capacity=4096, emitter_pos=(-50 * NM, -50 * NM),
                        emitter_dim=(100 * NM, 100 * NM), work=[[2.0]], emission=True, mh_jumps=40,
                        max_chains=300, quad_panels=8, quad_order=4, seed=31, atom_time_interval=2)
    rng = np.random.default_rng(31)
    n0 = 120
    pos = np.column_stack([rng.uniform(-60 * NM, 60 * NM, n0), rng.uniform(-60 * NM, 60 * NM, n0),
                           rng.uniform(2 * NM, 490 * NM, n0)])
    sp = np.where(np.arange(n0) % 3 == 0, 2, 1)
    dio.add_particles(pos, species=sp)
    for p, s in zip(pos, sp):
        o.add(p, species=int(s))
    o.set_tts(2)
    for step in range(1, 6):
        eng.step(step)
        o.step(step)
        c = dio.counters()
        assert dio.n == o.n, step
        assert c["emitted_step"] == o.s.emitted_step, step
        assert c["ramo_current_ion"] == pytest.approx(o.s.ramo_current_ion, rel=1e-9, abs=1e-30)
    p = dio.particles()
    assert np.max(np.abs(p["pos"] - o.arr("pos"))) < 1e-9 * NM
    assert nrel(p["vel"] + 1e-3, o.arr("vel") + 1e-3) < 1e-8
    assert c["emitted_total"] == o.s.emitted_total > 0
    _check_average_velocities(c, o)   # step 5: the ions did not move, their mean is 0
    assert c["n_ion_vel"] > 0 and c["avg_ion_vel"] == (0.0, 0.0, 0.0)
    assert all(v == 0 for v in eng.validate().values())
    eng.close()


def test_tip_image_term_survives_fp32(rg):
    """The tip sphere-image term carries the reference's extra factor
    K = q0 / (4 pi eps0) ~ 1.4e-9 (acc_tip_ic_force.inc), far below the FP32
    resolution of the direct sum.  The FP32 tiles keep it in separate sums
    scaled in FP64, so the image part of the acceleration and of the field
    (image charge on minus off) matches the FP64 form's."""
    rng = np.random.default_rng(5)
    tip = (900 * NM, 100 * NM, 100 * NM)
    n = 257
    pos = np.column_stack([rng.uniform(-300 * NM, 300 * NM, n), rng.uniform(-300 * NM, 300 * NM, n),
                           rng.uniform(105 * NM, 990 * NM, n)])
    pts = np.array([[0.0, 0.0, 102.0], [30.0, -10.0, 130.0], [-50.0, 40.0, 300.0]]) * NM
    diff = {}
    for prec in (rg.PREC_FP64, rg.PREC_FP32C):
        eng = rg.Engine(precision=prec, max_diodes=2, particle_capacity=4096)
        on = eng.add_diode(geometry=rg.GEOM_TIP, V_s=2e3, capacity=1024, tip_dim=tip, image_charge=True)
        off = eng.add_diode(geometry=rg.GEOM_TIP, V_s=2e3, capacity=1024, tip_dim=tip, image_charge=False)
        on.add_particles(pos)
        off.add_particles(pos)
        a_on = on.calculate_acceleration_particles()
        a_off = off.particles()["acc"]   # the same pass filled both diodes
        f_on = on.calc_field_at_batch(pts)
        diff[prec] = (a_on - a_off, f_on - off.calc_field_at_batch(pts), f_on)
        eng.close()
    da64, df64, f64 = diff[rg.PREC_FP64]
    da32, df32, _ = diff[rg.PREC_FP32C]
    assert np.all(np.linalg.norm(da64, axis=1) > 0)
    assert nrel(da32, da64) < 1e-3
    # the fields include the GV/m vacuum field: both forms round the total at its ulp, which is
    # ~1e-3 of the image part here, and the FP64 form adds each image term into the running sum
    tol = 1e-3 * np.abs(df64) + 16 * np.finfo(float).eps * np.linalg.norm(f64, axis=1)[:, None]
    assert np.all(np.abs(df32 - df64) <= tol), (df32, df64)


@pytest.mark.parametrize("nic", [0, 3])
def test_fp32c_mixed_electron_and_ion_tiles(rg, orc, nic):
    """Ions only among the first 64 particles: their j-tile takes the general
    FP32 tile, the all-electron tiles the variant without charge multiplies;
    accelerations and fields stay within the FP32 tolerance of the FP64 oracle."""
    rng = np.random.default_rng(12)
    n = 700
    pos = uniform_particles(rng, n)
    sp = np.where((np.arange(n) < 64) & (np.arange(n) % 4 == 1), 2, 1)
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=2, particle_capacity=4096)
    dio = eng.add_diode(V_s=2e3, gap=1000 * NM, capacity=1024, image_charge=True, N_ic_max=nic)
    dio.add_particles(pos, species=sp)
    o = orc.OracleDiode(cap=1024, V_s=2e3, d=1000 * NM, image_charge=True, N_ic_max=nic)
    for p, s in zip(pos, sp):
        o.add(p, species=int(s))
    assert nrel(dio.calculate_acceleration_particles(), o.accel("gather", True)) <= TOL32
    pts = np.vstack([uniform_particles(rng, 50),
                     np.column_stack([rng.uniform(-500 * NM, 500 * NM, 50), rng.uniform(-500 * NM, 500 * NM, 50),
                                      np.zeros(50)])])
    assert nrel(dio.calc_field_at_batch(pts), o.field_at(pts)) <= TOL32
    eng.close()


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-5)])
def test_emission_without_image_charges_and_lateral_field(rg, orc, prec, tol):
    """A planar diode without image charges: its supply points carry all three
    field components, so field.dt's mean field F_avg (Do_Surface_Integration_FE,
    src/mod_field_emission_v2.F90:644-651) has lateral parts; with image charges
    they cancel at the cathode.  Against the oracle: N_sup, the chain count
    and F_avg (relative to |F_avg_z|); in FP64 also the emitted electrons."""
    rng = np.random.default_rng(31)
    d, V, n0 = 500 * NM, 1.0e3, 150
    pos = np.column_stack([rng.uniform(-60 * NM, 60 * NM, n0), rng.uniform(-60 * NM, 60 * NM, n0),
                           rng.uniform(2 * NM, 490 * NM, n0)])
    eng = rg.Engine(precision=prec, max_diodes=2, particle_capacity=8192, chain_capacity=4096)
    dio = eng.add_diode(V_s=V, gap=d, capacity=4096, image_charge=False, emitter_pos=(-50 * NM, -50 * NM),
                        emitter_dim=(100 * NM, 100 * NM), work=[[2.0]], emission=True, mh_jumps=40,
                        max_chains=300, quad_panels=8, quad_order=4, seed=31)
    dio.add_particles(pos)
    o = orc.OracleDiode(cap=4096, V_s=V, d=d, image_charge=False)
    o.set_planar_emitter(-50 * NM, -50 * NM, 100 * NM, 100 * NM, [[2.0]])
    o.set_emission(True, seed=31, mh_jumps=40, max_chains=300, quad_panels=8, quad_order=4)
    for p in pos:
        o.add(p)
    eng.do_emission(1)
    o.emission(1)
    c = dio.counters()
    assert c["N_sup"] == pytest.approx(o.s.N_sup, rel=tol)
    ref = np.array([o.s.F_avg_x, o.s.F_avg_y, o.s.F_avg_z])
    assert abs(ref[0]) + abs(ref[1]) > 1e-6 * abs(ref[2])          # the lateral mean is there
    assert np.max(np.abs(np.array(c["F_avg"]) - ref)) <= tol * abs(ref[2]), (c["F_avg"], ref)
    if prec == 0:
        assert c["chains"] == o.s.last_chains and c["emitted_step"] == o.s.emitted_step
        np.testing.assert_array_equal(dio.particles()["id"], o.iarr("id"))
    eng.close()
