"""Serving (continuous batching) through the C ABI: requests admitted as slots
and pool memory free up, advanced together, retired on completion; each
result is bit-identical to the same diode simulated alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NM = 1e-9


def make_requests(n=6, seed=3):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        cap = int(rng.integers(200, 900))
        side = float(rng.uniform(100, 300)) * NM
        gap = float(rng.uniform(300, 800)) * NM
        kw = dict(V_s=float(rng.uniform(800, 2500)), gap=gap, capacity=cap,
                  emitter_pos=(-side / 2, -side / 2), emitter_dim=(side, side),
                  work=[[float(rng.uniform(2.0, 3.0))]], emission=True, mh_jumps=30,
                  max_chains=256, quad_panels=4, quad_order=4, seed=int(rng.integers(1, 1 << 40)))
        n0 = cap // 2
        pos = np.column_stack([rng.uniform(-side / 2, side / 2, n0), rng.uniform(-side / 2, side / 2, n0),
                               rng.uniform(1 * NM, gap - 1 * NM, n0)])
        out.append((int(rng.integers(4, 12)), pos, kw))
    return out


def alone(rg, prec, steps, pos, kw):
    eng = rg.Engine(precision=prec, max_diodes=1, particle_capacity=4096, chain_capacity=1024,
                    quad_capacity=1024)
    d = eng.add_diode(**kw)
    d.add_particles(pos, step=0)
    eng.run(1, steps)
    res = d.counters(), d.particles()
    eng.close()
    return res


@pytest.mark.parametrize("prec", [0, 1])
def test_served_equals_alone(rg, prec):
    reqs = make_requests()
    # pool for 3 diodes at a time: later requests wait for capacity
    eng = rg.Engine(precision=prec, max_diodes=3, particle_capacity=3 * 1024, chain_capacity=3 * 256,
                    quad_capacity=3 * 1024)
    ids = [eng.submit(steps, pos=pos, **kw) for steps, pos, kw in reqs]
    assert eng.poll(ids[-1])["state"] == rg.REQ_QUEUED
    finals = {}
    for _ in range(200):
        st = eng.serve(1)
        assert st["running"] <= 3
        for rid in ids:
            s = eng.poll(rid)
            if s["state"] == rg.REQ_DONE and rid not in finals:
                finals[rid] = s
        if len(finals) == len(ids):
            break
    assert len(finals) == len(ids)
    for rid, (steps, pos, kw) in zip(ids, reqs):
        c_alone, _ = alone(rg, prec, steps, pos, kw)
        c = finals[rid]["counters"]
        assert c["steps_done"] == steps
        for key in ("n", "emitted_total", "absorbed_top_total", "absorbed_bot_total",
                    "dropped_total", "electron_steps", "chains"):
            assert c[key] == c_alone[key], key
        for key in ("ramo_current", "N_sup", "MH_std", "residual"):
            assert c[key] == c_alone[key], key
        assert finals[rid]["done_s"] >= finals[rid]["admit_s"] >= finals[rid]["submit_s"]
    assert all(v == 0 for v in eng.validate().values())
    eng.close()


def test_cancel_and_poll(rg):
    reqs = make_requests(3, seed=9)
    eng = rg.Engine(precision=1, max_diodes=1, particle_capacity=2048, chain_capacity=512,
                    quad_capacity=1024)
    ids = [eng.submit(steps, pos=pos, **kw) for steps, pos, kw in reqs]
    eng.serve(1)
    assert eng.poll(ids[0])["state"] == rg.REQ_RUNNING
    assert eng.poll(ids[1])["state"] == rg.REQ_QUEUED
    eng.cancel(ids[1])
    assert eng.poll(ids[1])["state"] == rg.REQ_CANCELLED
    eng.cancel(ids[0])
    assert eng.poll(ids[0])["state"] == rg.REQ_CANCELLED
    st = eng.serve(1)     # the third request takes the freed slot
    assert eng.poll(ids[2])["state"] == rg.REQ_RUNNING and st["admitted"] == 1
    with pytest.raises(rg.RumdeedError):
        eng.poll(12345)
    eng.close()


def test_profile_step_reports_phases(rg):
    steps, pos, kw = make_requests(1, seed=4)[0]
    eng = rg.Engine(precision=1, max_diodes=2, particle_capacity=4096, chain_capacity=1024,
                    quad_capacity=2048)
    d = eng.add_diode(**kw)
    d.add_particles(pos, step=0)
    p = eng.profile_step(1)
    assert p["total_ms"] > 0 and p["mh_jump_launches"] == 30
    assert p["mh_pair_evals"] > 0 and p["force_pairs"] > 0
    parts = sum(p[k] for k in ("supply_ms", "mh_init_ms", "mh_jumps_ms", "emit_ms", "position_ms",
                               "force_ms", "velocity_ms", "compact_ms"))
    assert parts <= p["total_ms"] * 1.01 + 1e-3
    eng.close()


def test_served_two_time_step_diode_equals_alone(rg):
    """A two-time-step diode (atom_time_interval = 3, its force pass on the
    k_force_tts plan) served among standard diodes ends bit-identical to the
    same diode simulated alone, and so do its neighbours."""
    reqs = make_requests(n=4, seed=9)
    reqs[1][2]["atom_time_interval"] = 3
    eng = rg.Engine(precision=1, max_diodes=4, particle_capacity=4 * 1024, chain_capacity=4 * 256,
                    quad_capacity=4 * 1024)
    ids = [eng.submit(steps, pos=pos, **kw) for steps, pos, kw in reqs]
    finals = {}
    for _ in range(100):
        eng.serve(1)
        for rid in ids:
            s = eng.poll(rid)
            if s["state"] == rg.REQ_DONE and rid not in finals:
                finals[rid] = s
        if len(finals) == len(ids):
            break
    assert len(finals) == len(ids)
    for rid, (steps, pos, kw) in zip(ids, reqs):
        c, _ = alone(rg, 1, steps, pos, kw)
        got = finals[rid]["counters"]
        for key in ("n", "emitted_total", "absorbed_top_total", "absorbed_bot_total", "electron_steps"):
            assert got[key] == c[key], (rid, key)
        assert got["ramo_current"] == c["ramo_current"]
    eng.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_checkpoint_resume_equals_continuous_run(rg, prec):
    """rd_diode_save after 4 steps, rd_diode_load into a fresh diode of another
    engine (among other diodes), 4 more steps: the same particles, counters
    and life-time histogram as the run that went on without stopping."""
    (steps, pos, kw), (_, pos2, kw2) = make_requests(n=2, seed=21)
    a = rg.Engine(precision=prec, max_diodes=2, particle_capacity=4096, chain_capacity=1024, quad_capacity=2048)
    da = a.add_diode(**kw)
    da.add_particles(pos, step=0)
    a.run(1, 4)
    state = da.save_state()
    a.run(5, 4)
    b = rg.Engine(precision=prec, max_diodes=3, particle_capacity=8192, chain_capacity=2048, quad_capacity=4096)
    other = b.add_diode(**kw2)
    other.add_particles(pos2, step=0)
    db = b.add_diode(**kw)
    db.load_state(state)
    b.run(5, 4)
    ca, cb = da.counters(), db.counters()
    for key in ("n", "emitted_total", "absorbed_top_total", "absorbed_bot_total", "dropped_total",
                "electron_steps", "steps_done", "chains", "ramo_current", "N_sup", "MH_std", "residual"):
        assert ca[key] == cb[key], key
    pa, pb = da.particles(), db.particles()
    for key in ("pos", "vel", "acc", "charge", "id", "section"):
        np.testing.assert_array_equal(pa[key], pb[key], err_msg=key)
    np.testing.assert_array_equal(da.life_time(), db.life_time())
    with pytest.raises(rg.RumdeedError):
        db.load_state(state[:100])   # truncated
    a.close()
    b.close()
