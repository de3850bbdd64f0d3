"""Engine lifetime on the GPU: creating, stepping and destroying engines
returns their device memory (pools, scratch, graphs, streams), and a
destroyed engine's diodes leave no state behind for the next engine."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NM = 1e-9


def _free_bytes():
    torch = pytest.importorskip("torch")
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def _cycle(rg, seed):
    rng = np.random.default_rng(seed)
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=4, particle_capacity=1 << 16,
                    chain_capacity=1 << 14, quad_capacity=1 << 14)
    for k in range(3):
        d = eng.add_diode(V_s=2.0e3, gap=800 * NM, capacity=4096, emitter_pos=(-100 * NM, -100 * NM),
                          emitter_dim=(200 * NM, 200 * NM), work=[[2.5]], emission=True, mh_jumps=20,
                          max_chains=256, seed=seed + k)
        d.add_particles(np.column_stack([rng.uniform(-100 * NM, 100 * NM, 500), rng.uniform(-100 * NM, 100 * NM, 500),
                                         rng.uniform(2 * NM, 790 * NM, 500)]), step=0)
    eng.run(1, 3)                 # graph capture, both MH streams
    counters = [d.counters() for d in eng.diodes.values()]
    eng.close()
    return counters


def test_engines_release_device_memory(rg):
    first = _cycle(rg, 1)         # warm-up: context, module load, allocator caches
    base = _free_bytes()
    for k in range(8):
        again = _cycle(rg, 1)
        assert again == first     # same inputs, same results, engine after engine
    leaked = base - _free_bytes()
    assert leaked < 64 * 1024 * 1024, "%.1f MiB not returned" % (leaked / 2 ** 20)


def test_validate_reports_clean_and_corrupted_state(rg):
    """rd_validate: zero violations after steps; a non-finite position put in
    with rd_set_particles (no step runs on it) is counted, and the count
    returns to zero once the position is repaired."""
    rng = np.random.default_rng(3)
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=2, particle_capacity=8192, chain_capacity=2048,
                    quad_capacity=4096)
    d = eng.add_diode(V_s=2.0e3, gap=800 * NM, capacity=4096, emitter_pos=(-100 * NM, -100 * NM),
                      emitter_dim=(200 * NM, 200 * NM), work=[[2.5]], emission=True, mh_jumps=20,
                      max_chains=256, seed=7)
    d.add_particles(np.column_stack([rng.uniform(-100 * NM, 100 * NM, 300), rng.uniform(-100 * NM, 100 * NM, 300),
                                     rng.uniform(2 * NM, 790 * NM, 300)]), step=0)
    eng.run(1, 5)
    assert all(v == 0 for v in eng.validate().values())
    pos = d.particles()["pos"]
    bad = pos.copy()
    bad[7, 2] = np.nan
    d.set_particles(pos=bad)
    v = eng.validate()
    assert v["non_finite_state"] == 1 and sum(v.values()) == 1
    d.set_particles(pos=pos)
    assert all(v == 0 for v in eng.validate().values())
    eng.close()


def test_time_verlet_times_both_passes_and_keeps_state_valid(rg):
    """rd_time_verlet: positive device times for the position and the velocity
    pass; the passes it runs leave a state that rd_validate finds clean, with
    the Ramo / mean-velocity sums of the last velocity pass in the counters."""
    rng = np.random.default_rng(5)
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=3, particle_capacity=3 * 4096, chain_capacity=1024,
                    quad_capacity=1024)
    ds = []
    for k, n in enumerate((1000, 129, 4000)):   # ragged: partial 128-electron items
        d = eng.add_diode(V_s=2.0e3, gap=1000 * NM, capacity=4096, image_charge=True, N_ic_max=0)
        d.add_particles(np.column_stack([rng.uniform(-500 * NM, 500 * NM, n), rng.uniform(-500 * NM, 500 * NM, n),
                                         rng.uniform(450 * NM, 550 * NM, n)]), step=0)
        d.set_particles(vel=rng.normal(0.0, 1.0e5, (n, 3)))
        ds.append((d, n))
    pos_ms, vel_ms = eng.time_verlet(reps=3)
    assert pos_ms > 0.0 and vel_ms > 0.0
    assert all(v == 0 for v in eng.validate().values())
    for d, n in ds:
        c = d.counters()
        assert c["n_elec_vel"] == n and c["n_ion_vel"] == 0
        v = d.particles()["vel"]
        np.testing.assert_allclose(c["avg_elec_vel"], v.mean(axis=0), rtol=1e-12, atol=1e-9)
    eng.close()
