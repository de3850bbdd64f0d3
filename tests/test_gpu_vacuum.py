"""k_mh_vacuum: the batched MH sampling of a planar diode with no particle in
flight -- the chains' start and all their jumps -- runs in one launch (one
thread-block cluster per diode).  It must give exactly what the tiled jump
kernels give.  A diode holding one atom (charge 0: every pair sum adds exact
zeros, so its field is the vacuum field bit for bit) takes the tiled kernels;
the same diode without it takes the vacuum kernel.  One step of each must
agree in every emission counter and in every emitted electron's position, in
both precisions.  (The FP64 form of the empty one-diode deck is also checked
against the oracle chain for chain in test_gpu_config_parity.py.)

A uniform work function (one cell, or cells that all hold the same value)
makes every target equal, so every proposal is taken and the kernel walks the
chains without a barrier per jump; a checkerboard of different values takes
the jump-by-jump path with the cluster-wide acceptance counts.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NM = 1e-9


CHECKER = [[2.0, 2.3], [2.6, 2.1]]
UNIFORM = [[2.2]]
UNIFORM4 = [[2.2, 2.2], [2.2, 2.2]]


def _step(rg, prec, atom, jumps, work):
    eng = rg.Engine(precision=prec, max_diodes=2, particle_capacity=8192, chain_capacity=8192,
                    quad_capacity=65536, event_capacity=1 << 15)
    d = eng.add_diode(V_s=2.0e3, gap=1000 * NM, time_step=0.25e-15, capacity=8000,
                      emitter_pos=(-500 * NM, -500 * NM), emitter_dim=(1000 * NM, 1000 * NM),
                      work=work, emission=True, mh_jumps=jumps, seed=99)
    if atom:
        d.add_particles(np.array([[400 * NM, 400 * NM, 900 * NM]]), species=[rg.ATOM], step=0)
    eng.step(1)
    c = d.counters()
    ev, lost = eng.events_take()
    assert lost == 0
    sites = np.array(sorted(e["pos"][:2] for e in ev if e["kind"] == rg.EVENT_EMIT))
    eng.close()
    return c, sites


@pytest.mark.parametrize("prec,jumps,work", [(1, 200, CHECKER), (1, 37, CHECKER), (0, 60, CHECKER),
                                             (1, 200, UNIFORM), (1, 100, UNIFORM4), (0, 60, UNIFORM)])
def test_vacuum_kernel_equals_tiled_kernels(rg, prec, jumps, work):
    empty, s_empty = _step(rg, prec, False, jumps, work)
    atom, s_atom = _step(rg, prec, True, jumps, work)
    assert 1000 < empty["chains"] <= 8192 and empty["emitted_step"] > 50
    for key in ("N_sup", "chains", "chains_failed", "MH_std", "a_rate", "df_avg", "emitted_step", "residual"):
        assert empty[key] == atom[key], key
    assert empty["F_avg"] == atom["F_avg"]
    np.testing.assert_array_equal(s_empty, s_atom)


def _engine_of_two(rg, prec, atom, jumps, work, steps):
    eng = rg.Engine(precision=prec, max_diodes=2, particle_capacity=20000, chain_capacity=20000,
                    quad_capacity=131072, event_capacity=1 << 16)
    ds = []
    for seed in (5, 6):
        d = eng.add_diode(V_s=2.0e3, gap=1000 * NM, time_step=0.25e-15, capacity=9000,
                          emitter_pos=(-500 * NM, -500 * NM), emitter_dim=(1000 * NM, 1000 * NM),
                          work=work, emission=True, mh_jumps=jumps, seed=seed)
        if atom:
            d.add_particles(np.array([[400 * NM, 400 * NM, 900 * NM]]), species=[rg.ATOM], step=0)
        ds.append(d)
    out = []
    for s in range(1, steps + 1):
        eng.step(s)
        ev, lost = eng.events_take()
        assert lost == 0
        out.append([(d.counters(), sorted(tuple(e["pos"][:2]) for e in ev
                                          if e["kind"] == rg.EVENT_EMIT and e["diode"] == d.index)) for d in ds])
    eng.close()
    return out


@pytest.mark.parametrize("prec,work,steps", [(1, [[4.7]], 6), (0, [[4.7]], 3), (1, UNIFORM, 1)])
def test_vacuum_uniform_two_diodes_over_steps(rg, prec, work, steps):
    """Two vacuum-field diodes in one engine (the uniform kernel's second grid row),
    over several steps: at 4.7 eV nothing is emitted, so the diodes stay empty and
    MH_std climbs to its clamp, where the schedule takes its fixed point; at 2.2 eV
    one step emits.  Every counter and emission site equals the tiled kernels'."""
    empty = _engine_of_two(rg, prec, False, 100, work, steps)
    atom = _engine_of_two(rg, prec, True, 100, work, steps)
    for se, sa in zip(empty, atom):
        for (ce, ee), (ca, ea) in zip(se, sa):
            for key in ("N_sup", "chains", "chains_failed", "MH_std", "a_rate", "df_avg", "emitted_step"):
                assert ce[key] == ca[key], key
            assert ee == ea
    assert empty[-1][0][0]["MH_std"] != empty[0][0][0]["MH_std"] or steps == 1


def _serial_pair(rg, prec, atom, jumps, work, steps):
    eng = rg.Engine(precision=prec, max_diodes=2, particle_capacity=20000, chain_capacity=20000,
                    quad_capacity=131072, event_capacity=1 << 16)
    ds = []
    for seed in (11, 12):
        d = eng.add_diode(V_s=2.0e3, gap=1000 * NM, time_step=0.25e-15, capacity=9000,
                          emitter_pos=(-500 * NM, -500 * NM), emitter_dim=(1000 * NM, 1000 * NM),
                          work=work, emission=True, mh_jumps=jumps, seed=seed, mh_serial=True)
        if atom:
            d.add_particles(np.array([[400 * NM, 400 * NM, 900 * NM]]), species=[rg.ATOM], step=0)
        ds.append(d)
    out = []
    for s in range(1, steps + 1):
        eng.step(s)
        ev, lost = eng.events_take()
        assert lost == 0
        out.append([(d.counters(), sorted(tuple(e["pos"][:2]) for e in ev
                                          if e["kind"] == rg.EVENT_EMIT and e["diode"] == d.index)) for d in ds])
    eng.close()
    return out


@pytest.mark.parametrize("prec,work,steps", [(1, [[4.7]], 3), (0, [[4.7]], 2), (1, UNIFORM4, 1), (0, UNIFORM, 1)])
def test_serial_sampler_vacuum_pass_equals_serial_kernel(rg, prec, work, steps):
    """The serial sampler (mh_batch = .false.) on empty diodes with a uniform work
    function: the speculative parallel pass (k_mh_serial_vacuum) against the serial
    kernel itself, which a zero-charge atom forces (its field is the vacuum field bit
    for bit).  At 4.7 eV no chain emits and the parallel pass gives the step's
    results: every counter equals the serial kernel's bit for bit, the
    escape-probability mean included.  At 2.2 eV chains emit, the pass writes
    nothing and the serial kernel samples the diode: every counter and emission
    site equal."""
    fast = _serial_pair(rg, prec, False, 100, work, steps)
    slow = _serial_pair(rg, prec, True, 100, work, steps)
    for sf, ss in zip(fast, slow):
        for (cf, ef), (cs, es) in zip(sf, ss):
            for key in ("N_sup", "chains", "chains_failed", "MH_std", "a_rate", "emitted_step", "dropped_step"):
                assert cf[key] == cs[key], key
            assert cf["df_avg"] == cs["df_avg"]
            assert ef == es
    if work == [[4.7]]:
        assert all(c["emitted_step"] == 0 for s in fast for c, _ in s)
    else:
        assert sum(c["emitted_step"] for s in fast for c, _ in s) > 0
