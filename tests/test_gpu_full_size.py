"""Full-size checks through properties that do not need the oracle: the
force microbench sizes (262144 electrons), the 128-diode serving mix, and the
edge cases of the step (empty diodes, a full pool, every electron absorbed)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NM = 1e-9


def _box(n, seed):
    rng = np.random.default_rng(seed)
    return np.column_stack([rng.uniform(-500 * NM, 500 * NM, n), rng.uniform(-500 * NM, 500 * NM, n),
                            rng.uniform(1 * NM, 999 * NM, n)])


def _acc(rg, prec, pos, **kw):
    eng = rg.Engine(precision=prec, max_diodes=1, particle_capacity=len(pos) + 1024, chain_capacity=1024,
                    quad_capacity=1024)
    d = eng.add_diode(gap=1000 * NM, capacity=len(pos), **kw)
    d.add_particles(pos)
    a = d.calculate_acceleration_particles()
    eng.close()
    return a


def test_newton_third_law_at_262144(rg):
    """No images and no applied field: the pair forces cancel, sum m a = 0,
    to the FP32-compensated form's rounding at N = 262144."""
    pos = _box(262144, 3)
    a = _acc(rg, rg.PREC_FP32C, pos, V_s=0.0, image_charge=False)
    total = np.abs(a.sum(axis=0))
    scale = np.abs(a).sum(axis=0)
    assert np.all(total <= 1e-6 * scale), (total, scale)


def test_fp32c_force_error_at_262144(rg):
    """The force microbench at its largest size: max norm-relative error of the
    FP32-compensated accelerations against the FP64 form <= 1e-5."""
    pos = _box(262144, 3)
    a32 = _acc(rg, rg.PREC_FP32C, pos, V_s=2.0e3, image_charge=True, N_ic_max=0)
    a64 = _acc(rg, rg.PREC_FP64, pos, V_s=2.0e3, image_charge=True, N_ic_max=0)
    err = np.linalg.norm(a32 - a64, axis=1) / np.linalg.norm(a64, axis=1)
    assert err.max() <= 1e-5 and np.sqrt(np.mean(err ** 2)) <= 1e-7, (err.max(), np.sqrt(np.mean(err ** 2)))


def test_cathode_field_at_262144(rg):
    """Field at the 64 x 64 cathode midpoints from 262144 electrons: the
    FP32-compensated form within 1e-6 of the vacuum field's size of FP64."""
    pos = _box(262144, 3)
    c = (np.arange(64) + 0.5) / 64 * 1000 * NM - 500 * NM
    gx, gy = np.meshgrid(c, c, indexing="ij")
    grid = np.column_stack([gx.ravel(), gy.ravel(), np.zeros(4096)])
    out = {}
    for prec in (rg.PREC_FP32C, rg.PREC_FP64):
        eng = rg.Engine(precision=prec, max_diodes=1, particle_capacity=263168, chain_capacity=1024,
                        quad_capacity=1024)
        d = eng.add_diode(V_s=2.0e3, gap=1000 * NM, capacity=262144, image_charge=True, N_ic_max=0)
        d.add_particles(pos)
        out[prec] = d.calc_field_at_batch(grid)
        eng.close()
    e_vac = 2.0e3 / (1000 * NM)
    dev = np.linalg.norm(out[rg.PREC_FP32C] - out[rg.PREC_FP64], axis=1) / e_vac
    assert dev.max() <= 1e-6, dev.max()


def test_largest_diode_alone_equals_128_mix(rg):
    """The 128-diode serving mix at full size (the first 128 requests of the
    stream, 0.79 M electrons): one step of its largest diode is bit-identical
    alone and in the mix."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    st = bench.RequestStream(bench.SEED)
    reqs = [st.next() for _ in range(128)]
    big = max(range(128), key=lambda k: reqs[k]["capacity"])
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=128, particle_capacity=128 * 32768 + 4096,
                    chain_capacity=128 * 32768 + 4096, quad_capacity=128 * bench.MAX_SUPPLY_POINTS + 4096)
    ds = []
    for r in reqs:
        d = eng.add_diode(**bench.diode_kwargs(r))
        d.add_particles(bench.prefill(r), step=0)
        ds.append(d)
    eng.run(1, 1)
    mixed = ds[big].particles()
    assert all(v == 0 for v in eng.validate().values())   # 128 diodes, 0.79 M electrons
    eng.close()
    r = reqs[big]
    one = rg.Engine(precision=rg.PREC_FP32C, max_diodes=1, particle_capacity=r["capacity"] + 64,
                    chain_capacity=r["capacity"] + 64, quad_capacity=bench.MAX_SUPPLY_POINTS + 64)
    d = one.add_diode(**bench.diode_kwargs(r))
    d.add_particles(bench.prefill(r), step=0)
    one.run(1, 1)
    alone = d.particles()
    one.close()
    for key in mixed:
        np.testing.assert_array_equal(mixed[key], alone[key], err_msg=key)


def test_edge_cases_empty_full_and_absorb_all(rg):
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=3, particle_capacity=3 * 1024, chain_capacity=3 * 512,
                    quad_capacity=3 * 1024)
    empty = eng.add_diode(V_s=1.0e3, gap=500 * NM, capacity=512)                       # no particles, no emission
    full = eng.add_diode(V_s=1.0e3, gap=500 * NM, capacity=5, emitter_pos=(-50 * NM, -50 * NM),
                         emitter_dim=(100 * NM, 100 * NM), work=[[1.0]], emission=True, mh_jumps=20,
                         max_chains=50, quad_panels=4, quad_order=4, seed=3)            # emits past its capacity
    doomed = eng.add_diode(V_s=1.0e3, gap=500 * NM, capacity=512)
    rng = np.random.default_rng(4)
    n = 300
    doomed.add_particles(np.column_stack([rng.uniform(-50 * NM, 50 * NM, n), rng.uniform(-50 * NM, 50 * NM, n),
                                          np.full(n, 499.9 * NM)]),
                         vel=np.column_stack([np.zeros(n), np.zeros(n), np.full(n, 1e8)]))   # all cross the anode
    for step in (1, 2):
        eng.step(step)
    ce, cf, cd = empty.counters(), full.counters(), doomed.counters()
    assert ce["n"] == 0 and ce["emitted_total"] == 0
    assert cf["n"] == 5 and cf["dropped_total"] > 0 and cf["emitted_total"] == 5   # Add_Particle's drop rule
    assert cd["n"] == 0 and cd["absorbed_top_total"] == n
    eng.close()
