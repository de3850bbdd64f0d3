"""GPU against the oracle at the benchmark configurations' own sizes.

* Force/field microbench (N = 4096, 65536, 262144 electrons in a 1000 x 1000
  x 1000 nm box, 2 kV; N_ic_max 0, 7 and 8): the accelerations of 512 sampled
  particles and the field at 512 sampled points of the 64 x 64 cathode grid,
  each against the oracle's gather over all N particles (the rows of a gather
  are independent, so the sample checks the full-size system).  The FP64 form
  within 1e-12, the FP32-compensated form within 1e-5 (max norm-relative per
  particle; fields relative to max(|E|, V/d), since the space charge of
  262144 electrons cancels the vacuum field at the cathode to ~3e-5 of it).
  The FP64 form at N = 262144 with 29 or 33 image partners (~80 s per force
  evaluation on this GPU's FP64 pipe) is covered at N = 65536 instead.
* The one-diode deck (1 um gap, 2 kV, 1000 x 1000 nm emitter, 4.7 eV, MH
  with 200 and 100 jumps; and three steps of the populated 2.0 eV variant):
  the FP64 form emits the oracle's electrons chain for chain.
* The tip deck (h 500 nm, tip-anode gap 1000 nm, apex radius 10 and 50 nm,
  4.5 eV, a few thousand electrons in flight): two FP64 steps, chain for chain.

Each comparison prints its max and RMS error.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NM = 1e-9
TOL64, TOL32 = 1e-12, 1e-5
ROWS = 512


def _box(n, seed):
    rng = np.random.default_rng(seed)
    return np.column_stack([rng.uniform(-500 * NM, 500 * NM, n), rng.uniform(-500 * NM, 500 * NM, n),
                            rng.uniform(1 * NM, 999 * NM, n)])


def _grid(m=64):
    c = (np.arange(m) + 0.5) / m * 1000 * NM - 500 * NM
    gx, gy = np.meshgrid(c, c, indexing="ij")
    return np.column_stack([gx.ravel(), gy.ravel(), np.zeros(m * m)])


def _errs(got, ref, floor=0.0):
    e = np.linalg.norm(got - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), floor)
    return float(e.max()), float(np.sqrt(np.mean(e ** 2)))


_ORACLES = {}


def _oracle(orc, n, nic):
    """One oracle diode per (N, N_ic_max), positions seeded as the microbench's."""
    key = (n, nic)
    if key not in _ORACLES:
        _ORACLES.clear()   # keep one resident: the largest holds 262144 particles
        o = orc.OracleDiode(cap=n, V_s=2.0e3, d=1000 * NM, image_charge=True, N_ic_max=nic)
        o.add_many(_box(n, {4096: 1, 65536: 2, 262144: 3}[n]))
        _ORACLES[key] = o
    return _ORACLES[key]


def _gpu(rg, prec, n, nic):
    eng = rg.Engine(precision=prec, max_diodes=1, particle_capacity=n + 1024, chain_capacity=1024,
                    quad_capacity=1024)
    d = eng.add_diode(V_s=2.0e3, gap=1000 * NM, capacity=n, image_charge=True, N_ic_max=nic)
    d.add_particles(_box(n, {4096: 1, 65536: 2, 262144: 3}[n]))
    return eng, d


CASES = [(n, nic, prec) for n in (4096, 65536, 262144) for nic in (0, 7, 8) for prec in (0, 1)
         if not (n == 262144 and nic > 0 and prec == 0)]


@pytest.mark.parametrize("n,nic,prec", CASES)
def test_microbench_rows_match_oracle(rg, orc, n, nic, prec):
    o = _oracle(orc, n, nic)
    rng = np.random.default_rng(n + nic)
    rows = np.sort(rng.choice(n, ROWS, replace=False))
    grid = _grid()
    pts = grid[np.sort(rng.choice(len(grid), ROWS, replace=False))]
    eng, d = _gpu(rg, prec, n, nic)
    acc = d.calculate_acceleration_particles()[rows]
    fld = d.calc_field_at_batch(pts)
    eng.close()
    a_max, a_rms = _errs(acc, o.accel_rows(rows))
    f_max, f_rms = _errs(fld, o.field_at(pts), floor=2.0e3 / (1000 * NM))
    tol = TOL64 if prec == 0 else TOL32
    print("N=%d N_ic_max=%d %s: accel max %.2e rms %.2e; cathode field max %.2e rms %.2e"
          % (n, nic, "fp64" if prec == 0 else "fp32c", a_max, a_rms, f_max, f_rms))
    assert a_max <= tol and f_max <= tol, (a_max, f_max)


def _one_diode(rg, orc, phi, jumps, cap=8192):
    side = 1000 * NM
    kw = dict(V_s=2.0e3, gap=1000 * NM, time_step=0.25e-15, image_charge=True, N_ic_max=0, capacity=cap,
              emitter_pos=(-side / 2, -side / 2), emitter_dim=(side, side), work=[[phi]], emission=True,
              mh_jumps=jumps, seed=20261203)
    eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=1, particle_capacity=cap + 64, chain_capacity=cap + 64,
                    quad_capacity=rg.supply_points(**kw) + 64)
    d = eng.add_diode(**kw)
    o = orc.OracleDiode(cap=cap, V_s=2.0e3, d=1000 * NM, time_step=0.25e-15, image_charge=True, N_ic_max=0)
    o.set_planar_emitter(-side / 2, -side / 2, side, side, [[phi]])
    o.set_emission(True, seed=20261203, mh_jumps=jumps, max_chains=cap)   # the default supply rule
    return eng, d, o


def _same_step(d, o, step):
    c = d.counters()
    assert c["N_sup"] == pytest.approx(o.s.N_sup, rel=1e-12), step
    assert c["chains"] == o.s.last_chains and c["chains_failed"] == o.s.last_failed_chains, step
    assert c["MH_std"] == pytest.approx(o.s.MH_std, rel=1e-12), step
    assert c["emitted_step"] == o.s.emitted_step, step
    assert d.n == o.n, step
    return c


@pytest.mark.parametrize("jumps", [200, 100])
def test_one_diode_deck_empty_fp64_chain_for_chain(rg, orc, jumps):
    """4.7 eV as specified: ~1932 chains per step and an escape probability of
    ~3e-13, so nothing is emitted; the supply integral, the chain count, every
    chain's MH_std schedule and the (absent) emission agree."""
    eng, d, o = _one_diode(rg, orc, 4.7, jumps)
    for step in (1, 2):
        eng.step(step)
        o.step(step)
        c = _same_step(d, o, step)
        assert 1800 < c["chains"] < 2100 and c["emitted_step"] == 0
        print("4.7 eV, %d jumps, step %d: N_sup %.3f, chains %d, MH_std %.6f"
              % (jumps, step, c["N_sup"], c["chains"], c["MH_std"]))
    eng.close()


def test_one_diode_deck_populated_fp64_chain_for_chain(rg, orc):
    """The populated 2.0 eV variant, three full steps with 200 jumps: the
    emitted electrons (positions, ids), the space-charge-fed supply integral
    and the trajectories agree with the oracle."""
    eng, d, o = _one_diode(rg, orc, 2.0, 200)
    for step in (1, 2, 3):
        eng.step(step)
        o.step(step)
        c = _same_step(d, o, step)
        print("2.0 eV step %d: N_sup %.3f, chains %d, emitted %d, in flight %d"
              % (step, c["N_sup"], c["chains"], c["emitted_step"], d.n))
    assert d.n > 500
    p = d.particles()
    np.testing.assert_array_equal(p["id"], o.iarr("id"))
    assert np.max(np.abs(p["pos"] - o.arr("pos"))) < 1e-9 * NM
    assert c["ramo_current"] == pytest.approx(o.s.ramo_current, rel=1e-9)
    eng.close()


@pytest.mark.parametrize("r_apex,V", [(10 * NM, 1.0e3), (50 * NM, 1.5e3)])
def test_tip_deck_fp64_chain_for_chain(rg, orc, r_apex, V):
    """A hyperboloid tip of the 16-tip deck: h 500 nm, tip-anode gap 1000 nm,
    base radius R = sqrt(r (h^2 + 2 d h) / d) for apex radius r, 4.5 eV,
    80 MH jumps, 3000 electrons in flight.  Two FP64 steps against the oracle.
    The voltages, at the low end of the deck's 1-5 kV, keep the oracle's
    serial cost at seconds: ~2800 and ~4900 chains, a few hundred emitted."""
    h, dd, n0 = 500 * NM, 1000 * NM, 3000
    R = math.sqrt(r_apex * (h * h + 2.0 * dd * h) / dd)
    tip = (dd, R, h)
    rng = np.random.default_rng(int(r_apex / NM))
    pos = np.column_stack([rng.uniform(-R, R, n0), rng.uniform(-R, R, n0),
                           rng.uniform(h + 1 * NM, h + dd - 1 * NM, n0)])
    cap = 16384
    eng = rg.Engine(precision=rg.PREC_FP64, max_diodes=1, particle_capacity=cap + 64, chain_capacity=cap + 64,
                    quad_capacity=10000 + 64)
    d = eng.add_diode(geometry=rg.GEOM_TIP, V_s=V, time_step=0.25e-15, image_charge=True, capacity=cap,
                      tip_dim=tip, tip_work_function=4.5, emission=True, seed=7)
    d.add_particles(pos, step=0)
    o = orc.OracleDiode(orc.TIP, cap=cap, V_s=V, d=dd, time_step=0.25e-15, image_charge=True)
    o.set_tip(*tip, 4.5)
    o.set_emission(True, seed=7, max_chains=cap)
    for p in pos:
        o.add(p, step=0)
    assert o.s.r_tip == pytest.approx(r_apex, rel=1e-9)   # the apex radius recomputes exactly
    for step in (1, 2):
        eng.step(step)
        o.step(step)
        c = d.counters()
        assert c["N_sup"] == pytest.approx(o.s.N_sup, rel=1e-10), step
        assert c["chains"] == o.s.last_chains, step
        assert c["emitted_step"] == o.s.emitted_step, step
        assert d.n == o.n, step
        print("tip r=%.0f nm step %d: N_sup %.2f, chains %d, emitted %d, in flight %d"
              % (r_apex / NM, step, c["N_sup"], c["chains"], c["emitted_step"], d.n))
    p = d.particles()
    np.testing.assert_array_equal(p["id"], o.iarr("id"))
    assert np.max(np.abs(p["pos"] - o.arr("pos"))) < 1e-6 * NM
    eng.close()
