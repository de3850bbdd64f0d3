"""The supply-integral rule against a converged integral (oracle, CPU).

The reference integrates the emission supply N_sup (Do_Surface_Integration_FE,
src/mod_field_emission_v2.F90:635-656) with the adaptive Cuba library, asking
for an absolute error of 0.5 electron or a relative one of 1e-3
(src/mod_global.F90:84-92).  Here a composite Gauss-Legendre rule replaces it,
on the GPU and in the oracle alike.  This test integrates the same integrand
adaptively to convergence (orc_supply_planar_converged: bisection driven by
the Gauss-Legendre error and forced near every electron lower than half a
panel) and checks the default rule against it within the reference's
tolerance, max(0.5, 1e-3 N_sup), on states where the integrand has nm-scale
structure:

* a freshly emitted layer: 1136 electrons 1.0-1.2 nm above the 1000 x 1000 nm
  emitter of the one-diode deck (2 kV, 1 um gap, 2.0 eV), as after three
  steps of its populated variant;
* a space-charge-limited state: the central 500 x 500 nm of that deck after
  30 steps (tests/golden/supply_state_deck30.npy, made by
  tests/golden/make_supply_state.py), 2201 electrons, most within a few nm of
  the cathode;
* five diodes of the serving stream (pre-filled uniformly in the gap).

The former fixed rule (16 x 16 panels of 4 x 4 nodes) misses the tolerance on
the second state, which the test also asserts, so it would catch a regression
to it.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NM = 1e-9


def _diode(orc, pos, V, d, side, phi):
    o = orc.OracleDiode(cap=max(len(pos), 1), V_s=V, d=d, time_step=0.25e-15)
    o.set_planar_emitter(-side / 2, -side / 2, side, side, [[phi]])
    o.set_emission(True, seed=1)
    o.add_many(pos)
    return o


def _check(o, name, fixed16_fails=False):
    default = o.supply()
    conv, evals = o.supply_converged(0.01, 12)
    tol = max(0.5, 1e-3 * conv)
    print("%s: panels %d, default rule %+.3f, converged %.3f (%d evaluations), tolerance %.3f"
          % (name, o.L.orc_supply_panels(o.p), default - conv, conv, evals, tol))
    assert abs(default - conv) <= tol, (name, default, conv)
    if fixed16_fails:
        o.s.quad_panels = 16
        coarse = o.supply()
        o.s.quad_panels = 0
        assert abs(coarse - conv) > tol, (name, coarse, conv)


def test_supply_rule_fresh_emission_layer(orc):
    rng = np.random.default_rng(3)
    n = 1136
    pos = np.column_stack([rng.uniform(-500 * NM, 500 * NM, n), rng.uniform(-500 * NM, 500 * NM, n),
                           rng.uniform(1.0 * NM, 1.2 * NM, n)])
    _check(_diode(orc, pos, 2e3, 1000 * NM, 1000 * NM, 2.0), "fresh layer")


def test_supply_rule_space_charge_limited_state(orc):
    pos = np.load(os.path.join(ROOT, "tests", "golden", "supply_state_deck30.npy"))
    assert pos.shape == (2201, 3) and np.mean(pos[:, 2] < 8 * NM) > 0.7
    _check(_diode(orc, pos, 2e3, 1000 * NM, 500 * NM, 2.0), "deck after 30 steps", fixed16_fails=True)


def test_supply_rule_stream_diodes(orc):
    sys.path.insert(0, ROOT)
    import bench
    st = bench.RequestStream(bench.SEED)
    done = 0
    while done < 5:
        r = st.next()
        if r["capacity"] > 3000:
            continue
        _check(_diode(orc, bench.prefill(r), r["V_s"], r["gap"], r["side"], r["phi"]),
               "stream request %d" % r["index"])
        done += 1


def test_default_rule_spacing(orc):
    """Nodes at most 5 nm apart along the longer emitter side, 16 to 256 panels."""
    for side, panels in ((100 * NM, 16), (320 * NM, 16), (1000 * NM, 50), (2000 * NM, 100), (6000 * NM, 256)):
        o = orc.OracleDiode(cap=1)
        o.set_planar_emitter(-side / 2, -side / 2, side, side, [[4.7]])
        assert o.L.orc_supply_panels(o.p) == panels, side


def test_library_takes_the_same_rule(orc, rg):
    """rd_supply_points (the library's rule, no GPU needed) equals the oracle's."""
    for side in (100 * NM, 577 * NM, 1000 * NM, 1517 * NM, 2000 * NM):
        o = orc.OracleDiode(cap=1)
        o.set_planar_emitter(-side / 2, -side / 2, side, side, [[4.7]])
        P = o.L.orc_supply_panels(o.p)
        assert rg.supply_points(emitter_pos=(-side / 2, -side / 2), emitter_dim=(side, side), emission=True) \
            == (4 * P) ** 2, side
    o = orc.OracleDiode(cap=1, V_s=2e3, d=1000 * NM)
    o.set_planar_emitter(-500 * NM, -500 * NM, 1000 * NM, 1000 * NM, [[4.7]])
    o.set_ring(400 * NM, 50 * NM)
    P = o.L.orc_supply_panels(o.p)
    assert rg.supply_points(V_s=2e3, gap=1000 * NM, emitter_pos=(-500 * NM, -500 * NM),
                            emitter_dim=(400 * NM, 400 * NM), emitter_type=4, emitter_thickness=50 * NM,
                            emission=True) == (4 * P) ** 2
