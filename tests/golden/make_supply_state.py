"""Writes supply_state_deck30.npy: a space-charge-limited electron state for
the supply-rule convergence test (tests/test_oracle_supply.py).

The one-diode deck's populated variant (1 um gap, 2 kV, 1000 x 1000 nm
emitter centred on the axis, 2.0 eV, dt 0.25 fs, one image partner, 100 MH
jumps, Philox seed 20261203) is run for 30 full time steps in the oracle; the
electrons over the central 500 x 500 nm are kept (positions, m, (N, 3)).  Most
of them sit within a few nm of the cathode, where the supply integrand
varies on the nm scale.  Takes about two minutes on 8 cores:

    python tests/golden/make_supply_state.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import orc  # noqa: E402

NM = 1e-9


def main():
    side = 1000 * NM
    o = orc.OracleDiode(cap=20000, V_s=2e3, d=1000 * NM, time_step=0.25e-15)
    o.set_planar_emitter(-side / 2, -side / 2, side, side, [[2.0]])
    o.set_emission(True, seed=20261203, mh_jumps=100, max_chains=20000, quad_panels=16, quad_order=4)
    for step in range(1, 31):
        o.step(step)
    pos = o.arr("pos")
    keep = (np.abs(pos[:, 0]) < 250 * NM) & (np.abs(pos[:, 1]) < 250 * NM)
    path = os.path.join(HERE, "supply_state_deck30.npy")
    np.save(path, pos[keep])
    print("wrote %s: %d of %d electrons" % (path, keep.sum(), len(pos)))


if __name__ == "__main__":
    main()
