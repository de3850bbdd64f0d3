"""Emission statistics over seeds: the FP32-compensated GPU form against the
FP64 oracle.  The two draw different random numbers (the FP32 chains use FP32
draws from the same Philox counters), so they agree statistically, not run
for run: a populated planar diode runs STEPS full time steps per seed, and
over SEEDS the means of the emitted electrons, the electrons absorbed at the
anode and at the cathode, and the mean Ramo current agree within three
standard errors of the difference of the two means (src/mod_tests.F90
checks its planar system against bands in the same spirit, :2013-2119)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NM = 1e-9
STEPS = 40
SEEDS = range(1, 9)
KW = dict(V_s=1.0e3, gap=500 * NM, time_step=2.0e-15, image_charge=True, N_ic_max=0, capacity=4096,
          emitter_pos=(-50 * NM, -50 * NM), emitter_dim=(100 * NM, 100 * NM), work=[[2.0]],
          emission=True, mh_jumps=60, max_chains=300, quad_panels=8, quad_order=4)


def _gpu_run(rg, seed):
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=1, particle_capacity=4096 + 64,
                    chain_capacity=4096 + 64, quad_capacity=4096)
    d = eng.add_diode(seed=seed, **KW)
    ramo = []
    for s in range(1, STEPS + 1):
        eng.step(s)
        ramo.append(d.counters()["ramo_current"])
    c = d.counters()
    eng.close()
    return [c["emitted_total"], c["absorbed_top_total"], c["absorbed_bot_total"], float(np.mean(ramo))]


def _oracle_run(orc, seed):
    o = orc.OracleDiode(cap=4096, V_s=KW["V_s"], d=KW["gap"], time_step=KW["time_step"], image_charge=True,
                        N_ic_max=0)
    o.set_planar_emitter(-50 * NM, -50 * NM, 100 * NM, 100 * NM, KW["work"])
    o.set_emission(True, seed=seed, mh_jumps=60, max_chains=300, quad_panels=8, quad_order=4)
    ramo = []
    for s in range(1, STEPS + 1):
        o.step(s)
        ramo.append(o.s.ramo_current)
    return [o.s.emitted_total, o.s.absorbed_top_total, o.s.absorbed_bot_total, float(np.mean(ramo))]


def test_fp32c_emission_statistics_match_oracle_over_seeds(rg, orc):
    g = np.array([_gpu_run(rg, s) for s in SEEDS], dtype=float)
    o = np.array([_oracle_run(orc, s) for s in SEEDS], dtype=float)
    n = len(SEEDS)
    names = ["emitted", "absorbed_top", "absorbed_bot", "ramo_mean"]
    assert g[:, 0].mean() > 50, "the diode must emit for the comparison to mean anything"
    assert g[:, 1].mean() > 0, "electrons must reach the anode within the run"
    for k, name in enumerate(names):
        se = np.sqrt(g[:, k].var(ddof=1) / n + o[:, k].var(ddof=1) / n)
        floor = 1.0 if k < 3 else 1e-3 * abs(o[:, k].mean())   # integer counts; current scale
        diff = abs(g[:, k].mean() - o[:, k].mean())
        assert diff <= 3.0 * max(se, floor), (name, g[:, k].mean(), o[:, k].mean(), se)
