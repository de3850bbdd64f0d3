"""Emission statistics over seeds: the FP32-compensated GPU form against the
FP64 oracle.  The two draw different proposals (the FP32 chains step in FP32
from Gaussian pairs drawn in FP32 on the same Philox counters; their accept /
reject decisions are the FP64 form's), so they agree statistically, not run
for run.

Two diodes:
* a small one (100 x 100 nm emitter, 500 nm gap, 1 kV, 2.0 eV, 60 MH jumps),
  SEEDS x STEPS full time steps;
* the one-diode deck's populated variant (1000 x 1000 nm emitter, 1 um gap,
  2 kV, 2.0 eV, 100 MH jumps), fewer steps.
Over the seeds the means of the emitted electrons, the electrons absorbed at
the anode and at the cathode, and the mean Ramo current agree within three
standard errors of the difference of the two means (src/mod_tests.F90 checks
its planar system against bands in the same spirit, :2013-2119), and the
emission sites, pooled over seeds and steps in an 8 x 8 histogram over the
emitter, pass a chi-square test of homogeneity against the oracle's at the
1e-3 level (the emission-site density).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NM = 1e-9

SMALL = dict(kw=dict(V_s=1.0e3, gap=500 * NM, time_step=2.0e-15, image_charge=True, N_ic_max=0, capacity=4096,
                     emitter_pos=(-50 * NM, -50 * NM), emitter_dim=(100 * NM, 100 * NM), work=[[2.0]],
                     emission=True, mh_jumps=60, max_chains=300, quad_panels=8, quad_order=4),
             steps=60, seeds=range(1, 17))
DECK = dict(kw=dict(V_s=2.0e3, gap=1000 * NM, time_step=0.25e-15, image_charge=True, N_ic_max=0, capacity=8192,
                    emitter_pos=(-500 * NM, -500 * NM), emitter_dim=(1000 * NM, 1000 * NM), work=[[2.0]],
                    emission=True, mh_jumps=100, max_chains=8192, quad_panels=0, quad_order=0),
            steps=6, seeds=range(1, 9))
BINS = 8


def _site_bins(xy, kw):
    x0, y0 = kw["emitter_pos"]
    Lx, Ly = kw["emitter_dim"]
    ix = np.clip(((xy[:, 0] - x0) / Lx * BINS).astype(int), 0, BINS - 1)
    iy = np.clip(((xy[:, 1] - y0) / Ly * BINS).astype(int), 0, BINS - 1)
    return np.bincount(ix * BINS + iy, minlength=BINS * BINS)


def _gpu_run(rg, case, seed):
    kw = case["kw"]
    cap = kw["capacity"]
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=1, particle_capacity=cap + 64, chain_capacity=cap + 64,
                    quad_capacity=65536, event_capacity=1 << 17)
    d = eng.add_diode(seed=seed, **kw)
    ramo, sites = [], []
    for s in range(1, case["steps"] + 1):
        eng.step(s)
        ramo.append(d.counters()["ramo_current"])
        ev, lost = eng.events_take()
        assert lost == 0
        sites += [e["pos"][:2] for e in ev if e["kind"] == rg.EVENT_EMIT]
    c = d.counters()
    eng.close()
    assert len(sites) == c["emitted_total"]
    return ([c["emitted_total"], c["absorbed_top_total"], c["absorbed_bot_total"], float(np.mean(ramo))],
            _site_bins(np.array(sites).reshape(-1, 2), kw))


def _oracle_run(orc, case, seed):
    kw = case["kw"]
    o = orc.OracleDiode(cap=kw["capacity"], V_s=kw["V_s"], d=kw["gap"], time_step=kw["time_step"],
                        image_charge=True, N_ic_max=0)
    o.set_planar_emitter(*kw["emitter_pos"], *kw["emitter_dim"], kw["work"])
    o.set_emission(True, seed=seed, mh_jumps=kw["mh_jumps"], max_chains=kw["max_chains"],
                   quad_panels=kw["quad_panels"], quad_order=kw["quad_order"])
    ramo, sites = [], []
    for s in range(1, case["steps"] + 1):
        n0 = o.n
        o.emission(s)
        sites.append(o.arr("pos")[n0:, :2])
        o.verlet(s)
        o.remove(s)
        ramo.append(o.s.ramo_current)
    return ([o.s.emitted_total, o.s.absorbed_top_total, o.s.absorbed_bot_total, float(np.mean(ramo))],
            _site_bins(np.vstack(sites), kw))


def _compare(g, o, gh, oh, need_top=True):
    n = len(g)
    g = np.array(g, dtype=float)
    o = np.array(o, dtype=float)
    names = ["emitted", "absorbed_top", "absorbed_bot", "ramo_mean"]
    assert g[:, 0].mean() > 50, "the diode must emit for the comparison to mean anything"
    if need_top:
        assert g[:, 1].mean() > 0, "electrons must reach the anode within the run"
    for k, name in enumerate(names):
        se = np.sqrt(g[:, k].var(ddof=1) / n + o[:, k].var(ddof=1) / n)
        floor = 1.0 if k < 3 else 1e-3 * abs(o[:, k].mean())   # integer counts; current scale
        diff = abs(g[:, k].mean() - o[:, k].mean())
        print("%s: gpu %.4g oracle %.4g (3 se %.3g)" % (name, g[:, k].mean(), o[:, k].mean(), 3 * se))
        assert diff <= 3.0 * max(se, floor), (name, g[:, k].mean(), o[:, k].mean(), se)
    from scipy.stats import chi2
    G, O = gh.sum(axis=0).astype(float), oh.sum(axis=0).astype(float)
    keep = (G + O) > 0
    G, O = G[keep], O[keep]
    a, b = np.sqrt(O.sum() / G.sum()), np.sqrt(G.sum() / O.sum())
    stat = float(np.sum((a * G - b * O) ** 2 / (G + O)))   # two-sample chi-square, unequal totals
    p = float(chi2.sf(stat, keep.sum() - 1))
    print("emission sites: %d gpu, %d oracle, chi2 %.1f on %d dof, p %.3g"
          % (G.sum(), O.sum(), stat, keep.sum() - 1, p))
    assert p > 1e-3, (stat, p)


def test_fp32c_emission_statistics_match_oracle_over_seeds(rg, orc):
    pytest.importorskip("scipy")
    gr = [_gpu_run(rg, SMALL, s) for s in SMALL["seeds"]]
    orr = [_oracle_run(orc, SMALL, s) for s in SMALL["seeds"]]
    _compare([x[0] for x in gr], [x[0] for x in orr], np.array([x[1] for x in gr]), np.array([x[1] for x in orr]))


def test_fp32c_emission_statistics_one_diode_deck_populated(rg, orc):
    pytest.importorskip("scipy")
    gr = [_gpu_run(rg, DECK, s) for s in DECK["seeds"]]
    orr = [_oracle_run(orc, DECK, s) for s in DECK["seeds"]]
    _compare([x[0] for x in gr], [x[0] for x in orr], np.array([x[1] for x in gr]), np.array([x[1] for x in orr]),
             need_top=False)
