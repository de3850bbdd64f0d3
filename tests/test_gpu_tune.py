"""The pair-sum chunking, the MH launch shape and their autotuner
(rd_autotune / rd_set_chunking / rd_set_mh_launch).  The chunking sets the
j-chunk lengths of every pair sum; a result depends on it only in the last
FP32 bits, so: tuning leaves the particle state exactly as it was, a run
continued after tuning equals the same run continued under the chosen
chunking set by hand, and a diode is bit-identical alone and in a mix under
any one chunking.  The MH launch shape (plan parts on streams, FP32 thread
form) changes no bit at all."""
import numpy as np
import pytest

from test_gpu_serve import make_requests

pytestmark = pytest.mark.gpu

NM = 1e-9


def _engine(rg, reqs, **cfg):
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=len(reqs), particle_capacity=len(reqs) * 1024,
                    chain_capacity=len(reqs) * 256, quad_capacity=len(reqs) * 1024, **cfg)
    ds = []
    for steps, pos, kw in reqs:
        d = eng.add_diode(**kw)
        d.add_particles(pos, step=0)
        ds.append(d)
    return eng, ds


def _state(ds):
    return [d.particles() for d in ds]


def _same(a, b):
    for pa, pb in zip(a, b):
        for key in pa:
            np.testing.assert_array_equal(pa[key], pb[key], err_msg=key)


def test_autotune_keeps_state_and_matches_chosen_chunking(rg):
    reqs = make_requests(n=4, seed=11)
    e1, d1 = _engine(rg, reqs)
    e1.run(1, 3)
    before = _state(d1)
    t = e1.autotune()
    assert t["candidates"] == 15 + 4 * 2     # chunkings, then MH parts 1-4 x two thread forms
    assert 1 <= t["mh_parts"] <= 4 and t["mh_form"] in (0, 1)
    assert e1.get_mh_launch() == (t["mh_parts"], t["mh_form"])
    assert t["chunk_min"] in (128, 256, 512, 1024, 2048) and t["chunk_count_max"] in (8, 16, 32)
    assert 0 < t["ms_chosen"] <= t["ms_default"]
    assert e1.get_chunking() == (t["chunk_min"], t["chunk_count_max"])
    _same(before, _state(d1))                           # nothing moved
    e1.run(4, 3)
    e2, d2 = _engine(rg, reqs)
    e2.run(1, 3)
    e2.set_chunking(t["chunk_min"], t["chunk_count_max"])
    e2.run(4, 3)
    _same(_state(d1), _state(d2))
    e1.close()
    e2.close()


@pytest.mark.parametrize("chunking", [(512, 8), (2048, 32)])
def test_alone_equals_mix_under_a_chunking(rg, chunking):
    """A lone emitting diode runs the 64-thread, two-chains-per-thread MH jump
    form and a mix the 32-thread, four-chain form: the states must still be
    bit-equal."""
    reqs = make_requests(n=3, seed=5)
    eng, ds = _engine(rg, reqs, chunk_min=chunking[0], chunk_count_max=chunking[1])
    eng.run(1, 4)
    mixed = _state(ds)
    eng.close()
    for (steps, pos, kw), m in zip(reqs, mixed):
        one = rg.Engine(precision=rg.PREC_FP32C, max_diodes=1, particle_capacity=4096, chain_capacity=1024,
                        quad_capacity=1024, chunk_min=chunking[0], chunk_count_max=chunking[1])
        d = one.add_diode(**kw)
        d.add_particles(pos, step=0)
        one.run(1, 4)
        _same([m], [d.particles()])
        one.close()


def test_mh_launch_shapes_change_no_bit(rg):
    """Every planar MH launch shape -- 1 to 4 launches per jump over parts of
    the plan, 32 threads x 4 chains or 64 x 2 -- gives bit-identical states."""
    reqs = make_requests(n=5, seed=13)
    ref = None
    for parts, form in ((0, -1), (1, 0), (2, 1), (3, 0), (4, 1), (4, 0)):
        eng, ds = _engine(rg, reqs)
        eng.set_mh_launch(parts, form)
        eng.run(1, 3)
        if parts:
            assert eng.get_mh_launch() == (parts, form)
        st = _state(ds)
        eng.close()
        if ref is None:
            ref = st
        else:
            _same(ref, st)
