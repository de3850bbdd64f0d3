"""rd_field_at_noalloc: the field-at-points entry point for callers that
cannot allocate device memory while they run (their device memory belongs to
another runtime, or their memory budget is fixed up front).  It must give the
same fields as rd_field_at and as the oracle, on two calls in a row, using
only its static scratch, and commit no device memory.  This file is collected
last; it passes alone and after the others.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NM = 1e-9
TOL = {0: 1e-12, 1: 1e-5}   # FP64 plain form, FP32 compensated form (norm-relative per point)


def _nrel(a, b):
    return np.max(np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1))


def _box(rng, n, half=500 * NM, lo=1 * NM, hi=999 * NM):
    return np.column_stack([rng.uniform(-half, half, n), rng.uniform(-half, half, n), rng.uniform(lo, hi, n)])


def _setup(rg, orc, prec, n=700, nic=1, seed=17):
    rng = np.random.default_rng(seed)
    pos = _box(rng, n)
    eng = rg.Engine(precision=prec, max_diodes=3, particle_capacity=max(8192, 2 * n + 1024))
    other = eng.add_diode(V_s=1.0e3, gap=800 * NM, capacity=512)      # a second resident diode
    other.add_particles(pos[:200] * 0.8)
    d = eng.add_diode(V_s=2.0e3, gap=1000 * NM, capacity=max(2048, n), N_ic_max=nic)
    d.add_particles(pos)
    o = orc.OracleDiode(cap=max(2048, n), V_s=2.0e3, d=1000 * NM, N_ic_max=nic)
    for p in pos:
        o.add(p)
    return eng, d, o


def _noalloc(torch, d, pts):
    p_dev = torch.tensor(pts, dtype=torch.float64, device="cuda").contiguous()
    f_dev = torch.full((len(pts), 3), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()                       # the caller's writes are complete before the call
    d.calc_field_at_batch_noalloc(p_dev.data_ptr(), f_dev.data_ptr(), len(pts))
    return f_dev.cpu().numpy()


@pytest.mark.parametrize("prec", [0, 1])
def test_noalloc_matches_field_at_twice(rg, orc, prec):
    torch = pytest.importorskip("torch")
    eng, d, o = _setup(rg, orc, prec)
    rng = np.random.default_rng(5)
    for call in range(2):
        m = 3000 + 1000 * call
        pts = _box(rng, m, lo=0.0)
        pts[: m // 3, 2] = 0.0                                        # cathode points too
        ref = d.calc_field_at_batch(pts)
        got = _noalloc(torch, d, pts)
        assert _nrel(got, ref) <= TOL[prec], (call, _nrel(got, ref))
        sample = pts[::10]
        assert _nrel(got[::10], o.field_at(sample)) <= TOL[prec], call
    eng.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_noalloc_tip_diode(rg, orc, prec):
    """A hyperboloid tip: the sphere-image term of every point goes through the same scratch."""
    torch = pytest.importorskip("torch")
    tip = (900 * NM, 100 * NM, 100 * NM)
    rng = np.random.default_rng(11)
    n = 500
    pos = np.column_stack([rng.uniform(-300 * NM, 300 * NM, n), rng.uniform(-300 * NM, 300 * NM, n),
                           rng.uniform(105 * NM, 990 * NM, n)])
    eng = rg.Engine(precision=prec, max_diodes=2, particle_capacity=4096)
    d = eng.add_diode(geometry=rg.GEOM_TIP, V_s=2e3, capacity=1024, tip_dim=tip)
    d.add_particles(pos)
    o = orc.OracleDiode(orc.TIP, cap=1024, V_s=2e3, d=1000 * NM, image_charge=True)
    o.set_tip(*tip, 4.7)
    for p in pos:
        o.add(p)
    for call in range(2):
        pts = np.column_stack([rng.uniform(-200 * NM, 200 * NM, 700), rng.uniform(-200 * NM, 200 * NM, 700),
                               rng.uniform(110 * NM, 900 * NM, 700)])
        got = _noalloc(torch, d, pts)
        assert _nrel(got, d.calc_field_at_batch(pts)) <= TOL[prec], call
        assert _nrel(got, o.field_at(pts)) <= TOL[prec], call
    eng.close()


def test_noalloc_at_its_limit_allocates_nothing(rg, orc):
    """65536 points (the limit) against 20000 electrons: 512 point tiles x 20
    j-chunks exceed the scratch's 4096 partial-sum items, so the planner
    lengthens the chunks.  Two calls in a row match rd_field_at, a sample
    matches the oracle, and the device's free memory does not move across a
    call."""
    torch = pytest.importorskip("torch")
    prec = 1
    eng, d, o = _setup(rg, orc, prec, n=20000, nic=0, seed=23)
    rng = np.random.default_rng(29)
    for call in range(2):
        pts = _box(rng, 65536, lo=0.0)
        pts[::2, 2] = 0.0
        p_dev = torch.tensor(pts, dtype=torch.float64, device="cuda").contiguous()
        f_dev = torch.full((len(pts), 3), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        d.calc_field_at_batch_noalloc(p_dev.data_ptr(), f_dev.data_ptr(), len(pts))
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0, (call, free0 - free1)
        got = f_dev.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert _nrel(got, d.calc_field_at_batch(pts)) <= TOL[prec], call
        k = rng.choice(len(pts), 256, replace=False)
        assert _nrel(got[k], o.field_at(pts[k])) <= TOL[prec], call
    eng.close()


def test_noalloc_rejects_too_many_points(rg, orc):
    torch = pytest.importorskip("torch")
    eng, d, _ = _setup(rg, orc, 1, n=100)
    buf = torch.zeros((4, 3), dtype=torch.float64, device="cuda")
    with pytest.raises(rg.RumdeedError, match="65536"):
        d.calc_field_at_batch_noalloc(buf.data_ptr(), buf.data_ptr(), 65537)
    d.calc_field_at_batch_noalloc(buf.data_ptr(), buf.data_ptr(), 0)   # empty call is a no-op
    eng.close()
