"""rd_field_at_noalloc: the field-at-points entry point for callers that
cannot allocate device memory while they run (their device memory belongs to
another runtime, or their memory budget is fixed up front).  It must give the
same fields as rd_field_at, on two calls in a row, using only its static
scratch.  This file is collected last; it passes alone and after the others.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NM = 1e-9


def _setup(rg, prec, n=700, nic=1, seed=17):
    rng = np.random.default_rng(seed)
    pos = np.column_stack([rng.uniform(-500 * NM, 500 * NM, n), rng.uniform(-500 * NM, 500 * NM, n),
                           rng.uniform(1 * NM, 999 * NM, n)])
    eng = rg.Engine(precision=prec, max_diodes=3, particle_capacity=8192)
    other = eng.add_diode(V_s=1.0e3, gap=800 * NM, capacity=512)      # a second resident diode
    other.add_particles(pos[:200] * 0.8)
    d = eng.add_diode(V_s=2.0e3, gap=1000 * NM, capacity=2048, N_ic_max=nic)
    d.add_particles(pos)
    return eng, d


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-5)])
def test_noalloc_matches_field_at_twice(rg, prec, tol):
    torch = pytest.importorskip("torch")
    eng, d = _setup(rg, prec)
    rng = np.random.default_rng(5)
    for call in range(2):
        m = 3000 + 1000 * call
        pts = np.column_stack([rng.uniform(-500 * NM, 500 * NM, m), rng.uniform(-500 * NM, 500 * NM, m),
                               rng.uniform(0.0, 999 * NM, m)])
        pts[: m // 3, 2] = 0.0                                        # cathode points too
        ref = d.calc_field_at_batch(pts)
        p_dev = torch.tensor(pts, dtype=torch.float64, device="cuda").contiguous()
        f_dev = torch.full((m, 3), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        d.calc_field_at_batch_noalloc(p_dev.data_ptr(), f_dev.data_ptr(), m)
        got = f_dev.cpu().numpy()
        rel = np.max(np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1))
        assert rel <= tol, (call, rel)
    eng.close()


def test_noalloc_rejects_too_many_points(rg):
    torch = pytest.importorskip("torch")
    eng, d = _setup(rg, 1)
    buf = torch.zeros((4, 3), dtype=torch.float64, device="cuda")
    with pytest.raises(rg.RumdeedError, match="65536"):
        d.calc_field_at_batch_noalloc(buf.data_ptr(), buf.data_ptr(), 65537)
    d.calc_field_at_batch_noalloc(buf.data_ptr(), buf.data_ptr(), 0)   # empty call is a no-op
    eng.close()
