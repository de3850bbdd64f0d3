"""Engine lifetime on the GPU: creating, stepping and destroying engines
returns their device memory (pools, scratch, graphs, streams), and a
destroyed engine's diodes leave no state behind for the next engine."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NM = 1e-9


def _free_bytes():
    torch = pytest.importorskip("torch")
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def _cycle(rg, seed):
    rng = np.random.default_rng(seed)
    eng = rg.Engine(precision=rg.PREC_FP32C, max_diodes=4, particle_capacity=1 << 16,
                    chain_capacity=1 << 14, quad_capacity=1 << 14)
    for k in range(3):
        d = eng.add_diode(V_s=2.0e3, gap=800 * NM, capacity=4096, emitter_pos=(-100 * NM, -100 * NM),
                          emitter_dim=(200 * NM, 200 * NM), work=[[2.5]], emission=True, mh_jumps=20,
                          max_chains=256, seed=seed + k)
        d.add_particles(np.column_stack([rng.uniform(-100 * NM, 100 * NM, 500), rng.uniform(-100 * NM, 100 * NM, 500),
                                         rng.uniform(2 * NM, 790 * NM, 500)]), step=0)
    eng.run(1, 3)                 # graph capture, both MH streams
    counters = [d.counters() for d in eng.diodes.values()]
    eng.close()
    return counters


def test_engines_release_device_memory(rg):
    first = _cycle(rg, 1)         # warm-up: context, module load, allocator caches
    base = _free_bytes()
    for k in range(8):
        again = _cycle(rg, 1)
        assert again == first     # same inputs, same results, engine after engine
    leaked = base - _free_bytes()
    assert leaked < 64 * 1024 * 1024, "%.1f MiB not returned" % (leaked / 2 ** 20)
