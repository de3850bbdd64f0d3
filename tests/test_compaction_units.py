"""The index arithmetic of the in-place compaction (rd_step.cu: k_compact_count,
k_compact_scan, k_compact_move), restated on the host and checked on random removal
patterns: every moving survivor's destination lies below its own index, inside the
range of units the moving unit waits for or inside itself, so a unit never writes a
position an unfinished earlier unit has still to read, and the survivors end in
creation order (compact_array, src/mod_pair.F90:1180-1223)."""
import numpy as np
import pytest

UNIT = 256


def plan_units(mask):
    """Per 256-particle unit: survivors (cnt) and first destination (pre), as the
    count and scan kernels form them."""
    n = mask.size
    units = (n + UNIT - 1) // UNIT
    padded = np.zeros(units * UNIT, dtype=np.int64)
    padded[:n] = mask
    cnt = padded.reshape(units, UNIT).sum(axis=1)
    pre = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    return cnt, pre


def move_units(mask):
    """Destinations of the moving survivors and, per unit, the range of earlier
    units it waits for (t_lo .. t_hi), as k_compact_move forms them."""
    n = mask.size
    cnt, pre = plan_units(mask)
    dead = np.flatnonzero(mask == 0)
    fd = dead[0] if dead.size else n
    moves, waits = [], []
    for u in range(cnt.size):
        i0 = u * UNIT
        if i0 >= n or i0 + UNIT <= fd:
            waits.append((0, -1))
            continue
        before, ku = int(pre[u]), int(cnt[u])
        t_lo = before >> 8
        t_hi = min(u - 1, (before + ku - 1) >> 8) if ku > 0 else -1
        waits.append((t_lo, t_hi))
        idx = np.arange(i0, min(i0 + UNIT, n))
        m = mask[idx]
        pos = np.cumsum(m) - m   # survivors of the unit before each lane
        for i, mi, pi in zip(idx, m, pos):
            if mi and i >= fd:
                moves.append((int(i), before + int(pi), u))
    return moves, waits, fd


@pytest.mark.parametrize("n,pattern", [(5000, "quarter"), (24000, "quarter"), (30000, "scattered"),
                                       (777, "front"), (4096, "all"), (2500, "none"), (65536, "random")])
def test_compaction_units(n, pattern):
    rng = np.random.default_rng(n)
    mask = np.ones(n, dtype=np.int64)
    if pattern == "quarter":
        mask[(np.arange(n) % 4) != 0] = 0
    elif pattern == "scattered":
        mask[rng.choice(n, n // 100, replace=False)] = 0
    elif pattern == "front":
        mask[:5] = 0
    elif pattern == "all":
        mask[:] = 0
    elif pattern == "random":
        mask = (rng.random(n) < 0.6).astype(np.int64)
    moves, waits, fd = move_units(mask)
    state = np.arange(n)          # what sits at each position; compaction in place
    out = state.copy()
    for i, dst, u in moves:
        assert dst < i                                # below the survivor's own index
        du = dst // UNIT
        t_lo, t_hi = waits[u]
        assert du == u or t_lo <= du <= t_hi, (i, dst, u, waits[u])   # a unit it waits for, or itself
        assert du <= u
        out[dst] = state[i]
    keep = np.flatnonzero(mask)
    np.testing.assert_array_equal(out[:keep.size], keep)   # creation order
    # positions below the first removed particle never move
    np.testing.assert_array_equal(out[:min(fd, keep.size)], np.arange(min(fd, keep.size)))
