"""The headline's timed window (bench.py: fifo_schedule, steady_window) holds
continuous batching on the serving stream: the server is saturated (every slot
resident, requests queued), a resident runs its last step in the first timed
iteration and the queue head is admitted after it, and the first-come-first-served
schedule never holds more requests than slots."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _stream():
    st = bench.RequestStream(bench.SEED)
    reqs = []
    while True:
        r = st.next()
        if r is None:
            return reqs
        reqs.append(r)


def test_fifo_schedule_slots_and_order():
    reqs = _stream()
    S = 128
    sched = bench.fifo_schedule(reqs, S)
    admits = np.array([a for a, _ in sched])
    dones = np.array([d for _, d in sched])
    assert np.all(np.diff(admits) >= 0)                          # first come, first served
    assert np.all(dones - admits == np.array([r["steps"] for r in reqs]))
    assert all(a * bench.STEP_S_EST >= r["arrival"] - bench.STEP_S_EST for r, (a, _) in zip(reqs, sched))
    events = sorted([(a, 1) for a in admits] + [(d, -1) for d in dones], key=lambda e: (e[0], e[1]))
    live, peak = 0, 0
    for _, k in events:
        live += k
        peak = max(peak, live)
    assert peak <= S


def test_steady_window_holds_admission_and_retirement():
    reqs = _stream()
    S, lead = 128, 4
    T0, residents, queue = bench.steady_window(reqs, S, lead)
    assert T0 >= bench.WINDOW_AFTER
    assert len(residents) == S and len(queue) > 0                # saturated, requests waiting
    rems = [rem for _, rem in residents]
    assert min(rems) == lead + 1                                 # one runs its last step at T0
    assert all(rem > 0 for rem in rems)
