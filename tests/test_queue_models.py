"""The single-server queue models that the serving measurement reports beside
its p99 (first come first served, processor sharing, shortest remaining
service first, each at the requests' isolated service times), on traces whose
latencies follow by hand."""
import numpy as np

import bench_configs as bc

ARR = [0.0, 0.1, 0.1, 0.5]
SVC = [0.3, 0.1, 0.2, 0.05]


def test_fifo():
    assert np.allclose(bc.fifo_latencies(ARR, SVC), [0.3, 0.3, 0.5, 0.15])


def test_processor_sharing():
    # A alone to 0.1; A, B, C share until B ends at 0.4; A, C to 0.5; then
    # A, C, D with 0.05 each end together at 0.65
    assert np.allclose(bc.shared_latencies(ARR, SVC, "ps"), [0.65, 0.3, 0.55, 0.15])


def test_shortest_remaining_first():
    # B preempts A at 0.1; A (tie with C, earlier) to 0.4; D preempts C at 0.5
    assert np.allclose(bc.shared_latencies(ARR, SVC, "srpt"), [0.4, 0.1, 0.55, 0.05])


def test_work_conservation():
    rng = np.random.default_rng(3)
    arr = np.sort(rng.uniform(0, 10, 200))
    svc = rng.lognormal(-3, 1.5, 200)
    last = {}
    for name, lat in (("fifo", bc.fifo_latencies(arr, svc)), ("ps", bc.shared_latencies(arr, svc, "ps")),
                      ("srpt", bc.shared_latencies(arr, svc, "srpt"))):
        assert np.all(lat >= svc - 1e-9)
        last[name] = float(np.max(arr + lat))
    # every work-conserving single server empties at the same time
    assert abs(last["fifo"] - last["ps"]) < 1e-6 and abs(last["fifo"] - last["srpt"]) < 1e-6
