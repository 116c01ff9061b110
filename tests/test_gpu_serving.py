"""Continuous batching: requests arriving while others run are admitted into
new GPU batches that overlap with the running ones; every result equals the
same model run alone (bitwise), in FP64 and in mixed precision."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_served_results_equal_standalone_runs(gpu, mixed):
    from fedem_gb300 import models
    from fedem_gb300.batch import Batch, Model, Server

    cases = models.batch_c4(10, seed=77, n_max=300, steps=60)
    mods = [Model(f, o) for f, o, _ in cases]
    srv = Server(budget_bytes=8e9, mixed=mixed, min_batch=2, max_wait=0.005)
    ids, overlap = [], 0
    for k, m in enumerate(mods):
        ids.append(srv.submit(m))
        srv.pump()
        overlap = max(overlap, srv.status()["live_batches"])
        time.sleep(0.002)
    t0 = time.time()
    while any(srv.request(i)["state"] < 2 for i in ids):
        srv.pump()
        overlap = max(overlap, srv.status()["live_batches"])
        assert time.time() - t0 < 120
    assert overlap >= 2  # later arrivals ran while earlier batches were still on the GPU
    for k, i in enumerate(ids):
        r = srv.request(i)
        assert r["state"] == 2 and r["finished"] >= r["admitted"] >= r["arrival"]
        alone = Batch([mods[k]], mixed=mixed)
        alone.run()
        assert np.array_equal(srv.result(i), alone.triads(0)), k
        assert r["iterations"] == alone.info(0)["iterations"]
