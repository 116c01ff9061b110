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


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_slot_reuse_moves_running_models_bitwise(gpu, tmp_path, mixed):
    """Two engines of at most four models; when one model finishes and requests
    wait, the running models stop at their step end and move with their whole
    state into a new engine with the waiting requests.  Models of every kind
    (beams, joints, reduced parts, springs/dampers, prescribed motions with
    linear quasi-static steps) end bitwise as when run alone."""
    import os

    from conftest import GOLDEN_DIR
    from fedem_gb300 import models
    from fedem_gb300.batch import Batch, Model, Server

    cases = [(f, o) for f, o, _ in models.batch_c4(5, seed=91, n_max=200, steps=40)]
    cases += [(f, [x if not x.startswith("-timeEnd") else "-timeEnd=0.09" for x in o])
              for f, o, _ in models.batch_c4(2, seed=92, n_max=120, steps=90)]
    cases.append((models.hinged_beam(joint_type=1, load=2000.0)[0],
                  ["-timeInc=0.001", "-timeEnd=0.07", "-tolDispNorm=1.0e-10"]))
    fsi, opts, _ = models.superelement_chain_c3(str(tmp_path), n_parts=3, n_modes=6, nx=8, ny=2, nz=2, steps=50)
    cases.append((fsi, opts))
    cases.append((models.beam_chain_fsi(30, 0.25, 0.1, 0.01, clamp=0, load_node=30, load_dof=2, load=800.0,
                                        **models.STEEL, anchors=[(7.5, 1.0, 0.0)],
                                        springs=[(30, ("anchor", 0), 2.0e5, 1.0), (12, 27, 5.0e4, 3.75, 0.002)],
                                        dampers=[(5, 18, 120.0)]),
                  ["-timeInc=0.001", "-timeEnd=0.06"]))
    with open(os.path.join(GOLDEN_DIR, "cantilever_prescribed.fsi")) as f:
        cases.append((f.read(), ["-numit=-1", "-timeInc=0.2", "-timeEnd=2.0", "-quasiStatic=1.0"]))
    mods = [Model(f, o) for f, o in cases]
    srv = Server(budget_bytes=8e9, mixed=mixed, max_models_per_batch=4, min_batch=1, max_wait=0.0)
    srv.set_max_engines(2)
    srv.slot_reuse(0.25)
    ids = [srv.submit(m) for m in mods]
    t0 = time.time()
    while any(srv.request(i)["state"] < 2 for i in ids):
        srv.pump()
        assert time.time() - t0 < 180
    assert srv.slot_reuse() >= 1  # running models were moved at least once
    for k, i in enumerate(ids):
        r = srv.request(i)
        assert r["state"] == 2, (k, r)
        alone = Batch([mods[k]], mixed=mixed)
        alone.run()
        assert np.array_equal(srv.result(i), alone.triads(0)), k
        assert r["iterations"] == alone.info(0)["iterations"], k
        alone.close()
    srv.close()
