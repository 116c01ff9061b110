"""Results database of the primary response (the reference's writeSolverDB1,
src/vpmSolver/saveModule.f90:615-663): one file per model with a record of the
initial configuration and one per completed time step -- step, time, triad
position matrices, beam frames, reduced parts' frames and generalized DOFs.
Checked against the CPU oracle step by step (FP64 within 1e-10 of the largest
displacement over the run), against the batch's own final state bitwise, for
the single-precision form, and for a chain of reduced parts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1.0e-10


def _cases():
    from fedem_gb300 import models

    c1 = models.cantilever_c1()
    c1 = (c1[0], [o if not o.startswith("-timeEnd") else "-timeEnd=0.05" for o in c1[1]])
    return [c1] + [(f, o) for f, o, _ in models.batch_c4(2, seed=23, n_max=120, steps=40)]


def test_records_follow_every_step_and_match_the_oracle(gpu, oracle_lib, tmp_path):
    from fedem_gb300.batch import Batch, Model
    from fedem_gb300.results import read_results
    from oracle.oracle import OracleModel

    cases = _cases()
    b = Batch([Model(f, o) for f, o in cases], mixed=False)
    b.results_open(tmp_path)
    b.run()
    b.results_close()
    for k, (f, o) in enumerate(cases):
        r = read_results(tmp_path / f"model{k}.res")
        info = b.info(k)
        nrec = len(r["steps"])
        assert nrec == info["steps"] + 1
        np.testing.assert_array_equal(r["steps"], np.arange(nrec))
        assert r["times"][0] == 0.0 and np.all(np.diff(r["times"]) > 0.0)
        assert abs(r["times"][-1] - info["time"]) < 1e-12
        pos = r["triad_positions"]
        np.testing.assert_array_equal(pos[-1], b.triads(k))  # the final state, bit for bit
        # step by step against the oracle
        orc = OracleModel(f, o)
        np.testing.assert_allclose(pos[0], orc.triads(), rtol=0.0, atol=1e-14)  # initial configuration
        steps = [orc.triads()]
        while orc.solve_next():
            steps.append(orc.triads())
        steps.append(orc.triads())
        scale = orc.max_displacement()
        ref = np.stack(steps[:nrec])
        err = np.abs(pos[:, :, :, 3] - ref[:, :, :, 3]).max() / scale
        assert err <= FP64_TOL, (k, err)
        # one beam frame per element in every record
        assert r["beam_frames"].shape == (nrec, orc.nel, 3, 4)
        orc.close()
    b.close()


def test_single_precision_records(gpu, tmp_path):
    from fedem_gb300.batch import Batch, Model
    from fedem_gb300.results import read_results

    cases = _cases()[:2]
    d64, d32 = tmp_path / "d", tmp_path / "s"
    d64.mkdir()
    d32.mkdir()
    outs = []
    for d, dbl in ((d64, True), (d32, False)):
        b = Batch([Model(f, o) for f, o in cases], mixed=True)
        b.results_open(d, double=dbl)
        b.run()
        b.close()  # closes the database too
        outs.append([read_results(d / f"model{k}.res") for k in range(len(cases))])
    for a, s in zip(*outs):
        assert a["precision"] == "double" and s["precision"] == "single"
        np.testing.assert_array_equal(a["steps"], s["steps"])
        np.testing.assert_array_equal(a["values"].astype(np.float32).astype(np.float64), s["values"])


def test_reduced_parts_records(gpu, tmp_path):
    from fedem_gb300 import models
    from fedem_gb300.batch import Batch, Model
    from fedem_gb300.results import read_results

    fsi, opts, _ = models.superelement_chain_c3(str(tmp_path), n_parts=3, n_modes=6, nx=8, ny=2, nz=2, steps=20)
    b = Batch([Model(fsi, opts)], mixed=False)
    b.results_open(tmp_path)
    b.run()
    b.results_close()
    r = read_results(tmp_path / "model0.res")
    parts = [s for s in r["supels"] if s[0] == "part"]
    assert len(parts) == 3 and all(s[2] == 6 for s in parts)
    assert len(r["steps"]) == b.info(0)["steps"] + 1
    nt = len(r["triads"])
    ntv = sum(12 if kind == "position" else 3 for _, kind in r["triads"])
    assert r["values"].shape[1] == ntv + 3 * (12 + 6)
    # the triads' translations at the end equal the batch's final state
    last = r["values"][-1]
    tri = b.triads(0)
    off = 0
    for t, (_, kind) in enumerate(r["triads"]):
        if kind == "position":
            np.testing.assert_array_equal(last[off:off + 12].reshape(4, 3).T, tri[t])
            off += 12
        else:
            off += 3
    assert nt == tri.shape[0]
    b.close()


def test_frs1file_through_the_solver_abi(gpu, tmp_path):
    """The reference's own options on solverInit: -frs1file names the primary
    response database, -savestart skips the states before that time
    (solverModule.f90:352, solverRoutinesModule.f90:590-592); the records equal
    the triad positions getStateVar reports after each step."""
    from fedem_gb300 import models
    from fedem_gb300.results import read_results
    from fedem_gb300.solver import FedemSolver

    n_el = 16
    fsi = models.beam_chain_fsi(n_el, 0.25, 0.1, 0.01, clamp=0, load_node=n_el, load_dof=2, load=1500.0,
                                **models.STEEL)
    path = tmp_path / "primary.frs"
    opts = ["-timeInc=0.001", "-timeEnd=0.03", "-alphaNewmark=0.1", "-tolDispNorm=1.0e-10",
            f"-frs1file={path}", "-savestart=0.01"]
    s = FedemSolver(solver_options=opts, fsi=fsi)
    hist = []
    while s.solve_next():
        hist.append(np.array([s.get_state_var(t + 1) for t in range(n_el + 1)]))
    hist.append(np.array([s.get_state_var(t + 1) for t in range(n_el + 1)]))
    assert s.ierr.value == 0
    s.solver_done()
    r = read_results(path)
    assert r["precision"] == "double"
    np.testing.assert_array_equal(r["steps"], np.arange(10, 31))
    assert abs(r["times"][0] - 0.01) < 1e-12
    pos = r["triad_positions"][:, :, :, 3]
    for k, step in enumerate(r["steps"]):
        np.testing.assert_array_equal(pos[k], hist[step - 1])
