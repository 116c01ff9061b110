"""The linear-solver seam of one model (fgpu_batch_assemble_newton / _factor /
_solve: csAddEM + csSolve granularity, asmExtensionModule.f90:1227,
solExtensionModule.f90:153-505): the Newton matrix assembled on the GPU
matches the oracle's assembly, its factorisation solves N x = b like a dense
solve (FP64 within 1e-10, mixed precision with refinement within 1e-8),
negative pivots are counted, a singular matrix is reported as -3, and using
the seam between steps leaves the model's stepping bitwise unchanged."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _chain(clamp=0, n=24):
    from fedem_gb300 import models

    fsi = models.beam_chain_fsi(n, 0.25, 0.1, 0.01, clamp=clamp, load_node=n, load_dof=2, load=1200.0,
                                **models.STEEL)
    return fsi, ["-timeInc=0.001", "-timeEnd=0.02", "-alphaNewmark=0.1", "-tolDispNorm=1.0e-10"]


def _dense(m, vals):
    rp, ci = m.csr_pattern()
    a = np.zeros((m.neq, m.neq))
    for i in range(m.neq):
        a[i, ci[rp[i]:rp[i + 1]]] = vals[rp[i]:rp[i + 1]]
    return a


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_assembly_factor_and_solve(gpu, oracle_lib, mixed):
    from fedem_gb300.batch import Batch, Model
    from oracle.oracle import OracleModel

    fsi, opts = _chain()
    m = Model(fsi, opts)
    b = Batch([m], mixed=mixed)
    sM, sC, sK = 3.0e6, 0.0, 0.9
    b.assemble_newton(0, sM, sC, sK)
    n_gpu = _dense(m, b.newton_values(0))
    # the oracle's assembly of the same matrix (upper triangle)
    o = OracleModel(fsi, opts)
    rp_u, ci_u, v_u = o.newton_upper(sM, sC, sK)
    ref = np.zeros_like(n_gpu)
    for i in range(m.neq):
        ref[i, ci_u[rp_u[i]:rp_u[i + 1]]] = v_u[rp_u[i]:rp_u[i + 1]]
    ref = np.triu(ref) + np.triu(ref, 1).T
    assert np.abs(n_gpu - ref).max() <= 1e-13 * np.abs(ref).max()
    assert b.factor(0) == 0  # positive definite: no negative pivots
    rng = np.random.default_rng(11)
    rhs = rng.standard_normal((3, m.neq))
    x = b.solve(0, rhs)
    xd = np.linalg.solve(ref, rhs.T).T
    tol = 1e-8 if mixed else 1e-10
    assert np.abs(x - xd).max() <= tol * np.abs(xd).max()
    o.close()


def test_negative_pivots_and_singular(gpu):
    from fedem_gb300 import FedemException
    from fedem_gb300.batch import Batch, Model

    fsi, opts = _chain()
    m = Model(fsi, opts)
    b = Batch([m])
    b.assemble_newton(0, 0.0, 0.0, -1.0)  # -K: every pivot negative
    assert b.factor(0) == m.neq
    # an unclamped chain: K alone is singular (rigid-body motions)
    fsi2, opts2 = _chain(clamp=-1)
    m2 = Model(fsi2, opts2)
    b2 = Batch([m2])
    b2.assemble_newton(0, 0.0, 0.0, 1.0)
    with pytest.raises(FedemException):
        b2.factor(0)


def test_stepping_unchanged_by_the_seam(gpu):
    from fedem_gb300.batch import Batch, Model

    fsi, opts = _chain()
    ref = Batch([Model(fsi, opts)])
    ref.run()
    b = Batch([Model(fsi, opts)])
    b.run(max_batched=5)
    while b.info(0)["state"] == 1:  # to the end of the current step
        b.run(max_batched=1)
    b.assemble_newton(0, 1.0, 0.0, 1.0)
    b.factor(0)
    b.solve(0, np.ones(b.models[0].neq))
    b.run()
    np.testing.assert_array_equal(b.triads(0), ref.triads(0))
    assert b.info(0)["iterations"] == ref.info(0)["iterations"]
