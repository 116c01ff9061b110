"""Reduced parts (superelements with component modes) on the GPU path
against the oracle: FP64 within 1e-10 and mixed precision within 1e-8 of the
largest displacement over the run, equal FP64 iteration counts; a part that
holds a beam's own matrices equals the beam element; damped beams (Rayleigh
damping with the rigid-body filtering of the stiffness-proportional part)
against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1.0e-10
MIXED_TOL = 1.0e-8


def _oracle_run(fsi, opts):
    from oracle.oracle import OracleModel

    o = OracleModel(fsi, opts)
    o.run_all()
    out = o.triads().copy(), o.iterations(), o.max_displacement()
    o.close()
    return out


def _gpu_run(fsi, opts, mixed):
    from fedem_gb300.batch import Batch, Model

    m = Model(fsi, opts)
    b = Batch([m], mixed=mixed)
    st = b.run()
    assert st["models_done"] == 1 and st["models_failed"] == 0, b.info(0)
    out = b.triads(0).copy(), b.info(0)["iterations"]
    b.close()
    m.close()
    return out


def _check(fsi, opts, mixed):
    ref, iters, scale = _oracle_run(fsi, opts)
    ur, it = _gpu_run(fsi, opts, mixed)
    err = np.abs(ur[:, :, 3] - ref[:, :, 3]).max() / scale
    assert err <= (MIXED_TOL if mixed else FP64_TOL), err
    if not mixed:
        assert it == iters
    return err


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_superelement_chain_matches_oracle(gpu, oracle_lib, tmp_path, mixed):
    """16 Craig-Bampton parts (42 x 42), 15 revolute joints, gravity, harmonic end torque."""
    from fedem_gb300 import models

    fsi, opts, _ = models.superelement_chain_c3(str(tmp_path), steps=200)
    _check(fsi, opts, mixed)


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_damped_beams_match_oracle(gpu, oracle_lib, mixed):
    """Rayleigh-damped beams: the stiffness-proportional part is filtered of
    rigid-body motion in the predictor and the corrector passes."""
    from fedem_gb300 import models

    fsi = models.beam_chain_fsi(20, 0.25, 0.1, 0.01, clamp=0, load_node=20, load_dof=2, load=1500.0,
                                **models.STEEL)
    fsi = fsi.replace("  elPropId = 1\n", "  elPropId = 1\n  alpha1 = 0.5\n  alpha2 = 3.0e-4\n")
    _check(fsi, ["-timeInc=0.001", "-timeEnd=0.3", "-alphaNewmark=0.1", "-tolDispNorm=1.0e-10"], mixed)


def test_part_with_beam_matrices_equals_the_beam(gpu, oracle_lib, tmp_path):
    """A chain of parts whose files hold the beam elements' own K, M and
    gravity force vectors runs like the beam chain (damped, under gravity)."""
    from fedem_gb300 import models, reducer
    from oracle.oracle import OracleModel

    fsi = models.beam_chain_fsi(6, 0.5, 0.1, 0.01, clamp=0, load_node=6, load_dof=3, load=-2000.0,
                                shear_factor=0.5, **models.STEEL)
    fsi = fsi.replace("  elPropId = 1\n", "  elPropId = 1\n  alpha1 = 0.3\n  alpha2 = 2.0e-4\n")
    fsi += "&ENVIRONMENT\n  gravity = 0.0 0.0 -9.81\n/\n"
    opts = ["-timeInc=0.001", "-timeEnd=0.15", "-tolDispNorm=1.0e-10"]
    o = OracleModel(fsi, opts)
    K, M = o.element_matrix(0, 0), o.element_matrix(0, 1)
    o.close()
    paths = {}
    for k, a in (("K", K), ("M", M), ("G", M[:, 0:3] + M[:, 6:9])):
        paths[k] = str(tmp_path / f"beam_{k}.fmx")
        reducer.write_fmx(paths[k], reducer.FMX_TAGS[k], a)
    files = " ".join(f"'{paths[k]}'" for k in ("K", "M", "G"))
    part = fsi.replace("  elPropId = 1\n", f"  numGenDOFs = 0\n  inputFiles = {files}\n")
    ub, ib = _gpu_run(fsi, opts, False)
    up, ip = _gpu_run(part, opts, False)
    scale = np.abs(ub[:, :, 3] - ub[:, :, 3][0]).max()
    assert ib == ip
    assert np.abs(ub - up).max() <= 1.0e-12 * max(scale, 1.0)


def test_parts_batched_with_beams_same_as_alone(gpu, tmp_path):
    """A superelement chain batched with beam models gives bitwise its standalone result."""
    from fedem_gb300 import models
    from fedem_gb300.batch import Batch, Model

    fsi, opts, _ = models.superelement_chain_c3(str(tmp_path), n_parts=4, steps=60)
    cases = [(fsi, opts)] + [(f, o) for f, o, _ in models.batch_c4(3, seed=7, n_max=150, steps=60)]
    mix = Batch([Model(f, o) for f, o in cases], mixed=True)
    mix.run()
    alone = Batch([Model(fsi, opts)], mixed=True)
    alone.run()
    np.testing.assert_array_equal(mix.triads(0), alone.triads(0))
    mix.close()
    alone.close()


def _tilted():
    """A rotation turning global X away from every global axis."""
    a, b = np.radians(30.0), np.radians(20.0)
    Rz = np.array([[np.cos(a), -np.sin(a), 0.0], [np.sin(a), np.cos(a), 0.0], [0.0, 0.0, 1.0]])
    Ry = np.array([[np.cos(b), 0.0, np.sin(b)], [0.0, 1.0, 0.0], [-np.sin(b), 0.0, np.cos(b)]])
    return Ry @ Rz


@pytest.mark.parametrize("tilt", [False, True], ids=["along_x", "tilted"])
def test_part_newton_matrix_matches_oracle(gpu, oracle_lib, tmp_path, tilt):
    """The predictor's Newton matrix of a superelement chain (parts expanded
    through the revolute joints' constraint equations, part frames along the
    global axes or tilted) equals the oracle's assembly."""
    from fedem_gb300 import models
    from fedem_gb300.batch import Batch, Model
    from oracle.oracle import OracleModel

    fsi, opts, _ = models.superelement_chain_c3(str(tmp_path), n_parts=3, n_modes=6, nx=8, ny=2, nz=2, steps=10,
                                                axes=_tilted() if tilt else None)
    o = OracleModel(fsi, opts)
    beta, gamma, dt, alpha = 0.3025, 0.6, 5.0e-4, -0.1
    sM, sK = 1.0 / (beta * dt * dt), 1.0 + alpha
    rp_u, ci_u, v_u = o.newton_upper(sM, gamma / (beta * dt) * sK, sK)
    m = Model(fsi, opts)
    b = Batch([m])
    b.step(0)
    vals = b.newton_values(0)
    rp, ci = m.csr_pattern()
    dense_gpu = np.zeros((m.neq, m.neq))
    for i in range(m.neq):
        dense_gpu[i, ci[rp[i]:rp[i + 1]]] = vals[rp[i]:rp[i + 1]]
    dense_ref = np.zeros((m.neq, m.neq))
    for i in range(m.neq):
        dense_ref[i, ci_u[rp_u[i]:rp_u[i + 1]]] = v_u[rp_u[i]:rp_u[i + 1]]
    dense_ref = np.triu(dense_ref) + np.triu(dense_ref, 1).T
    scale = np.abs(dense_ref).max()
    # entry by entry: the mass terms of the generalized DOFs are far larger
    # than the torsional and coupling entries, so a bound on the largest entry
    # alone would hide errors in those
    # (1e-14 of the largest entry is the rounding floor of the cancelling sums)
    excess = np.abs(dense_gpu - dense_ref) - (1e-11 * np.abs(dense_ref) + 1e-14 * scale)
    i, j = np.unravel_index(np.argmax(excess), excess.shape)
    assert excess.max() <= 0.0, (i, j, dense_gpu[i, j], dense_ref[i, j], scale)
    assert np.array_equal(dense_gpu, dense_gpu.T)
    b.close()
    o.close()
