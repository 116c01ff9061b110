"""Reduced superelements (parts with component modes, matrices read from
binary matrix files) in the oracle, pinned to things outside it:

1. A part whose files hold a beam element's own K, M and gravity force
   vectors (no component modes) gives the beam model's results bitwise, in
   statics and in damped dynamics under gravity: the part path (ReadSupEls
   with inputFiles, initiateSupElTypeModule.f90:493-540, 962-1033) equals the
   beam path already pinned to the reference's goldens.
2. A Craig-Bampton reduced hex block (2 x 0.2 x 0.2 m, 40 x 4 x 4 elements,
   30 component modes) clamped at its first triad: the static tip deflection
   under a small tip load equals the full hexahedral model's solution with
   the same rigid face ties (the constraint modes reproduce static boundary
   loads exactly).
3. The same block's free vibration after a step load: the period measured
   from the oracle's time history equals the full model's first bending
   eigenfrequency within 0.5 %.
4. Matrix files with the wrong tag or size are refused at set-up.
"""
import numpy as np
import pytest

STATIC = ["-initEquilibrium", "-tolInitEquil=1.0e-12", "-timeInc=0.001", "-timeEnd=0.001"]


def _beam_vs_part(tmp_path, opts):
    from fedem_gb300 import models, reducer
    from oracle.oracle import OracleModel

    fsi = models.beam_chain_fsi(6, 0.5, 0.1, 0.01, clamp=0, load_node=6, load_dof=3, load=-2000.0,
                                shear_factor=0.5, **models.STEEL)
    fsi = fsi.replace("  elPropId = 1\n", "  elPropId = 1\n  alpha1 = 0.3\n  alpha2 = 2.0e-4\n")
    fsi += "&ENVIRONMENT\n  gravity = 0.0 0.0 -9.81\n/\n"
    o = OracleModel(fsi, opts)
    K, M = o.element_matrix(0, 0), o.element_matrix(0, 1)
    fg = M[:, 0:3] + M[:, 6:9]
    paths = {}
    for k, a in (("K", K), ("M", M), ("G", fg)):
        paths[k] = str(tmp_path / f"beam_{k}.fmx")
        reducer.write_fmx(paths[k], reducer.FMX_TAGS[k], a)
    files = " ".join(f"'{paths[k]}'" for k in ("K", "M", "G"))
    part = fsi.replace("  elPropId = 1\n", f"  numGenDOFs = 0\n  inputFiles = {files}\n")
    assert part.count("inputFiles") == 6
    p = OracleModel(part, opts)
    return o, p


def test_part_with_beam_matrices_is_the_beam_statics(oracle_lib, tmp_path):
    o, p = _beam_vs_part(tmp_path, STATIC)
    np.testing.assert_array_equal(o.triads(), p.triads())
    assert abs(o.state_var(7)[2]) > 1e-3
    o.close()
    p.close()


def test_part_with_beam_matrices_is_the_beam_dynamics(oracle_lib, tmp_path):
    o, p = _beam_vs_part(tmp_path, ["-timeInc=0.001", "-timeEnd=0.15", "-tolDispNorm=1.0e-10"])
    n = 0
    while o.solve_next():
        assert p.solve_next()
        n += 1
        np.testing.assert_array_equal(o.triads(), p.triads())
    assert not p.solve_next()  # the last step (solveNext returns false after it)
    np.testing.assert_array_equal(o.triads(), p.triads())
    assert n == 149 and o.iterations() == p.iterations()
    o.close()
    p.close()


# ---- a reduced hex block against the full hexahedral model ---------------------------
def _block_model(tmp_path, load, opts, n_modes=30):
    from fedem_gb300 import models, reducer

    paths, red = reducer.block_part_files(str(tmp_path), n_modes=n_modes)
    triads = [{"id": 1, "pos": (0.0, 0.0, 0.0), "bc": [0] * 6}, {"id": 2, "pos": (2.0, 0.0, 0.0)}]
    fsi = models.frame_fsi(triads, [], [], loads=[(2, 3, load)], title="block")
    fsi += models.part_records(10, [1, 2], (0.0, 0.0, 0.0), paths, n_modes, [(0, 0, 0), (2.0, 0, 0)],
                               ref_offset=2.0)
    return fsi, red


def _full_block_tip_system():
    """Full hex model, face x = 0 fixed, face x = 2 tied rigidly to a triad at
    its centre: (K, M) over [triad DOFs (6), interior DOFs]."""
    import scipy.sparse as sp

    from fedem_gb300 import reducer

    K, M, c = reducer.hex_block()
    nn = len(c)
    fa = np.abs(c[:, 0]) < 1e-9
    fb = np.abs(c[:, 0] - 2.0) < 1e-9
    interior = np.where(~(fa | fb))[0]
    rows, cols, vals = [], [], []
    for node in np.where(fb)[0]:
        r = c[node] - np.array([2.0, 0.0, 0.0])
        S = np.array([[0.0, -r[2], r[1]], [r[2], 0.0, -r[0]], [-r[1], r[0], 0.0]])
        for a in range(3):
            rows.append(3 * node + a), cols.append(a), vals.append(1.0)
            for b in range(3):
                if S[a, b] != 0.0:
                    rows.append(3 * node + a), cols.append(3 + b), vals.append(-S[a, b])
    idof = (3 * interior[:, None] + np.arange(3)).ravel()
    rows += idof.tolist()
    cols += (6 + np.arange(len(idof))).tolist()
    vals += [1.0] * len(idof)
    T = sp.coo_matrix((vals, (rows, cols)), shape=(3 * nn, 6 + len(idof))).tocsr()
    return (T.T @ K @ T).tocsc(), (T.T @ M @ T).tocsc()


def test_reduced_block_statics_equal_the_full_model(oracle_lib, tmp_path):
    import scipy.sparse.linalg as sla

    from oracle.oracle import OracleModel

    load = 10.0
    fsi, _ = _block_model(tmp_path, load, STATIC)
    o = OracleModel(fsi, STATIC)
    w = o.state_var(2)[2]
    Kf, _ = _full_block_tip_system()
    f = np.zeros(Kf.shape[0])
    f[2] = load
    u = sla.spsolve(Kf, f)
    assert abs(w / u[2] - 1.0) < 1.0e-6, (w, u[2])
    o.close()


def test_reduced_block_period_equals_the_full_model(oracle_lib, tmp_path):
    import scipy.sparse.linalg as sla

    from oracle.oracle import OracleModel

    load, dt, steps = 10.0, 2.0e-4, 600
    opts = [f"-timeInc={dt!r}", f"-timeEnd={steps * dt!r}", "-alphaNewmark=0.1", "-tolDispNorm=1.0e-12"]
    fsi, _ = _block_model(tmp_path, load, opts)
    o = OracleModel(fsi, opts)
    ws = []
    while o.solve_next():
        ws.append(o.state_var(2)[2])
    ws.append(o.state_var(2)[2])
    o.close()
    Kf, Mf = _full_block_tip_system()
    f = np.zeros(Kf.shape[0])
    f[2] = load
    static = sla.spsolve(Kf, f)[2]
    w2 = sla.eigsh(Kf, k=2, M=Mf, sigma=0.0, which="LM", return_eigenvectors=False)
    T1 = 2.0 * np.pi / np.sqrt(np.min(w2))
    y = np.array(ws) - static
    t = dt * np.arange(1, len(y) + 1)
    up = np.where((y[:-1] < 0.0) & (y[1:] >= 0.0))[0]
    tc = t[up] - y[up] * dt / (y[up + 1] - y[up])
    assert len(tc) >= 4
    T = (tc[-1] - tc[0]) / (len(tc) - 1)
    assert abs(T / T1 - 1.0) < 5.0e-3, (T, T1)


@pytest.mark.parametrize("which", ["tag", "size"])
def test_bad_matrix_files_are_refused(oracle_lib, tmp_path, which):
    from fedem_gb300 import reducer
    from oracle.oracle import OracleModel

    fsi, red = _block_model(tmp_path, 1.0, STATIC)
    bad = str(tmp_path / "bad_K.fmx")
    if which == "tag":
        reducer.write_fmx(bad, "mass matrix", red[0])
    else:
        reducer.write_fmx(bad, "stiffness matrix", red[0][:-1, :-1])
    fsi = fsi.replace(str(tmp_path / "block_K.fmx"), bad)
    with pytest.raises(RuntimeError):
        OracleModel(fsi, STATIC)
