"""Host-side set-up of the GPU solver (no GPU): element matrices, equation
numbering, sparsity pattern and symbolic factorisation, checked bit-exactly
against the oracle and for internal consistency."""
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN_DIR, ROOT


def _models():
    from fedem_gb300 import models

    out = [models.cantilever_c1()]
    for fsi, opts, _ in models.batch_c4(6, seed=11, n_max=300):
        out.append((fsi, opts))
    with open(os.path.join(GOLDEN_DIR, "cantilever_pipe.fsi")) as f:
        out.append((f.read(), ["-initEquilibrium"]))
    out.append((_frame_with_axials(), ["-timeInc=0.001", "-timeEnd=0.05"]))
    with open(os.path.join(GOLDEN_DIR, "cantilever_prescribed.fsi")) as f:
        out.append((f.read(), ["-numit=-1", "-timeInc=0.2", "-timeEnd=1.0", "-quasiStatic=1.0"]))
    # master-slave joints: a revolute hinge, a rigid joint, a pendulum on a grounded master
    out.append((models.hinged_beam(joint_type=1)[0], ["-timeInc=0.001", "-timeEnd=0.05"]))
    out.append((models.hinged_beam(joint_type=3)[0], ["-timeInc=0.001", "-timeEnd=0.05"]))
    out.append((models.pendulum()[0], ["-timeInc=0.001", "-timeEnd=0.05"]))
    return out


def _frame_with_axials():
    """Chain of 30 beams with anchors, axial springs (one with stiffness-
    proportional damping) and axial dampers across the chain and to ground."""
    from fedem_gb300 import models

    return models.beam_chain_fsi(30, 0.25, 0.1, 0.01, clamp=0, load_node=30, load_dof=2, load=800.0,
                                 **models.STEEL, anchors=[(7.5, 1.0, 0.0), (3.0, -1.0, 0.5)],
                                 springs=[(30, ("anchor", 0), 2.0e5, 1.0), (12, 27, 5.0e4, 3.75, 0.002),
                                          (20, ("anchor", 1), 1.0e5, 2.2)],
                                 dampers=[(30, ("anchor", 0), 300.0), (5, 18, 120.0)])


N_MODELS = 13


@pytest.mark.parametrize("idx", range(N_MODELS))
def test_setup_matches_oracle_bitwise(gpu_lib, oracle_lib, idx):
    from fedem_gb300.batch import Model
    from oracle.oracle import OracleModel

    fsi, opts = _models()[idx]
    m = Model(fsi, opts)
    o = OracleModel(fsi, opts)
    assert (m.ntri, m.ndof, m.neq, m.nel) == (o.ntri, o.ndof, o.neq, o.nel)
    # equation numbering (MEQN): bit-exact
    assert np.array_equal(m.meqn(), o.meqn())
    # element stiffness and mass matrices: bit-exact
    for e in range(m.nel):
        for which in (0, 1):
            assert np.array_equal(m.element_matrix(e, which), o.element_matrix(e, which)), (e, which)
    # sparsity pattern: the upper triangle of the GPU's full pattern is the oracle's pattern
    rp, ci = m.csr_pattern()
    orp, oci = o.csr_upper_pattern()
    upper_rows = [ci[rp[i]:rp[i + 1]] for i in range(m.neq)]
    for i in range(m.neq):
        r = upper_rows[i]
        assert np.array_equal(r[r >= i], oci[orp[i]:orp[i + 1]])
    # full pattern is symmetric
    a = set()
    for i in range(m.neq):
        for j in ci[rp[i]:rp[i + 1]]:
            a.add((i, int(j)))
    assert all((j, i) in a for (i, j) in a)


@pytest.mark.parametrize("idx", range(N_MODELS))
def test_symbolic_factorisation_is_consistent(gpu_lib, idx):
    from fedem_gb300.batch import Model

    fsi, opts = _models()[idx]
    m = Model(fsi, opts)
    perm, info = m.symbolic()
    assert sorted(perm.tolist()) == list(range(m.neq))
    npiv, nrow, parent, height = info[:, 0], info[:, 1], info[:, 2], info[:, 3]
    assert npiv.sum() == m.neq
    assert np.all(npiv >= 1) and np.all(nrow >= npiv)
    for f in range(m.nfront):
        if parent[f] >= 0:
            assert parent[f] > f  # post-order
            assert height[parent[f]] > height[f]
        else:
            assert nrow[f] == npiv[f]  # roots have no update rows
    assert nrow.max() == m.max_front
    assert height.max() + 1 == m.levels


def test_symbolic_is_deterministic(gpu_lib):
    from fedem_gb300 import models
    from fedem_gb300.batch import Model

    fsi, opts, _ = models.batch_c4(1, seed=3, n_min=500, n_max=600)[0]
    a, b = Model(fsi, opts), Model(fsi, opts)
    pa, ia = a.symbolic()
    pb, ib = b.symbolic()
    assert np.array_equal(pa, pb) and np.array_equal(ia, ib)


def test_nested_dissection_depth_is_logarithmic_for_chains(gpu_lib):
    from fedem_gb300 import models
    from fedem_gb300.batch import Model

    fsi, opts, n = models.batch_c4(1, seed=5, n_min=4000, n_max=4000)[0]
    m = Model(fsi, opts)
    assert m.levels <= 2 * int(np.ceil(np.log2(n))) and m.max_front <= 36


def _declared_functions():
    names = []
    for h in ("fedem_solver_core.h", "fgpu.h"):
        with open(os.path.join(ROOT, "include", h)) as f:
            text = f.read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for mt in re.finditer(r"^\s*(?!static)[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", text, flags=re.M):
            names.append(mt.group(1))
    return sorted(set(names) - {"if", "return"})


def test_library_exports_every_declared_symbol(gpu_lib):
    from fedem_gb300 import LIB_PATH

    import subprocess

    out = subprocess.run(["nm", "-D", "--defined-only", LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    declared = _declared_functions()
    assert len(declared) >= 60
    missing = [n for n in declared if n not in exported]
    assert not missing, missing


def test_fedempy_symbol_set_is_exported(gpu_lib):
    """Every symbol fedempy binds (PythonAPI/src/fedempy/solver.py:154-191) is present."""
    fedempy = ["solverInit", "restartFromState", "solveWindow", "getStateSize", "getTransformationStateSize",
               "getPartDeformationStateSize", "getPartStressStateSize", "getGagesSize", "saveState",
               "saveTransformationState", "savePartDeformationState", "savePartStressState", "saveGages",
               "solveNext", "startStep", "solveIteration", "solveEigenModes", "solveInverse", "solverDone",
               "setExtFunc", "getTime", "evalFunc", "getEquations", "getStateVar", "getSystemSize",
               "getSystemMatrix", "getElementStiffnessMatrix", "getRhsVector", "setRhsVector", "addRhsVector",
               "getBeamForcesFromDisp", "getStrainsFromDisp", "getRelDisp", "getRespVars", "getJointSprCoeff"]
    for name in fedempy:
        assert hasattr(gpu_lib, name), name
    # with the reference tree at hand, the names fedempy's own source binds
    ref = "/root/reference/PythonAPI/src/fedempy/solver.py"
    if os.path.exists(ref):
        with open(ref) as f:
            bound = set(re.findall(r"self\._solver\.(\w+)\.restype", f.read()))
        assert bound, "no bindings found in fedempy's solver.py"
        missing = sorted(n for n in bound if not hasattr(gpu_lib, n))
        assert not missing, missing


def test_invalid_model_fails_loudly(gpu_lib):
    from fedem_gb300 import FedemException
    from fedem_gb300.batch import Model

    with pytest.raises(FedemException):
        Model("&TRIAD\n id = 1\n/\n&SUP_EL\n id = 2\n numTriads = 2\n triadIds = 1 9\n/\n", [])


def test_prescribed_dofs_numbered_as_the_oracle(gpu_lib, oracle_lib):
    """A prescribed DOF gets MEQN = -ICEQ (samSolverModule.f90), the free DOFs
    are numbered around it, exactly as in the oracle."""
    from fedem_gb300.batch import Model
    from oracle.oracle import OracleModel

    with open(os.path.join(GOLDEN_DIR, "cantilever_prescribed.fsi")) as f:
        fsi = f.read()
    opts = ["-numit=-1", "-timeInc=0.2", "-timeEnd=1.0", "-quasiStatic=1.0"]
    g, o = Model(fsi, opts), OracleModel(fsi, opts)
    assert np.array_equal(g.meqn(), o.meqn())
    assert (g.meqn() < 0).sum() == 1 and g.neq == o.neq


def test_unsupported_records_fail_loudly_and_bc2_is_free(gpu_lib):
    """Input the GPU path does not implement (here a reference to an unknown
    engine, higher pairs, point-to-path joints) is refused with a message
    instead of being dropped; BC code 2 counts as a free DOF when the initial
    equilibrium iterations are off (initiateTriadTypeModule.f90:57-123)."""
    from fedem_gb300 import FedemException, models
    from fedem_gb300.batch import Model

    base = models.beam_chain_fsi(4, 1.0, 0.1, 0.01, clamp=0, load_node=4, load_dof=2, load=10.0, **models.STEEL)
    with pytest.raises(FedemException, match="unknown engine"):
        Model(base.replace("  f0 =", "  loadEngineId = 7\n  f0 ="), [])
    with pytest.raises(FedemException, match="HIGHER_PAIR|higher_pair"):
        Model(base + "&HIGHER_PAIR\n  id = 99\n/\n", [])
    with pytest.raises(FedemException, match="joints"):  # point-to-path joint types
        Model(base + "&MASTERSLAVEJOINT\n  id = 99\n  type = 6\n  slaveId = 5\n  masterId = 4\n/\n", [])
    free = Model(base, [])
    bc2 = Model(base.replace("&TRIAD\n  id = 5\n  nDOFs = 6\n", "&TRIAD\n  id = 5\n  nDOFs = 6\n  BC = 2 2 2 2 2 2\n"), [])
    assert bc2.neq == free.neq
    with pytest.raises(FedemException):
        Model(base.replace("&TRIAD\n  id = 5\n  nDOFs = 6\n", "&TRIAD\n  id = 5\n  nDOFs = 6\n  BC = 2 2 2 2 2 2\n"),
              ["-initEquilibrium"])


def test_external_function_records():
    """DEVICE_FUNCTION without a file is an external function (setExtFunc
    channel); with a file, or without a channel, the model is refused."""
    from fedem_gb300 import FedemException, models
    from fedem_gb300.batch import Model

    fsi = models.beam_chain_fsi(4, 0.25, 0.1, 0.01, clamp=0, load_node=4, load_dof=2, load=10.0,
                                load_ext=(2, 5, "tip"), **models.STEEL)
    Model(fsi, ["-timeInc=0.01", "-timeEnd=0.1"]).close()
    with pytest.raises(FedemException, match="file"):
        Model(fsi.replace("fileName = ''", "fileName = 'inputs.asc'"), ["-timeInc=0.01", "-timeEnd=0.1"])
    with pytest.raises(FedemException, match="channel"):
        Model(fsi.replace("channel = 2", "channel = 0"), ["-timeInc=0.01", "-timeEnd=0.1"])


@pytest.mark.parametrize("opt", ["-cutbackFactor=0.5", "-cutbackSing", "-lineSearch", "-stressStiffDyn",
                                 "-stressStiffEqu+", "-centripForceCorr", "-NewmarkFlag=100",
                                 "-tolUpdateFactor=10.0"])
def test_result_changing_options_are_refused(gpu_lib, opt):
    """Options that change the results and that this path does not implement
    (iteration cut-back, line search, geometric stiffness, centripetal
    correction, Newmark variants, tangent updates by tolerance) fail model
    creation with a message instead of being ignored; their defaults pass."""
    from fedem_gb300 import FedemException, models
    from fedem_gb300.batch import Model

    base = models.beam_chain_fsi(4, 1.0, 0.1, 0.01, clamp=0, load_node=4, load_dof=2, load=10.0, **models.STEEL)
    with pytest.raises(FedemException, match="not supported"):
        Model(base, ["-timeInc=0.01", opt])
    Model(base, ["-timeInc=0.01", "-cutbackFactor=1.0", "-lineSearch-", "-NewmarkFlag=0",
                 "-tolUpdateFactor=0.0"]).close()


def test_part_setup_matches_oracle(gpu_lib, oracle_lib, tmp_path):
    """Reduced parts (matrix files, generalized DOFs, revolute joints between
    them): the GPU host set-up numbers the generalized DOFs after the triads
    and before the joint DOFs as the oracle does, with the same sparsity
    pattern."""
    from fedem_gb300 import models
    from fedem_gb300.batch import Model
    from oracle.oracle import OracleModel

    fsi, opts, _ = models.superelement_chain_c3(str(tmp_path), n_parts=4, n_modes=8, nx=8, ny=2, nz=2, steps=10)
    m = Model(fsi, opts)
    o = OracleModel(fsi, opts)
    assert (m.ntri, m.ndof, m.neq) == (o.ntri, o.ndof, o.neq)
    assert np.array_equal(m.meqn(), o.meqn())
    rp, ci = m.csr_pattern()
    orp, oci = o.csr_upper_pattern()
    for i in range(m.neq):
        r = ci[rp[i]:rp[i + 1]]
        assert np.array_equal(r[r >= i], oci[orp[i]:orp[i + 1]])


def test_part_files_are_checked(gpu_lib, tmp_path):
    """A missing or mistagged part matrix file fails model creation loudly."""
    from fedem_gb300 import FedemException, models, reducer
    from fedem_gb300.batch import Model

    fsi, opts, info = models.superelement_chain_c3(str(tmp_path), n_parts=2, n_modes=4, nx=4, ny=2, nz=2, steps=10)
    bad = str(tmp_path / "bad_M.fmx")
    reducer.write_fmx(bad, "stiffness matrix", info["Mr"])
    with pytest.raises(FedemException, match="mass matrix"):
        Model(fsi.replace(info["files"]["M"], bad), opts)
    with pytest.raises(FedemException, match="cannot open"):
        Model(fsi.replace(info["files"]["K"], str(tmp_path / "none.fmx")), opts)
