"""Master-slave joints in the oracle, pinned to beam theory and rigid-body
dynamics (the reference's own tests hold no joint model).

- A revolute joint about Z in a beam clamped at one end and pinned at the
  other releases the bending moment there (a Gerber beam): a transverse load
  at the hinge is carried by the left cantilever alone, deflection P a^3/3EI.
- A rigid joint at the same place makes it a continuous propped cantilever:
  7 P L^3 / 768 EI under the mid-span load, and the same response, static and
  dynamic, as the model without the joint.
- A pipe hanging from a revolute joint swings with the period of a physical
  pendulum, 2 pi sqrt(2 L / 3 g) (1 + theta0^2 / 16).
Constraint semantics: masterSlaveJointRoutinesModule.f90:218-577 (slave
placement, constraint coefficients), samSolverModule.f90:581-860 (dependent
DOFs), sysMatrixTypeModule.f90:2099-2259 (assembly through the constraints).
"""
import numpy as np
import pytest

STATIC = ["-initEquilibrium", "-tolInitEquil=1.0e-12", "-timeInc=0.001", "-timeEnd=0.001"]


def _ei():
    from fedem_gb300 import models

    return 2.1e11 * models.pipe_section(0.1, 0.01)[1]


def _continuous(n=16, el_len=0.25, load=10.0, load_triad=9):
    """The hinged beam's geometry without the joint: one chain, clamped at
    x = 0, pinned at the end, load in Y at load_triad."""
    from fedem_gb300 import models

    triads = [{"id": k + 1, "pos": (k * el_len, 0.0, 0.0),
               "bc": [0] * 6 if k == 0 else ([0, 0, 0, 1, 1, 1] if k == n else None)} for k in range(n + 1)]
    beams = [(1000 + k, k + 1, k + 2, 1) for k in range(n)]
    return models.frame_fsi(triads, beams, [models.pipe_props(1, 0.1, 0.01)], loads=[(load_triad, 2, load)])


def test_revolute_hinge_releases_the_moment(oracle_lib):
    from fedem_gb300 import models
    from oracle.oracle import OracleModel

    fsi, master, slave = models.hinged_beam(joint_type=1, load=10.0)
    o = OracleModel(fsi, STATIC)
    y = o.state_var(master)[1]
    theory = 10.0 * 2.0 ** 3 / (3.0 * _ei())
    assert abs(y / theory - 1.0) < 1.0e-5, (y, theory)
    # the slave triad sits on the master (joint at the hinge point)
    assert np.allclose(o.state_var(slave), o.state_var(master), rtol=0, atol=1e-14)
    o.close()


def test_rigid_joint_is_a_continuous_beam(oracle_lib):
    from fedem_gb300 import models
    from oracle.oracle import OracleModel

    fsi, master, slave = models.hinged_beam(joint_type=3, load=10.0)
    o = OracleModel(fsi, STATIC)
    c = OracleModel(_continuous(), STATIC)
    y = o.state_var(master)[1]
    theory = 7.0 * 10.0 * 4.0 ** 3 / (768.0 * _ei())
    assert abs(y / theory - 1.0) < 1.0e-5, (y, theory)
    assert abs(y - c.state_var(9)[1]) <= 1.0e-10 * abs(y)
    o.close()
    c.close()


def test_rigid_joint_dynamics_equal_the_continuous_beam(oracle_lib):
    from fedem_gb300 import models
    from oracle.oracle import OracleModel

    opts = ["-timeInc=0.001", "-timeEnd=0.1", "-tolDispNorm=1.0e-12"]
    fsi, master, _ = models.hinged_beam(joint_type=3, load=2000.0)
    o = OracleModel(fsi, opts)
    c = OracleModel(_continuous(load=2000.0), opts)
    ho, hc = [], []
    while o.solve_next():
        c.solve_next()
        ho.append(o.state_var(master))
        hc.append(c.state_var(9))
    ho, hc = np.array(ho), np.array(hc)
    assert len(ho) == 99
    err = np.abs(ho - hc).max() / np.abs(hc[:, 1]).max()
    assert err < 1.0e-9, err
    o.close()
    c.close()


def test_pendulum_period(oracle_lib):
    from fedem_gb300 import models
    from oracle.oracle import OracleModel

    L, th0 = 1.0, 0.1
    fsi, tip = models.pendulum(length=L, theta0=th0)
    o = OracleModel(fsi, ["-timeInc=0.001", "-timeEnd=3.5", "-tolDispNorm=1.0e-10"])
    xs = []
    while o.solve_next():
        xs.append(o.state_var(tip)[0])
    o.close()
    x = np.array(xs)
    t = 0.001 * np.arange(1, len(x) + 1)
    i = np.where(np.sign(x[:-1]) != np.sign(x[1:]))[0]
    tc = t[i] - x[i] * 0.001 / (x[i + 1] - x[i])
    T = 2.0 * (tc[-1] - tc[0]) / (len(tc) - 1)
    T0 = 2.0 * np.pi * np.sqrt(2.0 * L / (3.0 * 9.81)) * (1.0 + th0 ** 2 / 16.0)
    assert len(tc) >= 4 and abs(T / T0 - 1.0) < 1.0e-4, (T, T0)
    assert abs(x.max() - L * np.sin(th0)) < 1e-3  # no energy gained or lost in two swings


@pytest.mark.parametrize("bad, msg", [
    ("  type = 1\n", "  type = 6\n"),  # point-to-path joint types
    ("  nJointVars = 1\n", "  nJointVars = 1\n  springId = 7\n"),  # joint springs
])
def test_unsupported_joint_input_is_refused(oracle_lib, bad, msg):
    from fedem_gb300 import models
    from oracle.oracle import OracleModel

    fsi, _, _ = models.hinged_beam(joint_type=1)
    with pytest.raises(RuntimeError):
        OracleModel(fsi.replace(bad, msg), STATIC)
