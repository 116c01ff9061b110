"""Writes the golden fixtures of the reference's own solver unit test.

Source: src/vpmSolver/vpmSolverTests/test_solver.C:93-262 and its models
cantilever-pipe.fsi / cantilever-noshear.fsi / cantilever-prescribed.fsi: a
10 m cantilever along Z made of five 2 m beams (A = 1.5394e-2,
Iy = Iz = 4.622e-4, It = 9.244e-4, shear factor 2 or 0, steel), clamped at
Z = 0 with a 1e5 N X-load at the tip, or (prescribed) with the tip X
deflection prescribed to 1.0 * time and solved as pure linear quasi-static
load steps.  The models are re-written here with this project's own
generator (same geometry, properties, load and motion; triad ids 1..6 along
the beam, so the reference's triad 25 at Z = 6 is triad 4 and its tip triad
17 is triad 6), and the expected positions are the reference test's values
with its tolerance.  A case lists the checked triads; each expected row
holds their (x, y, z) one after the other, the first row at the start time
unless "first_step" is 1.

Run:  python tests/golden/make_golden.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "fedem-solvers_gb300"))

from fedem_gb300.models import beam_chain_fsi  # noqa: E402

SECTION = (1.539380400e-02, 4.621989652e-04, 4.621989652e-04, 9.243979304e-04)
MAT = dict(E=2.1e11, G=8.139534884e+10, rho=7850.0)


def model(shear):
    return beam_chain_fsi(5, 2.0, 0.0, 0.0, clamp=0, load_node=5, load_dof=1, load=1.0e5, shear_factor=shear,
                          section=SECTION, axis="z", title="cantilever pipe along Z", **MAT)


DYNAMIC = ["-initEquilibrium", "-tolInitEquil=1.0e-8", "-tolDispNorm=1.0e-16", "-tolVelNorm=1.0e-15",
           "-tolEnerSum=1.0e-16", "-nupdat=5", "-timeInc=0.1", "-timeEnd=0.3"]
LINEAR = ["-initEquilibrium", "-tolInitEquil=0.0"]

PRESCRIBED = ["-numit=-1", "-timeInc=0.2", "-timeEnd=1.0", "-quasiStatic=1.0", "-tolDispNorm=1.0e-16",
              "-tolEnerSum=1.0e-16"]

CASES = [
    # test_solver.C:181-186: tip triad (u_x, u_y, u_z) at t = 0, 0.1, 0.2, 0.3
    {"name": "cantilever_pipe_dynamic", "model": "cantilever_pipe.fsi", "options": DYNAMIC, "triad": 6,
     "expected": [[0.344609, 0.0, 9.992951]] * 4, "abs_tol": 1.0e-6},
    {"name": "cantilever_pipe_linear", "model": "cantilever_pipe.fsi", "options": LINEAR, "triad": 6,
     "expected": [[0.345020, 0.0, 10.0]], "abs_tol": 1.0e-6},
    {"name": "cantilever_noshear_linear", "model": "cantilever_noshear.fsi", "options": LINEAR, "triad": 6,
     "expected": [[0.343424, 0.0, 10.0]], "abs_tol": 1.0e-6},
    # test_solver.C:196-262: triads at Z = 6 and Z = 10 after the steps t = 0.2, 0.4, 0.6, 0.8
    {"name": "cantilever_prescribed_quasistatic", "model": "cantilever_prescribed.fsi", "options": PRESCRIBED,
     "triads": [4, 6], "first_step": 1, "requires": ["prescribed_motion", "quasi_static"],
     "expected": [[0.086555, 0.0, 6.0, 0.2, 0.0, 10.0], [0.173111, 0.0, 6.0, 0.4, 0.0, 10.0],
                  [0.259666, 0.0, 6.0, 0.6, 0.0, 10.0], [0.346222, 0.0, 6.0, 0.8, 0.0, 10.0]],
     "abs_tol": 1.0e-6},
]

if __name__ == "__main__":
    with open(os.path.join(HERE, "cantilever_pipe.fsi"), "w") as f:
        f.write(model(2.0))
    with open(os.path.join(HERE, "cantilever_noshear.fsi"), "w") as f:
        f.write(model(0.0))
    with open(os.path.join(HERE, "cantilever_prescribed.fsi"), "w") as f:
        f.write(beam_chain_fsi(5, 2.0, 0.0, 0.0, clamp=0, load_node=5, load_dof=1, load=0.0, shear_factor=2.0,
                               section=SECTION, axis="z", title="cantilever with prescribed tip deflection",
                               motion=(5, 1, 1.0), **MAT))
    for c in CASES:
        c.setdefault("triads", [c.pop("triad", 6)])
        c.setdefault("first_step", 0)
        c.setdefault("requires", [])
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump({"source": "src/vpmSolver/vpmSolverTests/test_solver.C:93-262", "cases": CASES}, f, indent=1)
    print("wrote fixtures to", HERE)
