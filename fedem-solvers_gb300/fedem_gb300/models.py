"""Synthetic FEDEM models written as solver-input (.fsi) text.

The generators produce the workloads of the benchmark configurations with
seeded random properties; the text uses the record subset the reference
solver reads for beam models (&MECHANISM, &TRIAD, &SUP_EL, &TRIAD_UNDPOS,
&ELEMENT_PROPERTY, &LOAD; see src/vpmSolver/vpmSolverTests/models/
cantilever-pipe.fsi for the layout).  Every model is a straight chain of
2-noded beam superelements along the global X axis.
"""
import math

import numpy as np

STEEL = {"E": 2.1e11, "G": 8.1e10, "rho": 7850.0}


def pipe_section(od, wall):
    """Area, Iy, Iz, It of a circular pipe."""
    di = od - 2.0 * wall
    area = math.pi / 4.0 * (od * od - di * di)
    inertia = math.pi / 64.0 * (od ** 4 - di ** 4)
    return area, inertia, inertia, 2.0 * inertia


def _f(x):
    return repr(float(x))


def _bc_line(k, clamp, motion):
    if k == clamp:
        return "  BC = 0 0 0 0 0 0\n"
    if motion is not None and k == motion[0]:
        # BC 2 on the prescribed DOF: free, except in initial equilibrium iterations
        return "  BC = " + " ".join("2" if d + 1 == motion[1] else "1" for d in range(6)) + "\n"
    return ""


def _loads(n_el, load_node, load_dof, load, motion, load_ramp=None, load_ext=None):
    """&LOAD record, or with `motion` = (triad index, DOF, d1) a prescribed
    deflection d1 * time driven by a SCALE function of the TIME sensor
    (&MOTION, &ENGINE, &FUNCTION, &SENSOR as in the reference's
    cantilever-prescribed.fsi).  `load_ramp` = r makes the load
    load * r * time (F = f0 + f1 * engine with f0 = 0, f1 = load).
    `load_ext` = (channel, user id, tag) drives the load by an external
    function instead (DEVICE_FUNCTION without a file): F = load * value."""
    out = []
    if load_ext is not None:
        channel, uid, tag = load_ext
        base = 2 * n_el + 60
        out.append(f"&LOAD\n  id = {2 * n_el + 10}\n  triadId = {load_node + 1}\n  lDof = {int(load_dof)}\n"
                   f"  f0 = 0.0\n  f1 = {_f(load)}\n  loadEngineId = {base}\n/\n"
                   f"&ENGINE\n  id = {base}\n  extId = {int(uid)}\n  tag = '{tag}'\n  functionId = {base + 1}\n"
                   f"  nArg = 0\n/\n"
                   f"&FUNCTION\n  id = {base + 1}\n  type = 'DEVICE_FUNCTION'\n  channel = {int(channel)}\n"
                   f"  fileName = ''\n/\n")
    elif load_ramp is not None:
        base = 2 * n_el + 40
        out.append(f"&LOAD\n  id = {2 * n_el + 10}\n  triadId = {load_node + 1}\n  lDof = {int(load_dof)}\n"
                   f"  f0 = 0.0\n  f1 = {_f(load)}\n  loadEngineId = {base}\n/\n"
                   f"&ENGINE\n  id = {base}\n  functionId = {base + 1}\n  nArg = 1\n  argSensorId = {base + 2}\n/\n"
                   f"&FUNCTION\n  id = {base + 1}\n  type = 'SCALE'\n  realDataSize = 1\n  realData = {_f(load_ramp)}\n/\n"
                   f"&SENSOR\n  id = {base + 2}\n  type = 'TIME'\n/\n")
    elif motion is None or load != 0.0:
        out.append(f"&LOAD\n  id = {2 * n_el + 10}\n  triadId = {load_node + 1}\n  lDof = {int(load_dof)}\n"
                   f"  f0 = {_f(load)}\n/\n")
    if motion is not None:
        node, dof, d1 = motion
        base = 2 * n_el + 20
        out.append(f"&MOTION\n  id = {base}\n  triadId = {node + 1}\n  lDof = {int(dof)}\n  type = 'deflection'\n"
                   f"  motionEngineId = {base + 1}\n  d0 = 0.0\n  d1 = {_f(d1)}\n/\n"
                   f"&ENGINE\n  id = {base + 1}\n  functionId = {base + 2}\n  nArg = 1\n  argSensorId = {base + 3}\n/\n"
                   f"&FUNCTION\n  id = {base + 2}\n  type = 'SCALE'\n  realDataSize = 1\n  realData = 1.0\n/\n"
                   f"&SENSOR\n  id = {base + 3}\n  type = 'TIME'\n/\n")
    return out


def _axials(n_el, anchors, springs, dampers):
    """Fixed anchor triads and axial spring/damper records.  `anchors` are
    (x, y, z) points (triad ids 10*n_el + 100 + k, all DOFs fixed); springs are
    (triad a, triad b, stiffness, stress-free length[, alpha2]) and dampers
    (triad a, triad b, coefficient), with triads given as chain indices
    0..n_el or ("anchor", k)."""
    def tid(t):
        return 10 * n_el + 100 + t[1] if isinstance(t, tuple) else t + 1

    out = []
    for k, (x, y, z) in enumerate(anchors or ()):
        out.append(f"&TRIAD\n  id = {10 * n_el + 100 + k}\n  nDOFs = 6\n  ur = 1.0 0.0 0.0 {_f(x)} 0.0 1.0 0.0 "
                   f"{_f(y)} 0.0 0.0 1.0 {_f(z)}\n  BC = 0 0 0 0 0 0\n/\n")
    base = 20 * n_el + 200
    for k, sp in enumerate(springs or ()):
        a, b, stiff, l0 = sp[:4]
        alpha2 = sp[4] if len(sp) > 4 else 0.0
        out.append(f"&SPRING_BASE\n  id = {base + k}\n  l0 = {_f(l0)}\n  s0 = {_f(stiff)}\n/\n"
                   f"&SPRING_ELEMENT\n  id = {base + k}\n  triadIDs = {tid(a)} {tid(b)}\n"
                   f"  springBaseId = {base + k}\n  alpha2 = {_f(alpha2)}\n/\n")
    for k, (a, b, coeff) in enumerate(dampers or ()):
        out.append(f"&DAMPER\n  id = {base + 1000 + k}\n  triad1Id = {tid(a)}\n  triad2Id = {tid(b)}\n"
                   f"  d0 = {_f(coeff)}\n/\n")
    return out


def beam_chain_fsi(n_el, el_len, od, wall, E, G, rho, clamp, load_node, load_dof, load,
                   shear_factor=0.0, weights=(0.1, 1.0, 1.0), title="beam chain", section=None, axis="x",
                   motion=None, anchors=None, springs=None, dampers=None, load_ramp=None, load_ext=None):
    """Solver-input text for a straight chain of `n_el` beams along X (or Z).

    Triad k sits at k*el_len on the axis; triad `clamp` has all six DOFs
    fixed; a constant (step) load `load` acts on DOF `load_dof` (1..6) of
    triad `load_node`.  shear_factor = 0 gives Euler-Bernoulli beams.
    `section` = (A, Iy, Iz, It) overrides the pipe section from od/wall.
    `motion` = (triad index, DOF, d1) prescribes that DOF to d1 * time
    (the load record is then left out when `load` is 0); `load_ramp` = r
    makes the load grow as load * r * time; `load_ext` = (channel, user id,
    tag) makes it load * (external function value).  `anchors`,
    `springs` and `dampers` add fixed triads and axial springs/dampers
    (see _axials).
    """
    extra = _axials(n_el, anchors, springs, dampers)
    if axis == "z":
        return _chain_along_z(n_el, el_len, section or pipe_section(od, wall), E, G, rho, clamp, load_node,
                              load_dof, load, shear_factor, weights, title, motion, load_ramp) + "".join(extra)
    area, iy, iz, it = section or pipe_section(od, wall)
    out = [f"&HEADING\n  modelFile = '{title}'\n/\n",
           f"&MECHANISM\n  id = 1\n  weightTranslation = {_f(weights[0])}\n"
           f"  weightRotation = {_f(weights[1])}\n  weightGeneralized = {_f(weights[2])}\n/\n"]
    for k in range(n_el + 1):
        x = _f(k * el_len)
        bc = _bc_line(k, clamp, motion)
        out.append(f"&TRIAD\n  id = {k + 1}\n  nDOFs = 6\n  ur = 1.0 0.0 0.0 {x} 0.0 1.0 0.0 0.0 "
                   f"0.0 0.0 1.0 0.0\n{bc}/\n")
    L = _f(el_len)
    for e in range(n_el):
        a, b = e + 1, e + 2
        x0 = _f(e * el_len)
        sid = n_el + 2 + e
        out.append(
            f"&SUP_EL\n  id = {sid}\n  numTriads = 2\n  triadIds = {a} {b}\n  elPropId = 1\n  shadowPosAlg = 1\n"
            f"  refTriad1Id = {a}, offset1 = 0.0 0.0 0.0\n  refTriad2Id = {b}, offset2 = 0.0 0.0 0.0\n"
            f"  refTriad3Id = {a}, offset3 = 0.0 {L} 0.0\n"
            f"  supPos = 1.0 0.0 0.0 {x0} 0.0 1.0 0.0 0.0 0.0 0.0 1.0 0.0\n/\n"
            f"&TRIAD_UNDPOS\n  supElId = {sid}\n  triadId = {a}\n"
            f"  undPosInSupElSystem = 1.0 0.0 0.0 0.0 0.0 1.0 0.0 0.0 0.0 0.0 1.0 0.0\n/\n"
            f"&TRIAD_UNDPOS\n  supElId = {sid}\n  triadId = {b}\n"
            f"  undPosInSupElSystem = 1.0 0.0 0.0 {L} 0.0 1.0 0.0 0.0 0.0 0.0 1.0 0.0\n/\n")
    out.append(f"&ELEMENT_PROPERTY\n  id = 1\n  geometry = {_f(area)} {_f(iy)} {_f(iz)} {_f(it)} "
               f"{_f(shear_factor)} {_f(shear_factor)} 0.0 0.0\n  material = {_f(rho)} {_f(E)} {_f(G)}\n/\n")
    out += _loads(n_el, load_node, load_dof, load, motion, load_ramp, load_ext)
    return "".join(out + extra)


def _chain_along_z(n_el, el_len, section, E, G, rho, clamp, load_node, load_dof, load, shear_factor, weights,
                   title, motion, load_ramp=None):
    """Chain along global Z; the superelement X axis is the beam axis, so the
    superelement frame rotates global Z onto local X."""
    area, iy, iz, it = section
    rot = "0.0 0.0 -1.0 {p0} 0.0 1.0 0.0 {p1} 1.0 0.0 0.0 {p2}"
    out = [f"&HEADING\n  modelFile = '{title}'\n/\n",
           f"&MECHANISM\n  id = 1\n  weightTranslation = {_f(weights[0])}\n"
           f"  weightRotation = {_f(weights[1])}\n  weightGeneralized = {_f(weights[2])}\n/\n"]
    for k in range(n_el + 1):
        bc = _bc_line(k, clamp, motion)
        out.append(f"&TRIAD\n  id = {k + 1}\n  nDOFs = 6\n  ur = 1.0 0.0 0.0 0.0 0.0 1.0 0.0 0.0 "
                   f"0.0 0.0 1.0 {_f(k * el_len)}\n{bc}/\n")
    L = _f(el_len)
    for e in range(n_el):
        a, b = e + 1, e + 2
        sid = n_el + 2 + e
        out.append(
            f"&SUP_EL\n  id = {sid}\n  numTriads = 2\n  triadIds = {a} {b}\n  elPropId = 1\n  shadowPosAlg = 1\n"
            f"  refTriad1Id = {a}, offset1 = 0.0 0.0 0.0\n  refTriad2Id = {b}, offset2 = 0.0 0.0 0.0\n"
            f"  refTriad3Id = {a}, offset3 = 0.0 {L} 0.0\n"
            f"  supPos = {rot.format(p0='0.0', p1='0.0', p2=_f(e * el_len))}\n/\n"
            f"&TRIAD_UNDPOS\n  supElId = {sid}\n  triadId = {a}\n"
            f"  undPosInSupElSystem = {rot.format(p0='0.0', p1='0.0', p2='0.0')}\n/\n"
            f"&TRIAD_UNDPOS\n  supElId = {sid}\n  triadId = {b}\n"
            f"  undPosInSupElSystem = {rot.format(p0=L, p1='0.0', p2='0.0')}\n/\n")
    out.append(f"&ELEMENT_PROPERTY\n  id = 1\n  geometry = {_f(area)} {_f(iy)} {_f(iz)} {_f(it)} "
               f"{_f(shear_factor)} {_f(shear_factor)} 0.0 0.0\n  material = {_f(rho)} {_f(E)} {_f(G)}\n/\n")
    out += _loads(n_el, load_node, load_dof, load, motion, load_ramp)
    return "".join(out)


def cantilever_c1():
    """Plain method, FP64: 5 m cantilever pipe, 20 Euler-Bernoulli beams, 1 kN tip step load."""
    fsi = beam_chain_fsi(20, 0.25, 0.1, 0.01, clamp=0, load_node=20, load_dof=2, load=1000.0, **STEEL,
                         title="cantilever pipe, 20 beams")
    opts = ["-timeInc=0.001", "-timeEnd=1.0", "-alphaNewmark=0.1", "-tolDispNorm=1.0e-8"]
    return fsi, opts


def served_pool_c5(n_models=64, seed=5, dof_min=1000, dof_max=200000, steps_min=100, steps_max=2000,
                   steps_scale=1.0):
    """Request pool of the served workload: the batch generator's beam chains with
    sizes log-uniform in [dof_min, dof_max] DOF and time steps log-uniform in
    [steps_min, steps_max] (times steps_scale).  Returns (fsi, options, elements, steps)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_models):
        dof = math.exp(rng.uniform(math.log(dof_min), math.log(dof_max)))
        n_el = max(2, int(round(dof / 6.0)))
        steps = max(1, int(round(steps_scale * math.exp(rng.uniform(math.log(steps_min), math.log(steps_max))))))
        sub = batch_c4(1, seed=int(rng.integers(1 << 30)), n_min=n_el, n_max=n_el, steps=steps)[0]
        out.append((sub[0], sub[1], n_el, steps))
    return out


def batch_c4(n_models=256, seed=4, n_min=10, n_max=4000, steps=500):
    """Batched workload: chains with log-uniform element counts, +/-20% properties,
    random clamp and load triads, step loads uniform in [0.1, 10] kN.
    Returns a list of (fsi text, options, element count)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_models):
        n_el = int(math.floor(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        n_el = max(n_min, min(n_max, n_el))
        s = rng.uniform(0.8, 1.2, size=5)
        od = 0.1 * s[0]
        clamp = int(rng.integers(0, n_el + 1))
        load_node = int(rng.integers(0, n_el))
        if load_node >= clamp:
            load_node += 1
        load_dof = int(rng.choice([2, 3]))
        load = float(rng.uniform(100.0, 10000.0)) * (1.0 if rng.random() < 0.5 else -1.0)
        fsi = beam_chain_fsi(n_el, 0.25, od, od / 10.0, E=STEEL["E"] * s[1], G=STEEL["G"] * s[2],
                             rho=STEEL["rho"] * s[3], clamp=clamp, load_node=load_node, load_dof=load_dof,
                             load=load, title=f"batch model, {n_el} beams")
        opts = ["-timeInc=0.001", f"-timeEnd={steps * 0.001!r}", "-alphaNewmark=0.1", "-tolDispNorm=1.0e-8"]
        out.append((fsi, opts, n_el))
    return out


# ---------------------------------------------------------------------------
# General frames: beams in any direction, master-slave joints, springs, dampers
# ---------------------------------------------------------------------------
def _beam_frame(a, b):
    """Superelement axes of a beam from point a to b: x along the beam, y and z
    completing a right-handed frame (the beam element takes its local axes from
    these).  Returns the 3x3 rotation (columns ex, ey, ez) and the length."""
    a, b = np.asarray(a, float), np.asarray(b, float)
    ex = b - a
    L = float(np.linalg.norm(ex))
    ex = ex / L
    # the global axis least aligned with the beam completes the frame
    ref = np.eye(3)[int(np.argmin(np.abs(ex)))]
    ez = np.cross(ex, ref)
    ez /= np.linalg.norm(ez)
    ey = np.cross(ez, ex)
    return np.stack([ex, ey, ez], 1), L


def _rows34(R, p):
    """3x4 position matrix [R | p] as the file writes it: row by row."""
    return " ".join(_f(R[r, c]) if c < 3 else _f(p[r]) for r in range(3) for c in range(4))


def frame_fsi(triads, beams, props, joints=(), loads=(), springs=(), dampers=(), gravity=None,
              weights=(0.1, 1.0, 1.0), title="frame"):
    """Solver-input text of a general frame.

    triads:  dicts {id, pos (3), bc (6 ints, default free)}; global axes.
    beams:   (id, triad a, triad b, property id) 2-noded beam superelements.
    props:   dicts {id, A, Iy, Iz, It, rho, E, G, shear (0 = Euler-Bernoulli)}.
    joints:  dicts {id, type (1 revolute, 3 rigid, 4 free), slave, master,
             pos (3), rot (3x3, columns = joint axes; default identity),
             dofs [(lDof, iMat), ...], bc [..], init [..]}: &MASTERSLAVEJOINT.
    loads:   (triad id, DOF 1..6, f0) constant point loads.
    springs: (triad a, triad b, stiffness, stress-free length[, alpha2]).
    dampers: (triad a, triad b, coefficient).
    gravity: (gx, gy, gz) or None.
    """
    pos = {t["id"]: np.asarray(t["pos"], float) for t in triads}
    out = [f"&HEADING\n  modelFile = '{title}'\n/\n",
           f"&MECHANISM\n  id = 1\n  weightTranslation = {_f(weights[0])}\n"
           f"  weightRotation = {_f(weights[1])}\n  weightGeneralized = {_f(weights[2])}\n/\n"]
    if gravity is not None:
        out.append("&ENVIRONMENT\n  gravity = " + " ".join(_f(g) for g in gravity) + "\n/\n")
    for t in triads:
        bc = t.get("bc")
        bcl = ("  BC = " + " ".join(str(int(v)) for v in bc) + "\n") if bc is not None else ""
        out.append(f"&TRIAD\n  id = {t['id']}\n  nDOFs = 6\n  ur = {_rows34(np.eye(3), pos[t['id']])}\n{bcl}/\n")
    for (sid, ta, tb, pid) in beams:
        R, L = _beam_frame(pos[ta], pos[tb])
        out.append(
            f"&SUP_EL\n  id = {sid}\n  numTriads = 2\n  triadIds = {ta} {tb}\n  elPropId = {pid}\n  shadowPosAlg = 1\n"
            f"  refTriad1Id = {ta}, offset1 = 0.0 0.0 0.0\n  refTriad2Id = {tb}, offset2 = 0.0 0.0 0.0\n"
            f"  refTriad3Id = {ta}, offset3 = 0.0 {_f(L)} 0.0\n"
            f"  supPos = {_rows34(R, pos[ta])}\n/\n"
            f"&TRIAD_UNDPOS\n  supElId = {sid}\n  triadId = {ta}\n"
            f"  undPosInSupElSystem = {_rows34(R, (0.0, 0.0, 0.0))}\n/\n"
            f"&TRIAD_UNDPOS\n  supElId = {sid}\n  triadId = {tb}\n"
            f"  undPosInSupElSystem = {_rows34(R, (L, 0.0, 0.0))}\n/\n")
    for p in props:
        out.append(f"&ELEMENT_PROPERTY\n  id = {p['id']}\n  geometry = {_f(p['A'])} {_f(p['Iy'])} {_f(p['Iz'])} "
                   f"{_f(p['It'])} {_f(p.get('shear', 0.0))} {_f(p.get('shear', 0.0))} 0.0 0.0\n"
                   f"  material = {_f(p['rho'])} {_f(p['E'])} {_f(p['G'])}\n/\n")
    for j in joints:
        R = np.asarray(j.get("rot", np.eye(3)), float)
        dofs = list(j.get("dofs", []))
        bc = list(j.get("bc", [1] * len(dofs)))
        init = list(j.get("init", [0.0] * len(dofs)))
        lines = [f"&MASTERSLAVEJOINT\n  id = {j['id']}\n  type = {int(j.get('type', 1))}\n"
                 f"  slaveId = {j['slave']}\n  masterId = {j['master']}\n"
                 f"  initPosInGlobal = {_rows34(R, j['pos'])}\n  nJointVars = {len(dofs)}\n"]
        if dofs:
            lines.append("  JointVarDefs = " + " ".join(f"{int(a)} {int(b)}" for a, b in dofs) + "\n")
            lines.append("  BC = " + " ".join(str(int(v)) for v in bc) + "\n")
            lines.append("  JVarInitVal = " + " ".join(_f(v) for v in init) + "\n")
        out.append("".join(lines) + "/\n")
    for k, (tid, dof, f0) in enumerate(loads):
        out.append(f"&LOAD\n  id = {900000 + k}\n  triadId = {tid}\n  lDof = {int(dof)}\n  f0 = {_f(f0)}\n/\n")
    for k, sp in enumerate(springs):
        a, b, stiff, l0 = sp[:4]
        alpha2 = sp[4] if len(sp) > 4 else 0.0
        out.append(f"&SPRING_BASE\n  id = {800000 + k}\n  l0 = {_f(l0)}\n  s0 = {_f(stiff)}\n/\n"
                   f"&SPRING_ELEMENT\n  id = {800000 + k}\n  triadIDs = {a} {b}\n"
                   f"  springBaseId = {800000 + k}\n  alpha2 = {_f(alpha2)}\n/\n")
    for k, (a, b, coeff) in enumerate(dampers):
        out.append(f"&DAMPER\n  id = {850000 + k}\n  triad1Id = {a}\n  triad2Id = {b}\n  d0 = {_f(coeff)}\n/\n")
    return "".join(out)


def pipe_props(pid, od, wall, E=STEEL["E"], G=STEEL["G"], rho=STEEL["rho"]):
    area, iy, iz, it = pipe_section(od, wall)
    return {"id": pid, "A": area, "Iy": iy, "Iz": iz, "It": it, "rho": rho, "E": E, "G": G}


def hinged_beam(n_left=8, n_right=8, el_len=0.25, load=10.0, joint_type=1):
    """Two beam segments along X joined at x = n_left * el_len: the left one
    clamped at x = 0, the right one pinned (translations fixed) at its end.
    The joint's master is the left segment's end triad, its slave the right
    segment's first triad (same point).  joint_type 1: revolute about global Z
    (bending about Z released: a Gerber beam, which carries a transverse Y load
    at the hinge on the left cantilever alone); 3: rigid (a continuous beam).
    The load acts on the master triad in Y."""
    triads, beams = [], []
    nid = 1
    for k in range(n_left + 1):
        triads.append({"id": nid, "pos": (k * el_len, 0.0, 0.0), "bc": [0] * 6 if k == 0 else None})
        nid += 1
    master = nid - 1
    slave = nid
    for k in range(n_right + 1):
        bc = [0, 0, 0, 1, 1, 1] if k == n_right else None
        triads.append({"id": nid, "pos": ((n_left + k) * el_len, 0.0, 0.0), "bc": bc})
        nid += 1
    sid = 1000
    for k in range(n_left):
        beams.append((sid, k + 1, k + 2, 1))
        sid += 1
    for k in range(n_right):
        beams.append((sid, slave + k, slave + k + 1, 1))
        sid += 1
    j = {"id": 500, "type": joint_type, "slave": slave, "master": master, "pos": (n_left * el_len, 0.0, 0.0)}
    if joint_type == 1:
        j["dofs"] = [(6, 1)]
    fsi = frame_fsi(triads, beams, [pipe_props(1, 0.1, 0.01)], joints=[j], loads=[(master, 2, load)],
                    title="hinged beam")
    return fsi, master, slave


def pendulum(length=1.0, n_el=4, theta0=0.1, g=9.81):
    """A pipe hanging from a revolute joint (axis global Z) at the origin,
    released at rest theta0 from the vertical under gravity -Y.  The joint's
    master is a clamped ground triad, its slave the pipe's top triad."""
    d = np.array([np.sin(theta0), -np.cos(theta0), 0.0])
    triads = [{"id": 1, "pos": (0.0, 0.0, 0.0), "bc": [0] * 6}]
    for k in range(n_el + 1):
        triads.append({"id": 2 + k, "pos": tuple(d * length * k / n_el)})
    beams = [(100 + k, 2 + k, 3 + k, 1) for k in range(n_el)]
    j = {"id": 50, "type": 1, "slave": 2, "master": 1, "pos": (0.0, 0.0, 0.0), "dofs": [(6, 1)]}
    fsi = frame_fsi(triads, beams, [pipe_props(1, 0.05, 0.005)], joints=[j], gravity=(0.0, -g, 0.0),
                    title="pendulum")
    return fsi, 2 + n_el


def space_frame_c2(seed=2, storeys=12, bays=4, h=3.0, bay=3.0, n_joints=40, n_springs=40, load=10.0e3,
                   freq=2.0, steps=2000, dt=1.0e-3):
    """Space-frame tower: `storeys` x (`bays` x `bays`) lattice of steel pipes
    (3 m storeys and bays), base clamped.  Members: columns, floor beams in X
    and Y, one floor diagonal per bay and one diagonal brace per panel of the
    four outer faces (1,164 beams at the default size).  Pipe OD uniform in
    [0.05, 0.2] m per member, wall OD/10.  `n_joints` revolute joints at
    random floor nodes release one X floor beam's end rotation about global Y
    (a pinned beam end: the beam attaches to a dependent triad at the node).
    `n_springs` axial spring + damper pairs, each between a random node and
    another random node at most one storey away (k uniform in [1e5, 1e7] N/m,
    c = 1e-3 k, stress-free at the start).
    Lateral top load: `load` N in X spread over the top floor's nodes,
    sinusoidal at `freq` Hz.  Returns (fsi, options)."""
    rng = np.random.default_rng(seed)
    n = bays + 1

    def nid(i, j, k):
        return 1 + i + n * (j + n * k)

    triads = []
    for k in range(storeys + 1):
        for j in range(n):
            for i in range(n):
                triads.append({"id": nid(i, j, k), "pos": (i * bay, j * bay, k * h),
                               "bc": [0] * 6 if k == 0 else None})
    members = []
    for k in range(storeys):
        for j in range(n):
            for i in range(n):
                members.append((nid(i, j, k), nid(i, j, k + 1)))
    for k in range(1, storeys + 1):
        for j in range(n):
            for i in range(bays):
                members.append((nid(i, j, k), nid(i + 1, j, k)))
        for j in range(bays):
            for i in range(n):
                members.append((nid(i, j, k), nid(i, j + 1, k)))
        for j in range(bays):
            for i in range(bays):
                members.append((nid(i, j, k), nid(i + 1, j + 1, k)))
    for k in range(storeys):  # outer faces: one diagonal per panel
        for i in range(bays):
            members.append((nid(i, 0, k), nid(i + 1, 0, k + 1)))
            members.append((nid(i, bays, k), nid(i + 1, bays, k + 1)))
        for j in range(bays):
            members.append((nid(0, j, k), nid(0, j + 1, k + 1)))
            members.append((nid(bays, j, k), nid(bays, j + 1, k + 1)))
    ods = rng.uniform(0.05, 0.2, size=len(members))
    props = [pipe_props(1 + e, ods[e], ods[e] / 10.0) for e in range(len(members))]
    # revolute joints: the far end of an X floor beam gets its own (dependent) triad
    xbeams = [e for e, (a, b) in enumerate(members)
              if triads[a - 1]["pos"][2] == triads[b - 1]["pos"][2] and triads[b - 1]["pos"][0] > triads[a - 1]["pos"][0]
              and triads[b - 1]["pos"][1] == triads[a - 1]["pos"][1]]
    picks = rng.permutation(xbeams)
    joints, used = [], set()
    next_id = nid(bays, bays, storeys) + 1
    rot = np.array([[0.0, 1.0, 0.0], [0.0, 0.0, 1.0], [1.0, 0.0, 0.0]])  # joint Z = global Y
    for e in picks:
        if len(joints) == n_joints:
            break
        a, b = members[e]
        if b in used:
            continue
        used.add(b)
        slave = next_id
        next_id += 1
        triads.append({"id": slave, "pos": triads[b - 1]["pos"]})
        members[e] = (a, slave)
        joints.append({"id": 700000 + len(joints), "type": 1, "slave": slave, "master": b,
                       "pos": triads[b - 1]["pos"], "rot": rot, "dofs": [(6, 1)]})
    free = [t["id"] for t in triads if t.get("bc") is None and t["id"] <= nid(bays, bays, storeys)]
    springs, dampers = [], []
    for _ in range(n_springs):
        # a random node tied to another random node at most one storey away
        a = int(rng.choice(free))
        za = triads[a - 1]["pos"][2]
        near = [t for t in free if t != a and abs(triads[t - 1]["pos"][2] - za) <= h + 1e-9]
        b = int(rng.choice(near))
        pa, pb = np.array(triads[a - 1]["pos"]), np.array(triads[b - 1]["pos"])
        kk = rng.uniform(1.0e5, 1.0e7)
        springs.append((int(a), int(b), kk, float(np.linalg.norm(pb - pa))))
        dampers.append((int(a), int(b), 1.0e-3 * kk))
    beams = [(100000 + e, a, b, 1 + e) for e, (a, b) in enumerate(members)]
    top = [nid(i, j, storeys) for j in range(n) for i in range(n)]
    fsi = frame_fsi(triads, beams, props, joints=joints, springs=springs, dampers=dampers,
                    title=f"space frame {storeys}x{bays}x{bays}")
    # sinusoidal lateral top load (engine of a SINUSOIDAL function of the TIME sensor)
    eng = 990000
    fsi += (f"&FUNCTION\n  id = {eng + 1}\n  type = 'SINUSOIDAL'\n  realDataSize = 4\n"
            f"  realData = {_f(freq)} 0.0 1.0 0.0\n/\n"
            f"&SENSOR\n  id = {eng + 2}\n  type = 'TIME'\n/\n"
            f"&ENGINE\n  id = {eng}\n  functionId = {eng + 1}\n  nArg = 1\n  argSensorId = {eng + 2}\n/\n")
    for k, t in enumerate(top):
        fsi += (f"&LOAD\n  id = {980000 + k}\n  triadId = {t}\n  lDof = 1\n  f0 = 0.0\n"
                f"  f1 = {_f(load / len(top))}\n  loadEngineId = {eng}\n/\n")
    opts = ["-timeInc=%r" % dt, "-timeEnd=%r" % (steps * dt), "-alphaNewmark=0.1", "-tolDispNorm=1.0e-8"]
    return fsi, opts


def part_records(pid, triad_ids, origin, files, n_gen, undpos, R=None, alpha1=0.0, alpha2=0.0, gen_bc=None,
                 ref_offset=1.0):
    """&SUP_EL and &TRIAD_UNDPOS records of a reduced part: triads
    `triad_ids`, generalized DOFs `n_gen`, matrices from `files` (K, M, G
    paths), part axes R (columns; default global) at `origin`, each triad's
    position in part axes in `undpos`.  The corotated frame follows the first
    two triads and a point `ref_offset` along part Y from the first one
    (shadowPosAlg 1)."""
    R = np.eye(3) if R is None else np.asarray(R, float)
    ta, tb = triad_ids[0], triad_ids[1]
    files_line = " ".join(f"'{files[k]}'" for k in ("K", "M", "G"))
    bc = "" if gen_bc is None else "  BC = " + " ".join(str(int(v)) for v in gen_bc) + "\n"
    out = [f"&SUP_EL\n  id = {pid}\n  numTriads = {len(triad_ids)}\n  triadIds = {' '.join(map(str, triad_ids))}\n"
           f"  numGenDOFs = {n_gen}\n{bc}  inputFiles = {files_line}\n  shadowPosAlg = 1\n"
           f"  refTriad1Id = {ta}, offset1 = 0.0 0.0 0.0\n  refTriad2Id = {tb}, offset2 = 0.0 0.0 0.0\n"
           f"  refTriad3Id = {ta}, offset3 = 0.0 {_f(ref_offset)} 0.0\n"
           f"  alpha1 = {_f(alpha1)}\n  alpha2 = {_f(alpha2)}\n"
           f"  supPos = {_rows34(R, origin)}\n/\n"]
    # a triad in global axes sits in the part axes R with orientation R
    for t, p in zip(triad_ids, undpos):
        out.append(f"&TRIAD_UNDPOS\n  supElId = {pid}\n  triadId = {t}\n"
                   f"  undPosInSupElSystem = {_rows34(R, p)}\n/\n")
    return "".join(out)


def superelement_chain_c3(directory, n_parts=16, n_modes=30, length=2.0, width=0.2, height=0.2, nx=40, ny=4,
                          nz=4, torque=500.0, freq=2.0, damping=0.01, damping_hz=10.0, steps=4000, dt=5.0e-4,
                          g=9.81, axes=None):
    """Superelement chain: `n_parts` steel blocks (length x width x height,
    meshed with nx x ny x nz hexahedra) in series along global X, each reduced
    by the Craig-Bampton reducer to its two end-face triads plus `n_modes`
    component modes ((12 + n_modes)^2 K and M, written as binary matrix files
    into `directory`).  Consecutive parts are joined by revolute joints whose
    axis is the chain axis X (the master is the end triad of part k, the
    slave the first triad of part k + 1): every part is free to turn about
    the axis, bending and shear pass through.  The first triad is clamped,
    the last one pinned (translations fixed).  Gravity -Z; a harmonic torque
    `torque` sin(2 pi freq t) about X at the last triad; Rayleigh damping
    `damping` at `damping_hz`, half mass- and half stiffness-proportional.
    `axes` (3 x 3 rotation, columns) turns the whole chain (not gravity) so
    that its axis is axes[:, 0].  Returns (fsi, options, info)."""
    from . import reducer

    paths, (Kr, Mr, fg, w2) = reducer.block_part_files(directory, length, width, height, nx, ny, nz, n_modes)
    w0 = 2.0 * np.pi * damping_hz
    a1, a2 = damping * w0, damping / w0
    triads, joints, parts = [], [], []
    A = np.eye(3) if axes is None else np.asarray(axes, float)
    rot = A @ np.array([[0.0, 0.0, 1.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])  # joint Z = the chain axis
    for k in range(n_parts):
        ta, tb = 1 + 2 * k, 2 + 2 * k
        x0 = k * length
        pa, pb = A @ np.array([x0, 0.0, 0.0]), A @ np.array([x0 + length, 0.0, 0.0])
        triads.append({"id": ta, "pos": tuple(pa), "bc": [0] * 6 if k == 0 else None})
        triads.append({"id": tb, "pos": tuple(pb), "bc": [0, 0, 0, 1, 1, 1] if k == n_parts - 1 else None})
        parts.append(part_records(5000 + k, [ta, tb], tuple(pa), paths, n_modes,
                                  [(0.0, 0.0, 0.0), (length, 0.0, 0.0)], R=A, alpha1=a1, alpha2=a2,
                                  ref_offset=length))
        if k > 0:
            joints.append({"id": 600 + k, "type": 1, "slave": ta, "master": ta - 1, "pos": tuple(pa),
                           "rot": rot, "dofs": [(6, 1)]})
    fsi = frame_fsi(triads, [], [], joints=joints, gravity=(0.0, 0.0, -g), title="superelement chain")
    fsi += "".join(parts)
    eng = 990000
    fsi += (f"&FUNCTION\n  id = {eng + 1}\n  type = 'SINUSOIDAL'\n  realDataSize = 4\n"
            f"  realData = {_f(freq)} 0.0 1.0 0.0\n/\n"
            f"&SENSOR\n  id = {eng + 2}\n  type = 'TIME'\n/\n"
            f"&ENGINE\n  id = {eng}\n  functionId = {eng + 1}\n  nArg = 1\n  argSensorId = {eng + 2}\n/\n"
            + "".join(f"&LOAD\n  id = {980000 + c}\n  triadId = {2 * n_parts}\n  lDof = {4 + c}\n  f0 = 0.0\n"
                      f"  f1 = {_f(torque * A[c, 0])}\n  loadEngineId = {eng}\n/\n" for c in range(3) if A[c, 0] != 0.0))
    opts = ["-timeInc=%r" % dt, "-timeEnd=%r" % (steps * dt), "-alphaNewmark=0.1", "-tolDispNorm=1.0e-8"]
    info = {"Kr": Kr, "Mr": Mr, "fg": fg, "w2": w2, "files": paths, "tip": 2 * n_parts}
    return fsi, opts, info
