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
