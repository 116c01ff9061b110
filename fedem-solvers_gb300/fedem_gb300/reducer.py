"""Reduced superelements for the solver: a Craig-Bampton reducer of a block
of 8-node hexahedra and the FEDEM binary matrix files it writes.

The reference's part reducer (src/vpmReducer/reducer.f90, cfemReducer.f90:
188-467) condenses an FE part onto its external nodes (static condensation)
and adds fixed-interface component modes, then writes the reduced stiffness
and mass matrices and the gravity force vectors with writeDoubleDBfile
(src/vpmUtilities/binaryDBInterface.f90:452-500).  The solver reads them back
per part (ReadSupElMatrices, src/vpmSolver/initiateSupElTypeModule.f90:
962-1033).  This module does the same for one family of parts:

- a box of nx x ny x nz equal trilinear hexahedra (isotropic, consistent
  mass, 2 x 2 x 2 Gauss points);
- each end face (x = 0 and x = length) tied rigidly to a triad at the face
  centre (u_node = t + theta x r, a linear rigid spider);
- Craig-Bampton reduction onto the two triads' 12 DOFs (static constraint
  modes) plus n_modes fixed-interface normal modes (mass-normalised), so that
  the reduced matrices have the solver's DOF order [triad 1 (6), triad 2 (6),
  modes]: K_r = [[K_bb - K_bi K_ii^-1 K_ib, 0], [0, diag(w^2)]], M_r dense
  with the boundary-mode coupling, and the gravity force vectors
  fg = T^T M r_j of the rigid translations r_j (solver: Q = fg (g R)).

Static loads on the triads are reproduced exactly by the constraint modes.

Matrix files: the tag text '#FEDEM <type>' opens the file, the version field
';1.0;' ends its header line, and the values follow as raw little-endian
doubles, column by column (binaryDB.c:643-731 writes the tag, the version
field and then the data the same way).  The reference's tag block also holds
an endian mark and a checksum in the layout of its fedem-foundation library
(absent here); this writer puts a newline there instead, and both readers in
this project take the tag text from the start and the values from the end of
the file.
"""
import os

import numpy as np

FMX_TAGS = {"K": "stiffness matrix", "M": "mass matrix", "G": "gravity force vectors"}


def write_fmx(path, dtype, a):
    """Writes a double matrix (column-major) as a FEDEM binary matrix file."""
    a = np.asarray(a, dtype="<f8")
    with open(path, "wb") as f:
        f.write(("#FEDEM " + dtype + "\n;1.0;\n").encode("ascii"))
        f.write(np.asfortranarray(a).tobytes(order="F"))


def read_fmx(path, dtype, shape):
    """Reads a matrix of the given shape from a FEDEM binary matrix file."""
    with open(path, "rb") as f:
        buf = f.read()
    n = int(np.prod(shape))
    tag = ("#FEDEM " + dtype).encode("ascii")
    if not buf.startswith(tag) or len(buf) < len(tag) + 6 + 8 * n:
        raise ValueError(f"{path} is not a {dtype} file of {n} values")
    head = len(buf) - 8 * n
    if buf[head - 6:head] != b";1.0;\n":
        raise ValueError(f"{path}: no version field before the data")
    return np.frombuffer(buf[head:], dtype="<f8").reshape(shape, order="F").copy()


def _hex_matrices(ax, ay, az, E, nu, rho):
    """Stiffness and consistent mass (24 x 24, DOFs node by node) of a box
    hexahedron with edge lengths ax, ay, az."""
    s = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                  [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], float)
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    mu = E / (2.0 * (1.0 + nu))
    D = np.zeros((6, 6))
    D[:3, :3] = lam
    D[np.arange(3), np.arange(3)] += 2.0 * mu
    D[np.arange(3, 6), np.arange(3, 6)] = mu
    detJ = ax * ay * az / 8.0
    g = 1.0 / np.sqrt(3.0)
    Ke = np.zeros((24, 24))
    Me = np.zeros((24, 24))
    for xi in (-g, g):
        for eta in (-g, g):
            for zeta in (-g, g):
                N = (1 + s[:, 0] * xi) * (1 + s[:, 1] * eta) * (1 + s[:, 2] * zeta) / 8.0
                dx = s[:, 0] * (1 + s[:, 1] * eta) * (1 + s[:, 2] * zeta) / 8.0 * (2.0 / ax)
                dy = s[:, 1] * (1 + s[:, 0] * xi) * (1 + s[:, 2] * zeta) / 8.0 * (2.0 / ay)
                dz = s[:, 2] * (1 + s[:, 0] * xi) * (1 + s[:, 1] * eta) / 8.0 * (2.0 / az)
                B = np.zeros((6, 24))
                B[0, 0::3], B[1, 1::3], B[2, 2::3] = dx, dy, dz
                B[3, 0::3], B[3, 1::3] = dy, dx
                B[4, 1::3], B[4, 2::3] = dz, dy
                B[5, 0::3], B[5, 2::3] = dz, dx
                Ke += B.T @ D @ B * detJ
                Nm = np.zeros((3, 24))
                for c in range(3):
                    Nm[c, c::3] = N
                Me += rho * Nm.T @ Nm * detJ
    return Ke, Me


def hex_block(length=2.0, width=0.2, height=0.2, nx=40, ny=4, nz=4, E=2.1e11, nu=0.3, rho=7850.0):
    """Sparse K and M (3 DOFs per node) of a box of nx x ny x nz hexahedra
    spanning x in [0, length], y in [-width/2, width/2], z in [-height/2,
    height/2], and the node coordinates.  Node (i, j, k) is i + (nx+1)(j + (ny+1) k)."""
    import scipy.sparse as sp

    ax, ay, az = length / nx, width / ny, height / nz
    Ke, Me = _hex_matrices(ax, ay, az, E, nu, rho)
    xs = np.linspace(0.0, length, nx + 1)
    ys = np.linspace(-width / 2, width / 2, ny + 1)
    zs = np.linspace(-height / 2, height / 2, nz + 1)
    K_, J_, I_ = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    coords = np.stack([xs[I_.ravel()], ys[J_.ravel()], zs[K_.ravel()]], 1)

    def nid(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)

    ek, ej, ei = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ei, ej, ek = ei.ravel(), ej.ravel(), ek.ravel()
    conn = np.stack([nid(ei, ej, ek), nid(ei + 1, ej, ek), nid(ei + 1, ej + 1, ek), nid(ei, ej + 1, ek),
                     nid(ei, ej, ek + 1), nid(ei + 1, ej, ek + 1), nid(ei + 1, ej + 1, ek + 1),
                     nid(ei, ej + 1, ek + 1)], 1)
    dofs = (3 * conn[:, :, None] + np.arange(3)[None, None, :]).reshape(len(conn), 24)
    rows = np.repeat(dofs, 24, axis=1).ravel()
    cols = np.tile(dofs, (1, 24)).ravel()
    n = 3 * len(coords)
    K = sp.coo_matrix((np.tile(Ke.ravel(), len(conn)), (rows, cols)), shape=(n, n)).tocsr()
    M = sp.coo_matrix((np.tile(Me.ravel(), len(conn)), (rows, cols)), shape=(n, n)).tocsr()
    return K, M, coords


def craig_bampton_two_faces(K, M, coords, length, n_modes=30):
    """Craig-Bampton reduction of a block onto triads at its end-face centres
    (0, 0, 0) and (length, 0, 0), in the block's axes.  Returns (K_r, M_r,
    fg, w2): the (12 + n_modes)^2 reduced matrices, the (12 + n_modes) x 3
    gravity force vectors and the squared fixed-interface frequencies."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla

    nn = len(coords)
    tol = 1e-9 * length
    face = [np.where(np.abs(coords[:, 0]) < tol)[0], np.where(np.abs(coords[:, 0] - length) < tol)[0]]
    centre = [np.zeros(3), np.array([length, 0.0, 0.0])]
    on_face = np.zeros(nn, bool)
    on_face[face[0]] = on_face[face[1]] = True
    interior = np.where(~on_face)[0]
    n_int = 3 * len(interior)
    # u_full = T q', q' = [triad 1 (t, theta), triad 2 (t, theta), interior DOFs]
    rows, cols, vals = [], [], []
    for f in range(2):
        for node in face[f]:
            r = coords[node] - centre[f]
            # u = t + theta x r = t - skew(r) theta
            S = np.array([[0.0, -r[2], r[1]], [r[2], 0.0, -r[0]], [-r[1], r[0], 0.0]])
            for a in range(3):
                rows.append(3 * node + a)
                cols.append(6 * f + a)
                vals.append(1.0)
                for b in range(3):
                    if S[a, b] != 0.0:
                        rows.append(3 * node + a)
                        cols.append(6 * f + 3 + b)
                        vals.append(-S[a, b])
    idof = (3 * interior[:, None] + np.arange(3)[None, :]).ravel()
    rows.extend(idof.tolist())
    cols.extend((12 + np.arange(n_int)).tolist())
    vals.extend([1.0] * n_int)
    T = sp.coo_matrix((vals, (rows, cols)), shape=(3 * nn, 12 + n_int)).tocsr()
    Kq = (T.T @ K @ T).tocsc()
    Mq = (T.T @ M @ T).tocsc()
    b, i = np.arange(12), 12 + np.arange(n_int)
    Kii, Kib = Kq[i][:, i].tocsc(), Kq[i][:, b].toarray()
    Mii = Mq[i][:, i].tocsc()
    lu = sla.splu(Kii)
    Psi = -lu.solve(Kib)
    if n_modes > 0:
        w2, Phi = sla.eigsh(Kii, k=n_modes, M=Mii, sigma=0.0, which="LM")
        order = np.argsort(w2)
        w2, Phi = w2[order], Phi[:, order]
        Phi = Phi / np.sqrt(np.einsum("ij,ij->j", Phi, Mii @ Phi))
    else:  # static condensation alone (Guyan)
        w2, Phi = np.zeros(0), np.zeros((n_int, 0))
    Tcb = np.zeros((12 + n_int, 12 + n_modes))
    Tcb[:12, :12] = np.eye(12)
    Tcb[12:, :12] = Psi
    Tcb[12:, 12:] = Phi
    Kr = Tcb.T @ (Kq @ Tcb)
    Mr = Tcb.T @ (Mq @ Tcb)
    Kr = 0.5 * (Kr + Kr.T)
    Mr = 0.5 * (Mr + Mr.T)
    # the constraint modes are K-orthogonal to the fixed-interface modes
    Kr[:12, 12:] = 0.0
    Kr[12:, :12] = 0.0
    fg = np.zeros((12 + n_modes, 3))
    for j in range(3):
        r = np.zeros(12 + n_int)
        r[j] = r[6 + j] = 1.0
        r[12:] = np.tile(np.eye(3)[j], len(interior))
        fg[:, j] = Tcb.T @ (Mq @ r)
    return Kr, Mr, fg, w2


_CACHE = {}


def block_part_files(directory, length=2.0, width=0.2, height=0.2, nx=40, ny=4, nz=4, n_modes=30, E=2.1e11,
                     nu=0.3, rho=7850.0, prefix="block"):
    """Reduces the block and writes <prefix>_K.fmx, _M.fmx and _G.fmx into
    `directory`; returns the three paths and the reduced matrices (cached per
    process for equal arguments)."""
    key = (length, width, height, nx, ny, nz, n_modes, E, nu, rho)
    if key not in _CACHE:
        K, M, coords = hex_block(length, width, height, nx, ny, nz, E, nu, rho)
        _CACHE[key] = craig_bampton_two_faces(K, M, coords, length, n_modes)
    Kr, Mr, fg, w2 = _CACHE[key]
    os.makedirs(directory, exist_ok=True)
    paths = {}
    for k, a in (("K", Kr), ("M", Mr), ("G", fg)):
        paths[k] = os.path.join(directory, f"{prefix}_{k}.fmx")
        write_fmx(paths[k], FMX_TAGS[k], a)
    return paths, (Kr, Mr, fg, w2)
