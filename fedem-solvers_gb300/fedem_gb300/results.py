"""Reader of the results database files the GPU solver core writes
(fgpu_batch_results_open): a text header naming the record layout, then one
binary record per saved state -- step (int32), time (float64), the triads'
position matrices (3 x 4, column by column; the translation only for triads
with three DOFs), the beam superelements' frames (3 x 4) and the reduced
parts' frames and generalized DOF values -- in the precision the header names.
The record contents and order follow the reference's primary response output
(src/vpmSolver/saveModule.f90:615-663)."""
import numpy as np


def read_results(path):
    """Returns a dict: steps (int array), times, triads (list of (id, kind)),
    supels (list of (kind, id, ngen)), values (records x values array in the
    file's precision, converted to float64), and per-object views:
    triad_positions (records x triads-with-6-DOFs x 3 x 4, column-major as
    stored, i.e. [..., row, column]) when every saved triad has six DOFs."""
    with open(path, "rb") as f:
        blob = f.read()
    end = blob.index(b"#data\n") + len(b"#data\n")
    header = blob[:end].decode().splitlines()
    data = blob[end:]
    precision, rec_bytes = "double", None
    triads, supels = [], []
    for line in header:
        w = line[1:].split()
        if not w:
            continue
        if w[0] == "precision":
            precision = w[1]
        elif w[0] == "record" and w[1] == "bytes":
            rec_bytes = int(w[2].rstrip(":"))
        elif w[0] == "triad":
            triads.append((int(w[1]), w[2]))
        elif w[0] == "supel":
            supels.append(("beam", int(w[1]), 0))
        elif w[0] == "part":
            supels.append(("part", int(w[1]), int(w[w.index("generalized") + 1])))
    vt = np.float64 if precision == "double" else np.float32
    nval = (rec_bytes - 12) // np.dtype(vt).itemsize
    rec = np.dtype([("step", "<i4"), ("time", "<f8"), ("v", vt, (nval,))])
    arr = np.frombuffer(data, dtype=rec, count=len(data) // rec_bytes)
    out = {"steps": arr["step"].astype(np.int64), "times": arr["time"].astype(np.float64),
           "triads": triads, "supels": supels, "values": arr["v"].astype(np.float64), "precision": precision}
    if triads and all(k == "position" for _, k in triads):
        nt = len(triads)
        # stored column by column: value 3 c + r is (row r, column c)
        out["triad_positions"] = out["values"][:, :12 * nt].reshape(-1, nt, 4, 3).transpose(0, 1, 3, 2)
    nb = sum(1 for s in supels if s[0] == "beam")
    if nb and not any(s[0] == "part" for s in supels):
        off = 12 * len(triads) if triads and all(k == "position" for _, k in triads) else None
        if off is not None:
            out["beam_frames"] = out["values"][:, off:off + 12 * nb].reshape(-1, nb, 4, 3).transpose(0, 1, 3, 2)
    return out
