"""The results-database reader (fedem_gb300.results.read_results) on files
written here in the layout the GPU writer uses: text header naming the record
layout, then binary records of step (int32), time (float64) and the values
(double or single precision).  No GPU needed."""
import struct

import numpy as np


def _write(path, triads, supels, records, double=True):
    nval = sum(12 if k == "position" else 3 for _, k in triads) + sum(12 + g for _, _, g in supels)
    rec_bytes = 4 + 8 + nval * (8 if double else 4)
    with open(path, "wb") as f:
        f.write(b"#FEDEM results database: primary response\n#model 0\n")
        f.write(f"#precision {'double' if double else 'single'}\n".encode())
        f.write(f"#record bytes {rec_bytes}: step int32, time float64, then in this order:\n".encode())
        for tid, kind in triads:
            f.write(f"#triad {tid} {'position 3x4' if kind == 'position' else 'translation 3'}\n".encode())
        for kind, sid, ng in supels:
            if kind == "beam":
                f.write(f"#supel {sid} frame 3x4\n".encode())
            else:
                f.write(f"#part {sid} frame 3x4 generalized {ng}\n".encode())
        f.write(b"#data\n")
        for step, t, vals in records:
            f.write(struct.pack("<id", step, t))
            f.write(np.asarray(vals, dtype=np.float64 if double else np.float32).tobytes())


def test_reads_positions_and_frames(tmp_path):
    from fedem_gb300.results import read_results

    rng = np.random.default_rng(3)
    triads = [(1, "position"), (2, "position")]
    supels = [("beam", 7, 0)]
    recs = [(k, 0.001 * k, rng.standard_normal(36)) for k in range(5)]
    p = tmp_path / "model0.res"
    _write(p, triads, supels, recs)
    r = read_results(p)
    np.testing.assert_array_equal(r["steps"], np.arange(5))
    np.testing.assert_array_equal(r["times"], [0.001 * k for k in range(5)])
    assert r["triads"] == triads and r["supels"] == supels
    pos = r["triad_positions"]
    assert pos.shape == (5, 2, 3, 4)
    # stored column by column: value 3 c + row is (row, c)
    for k, (_, _, v) in enumerate(recs):
        np.testing.assert_array_equal(pos[k, 1], v[12:24].reshape(4, 3).T)
        np.testing.assert_array_equal(r["beam_frames"][k, 0], v[24:36].reshape(4, 3).T)


def test_single_precision_and_parts(tmp_path):
    from fedem_gb300.results import read_results

    triads = [(4, "position"), (5, "translation")]
    supels = [("part", 1, 6)]
    vals = np.arange(12 + 3 + 18, dtype=np.float64) * 0.5
    p = tmp_path / "model0.res"
    _write(p, triads, supels, [(0, 0.0, vals), (1, 0.25, vals + 1.0)], double=False)
    r = read_results(p)
    assert r["precision"] == "single"
    assert r["values"].shape == (2, 33)
    np.testing.assert_array_equal(r["values"][1], (vals + 1.0).astype(np.float32))
    assert "triad_positions" not in r  # a three-DOF triad in the record
