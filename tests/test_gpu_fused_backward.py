"""The first solve's back substitution runs inside the factorisation's launch
in batches without large fronts (a warp that finds no leaf left serves the
back-substitution queue, waiting for each root's elimination); with
FGPU_NO_FUSED_BACKWARD set at batch creation it is a launch of its own.  Both
give bitwise the same results and iteration counts, in FP64 and in mixed
precision, and the fused batch has one launch fewer per batched iteration."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KNOB = "FGPU_NO_FUSED_BACKWARD"


def _run(cases, mixed, fused):
    from fedem_gb300.batch import Batch, Model

    old = os.environ.pop(KNOB, None)
    try:
        if not fused:
            os.environ[KNOB] = "1"
        b = Batch([Model(f, o) for f, o in cases], mixed=mixed)
    finally:
        os.environ.pop(KNOB, None)
        if old is not None:
            os.environ[KNOB] = old
    st = b.run()
    assert st["models_failed"] == 0
    out = (b.all_triads().copy(), [b.info(k)["iterations"] for k in range(len(cases))], st["kernels_per_iteration"])
    b.close()
    return out


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_fused_back_substitution_gives_the_same_bits(gpu, mixed):
    from fedem_gb300 import models

    cases = [(f, o) for f, o, _ in models.batch_c4(12, seed=23, n_max=2000, steps=40)]
    x1, it1, k1 = _run(cases, mixed, True)
    x0, it0, k0 = _run(cases, mixed, False)
    np.testing.assert_array_equal(x1, x0)
    assert it1 == it0
    assert k1 == k0 - 1
