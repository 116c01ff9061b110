"""The launch-shape autotuner: before a batch's first iteration it times the
candidate shapes of the multifrontal kernels (panel variant of the small-front
factorisation, warps per block of the forward and backward solves, cluster
size of the large-front factorisation) on the batch's own fronts and keeps the
fastest.  Only shapes that leave every result bit unchanged are candidates
(the three panel variants perform the same multiply-subtracts in the same
order), so a batch run with the tuned shapes, with any fixed shape, or with
the shapes reused from an earlier batch of the same structure gives bitwise
the same results.  Checked on beam chains (small fronts only) and on the space-frame
tower (large fronts on clusters), FP64 and mixed precision."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(1, 4, 16, 2), (0, 16, 4, 4), (2, 8, 8, 16)]


def _cases(kind):
    from fedem_gb300 import models

    if kind == "chains":
        return [(f, o) for f, o, _ in models.batch_c4(6, seed=17, n_max=1500, steps=30)]
    return [models.space_frame_c2(steps=6)]


def _run(cases, mixed, shape=None):
    from fedem_gb300.batch import Batch, Model

    b = Batch([Model(f, o) for f, o in cases], mixed=mixed)
    if shape is not None:
        b.set_launch_shape(*shape)
    st = b.run()
    assert st["models_failed"] == 0
    sh, ms, tuned = b.launch_shape()
    out = (b.all_triads().copy(), [b.info(k)["iterations"] for k in range(len(cases))], sh, ms, tuned)
    b.close()
    return out


@pytest.mark.parametrize("kind", ["chains", "space_frame"])
@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_every_shape_gives_the_same_bits(gpu, kind, mixed):
    cases = _cases(kind)
    ref, its, sh, ms, tuned = _run(cases, mixed)
    assert tuned
    assert sh["panel"] in (0, 1, 2) and sh["forward_warps"] in (4, 8, 16)
    assert sh["backward_warps"] in (4, 8, 16) and sh["large_cluster"] in (2, 4, 8, 16)
    for shape in SHAPES:
        x, it, sh2, ms2, tuned2 = _run(cases, mixed, shape)
        assert tuned2 and ms2 == 0.0
        assert (sh2["panel"], sh2["forward_warps"], sh2["backward_warps"], sh2["large_cluster"]) == shape
        np.testing.assert_array_equal(x, ref)
        assert it == its
    # a second batch of the same structure reuses the tuned shapes (no probe)
    x, it, sh3, ms3, _ = _run(cases, mixed)
    assert sh3 == sh and ms3 == 0.0
    np.testing.assert_array_equal(x, ref)


def test_shape_is_fixed_once_iterating(gpu):
    from fedem_gb300 import FedemException
    from fedem_gb300.batch import Batch, Model

    f, o = _cases("chains")[0]
    b = Batch([Model(f, o)], mixed=True)
    with pytest.raises(FedemException):
        b.set_launch_shape(0, 3, 8, 8)  # 3 warps per block is not a candidate
    b.run(max_batched=3)
    with pytest.raises(FedemException):
        b.set_launch_shape(0, 8, 8, 8)
    b.close()
