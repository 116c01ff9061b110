"""fgpu_batch_norms_noalloc (convergence norms into a fixed scratch array,
no device allocation) against fgpu_batch_get_norms, the norms the batch's own
pass stored, both through the C ABI.  The file name keeps it last in
collection; it needs nothing from the other test files."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# same chunks, thread mapping, expressions, reduction order and weight sums as
# the batch's own norms pass: the values are compared bit for bit


def _norms(lib, batch, model, noalloc):
    out = np.full(18, np.nan)
    fn = lib.fgpu_batch_norms_noalloc if noalloc else lib.fgpu_batch_get_norms
    rc = fn(batch._h, model, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert rc == 0, lib.fgpu_last_error().decode()
    return out


def _close(a, b):
    return np.array_equal(a, b, equal_nan=True)


def test_noalloc_norms_match_stored_norms_on_two_calls_in_a_row(gpu):
    from fedem_gb300 import load_library, models
    from fedem_gb300.batch import Batch, Model

    lib = load_library()
    # a 20-beam cantilever and a 3000-beam chain (18,006 DOFs: 9 norm chunks)
    fsi1, opts = models.cantilever_c1()
    fsi2 = models.beam_chain_fsi(3000, 0.25, 0.1, 0.01, clamp=0, load_node=3000, load_dof=2, load=1000.0,
                                 **models.STEEL)
    ms = [Model(fsi1, opts), Model(fsi2, opts)]
    for mixed in (False, True):
        b = Batch(ms, mixed=mixed)
        for _ in range(3):
            for k in range(len(ms)):
                b.step(k)
                ref = _norms(lib, b, k, noalloc=False)
                first = _norms(lib, b, k, noalloc=True)
                second = _norms(lib, b, k, noalloc=True)
                assert np.all(np.isfinite(ref)) and ref[0] > 0.0
                assert _close(first, ref), (k, first, ref)
                assert _close(second, ref), (k, second, ref)
        b.close()


def test_noalloc_norms_refuse_models_above_the_scratch_limit(gpu):
    from fedem_gb300 import load_library, models
    from fedem_gb300.batch import Batch, Model

    lib = load_library()
    fsi, opts = models.cantilever_c1()
    big = models.beam_chain_fsi(90000, 0.25, 0.1, 0.01, clamp=0, load_node=90000, load_dof=2, load=1000.0,
                                **models.STEEL)  # 540,006 DOFs > 524,288
    b = Batch([Model(fsi, opts), Model(big, opts)])
    out = np.zeros(18)
    rc = lib.fgpu_batch_norms_noalloc(b._h, 1, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert rc != 0
    assert "524,288" in lib.fgpu_last_error().decode()
    # the small model of the same batch still works after the refusal
    b.step(0)
    assert _close(_norms(lib, b, 0, noalloc=True), _norms(lib, b, 0, noalloc=False))
    b.close()


def test_noalloc_norms_keep_a_nan_like_the_stored_norms(gpu):
    """A model whose residual turned NaN (NaN point load): the batch's stored
    norms carry the NaN in its maxima, and the no-allocation norms are the
    same values, NaN in the same places."""
    from fedem_gb300 import load_library, models
    from fedem_gb300.batch import Batch, Model

    lib = load_library()
    fsi, opts = models.cantilever_c1()
    bad = models.beam_chain_fsi(3000, 0.25, 0.1, 0.01, clamp=0, load_node=3000, load_dof=2, load=1000.0,
                                **models.STEEL).replace("f0 = ", "f0 = nan ! ", 1)
    b = Batch([Model(fsi, opts), Model(bad, opts)])
    b.step(1)
    ref = _norms(lib, b, 1, noalloc=False)
    assert np.isnan(ref).any()
    assert _close(_norms(lib, b, 1, noalloc=True), ref)
    assert _close(_norms(lib, b, 1, noalloc=True), ref)
    b.close()
