"""The measured peaks the bench quotes kernels against: the FP64 FMA rate and
the TF32 rate of mma.sync m16n8k8.  Both come from timed kernels of the
library itself; the test checks that they run and give plausible GB300-class
figures (no exact value: clocks vary)."""
import pytest

pytestmark = pytest.mark.gpu


def test_fp64_peak_is_plausible(gpu_lib):
    from fedem_gb300.batch import measure_fp64_peak

    tf, ms = measure_fp64_peak(gpu_lib)
    assert ms > 0.0
    assert 0.1 < tf < 100.0


def test_tf32_mma_peak_is_plausible(gpu_lib):
    from fedem_gb300.batch import measure_tf32_mma_peak

    tf, ms = measure_tf32_mma_peak(gpu_lib)
    assert ms > 0.0
    # far above the FP64 rate, below the tcgen05 dense TF32 figure
    assert 5.0 < tf < 2000.0
