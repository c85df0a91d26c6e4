"""The bounded waits of the step kernels end in an error status, not a hang.

The 3D hydro kernel waits on an mbarrier for each tensor copy with a time
limit (1 s); on expiry it reports EK_DEVERR_TMA_TIMEOUT and leaves.  The
diagnostic entry point runs the same wait on a barrier nothing completes,
with a short limit, so the expiry path runs without any fault.
"""

import pytest

import euler_kokkos_gb300 as ek

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("limit_us", [500, 5000])
def test_mbarrier_wait_expires_and_returns(limit_us):
    expired, elapsed_us = ek.selftest_bounded_wait(limit_us)
    assert expired
    assert limit_us <= elapsed_us < limit_us + 200000  # gave up after the limit, no hang


def test_selftest_arguments_checked():
    with pytest.raises(ek.EkError):
        ek.selftest_bounded_wait(0)


def test_fma_rate_diagnostic():
    # the FLOP roofline's denominators: CUDA-core FMA throughput; GB300 runs
    # FP64 at a small fraction of the FP32 rate
    f32 = ek.measure_fma_rate(ek.EK_PREC_MIXED)
    f64 = ek.measure_fma_rate(ek.EK_PREC_FP64)
    assert 1.0 < f32 < 500.0 and 0.01 < f64 < 100.0
    assert f32 > 8 * f64
