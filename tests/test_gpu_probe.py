"""GPU: the FMA-pipe probe that the FP64 form's compute roofline divides by
measures a plausible rate, and FP32 above FP64 (GB300's FP64 pipe is a small
fraction of its FP32 rate)."""
import pytest

import sks

pytestmark = pytest.mark.gpu


def test_fma_peaks_are_measured():
    p64 = sks.probe_fma_peak(sks.FP64)
    p32 = sks.probe_fma_peak(sks.FP32C)
    assert 0.05 < p64 < 200.0
    assert 1.0 < p32 < 1000.0
    assert p32 > 4 * p64
    with pytest.raises(sks.SksError):
        sks.probe_fma_peak(7)
