"""CPU: the band-pass design (SAC's `bp bu co f1 f2 n N`) is the Butterworth
band-pass of the published bilinear design; scipy.signal designs the same
filter independently, so their responses must agree."""
import numpy as np
import pytest

import sks

signal = pytest.importorskip("scipy.signal")


@pytest.mark.parametrize("f_lo,f_hi,poles,dt", [(0.02, 0.5, 2, 0.005), (0.05, 0.3, 4, 0.01), (0.1, 1.0, 3, 0.005),
                                                (0.02, 0.5, 1, 0.05)])
def test_bandpass_response_matches_scipy_butter(f_lo, f_hi, poles, dt):
    ours = sks.bandpass_design(f_lo, f_hi, poles, dt)
    assert ours.shape == (poles, 6)
    ref = signal.butter(poles, [f_lo, f_hi], btype="bandpass", fs=1.0 / dt, output="sos")
    f = np.geomspace(f_lo / 20, min(0.45 / dt, f_hi * 20), 400)
    _, h1 = signal.sosfreqz(ours, worN=f, fs=1.0 / dt)
    _, h2 = signal.sosfreqz(ref, worN=f, fs=1.0 / dt)
    # the same poles and gain; evaluation near z = 1 (poles within 1e-3 of the
    # unit circle) rounds differently for the two numerator factorisations
    assert np.abs(h1 - h2).max() <= 1e-7 * np.abs(h2).max()
    # unit gain at the centre of the band (geometric mean of the prewarped corners)
    fc = np.arctan(np.sqrt(np.tan(np.pi * f_lo * dt) * np.tan(np.pi * f_hi * dt))) / (np.pi * dt)
    _, hc = signal.sosfreqz(ours, worN=[fc], fs=1.0 / dt)
    assert abs(abs(hc[0]) - 1.0) < 1e-9


def test_bandpass_rejects_bad_corners():
    for args in ((0.5, 0.02, 2, 0.005), (0.0, 0.5, 2, 0.005), (0.02, 150.0, 2, 0.005), (0.02, 0.5, 9, 0.005)):
        with pytest.raises(sks.SksError):
            sks.bandpass_design(*args)
