"""CPU: the Silver-Chan splitting estimate recovers known splitting parameters."""
import numpy as np
import pytest

import splitting
import synth


@pytest.mark.parametrize("phi,delay", [(45.0, 1.0), (-30.0, 0.6), (10.0, 1.75), (-80.0, 0.35)])
def test_recovers_imposed_splitting(phi, delay):
    dt = 0.01
    t = np.arange(6000) * dt
    radial = synth.ricker(t - 25.0, 0.3)           # SKS arrives radially polarised
    x, y = splitting.apply_splitting(radial, np.zeros_like(radial), phi, delay, dt)
    w = splitting.sks_window(x, dt, 12.0)
    r = splitting.splitting(x, y, dt, w, max_delay=3.0, dphi=0.25)
    assert abs(r["phi_deg"] - phi) <= 0.5
    assert abs(r["delay_s"] - delay) <= 2 * dt
    assert r["lambda_ratio"] < 1e-3


def test_unsplit_wave_has_no_transverse_energy_to_remove():
    dt = 0.01
    t = np.arange(4000) * dt
    x = synth.ricker(t - 20.0, 0.3)
    y = np.zeros_like(x)
    r = splitting.splitting(x, y, dt, splitting.sks_window(x, dt, 10.0))
    # with no transverse energy, lambda2 vanishes for the null directions (delay 0, or phi along x or y)
    assert r["lambda_ratio"] < 1e-12
    assert r["delay_s"] == 0.0 or abs(abs(r["phi_deg"]) % 90.0) < 1e-9


def test_window_is_checked():
    with pytest.raises(ValueError):
        splitting.splitting(np.zeros(10), np.zeros(10), 0.1, (5, 20))
