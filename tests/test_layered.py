"""CPU: plane waves through a layered stack (sks_layered_coefficients,
sks_layered_series), the boundary-trace producer for layered structure below
the box.  The reference's generator is a ray sum with a Fortran core that does
not build here (semsyn/src/aser.rout_noplot.f), so nothing pins these numbers
to it; they are checked against what the physics fixes:
- a stack of identical media passes the wave unchanged;
- energy flux is conserved at every frequency (all modes propagate);
- a single SH layer over a half-space has a closed form (transmission through
  two interfaces times the reverberation series);
- vertical incidence does not convert P and SV, and SV then behaves as SH;
- a single interface has frequency-independent coefficients, so the series is
  the Ricker pulse scaled.
"""
import math

import numpy as np
import pytest

import sks
import synth

A = (8.1, 4.5, 3.4)           # mantle-like half-space
T = (7.6, 4.3, 3.3)           # the box's bottom medium
B = (6.5, 3.7, 2.9, 20.0)
C3 = (7.4, 4.1, 3.2, 35.0)
STACKS = [[T, A], [T, B, A], [T, B, C3, A], [T, (5.8, 3.2, 2.6, 3.0), B, C3, (9.0, 5.0, 3.6, 50.0), A]]


def _eta(v, p):
    return math.sqrt(1.0 / v ** 2 - p ** 2)


@pytest.mark.parametrize("stack", STACKS, ids=lambda s: f"{len(s)}media")
def test_energy_flux_is_conserved(stack):
    top, hs = stack[0], stack[-1]
    for p in (0.0, 0.021, 0.042, 0.06):
        for w in (0.0, 0.7, 3.1, 12.0, 55.0):
            c = sks.layered_coefficients(stack, p, w)
            for inc in (0, 1):
                vin = hs[0] if inc == 0 else hs[1]
                f_in = hs[2] * vin ** 2 * _eta(vin, p)
                f_out = sum(top[2] * v ** 2 * _eta(v, p) * abs(c["t_psv"][m, inc]) ** 2 +
                            hs[2] * u ** 2 * _eta(u, p) * abs(c["r_psv"][m, inc]) ** 2
                            for m, (v, u) in enumerate(((top[0], hs[0]), (top[1], hs[1]))))
                assert abs(f_out / f_in - 1.0) < 1e-12, (p, w, inc)
            f_in = hs[2] * hs[1] ** 2 * _eta(hs[1], p)
            f_out = (top[2] * top[1] ** 2 * _eta(top[1], p) * abs(c["t_sh"]) ** 2 +
                     hs[2] * hs[1] ** 2 * _eta(hs[1], p) * abs(c["r_sh"]) ** 2)
            assert abs(f_out / f_in - 1.0) < 1e-12, (p, w)


def test_identical_media_pass_the_wave_unchanged():
    same = [A, A + (10.0,), A + (7.0,), A]
    for p in (0.0, 0.04):
        for w in (0.0, 2.0, 30.0):
            c = sks.layered_coefficients(same, p, w)
            assert np.allclose(c["t_psv"], np.eye(2), rtol=0, atol=1e-13)
            assert np.abs(c["r_psv"]).max() < 1e-13
            assert abs(c["t_sh"] - 1.0) < 1e-13 and abs(c["r_sh"]) < 1e-13


def test_sh_layer_closed_form():
    for p in (0.0, 0.035):
        for w in (0.5, 2.7, 9.0):
            def z(m):
                return m[2] * m[1] ** 2 * _eta(m[1], p)
            h = B[3]
            t_ab = 2 * z(A) / (z(A) + z(B))
            t_bt = 2 * z(B) / (z(B) + z(T))
            r_bt = (z(B) - z(T)) / (z(B) + z(T))
            r_ba = (z(B) - z(A)) / (z(B) + z(A))
            ph = np.exp(-1j * w * _eta(B[1], p) * h)
            want = t_ab * t_bt * ph / (1 - r_bt * r_ba * ph * ph) * np.exp(1j * w * _eta(A[1], p) * h)
            got = sks.layered_coefficients([T, B, A], p, w)["t_sh"]
            assert abs(got - want) < 1e-13 * abs(want), (p, w)


def test_vertical_incidence_does_not_convert():
    for stack in STACKS[1:]:
        c = sks.layered_coefficients(stack, 0.0, 3.0)
        assert abs(c["t_psv"][0, 1]) < 1e-14 and abs(c["t_psv"][1, 0]) < 1e-14
        assert abs(c["t_psv"][1, 1] - c["t_sh"]) < 1e-13


@pytest.mark.parametrize("f0", [0.5, 1.5])
def test_series_of_one_interface_is_the_scaled_pulse(f0):
    p, dt = 0.042, 0.00125
    s = sks.layered_series([T, A], p, f0, dt, 40.0, p_amp=0.4, sv_amp=1.0, sh_amp=0.7)
    c = sks.layered_coefficients([T, A], p, 1.0)
    assert abs(c["t_psv"][1, 1].imag) < 1e-15 and abs(c["t_psv"][0, 1].imag) < 1e-15
    t = np.arange(s.shape[1]) * dt
    r = synth.ricker(t - 1.5 / f0, f0)
    want = [0.4 * c["t_psv"][0, 0].real + c["t_psv"][0, 1].real,
            0.4 * c["t_psv"][1, 0].real + c["t_psv"][1, 1].real, 0.7 * c["t_sh"].real]
    for m in range(3):
        assert np.abs(s[m] - want[m] * r).max() < 1e-7, m


def test_series_of_identical_media_is_the_pulse():
    f0, dt = 0.5, 0.00125
    s = sks.layered_series([A, A + (30.0,), A], 0.04, f0, dt, 120.0, p_amp=0.3, sv_amp=1.0, sh_amp=0.7)
    assert s.shape[1] & (s.shape[1] - 1) == 0
    r = synth.ricker(np.arange(s.shape[1]) * dt - 1.5 / f0, f0)
    for m, a in enumerate((0.3, 1.0, 0.7)):
        assert np.abs(s[m] - a * r).max() < 1e-7


def test_layered_series_delays_and_reverberates():
    """A slow layer delays the transmitted SH pulse by its extra vertical
    time, and its first reverberation follows one two-way time later with
    the sign and size of r_bt * r_ba."""
    p, f0, dt = 0.03, 1.0, 0.001
    s = sks.layered_series([T, B, A], p, f0, dt, 60.0, sv_amp=0.0, sh_amp=1.0)[2]
    t = np.arange(s.size) * dt
    lag = B[3] * (_eta(B[1], p) - _eta(A[1], p))
    direct = synth.ricker(t - 1.5 / f0 - lag, f0)
    k = np.dot(s, direct) / np.dot(direct, direct)

    def z(m):
        return m[2] * m[1] ** 2 * _eta(m[1], p)
    t_ab = 2 * z(A) / (z(A) + z(B))
    t_bt = 2 * z(B) / (z(B) + z(T))
    assert abs(k - t_ab * t_bt) < 2e-3
    two_way = 2 * B[3] * _eta(B[1], p)
    rev = synth.ricker(t - 1.5 / f0 - lag - two_way, f0)
    r_bt = (z(B) - z(T)) / (z(B) + z(T))
    r_ba = (z(B) - z(A)) / (z(B) + z(A))
    k2 = np.dot(s, rev) / np.dot(rev, rev)
    assert abs(k2 - t_ab * t_bt * r_bt * r_ba) < 2e-3 * abs(t_ab * t_bt)


def test_refusals():
    good = [T, B, A]
    for bad, p in (([T], 0.04), (good, 1.0 / 6.4), ([T, (3.0, 4.0, 3.0, 5.0), A], 0.04),
                   ([T, (6.5, 3.7, 2.9, 0.0), A], 0.04), ([T, (6.5, 3.7, -1.0, 5.0), A], 0.04), (good, -0.01)):
        with pytest.raises(sks.SksError):
            sks.layered_coefficients(bad, p, 1.0)
    with pytest.raises(sks.SksError):
        sks.layered_series(good, 0.04, 0.0, 0.001, 10.0)
