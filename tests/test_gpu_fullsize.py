"""GPU: size-independent properties of the solve at the benchmark sizes.

The oracle finishes in seconds only on small meshes, so at the full sizes of
the benchmark workloads -- the 800 x 300-element anisotropic mesh
(3,844,401 points) and the 4000 x 1000-element mesh (64,020,001 points) --
the checks are properties that hold at any size, on the whole saved wavefield
(both displacement buffers and, for FP32C, the (d, c) state):

* linearity: the wavefield of a plane wave with amplitudes (2, -0.5) equals
  2 x (1, 0) - 0.5 x (0, 1) to the form's rounding (relative L2 <= 1e-10 for
  FP64, <= 1e-4 for FP32C: the parity bars);
* a run split across calls equals one run, bit for bit, and repeats bit for bit;
* FP32C against FP64: relative L2 of the displacement <= 1e-4.
"""
import tempfile

import numpy as np
import pytest

import sks
import synth
from util import chdir

pytestmark = pytest.mark.gpu

HDR = 88            # bytes of the saved-state header
STEPS = 800         # 4 s at 5 ms: the Ricker pulse has entered the mesh


@pytest.fixture(scope="module")
def c1_dir():
    with tempfile.TemporaryDirectory() as d:
        c = synth.config_aniso_3c(nst=STEPS + 10)
        c.write_records = False
        summ = synth.write_case(c, d)
        yield d, c, summ


def _solve(d, c, summ, prec, amps, splits=(STEPS,)):
    with chdir(d):
        s = sks.Solver(["par=run.par"], precision=prec)
    s.set_boundary_plane_wave(summ["vs"], c.p, c.f0, amps[0], amps[1])
    for n in splits:
        assert sks.lib().sks_run(s.h, n, None, None, None) == n     # no seismograms copied out
    st = s.save_state()
    info = s.info()
    s.close()
    return st, info


def _fields(state, info, prec):
    """(U0, U1, d) of a saved state as float64 arrays; d is None for FP64."""
    np_ = info["nx"] * info["nz"]
    dt = np.float64 if prec == sks.FP64 else np.float32
    el = np.dtype(dt).itemsize
    o = HDR
    u0 = np.frombuffer(state[o:o + 3 * np_ * el].tobytes(), dt).astype(np.float64)
    o += 3 * np_ * el
    u1 = np.frombuffer(state[o:o + 3 * np_ * el].tobytes(), dt).astype(np.float64)
    o += 3 * np_ * el
    d = None
    if prec == sks.FP32C:
        dc = np.frombuffer(state[o:o + 6 * np_ * el].tobytes(), np.float32).astype(np.float64)
        d = dc[0::2]                       # (d, c) pairs: the increment, then its compensation
    return u0, u1, d


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("prec,tol", [(sks.FP64, 1e-10), (sks.FP32C, 1e-4)])
def test_linearity_in_the_incident_wave(c1_dir, prec, tol):
    d, c, summ = c1_dir
    sa, info = _solve(d, c, summ, prec, (1.0, 0.0))
    sb, _ = _solve(d, c, summ, prec, (0.0, 1.0))
    sc, _ = _solve(d, c, summ, prec, (2.0, -0.5))
    fa, fb, fc = (_fields(x, info, prec) for x in (sa, sb, sc))
    assert info["step"] == STEPS
    for i in range(3):
        if fc[i] is None:
            continue
        assert np.linalg.norm(fc[i]) > 0
        assert np.linalg.norm(fa[i]) > 0 and np.linalg.norm(fb[i]) > 0
        assert _rel(2.0 * fa[i] - 0.5 * fb[i], fc[i]) <= tol, (prec, i)


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C])
def test_split_runs_and_repeats_are_bit_identical(c1_dir, prec):
    d, c, summ = c1_dir
    one, _ = _solve(d, c, summ, prec, (1.0, 0.4))
    again, _ = _solve(d, c, summ, prec, (1.0, 0.4))
    split, _ = _solve(d, c, summ, prec, (1.0, 0.4), splits=(1, 63, 300, STEPS - 364))
    assert np.array_equal(one, again)
    assert np.array_equal(one, split)


def test_fp32c_tracks_fp64_on_the_whole_wavefield(c1_dir):
    d, c, summ = c1_dir
    s64, info = _solve(d, c, summ, sks.FP64, (1.0, 0.4))
    s32, _ = _solve(d, c, summ, sks.FP32C, (1.0, 0.4))
    f64 = _fields(s64, info, sks.FP64)
    f32 = _fields(s32, info, sks.FP32C)
    for i in range(2):
        assert np.linalg.norm(f64[i]) > 0
        assert _rel(f32[i], f64[i]) <= 1e-4, i


def test_largest_mesh_split_run_is_bit_identical():
    """The 64,020,001-point mesh (4000 x 1000 elements of 250 m), FP32C: a run
    split across calls equals one run, and the wavefield is finite and moving."""
    with tempfile.TemporaryDirectory() as d:
        c = synth.config_large(nst=520)
        c.write_records = False
        summ = synth.write_case(c, d)
        one, info = _solve(d, c, summ, sks.FP32C, (1.0, 0.3), splits=(500,))
        split, _ = _solve(d, c, summ, sks.FP32C, (1.0, 0.3), splits=(170, 330))
        assert info["nx"] * info["nz"] == 64020001
        assert np.array_equal(one, split)
        u0, u1, dd = _fields(one, info, sks.FP32C)
        assert np.isfinite(u0).all() and np.isfinite(u1).all() and np.isfinite(dd).all()
        assert np.abs(dd).max() > 0
