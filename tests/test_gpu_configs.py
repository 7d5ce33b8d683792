"""GPU parity at the benchmark configurations' own sizes, against the FP64 oracle.

* The plain isotropic P-SV case, whole: 200 x 100 elements of 2 km (801 x 401 =
  321,201 points), crust over mantle, SV plane wave p = 0.045 s/km, Ricker
  0.2 Hz, dt 10 ms, all 6000 steps, 101 surface receivers, P-SV only (the
  reference's `sem2d`).  Seismograms of the FP64 form within relative L2 1e-10
  of the FP64 oracle on every component, the FP32C form within 1e-4.
* The anisotropic 3-component case on its full mesh: 800 x 300 elements of
  1 km (3201 x 1201 = 3,844,401 points), 100 km hexagonal layer (4 %,
  azimuth 45 deg, tilt 20 deg: full c_ij), p = 0.042 s/km, Ricker 0.5 Hz,
  dt 5 ms, 201 receivers, over a window of 240 steps whose boundary records
  start 2 s into the plane wave, so the pulse's main lobe enters the mesh
  inside the window.  The receivers at the surface see almost nothing in
  1.2 s, so the check is on the whole displacement field u^n at the window's
  end: relative L2 of the 3-component field over all points, FP64 within
  1e-10, FP32C within 1e-4; the seismograms must agree to the same fraction of
  the field's peak amplitude.

The oracle needs minutes of CPU at these sizes; both oracle runs start in
threads when the module's fixture is built (ctypes releases the GIL), so they
overlap the GPU solves.
"""
import os
import threading

import numpy as np
import pytest

import sks
import synth
from oracle.oracle import Oracle
from util import rel_l2, seis_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
FP32C_TOL = 1e-4
C1_STEPS = 240
C1_RECORD_T0 = 400          # 2 s of the plane wave at 5 ms: the pulse's main lobe lies in the window
HDR = 88                    # bytes of a saved solver state's header; int32 `cur` at byte 32


class _Background:
    """One oracle solve in a thread: seismograms and, optionally, the final field."""

    def __init__(self, d, nsteps, want_field):
        self.d, self.nsteps, self.want_field = d, nsteps, want_field
        self.result = None
        self.error = None
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()

    def _run(self):
        try:
            # absolute paths: the working directory is the process's, shared with the tests
            o = Oracle([f"par={os.path.join(self.d, 'run.par')}"], fp64=True)
            seis = o.run(self.nsteps)
            field = o.field() if self.want_field else None
            o.close()
            self.result = (seis, field)
        except Exception as e:     # re-raised in the test
            self.error = e

    def get(self):
        self.t.join()
        if self.error:
            raise self.error
        return self.result


@pytest.fixture(scope="module")
def configs(tmp_path_factory):
    c0 = synth.config_isotropic_psv()
    d0 = str(tmp_path_factory.mktemp("c0_iso_psv"))
    synth.write_case(c0, d0, absolute=True)
    c1 = synth.config_aniso_3c(nst=C1_STEPS)
    c1.record_t0 = C1_RECORD_T0
    d1 = str(tmp_path_factory.mktemp("c1_aniso_window"))
    synth.write_case(c1, d1, absolute=True)
    return {"c0": (d0, c0, _Background(d0, c0.nst, False)),
            "c1": (d1, c1, _Background(d1, C1_STEPS, True))}


def _gpu(d, prec, nsteps):
    """Seismograms and the final displacement [nz][nx][3] (x, y, z) of a GPU solve."""
    with sks.Solver([f"par={os.path.join(d, 'run.par')}"], precision=prec, device=0) as s:
        s.load_boundary_files()
        seis = s.run(nsteps)
        info = s.info()
        st = s.save_state()
    nx, nz = info["nx"], info["nz"]
    n = nx * nz
    cur = int(np.frombuffer(st[32:36].tobytes(), np.int32)[0])
    dt = np.float64 if prec == sks.FP64 else np.float32
    el = np.dtype(dt).itemsize
    o = HDR + cur * 3 * n * el
    buf = np.frombuffer(st[o:o + 3 * n * el].tobytes(), dt).astype(np.float64)
    pairs = buf[:2 * n].reshape(n, 2)
    field = np.stack([pairs[:, 0], buf[2 * n:3 * n], pairs[:, 1]], axis=1).reshape(nz, nx, 3)
    return seis, field, info


@pytest.mark.parametrize("prec,tol", [(sks.FP64, FP64_TOL), (sks.FP32C, FP32C_TOL)], ids=["fp64", "fp32c"])
def test_isotropic_psv_whole_solve(configs, prec, tol):
    d, c, bg = configs["c0"]
    out, _, info = _gpu(d, prec, c.nst)
    assert (info["nx"], info["nz"]) == (801, 401) and out[0].shape == (6000, 101)
    ref, _ = bg.get()
    assert max(np.abs(r).max() for r in ref) > 0.1, "the case produced no signal at the receivers"
    err = seis_err(out, ref)
    assert np.isfinite(err) and err <= tol, f"isotropic P-SV, 6000 steps: rel L2 {err:.3e} > {tol:g}"


@pytest.mark.parametrize("prec,tol", [(sks.FP64, FP64_TOL), (sks.FP32C, FP32C_TOL)], ids=["fp64", "fp32c"])
def test_anisotropic_full_mesh_window(configs, prec, tol):
    d, c, bg = configs["c1"]
    out, field, info = _gpu(d, prec, C1_STEPS)
    assert info["nx"] * info["nz"] == 3_844_401 and info["step"] == C1_STEPS
    ref, rfield = bg.get()
    assert np.abs(rfield).max() > 0.1, "the pulse has not entered the mesh"
    err = rel_l2(field, rfield)
    assert np.isfinite(err) and err <= tol, f"field rel L2 {err:.3e} > {tol:g}"
    dev = max(float(np.abs(out[k].astype(np.float64) - ref[k]).max()) for k in range(3))
    assert dev <= tol * np.abs(rfield).max(), f"seismograms differ by {dev:.3e}"
