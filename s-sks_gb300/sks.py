"""Python binding of the C ABI in include/sks.h (ctypes, no torch types).

    import sks
    with sks.Setup(["par=run.par"]) as su:          # host-only set-up
        info = su.info()
    s = sks.Solver(["par=run.par"], precision=sks.FP32C)
    s.load_boundary_files()
    u, v, w = s.run(s.info()["nst"])               # seismograms [nst, ntrace]

The library is the in-tree build s-sks_gb300/_build/libsks_gb300.so; there is
no fallback: a missing library raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

FP64 = 0
FP32C = 1

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libsks_gb300.so")

ERRORS = {0: "OK", -1: "ERR_ARG", -2: "ERR_IO", -3: "ERR_MODEL", -4: "ERR_UNSUPPORTED", -5: "ERR_CUDA",
          -6: "ERR_NOMEM", -7: "ERR_BOUNDARY", -8: "ERR_STATE", -9: "ERR_NONFINITE"}

EXPORTS = ["sks_open_par", "sks_load_boundary_files", "sks_set_boundary", "sks_run", "sks_reset",
           "sks_wavefield_finite", "sks_test_stall_pipeline", "sks_batch_test_stall_pipeline",
           "sks_get_info", "sks_setup_open", "sks_setup_info", "sks_setup_material", "sks_setup_mass",
           "sks_setup_receivers", "sks_setup_schedule", "sks_setup_close", "sks_open_setup",
           "sks_kernel_launches", "sks_last_run_ms", "sks_enable_kernel_timing", "sks_kernel_timing",
           "sks_probe_fma_peak",
           "sks_set_tuning", "sks_get_tuning", "sks_autotune", "sks_line_increments",
           "sks_line_increments_noalloc", "sks_set_boundary_plane_wave", "sks_snapshot",
           "sks_layered_coefficients", "sks_layered_series_length", "sks_layered_series",
           "sks_set_boundary_layered_wave",
           "sks_state_bytes", "sks_state_save", "sks_state_load",
           "sks_elastic_rotate", "sks_elastic_dip", "sks_christoffel", "sks_semmodel_write",
           "sks_bandpass_design", "sks_split_scratch", "sks_split_traces",
           "sks_sac_fields_init", "sks_sac_write", "sks_uvw2sac",
           "sks_batch_create", "sks_batch_add", "sks_batch_remove", "sks_batch_size", "sks_batch_run",
           "sks_batch_set_tuning", "sks_batch_get_tuning", "sks_batch_autotune", "sks_batch_last_run_ms",
           "sks_batch_kernel_launches", "sks_batch_destroy",
           "sks_server_create", "sks_server_set_tuning", "sks_server_set_active_points", "sks_server_submit", "sks_server_submit_layered", "sks_server_step",
           "sks_server_request_info", "sks_server_release", "sks_server_clock", "sks_server_device_bytes",
           "sks_server_destroy",
           "sks_destroy", "sks_last_error"]

KERNEL_CLASSES = ["element", "seam", "inject", "record", "interp"]


class SksError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Info(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("nex", "nez", "hpn", "nx", "nz", "nst", "nt_inject", "ntrace",
                                         "mtotal", "shtotal", "nrec_psv", "nrec_sh", "nmat", "anisotropic",
                                         "precision", "step")] + \
               [("eh", C.c_double), ("h", C.c_double), ("sdt", C.c_double), ("device_bytes", C.c_int64),
                ("seam_points", C.c_int64), ("tile_rows", C.c_int32), ("neh", C.c_int32), ("iso_rows", C.c_int32)]

    def asdict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3


class RequestInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("status", C.c_int32), ("precision", C.c_int32), ("step", C.c_int32),
                ("nst", C.c_int32), ("ntrace", C.c_int32), ("submit_s", C.c_double), ("admit_s", C.c_double),
                ("done_s", C.c_double), ("device_bytes", C.c_int64)]

    def asdict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Layer(C.Structure):
    _fields_ = [("c", C.c_double * 36), ("rho", C.c_double), ("npts", C.c_int32),
                ("x", C.POINTER(C.c_double)), ("z", C.POINTER(C.c_double))]


class SplitOpts(C.Structure):
    _fields_ = [("f_lo", C.c_double), ("f_hi", C.c_double), ("poles", C.c_int32), ("passes", C.c_int32),
                ("before", C.c_double), ("after", C.c_double), ("max_delay", C.c_double), ("dphi", C.c_double)]


class PlaneWave(C.Structure):
    _fields_ = [("vs", C.c_double), ("p", C.c_double), ("f0", C.c_double), ("sv_amp", C.c_double),
                ("sh_amp", C.c_double)]


class StackLayer(C.Structure):
    _fields_ = [("vp", C.c_double), ("vs", C.c_double), ("rho", C.c_double), ("thickness", C.c_double)]


class LayeredWave(C.Structure):
    _fields_ = [("p", C.c_double), ("f0", C.c_double), ("p_amp", C.c_double), ("sv_amp", C.c_double),
                ("sh_amp", C.c_double)]


class LayeredCoef(C.Structure):
    _fields_ = [("t_psv", C.c_double * 8), ("r_psv", C.c_double * 8), ("t_sh", C.c_double * 2),
                ("r_sh", C.c_double * 2)]


class SacFields(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("delta", "b", "e", "o", "evla", "evlo", "evdp", "stla", "stlo", "stel",
                                          "gcarc", "cmpaz", "cmpinc")] + \
               [(n, C.c_int32) for n in ("nzyear", "nzjday", "nzhour", "nzmin", "nzsec", "nzmsec")] + \
               [("kstnm", C.c_char * 9)]


class Tuning(C.Structure):
    _fields_ = [("warps_per_block", C.c_int32), ("band_rows", C.c_int32), ("zseam", C.c_int32),
                ("register_cap", C.c_int32), ("waves", C.c_int32), ("blocks", C.c_int32),
                ("ms_per_step", C.c_float), ("pipeline", C.c_int32)]

    def asdict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} is not built; run s-sks_gb300/sks_build.py")
        L = C.CDLL(LIB_PATH)
        vp, ip, dp, fp = C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_double), C.POINTER(C.c_float)
        argv_t = C.POINTER(C.c_char_p)
        L.sks_open_par.argtypes = [C.c_int, argv_t, C.c_int, C.c_int, C.POINTER(vp)]
        L.sks_load_boundary_files.argtypes = [vp]
        L.sks_set_boundary.argtypes = [vp, fp, C.c_int32, fp, C.c_int32]
        L.sks_run.argtypes = [vp, C.c_int32, fp, fp, fp]
        L.sks_reset.argtypes = [vp]
        L.sks_wavefield_finite.argtypes = [vp]
        L.sks_test_stall_pipeline.argtypes = [vp, C.c_int32, C.c_int32]
        L.sks_batch_test_stall_pipeline.argtypes = [vp, C.c_int32, C.c_int32]
        L.sks_get_info.argtypes = [vp, C.POINTER(Info)]
        L.sks_setup_open.argtypes = [C.c_int, argv_t, C.POINTER(vp)]
        L.sks_setup_info.argtypes = [vp, C.POINTER(Info)]
        L.sks_setup_material.argtypes = [vp, dp]
        L.sks_setup_mass.argtypes = [vp, dp, dp]
        L.sks_setup_receivers.argtypes = [vp, C.POINTER(C.c_int64)]
        L.sks_setup_schedule.argtypes = [vp, ip, dp, ip, dp]
        L.sks_setup_close.argtypes = [vp]
        L.sks_setup_close.restype = None
        L.sks_open_setup.argtypes = [vp, C.c_int, C.c_int, C.POINTER(vp)]
        L.sks_kernel_launches.argtypes = [vp]
        L.sks_kernel_launches.restype = C.c_int64
        L.sks_last_run_ms.argtypes = [vp]
        L.sks_last_run_ms.restype = C.c_double
        L.sks_enable_kernel_timing.argtypes = [vp, C.c_int]
        L.sks_kernel_timing.argtypes = [vp, dp, C.POINTER(C.c_int64)]
        L.sks_probe_fma_peak.argtypes = [C.c_int, C.c_int, dp]
        L.sks_sac_fields_init.argtypes = [C.POINTER(SacFields)]
        L.sks_sac_fields_init.restype = None
        L.sks_sac_write.argtypes = [C.c_char_p, C.c_int32, C.POINTER(C.c_float), C.POINTER(SacFields)]
        L.sks_uvw2sac.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.c_char_p]
        L.sks_set_tuning.argtypes = [vp, C.POINTER(Tuning)]
        L.sks_get_tuning.argtypes = [vp, C.POINTER(Tuning)]
        L.sks_autotune.argtypes = [vp, C.c_int32, C.POINTER(Tuning)]
        L.sks_line_increments.argtypes = [vp, C.c_int32, C.c_int32, dp]
        L.sks_line_increments_noalloc.argtypes = [vp, vp, C.c_int32, C.c_int32, C.c_int32, vp, vp, vp, vp,
                                                  C.c_int32, vp, vp]
        L.sks_set_boundary_plane_wave.argtypes = [vp, C.POINTER(PlaneWave)]
        L.sks_layered_coefficients.argtypes = [C.POINTER(StackLayer), C.c_int32, C.c_double, C.c_double,
                                               C.POINTER(LayeredCoef)]
        L.sks_layered_series_length.argtypes = [C.POINTER(StackLayer), C.c_int32, C.c_double, C.c_double,
                                                C.c_double, C.c_double]
        L.sks_layered_series_length.restype = C.c_int64
        L.sks_layered_series.argtypes = [C.POINTER(StackLayer), C.c_int32, C.POINTER(LayeredWave), C.c_double,
                                         C.c_int64, dp]
        L.sks_set_boundary_layered_wave.argtypes = [vp, C.POINTER(StackLayer), C.c_int32, C.POINTER(LayeredWave)]
        L.sks_snapshot.argtypes = [vp, C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_int32)]
        L.sks_elastic_rotate.argtypes = [dp, C.c_double, dp]
        L.sks_elastic_dip.argtypes = [dp, C.c_double, dp]
        L.sks_christoffel.argtypes = [dp, C.c_double, dp, dp]
        L.sks_semmodel_write.argtypes = [C.c_char_p, C.c_int32, C.POINTER(Layer), C.c_int32]
        L.sks_bandpass_design.argtypes = [C.c_double, C.c_double, C.c_int32, C.c_double, dp]
        L.sks_split_scratch.argtypes = [C.c_int32, C.c_int32, C.c_double, C.POINTER(SplitOpts),
                                        C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.sks_split_traces.argtypes = [vp, vp, C.c_int32, C.c_int32, C.c_int64, C.c_double, C.POINTER(SplitOpts),
                                       vp, vp, vp, vp]
        L.sks_state_bytes.argtypes = [vp]
        L.sks_state_bytes.restype = C.c_int64
        L.sks_state_save.argtypes = [vp, vp, C.c_int64]
        L.sks_state_load.argtypes = [vp, vp, C.c_int64]
        L.sks_destroy.argtypes = [vp]
        L.sks_destroy.restype = None
        fpp = C.POINTER(C.POINTER(C.c_float))
        L.sks_batch_create.argtypes = [C.c_int, C.c_int, C.POINTER(vp)]
        L.sks_batch_add.argtypes = [vp, vp]
        L.sks_batch_remove.argtypes = [vp, vp]
        L.sks_batch_size.argtypes = [vp]
        L.sks_batch_run.argtypes = [vp, C.c_int32, fpp, fpp, fpp]
        L.sks_batch_set_tuning.argtypes = [vp, C.POINTER(Tuning)]
        L.sks_batch_get_tuning.argtypes = [vp, C.POINTER(Tuning)]
        L.sks_batch_autotune.argtypes = [vp, C.c_int32, C.POINTER(Tuning)]
        L.sks_batch_last_run_ms.argtypes = [vp]
        L.sks_batch_last_run_ms.restype = C.c_double
        L.sks_batch_kernel_launches.argtypes = [vp]
        L.sks_batch_kernel_launches.restype = C.c_int64
        L.sks_batch_destroy.argtypes = [vp]
        L.sks_batch_destroy.restype = None
        L.sks_server_create.argtypes = [C.c_int, C.c_int64, C.c_int32, C.POINTER(vp)]
        L.sks_server_set_tuning.argtypes = [vp, C.c_int, C.POINTER(Tuning)]
        L.sks_server_set_active_points.argtypes = [vp, C.c_int, C.c_int64]
        L.sks_server_submit.argtypes = [vp, vp, C.c_int, C.POINTER(PlaneWave), fp, fp, fp, C.POINTER(C.c_int64)]
        L.sks_server_submit_layered.argtypes = [vp, vp, C.c_int, C.POINTER(StackLayer), C.c_int32,
                                                C.POINTER(LayeredWave), fp, fp, fp, C.POINTER(C.c_int64)]
        L.sks_server_step.argtypes = [vp]
        L.sks_server_request_info.argtypes = [vp, C.c_int64, C.POINTER(RequestInfo)]
        L.sks_server_release.argtypes = [vp, C.c_int64]
        L.sks_server_clock.argtypes = [vp]
        L.sks_server_clock.restype = C.c_double
        L.sks_server_device_bytes.argtypes = [vp]
        L.sks_server_device_bytes.restype = C.c_int64
        L.sks_server_destroy.argtypes = [vp]
        L.sks_server_destroy.restype = None
        L.sks_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def _check(rc: int) -> int:
    if rc < 0:
        raise SksError(rc, lib().sks_last_error().decode())
    return rc


def _argv(words) -> tuple:
    words = ["sks"] + [str(w) for w in words]
    arr = (C.c_char_p * len(words))(*[w.encode() for w in words])
    return len(words), arr


def _f32(a):
    return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None


class Setup:
    """Host-only set-up of a par file (mesh, materials, mass, receivers, schedule)."""

    def __init__(self, words):
        self.h = C.c_void_p()
        n, arr = _argv(words)
        _check(lib().sks_setup_open(n, arr, C.byref(self.h)))

    def info(self) -> dict:
        i = Info()
        _check(lib().sks_setup_info(self.h, C.byref(i)))
        return i.asdict()

    def material(self) -> np.ndarray:
        i = self.info()
        out = np.zeros((i["nx"] * i["nz"], 16))
        _check(lib().sks_setup_material(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def mass(self):
        i = self.info()
        np_ = i["nx"] * i["nz"]
        m = np.zeros(np_)
        ab = np.zeros(3 * np_)
        _check(lib().sks_setup_mass(self.h, m.ctypes.data_as(C.POINTER(C.c_double)),
                                    ab.ctypes.data_as(C.POINTER(C.c_double))))
        return m, ab.reshape(np_, 3)

    def receivers(self) -> np.ndarray:
        off = np.zeros(max(1, self.info()["ntrace"]), dtype=np.int64)
        _check(lib().sks_setup_receivers(self.h, off.ctypes.data_as(C.POINTER(C.c_int64))))
        return off[: self.info()["ntrace"]]

    def schedule(self):
        n = self.info()["nt_inject"]
        tp, ts = np.zeros(4 * n + 1, np.int32), np.zeros(4 * n + 1, np.int32)
        wp, ws = np.zeros(4 * n + 1), np.zeros(4 * n + 1)
        ip, dp = C.POINTER(C.c_int32), C.POINTER(C.c_double)
        _check(lib().sks_setup_schedule(self.h, tp.ctypes.data_as(ip), wp.ctypes.data_as(dp),
                                        ts.ctypes.data_as(ip), ws.ctypes.data_as(dp)))
        return (tp[:4 * n].reshape(n, 4), wp[:4 * n].reshape(n, 4),
                ts[:4 * n].reshape(n, 4), ws[:4 * n].reshape(n, 4))

    def close(self):
        if self.h:
            lib().sks_setup_close(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver:
    """Device solver of one par file (sks_open_par), or of an open Setup
    (sks_open_setup, which takes the set-up over)."""

    def __init__(self, words=None, precision: int = FP64, device: int = 0, setup: "Setup | None" = None):
        self.h = C.c_void_p()
        if setup is not None:
            h, setup.h = setup.h, C.c_void_p()
            _check(lib().sks_open_setup(h, precision, device, C.byref(self.h)))
        else:
            n, arr = _argv(words)
            _check(lib().sks_open_par(n, arr, precision, device, C.byref(self.h)))

    def info(self) -> dict:
        i = Info()
        _check(lib().sks_get_info(self.h, C.byref(i)))
        return i.asdict()

    def load_boundary_files(self):
        _check(lib().sks_load_boundary_files(self.h))

    def set_boundary(self, psv: np.ndarray, sh: np.ndarray | None):
        psv = np.ascontiguousarray(psv, dtype=np.float32)
        i = self.info()
        nps = psv.size // max(1, i["mtotal"])
        if sh is not None:
            sh = np.ascontiguousarray(sh, dtype=np.float32)
            nsh = sh.size // max(1, i["shtotal"])
        else:
            nsh = 0
        _check(lib().sks_set_boundary(self.h, _f32(psv), nps, _f32(sh), nsh))

    def set_boundary_plane_wave(self, vs: float, p: float, f0: float, sv_amp: float = 1.0, sh_amp: float = 0.0):
        pw = PlaneWave(vs, p, f0, sv_amp, sh_amp)
        _check(lib().sks_set_boundary_plane_wave(self.h, C.byref(pw)))

    def set_boundary_layered_wave(self, layers, p: float, f0: float, p_amp: float = 0.0, sv_amp: float = 1.0,
                                  sh_amp: float = 0.0):
        """layers: (vp, vs, rho, thickness) from the box's bottom medium down to the half-space."""
        st = _stack(layers)
        w = LayeredWave(p, f0, p_amp, sv_amp, sh_amp)
        _check(lib().sks_set_boundary_layered_wave(self.h, st, len(layers), C.byref(w)))

    def run(self, nsteps: int, out=None):
        nt = self.info()["ntrace"]
        if out is None:
            out = tuple(np.zeros((nsteps, max(nt, 0)), np.float32) for _ in range(3))
        u, v, w = out
        n = _check(lib().sks_run(self.h, nsteps, _f32(u), _f32(v), _f32(w)))
        return u[:n], v[:n], w[:n]

    def reset(self):
        _check(lib().sks_reset(self.h))

    def wavefield_finite(self) -> bool:
        """False once a step produced a non-finite displacement (until reset)."""
        return _check(lib().sks_wavefield_finite(self.h)) == 1

    def test_stall_pipeline(self, tile: int, spin_limit: int):
        """Failure-path tests only: the next run's pipelined wait on `tile` runs out."""
        _check(lib().sks_test_stall_pipeline(self.h, tile, spin_limit))

    def save_state(self) -> np.ndarray:
        n = _check(lib().sks_state_bytes(self.h))
        buf = np.zeros(n, np.uint8)
        _check(lib().sks_state_save(self.h, buf.ctypes.data_as(C.c_void_p), n))
        return buf

    def load_state(self, buf: np.ndarray):
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        _check(lib().sks_state_load(self.h, buf.ctypes.data_as(C.c_void_p), buf.size))

    def snapshot(self, k: int):
        """(step, [nx/2][nz/2][2] float32 of (u_x, u_y)) of snapshot k, or None when not taken."""
        dims = (C.c_int32 * 2)()
        lib().sks_snapshot(self.h, k, None, dims)
        out = np.zeros((dims[0], dims[1], 2), np.float32)
        st = lib().sks_snapshot(self.h, k, out.ctypes.data_as(C.POINTER(C.c_float)), dims)
        return None if st < 0 else (st, out)

    def nline(self) -> int:
        i = self.info()
        nbl = i["neh"] * i["hpn"]
        return (i["nx"] - nbl) + (i["nz"] - nbl - 1)

    def line_increments(self, it0: int, nsteps: int) -> np.ndarray:
        """FP64 boundary increments g(it+1)-g(it) of steps [it0, it0+nsteps): [nsteps, nline, 3]."""
        out = np.zeros((nsteps, self.nline(), 3))
        _check(lib().sks_line_increments(self.h, it0, nsteps, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def tuning(self) -> dict:
        t = Tuning()
        _check(lib().sks_get_tuning(self.h, C.byref(t)))
        return t.asdict()

    def set_tuning(self, warps_per_block: int, band_rows: int, zseam: int = 1, register_cap: int = 0,
                   waves: int = 0, pipeline: int = 0):
        t = Tuning(warps_per_block, band_rows, zseam, register_cap, waves, 0, 0.0, pipeline)
        _check(lib().sks_set_tuning(self.h, C.byref(t)))

    def autotune(self, steps: int = 8) -> dict:
        t = Tuning()
        _check(lib().sks_autotune(self.h, steps, C.byref(t)))
        return t.asdict()

    def launches(self) -> int:
        return lib().sks_kernel_launches(self.h)

    def last_run_ms(self) -> float:
        return lib().sks_last_run_ms(self.h)

    def enable_kernel_timing(self, on: bool = True):
        _check(lib().sks_enable_kernel_timing(self.h, 1 if on else 0))

    def kernel_timing(self) -> dict:
        ms = (C.c_double * 5)()
        cnt = (C.c_int64 * 5)()
        _check(lib().sks_kernel_timing(self.h, ms, cnt))
        return {k: (ms[i], cnt[i]) for i, k in enumerate(KERNEL_CLASSES)}

    def close(self):
        if self.h:
            lib().sks_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Solvers of one form advanced together (sks_batch_*)."""

    def __init__(self, precision: int = FP32C, device: int = 0):
        self.h = C.c_void_p()
        _check(lib().sks_batch_create(precision, device, C.byref(self.h)))
        self.members: list[Solver] = []

    def add(self, s: Solver):
        _check(lib().sks_batch_add(self.h, s.h))
        self.members.append(s)

    def remove(self, s: Solver):
        _check(lib().sks_batch_remove(self.h, s.h))
        self.members.remove(s)

    def __len__(self) -> int:
        return _check(lib().sks_batch_size(self.h))

    def run(self, nsteps: int, want: bool = True, status: bool = False):
        """Advance every member; returns per member (u, v, w) of the rows it took
        (with status=True: (that list, the call's status) instead of raising)."""
        infos = [m.info() for m in self.members]
        n = len(self.members)
        fpp = C.POINTER(C.c_float) * max(1, n)
        outs, arrs = [], [fpp(), fpp(), fpp()]
        for i, inf in enumerate(infos):
            rows = max(0, min(inf["nst"], inf["step"] + nsteps) - inf["step"])
            o = tuple(np.zeros((rows, max(inf["ntrace"], 0)), np.float32) for _ in range(3))
            outs.append(o)
            for c in range(3):
                arrs[c][i] = _f32(o[c]) if want and o[c].size else None
        rc = lib().sks_batch_run(self.h, nsteps, arrs[0], arrs[1], arrs[2])
        if status:
            return outs, rc
        _check(rc)
        return outs

    def test_stall_pipeline(self, tile: int, spin_limit: int):
        """Failure-path tests only: the next run's pipelined wait on `tile` runs out."""
        _check(lib().sks_batch_test_stall_pipeline(self.h, tile, spin_limit))

    def tuning(self) -> dict:
        t = Tuning()
        _check(lib().sks_batch_get_tuning(self.h, C.byref(t)))
        return t.asdict()

    def set_tuning(self, warps_per_block: int, band_rows: int, zseam: int = 0, register_cap: int = 1,
                   pipeline: int = 0):
        t = Tuning(warps_per_block, band_rows, zseam, register_cap, 0, 0, 0.0, pipeline)
        _check(lib().sks_batch_set_tuning(self.h, C.byref(t)))

    def autotune(self, steps: int = 4) -> dict:
        t = Tuning()
        _check(lib().sks_batch_autotune(self.h, steps, C.byref(t)))
        return t.asdict()

    def last_run_ms(self) -> float:
        return lib().sks_batch_last_run_ms(self.h)

    def launches(self) -> int:
        return lib().sks_batch_kernel_launches(self.h)

    def close(self):
        if self.h:
            lib().sks_batch_destroy(self.h)
            self.h = C.c_void_p()
        self.members = []

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """The serving loop (sks_server_*): submit() from any thread, step() in a loop."""

    def __init__(self, device: int = 0, budget: int = 0, quantum: int = 64):
        self.h = C.c_void_p()
        _check(lib().sks_server_create(device, budget, quantum, C.byref(self.h)))
        self.outputs: dict[int, tuple] = {}

    def set_tuning(self, precision: int, warps_per_block: int, band_rows: int, zseam: int, register_cap: int,
                   pipeline: int = 0):
        t = Tuning(warps_per_block, band_rows, zseam, register_cap, 0, 0, 0.0, pipeline)
        _check(lib().sks_server_set_tuning(self.h, precision, C.byref(t)))

    def set_active_points(self, precision: int, max_points: int):
        _check(lib().sks_server_set_active_points(self.h, precision, max_points))

    def submit(self, setup: "Setup", precision: int, plane_wave: tuple | None = None, want: bool = True,
               layered: tuple | None = None) -> int:
        """plane_wave = (vs, p, f0, sv_amp, sh_amp); layered = (layers, p, f0, p_amp, sv_amp, sh_amp) with
        layers as for Solver.set_boundary_layered_wave; neither: the par's boundary files."""
        i = setup.info()
        out = tuple(np.zeros((i["nst"], max(i["ntrace"], 0)), np.float32) for _ in range(3)) if want else None
        pw = C.byref(PlaneWave(*plane_wave)) if plane_wave is not None else None
        h, setup.h = setup.h, C.c_void_p()
        rid = C.c_int64()
        ptrs = [_f32(o) for o in out] if out else [None, None, None]
        if layered is not None:
            layers, wave = layered[0], LayeredWave(*layered[1:])
            _check(lib().sks_server_submit_layered(self.h, h, precision, _stack(layers), len(layers), C.byref(wave),
                                                   ptrs[0], ptrs[1], ptrs[2], C.byref(rid)))
        else:
            _check(lib().sks_server_submit(self.h, h, precision, pw, ptrs[0], ptrs[1], ptrs[2], C.byref(rid)))
        self.outputs[rid.value] = out
        return rid.value

    def step(self) -> int:
        return _check(lib().sks_server_step(self.h))

    def info(self, rid: int) -> dict:
        r = RequestInfo()
        _check(lib().sks_server_request_info(self.h, rid, C.byref(r)))
        return r.asdict()

    def result(self, rid: int):
        return self.outputs[rid]

    def release(self, rid: int):
        _check(lib().sks_server_release(self.h, rid))
        self.outputs.pop(rid, None)

    def clock(self) -> float:
        return lib().sks_server_clock(self.h)

    def device_bytes(self) -> int:
        return lib().sks_server_device_bytes(self.h)

    def close(self):
        if self.h:
            lib().sks_server_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- model builder --------------------------------------------------------
def sac_write(path: str, data, **fields):
    """One SAC file (sks_sac_write): header fields by name (SacFields), the rest unset."""
    f = SacFields()
    lib().sks_sac_fields_init(C.byref(f))
    for k, v in fields.items():
        setattr(f, k, v.encode() if k == "kstnm" else v)
    a = np.ascontiguousarray(data, dtype=np.float32)
    _check(lib().sks_sac_write(path.encode(), a.size, a.ctypes.data_as(C.POINTER(C.c_float)), C.byref(f)))


def uvw2sac(words, directory: str | None = None):
    """The uvw2sac program (sks_uvw2sac) on par words, reading seis.u/v/w in `directory`."""
    n, arr = _argv(words)
    _check(lib().sks_uvw2sac(n, arr, directory.encode() if directory else None))


def probe_fma_peak(precision: int, device: int = 0) -> float:
    """Measured peak FMA throughput of the device's CUDA cores (TFLOP/s) for the FP64 or FP32 pipe."""
    t = C.c_double(0.0)
    _check(lib().sks_probe_fma_peak(device, precision, C.byref(t)))
    return t.value


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _stack(layers):
    st = (StackLayer * len(layers))()
    for i, l in enumerate(layers):
        vp, vs, rho = l[0], l[1], l[2]
        st[i] = StackLayer(vp, vs, rho, l[3] if len(l) > 3 else 0.0)
    return st


def layered_coefficients(layers, p: float, omega: float) -> dict:
    """Plane-wave coefficients of a layered stack at angular frequency omega:
    t_psv/r_psv [out][in] (0 = P, 1 = SV) complex 2x2, t_sh, r_sh complex."""
    c = LayeredCoef()
    _check(lib().sks_layered_coefficients(_stack(layers), len(layers), p, omega, C.byref(c)))
    t = np.array(c.t_psv[:]).reshape(2, 2, 2)
    r = np.array(c.r_psv[:]).reshape(2, 2, 2)
    return {"t_psv": t[..., 0] + 1j * t[..., 1], "r_psv": r[..., 0] + 1j * r[..., 1],
            "t_sh": c.t_sh[0] + 1j * c.t_sh[1], "r_sh": c.r_sh[0] + 1j * c.r_sh[1]}


def layered_series(layers, p: float, f0: float, dt: float, span: float, p_amp: float = 0.0, sv_amp: float = 1.0,
                   sh_amp: float = 0.0) -> np.ndarray:
    """Upgoing P, SV, SH series (3, nt) at the base of the top medium, sample i at i*dt (periodic)."""
    st = _stack(layers)
    nt = lib().sks_layered_series_length(st, len(layers), p, f0, dt, span)
    _check(int(nt) if nt < 0 else 0)
    out = np.zeros(3 * nt)
    w = LayeredWave(p, f0, p_amp, sv_amp, sh_amp)
    _check(lib().sks_layered_series(st, len(layers), C.byref(w), dt, nt, _d(out)))
    return out.reshape(3, nt)


def elastic_rotate(c, angle_deg: float) -> np.ndarray:
    """6x6 Voigt matrix in axes turned by angle_deg about x3 (new x1 from old x1, counter-clockwise)."""
    c = np.ascontiguousarray(c, dtype=np.float64).reshape(6, 6)
    out = np.zeros((6, 6))
    _check(lib().sks_elastic_rotate(_d(c), angle_deg, _d(out)))
    return out


def elastic_dip(c, angle_deg: float) -> np.ndarray:
    """6x6 Voigt matrix in axes turned by angle_deg about x2 (new x1 from old x1 toward old x3)."""
    c = np.ascontiguousarray(c, dtype=np.float64).reshape(6, 6)
    out = np.zeros((6, 6))
    _check(lib().sks_elastic_dip(_d(c), angle_deg, _d(out)))
    return out


def christoffel(c, rho: float, direction) -> np.ndarray:
    """Phase velocities (descending) along direction."""
    c = np.ascontiguousarray(c, dtype=np.float64).reshape(6, 6)
    n = np.ascontiguousarray(direction, dtype=np.float64)
    v = np.zeros(3)
    _check(lib().sks_christoffel(_d(c), rho, _d(n), _d(v)))
    return v


def semmodel_write(path: str, layers, full: bool = True):
    """layers: (c 6x6, rho, x control points, z heights) bottom to top."""
    keep = []
    arr = (Layer * len(layers))()
    for i, (c, rho, x, z) in enumerate(layers):
        x = np.ascontiguousarray(x, dtype=np.float64)
        z = np.ascontiguousarray(z, dtype=np.float64)
        keep += [x, z]
        arr[i].c[:] = list(np.asarray(c, dtype=np.float64).reshape(36))
        arr[i].rho = rho
        arr[i].npts = len(x)
        arr[i].x = _d(x)
        arr[i].z = _d(z)
    _check(lib().sks_semmodel_write(path.encode(), len(layers), arr, 1 if full else 0))


# ---- post-processing ------------------------------------------------------
def bandpass_design(f_lo: float, f_hi: float, poles: int, dt: float) -> np.ndarray:
    """Second-order sections [poles][6] (b0 b1 b2 1 a1 a2) of the Butterworth band-pass."""
    sos = np.zeros((max(1, poles), 6))
    n = _check(lib().sks_bandpass_design(f_lo, f_hi, poles, dt, _d(sos)))
    return sos[:n]


def split_traces_device(radial_ptr: int, transverse_ptr: int, ntrace: int, nt: int, ld: int, dt: float,
                        opts: SplitOpts, work_ptr: int, sums_ptr: int, out_ptr: int, stream: int = 0):
    """sks_split_traces on device pointers (integers, e.g. torch data_ptr())."""
    _check(lib().sks_split_traces(C.c_void_p(radial_ptr), C.c_void_p(transverse_ptr), ntrace, nt, ld, dt,
                                  C.byref(opts), C.c_void_p(work_ptr), C.c_void_p(sums_ptr), C.c_void_p(out_ptr),
                                  C.c_void_p(stream)))


def split_scratch(ntrace: int, nt: int, dt: float, opts: SplitOpts):
    w, s = C.c_int64(), C.c_int64()
    _check(lib().sks_split_scratch(ntrace, nt, dt, C.byref(opts), C.byref(w), C.byref(s)))
    return w.value, s.value
