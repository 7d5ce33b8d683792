"""ORACLE binding — test infrastructure, not product code.

ctypes access to the C restatement in oracle/sem_oracle.c (built by
oracle/Makefile).  Only tests/, the smoke entry and bench.py's CPU-baseline
leg use it, as the checker.

    from oracle import Oracle
    o = Oracle(["par=run.par"], fp64=True)
    u, v, w = o.run(o.nst)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")


def build(reference_root: str | None = None, with_reference: bool = True) -> None:
    """Compile the restatement; with_reference: also the reference binaries
    (oracle/_ref) where the reference's sources are present.  Their location:
    reference_root, else $SKS_REFERENCE_ROOT, else the Makefile's default."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True, capture_output=True)
    if not with_reference:
        return
    root = reference_root or os.environ.get("SKS_REFERENCE_ROOT")
    cmd = ["make", "-s", "-C", HERE, "ref-if-present"] + ([f"REF={root}"] if root else [])
    subprocess.run(cmd, check=True, capture_output=True)


_libs: dict = {}


def _lib(fp64: bool) -> C.CDLL:
    key = "liboracle64.so" if fp64 else "liboracle32.so"
    if key not in _libs:
        path = os.path.join(BUILD, key)
        if not os.path.exists(path):
            build(with_reference=False)
        L = C.CDLL(path)
        L.oracle_create.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
        L.oracle_create.restype = C.c_void_p
        L.oracle_dims.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
        L.oracle_eh.argtypes = [C.c_void_p]
        L.oracle_eh.restype = C.c_double
        L.oracle_run.argtypes = [C.c_void_p, C.c_int] + [C.POINTER(C.c_float)] * 3
        L.oracle_material.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.oracle_mass.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.oracle_receivers.argtypes = [C.c_void_p, C.POINTER(C.c_longlong)]
        L.oracle_field.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.oracle_snapshot.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_int)]
        L.oracle_destroy.argtypes = [C.c_void_p]
        L.oracle_destroy.restype = None
        L.oracle_last_error.restype = C.c_char_p
        _libs[key] = L
    return _libs[key]


class Oracle:
    def __init__(self, words, fp64: bool = True):
        self.L = _lib(fp64)
        w = ["oracle"] + [str(x) for x in words]
        arr = (C.c_char_p * len(w))(*[x.encode() for x in w])
        self.h = self.L.oracle_create(len(w), arr)
        if not self.h:
            raise RuntimeError("oracle: " + self.L.oracle_last_error().decode())
        d = (C.c_int * 8)()
        self.L.oracle_dims(self.h, d)
        self.nx, self.nz, self.nez, self.ntrace, self.nst, self.nt_sem, self.mtotal, self.shtotal = list(d)
        self.eh = self.L.oracle_eh(self.h)

    def run(self, nsteps: int):
        out = [np.zeros((nsteps, max(1, self.ntrace)), np.float32) for _ in range(3)]
        p = [o.ctypes.data_as(C.POINTER(C.c_float)) for o in out]
        n = self.L.oracle_run(self.h, nsteps, *p)
        if n < 0:
            raise RuntimeError("oracle: " + self.L.oracle_last_error().decode())
        return tuple(o[:n, : self.ntrace] for o in out)

    def material(self) -> np.ndarray:
        out = np.zeros((self.nx * self.nz, 16))
        self.L.oracle_material(self.h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def mass(self):
        n = self.nx * self.nz
        m, ab = np.zeros(n), np.zeros(3 * n)
        self.L.oracle_mass(self.h, m.ctypes.data_as(C.POINTER(C.c_double)), ab.ctypes.data_as(C.POINTER(C.c_double)))
        return m, ab.reshape(n, 3)

    def receivers(self) -> np.ndarray:
        off = np.zeros(max(1, self.ntrace), np.int64)
        self.L.oracle_receivers(self.h, off.ctypes.data_as(C.POINTER(C.c_longlong)))
        return off[: self.ntrace]

    def field(self) -> np.ndarray:
        """The newest displacement u^n as [nz][nx][3] float64 (x, y, z components)."""
        out = np.zeros(self.nx * self.nz * 3)
        self.L.oracle_field(self.h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out.reshape(self.nz, self.nx, 3)

    def snapshot(self, k: int):
        """(step, [nx/2][nz/2][2] float32) of snapshot k (plot_snap), or None."""
        dims = (C.c_int * 2)()
        self.L.oracle_snapshot(self.h, k, None, dims)
        out = np.zeros((dims[0], dims[1], 2), np.float32)
        st = self.L.oracle_snapshot(self.h, k, out.ctypes.data_as(C.POINTER(C.c_float)), dims)
        return None if st < 0 else (st, out)

    def close(self):
        if self.h:
            self.L.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
