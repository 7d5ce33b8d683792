"""Golden vectors of the reference's model tools (semsyn/model/src/elastic_rotate.c
and elastic_dip.c): their rotate() on seeded 6x6 Voigt matrices and angles.

The tools are compiled from the reference sources into oracle/_ref/libela_rotate.so
and libela_dip.so (`make -C oracle ref`; their main() renamed).  rotate() is a
K&R definition, so its float angle arrives as a double.

    python tests/golden/make_golden_elastic.py
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REFBIN = os.path.join(ROOT, "oracle", "_ref")
PAIR = [(0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1)]


def reference_rotate(lib_name: str, c: np.ndarray, angle: float) -> np.ndarray:
    lib = C.CDLL(os.path.join(REFBIN, lib_name))
    f = lib.rotate
    f.restype = C.c_float
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float), C.c_double]
    cf = np.ascontiguousarray(c, dtype=np.float32)
    out = np.zeros((6, 6), np.float32)
    for jk, (j, k) in enumerate(PAIR):
        for mn, (m, n) in enumerate(PAIR):
            out[jk, mn] = f(j, k, m, n, cf.ctypes.data_as(C.POINTER(C.c_float)), float(np.float32(angle)))
    return out


def inputs(seed: int = 11, n: int = 6):
    rng = np.random.default_rng(seed)
    mats, angles = [], []
    for _ in range(n):
        a = rng.uniform(-30, 30, (6, 6))
        m = a @ a.T / 6 + np.diag(rng.uniform(50, 250, 6))     # symmetric positive definite
        mats.append(m.astype(np.float32).astype(np.float64))
        angles.append(float(np.float32(rng.uniform(-180, 180))))
    return np.array(mats), np.array(angles)


if __name__ == "__main__":
    if not os.path.exists(os.path.join(REFBIN, "libela_rotate.so")):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    mats, angles = inputs()
    rot = np.array([reference_rotate("libela_rotate.so", m, a) for m, a in zip(mats, angles)])
    dip = np.array([reference_rotate("libela_dip.so", m, a) for m, a in zip(mats, angles)])
    np.savez_compressed(os.path.join(HERE, "model", "elastic_tools.npz"), mats=mats, angles=angles, rotate=rot, dip=dip)
    print("elastic_tools", mats.shape, rot.shape, dip.shape)
