"""Shared helpers of the tests: synthetic cases in temp dirs, error norms."""
import contextlib
import glob
import os

import numpy as np


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a - b))


def seis_err(out, ref) -> float:
    return max(rel_l2(out[i], ref[i]) for i in range(3))


@contextlib.contextmanager
def chdir(d):
    old = os.getcwd()
    os.chdir(d)
    try:
        yield
    finally:
        os.chdir(old)


def solver_fixtures():
    """The golden solver fixtures (tests/golden/*.npz holding a par file),
    sorted; the uvw2sac fixture, which holds none, is left out."""
    out = []
    for p in sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))):
        with np.load(p) as z:
            if "in_run_par" in z.files:
                out.append(p)
    return out
