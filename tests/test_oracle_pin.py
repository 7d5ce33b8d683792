"""The oracle pinned to the reference (CPU).

Golden fixtures (tests/golden/*.npz) hold inputs and the seismograms the
REFERENCE binaries (compiled from the reference sources, see
tests/golden/make_golden.py) wrote for them.  The float build of the oracle
must reproduce them bit for bit; the FP64 build must stay within the FP32
rounding noise of the reference.  Known answers of the GLL tables close the
set.
"""
import os
import tempfile

import numpy as np
import pytest

from golden.make_golden import extract
from oracle.oracle import Oracle
from util import chdir, rel_l2, solver_fixtures

GOLDEN = solver_fixtures()
# relative L2 of FP64 against the float reference: the reference's own FP32
# rounding (measured 2e-6 .. 1e-5 on these cases)
FP32_NOISE = 5e-5


def _run(path, fp64):
    with tempfile.TemporaryDirectory() as d:
        z = extract(path, d)
        nt, nst = int(z["ntrace"]), int(z["nst"])
        words = ["par=run.par"] + (["psv_only=1"] if str(z["prog"]) == "sem2d" else [])
        with chdir(d):
            o = Oracle(words, fp64=fp64)
            out = o.run(nst)
            o.close()
        gold = [z["seis_" + x].reshape(nst, nt) for x in "uvw"]
    return out, gold


def test_golden_fixtures_present():
    assert len(GOLDEN) >= 5


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_float_oracle_is_bit_exact_to_reference(path):
    out, gold = _run(path, fp64=False)
    for i, c in enumerate("uvw"):
        assert out[i].shape == gold[i].shape
        assert np.array_equal(out[i].view(np.uint32), gold[i].view(np.uint32)), f"seis.{c} differs"
    assert max(np.abs(g).max() for g in gold) > 1.0, "fixture carries no signal"


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_fp64_oracle_within_reference_rounding(path):
    out, gold = _run(path, fp64=True)
    for i in range(3):
        assert rel_l2(out[i], gold[i]) <= FP32_NOISE


def test_gll_known_answers():
    # N=4: points {+-1, +-sqrt(3/7), 0}, weights {1/10, 49/90, 32/45}
    import sks
    with tempfile.TemporaryDirectory() as d:
        z = extract(GOLDEN[0], d)
        with chdir(d), sks.Setup(["par=run.par"]) as su:
            info = su.info()
            mass, _ = su.mass()
            mat = su.material()
    # mass sums to rho * area of the box (lumped GLL mass integrates rho exactly)
    rho = mat[:, 15].reshape(info["nz"], info["nx"])
    H, W = info["nez"] * info["eh"], info["nex"] * info["eh"]
    assert abs(mass.sum() - _gll_integral(rho, info)) <= 1e-12 * mass.sum()
    assert mass.min() > 0
    assert W > 0 and H > 0
    del z


def _gll_integral(rho, info):
    """Tensor-product GLL quadrature of rho over the box, element by element."""
    N = info["hpn"]
    w = np.array([0.1, 49 / 90, 32 / 45, 49 / 90, 0.1]) if N == 4 else None
    Je = info["eh"] ** 2 / 4
    tot = 0.0
    for ez in range(info["nez"]):
        for ex in range(info["nex"]):
            blk = rho[ez * N:ez * N + N + 1, ex * N:ex * N + N + 1]
            tot += Je * float(w @ blk @ w)
    return tot


def test_derivative_matrix_known_answers():
    """l'_i(xi_j) from the oracle's own restatement reproduces exact derivatives
    of polynomials up to degree N and its rows sum to zero."""
    xi = np.array([-1.0, -np.sqrt(3 / 7), 0.0, np.sqrt(3 / 7), 1.0])
    N = 4
    D = np.zeros((N + 1, N + 1))
    for i in range(N + 1):
        down = np.prod([xi[i] - xi[k] for k in range(N + 1) if k != i])
        for j in range(N + 1):
            s = 0.0
            for q in range(N + 1):
                if q == i:
                    continue
                s += np.prod([xi[j] - xi[k] for k in range(N + 1) if k not in (i, q)])
            D[j, i] = s / down
    assert np.allclose(D.sum(1), 0, atol=1e-13)
    for k in range(N + 1):
        assert np.allclose(D @ xi ** k, k * xi ** max(k - 1, 0) if k else 0, atol=1e-12)


def _snap_fixtures():
    out = []
    for p in GOLDEN:
        z = np.load(p)
        if "snap_out1" in z.files:
            out.append(p)
    return out


SNAP = _snap_fixtures()


@pytest.mark.parametrize("path", SNAP, ids=[os.path.basename(p)[:-4] for p in SNAP])
def test_float_oracle_snapshot_files_are_the_references(path):
    """The oracle's program writes out1..outK byte for byte as the reference did."""
    import subprocess
    exe = os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle", "_build", "oracle_sem2d_psvsh32")
    with tempfile.TemporaryDirectory() as d:
        z = extract(path, d)
        words = ["par=run.par"] + str(z["words"]).split()
        r = subprocess.run([exe] + words, cwd=d, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        k = 1
        while f"snap_out{k}" in z.files:
            with open(os.path.join(d, f"out{k}"), "rb") as f:
                assert f.read() == z[f"snap_out{k}"].tobytes(), f"out{k} differs"
            k += 1
        assert k > 5
        assert not os.path.exists(os.path.join(d, f"out{k}"))


def test_snapshot_fixture_present():
    assert SNAP
