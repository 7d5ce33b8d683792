"""CPU: the model builder (FP64 tensor rotations, Christoffel velocities, SEM
model writer) against the reference's model tools and known answers."""
import os

import numpy as np
import pytest

import sks
import synth
from golden import make_golden_elastic as mge
from util import chdir

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = np.load(os.path.join(ROOT, "tests", "golden", "model", "elastic_tools.npz"))
HAVE_REF = os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libela_rotate.so"))


def _close_to_float_reference(ours, ref):
    # the reference sums 81 float products per entry
    return np.abs(ours - ref).max() <= 2e-6 * np.abs(ref).max() * 81 ** 0.5


def test_rotations_match_the_reference_golden_vectors():
    for m, a, r, d in zip(GOLD["mats"], GOLD["angles"], GOLD["rotate"], GOLD["dip"]):
        assert _close_to_float_reference(sks.elastic_rotate(m, a), r)
        assert _close_to_float_reference(sks.elastic_dip(m, a), d)


@pytest.mark.skipif(not HAVE_REF, reason="reference model tools not built here")
def test_rotations_match_the_reference_tools():
    mats, angles = mge.inputs(seed=5, n=4)
    for m, a in zip(mats, angles):
        assert _close_to_float_reference(sks.elastic_rotate(m, a), mge.reference_rotate("libela_rotate.so", m, a))
        assert _close_to_float_reference(sks.elastic_dip(m, a), mge.reference_rotate("libela_dip.so", m, a))


def test_rotation_identities():
    m = GOLD["mats"][0]
    assert np.allclose(sks.elastic_rotate(m, 360.0), m, rtol=0, atol=1e-11 * np.abs(m).max())
    assert np.allclose(sks.elastic_rotate(sks.elastic_rotate(m, 37.0), -37.0), m, rtol=0, atol=1e-11 * np.abs(m).max())
    assert np.allclose(sks.elastic_dip(sks.elastic_dip(m, 12.5), -12.5), m, rtol=0, atol=1e-11 * np.abs(m).max())
    iso = synth.iso_cij(8.1, 4.5, 3.4)
    assert np.allclose(sks.elastic_rotate(sks.elastic_dip(iso, 23.0), 71.0), iso, rtol=0, atol=1e-11 * iso.max())


@pytest.mark.parametrize("az,tilt", [(45.0, 20.0), (0.0, 0.0), (130.0, 35.0), (-60.0, 10.0)])
def test_tilted_hexagonal_is_dip_then_rotate(az, tilt):
    """An axis at azimuth az, tilted up by tilt: dip the axis-aligned tensor by
    -tilt, then rotate by -az (the tools turn the axes, not the medium)."""
    h0 = synth.hexagonal_cij(8.1, 4.5, 3.4, 0.05, 0.0, 0.0)
    want = synth.hexagonal_cij(8.1, 4.5, 3.4, 0.05, az, tilt)
    got = sks.elastic_rotate(sks.elastic_dip(h0, -tilt), -az)
    assert np.allclose(got, want, rtol=0, atol=1e-10 * np.abs(want).max())


def test_christoffel_velocities():
    assert np.allclose(sks.christoffel(synth.iso_cij(8.1, 4.5, 3.4), 3.4, [0.3, -0.2, 1.0]), [8.1, 4.5, 4.5])
    h = synth.hexagonal_cij(8.1, 4.5, 3.4, 0.04, 0.0, 0.0)
    assert np.allclose(sks.christoffel(h, 3.4, [1, 0, 0]), [8.1 * 1.02, 4.5 * 1.02, 4.5 * 1.02])
    assert np.allclose(sks.christoffel(h, 3.4, [0, 0, 2]), [8.1 * 0.98, 4.5 * 1.02, 4.5 * 0.98])
    rng = np.random.default_rng(3)
    m = GOLD["mats"][2]
    for _ in range(5):
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        t = np.zeros((3, 3))
        V = [[0, 5, 4], [5, 1, 3], [4, 3, 2]]
        for i in range(3):
            for k in range(3):
                t[i, k] = sum(m[V[i][j], V[k][l]] * n[j] * n[l] for j in range(3) for l in range(3)) / 3.3
        want = np.sqrt(np.sort(np.linalg.eigvalsh(t))[::-1])
        assert np.allclose(sks.christoffel(m, 3.3, n), want, rtol=1e-12)
    with pytest.raises(sks.SksError):
        sks.christoffel(m, 3.3, [0, 0, 0])


@pytest.mark.parametrize("full", [True, False])
def test_semmodel_written_is_what_the_solver_reads(tmp_path, full):
    d = str(tmp_path)
    H = 16.002
    tilt = 25.0 if full else 0.0           # the 13-constant form cannot hold a tilted axis
    layers = [synth.SemLayer(H - 6, synth.iso_cij(8.1, 4.5, 3.4), 3.4),
              synth.SemLayer(H - 3, synth.hexagonal_cij(8.1, 4.5, 3.4, 0.05, 40.0, tilt), 3.4),
              synth.SemLayer(H + 1, synth.iso_cij(6.4, 3.6, 2.8), 2.8)]
    c = synth.Case(nex=12, nez=8, eh=2.0, sdt=0.01, nst=10, layers=layers, p=0.05, f0=1.0, ntrace=5,
                   rec_dx=4.0, semmodel_full=full)
    synth.write_case(c, d)
    path = os.path.join(d, "semmodel")
    xmax = c.nex * c.eh * 1.001 + 10.0
    sks.semmodel_write(path, [(L.C, L.rho, [-10.0, xmax], [L.top, L.top]) for L in layers], full=full)
    with chdir(d):
        su = sks.Setup(["par=run.par"])
        info = su.info()
        mat = su.material()
        su.close()
    V = [0, 5, 4, 3, 2]
    rows = {}
    for L in layers:
        rows[L.top] = [L.C[V[a], V[b]] for a in range(5) for b in range(a, 5)] + [1.0 / L.rho]
    h = info["h"]
    for iz in (1, info["nz"] // 2, info["nz"] - 2):
        z = iz * h
        L = next(L for L in layers if z < L.top)
        got = mat[iz * info["nx"] + 3]
        want = np.array([L.C[V[a], V[b]] for a in range(5) for b in range(a, 5)])
        assert np.allclose(got[:15], want, rtol=1e-12, atol=1e-9), (iz, got[:15], want)
