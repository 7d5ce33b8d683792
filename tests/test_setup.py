"""Host set-up of the library against the oracle and the reference's rules (CPU).

sks_setup_open() is the set-up half of the reference's main(): par words,
ray/SEM models, mesh, per-point materials, GLL tables, mass, Stacey matrix,
receivers and the boundary-record schedule.  These tests need no GPU.
"""
import os
import tempfile

import numpy as np
import pytest

import sks
import synth
from golden.make_golden import extract
from oracle.oracle import Oracle
from util import chdir, solver_fixtures

GOLDEN = solver_fixtures()
IDS = [os.path.basename(p)[:-4] for p in GOLDEN]


def _words(z):
    return ["par=run.par"] + (["psv_only=1"] if str(z["prog"]) == "sem2d" else [])


@pytest.fixture(scope="module")
def golden_dirs(tmp_path_factory):
    out = {}
    for p in GOLDEN:
        d = str(tmp_path_factory.mktemp(os.path.basename(p)[:-4]))
        z = extract(p, d)
        out[p] = (d, _words(z))
    return out


@pytest.mark.parametrize("path", GOLDEN, ids=IDS)
def test_setup_matches_oracle(golden_dirs, path):
    d, words = golden_dirs[path]
    with chdir(d):
        o = Oracle(words, fp64=True)
        with sks.Setup(words) as su:
            info = su.info()
            assert (info["nx"], info["nz"], info["nez"], info["ntrace"], info["nt_inject"]) == \
                   (o.nx, o.nz, o.nez, o.ntrace, o.nt_sem)
            assert info["eh"] == o.eh
            # materials: identical per point (the table + index reproduces discret())
            assert np.array_equal(su.material(), o.material())
            m, ab = su.mass()
            mo, abo = o.mass()
            assert np.max(np.abs(m - mo)) <= 1e-15 * np.abs(mo).max()
            assert np.max(np.abs(ab - abo)) <= 1e-14 * max(np.abs(abo).max(), 1e-300)
            assert np.array_equal(su.receivers(), o.receivers())
        o.close()


def _ring_schedule(nt_sem, sdt, dp, psv_only):
    """Restatement of interpl()/interp_const() with the ns[] ring shared by the
    P-SV and SH calls (interpl.c:16-91, sem2d_psvsh.c:428-431): record index of
    each tap and the weights, per step."""
    f32 = np.float32
    rdt_f = f32(sdt) / f32(dp)
    rdt = sdt / dp
    ns = [0, 1, 2, 3]
    slots = {0: [-1] * 4, 1: [-1] * 4}
    cnt = {0: 0, 1: 0}
    taps = {0: [], 1: []}
    ws = []
    for it in range(nt_sem):
        t_f = f32(f32(it) * rdt_f)
        ns0 = int(np.float64(t_f) + 0.00001)
        prev = int(np.float64(f32(f32(f32(it) - f32(1)) * rdt_f)) + 0.00001)
        adv = ns0 > prev or it == 0
        d = it * rdt - ns0
        w = [-0.5 * d ** 3 + d * d - 0.5 * d, 3 * d ** 3 - 2.5 * d * d + 1, -3 * d ** 3 + 2 * d * d + 0.5 * d,
             0.5 * (d ** 3 - d * d)]
        ws.append(w)
        for fam in (0, 1):
            if fam == 1 and psv_only:
                taps[1].append([-1] * 4)
                continue
            if adv:
                ns = ns[1:] + ns[:1]
                slots[fam][ns[3]] = cnt[fam]
                cnt[fam] += 1
            taps[fam].append([slots[fam][ns[j]] for j in range(4)])
    return np.array(taps[0]), np.array(taps[1]), np.array(ws), cnt


@pytest.mark.parametrize("path", GOLDEN, ids=IDS)
def test_schedule_is_the_shared_ring(golden_dirs, path):
    d, words = golden_dirs[path]
    with chdir(d), sks.Setup(words) as su:
        info = su.info()
        tp, wp, ts, ws = su.schedule()
        par = dict(line.strip().split("=", 1) for line in open("run.par") if "=" in line)
    sdt, dp = float(par["sdt"]), float(par["dp"])
    rp, rs, rw, cnt = _ring_schedule(info["nt_inject"], sdt, dp, "psv_only=1" in words)
    assert np.array_equal(tp, rp)
    assert np.array_equal(ts, rs)
    assert np.allclose(wp, rw, rtol=0, atol=1e-12)
    assert info["nrec_psv"] == cnt[0]


def test_shared_ring_lag():
    """With dp == sdt the two calls turn the shared ring twice a step: step it
    reads record it-1 (P-SV and SH) instead of it-2 for a single call."""
    tp, ts, w, _ = _ring_schedule(6, 0.01, 0.01, False)
    assert [row[1] for row in tp[1:]] == [0, 1, 2, 3, 4]
    assert [row[1] for row in ts[1:]] == [0, 1, 2, 3, 4]
    assert np.allclose(w, [[0, 1, 0, 0]] * 6)
    tp1, _, _, _ = _ring_schedule(6, 0.01, 0.01, True)
    assert [row[1] for row in tp1[2:]] == [0, 1, 2, 3]


def _small_case(d, **kw):
    kw.setdefault("ntrace", 4)
    kw.setdefault("rec_dx", 3.0)
    c = synth.Case(nex=8, nez=6, eh=2.0, sdt=0.01, nst=20, layers=synth.layered_two(12.0, 3.0), **kw)
    synth.write_case(c, d)
    return c


def _err(words):
    with pytest.raises(sks.SksError) as e:
        sks.Setup(words)
    return e.value.code


def test_errors_are_status_codes(tmp_path):
    d = str(tmp_path)
    _small_case(d)
    with chdir(d):
        assert _err(["par=missing.par"]) == -2                      # ERR_IO
        assert _err(["par=run.par", "raymodel=nope"]) == -2
        assert _err(["par=run.par", "semmodel=nope"]) == -2
        assert _err(["par=run.par", "rec_file=nope"]) == -2
        assert _err(["par=run.par", "msource=1"]) == -4             # ERR_UNSUPPORTED
        assert _err(["par=run.par", "atten=2", "ass=0"]) == -1       # the taper needs ass > 0
        with sks.Setup(["par=run.par", "atten=4", "ass=0.9"]) as su:   # the boundary taper is supported
            assert su.info()["nx"] > 0
        assert _err(["par=run.par", "hpn=9"]) == -1                 # ERR_ARG
        with open("bad.par", "w") as f:
            f.write("".join(line for line in open("run.par") if not line.startswith("nex=")))
        assert _err(["par=bad.par"]) == -1                          # must-have key missing
        with open("semmodel.short", "w") as f:
            f.write("".join(open("semmodel").read().split("\n")[:2]))
        assert _err(["par=run.par", "semmodel=semmodel.short"]) == -3   # ERR_MODEL
        with open("semmodel.narrow", "w") as f:
            f.write(open("semmodel").read().replace("-10.0", "5.0"))
        assert _err(["par=run.par", "semmodel=semmodel.narrow"]) == -3  # x outside a layer
        with open("rec_far", "w") as f:
            f.write("2\n1.0 500.0\n")
        assert _err(["par=run.par", "rec_file=rec_far"]) == -3      # receiver off the mesh


def test_par_words_last_wins_and_nest(tmp_path):
    d = str(tmp_path)
    _small_case(d)
    with chdir(d):
        with open("outer.par", "w") as f:
            f.write("# comment line\npar=run.par nst=33   # trailing comment\n")
        with sks.Setup(["par=outer.par"]) as su:
            assert su.info()["nst"] == 33
        with sks.Setup(["par=outer.par", "nst=44"]) as su:
            assert su.info()["nst"] == 44
        with sks.Setup(["nst=55", "par=outer.par"]) as su:
            assert su.info()["nst"] == 33


def test_mass_integrates_density(tmp_path):
    """The lumped GLL mass sums to the GLL quadrature of rho over the box."""
    d = str(tmp_path)
    _small_case(d)
    with chdir(d), sks.Setup(["par=run.par"]) as su:
        info = su.info()
        mass, _ = su.mass()
        rho = su.material()[:, 15].reshape(info["nz"], info["nx"])
    N = info["hpn"]
    w = np.array([0.1, 49 / 90, 32 / 45, 49 / 90, 0.1])
    Je = info["eh"] ** 2 / 4
    tot = sum(Je * float(w @ rho[ez * N:ez * N + N + 1, ex * N:ex * N + N + 1] @ w)
              for ez in range(info["nez"]) for ex in range(info["nex"]))
    assert abs(mass.sum() - tot) <= 1e-12 * tot


def test_materials_are_deduplicated(tmp_path):
    d = str(tmp_path)
    _small_case(d)
    with chdir(d), sks.Setup(["par=run.par"]) as su:
        info = su.info()
        mat = su.material()
    assert info["nmat"] <= 4
    assert len(np.unique(mat, axis=0)) <= info["nmat"]
    assert info["anisotropic"] == 0


def _iso_rows_numpy(mat, info):
    """Element rows whose points all carry an exactly isotropic material:
    zero coupling entries, C11 = C33, C44 = C55 = C66 (the 15-entry row is
    C11 C16 C15 C14 C13 | C66 C56 C46 C36 | C55 C45 C35 | C44 C34 | C33)."""
    m = mat[:, :15]
    iso = ((m[:, [1, 2, 3, 6, 7, 8, 10, 11, 13]] == 0).all(axis=1) & (m[:, 0] == m[:, 14]) &
           (m[:, 5] == m[:, 9]) & (m[:, 9] == m[:, 12]))
    iso = iso.reshape(info["nz"], info["nx"])
    N = info["hpn"]
    return sum(bool(iso[ez * N:ez * N + N + 1].all()) for ez in range(info["nez"]))


@pytest.mark.parametrize("tilt", [0.0, 20.0])
def test_isotropic_element_rows_are_counted_as_the_materials_say(tmp_path, tilt):
    """sks_info_t.iso_rows (the rows the FP64 kernels give the isotropic
    stress) equals a numpy classification of the per-point materials; an
    anisotropic layer between isotropic ones leaves its rows and the rows
    across its interfaces out."""
    d = str(tmp_path)
    H = 24.002
    layers = [synth.SemLayer(H - 12, synth.iso_cij(8.1, 4.5, 3.4), 3.4),
              synth.SemLayer(H - 5, synth.hexagonal_cij(8.1, 4.5, 3.4, 0.05, 40.0, tilt), 3.4),
              synth.SemLayer(H + 1, synth.iso_cij(6.4, 3.6, 2.8), 2.8)]
    c = synth.Case(nex=10, nez=12, eh=2.0, sdt=0.01, nst=10, layers=layers, p=0.05, f0=1.0, ntrace=3,
                   rec_dx=4.0, semmodel_full=True)
    synth.write_case(c, d)
    with chdir(d), sks.Setup(["par=run.par"]) as su:
        info = su.info()
        mat = su.material()
    want = _iso_rows_numpy(mat, info)
    assert info["iso_rows"] == want
    assert 0 < want < info["nez"]
    assert info["anisotropic"] == 1


def _config_case(name):
    if name == "c0_iso_psv":
        return synth.config_isotropic_psv(nst=8), ["psv_only=1"]
    c = synth.config_aniso_3c(nst=8)
    c.semmodel_full = name == "c1_aniso_21"
    return c, []


@pytest.mark.parametrize("name", ["c0_iso_psv", "c1_aniso_21", "c1_aniso_13"])
def test_setup_matches_oracle_on_configuration_meshes(tmp_path, name):
    """The set-up on the benchmark configurations' own meshes: the plain
    isotropic P-SV case (321,201 points) and the anisotropic 3-component mesh
    (3,844,401 points) with its SEM model in 21 constants per layer (tilted
    axis) and in the reference's 13: mesh, materials per point, mass, Stacey
    matrix, receivers and the record schedule against the FP64 oracle."""
    d = str(tmp_path)
    c, extra = _config_case(name)
    synth.write_case(c, d)
    words = ["par=run.par"] + extra
    with chdir(d):
        o = Oracle(words, fp64=True)
        with sks.Setup(words) as su:
            info = su.info()
            assert (info["nx"], info["nz"]) == (c.nex * 4 + 1, c.nez * 4 + 1)
            assert (info["nx"], info["nz"], info["nez"], info["ntrace"], info["nt_inject"]) == \
                   (o.nx, o.nz, o.nez, o.ntrace, o.nt_sem)
            assert info["eh"] == o.eh
            mat = su.material()
            assert np.array_equal(mat, o.material())
            m, ab = su.mass()
            mo, abo = o.mass()
            assert np.max(np.abs(m - mo)) <= 1e-15 * np.abs(mo).max()
            assert np.max(np.abs(ab - abo)) <= 1e-14 * max(np.abs(abo).max(), 1e-300)
            assert np.array_equal(su.receivers(), o.receivers())
            tp, wp, ts, ws = su.schedule()
        o.close()
    rp, rs, rw, cnt = _ring_schedule(info["nt_inject"], c.sdt, c.dp or c.sdt, bool(extra))
    assert np.array_equal(tp, rp) and np.array_equal(ts, rs)
    assert np.allclose(wp, rw, rtol=0, atol=1e-12)
    # the tilted axis's entries that the reference's 13 constants drop (C15,
    # C14, C56, C46, C35, C34 of the 15-entry rows) exist in the 21-constant
    # model only; both models keep the azimuthal ones (C16, C36, C45)
    tilt_only = np.abs(mat[:, [2, 3, 6, 7, 11, 13]]).max() > 0
    assert tilt_only == (name == "c1_aniso_21")
    if name != "c0_iso_psv":
        assert np.abs(mat[:, [1, 8, 10]]).max() > 0
