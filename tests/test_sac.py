"""CPU: SAC output of the seismograms (sks_sac_write, sks_uvw2sac and the
uvw2sac_gb300 program) as the reference's uvw2sac writes it
(semsyn/plot/uvw2sac.c): the published SAC version 6 binary layout, the
header words the program sets, every second record times `enlarge`, the
receivers' distances in float as the program computes them, log.txt and
pm.xy."""
import os
import subprocess

import numpy as np
import pytest

import sks
import synth
from util import chdir

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROG = os.path.join(ROOT, "s-sks_gb300", "_build", "uvw2sac_gb300")

# SAC v6 header: float words, integer words (after the 70 floats), by name
FW = {"delta": 0, "depmin": 1, "b": 5, "e": 6, "o": 7, "a": 8, "stla": 31, "stlo": 32, "stel": 33, "evla": 35,
      "evlo": 36, "evdp": 38, "mag": 39, "gcarc": 53, "cmpaz": 57, "cmpinc": 58}
IW = {"nzyear": 0, "nzjday": 1, "nzhour": 2, "nzmin": 3, "nzsec": 4, "nzmsec": 5, "nvhdr": 6, "npts": 9,
      "iftype": 15, "idep": 16, "leven": 35}


def read_sac(path):
    raw = open(path, "rb").read()
    f = np.frombuffer(raw[:280], np.float32)
    i = np.frombuffer(raw[280:440], np.int32)
    c = raw[440:632]
    h = {k: float(f[v]) for k, v in FW.items()}
    h.update({k: int(i[v]) for k, v in IW.items()})
    h["kstnm"] = c[:8].split(b"\0")[0].decode().strip()
    h["kstnm_raw"] = c[:8]
    h["kevnm"] = c[8:24].decode()
    h["kcmpnm"] = c[8 * 20:8 * 21].decode()
    data = np.frombuffer(raw[632:], np.float32)
    assert data.size == h["npts"]
    return h, data


def test_sac_write_layout(tmp_path):
    p = str(tmp_path / "a.sac")
    x = np.arange(17, dtype=np.float32) * 0.5
    sks.sac_write(p, x, delta=0.02, b=0.0, e=0.34, kstnm="ST1", cmpaz=90.0)
    h, d = read_sac(p)
    assert os.path.getsize(p) == 632 + 4 * 17
    assert np.array_equal(d, x)
    assert h["delta"] == np.float32(0.02) and h["b"] == 0.0 and h["e"] == np.float32(0.34) and h["cmpaz"] == 90.0
    assert h["npts"] == 17 and h["iftype"] == 1 and h["leven"] == 1 and h["nvhdr"] == 6
    assert h["kstnm"] == "ST1" and h["kstnm_raw"] == b"ST1\x0045  "
    for k in ("depmin", "a", "mag", "stla", "evdp", "gcarc"):
        assert h[k] == -12345.0, k
    assert h["idep"] == -12345 and h["nzyear"] == -12345
    assert h["kevnm"] == "-12345          " and h["kcmpnm"] == "-12345  "


def _case(d, get_rec):
    c = synth.Case(nex=20, nez=8, eh=2.0, sdt=0.01, nst=101, layers=synth.layered_two(16.0, 5.0), p=0.04, f0=1.0,
                   ntrace=6, rec_dx=4.0)
    synth.write_case(c, d)
    rng = np.random.default_rng(4)
    seis = [rng.normal(size=(c.nst, c.ntrace)).astype(np.float32) for _ in range(3)]
    for name, a in zip(("seis.u", "seis.v", "seis.w"), seis):
        a.tofile(os.path.join(d, name))
    words = ["par=run.par", "zbeg=0", "idzplot=1", "zs=12.5", "Conv_Source=0", "tstart=3.5", f"get_rec={get_rec}",
             "xmin=100.0", "xbeg=3.0"]
    return c, seis, words


def _expected_h(d):
    with chdir(d):
        su = sks.Setup(["par=run.par"])
        h = su.info()["h"]
        su.close()
    return np.float32(h)


@pytest.mark.parametrize("get_rec", [0, 1])
def test_uvw2sac_files_as_the_reference_writes_them(tmp_path, get_rec):
    d = str(tmp_path)
    c, seis, words = _case(d, get_rec)
    with chdir(d):
        sks.uvw2sac(words)
    h = _expected_h(d)
    num = c.nst // 2                          # every second record; the last odd one dropped
    f32 = np.float32
    if get_rec:
        xs = [float(x) for x in open(os.path.join(d, "rec_file")).read().split()[1:]]
        ix1 = [int(f32(x) / h) for x in xs]
        gc = [(f32(100.0) + f32(ix) * h) / f32(111.2) for ix in ix1]
    else:
        ixbeg = int(f32(3.0) / h)
        gc = [(f32(100.0) + f32(3.0) + f32(8 * i) * h) / f32(111.2) for i in range(c.ntrace)]
        assert ixbeg >= 0
    for n in range(c.ntrace):
        for ext, comp, az, inc in ((".ce", 0, 90.0, 90.0), (".cn", 1, 0.0, 90.0), (".cz", 2, 0.0, 0.0)):
            hd, data = read_sac(os.path.join(d, f"{n}{ext}"))
            want = seis[comp][0:2 * num:2, n] * f32(4.0)
            assert np.array_equal(data, want), (n, ext)
            assert hd["npts"] == num and hd["delta"] == f32(2) * f32(0.01)
            assert hd["b"] == 0.0 and hd["e"] == f32(num) * hd["delta"] and hd["o"] == f32(-3.5)
            assert hd["evdp"] == f32(12.5) and hd["evla"] == 0.0 and hd["evlo"] == 0.0 and hd["stla"] == 0.0
            assert hd["cmpaz"] == az and hd["cmpinc"] == inc
            assert hd["nzyear"] == 2006 and hd["nzjday"] == 0 and hd["nzmsec"] == 0
            assert hd["kstnm"] == str(n)
            assert hd["gcarc"] == pytest.approx(float(gc[n]), rel=1e-6) and hd["stlo"] == hd["gcarc"]
    log = open(os.path.join(d, "log.txt")).read().split()
    assert float(log[0]) == pytest.approx(3.5) and float(log[1]) == pytest.approx(3.5 + c.nst * 0.01, abs=1e-3)
    assert float(log[2]) == pytest.approx(float(gc[0]), abs=1e-3)
    pm = open(os.path.join(d, "pm.xy")).read().splitlines()
    assert pm[0].startswith(">>") and len(pm) == c.ntrace * (num + 1)
    u0, w0 = (float(x) for x in pm[1].split())
    assert u0 == pytest.approx(float(seis[0][0, 0] * 4), rel=1e-4) and w0 == pytest.approx(float(seis[2][0, 0] * 4), rel=1e-4)


def test_uvw2sac_program_and_refusals(tmp_path):
    d = str(tmp_path)
    c, seis, words = _case(d, 1)
    r = subprocess.run([PROG] + words, cwd=d, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.exists(os.path.join(d, "5.cz"))
    with chdir(d):
        with pytest.raises(sks.SksError):
            sks.uvw2sac([w for w in words if not w.startswith("Conv_Source")] + ["Conv_Source=1"])
        with pytest.raises(sks.SksError):
            sks.uvw2sac([w for w in words if not w.startswith("zs=")])          # zs is required
        with pytest.raises(sks.SksError):
            sks.uvw2sac(words + ["nst=500"])                                   # more records than the files hold
    r = subprocess.run([PROG] + words + ["Conv_Source=1"], cwd=d, capture_output=True, text=True)
    assert r.returncode == 1 and "Conv_Source" in r.stderr


@pytest.mark.parametrize("get_rec", [0, 1])
def test_uvw2sac_byte_identical_to_the_reference_program(tmp_path, get_rec):
    """Every file uvw2sac_gb300 writes -- the 18 SAC files, log.txt, pm.xy,
    tt.txt -- is byte-identical to what the reference's uvw2sac writes from
    the same inputs (tests/golden/uvw2sac.npz, made by make_golden_sac.py from
    the program compiled out of semsyn/plot)."""
    z = np.load(os.path.join(ROOT, "tests", "golden", "uvw2sac.npz"))
    d = str(tmp_path)
    for k in z.files:
        if k.startswith("in/"):
            z[k].tofile(os.path.join(d, k[3:]))
    words = ["par=run.par", "zbeg=0", "idzplot=1", "zs=12.5", "Conv_Source=0", "tstart=3.5", "xmin=100.0",
             "xbeg=3.0", f"get_rec={get_rec}"]
    r = subprocess.run([PROG] + words, cwd=d, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    want = {k.split("/", 1)[1]: z[k].tobytes() for k in z.files if k.startswith(f"get_rec{get_rec}/")}
    assert len(want) == 21
    for name, data in want.items():
        got = open(os.path.join(d, name), "rb").read()
        assert got == data, name
