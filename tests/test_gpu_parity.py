"""GPU parity: the CUDA solver through the C ABI against the FP64 oracle.

Bars: the plain FP64 form within relative L2 1e-10 of the FP64 oracle on every
seismogram component; the FP32-compensated form within 1e-4.  Cases cover the
isotropic and anisotropic stress kernels, P-SV+SH and P-SV-only injection,
Stacey on/off, a GRT record step different from the SEM step with injection
ending inside the run, Earth flattening, both receiver layouts, many warp-tile
seams, runs split across calls, determinism and the drop-in CLI.
"""
import os
import subprocess

import numpy as np
import pytest

import sks
import synth
from oracle.oracle import Oracle
from golden.make_golden import extract
from util import chdir, seis_err, solver_fixtures

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
FP32C_TOL = 1e-4


def _aniso_layers(H, tilt=20.0):
    return [synth.SemLayer(H - 6, synth.iso_cij(8.1, 4.5, 3.4), 3.4),
            synth.SemLayer(H - 3, synth.hexagonal_cij(8.1, 4.5, 3.4, 0.06, 30.0, tilt), 3.4),
            synth.SemLayer(H + 1, synth.iso_cij(6.4, 3.6, 2.8), 2.8)]


CASES = {
    "aniso_full_sh": lambda: synth.Case(nex=16, nez=10, eh=2.0, sdt=0.01, nst=800, layers=_aniso_layers(20.0),
                                        p=0.05, f0=1.0, sv_amp=1.0, sh_amp=0.5, ntrace=7, rec_x0=1.0,
                                        rec_dx=4.0, semmodel_full=True),
    "aniso_13_sh": lambda: synth.Case(nex=18, nez=9, eh=2.0, sdt=0.01, nst=760,
                                      layers=_aniso_layers(18.0, tilt=0.0), p=0.05, f0=1.0, sv_amp=1.0,
                                      sh_amp=0.7, ntrace=9, rec_x0=0.5, rec_dx=3.7),
    "iso_psv": lambda: synth.Case(nex=30, nez=10, eh=2.0, sdt=0.01, nst=800, layers=synth.layered_two(20.0, 6.0),
                                  p=0.045, f0=1.0, ntrace=15, rec_dx=4.0),
    "seams_many": lambda: synth.Case(nex=40, nez=24, eh=1.0, sdt=0.005, nst=1400, layers=_aniso_layers(24.0),
                                     p=0.045, f0=1.5, sv_amp=1.0, sh_amp=0.3, ntrace=21, rec_dx=1.9,
                                     semmodel_full=True),
    "rdt_half_short_grt": lambda: synth.Case(nex=16, nez=10, eh=2.0, sdt=0.005, dp=0.01, nt=300, nst=1500,
                                             layers=_aniso_layers(20.0), p=0.05, f0=1.0, sh_amp=0.5,
                                             ntrace=7, rec_dx=4.0, semmodel_full=True),
    "psv_only_no_absorb": lambda: synth.Case(nex=16, nez=10, eh=2.0, sdt=0.01, nst=800, layers=_aniso_layers(20.0),
                                             p=0.05, f0=1.0, ntrace=7, rec_dx=4.0, psv_only=True, absorb=0,
                                             semmodel_full=True),
    # boundary taper (atten_wave2): bottom, left and right zones two elements wide
    "atten3_neh2": lambda: synth.Case(nex=20, nez=10, eh=2.0, sdt=0.01, nst=800, layers=_aniso_layers(20.0),
                                      p=0.05, f0=1.0, sv_amp=2.0, sh_amp=1.0, neh=2, ntrace=9, rec_x0=1.0,
                                      rec_dx=4.0, semmodel_full=True, extra={"atten": 3, "ass": "0.85"}),
    # the default taper: the bottom zone only, ass = 0.93
    "atten1": lambda: synth.Case(nex=18, nez=9, eh=2.0, sdt=0.01, nst=760, layers=_aniso_layers(18.0, tilt=0.0),
                                 p=0.05, f0=1.0, sv_amp=1.0, sh_amp=0.7, ntrace=9, rec_x0=0.5, rec_dx=3.7,
                                 extra={"atten": 1}),
    # GLL degree 5 (the reference's default hpn): 5 elements per warp
    "hpn5_aniso": lambda: synth.Case(nex=23, nez=8, eh=2.0, sdt=0.008, nst=900, layers=_aniso_layers(16.0),
                                     p=0.05, f0=1.0, sv_amp=1.0, sh_amp=0.5, hpn=5, ntrace=9, rec_x0=1.0,
                                     rec_dx=4.5, semmodel_full=True),
    # GLL degrees 3 (7 elements per warp) and 6 (4 elements per warp)
    "hpn3_aniso": lambda: synth.Case(nex=27, nez=9, eh=1.5, sdt=0.008, nst=900, layers=_aniso_layers(13.5),
                                     p=0.05, f0=1.2, sv_amp=1.0, sh_amp=0.5, hpn=3, ntrace=9, rec_x0=1.0,
                                     rec_dx=4.0, semmodel_full=True),
    "hpn6_aniso": lambda: synth.Case(nex=17, nez=7, eh=2.5, sdt=0.006, nst=1100, layers=_aniso_layers(17.5),
                                     p=0.05, f0=1.0, sv_amp=1.0, sh_amp=0.5, hpn=6, ntrace=9, rec_x0=1.0,
                                     rec_dx=4.5, semmodel_full=True),
    # degree 3 with the boundary taper's bottom and left zones, degree 6 with the bottom, left and right
    # ones (the top zone would hold the surface receivers)
    "hpn3_atten2": lambda: synth.Case(nex=30, nez=12, eh=1.5, sdt=0.008, nst=900, layers=_aniso_layers(18.0),
                                      p=0.05, f0=1.2, sv_amp=2.0, sh_amp=1.0, hpn=3, neh=2, ntrace=9, rec_x0=1.0,
                                      rec_dx=4.0, semmodel_full=True, extra={"atten": 2, "ass": "0.9"}),
    "hpn6_atten3": lambda: synth.Case(nex=18, nez=8, eh=2.5, sdt=0.006, nst=1100, layers=_aniso_layers(20.0),
                                      p=0.05, f0=1.0, sv_amp=2.0, sh_amp=1.0, hpn=6, neh=2, ntrace=9, rec_x0=1.0,
                                      rec_dx=4.5, semmodel_full=True, extra={"atten": 3, "ass": "0.85"}),
    "flat0_raymodel_xbeg": lambda: synth.Case(nex=20, nez=8, eh=2.0, sdt=0.01, nst=700,
                                              layers=synth.layered_two(16.0, 5.0), p=0.04, f0=1.0, flat=0,
                                              readpars=0, get_rec=0, ntrace=6, sh_amp=0.4,
                                              extra={"xbeg": "0.0", "idxplot": 13}),
}


@pytest.fixture(scope="module")
def casedirs(tmp_path_factory):
    out = {}
    for name, mk in CASES.items():
        d = str(tmp_path_factory.mktemp(name))
        c = mk()
        synth.write_case(c, d)
        with chdir(d):
            o = Oracle(["par=run.par"], fp64=True)
            ref = o.run(c.nst)
            o.close()
        out[name] = (d, c, ref)
    return out


def _gpu_run(d, prec, nsteps, pieces=None):
    with chdir(d), sks.Solver(["par=run.par"], precision=prec, device=0) as s:
        s.load_boundary_files()
        if not pieces:
            return s.run(nsteps), s.info()
        parts = []
        done = 0
        for p in pieces:
            parts.append(s.run(p))
            done += len(parts[-1][0])
        rest = nsteps - done
        if rest > 0:
            parts.append(s.run(rest))
        return tuple(np.concatenate([q[i] for q in parts]) for i in range(3)), s.info()


@pytest.mark.parametrize("name", list(CASES))
def test_fp64_matches_oracle(casedirs, name):
    d, c, ref = casedirs[name]
    out, info = _gpu_run(d, sks.FP64, c.nst)
    assert out[0].shape == ref[0].shape
    err = seis_err(out, ref)
    assert np.isfinite(err) and err <= FP64_TOL, f"{name}: FP64 rel L2 {err:.3e}"
    assert max(np.abs(r).max() for r in ref) > 0.5, "case produced no signal"


@pytest.mark.parametrize("name", list(CASES))
def test_fp32c_matches_oracle(casedirs, name):
    d, c, ref = casedirs[name]
    out, _ = _gpu_run(d, sks.FP32C, c.nst)
    err = seis_err(out, ref)
    assert np.isfinite(err) and err <= FP32C_TOL, f"{name}: FP32C rel L2 {err:.3e}"


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C])
def test_split_runs_equal_one_run(casedirs, prec):
    d, c, _ = casedirs["seams_many"]
    whole, _ = _gpu_run(d, prec, c.nst)
    split, _ = _gpu_run(d, prec, c.nst, pieces=[1, 63, 64, 5, 70])
    for i in range(3):
        assert np.array_equal(whole[i], split[i])


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C])
def test_taper_under_every_grid_and_in_a_batch(casedirs, prec):
    """The boundary taper is applied where the point is updated, so it must
    not depend on the CTA grid (band seams, pipelined chunks, balanced waves)
    nor on running as a batch member."""
    d, c, _ = casedirs["atten3_neh2"]
    ref = None
    with chdir(d):
        for t in ((4, 8, 1, 0, 0, 0), (2, 1, 0, 1, 0, 1), (4, 3, 1, 1, 0, 1), (4, 4, 0, 1, 2, 0)):
            with sks.Solver(["par=run.par"], precision=prec) as s:
                s.load_boundary_files()
                s.set_tuning(*t)
                out = s.run(c.nst)
            if ref is None:
                ref = out
            for i in range(3):
                assert np.array_equal(out[i], ref[i]), (t, i)
        with sks.Solver(["par=run.par"], precision=prec) as s:
            s.load_boundary_files()
            with sks.Batch(prec) as b:
                b.add(s)
                got = b.run(c.nst)[0]
                b.remove(s)
    for i in range(3):
        assert np.array_equal(got[i], ref[i]), i


@pytest.mark.parametrize("deg", [3, 5, 6])
@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C])
def test_other_degrees_tunings_bit_identical_and_refusals(casedirs, prec, deg):
    """Degrees 3, 5 and 6 compile 4-warp CTAs with register cap 0 or 1: every
    such grid (seams or halo rows, per-step or pipelined, balanced waves)
    gives the same bits; other tunings are refused; batches take them."""
    d, c, _ = casedirs[f"hpn{deg}_aniso"]
    ref = None
    with chdir(d):
        for t in ((4, 3, 0, 0, 0, 0), (4, 1, 1, 1, 0, 0), (4, 8, 0, 1, 0, 1), (4, 2, 1, 0, 0, 1), (4, 4, 0, 1, 2, 0)):
            with sks.Solver(["par=run.par"], precision=prec) as s:
                s.load_boundary_files()
                s.set_tuning(*t)
                out = s.run(c.nst)
            if ref is None:
                ref = out
            for i in range(3):
                assert np.array_equal(out[i], ref[i]), (t, i)
        with sks.Solver(["par=run.par"], precision=prec) as s:
            for bad in ((2, 4, 0, 1, 0, 0), (4, 4, 0, 2, 0, 0)):
                with pytest.raises(sks.SksError):
                    s.set_tuning(*bad)
            s.load_boundary_files()
            with sks.Batch(prec) as b:
                b.add(s)                                # batches take these degrees too
                b.remove(s)
        with pytest.raises(sks.SksError):
            sks.Solver(["par=run.par", "hpn=7"], precision=prec)


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C])
def test_deterministic(casedirs, prec):
    d, c, _ = casedirs["aniso_full_sh"]
    a, _ = _gpu_run(d, prec, c.nst)
    b, _ = _gpu_run(d, prec, c.nst)
    for i in range(3):
        assert np.array_equal(a[i], b[i])


def test_reset_replays(casedirs):
    d, c, _ = casedirs["aniso_13_sh"]
    with chdir(d), sks.Solver(["par=run.par"], precision=sks.FP64) as s:
        s.load_boundary_files()
        a = s.run(c.nst)
        s.reset()
        b = s.run(c.nst)
    for i in range(3):
        assert np.array_equal(a[i], b[i])


def test_set_boundary_from_memory_equals_files(casedirs):
    d, c, _ = casedirs["aniso_full_sh"]
    with chdir(d):
        with sks.Solver(["par=run.par"], precision=sks.FP64) as s:
            info = s.info()
            psv = np.fromfile("greenfile", np.float32)[: info["nrec_psv"] * info["mtotal"]]
            sh = np.fromfile("shgreenfile", np.float32)[: info["nrec_sh"] * info["shtotal"]]
            s.set_boundary(psv, sh)
            a = s.run(c.nst)
        b, _ = _gpu_run(d, sks.FP64, c.nst)
    for i in range(3):
        assert np.array_equal(a[i], b[i])


def test_cli_drop_in_writes_reference_files(casedirs):
    d, c, ref = casedirs["aniso_13_sh"]
    cli = os.path.join(os.path.dirname(sks.LIB_PATH), "sem2d_psvsh_gb300")
    r = subprocess.run([cli, "par=run.par"], cwd=d, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nt = c.ntrace
    got = [np.fromfile(os.path.join(d, f"seis.{x}"), np.float32).reshape(-1, nt) for x in "uvw"]
    assert got[0].shape[0] == c.nst
    assert seis_err(got, ref) <= FP64_TOL


GOLDEN = solver_fixtures()


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_golden_inputs_fp64_vs_oracle_and_reference(path, tmp_path):
    """On the reference-generated fixtures: FP64 GPU within 1e-10 of the FP64
    oracle, and within the reference's own FP32 rounding of its seismograms."""
    d = str(tmp_path)
    z = extract(path, d)
    nt, nst = int(z["ntrace"]), int(z["nst"])
    words = ["par=run.par"] + (["psv_only=1"] if str(z["prog"]) == "sem2d" else [])
    gold = [z["seis_" + x].reshape(nst, nt) for x in "uvw"]
    with chdir(d):
        o = Oracle(words, fp64=True)
        ref = o.run(nst)
        o.close()
        for prec, tol in ((sks.FP64, FP64_TOL), (sks.FP32C, FP32C_TOL)):
            with sks.Solver(words, precision=prec) as s:
                s.load_boundary_files()
                out = s.run(nst)
            assert seis_err(out, ref) <= tol
            assert seis_err(out, gold) <= 5e-5


def _ring_traces(d, info, tp, wp, ts, ws, it):
    """g(it) from the files and the schedule: four taps, then the |g| >= 10 guard."""
    L = info["mtotal"]
    psv = np.fromfile(os.path.join(d, "greenfile"), np.float32).reshape(-1, L).astype(np.float64)
    sh = np.fromfile(os.path.join(d, "shgreenfile"), np.float32).reshape(-1, info["shtotal"]).astype(np.float64)
    out = []
    for rec, taps, w in ((psv, tp, wp), (sh, ts, ws)):
        g = np.zeros(rec.shape[1])
        for j in range(4):
            if taps[it, j] >= 0:
                g += w[it, j] * rec[taps[it, j]]
        assert np.all(np.abs(g) < 10)
        out.append(g)
    return out


def test_line_increments_match_schedule(casedirs):
    """sks_line_increments = g(it+1) - g(it) of the four-tap interpolation."""
    d, c, _ = casedirs["rdt_half_short_grt"]
    with chdir(d), sks.Solver(["par=run.par"], precision=sks.FP64) as s, sks.Setup(["par=run.par"]) as su:
        s.load_boundary_files()
        info = s.info()
        tp, wp, ts, ws = su.schedule()
        it0, n = 3, 40
        got = s.line_increments(it0, n)
        nx, nz, nbl = info["nx"], info["nz"], info["neh"] * info["hpn"]
        for k in range(n):
            it = it0 + k
            if it + 1 >= info["nt_inject"]:
                assert not got[k].any()
                continue
            g0, v0 = _ring_traces(d, info, tp, wp, ts, ws, it)
            g1, v1 = _ring_traces(d, info, tp, wp, ts, ws, it + 1)
            row = np.stack([-g0[nbl:nx] + g1[nbl:nx], -v0[nbl:nx] + v1[nbl:nx],
                            g0[nx + nbl:2 * nx] - g1[nx + nbl:2 * nx]], axis=1)
            iz = np.arange(nbl + 1, nz)
            col = np.stack([-g0[2 * nx + iz] + g1[2 * nx + iz], -v0[nx + iz] + v1[nx + iz],
                            g0[2 * nx + nz + iz] - g1[2 * nx + nz + iz]], axis=1)
            ref = np.concatenate([row, col])
            assert np.allclose(got[k], ref, rtol=0, atol=1e-12 * max(1.0, np.abs(ref).max()))
        # the injection window ends: the tail is zeros
        tail = s.line_increments(info["nt_inject"] - 2, 5)
        assert tail[0].any() and not tail[1:].any()


SNAP_FIXTURES = [p for p in GOLDEN if "snap_out1" in np.load(p).files]


def _parse_snapshot_text(b: bytes):
    rows = np.array([line.split() for line in b.decode().splitlines()], dtype=np.float64)
    return rows[:, :2].astype(int), rows[:, 2:]


@pytest.mark.parametrize("path", SNAP_FIXTURES, ids=[os.path.basename(p)[:-4] for p in SNAP_FIXTURES])
def test_snapshots_vs_oracle_and_reference_files(path, tmp_path):
    """plot_snap: both forms, per-step and pipelined launches, against the
    FP64 oracle's snapshots; the drop-in program's out files against the
    reference's (same points, values within its FP32 rounding)."""
    d = str(tmp_path)
    z = extract(path, d)
    nst = int(z["nst"])
    words = ["par=run.par"] + str(z["words"]).split()
    with chdir(d):
        o = Oracle(words, fp64=True)
        o.run(nst)
        ref = []
        k = 0
        while True:
            r = o.snapshot(k)
            if r is None:
                break
            ref.append(r)
            k += 1
        o.close()
        assert len(ref) >= 5 and max(np.abs(r[1]).max() for r in ref) > 0.05
        for prec, tol in ((sks.FP64, FP64_TOL), (sks.FP32C, FP32C_TOL)):
            for tuning in ((4, 3, 0, 1, 0, 0), (4, 3, 0, 1, 0, 1), (2, 2, 1, 0, 0, 0)):
                with sks.Solver(words, precision=prec) as s:
                    s.load_boundary_files()
                    s.set_tuning(*tuning)
                    s.run(nst // 3)
                    s.run(nst)
                    for k, (step, a) in enumerate(ref):
                        got = s.snapshot(k)
                        assert got is not None and got[0] == step
                        na = np.linalg.norm(a)
                        if na == 0.0:                  # before the wave arrives: exactly zero
                            assert not np.any(got[1]), (prec, tuning, k)
                            continue
                        err = np.linalg.norm(got[1].astype(np.float64) - a) / na
                        assert err <= tol, (prec, tuning, k, err)
                    assert s.snapshot(len(ref)) is None
        cli = os.path.join(os.path.dirname(sks.LIB_PATH), "sem2d_psvsh_gb300")
        r = subprocess.run([cli] + words, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    k = 1
    while f"snap_out{k}" in z.files:
        pos_ref, val_ref = _parse_snapshot_text(z[f"snap_out{k}"].tobytes())
        with open(os.path.join(d, f"out{k}"), "rb") as f:
            pos, val = _parse_snapshot_text(f.read())
        assert np.array_equal(pos, pos_ref)
        # the reference's %e text keeps 7 significant digits
        assert np.linalg.norm(val - val_ref) <= 5e-5 * np.linalg.norm(val_ref) + 1e-30
        k += 1
    assert not os.path.exists(os.path.join(d, f"out{k}"))


def test_snapshots_need_plot_snap(tmp_path):
    d = str(tmp_path)
    c = CASES["aniso_full_sh"]()
    synth.write_case(c, d)
    with chdir(d), sks.Solver(["par=run.par"], precision=sks.FP32C) as s:
        s.load_boundary_files()
        s.run(50)
        assert s.snapshot(0) is None
        assert "plot_snap" in sks.lib().sks_last_error().decode()
