"""GPU: batches of uneven solves give each member the seismograms of the same
solver run alone with the batch's tuning, bit for bit.

Members differ in mesh size, time step, ray parameter, anisotropy (none,
hexagonal with a tilted axis), step count and the step they join at; runs are
split across calls; members leave and join between calls; the batch autotuner
leaves every member where it was.
"""
import os

import numpy as np
import pytest

import sks
import synth
from util import chdir

pytestmark = pytest.mark.gpu

TUNING = (4, 3, 0, 1)          # warps per CTA, band rows, band seams, register cap


def _layers(H, aniso):
    mid = synth.hexagonal_cij(8.1, 4.5, 3.4, 0.05, 40.0, 25.0) if aniso else synth.iso_cij(8.0, 4.45, 3.35)
    return [synth.SemLayer(H - 6, synth.iso_cij(8.1, 4.5, 3.4), 3.4),
            synth.SemLayer(H - 3, mid, 3.4),
            synth.SemLayer(H + 1, synth.iso_cij(6.4, 3.6, 2.8), 2.8)]


CASES = [
    dict(nex=31, nez=10, eh=1.0, sdt=0.005, nst=850, p=0.045, f0=1.5, aniso=True, ntrace=11, rec_dx=2.5),
    dict(nex=17, nez=6, eh=2.0, sdt=0.01, nst=620, p=0.05, f0=0.8, aniso=False, ntrace=5, rec_dx=6.0),
    dict(nex=53, nez=12, eh=1.0, sdt=0.004, nst=1200, p=0.038, f0=1.2, aniso=True, ntrace=25, rec_dx=2.0),
    dict(nex=24, nez=10, eh=1.5, sdt=0.006, nst=960, p=0.042, f0=1.0, aniso=True, ntrace=9, rec_dx=3.5),
]


@pytest.fixture(scope="module")
def cases(tmp_path_factory):
    dirs = []
    for i, k in enumerate(CASES):
        d = str(tmp_path_factory.mktemp(f"batch{i}"))
        H = k["nez"] * k["eh"] + 0.002
        c = synth.Case(nex=k["nex"], nez=k["nez"], eh=k["eh"], sdt=k["sdt"], nst=k["nst"],
                       layers=_layers(H, k["aniso"]), p=k["p"], f0=k["f0"], sv_amp=1.0, sh_amp=0.4,
                       ntrace=k["ntrace"], rec_dx=k["rec_dx"], semmodel_full=True)
        synth.write_case(c, d)
        dirs.append(d)
    return dirs


def _open(d, prec):
    with chdir(d):
        s = sks.Solver(["par=run.par"], precision=prec)
        s.load_boundary_files()
    return s


def _alone(d, prec, nst):
    s = _open(d, prec)
    s.set_tuning(*TUNING, 0)
    out = s.run(nst)
    s.close()
    return out


def _cat(parts):
    return tuple(np.concatenate([p[c] for p in parts]) for c in range(3))


@pytest.mark.parametrize("prec,tuning", [(sks.FP64, TUNING + (0,)), (sks.FP32C, TUNING + (0,)),
                                         (sks.FP64, (4, 3, 1, 0, 1)), (sks.FP32C, (4, 3, 0, 1, 1)),
                                         (sks.FP32C, (2, 5, 1, 0, 1))])
def test_batch_matches_members_alone(cases, prec, tuning):
    """Per-step launches and pipelined chunks (tuning[4] = 1), with halo rows
    and with band seams."""
    nst = [k["nst"] for k in CASES]
    ref = [_alone(d, prec, n) for d, n in zip(cases, nst)]
    assert all(max(np.abs(x).max() for x in r) > 0.05 for r in ref)
    with sks.Batch(prec) as b:
        sol = [_open(d, prec) for d in cases]
        for s in sol:
            b.add(s)
        b.set_tuning(*tuning)
        assert b.tuning()["pipeline"] == tuning[4]
        parts = [[] for _ in sol]
        for n in (1, 63, 200, 1000):            # split calls; members finish at different calls
            outs = b.run(n)
            for i, o in enumerate(outs):
                parts[i].append(o)
        assert b.launches() > 0
        for i, s in enumerate(sol):
            assert s.info()["step"] == nst[i]
            got = _cat(parts[i])
            for c in range(3):
                assert got[c].shape == ref[i][c].shape
                assert np.array_equal(got[c], ref[i][c]), f"member {i} component {c}"
        for s in sol:
            b.remove(s)
            s.close()


@pytest.mark.parametrize("pipeline", [0, 1])
def test_batch_members_join_and_leave_between_calls(cases, pipeline):
    prec = sks.FP32C
    ref = [_alone(d, prec, k["nst"]) for d, k in zip(cases, CASES)]
    with sks.Batch(prec) as b:
        b.set_tuning(*TUNING, pipeline)
        a = _open(cases[0], prec)
        c = _open(cases[2], prec)
        b.add(a)
        b.add(c)
        pa, pc = [], []
        o = b.run(150)
        pa.append(o[0]); pc.append(o[1])
        # a member leaves, runs 40 steps alone with the same tuning, comes back
        b.remove(a)
        pa.append(a.run(40))
        late = _open(cases[3], prec)            # joins at step 0 while c is at step 150
        b.add(late)
        b.add(a)
        pl = []
        o = b.run(10000)
        pc.append(o[0]); pl.append(o[1]); pa.append(o[2])
        for got, want in ((_cat(pa), ref[0]), (_cat(pc), ref[2]), (_cat(pl), ref[3])):
            for k in range(3):
                assert np.array_equal(got[k], want[k])
        for s in (a, c, late):
            s.close()                           # a member leaves its batch when destroyed
        assert len(b) == 0


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C])
def test_batch_autotune_restores_members(cases, prec):
    with sks.Batch(prec) as b:
        sol = [_open(d, prec) for d in cases[:3]]
        for s in sol:
            b.add(s)
        first = b.run(20)
        best = b.autotune(4)
        assert best["ms_per_step"] > 0
        t = b.tuning()
        assert (t["warps_per_block"], t["band_rows"], t["zseam"], t["register_cap"]) == \
               (best["warps_per_block"], best["band_rows"], best["zseam"], best["register_cap"])
        rest = b.run(10000)
        for i, d in enumerate(cases[:3]):
            s = _open(d, prec)
            s.set_tuning(best["warps_per_block"], best["band_rows"], best["zseam"], best["register_cap"], 0)
            want = s.run(CASES[i]["nst"])
            s.close()
            got = _cat([first[i], rest[i]])
            for c in range(3):
                assert np.array_equal(got[c], want[c])
        for s in sol:
            b.remove(s)
            s.close()


def test_batch_rejects_mixed_forms_and_double_membership(cases):
    with sks.Batch(sks.FP32C) as b, sks.Batch(sks.FP32C) as b2:
        s64 = _open(cases[1], sks.FP64)
        with pytest.raises(sks.SksError):
            b.add(s64)
        s = _open(cases[1], sks.FP32C)
        b.add(s)
        with pytest.raises(sks.SksError):
            b2.add(s)
        with pytest.raises(sks.SksError):
            s.set_tuning(4, 3, 0, 1, 0)        # a member's tuning belongs to its batch
        b.remove(s)
        s.set_tuning(4, 3, 0, 1, 0)
        s.close()
        s64.close()


# per degree: the members' (nex, nez, eh, dt, steps)
DEG_MEMBERS = {3: ((30, 9, 1.5, 0.008, 700), (20, 8, 2.0, 0.01, 560)),
               5: ((23, 7, 2.0, 0.008, 700), (14, 6, 2.5, 0.01, 560)),
               6: ((19, 6, 2.5, 0.006, 900), (12, 5, 3.0, 0.007, 720))}


@pytest.mark.parametrize("deg", [5, 3, 6])
@pytest.mark.parametrize("prec,tuning", [(sks.FP64, (4, 3, 1, 0, 0)), (sks.FP32C, (4, 3, 0, 1, 0)),
                                         (sks.FP32C, (4, 4, 1, 1, 1))])
def test_other_degrees_batch_matches_members_alone(cases, tmp_path, prec, tuning, deg):
    """Members of GLL degree 5 (the reference's default hpn), 3 or 6 in a
    batch equal their solo runs; a batch holds one degree and that degree's
    compiled tunings."""
    dirs, nst = [], []
    for i, (nex, nez, eh, sdt, n) in enumerate(DEG_MEMBERS[deg]):
        d = str(tmp_path / f"d{deg}_{i}")
        H = nez * eh + 0.002
        c = synth.Case(nex=nex, nez=nez, eh=eh, sdt=sdt, nst=n, layers=_layers(H, True), p=0.045, f0=1.0,
                       sv_amp=1.0, sh_amp=0.4, hpn=deg, ntrace=7, rec_dx=3.0, semmodel_full=True)
        synth.write_case(c, d)
        dirs.append(d)
        nst.append(n)
    ref = []
    for d, n in zip(dirs, nst):
        s = _open(d, prec)
        s.set_tuning(*tuning[:4], 0, tuning[4])
        ref.append(s.run(n))
        s.close()
    assert all(max(np.abs(x).max() for x in r) > 0.05 for r in ref)
    with sks.Batch(prec) as b:
        sol = [_open(d, prec) for d in dirs]
        for s in sol:
            b.add(s)
        b.set_tuning(*tuning)
        with pytest.raises(sks.SksError):
            b.set_tuning(2, 3, 0, 1, 0)                 # not compiled for degrees other than 4
        other = _open(cases[0], prec)                    # degree 4
        with pytest.raises(sks.SksError):
            b.add(other)
        other.close()
        outs = b.run(max(nst))
        for i, s in enumerate(sol):
            for c in range(3):
                assert np.array_equal(outs[i][c], ref[i][c]), f"member {i} component {c}"
        for s in sol:
            b.remove(s)
            s.close()
