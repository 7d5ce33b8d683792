"""GPU: failure detection without a GPU fault.

* A non-finite wavefield.  The reference's only guard replaces an
  interpolated boundary value outside (-10, 10) -- NaN included -- by the
  mean of its neighbours (sem2d_psvsh.c:432-444); a NaN whose neighbours are
  not finite either (a whole NaN record) survives it and would poison the
  field for the rest of the solve.  The step kernels flag it:
  sks_run returns SKS_ERR_NONFINITE, the flag stays until sks_reset, and a
  clean run afterwards is bit-identical to a fresh solver's.  In a batch only
  the bad member is flagged and its batch mates' seismograms are bit-identical
  to their runs alone; the serving loop fails that request alone.
* A wait that runs out.  The pipelined chunks start a tile once its
  neighbours finished the previous step; every wait is bounded.  A test hook
  makes one tile never publish its progress, with a short poll limit: the run
  returns the error, the device stays usable, and the next run (after a
  reset) is bit-identical to a clean one.

The failures are made on the host (a NaN in the caller's records, a counter
nothing sets); nothing faults, traps or hangs the GPU.
"""
import os

import numpy as np
import pytest

import sks
import synth
from util import chdir

pytestmark = pytest.mark.gpu

TUNING = (4, 3, 0, 1)          # warps per CTA, band rows, band seams, register cap
PIPE = TUNING + (0, 1)         # ... waves 0, pipelined chunks
SPINS = 1 << 14                # polls before a stalled wait gives up (a few ms)
BAD_RECORD = 60                # a record every case injects


def _layers(H):
    return [synth.SemLayer(H - 6, synth.iso_cij(8.1, 4.5, 3.4), 3.4),
            synth.SemLayer(H - 3, synth.hexagonal_cij(8.1, 4.5, 3.4, 0.05, 40.0, 25.0), 3.4),
            synth.SemLayer(H + 1, synth.iso_cij(6.4, 3.6, 2.8), 2.8)]


CASES = [
    dict(nex=31, nez=10, eh=1.0, sdt=0.005, nst=500, p=0.045, f0=1.5, ntrace=11, rec_dx=2.5),
    dict(nex=17, nez=6, eh=2.0, sdt=0.01, nst=400, p=0.05, f0=0.8, ntrace=5, rec_dx=6.0),
    dict(nex=24, nez=10, eh=1.5, sdt=0.006, nst=450, p=0.042, f0=1.0, ntrace=9, rec_dx=3.5),
]


def _records(d):
    """The case's P-SV and SH record tables, [nrec][values] float32."""
    with chdir(d), sks.Setup(["par=run.par"]) as su:
        i = su.info()
    psv = np.fromfile(os.path.join(d, "greenfile"), np.float32).reshape(-1, i["mtotal"])
    sh = np.fromfile(os.path.join(d, "shgreenfile"), np.float32).reshape(-1, i["shtotal"])
    assert psv.shape[0] > BAD_RECORD + 2
    return psv, sh


@pytest.fixture(scope="module")
def cases(tmp_path_factory):
    out = []
    for i, k in enumerate(CASES):
        d = str(tmp_path_factory.mktemp(f"fail{i}"))
        H = k["nez"] * k["eh"] + 0.002
        c = synth.Case(nex=k["nex"], nez=k["nez"], eh=k["eh"], sdt=k["sdt"], nst=k["nst"], layers=_layers(H),
                       p=k["p"], f0=k["f0"], sv_amp=1.0, sh_amp=0.4, ntrace=k["ntrace"], rec_dx=k["rec_dx"],
                       semmodel_full=True)
        synth.write_case(c, d)
        out.append((d, k["nst"]))
    return out


def _open(d, prec, tuning=TUNING + (0, 0), records=None):
    with chdir(d):
        s = sks.Solver(["par=run.par"], precision=prec)
        if records is None:
            s.load_boundary_files()
    if records is not None:
        s.set_boundary(*records)
    s.set_tuning(*tuning)
    return s


def _same(a, b):
    return all(np.array_equal(x.view(np.uint32), y.view(np.uint32)) for x, y in zip(a, b))


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C], ids=["fp64", "fp32c"])
def test_nan_record_flags_the_solve_and_reset_clears_it(cases, prec):
    d, nst = cases[0]
    psv, sh = _records(d)
    with _open(d, prec) as s:
        assert s.wavefield_finite()             # before any run
        ref = s.run(nst)
        assert s.wavefield_finite()
    assert max(np.abs(x).max() for x in ref) > 0.05
    bad = psv.copy()
    bad[BAD_RECORD, :] = np.nan
    with _open(d, prec, records=(bad, sh)) as s:
        with pytest.raises(sks.SksError) as e:
            s.run(nst)
        assert e.value.code == -9, str(e.value)
        assert not s.wavefield_finite()
        s.reset()
        assert s.wavefield_finite()
        s.set_boundary(psv, sh)
        again = s.run(nst)
        assert s.wavefield_finite()
    assert _same(again, ref)


def _line_value(d):
    """Index of u_x of the interface row's point ix = nbl + 2 in a P-SV record."""
    with chdir(d), sks.Setup(["par=run.par"]) as su:
        i = su.info()
    return i["neh"] * i["hpn"] + 2


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C], ids=["fp64", "fp32c"])
def test_one_nan_value_is_mended_by_the_guard_as_the_reference_does(cases, prec, tmp_path):
    """One NaN value on the interface line: the guard replaces it by its
    neighbours' mean, the run stays finite, and the seismograms meet the
    parity bars against the FP64 oracle reading the same file."""
    from oracle.oracle import Oracle
    from util import seis_err
    d0, nst = cases[2]
    d = str(tmp_path)
    for f in os.listdir(d0):
        if os.path.isfile(os.path.join(d0, f)):
            with open(os.path.join(d0, f), "rb") as fi, open(os.path.join(d, f), "wb") as fo:
                fo.write(fi.read())
    psv, _ = _records(d)
    psv = psv.copy()
    psv[BAD_RECORD, _line_value(d)] = np.nan
    psv.tofile(os.path.join(d, "greenfile"))
    with chdir(d):
        o = Oracle(["par=run.par"], fp64=True)
        ref = o.run(nst)
        o.close()
    assert all(np.isfinite(x).all() for x in ref)
    with _open(d, prec, tuning=PIPE) as s:
        out = s.run(nst)
        assert s.wavefield_finite()
    assert seis_err(out, ref) <= (1e-10 if prec == sks.FP64 else 1e-4)


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C], ids=["fp64", "fp32c"])
def test_two_adjacent_nan_values_are_flagged_in_a_pipelined_run(cases, prec):
    """Two neighbouring NaN values: the guard's mean of the first takes the
    second's NaN, so NaN reaches the field, which is flagged."""
    d, nst = cases[2]
    psv, sh = _records(d)
    k = _line_value(d)
    bad = psv.copy()
    bad[BAD_RECORD, k:k + 2] = np.nan
    with _open(d, prec, tuning=PIPE, records=(bad, sh)) as s:
        with pytest.raises(sks.SksError) as e:
            s.run(nst)
        assert e.value.code == -9, str(e.value)


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C], ids=["fp64", "fp32c"])
def test_batch_flags_only_the_bad_member(cases, prec):
    alone = []
    for d, nst in cases:
        with _open(d, prec) as s:
            alone.append(s.run(nst))
    solvers = []
    for i, (d, nst) in enumerate(cases):
        if i == 1:
            psv, sh = _records(d)
            psv = psv.copy()
            psv[BAD_RECORD, :] = np.nan
            solvers.append(_open(d, prec, records=(psv, sh)))
        else:
            solvers.append(_open(d, prec))
    with sks.Batch(prec) as b:
        b.set_tuning(*TUNING, 0)
        for s in solvers:
            b.add(s)
        outs, rc = b.run(max(n for _, n in cases), status=True)
        assert rc == -9
        assert "member 1" in sks.lib().sks_last_error().decode()
        assert [s.wavefield_finite() for s in solvers] == [True, False, True]
        for i in (0, 2):
            assert _same(outs[i], alone[i]), f"member {i} changed"
    for s in solvers:
        s.close()


def test_server_fails_only_the_bad_request(cases, tmp_path):
    prec = sks.FP32C
    # the bad request: case 1 with a NaN record in its P-SV file
    d1, _ = cases[1]
    bad_dir = str(tmp_path / "bad")
    os.makedirs(bad_dir)
    for f in os.listdir(d1):
        src = os.path.join(d1, f)
        if os.path.isfile(src):
            with open(src, "rb") as fi, open(os.path.join(bad_dir, f), "wb") as fo:
                fo.write(fi.read())
    psv, _ = _records(bad_dir)
    psv = psv.copy()
    psv[BAD_RECORD, :] = np.nan
    psv.tofile(os.path.join(bad_dir, "greenfile"))
    dirs = [cases[0][0], bad_dir, cases[2][0]]
    alone = {}
    for i in (0, 2):
        with _open(dirs[i], prec) as s:
            alone[i] = s.run(cases[i][1])
    srv = sks.Server(0, 0, 64)
    srv.set_tuning(prec, *TUNING)
    ids = {}
    for i, d in enumerate(dirs):
        with chdir(d):
            ids[i] = srv.submit(sks.Setup(["par=run.par"]), prec, None)
    rounds = 0
    while srv.step() > 0:
        rounds += 1
        assert rounds < 100000
    st = {i: srv.info(r) for i, r in ids.items()}
    assert st[1]["state"] == sks.REQ_FAILED and st[1]["status"] == -9
    for i in (0, 2):
        assert st[i]["state"] == sks.REQ_DONE and st[i]["status"] == 0
        assert _same(srv.result(ids[i]), alone[i]), f"request {i} changed"
    srv.close()


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C], ids=["fp64", "fp32c"])
def test_pipelined_wait_runs_out_and_the_next_run_is_clean(cases, prec):
    d, nst = cases[0]
    with _open(d, prec, tuning=PIPE) as s:
        ref = s.run(nst)
    with _open(d, prec, tuning=PIPE) as s:
        s.test_stall_pipeline(1, SPINS)
        with pytest.raises(sks.SksError) as e:
            s.run(nst)
        assert e.value.code == -5 and "ran out" in str(e.value)
        s.reset()
        again = s.run(nst)
    assert _same(again, ref)


def test_batch_pipelined_wait_runs_out_and_the_next_run_is_clean(cases):
    prec = sks.FP32C
    alone = []
    for d, nst in cases:
        with _open(d, prec, tuning=PIPE) as s:
            alone.append(s.run(nst))
    solvers = [_open(d, prec) for d, _ in cases]
    nmax = max(n for _, n in cases)
    with sks.Batch(prec) as b:
        b.set_tuning(*TUNING, pipeline=1)
        for s in solvers:
            b.add(s)
        b.test_stall_pipeline(2, SPINS)
        _, rc = b.run(nmax, status=True)
        assert rc == -5 and "ran out" in sks.lib().sks_last_error().decode()
        for s in solvers:
            s.reset()
        outs = b.run(nmax)
        for i in range(len(cases)):
            assert _same(outs[i], alone[i]), f"member {i} differs after the failed run"
    for s in solvers:
        s.close()
