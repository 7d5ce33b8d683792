"""GPU: a solve's state saved mid-run and loaded into a fresh solver (or back
into the same one) continues exactly: the remaining seismogram rows and the
snapshots are bit-identical, under any tuning; states of other solves are
refused."""
import numpy as np
import pytest

import sks
import synth
from util import chdir

pytestmark = pytest.mark.gpu


def _layers(H):
    return [synth.SemLayer(H - 6, synth.iso_cij(8.1, 4.5, 3.4), 3.4),
            synth.SemLayer(H - 3, synth.hexagonal_cij(8.1, 4.5, 3.4, 0.05, 35.0, 15.0), 3.4),
            synth.SemLayer(H + 1, synth.iso_cij(6.4, 3.6, 2.8), 2.8)]


@pytest.fixture(scope="module")
def case(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("restart"))
    c = synth.Case(nex=33, nez=11, eh=1.0, sdt=0.005, nst=900, layers=_layers(11.002), p=0.045, f0=1.5,
                   sv_amp=1.0, sh_amp=0.4, ntrace=9, rec_dx=3.0, semmodel_full=True,
                   extra={"plot_snap": 1, "startsnap": 100, "incresnap": 150})
    synth.write_case(c, d)
    return d, c


def _open(d, prec):
    with chdir(d):
        s = sks.Solver(["par=run.par"], precision=prec)
        s.load_boundary_files()
    return s


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C])
def test_state_round_trip_continues_bit_identically(case, prec):
    d, c = case
    k = 333
    a = _open(d, prec)
    a.set_tuning(4, 3, 0, 1, 0, 0)
    first = a.run(k)
    state = a.save_state()
    rest = a.run(c.nst)
    assert max(np.abs(x).max() for x in rest) > 0.05
    snaps_a = [a.snapshot(i) for i in range(6)]
    for tuning in ((4, 8, 0, 1, 0, 1), (2, 2, 1, 0, 0, 0)):
        b = _open(d, prec)
        b.set_tuning(*tuning)
        b.load_state(state)
        assert b.info()["step"] == k
        got = b.run(c.nst)
        for i in range(3):
            assert np.array_equal(got[i], rest[i]), (prec, tuning, i)
        for i, sa in enumerate(snaps_a):
            sb = b.snapshot(i)
            assert (sa is None) == (sb is None)
            if sa is not None:
                assert sa[0] == sb[0] and np.array_equal(sa[1], sb[1])
        b.close()
    # back into the same solver: it rewinds to step k
    a.load_state(state)
    again = a.run(c.nst)
    for i in range(3):
        assert np.array_equal(again[i], rest[i])
    assert first[0].shape[0] == k
    a.close()


def test_state_of_another_solve_is_refused(case, tmp_path):
    d, c = case
    a64 = _open(d, sks.FP64)
    a64.run(10)
    s64 = a64.save_state()
    a32 = _open(d, sks.FP32C)
    with pytest.raises(sks.SksError):
        a32.load_state(s64)                     # another form
    with pytest.raises(sks.SksError):
        a64.load_state(s64[:100])               # truncated
    bad = s64.copy()
    bad[:8] = 0
    with pytest.raises(sks.SksError):
        a64.load_state(bad)                     # not a state
    # damaged header words: step (int32 at byte 28), buffer index (byte 32),
    # field bytes (int64 at byte 40)
    for off, val, dt in ((28, -1, np.int32), (28, c.nst + 1, np.int32), (32, 2, np.int32), (40, 8, np.int64)):
        bad = s64.copy()
        bad[off:off + np.dtype(dt).itemsize] = np.frombuffer(np.array([val], dt).tobytes(), np.uint8)
        with pytest.raises(sks.SksError):
            a64.load_state(bad)
    a64.load_state(s64)                         # the solver is unchanged and runs on
    assert a64.info()["step"] == 10
    more = a64.run(5)
    assert more[0].shape[0] == 5 and all(np.isfinite(x).all() for x in more)
    d2 = str(tmp_path)
    c2 = synth.Case(nex=21, nez=11, eh=1.0, sdt=0.005, nst=900, layers=_layers(11.002), p=0.045, f0=1.5,
                    ntrace=5, rec_dx=3.0, semmodel_full=True)
    synth.write_case(c2, d2)
    other = _open(d2, sks.FP64)
    with pytest.raises(sks.SksError):
        other.load_state(s64)                   # another mesh
    for s in (a64, a32, other):
        s.close()
