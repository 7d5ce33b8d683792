"""GPU: every tuning of the step kernel gives bit-identical seismograms, and the
autotuner leaves the solve where it found it.

The CTA grid (warps per CTA, band height, band-seam method, register cap,
pipelined chunks) changes which CTA computes an element and when, never the
arithmetic: a halo element is recomputed with the same inputs and code, and
each point's force is summed in the same order.
"""
import numpy as np
import pytest

import sks
import synth
from util import chdir

pytestmark = pytest.mark.gpu


def _layers(H):
    return [synth.SemLayer(H - 6, synth.iso_cij(8.1, 4.5, 3.4), 3.4),
            synth.SemLayer(H - 3, synth.hexagonal_cij(8.1, 4.5, 3.4, 0.06, 30.0, 20.0), 3.4),
            synth.SemLayer(H + 1, synth.iso_cij(6.4, 3.6, 2.8), 2.8)]


@pytest.fixture(scope="module")
def case(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("tuning"))
    c = synth.Case(nex=53, nez=23, eh=1.0, sdt=0.005, nst=900, layers=_layers(23.0), p=0.045, f0=1.5,
                   sv_amp=1.0, sh_amp=0.3, ntrace=25, rec_dx=2.1, semmodel_full=True)
    synth.write_case(c, d)
    return d, c


def _run(d, prec, nst, tuning=None, autotune=False):
    with chdir(d), sks.Solver(["par=run.par"], precision=prec) as s:
        s.load_boundary_files()
        if tuning:
            s.set_tuning(*tuning)
        got = None
        if autotune:
            a = s.run(37)
            before = s.info()["step"]
            got = s.autotune(6)
            assert s.info()["step"] == before
            b = s.run(nst - 37)
            out = tuple(np.concatenate([a[i], b[i]]) for i in range(3))
        else:
            out = s.run(nst)
        return out, got, s.tuning()


TUNINGS = ([(nw, hz, zs, cap, wv, 0) for nw in (2, 4) for hz in (1, 3, 23) for zs in (0, 1) for cap in (0, 1, 2)
            for wv in (0,)] + [(nw, 4, zs, 1, wv, 0) for nw in (2, 4) for zs in (0, 1) for wv in (1, 2, 5)]
           + [(nw, hz, zs, cap, 0, 1) for nw in (2, 4) for hz in (1, 3, 23) for zs in (0, 1) for cap in (0, 1, 2)])


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C])
def test_all_tunings_bit_identical(case, prec):
    d, c = case
    ref, _, _ = _run(d, prec, c.nst, tuning=(4, 8, 1, 0, 0, 0))
    assert max(np.abs(x).max() for x in ref) > 0.1
    for t in TUNINGS:
        out, _, used = _run(d, prec, c.nst, tuning=t)
        got = (used["warps_per_block"], used["zseam"], used["register_cap"], used["waves"], used["pipeline"])
        assert got == (t[0], t[2], t[3], t[4], t[5])
        if t[4] == 0:
            assert used["band_rows"] == t[1]
        for i in range(3):
            assert np.array_equal(out[i], ref[i]), f"tuning {t} differs in component {i}"


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C])
def test_autotune_restores_state(case, prec):
    d, c = case
    ref, _, _ = _run(d, prec, c.nst)
    out, best, used = _run(d, prec, c.nst, autotune=True)
    assert best["ms_per_step"] > 0
    assert (used["warps_per_block"], used["band_rows"], used["zseam"]) == \
           (best["warps_per_block"], best["band_rows"], best["zseam"])
    for i in range(3):
        assert np.array_equal(out[i], ref[i])
