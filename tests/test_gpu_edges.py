"""GPU: edge cases of the solve against the FP64 oracle: the smallest mesh the
solver accepts (3 x 2 elements), a run of a single step (step 0 only) and of
single steps one call at a time, and a solve without receivers (alone, in a
batch, saved and restored)."""
import numpy as np
import pytest

import sks
import synth
from oracle.oracle import Oracle
from util import chdir, seis_err

pytestmark = pytest.mark.gpu


def _case(d, **kw):
    nez = kw.pop("nez")
    c = synth.Case(eh=2.0, sdt=0.01, layers=synth.layered_two(nez * 2.0 + 0.002, 2.0), p=0.04, f0=1.0, nez=nez,
                   sh_amp=0.5, **kw)
    synth.write_case(c, d)
    return c


def _oracle(d, nst):
    with chdir(d):
        o = Oracle(["par=run.par"], fp64=True)
        ref = o.run(nst)
        o.close()
    return ref


def _open(d, prec):
    with chdir(d):
        s = sks.Solver(["par=run.par"], precision=prec)
        s.load_boundary_files()
    return s


@pytest.mark.parametrize("prec,tol", [(sks.FP64, 1e-10), (sks.FP32C, 1e-4)])
def test_smallest_mesh_matches_oracle(tmp_path, prec, tol):
    d = str(tmp_path)
    c = _case(d, nex=3, nez=2, nst=300, ntrace=2, rec_dx=4.0)
    ref = _oracle(d, c.nst)
    assert max(np.abs(r).max() for r in ref) > 1e-3
    s = _open(d, prec)
    for t in ((4, 1, 0, 0, 0, 0), (2, 2, 1, 1, 0, 1), (4, 2, 0, 1, 0, 1)):
        s.reset()
        s.set_tuning(*t)
        out = s.run(c.nst)
        assert seis_err(out, ref) <= tol, t
    s.close()


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C])
def test_single_steps(tmp_path, prec):
    d = str(tmp_path)
    c = _case(d, nex=12, nez=6, nst=450, ntrace=5, rec_dx=4.0)
    ref = _oracle(d, c.nst)
    assert max(np.abs(r).max() for r in ref) > 0.05
    first = _oracle(d, 1)
    s = _open(d, prec)
    one = s.run(1)                                   # step 0 alone
    for i in range(3):
        assert one[i].shape == (1, 5)
        assert np.allclose(one[i], first[i], rtol=0, atol=1e-6 * max(1e-30, np.abs(ref[i]).max()))
    rows = [one] + [s.run(1) for _ in range(c.nst - 1)]
    got = tuple(np.concatenate([r[i] for r in rows]) for i in range(3))
    assert seis_err(got, ref) <= (1e-10 if prec == sks.FP64 else 1e-4)
    assert s.run(5)[0].shape == (0, 5)                # the run is over
    s.close()


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C])
def test_solve_without_receivers(tmp_path, prec):
    d = str(tmp_path)
    c = _case(d, nex=12, nez=5, nst=120, ntrace=0, rec_dx=4.0)
    s = _open(d, prec)
    assert s.info()["ntrace"] == 0
    out = s.run(60)
    assert all(o.shape == (60, 0) for o in out)
    st = s.save_state()
    rest = s.run(c.nst)
    assert all(o.shape == (60, 0) for o in rest)
    s.load_state(st)
    assert s.info()["step"] == 60
    s.reset()
    with sks.Batch(prec) as b:
        b.add(s)
        got = b.run(c.nst)
        assert got[0][0].shape == (c.nst, 0)
        assert s.info()["step"] == c.nst
        b.remove(s)
    s.close()
