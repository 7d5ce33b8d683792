"""GPU: the allocation-free boundary increments agree with the allocating ones.

sks_line_increments_noalloc() serves callers that must not allocate device
memory when they run (their memory is already divided up by a serving process
or a host plugin interface, or they cannot afford cudaMalloc's device-wide
synchronization).  The caller hands it device buffers it already owns; the
FP64 interpolation rows go to a fixed scratch array inside the library.  Here
the caller's buffers are made with torch, the call is made twice in a row
(different step ranges, so the second call runs over the first one's scratch
contents), and each result is compared with sks_line_increments() on the same
solve.  A third call comes from a fresh host thread, in which no CUDA context
is current yet when the call starts.  This file is collected last on purpose.
"""
import ctypes as C
import threading

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


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def test_noalloc_matches_allocating_entry_point(tmp_path):
    torch = pytest.importorskip("torch")
    d = str(tmp_path)
    c = synth.Case(nex=16, nez=10, eh=2.0, sdt=0.005, dp=0.01, nt=300, nst=700, layers=_layers(20.0),
                   p=0.05, f0=1.0, sh_amp=0.5, ntrace=7, rec_dx=4.0, semmodel_full=True)
    synth.write_case(c, d)
    with chdir(d), sks.Solver(["par=run.par"], precision=sks.FP64) as s, sks.Setup(["par=run.par"]) as su:
        s.load_boundary_files()
        info = s.info()
        nx, nz, nbl = info["nx"], info["nz"], info["neh"] * info["hpn"]
        tp, wp, ts, ws = su.schedule()
        dev = torch.device("cuda:0")
        psv = torch.from_numpy(np.fromfile("greenfile", np.float32)).to(dev)
        sh = torch.from_numpy(np.fromfile("shgreenfile", np.float32)).to(dev)
        stream = torch.cuda.current_stream(dev)
        for it0, n, fresh in ((5, 60, False), (120, 37, False), (5, 60, True)):   # calls in a row
            ref = s.line_increments(it0, n)
            assert np.abs(ref).max() > 0
            sl = slice(it0, it0 + n + 1)           # the schedule of steps it0..it0+n
            tap_p = torch.from_numpy(np.ascontiguousarray(tp[sl])).to(dev)
            w_p = torch.from_numpy(np.ascontiguousarray(wp[sl])).to(dev)
            tap_s = torch.from_numpy(np.ascontiguousarray(ts[sl])).to(dev)
            w_s = torch.from_numpy(np.ascontiguousarray(ws[sl])).to(dev)
            out = torch.full((n, ref.shape[1], 3), float("nan"), dtype=torch.float64, device=dev)
            res = {}

            def call():
                res["rc"] = sks.lib().sks_line_increments_noalloc(_ptr(psv), _ptr(sh), nx, nz, nbl, _ptr(tap_p),
                                                                  _ptr(w_p), _ptr(tap_s), _ptr(w_s), n, _ptr(out),
                                                                  C.c_void_p(stream.cuda_stream))
                res["err"] = sks.lib().sks_last_error().decode()   # the error text is per host thread

            if fresh:
                t = threading.Thread(target=call)
                t.start()
                t.join()
            else:
                call()
            assert res["rc"] == 0, res["err"]
            torch.cuda.synchronize(dev)
            got = out.cpu().numpy()
            assert np.allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def test_noalloc_rejects_sizes_beyond_its_scratch():
    # (nsteps+2) * 3*(nx+nz) above the 1 Mi-double scratch: refused before any GPU work
    one = C.c_void_p(1)
    rc = sks.lib().sks_line_increments_noalloc(one, one, 3201, 1201, 4, one, one, one, one, 100, one, None)
    assert rc == -1
    assert "scratch" in sks.lib().sks_last_error().decode()
