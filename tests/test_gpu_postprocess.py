"""GPU: device band-pass and Silver-Chan splitting of many receivers against
the host restatement (scipy sections forward and backward; splitting.py), on
synthetic split waves with known parameters and on a solve's seismograms."""
import numpy as np
import pytest

import sks
import splitting
import synth
from util import chdir

pytestmark = pytest.mark.gpu
signal = pytest.importorskip("scipy.signal")


def _device_split(rad, trn, dt, opts):
    torch = pytest.importorskip("torch")
    nt, ntrace = rad.shape                      # time-major [nt][ntrace]
    dev = torch.device("cuda:0")
    a = torch.from_numpy(np.ascontiguousarray(rad, dtype=np.float32)).to(dev)
    b = torch.from_numpy(np.ascontiguousarray(trn, dtype=np.float32)).to(dev)
    wf, sd = sks.split_scratch(ntrace, nt, dt, opts)
    work = torch.zeros(wf, dtype=torch.float32, device=dev)
    sums = torch.zeros(sd, dtype=torch.float64, device=dev)
    out = torch.zeros(4 * ntrace, dtype=torch.float32, device=dev)
    sks.split_traces_device(a.data_ptr(), b.data_ptr(), ntrace, nt, ntrace, dt, opts, work.data_ptr(),
                            sums.data_ptr(), out.data_ptr(), torch.cuda.current_stream(dev).cuda_stream)
    torch.cuda.synchronize(dev)
    filt = work.cpu().numpy().reshape(2, ntrace, nt)
    return out.cpu().numpy().reshape(ntrace, 4), filt


def _host_filter(x, sos, passes):
    y = signal.sosfilt(sos, x.astype(np.float64))
    if passes == 2:
        y = signal.sosfilt(sos, y[::-1])[::-1]
    return y


def test_known_splits_recovered_on_device():
    dt = 0.01
    t = np.arange(6000) * dt
    truth = [(45.0, 1.0), (-30.0, 0.6), (10.0, 1.75), (-80.0, 0.35), (65.0, 1.2), (0.5, 0.9)]
    rad, trn = [], []
    for phi, dl in truth:
        x, y = splitting.apply_splitting(synth.ricker(t - 25.0, 0.3), np.zeros_like(t), phi, dl, dt)
        rad.append(x)
        trn.append(y)
    rad, trn = np.array(rad).T, np.array(trn).T
    opts = sks.SplitOpts(0.0, 0.0, 2, 1, 12.0, 12.0, 3.0, 0.25)      # no filter
    out, _ = _device_split(rad, trn, dt, opts)
    for r, (phi, dl) in enumerate(truth):
        assert abs(out[r, 0] - phi) <= 0.5, (r, out[r])
        assert abs(out[r, 1] * dt - dl) <= 2 * dt, (r, out[r])
        assert out[r, 2] < 1e-3


def test_filter_and_splitting_match_the_host_on_a_solve(tmp_path):
    d = str(tmp_path)
    H = 20.002
    layers = [synth.SemLayer(H - 8, synth.iso_cij(8.1, 4.5, 3.4), 3.4),
              synth.SemLayer(H - 3, synth.hexagonal_cij(8.1, 4.5, 3.4, 0.06, 50.0, 15.0), 3.4),
              synth.SemLayer(H + 1, synth.iso_cij(6.4, 3.6, 2.8), 2.8)]
    c = synth.Case(nex=40, nez=10, eh=2.0, sdt=0.01, nst=1500, layers=layers, p=0.045, f0=0.6, ntrace=16,
                   rec_dx=4.0, semmodel_full=True)
    synth.write_case(c, d)
    with chdir(d), sks.Solver(["par=run.par"], precision=sks.FP64) as s:
        s.load_boundary_files()
        u, v, w = s.run(c.nst)
    opts = sks.SplitOpts(0.05, 1.5, 2, 2, 5.0, 8.0, 2.0, 0.5)
    out, filt = _device_split(u, v, c.sdt, opts)
    sos = sks.bandpass_design(0.05, 1.5, 2, c.sdt)
    agree = 0
    for r in range(c.ntrace):
        hx = _host_filter(u[:, r], sos, 2)
        hy = _host_filter(v[:, r], sos, 2)
        assert np.linalg.norm(filt[0, r] - hx) <= 1e-5 * np.linalg.norm(hx)
        assert np.linalg.norm(filt[1, r] - hy) <= 1e-5 * max(np.linalg.norm(hy), 1e-30)
        x32, y32 = filt[0, r].astype(np.float64), filt[1, r].astype(np.float64)
        i = int(np.argmax(np.abs(x32)))
        win = (max(0, i - 500), min(len(x32), i + 800))
        assert int(out[r, 3]) == win[0]
        ref = splitting.splitting(x32, y32, c.sdt, win, max_delay=2.0, dphi=0.5)
        _, lam2, lam1 = splitting.eigen_grid(x32, y32, c.sdt, win, max_delay=2.0, dphi=0.5)
        jp, k = int(round((out[r, 0] + 90.0) / 0.5)), int(out[r, 1])
        jm = np.unravel_index(int(np.argmin(lam2)), lam2.shape)
        # the device's cell is a minimum of the host's grid to rounding (the
        # valley can be flat enough for rounding to pick a neighbouring cell)
        assert lam2[jp, k] <= lam2[jm] + 1e-10 * lam1[jm], (r, out[r], ref)
        assert abs(out[r, 2] - ref["lambda_ratio"]) <= 1e-6 + 1e-3 * ref["lambda_ratio"]
        agree += (jp, k) == jm
    assert agree >= c.ntrace // 2
