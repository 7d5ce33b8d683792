"""GPU: boundary records from a plane wave through a layered stack
(sks_set_boundary_layered_wave).

- A stack of identical media gives the plane-wave records: the interpolated
  line increments and the solves agree to the series' interpolation error.
- The device evaluation of the mode series equals a host evaluation of the
  same series at the same node positions and times.
- The SEM itself checks the physics: a box holding a low-impedance layer,
  driven by the half-space plane wave below it, must show above the layer the
  upgoing waves the layered generator predicts.  What the injection line
  actually sends up (its constant scale, its small lag and the P it radiates
  with an SV record) is read from a homogeneous box driven the same way, so
  the layered prediction has no free parameter.
"""
import math

import numpy as np
import pytest

import sks
import synth
from util import chdir

pytestmark = pytest.mark.gpu

VP, VS, RHO = 8.1, 4.5, 3.4


def _case(d, layers, nex, nez, nst, p, f0, ntrace, rec_x0, rec_dx, sv, sh, extra=None):
    c = synth.Case(nex=nex, nez=nez, eh=1.0, sdt=0.005, nst=nst, layers=layers, p=p, f0=f0, sv_amp=sv, sh_amp=sh,
                   ntrace=ntrace, rec_x0=rec_x0, rec_dx=rec_dx, write_records=False, extra=extra or {})
    synth.write_case(c, d)
    return c


def _iso(vp, vs, rho, top):
    return synth.SemLayer(top, synth.iso_cij(vp, vs, rho), rho)


def test_identical_media_give_the_plane_wave(tmp_path):
    d = str(tmp_path)
    p, f0 = 0.044, 1.3
    c = _case(d, [_iso(VP, VS, RHO, 13.0)], 29, 12, 700, p, f0, 9, 2.0, 3.0, 1.0, 0.6)
    with chdir(d):
        a = sks.Solver(["par=run.par"], precision=sks.FP64)
        b = sks.Solver(["par=run.par"], precision=sks.FP64)
    a.set_boundary_plane_wave(VS, p, f0, 1.0, 0.6)
    b.set_boundary_layered_wave([(VP, VS, RHO), (VP, VS, RHO, 12.0), (VP, VS, RHO, 5.0), (VP, VS, RHO)], p, f0,
                                0.0, 1.0, 0.6)
    la, lb = a.line_increments(0, 400), b.line_increments(0, 400)
    scale = float(np.abs(la).max())
    assert scale > 0
    assert np.abs(la - lb).max() <= 2e-6 * scale
    ua, ub = a.run(c.nst), b.run(c.nst)
    for k in range(3):
        assert np.linalg.norm(ua[k] - ub[k]) <= 1e-5 * np.linalg.norm(ua[k]), k
    a.close()
    b.close()


def _cubic(f, tt):
    """cubic Lagrange on a periodic series at fractional sample positions tt"""
    nt = f.size
    fl = np.floor(tt)
    dd = tt - fl
    i0 = fl.astype(np.int64) % nt
    w = (-dd * (dd - 1) * (dd - 2) / 6, (dd + 1) * (dd - 1) * (dd - 2) / 2, -(dd + 1) * dd * (dd - 2) / 2,
         (dd + 1) * dd * (dd - 1) / 6)
    return sum(wk * f[(i0 + k - 1) % nt] for k, wk in enumerate(w))


def test_device_records_equal_a_host_evaluation(tmp_path):
    d = str(tmp_path)
    p, f0 = 0.04, 1.1
    top = (7.9, 4.4, 3.35)
    stack = [top, (6.6, 3.8, 2.9, 6.0), (7.2, 4.0, 3.1, 9.0), (VP, VS, RHO)]
    c = _case(d, [_iso(*top, 13.0)], 29, 12, 600, p, f0, 5, 2.0, 4.0, 1.0, 0.5)
    with chdir(d):
        host = sks.Solver(["par=run.par"], precision=sks.FP64)
        dev = sks.Solver(["par=run.par"], precision=sks.FP64)
    i = host.info()
    nx, nz, eh, dp = i["nx"], i["nz"], i["eh"], c.sdt
    nbl = i["neh"] * i["hpn"]
    nrec = max(i["nrec_psv"], i["nrec_sh"])
    dts = dp / 4
    xmax, zmax = (nx - 1) * i["h"] + eh, (nz - 1) * i["h"] + eh
    span = nrec * dp + p * xmax + zmax / top[1]
    ser = sks.layered_series(stack, p, f0, dts, span, 0.0, 1.0, 0.5)
    ep, es = math.sqrt(1 / top[0] ** 2 - p ** 2), math.sqrt(1 / top[1] ** 2 - p ** 2)
    line = synth.gll_positions(nbl + 1, eh)[nbl]
    xs = np.concatenate([synth.gll_positions(nx, eh), np.full(nz, line)])
    zs = np.concatenate([np.full(nx, line), synth.gll_positions(nz, eh)])
    t = (np.arange(nrec) * dp)[:, None]
    fp = _cubic(ser[0], (t - p * xs - ep * zs) / dts)
    fs = _cubic(ser[1], (t - p * xs - es * zs) / dts)
    fh = _cubic(ser[2], (t - p * xs - es * zs) / dts)
    ux = fp * p * top[0] + fs * es * top[1]
    uz = fp * ep * top[0] - fs * p * top[1]
    psv = np.concatenate([ux[:, :nx], -uz[:, :nx], ux[:, nx:], -uz[:, nx:]], axis=1).astype(np.float32)
    host.set_boundary(psv[:i["nrec_psv"]], fh[:i["nrec_sh"]].astype(np.float32))
    dev.set_boundary_layered_wave(stack, p, f0, 0.0, 1.0, 0.5)
    la, lb = host.line_increments(0, 400), dev.line_increments(0, 400)
    scale = float(np.abs(la).max())
    assert scale > 0
    assert np.abs(la - lb).max() <= 4 * np.finfo(np.float32).eps * scale
    host.close()
    dev.close()


def test_sem_through_a_layer_matches_the_layered_generator(tmp_path):
    """Box 280 x 100 km (1 km elements), SV + SH plane wave (p = 0.04 s/km,
    0.5 Hz) from the half-space medium below; the layered box holds a 10 km
    low-impedance layer at 16-26 km under a third medium.  Receivers 36 km up
    at x = 160..200 km; the window closes before anything from the left
    column, the right and bottom edges or the free surface can reach them."""
    p, f0, nst, dt = 0.04, 0.5, 4700, 0.005
    A = (VP, VS, RHO)
    Bm = (7.0, 4.0, 2.6)
    Tm = (7.5, 4.2, 3.1)
    z1, z2, zr, H = 16.0, 26.0, 36.0, 100.0
    runs = {}
    for name, layers in (("homogeneous", [_iso(*A, H + 1.0)]),
                         ("layered", [_iso(*A, z1), _iso(*Bm, z2), _iso(*Tm, H + 1.0)])):
        d = str(tmp_path / name)
        c = _case(d, layers, 280, 100, nst, p, f0, 5, 160.0, 10.0, 1.0, 0.7, extra={"zbeg": -(H - zr)})
        with chdir(d):
            s = sks.Solver(["par=run.par"], precision=sks.FP64)
        i = s.info()
        s.set_boundary_plane_wave(VS, p, f0, 1.0, 0.7)
        runs[name] = s.run(c.nst)
        s.close()
    # receiver nodes as the par words place them (float arithmetic, sem2d_psvsh.c:333-357)
    f32 = np.float32
    hf = f32(i["h"])
    ix = [int(f32(160.0 + 10.0 * k) / hf) for k in range(5)]
    iz = int(f32(-(H - zr)) / hf) + i["nz"] - 1
    xr = synth.gll_positions(i["nx"], i["eh"])[ix]
    zr = float(synth.gll_positions(i["nz"], i["eh"])[iz])
    assert abs(zr - 36.0) < 0.5 and np.abs(xr - (160.0 + 10.0 * np.arange(5))).max() < 0.5
    t = np.arange(nst) * dt
    # window: until 3.5 s after the direct S pulse's centre at the last receiver
    eta_s = [math.sqrt(1 / m[1] ** 2 - p ** 2) for m in (A, Bm, Tm)]
    t_s = 1.5 / f0 + p * xr + eta_s[0] * z1 + eta_s[1] * (z2 - z1) + eta_s[2] * (zr - z2)
    win = t[:, None] <= (t_s + 3.5)[None, :]
    assert t_s.max() + 3.5 <= t[-1]

    ho = [runs["homogeneous"][k].astype(np.float64) for k in (0, 2, 1)]   # seis.u (u_x), seis.w (-u_z), seis.v
    la = [runs["layered"][k].astype(np.float64) for k in (0, 2, 1)]

    def misfit(got, want):
        num = sum(np.sum(((g - q) * win) ** 2) for g, q in zip(got, want))
        return math.sqrt(num / sum(np.sum((g * win) ** 2) for g in got))

    # the homogeneous box is close to the scaled pulse (the injection's constant, as for SH in a
    # homogeneous box); the line's displacement increments also radiate some P with the SV record,
    # which is why the comparison below splits what the box records into P and SV
    pulse = synth.ricker(t[:, None] - 1.5 / f0 - p * xr[None, :] - eta_s[0] * zr, f0)
    pol = (eta_s[0] * VS, p * VS)                 # SV: u_x, -u_z per unit amplitude
    k_sv = sum(np.sum(g * q * pulse * win) for g, q in zip(ho[:2], pol)) / (np.sum(pulse * pulse * win) * 1.0)
    k_sh = np.sum(ho[2] * pulse * win) / np.sum(pulse * pulse * win) / 0.7
    print(f"homogeneous box: scale SV {k_sv:.4f} SH {k_sh:.4f}, misfit to the scaled pulse "
          f"{misfit(ho, (k_sv * pol[0] * pulse, k_sv * pol[1] * pulse, 0.7 * k_sh * pulse)):.4f}")
    assert 1.5 < k_sv < 3.0 and abs(k_sh / k_sv - 1.0) < 0.02

    # what the line injects, as the homogeneous box records it at each receiver
    # (split into its upgoing P and SV parts; SH apart), carried through the
    # stack [third medium, layer, half-space medium]: each incident mode is
    # moved back to the stack's top (26 km up), transferred, and each upgoing
    # mode moved up to the receivers, exact delays in the frequency domain
    stack = [Tm, Bm + (z2 - z1,), A]
    nfft = 1 << int(math.ceil(math.log2(3 * nst)))
    om = 2 * math.pi * np.fft.rfftfreq(nfft, dt)
    coef = [sks.layered_coefficients(stack, p, float(w)) for w in om]
    tpsv = np.array([c["t_psv"] for c in coef])          # [w][out][in]
    t_hh = np.array([c["t_sh"] for c in coef])
    ep_a, es_a = math.sqrt(1 / VP ** 2 - p ** 2), eta_s[0]
    ep_t, es_t = math.sqrt(1 / Tm[0] ** 2 - p ** 2), math.sqrt(1 / Tm[1] ** 2 - p ** 2)
    dz = zr - z2
    back = (np.exp(1j * om * ep_a * (zr - z2)), np.exp(1j * om * es_a * (zr - z2)))   # incident P, SV to the top
    up = (np.exp(-1j * om * ep_t * dz), np.exp(-1j * om * es_t * dz))                   # upgoing P, SV to the receivers
    # (u_x, -u_z) of a unit upgoing P and SV in the half-space medium
    mode = np.array([[p * VP, es_a * VS], [-ep_a * VP, p * VS]])
    split = np.linalg.inv(mode)
    want = [np.zeros_like(ho[0]) for _ in range(3)]
    for k in range(5):
        a_p = split[0, 0] * ho[0][:, k] + split[0, 1] * ho[1][:, k]
        a_s = split[1, 0] * ho[0][:, k] + split[1, 1] * ho[1][:, k]
        inc = (np.fft.rfft(a_p, nfft) * back[0], np.fft.rfft(a_s, nfft) * back[1])
        out = [np.fft.irfft((tpsv[:, m, 0] * inc[0] + tpsv[:, m, 1] * inc[1]) * up[m], nfft)[:nst] for m in (0, 1)]
        want[0][:, k] = out[0] * p * Tm[0] + out[1] * es_t * Tm[1]
        want[1][:, k] = -(out[0] * ep_t * Tm[0] - out[1] * p * Tm[1])
        want[2][:, k] = np.fft.irfft(np.fft.rfft(ho[2][:, k], nfft) * t_hh * back[1] * up[1], nfft)[:nst]
    for name, g, q in zip(("u_x", "-u_z", "u_y"), la, want):
        print(f"  {name}: misfit {math.sqrt(np.sum(((g - q) * win) ** 2) / np.sum((g * win) ** 2)):.4f}")
    e_layered = misfit(la, want)
    e_naive = misfit(la, ho)                         # as if the layer were not there
    print(f"layered box: misfit {e_layered:.4f} to the layered generator, {e_naive:.4f} to the unlayered wave")
    assert e_layered < 0.015, (e_layered, e_naive)
    assert e_naive > 30 * e_layered, (e_layered, e_naive)


@pytest.mark.parametrize("form", ["plane", "stack"])
def test_program_generator_words(tmp_path, form):
    """The drop-in program with sks_plane_wave= or sks_stack= / sks_wave=
    writes the seismograms the library gives with the same generator."""
    import os
    import subprocess
    d = str(tmp_path)
    p, f0 = 0.04, 1.2
    top = (7.9, 4.4, 3.35)
    c = _case(d, [_iso(*top, 13.0)], 29, 12, 500, p, f0, 6, 2.0, 4.0, 1.0, 0.5)
    stack = [top, (6.6, 3.8, 2.9, 6.0), (VP, VS, RHO)]
    with open(os.path.join(d, "stack.txt"), "w") as f:
        f.write("# box bottom medium, layer, half-space\n")
        for m in stack:
            f.write(" ".join(repr(float(v)) for v in (tuple(m) + (0.0,))[:4]) + "\n")
    words = (["sks_plane_wave=4.4,0.04,1.2,1.0,0.5"] if form == "plane"
             else ["sks_stack=stack.txt", "sks_wave=0.04,1.2,0.0,1.0,0.5"])
    cli = os.path.join(os.path.dirname(sks.LIB_PATH), "sem2d_psvsh_gb300")
    r = subprocess.run([cli, "par=run.par"] + words, cwd=d, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    with chdir(d):
        s = sks.Solver(["par=run.par"], precision=sks.FP64)
    if form == "plane":
        s.set_boundary_plane_wave(4.4, p, f0, 1.0, 0.5)
    else:
        s.set_boundary_layered_wave(stack, p, f0, 0.0, 1.0, 0.5)
    u, v, w = s.run(c.nst)
    s.close()
    for name, want in (("seis.u", u), ("seis.v", v), ("seis.w", w)):
        got = np.fromfile(os.path.join(d, name), np.float32).reshape(c.nst, -1)
        assert np.abs(want).max() > 0
        assert np.array_equal(got, want), name
