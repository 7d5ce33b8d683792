"""GPU: a known answer of the physics.  A vertically incident SV plane wave
(the SKS geometry, p = 0) crossing a hexagonal layer of thickness L whose
symmetry axis is horizontal at azimuth az splits into a fast S wave polarised
along the axis and a slow one across it: Silver-Chan analysis of the surface
seismograms recovers the fast axis at az and the delay
L (1/vs_slow - 1/vs_fast).  Both forms, through the C ABI, on receivers away
from the injection column (which carries the isotropic half-space plane wave
through the layer)."""
import numpy as np
import pytest

import sks
import splitting
import synth
from util import chdir

pytestmark = pytest.mark.gpu

H, L, AZ, S, VS = 120.002, 50.0, 30.0, 0.04, 4.5


@pytest.fixture(scope="module")
def case(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("sks_split"))
    layers = [synth.SemLayer(H - L, synth.iso_cij(8.1, VS, 3.4), 3.4),
              synth.SemLayer(H + 1, synth.hexagonal_cij(8.1, VS, 3.4, S, AZ, 0.0), 3.4)]
    c = synth.Case(nex=40, nez=60, eh=2.0, sdt=0.01, nst=3700, layers=layers, p=0.0, f0=0.4, sv_amp=1.0,
                   sh_amp=0.0, ntrace=5, rec_x0=20.0, rec_dx=10.0, semmodel_full=True)
    synth.write_case(c, d)
    return d, c


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C])
def test_vertical_sks_splits_by_the_layer(case, prec):
    d, c = case
    with chdir(d), sks.Solver(["par=run.par"], precision=prec) as s:
        s.load_boundary_files()
        u, v, _ = s.run(c.nst)
    want = L * (1.0 / (VS * (1 - S / 2)) - 1.0 / (VS * (1 + S / 2)))        # 0.445 s
    for r in (2, 3, 4):                                                     # x = 40, 50, 60 km
        x, y = u[:, r].astype(np.float64), v[:, r].astype(np.float64)
        assert np.abs(x).max() > 1.0
        res = splitting.splitting(x, y, c.sdt, splitting.sks_window(x, c.sdt, 6.0), max_delay=2.0, dphi=0.5)
        assert abs(res["phi_deg"] - AZ) <= 2.0, (r, res)
        assert abs(res["delay_s"] - want) <= 0.03, (r, res, want)
        assert res["lambda_ratio"] < 0.01


def _state_fields(st, nx, nz, prec):
    """views into a saved state: U0, U1 as [3][np] arrays in the buffer's
    layout ((u_x, u_z) pairs, then u_y) and, for FP32C, the (d, c) pairs"""
    np_ = nx * nz
    dt = np.float64 if prec == sks.FP64 else np.float32
    el = np.dtype(dt).itemsize
    o = 88
    u0 = np.frombuffer(st, dtype=dt, count=3 * np_, offset=o)
    u1 = np.frombuffer(st, dtype=dt, count=3 * np_, offset=o + 3 * np_ * el)
    dv = np.frombuffer(st, dtype=np.float32, count=6 * np_, offset=o + 6 * np_ * el) if prec == sks.FP32C else None
    return u0, u1, dv


def _layout(ux, uy, uz):
    return np.concatenate([np.stack([ux, uz], axis=1).ravel(), uy])


@pytest.mark.parametrize("prec,tol", [(sks.FP64, 1e-12), (sks.FP32C, 2e-5)])
@pytest.mark.parametrize("motion", ["translation", "rotation"])
def test_rigid_motions_stay_at_rest(tmp_path, prec, tol, motion):
    """K annihilates rigid motions: a uniform displacement, or a small rigid
    rotation of the x-z plane (zero strain; exact through the degree-4 GLL
    derivatives), loaded as the state of a solve with no incident wave, stays
    where it is -- inside, on the free surface and on the absorbing edges."""
    d = str(tmp_path)
    layers = [synth.SemLayer(10.0, synth.iso_cij(8.1, 4.5, 3.4), 3.4),
              synth.SemLayer(20.5, synth.hexagonal_cij(7.0, 4.0, 3.0, 0.05, 35.0, 20.0), 3.0)]
    c = synth.Case(nex=24, nez=10, eh=2.0, sdt=0.01, nst=260, layers=layers, p=0.04, f0=1.0, ntrace=5, rec_dx=4.0,
                   semmodel_full=True, write_records=False)
    summ = synth.write_case(c, d)
    with chdir(d):
        s = sks.Solver(["par=run.par"], precision=prec)
    s.set_boundary_plane_wave(summ["vs"], c.p, c.f0, 0.0, 0.0)      # no incident wave
    s.run(10)
    info = s.info()
    nx, nz = info["nx"], info["nz"]
    st = s.save_state().copy()
    u0, u1, dv = _state_fields(st, nx, nz, prec)
    # node coordinates: GLL points of degree 4 inside each element (not evenly spaced)
    eh = info["eh"]
    xi = np.array([-1.0, -np.sqrt(3.0 / 7.0), 0.0, np.sqrt(3.0 / 7.0), 1.0])

    def coord(i):
        e, a = np.divmod(i, 4)
        return e * eh + (xi[a] + 1.0) * eh / 2.0

    z, x = np.meshgrid(coord(np.arange(nz)), coord(np.arange(nx)), indexing="ij")
    if motion == "translation":
        ux, uy, uz = np.full(nx * nz, 0.7), np.full(nx * nz, -0.4), np.full(nx * nz, 0.25)
    else:
        a = 1e-3                                                   # radians
        ux, uy, uz = (a * (z - 10.0)).ravel(), np.zeros(nx * nz), (-a * (x - 24.0)).ravel()
    field = _layout(ux, uy, uz)
    np.copyto(u0, field.astype(u0.dtype))
    np.copyto(u1, field.astype(u1.dtype))
    if dv is not None:
        np.copyto(dv, 0.0)
    s.load_state(st)
    s.run(200)
    after = s.save_state()
    a0, a1, _ = _state_fields(after, nx, nz, prec)
    scale = np.abs(field).max()
    for arr in (a0, a1):
        err = np.abs(arr.astype(np.float64) - field).max() / scale
        assert err <= tol, (motion, err)
    s.close()


def _uvec(arr, np_):
    """(u_x, u_y, u_z) of a state buffer array in the device layout, [np][3]"""
    a = arr.astype(np.float64)
    pairs = a[:2 * np_].reshape(np_, 2)
    return np.stack([pairs[:, 0], a[2 * np_:3 * np_], pairs[:, 1]], axis=1)


def test_energy_is_conserved_without_absorbing_edges(tmp_path):
    """absorb=0 and no incident wave: the leapfrog's discrete energy
    E = 1/2 |(u^{n+1} - u^n)/dt|^2_M + 1/2 (u^n)^T K u^{n+1} is constant; K u^n
    follows from the FP64 update itself, K u^n = M (2u^n - u^{n-1} - u^{n+1})/dt^2,
    with the lumped mass M of the set-up.  Starting from a Gaussian displacement
    in an anisotropic layered box, E stays within 1e-10 over 400 steps."""
    d = str(tmp_path)
    layers = [synth.SemLayer(12.0, synth.iso_cij(8.1, 4.5, 3.4), 3.4),
              synth.SemLayer(24.5, synth.hexagonal_cij(7.0, 4.0, 3.0, 0.05, 35.0, 20.0), 3.0)]
    c = synth.Case(nex=20, nez=12, eh=2.0, sdt=0.01, nst=440, layers=layers, p=0.04, f0=1.0, ntrace=3, rec_dx=4.0,
                   semmodel_full=True, write_records=False, absorb=0)
    summ = synth.write_case(c, d)
    with chdir(d):
        su = sks.Setup(["par=run.par"])
        mass, _ = su.mass()
        su.close()
        s = sks.Solver(["par=run.par"], precision=sks.FP64)
    s.set_boundary_plane_wave(summ["vs"], c.p, c.f0, 0.0, 0.0)
    s.run(2)
    info = s.info()
    nx, nz, dt = info["nx"], info["nz"], info["sdt"]
    np_ = nx * nz
    st = s.save_state().copy()
    u0, u1, _ = _state_fields(st, nx, nz, sks.FP64)
    xi = np.array([-1.0, -np.sqrt(3.0 / 7.0), 0.0, np.sqrt(3.0 / 7.0), 1.0])
    eh = info["eh"]
    e, a = np.divmod(np.arange(max(nx, nz)), 4)
    co = e * eh + (xi[a] + 1.0) * eh / 2.0
    z, x = np.meshgrid(co[:nz], co[:nx], indexing="ij")
    g = np.exp(-((x - 20.0) ** 2 + (z - 12.0) ** 2) / (2 * 3.0 ** 2)).ravel()
    field = _layout(0.8 * g, 0.5 * g, -0.3 * g)
    np.copyto(u0, field)
    np.copyto(u1, field)
    s.load_state(st)

    def energy():
        a = s.save_state()
        s.run(1)
        b = s.save_state()
        ua, ub, _ = _state_fields(a, nx, nz, sks.FP64)
        vb0, vb1, _ = _state_fields(b, nx, nz, sks.FP64)
        # consecutive fields: with k steps done, the state holds the newest
        # level in buffer (k-1)&1 and the one before in k&1 (the header's step
        # is the int32 at byte 28); one step later the newest is in k&1
        step = int(np.frombuffer(a, np.int32, count=1, offset=28)[0])
        un, unm1 = (ua, ub) if (step - 1) % 2 == 0 else (ub, ua)
        unp1 = vb0 if step % 2 == 0 else vb1
        un, unm1, unp1 = _uvec(un, np_), _uvec(unm1, np_), _uvec(unp1, np_)
        ku = mass[:, None] * (2 * un - unm1 - unp1) / dt ** 2
        v = (unp1 - un) / dt
        return 0.5 * np.sum(mass[:, None] * v * v) + 0.5 * np.sum(ku * unp1)

    e0 = energy()
    s.run(400)
    e1 = energy()
    assert e0 > 0
    assert abs(e1 - e0) <= 1e-10 * e0, (e0, e1)
    s.close()


@pytest.mark.parametrize("prec", [sks.FP64, sks.FP32C])
def test_plane_sh_wave_in_a_homogeneous_box(tmp_path, prec):
    """A plane SH wave (p = 0.04 s/km, 0.3 Hz Ricker) in a homogeneous box
    against the analytic solution.  Inside the box, before the free-surface
    reflection comes back down, the snapshots follow R(t - t0 - p x - eta z)
    with eta = sqrt(1/vs^2 - p^2): same shape and timing, amplitude constant in
    time (the injection of the line's record increments scales the incident
    wave by a constant, 2.24 here, the same in the reference's scheme).  At the
    free surface the seismogram is the incident wave doubled."""
    import math
    d = str(tmp_path)
    vs, p, f0, dt = 4.5, 0.04, 0.3, 0.005
    layers = [synth.SemLayer(41.002, synth.iso_cij(8.1, vs, 3.4), 3.4)]
    c = synth.Case(nex=80, nez=40, eh=1.0, sdt=dt, nst=3300, layers=layers, p=p, f0=f0, sv_amp=0.0, sh_amp=1.0,
                   ntrace=3, rec_x0=30.0, rec_dx=10.0, write_records=False,
                   extra={"plot_snap": 1, "startsnap": 1900, "incresnap": 100})
    summ = synth.write_case(c, d)
    with chdir(d):
        s = sks.Solver(["par=run.par"], precision=prec)
    s.set_boundary_plane_wave(summ["vs"], p, f0, 0.0, 1.0)
    _, v, _ = s.run(c.nst)
    info = s.info()
    nx, nz, eh = info["nx"], info["nz"], info["eh"]
    xs, zs = synth.gll_positions(nx, eh), synth.gll_positions(nz, eh)
    eta = math.sqrt(1.0 / vs ** 2 - p ** 2)
    amps = []
    for k in range(7):                                   # steps 1900 .. 2500: the pulse between 13 and 27 km
        step, snap = s.snapshot(k)
        col = snap[80, :, 1].astype(np.float64)          # u_y on the column x = 40 km (every second point)
        want = synth.ricker(step * dt - 1.5 / f0 - (p * xs[160] + eta * zs[0::2][:col.size]), f0)
        assert np.dot(col, want) / np.linalg.norm(col) / np.linalg.norm(want) >= 0.999, step
        assert abs(np.argmax(np.abs(col)) - np.argmax(np.abs(want))) <= 1, step
        amps.append(np.dot(col, want) / np.dot(want, want))
    A = float(np.mean(amps))
    assert max(abs(a - A) for a in amps) <= 0.01 * A
    # the receiver at x = 50 km on the free surface: twice the incident wave
    ix = int(round(50.0 / info["h"]))
    t = np.arange(c.nst) * dt
    want = synth.ricker(t - 1.5 / f0 - (p * xs[ix] + eta * zs[-1]), f0)
    got = v[:, 2].astype(np.float64)
    lag = max(range(-4, 5), key=lambda L: np.dot(np.roll(want, L), got))
    w = np.roll(want, lag)
    assert np.dot(w, got) / np.linalg.norm(w) / np.linalg.norm(got) >= 0.999
    assert abs(np.dot(w, got) / np.dot(w, w) / A - 2.0) <= 0.02
    s.close()
