"""Synthetic inputs for the semsyn SEM solver, in the reference's own file formats.

A case directory holds what `sem2d_psvsh par=run.par` reads:

* ``run.par``      getpar words (keys of semsyn/src/sem2d_psvsh.c:154-205);
* ``raymodel``     1-D ray model: ``jo nb`` / jo lines ``vp vs rho thk`` (top down)
                   / ``lfinal`` / rays (semsyn/src/readmodel.c:61-107);
* ``semmodel``     layer table: ``nll`` then per layer ``np c11 c12 c13 c16 c22 c23
                   c26 c33 c36 c44 c45 c55 c66 rho``, an x line and a height line
                   (sem2d_psvsh.c:703-738); with ``semmodel_full=1`` the layer line
                   carries all 21 Voigt constants then rho;
* ``greenfile``    time-major float32 records of 2(nx+nz) values
                   [u_bottom(nx), w_bottom(nx), u_left(nz), w_left(nz)], w positive
                   down (the demultiplexed GRT output, semsyn/src/demult.c:63-78);
* ``shgreenfile``  time-major float32 records of (nx+nz) values [v_bottom, v_left];
* ``rec_file``     ``n`` then n receiver x positions in km (sem2d_psvsh.c:347-357).

The boundary traces are an analytic upgoing plane wave (SV and/or SH, Ricker
wavelet) in the homogeneous layer that holds the injection line; the GRT
generator of the reference (Fortran) is not part of this path.  Elastic
constants are in (km/s)^2 * g/cc, lengths in km, times in s, as in the
reference.  Anisotropic layers are hexagonal with a fast symmetry axis rotated
to a given azimuth (from +x toward +y) and tilt (up from horizontal) in FP64.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

VOIGT = {(0, 0): 0, (1, 1): 1, (2, 2): 2, (1, 2): 3, (2, 1): 3, (0, 2): 4, (2, 0): 4, (0, 1): 5, (1, 0): 5}


def iso_cij(vp: float, vs: float, rho: float) -> np.ndarray:
    """6x6 Voigt stiffness of an isotropic solid (c11 = rho vp^2, c44 = rho vs^2)."""
    c11 = rho * vp * vp
    c44 = rho * vs * vs
    c12 = c11 - 2.0 * c44
    C = np.zeros((6, 6))
    C[:3, :3] = c12
    for i in range(3):
        C[i, i] = c11
        C[i + 3, i + 3] = c44
    return C


def _voigt_to_tensor(C: np.ndarray) -> np.ndarray:
    c = np.zeros((3, 3, 3, 3))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                for l in range(3):
                    c[i, j, k, l] = C[VOIGT[i, j], VOIGT[k, l]]
    return c


def _tensor_to_voigt(c: np.ndarray) -> np.ndarray:
    C = np.zeros((6, 6))
    for (i, j), m in VOIGT.items():
        for (k, l), n in VOIGT.items():
            C[m, n] = c[i, j, k, l]
    return 0.5 * (C + C.T)


def hexagonal_cij(vp: float, vs: float, rho: float, strength: float,
                  azimuth_deg: float, tilt_deg: float) -> np.ndarray:
    """Hexagonal (transversely isotropic) stiffness with a FAST symmetry axis.

    P and S velocities along the axis are v(1+s/2), across it v(1-s/2), so the
    S splitting strength for propagation across the axis is ``strength``
    (elliptical condition for c13).  The axis points at ``azimuth`` from +x
    toward +y and ``tilt`` up from the horizontal; the rotation is done on the
    4th-order tensor in FP64.
    """
    s = strength
    vpf, vps = vp * (1 + s / 2), vp * (1 - s / 2)
    vsf, vss = vs * (1 + s / 2), vs * (1 - s / 2)
    C = np.zeros((6, 6))
    C[0, 0] = rho * vpf ** 2                   # along the axis (local x1)
    C[1, 1] = C[2, 2] = rho * vps ** 2
    C[4, 4] = C[5, 5] = rho * vsf ** 2         # shear polarised along the axis
    C[3, 3] = rho * vss ** 2                   # shear in the isotropy plane
    C[1, 2] = C[2, 1] = C[1, 1] - 2 * C[3, 3]
    c13 = math.sqrt((C[0, 0] - C[4, 4]) * (C[1, 1] - C[4, 4])) - C[4, 4]
    C[0, 1] = C[1, 0] = C[0, 2] = C[2, 0] = c13
    az, tl = math.radians(azimuth_deg), math.radians(tilt_deg)
    a = np.array([math.cos(tl) * math.cos(az), math.cos(tl) * math.sin(az), math.sin(tl)])
    b = np.array([-math.sin(az), math.cos(az), 0.0])
    c = np.cross(a, b)
    R = np.stack([a, b, c], axis=1)           # local -> global
    cl = _voigt_to_tensor(C)
    cg = np.einsum("ip,jq,kr,ls,pqrs->ijkl", R, R, R, R, cl)
    return _tensor_to_voigt(cg)


@dataclass
class SemLayer:
    """One SEM-model layer: material up to a flat top at ``top`` km above the box bottom."""
    top: float
    C: np.ndarray
    rho: float


@dataclass
class Case:
    nex: int
    nez: int
    eh: float                      # requested element size (km)
    sdt: float                     # SEM time step (s)
    nst: int                       # SEM steps
    layers: list                   # SemLayer, bottom to top
    p: float = 0.045               # ray parameter (s/km)
    f0: float = 0.2                # Ricker dominant frequency (Hz)
    sv_amp: float = 1.0
    sh_amp: float = 0.0
    hpn: int = 4
    neh: int = 1
    absorb: int = 1
    ntrace: int = 11
    rec_x0: float = 0.0
    rec_dx: float = 4.0
    dp: float | None = None        # GRT record step (default sdt)
    nt: int | None = None          # GRT records in the file (default nst + 3)
    readpars: int = 1
    get_rec: int = 1
    semmodel_full: bool = False
    psv_only: bool = False
    flat: int = 1
    write_records: bool = True     # False: no greenfile/shgreenfile (records generated on the device)
    record_t0: int = 0             # the file's record 0 is the plane wave's record record_t0 (pulse earlier)
    extra: dict = field(default_factory=dict)

    @property
    def thickness(self) -> float:
        return self.nez * self.eh + 0.002


def _fmt(v: float) -> str:
    return repr(float(v))


def write_case(case: Case, d: str, absolute: bool = False) -> dict:
    """Write the input files of ``case`` into directory ``d``; returns a summary.
    absolute: the par file names its inputs by absolute path (readable from
    any working directory)."""
    os.makedirs(d, exist_ok=True)
    N = case.hpn
    H = case.thickness
    # ray model: two layers inside the SEM box (crust-like top 10% and the rest)
    # plus the half-space; nrec = 3 via the first ray's layer list.
    top = case.layers[-1]
    bot = case.layers[0]
    vp_b = math.sqrt(bot.C[0, 0] / bot.rho)
    vs_b = math.sqrt(bot.C[3, 3] / bot.rho)
    vp_t = math.sqrt(top.C[0, 0] / top.rho)
    vs_t = math.sqrt(top.C[3, 3] / top.rho)
    t0 = round(0.1 * H, 3)
    with open(os.path.join(d, "raymodel"), "w") as f:
        f.write("3 2\n")
        f.write(f"{vp_t:.6f} {vs_t:.6f} {top.rho:.6f} {t0:.3f}\n")
        f.write(f"{vp_b:.6f} {vs_b:.6f} {bot.rho:.6f} {H - t0:.3f}\n")
        f.write(f"{vp_b:.6f} {vs_b:.6f} {bot.rho:.6f} 0.000\n")
        f.write("1\n3 3 3 3\n1 1 1 1\n")
    # SEM model: flat interfaces spanning the box
    xmax = case.nex * case.eh * 1.001 + 10.0
    with open(os.path.join(d, "semmodel"), "w") as f:
        f.write(f"{len(case.layers)}\n")
        for L in case.layers:
            C = L.C
            if case.semmodel_full:
                vals = [C[i, j] for i in range(6) for j in range(i, 6)] + [L.rho]
            else:
                vals = [C[0, 0], C[0, 1], C[0, 2], C[0, 5], C[1, 1], C[1, 2], C[1, 5],
                        C[2, 2], C[2, 5], C[3, 3], C[3, 4], C[4, 4], C[5, 5], L.rho]
            f.write("2 " + " ".join(_fmt(v) for v in vals) + "\n")
            f.write(f"-10.0 {xmax:.3f}\n")
            f.write(f"{L.top:.4f} {L.top:.4f}\n")
    # receivers at the surface
    with open(os.path.join(d, "rec_file"), "w") as f:
        f.write(f"{case.ntrace}\n")
        f.write(" ".join(f"{case.rec_x0 + i * case.rec_dx:.4f}" for i in range(case.ntrace)) + "\n")
    # boundary traces: upgoing plane wave in the bottom layer
    dp = case.dp if case.dp is not None else case.sdt
    nt = case.nt if case.nt is not None else case.nst + 3
    eh_eff = (np.float32(H) - 1e-3) / case.nez          # as the solver re-derives it
    h = float(eh_eff) / N
    nx, nz = case.nex * N + 1, case.nez * N + 1
    nbl = case.neh * N
    if case.write_records:
        write_plane_wave(os.path.join(d, "greenfile"), os.path.join(d, "shgreenfile"),
                         nx=nx, nz=nz, h=h, nbl=nbl, vs=vs_b, p=case.p, f0=case.f0,
                         dp=dp, nt=nt, sv_amp=case.sv_amp, sh_amp=case.sh_amp, eh=float(eh_eff), deg=N,
                         r_first=case.record_t0)
    name = (lambda f: os.path.join(os.path.abspath(d), f)) if absolute else (lambda f: f)
    par = {
        "greenfile": name("greenfile"), "shgreenfile": name("shgreenfile"), "raymodel": name("raymodel"),
        "semmodel": name("semmodel"), "nt": nt, "dp": _fmt(dp), "nex": case.nex, "eh": _fmt(case.eh),
        "xmin": "0.0", "nst": case.nst, "sdt": _fmt(case.sdt), "hpn": N, "neh": case.neh,
        "absorb": case.absorb, "readpars": case.readpars, "xbeg": "0.0", "idxplot": 8,
        "xtrace": case.ntrace, "get_rec": case.get_rec, "rec_file": name("rec_file"), "plot_trace": 1,
        "msource": 0, "check": 0, "flat": case.flat, "nfil": 1,
    }
    if case.semmodel_full:
        par["semmodel_full"] = 1
    if case.psv_only:
        par["psv_only"] = 1
    par.update(case.extra)
    with open(os.path.join(d, "run.par"), "w") as f:
        for k, v in par.items():
            f.write(f"{k}={v}\n")
    return {"nx": nx, "nz": nz, "h": h, "nt": nt, "dp": dp, "vs": vs_b}


def ricker(t: np.ndarray, f0: float) -> np.ndarray:
    a = (math.pi * f0 * t) ** 2
    return (1.0 - 2.0 * a) * np.exp(-a)


GLL3 = (-1.0, -0.4472135954999579, 0.4472135954999579, 1.0)         # GLL points of degree 3: +-1/sqrt(5)
GLL4 = (-1.0, -0.6546536707079771, 0.0, 0.6546536707079771, 1.0)    # GLL points of degree 4
GLL5 = (-1.0, -0.7650553239294647, -0.2852315164806451, 0.2852315164806451, 0.7650553239294647, 1.0)
# degree 6: 0 and +-sqrt((15 -+ 2 sqrt(15))/33)
GLL6 = (-1.0, -0.8302238962785669, -0.46884879347071423, 0.0, 0.46884879347071423, 0.8302238962785669, 1.0)
GLL_POINTS = {3: GLL3, 4: GLL4, 5: GLL5, 6: GLL6}


def gll_positions(n: int, eh: float, deg: int = 4) -> np.ndarray:
    """Coordinates of grid points 0..n-1 along a row or column of degree-deg
    elements of size eh: point deg*e+m at e*eh + (xi_m + 1)*eh/2, the node
    positions the reference's boundary-trace generator uses
    (semsyn/src/aserpsv_sem.c:887-920, Grid_Point)."""
    if deg in GLL_POINTS:
        xi = np.array(GLL_POINTS[deg])
    else:                                        # +-1 and the roots of P_deg'
        inner = np.sort(np.polynomial.legendre.Legendre.basis(deg).deriv().roots().real)
        xi = np.concatenate([[-1.0], inner, [1.0]])
    e, m = np.divmod(np.arange(n), deg)
    return e * eh + (xi[m] + 1.0) * eh / 2.0


def plane_wave_records(nx, nz, h, nbl, vs, p, f0, dp, r0, r1, sv_amp=1.0, sh_amp=0.0, eh=None, deg=4):
    """Records r0..r1-1 of the boundary traces (float32, time-major), the
    plane wave timed at the GLL node positions of the line (eh: the element
    size, deg*h when not given; deg: the GLL degree)."""
    eh = deg * h if eh is None else eh
    eta = math.sqrt(max(1.0 / vs ** 2 - p ** 2, 0.0))
    delay = 1.5 / f0
    xb = gll_positions(nx, eh, deg)            # bottom line, at the height of row nbl
    zl = gll_positions(nz, eh, deg)            # left column, at the position of column nbl
    line = gll_positions(nbl + 1, eh, deg)[nbl]
    tau_b = p * xb + eta * line
    tau_l = p * line + eta * zl
    t = (np.arange(r0, r1) * dp)[:, None]
    rb = ricker(t - delay - tau_b[None, :], f0)
    rl = ricker(t - delay - tau_l[None, :], f0)
    ux, uz = sv_amp * eta * vs, -sv_amp * p * vs   # SV polarisation, z up
    psv = np.concatenate([ux * rb, -uz * rb, ux * rl, -uz * rl], axis=1).astype(np.float32)
    sh = np.concatenate([sh_amp * rb, sh_amp * rl], axis=1).astype(np.float32)
    return psv, sh


def write_plane_wave(psv_path, sh_path, *, nx, nz, h, nbl, vs, p, f0, dp, nt,
                     sv_amp=1.0, sh_amp=0.0, chunk=1024, eh=None, deg=4, r_first=0):
    """Records r_first .. r_first+nt-1 of the plane wave as the files' records 0 .. nt-1."""
    with open(psv_path, "wb") as fp, open(sh_path, "wb") as fs:
        for r0 in range(r_first, r_first + nt, chunk):
            psv, sh = plane_wave_records(nx, nz, h, nbl, vs, p, f0, dp, r0, min(r_first + nt, r0 + chunk),
                                         sv_amp, sh_amp, eh, deg)
            fp.write(psv.tobytes())
            fs.write(sh.tobytes())


# ---------------------------------------------------------------------------
# the benchmark configurations, restated with their sizes
# ---------------------------------------------------------------------------
CRUST = dict(vp=6.4, vs=3.6, rho=2.8)
MANTLE = dict(vp=8.1, vs=4.5, rho=3.4)


def layered_two(H: float, crust_km: float = 35.0):
    return [SemLayer(H - crust_km, iso_cij(**MANTLE), MANTLE["rho"]),
            SemLayer(H + 1.0, iso_cij(**CRUST), CRUST["rho"])]


def layered_aniso(H: float, crust_km=35.0, aniso_km=100.0, strength=0.04, az=45.0, tilt=20.0):
    m = MANTLE
    return [SemLayer(H - crust_km - aniso_km, iso_cij(**m), m["rho"]),
            SemLayer(H - crust_km, hexagonal_cij(m["vp"], m["vs"], m["rho"], strength, az, tilt), m["rho"]),
            SemLayer(H + 1.0, iso_cij(**CRUST), CRUST["rho"])]


def config_isotropic_psv(nst=6000) -> Case:
    """The plain isotropic P-SV case: 400x200 km, 200x100 elements of 2 km, GLL
    degree 4, a 35 km crust over the mantle, SV plane wave p=0.045 s/km, Ricker
    0.2 Hz, dt 10 ms, 101 receivers every 4 km, Stacey on the sides and bottom;
    P-SV only (the reference's `sem2d` program: no SH record file)."""
    H = 200.0
    return Case(nex=200, nez=100, eh=2.0, sdt=0.01, nst=nst, layers=layered_two(H),
                p=0.045, f0=0.2, ntrace=101, rec_x0=0.0, rec_dx=4.0, psv_only=True)


def config_aniso_3c(nst=24000) -> Case:
    """800x300 km, 800x300 elements of 1 km, 100 km hexagonal layer (4%, az 45, tilt 20)."""
    H = 300.0
    return Case(nex=800, nez=300, eh=1.0, sdt=0.005, nst=nst, layers=layered_aniso(H),
                p=0.042, f0=0.5, ntrace=201, rec_x0=0.0, rec_dx=4.0, semmodel_full=True)


def config_large(nst=40000) -> Case:
    """1000x250 km, 4000x1000 elements of 250 m, anisotropic layer as above, 2 Hz."""
    H = 250.0
    return Case(nex=4000, nez=1000, eh=0.25, sdt=0.0015, nst=nst, layers=layered_aniso(H),
                p=0.045, f0=2.0, ntrace=1001, rec_x0=0.0, rec_dx=1.0, semmodel_full=True)


GLL4_MIN_SPACING = (1.0 - math.sqrt(3.0 / 7.0)) / 2.0   # smallest GLL gap of degree 4, in element sizes


def vp_max(layers) -> float:
    """Largest diagonal P velocity sqrt(C_ii / rho) over the layers (i = 1..3)."""
    return max(math.sqrt(max(L.C[0, 0], L.C[1, 1], L.C[2, 2]) / L.rho) for L in layers)


def stable_dt(eh: float, layers, courant: float = 0.4) -> float:
    """dt = courant * h_min / vp_max, h_min the smallest GLL spacing of an element of size eh."""
    return courant * GLL4_MIN_SPACING * eh / vp_max(layers)


def layered_aniso_box(H: float, strength: float, az: float, tilt: float, crust_km=35.0, aniso_km=100.0):
    """Crust over a hexagonal layer over the mantle, for a box of height H;
    layers that would lie below the box bottom are left out."""
    out = [L for L in layered_aniso(H, crust_km, aniso_km, strength, az, tilt) if L.top > 0.0]
    return out


def draw_instance(rng: np.random.Generator, nex: int, nez: int, eh: float, seconds: float = 60.0,
                  ntrace: int = 101) -> dict:
    """One SKS solve with the draws of the batched and served workloads: ray
    parameter U[0.038, 0.052] s/km, anisotropy U[0, 6] %, fast-axis azimuth
    U[0, 180) deg, tilt U[0, 30) deg, Ricker U[0.2, 0.5] Hz; dt = 0.4 h_min /
    vp_max and `seconds` of simulated time."""
    p = float(rng.uniform(0.038, 0.052))
    strength = float(rng.uniform(0.0, 0.06))
    az = float(rng.uniform(0.0, 180.0))
    tilt = float(rng.uniform(0.0, 30.0))
    f0 = float(rng.uniform(0.2, 0.5))
    H = nez * eh
    layers = layered_aniso_box(H, strength, az, tilt)
    dt = stable_dt(eh, layers)
    nst = int(math.ceil(seconds / dt))
    width = nex * eh
    dx = width * 0.9 / max(1, ntrace - 1)
    case = Case(nex=nex, nez=nez, eh=eh, sdt=dt, nst=nst, layers=layers, p=p, f0=f0, sv_amp=1.0, sh_amp=0.0,
                ntrace=ntrace, rec_x0=0.05 * width, rec_dx=dx, semmodel_full=True, write_records=False)
    return {"case": case, "p": p, "strength": strength, "az": az, "tilt": tilt, "f0": f0, "dt": dt, "nst": nst,
            "vs_bottom": math.sqrt(layers[0].C[3, 3] / layers[0].rho)}


def config_batch(n: int = 64, seed: int = 20240601, seconds: float = 60.0) -> list:
    """The batched workload: n instances, nex U{200..1000}, nez U{100..400},
    element size U[1, 2] km, the physics draws of draw_instance."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nex = int(rng.integers(200, 1001))
        nez = int(rng.integers(100, 401))
        eh = float(rng.uniform(1.0, 2.0))
        out.append(draw_instance(rng, nex, nez, eh, seconds))
    return out


def draw_served_size(rng: np.random.Generator) -> tuple:
    """Served request mesh: lognormal element counts with median 400 x 200,
    clipped to 100 x 50 .. 2000 x 600 (one shared log-normal factor keeps the
    aspect near 2:1, plus a small independent spread)."""
    g = rng.normal(0.0, 0.6)
    nex = int(np.clip(round(400 * math.exp(g + rng.normal(0.0, 0.15))), 100, 2000))
    nez = int(np.clip(round(200 * math.exp(g + rng.normal(0.0, 0.15))), 50, 600))
    return nex, nez
