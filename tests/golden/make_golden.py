"""Generate the golden fixtures in this directory from the REFERENCE solver.

Each fixture <case>.npz holds the input files of one small run (run.par,
raymodel, semmodel, greenfile, shgreenfile, rec_file) and the seis.u / seis.v /
seis.w the reference binaries wrote for them.  The binaries are compiled from
the reference sources by `make -C oracle ref` (oracle/_ref/sem2d_psvsh and
oracle/_ref/sem2d, the P-SV-only program).  Inputs are stored, not
regenerated, so the fixtures do not depend on numpy's math library.

    python tests/golden/make_golden.py        # needs oracle/_ref built here
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "s-sks_gb300"))
import synth  # noqa: E402

REFBIN = os.path.join(ROOT, "oracle", "_ref")
FILES = ["run.par", "raymodel", "semmodel", "greenfile", "shgreenfile", "rec_file"]


def aniso_layers(H, az=30.0, tilt=0.0, s=0.06):
    return [synth.SemLayer(H - 6, synth.iso_cij(8.1, 4.5, 3.4), 3.4),
            synth.SemLayer(H - 3, synth.hexagonal_cij(8.1, 4.5, 3.4, s, az, tilt), 3.4),
            synth.SemLayer(H + 1, synth.iso_cij(6.4, 3.6, 2.8), 2.8)]


def ratio_semmodel(path, H):
    """A SEM model with a layer of multiplying coefficients (negative control-
    point count, sem2d_psvsh.c:730-733,758-763) and a sloping interface."""
    iso = synth.iso_cij(8.1, 4.5, 3.4)
    cr = synth.iso_cij(6.4, 3.6, 2.8)
    v = lambda C, rho: [C[0, 0], C[0, 1], C[0, 2], C[0, 5], C[1, 1], C[1, 2], C[1, 5],
                        C[2, 2], C[2, 5], C[3, 3], C[3, 4], C[4, 4], C[5, 5], rho]
    with open(path, "w") as f:
        f.write("3\n")
        f.write("2 " + " ".join(repr(float(x)) for x in v(iso, 3.4)) + "\n-10.0 200.0\n8.0 11.0\n")
        f.write("-2 " + " ".join(repr(float(x)) for x in [1.05, 1.0, 1.0, 0.0, 1.05, 1.0, 0.0, 1.02, 0.0, 0.97,
                                                              0.0, 0.97, 0.95, 1.01]) + "\n-10.0 200.0\n12.0 12.0\n")
        f.write("3 " + " ".join(repr(float(x)) for x in v(cr, 2.8)) + f"\n-10.0 60.0 200.0\n{H + 1:.3f} {H + 1:.3f} {H + 1:.3f}\n")


CASES = {
    # anisotropic layer through the reference's 13-constant SEM model, P-SV + SH
    "psvsh_aniso13": dict(prog="sem2d_psvsh", case=lambda: synth.Case(
        nex=14, nez=9, eh=2.0, sdt=0.01, nst=720, layers=aniso_layers(18.0), p=0.05, f0=1.0,
        sv_amp=1.0, sh_amp=0.5, ntrace=7, rec_x0=1.0, rec_dx=4.0)),
    # GRT step twice the SEM step, injection ends before the run does,
    # receivers from xbeg/idxplot (the first one wraps to the row below)
    "psvsh_rdt_half": dict(prog="sem2d_psvsh", case=lambda: synth.Case(
        nex=12, nez=8, eh=2.0, sdt=0.005, dp=0.01, nt=260, nst=1200, layers=aniso_layers(16.0, 60.0),
        p=0.045, f0=1.0, sv_amp=1.0, sh_amp=0.8, ntrace=5, get_rec=0,
        extra={"xbeg": "0.0", "idxplot": 11})),
    # the P-SV-only program sem2d (no SH file)
    "psv_sem2d": dict(prog="sem2d", case=lambda: synth.Case(
        nex=14, nez=9, eh=2.0, sdt=0.01, nst=720, layers=aniso_layers(18.0, 45.0), p=0.05, f0=1.0,
        ntrace=7, rec_x0=2.0, rec_dx=4.0)),
    # 1-D ray model only (readpars=0) with Earth flattening
    "flat0_raymodel": dict(prog="sem2d_psvsh", case=lambda: synth.Case(
        nex=14, nez=8, eh=2.0, sdt=0.01, nst=640, layers=synth.layered_two(16.0, 5.0), p=0.04,
        f0=1.0, flat=0, readpars=0, sh_amp=0.4, ntrace=6, rec_dx=4.5)),
    # SEM model with a coefficient layer and a sloping interface
    "ratio_layers": dict(prog="sem2d_psvsh", semmodel=ratio_semmodel, case=lambda: synth.Case(
        nex=14, nez=8, eh=2.0, sdt=0.01, nst=640, layers=synth.layered_two(16.0, 5.0), p=0.05,
        f0=1.0, sh_amp=0.3, ntrace=8, rec_dx=3.3)),
    # boundary taper in all four zones (atten=4, ass=0.9), two elements wide (neh=2)
    "psvsh_atten": dict(prog="sem2d_psvsh", case=lambda: synth.Case(
        nex=14, nez=9, eh=2.0, sdt=0.01, nst=720, layers=aniso_layers(18.0, 40.0), p=0.05, f0=1.0,
        sv_amp=3.0, sh_amp=1.5, neh=2, ntrace=7, rec_x0=1.0, rec_dx=4.0, extra={"atten": 4, "ass": "0.9"})),
    # GLL degree 5, the reference's default hpn (records at the degree-5 node positions)
    "psvsh_hpn5": dict(prog="sem2d_psvsh", case=lambda: synth.Case(
        nex=12, nez=7, eh=2.5, sdt=0.01, nst=640, layers=aniso_layers(17.5, 50.0), p=0.05, f0=1.0,
        sv_amp=1.0, sh_amp=0.6, hpn=5, ntrace=7, rec_x0=1.0, rec_dx=4.0)),
    # GLL degrees 3 and 6, the ends of the range the reference accepts (lagrange.c:323-328)
    "psvsh_hpn3": dict(prog="sem2d_psvsh", case=lambda: synth.Case(
        nex=16, nez=9, eh=2.0, sdt=0.01, nst=700, layers=aniso_layers(18.0, 35.0), p=0.05, f0=1.0,
        sv_amp=1.0, sh_amp=0.6, hpn=3, ntrace=7, rec_x0=1.0, rec_dx=4.0)),
    "psvsh_hpn6": dict(prog="sem2d_psvsh", case=lambda: synth.Case(
        nex=10, nez=6, eh=3.0, sdt=0.008, nst=800, layers=aniso_layers(18.0, 55.0), p=0.05, f0=1.0,
        sv_amp=1.0, sh_amp=0.6, hpn=6, ntrace=7, rec_x0=1.0, rec_dx=4.0)),
    # snapshots (plot_snap): the reference's text files out1..outK
    "psvsh_snap": dict(prog="sem2d_psvsh", words=["plot_snap=1", "startsnap=40", "incresnap=60"],
                       case=lambda: synth.Case(
        nex=14, nez=9, eh=2.0, sdt=0.01, nst=720, layers=aniso_layers(18.0, 20.0), p=0.05, f0=1.0,
        sv_amp=1.0, sh_amp=0.5, ntrace=7, rec_x0=1.0, rec_dx=4.0)),
}


def quantize_traces(d):
    """Round the boundary traces to multiples of 2^-12 so the stored fixture
    compresses; the reference then runs on exactly these values."""
    for fn in ("greenfile", "shgreenfile"):
        p = os.path.join(d, fn)
        a = np.fromfile(p, np.float32)
        np.round(a.astype(np.float64) * 4096.0).astype(np.float32).__truediv__(np.float32(4096.0)).astype(np.float32).tofile(p)


def make(name, spec):
    with tempfile.TemporaryDirectory() as d:
        c = spec["case"]()
        synth.write_case(c, d)
        if "semmodel" in spec:
            spec["semmodel"](os.path.join(d, "semmodel"), c.thickness)
        quantize_traces(d)
        r = subprocess.run([os.path.join(REFBIN, spec["prog"]), "par=run.par"] + spec.get("words", []), cwd=d,
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{name}: reference failed\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        out = {}
        for fn in FILES:
            with open(os.path.join(d, fn), "rb") as f:
                out["in_" + fn.replace(".", "_")] = np.frombuffer(f.read(), np.uint8)
        for x in "uvw":
            out["seis_" + x] = np.fromfile(os.path.join(d, "seis." + x), np.float32)
        out["ntrace"] = np.array(c.ntrace)
        out["nst"] = np.array(c.nst)
        out["prog"] = np.array(spec["prog"])
        out["words"] = np.array(" ".join(spec.get("words", [])))
        k = 1
        while os.path.exists(os.path.join(d, f"out{k}")):
            with open(os.path.join(d, f"out{k}"), "rb") as f:
                out[f"snap_out{k}"] = np.frombuffer(f.read(), np.uint8)
            k += 1
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, {k: v.shape for k, v in out.items() if k.startswith("seis")})


def extract(npz_path, d):
    """Write the input files of a fixture into directory d; returns the npz."""
    z = np.load(npz_path)
    for fn in FILES:
        with open(os.path.join(d, fn), "wb") as f:
            f.write(z["in_" + fn.replace(".", "_")].tobytes())
    return z


if __name__ == "__main__":
    if not os.path.exists(os.path.join(REFBIN, "sem2d_psvsh")):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    for n, s in CASES.items():
        if len(sys.argv) > 1 and n not in sys.argv[1:]:
            continue
        make(n, s)
