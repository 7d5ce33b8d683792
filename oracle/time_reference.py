"""Per-step CPU time of the reference solver binaries (oracle/_ref, built by
`make -C oracle ref` from the reference's sources) beside the oracle's float
build (oracle/_build), on the anisotropic 3-component mesh of 800 x 300
elements (3,844,401 points) with its SEM model written as the reference's
13 constants per layer (the reference reads no more).  One process at a
time, one thread each; the time of a step is (T(6 steps) - T(2 steps)) / 4,
so set-up and file reading cancel.  Test infrastructure: it justifies which
CPU code the benchmark's CPU baseline times on a host where the reference
binaries cannot be built.

    python oracle/time_reference.py
"""
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [os.path.join(ROOT, "s-sks_gb300"), ROOT]

import synth  # noqa: E402

PROGRAMS = {
    "sem2dMP -O2 (the OpenMP variant; its pragmas are commented out)": os.path.join(HERE, "_ref", "sem2dMP"),
    "sem2d_psvsh -O2": os.path.join(HERE, "_ref", "sem2d_psvsh"),
    "sem2d_psvsh, the makefile's flags (no -O)": os.path.join(HERE, "_ref", "sem2d_psvsh_O0"),
    "oracle float build (bit-exact to the reference binary)": os.path.join(HERE, "_build", "oracle_sem2d_psvsh32"),
}


def main() -> None:
    d = tempfile.mkdtemp(prefix="sks_cpu_")
    c = synth.config_aniso_3c(nst=12)
    c.semmodel_full = False
    synth.write_case(c, d)
    npts = (c.nex * 4 + 1) * (c.nez * 4 + 1)
    for name, exe in PROGRAMS.items():
        if not os.path.exists(exe):
            print(f"{name}: not built ({exe})")
            continue
        t = {}
        for n in (2, 6):
            t0 = time.perf_counter()
            r = subprocess.run([exe, "par=run.par", f"nst={n}"], cwd=d, capture_output=True, text=True)
            t[n] = time.perf_counter() - t0
            if r.returncode:
                raise RuntimeError(f"{name}: exit {r.returncode}\n{r.stdout[-500:]}{r.stderr[-500:]}")
        per = (t[6] - t[2]) / 4
        print(f"{name}: {per * 1e3:.0f} ms per step, {npts / per / 1e6:.2f} M point-updates/s", flush=True)


if __name__ == "__main__":
    main()
