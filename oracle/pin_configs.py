"""Pin the oracle's float build to the reference binaries at the benchmark
configurations' own sizes (test infrastructure).

The golden fixtures pin the oracle on small meshes; this script repeats the
check on the two workloads the GPU parity tests compare with the FP64 oracle
at full size, so the chain GPU -> oracle -> reference holds there too:

  c0  the plain isotropic P-SV case, whole: 200 x 100 elements of 2 km
      (801 x 401 = 321,201 points), 6000 steps, 101 receivers, run by the
      reference's P-SV-only program sem2d;
  c1  the anisotropic 3-component mesh: 800 x 300 elements of 1 km
      (3201 x 1201 = 3,844,401 points), its SEM model written as the
      reference's 13 constants per layer (the reference reads no more), over
      a window of 240 steps whose boundary records start 2 s into the plane
      wave, with snapshots (plot_snap) at steps 120 and 239, so the displacement
      field of every second point is compared as well as the seismograms.

c0_short and c1_short are the same meshes over 300 and 8 steps with
snapshots inside the window.  `--record` writes each case's input and
output digests to tests/golden/config_pins.json; the CPU tests compare the
float oracle with the short cases' digests (tests/test_oracle_pin_configs.py),
and the long cases' digests are kept there as the record of those runs.

Each program runs on the same input files in a directory of its own, both at
once; seis.u / seis.v / seis.w and the snapshot files out1.. must be equal
byte for byte.  The reference binaries are built by `make -C oracle ref` from
the reference's sources; this takes minutes of CPU (c0: about 15 min for the
reference at -O2, c1: a few minutes).

    python oracle/pin_configs.py [c0] [c1] [c0_short] [c1_short] [--record]
"""
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [os.path.join(ROOT, "s-sks_gb300"), ROOT]

import synth  # noqa: E402

REFBIN = os.path.join(HERE, "_ref")
ORACLE = os.path.join(HERE, "_build", "oracle_sem2d_psvsh32")
INPUTS = ["run.par", "raymodel", "semmodel", "greenfile", "shgreenfile", "rec_file"]


def _c0():
    return synth.config_isotropic_psv(), "sem2d", ["psv_only=1"], []


def _c1():
    c = synth.config_aniso_3c(nst=240)
    c.record_t0 = 400            # 2 s of the plane wave at 5 ms
    c.semmodel_full = False      # the reference's 13 constants per layer
    snap = ["plot_snap=1", "startsnap=120", "incresnap=119"]
    return c, "sem2d_psvsh", [], snap


def _c0_short():
    c = synth.config_isotropic_psv(nst=300)
    return c, "sem2d", ["psv_only=1"], ["plot_snap=1", "startsnap=150", "incresnap=149"]


def _c1_short():
    c, prog, ow, _ = _c1()
    c.nst = 8
    return c, prog, ow, ["plot_snap=1", "startsnap=3", "incresnap=4"]


CASES = {"c0": _c0, "c1": _c1,
         # the same meshes over short windows, whose snapshots the CPU tests
         # compare with the reference's (tests/golden/config_pins.json)
         "c0_short": _c0_short, "c1_short": _c1_short}


def _sha(path):
    h = hashlib.sha256()
    with open(path, "rb") as f:
        for b in iter(lambda: f.read(1 << 20), b""):
            h.update(b)
    return h.hexdigest()


def pin(name):
    case, prog, oracle_words, words = CASES[name]()
    base = tempfile.mkdtemp(prefix=f"sks_pin_{name}_")
    try:
        dirs = {k: os.path.join(base, k) for k in ("reference", "oracle")}
        synth.write_case(case, dirs["reference"])
        shutil.copytree(dirs["reference"], dirs["oracle"])
        cmds = {"reference": [os.path.join(REFBIN, prog), "par=run.par"] + words,
                "oracle": [ORACLE, "par=run.par"] + oracle_words + words}
        t0 = time.perf_counter()
        logs = {k: open(os.path.join(base, k + ".log"), "w+b") for k in cmds}
        procs = {k: subprocess.Popen(cmds[k], cwd=dirs[k], stdout=subprocess.DEVNULL, stderr=logs[k]) for k in cmds}
        secs = {}
        while len(secs) < len(procs):           # each program's own wall time
            for k, p in procs.items():
                if k not in secs and p.poll() is not None:
                    secs[k] = round(time.perf_counter() - t0, 1)
            time.sleep(0.5)
        for k, p in procs.items():
            logs[k].seek(0)
            err = logs[k].read().decode(errors="replace")
            logs[k].close()
            if p.returncode:
                raise RuntimeError(f"{name}: {k} exit {p.returncode}: {err[-500:]}")
        outs = ["seis.u", "seis.v", "seis.w"]
        k = 1
        while os.path.exists(os.path.join(dirs["reference"], f"out{k}")):
            outs.append(f"out{k}")
            k += 1
        result = {"case": name, "program": prog, "steps": case.nst,
                  "points": (case.nex * case.hpn + 1) * (case.nez * case.hpn + 1),
                  "inputs_sha256": {f: _sha(os.path.join(dirs["reference"], f)) for f in INPUTS
                                    if os.path.exists(os.path.join(dirs["reference"], f))},
                  "wall_s": secs, "files": {}}
        same = True
        for f in outs:
            a, b = os.path.join(dirs["reference"], f), os.path.join(dirs["oracle"], f)
            ha = _sha(a)
            hb = _sha(b) if os.path.exists(b) else None
            result["files"][f] = {"bytes": os.path.getsize(a), "reference_sha256": ha, "identical": ha == hb}
            if f.startswith("seis."):      # how much signal the trace file carries
                result["files"][f]["max_abs"] = float(np.abs(np.fromfile(a, np.float32)).max(initial=0.0))
            same = same and ha == hb
        result["bit_exact"] = same
        return result
    finally:
        shutil.rmtree(base, ignore_errors=True)


RECORD = os.path.join(ROOT, "tests", "golden", "config_pins.json")


def main():
    record = "--record" in sys.argv[1:]
    names = [a for a in sys.argv[1:] if a != "--record"] or list(CASES)
    if not os.path.exists(ORACLE):
        subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if not os.path.exists(os.path.join(REFBIN, "sem2d_psvsh")):
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)
    ok = True
    rec = {}
    if record and os.path.exists(RECORD):
        with open(RECORD) as f:
            rec = json.load(f)
    for n in names:
        r = pin(n)
        print(json.dumps(r), flush=True)
        ok = ok and r["bit_exact"]
        if record:
            case, prog, oracle_words, words = CASES[n]()
            rec[n] = {"program": prog, "steps": case.nst, "points": r["points"], "words": oracle_words + words,
                      "inputs_sha256": r["inputs_sha256"],
                      "outputs_sha256": {f: v["reference_sha256"] for f, v in r["files"].items()}}
    if record:
        with open(RECORD, "w") as f:
            json.dump(rec, f, indent=1, sort_keys=True)
            f.write("\n")
    sys.exit(0 if ok else 1)


if __name__ == "__main__":
    main()
