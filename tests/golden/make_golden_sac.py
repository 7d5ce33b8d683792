"""Golden files of the reference's seismogram converter (semsyn/plot/uvw2sac.c).

Runs oracle/_ref/uvw2sac -- the reference program compiled from its own
sources by `make -C oracle ref` (restated sachead.h, a declaration of
open_file, stand-ins for the Fortran source routines it calls only with
Conv_Source=1) -- on seeded seismograms of a small mesh, with receivers from
the par words (get_rec=0) and from a receiver file (get_rec=1), and stores
the inputs and every file it writes in tests/golden/uvw2sac.npz.

    python tests/golden/make_golden_sac.py     # needs oracle/_ref/uvw2sac
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "s-sks_gb300")]
import synth  # noqa: E402

WORDS = ["par=run.par", "zbeg=0", "idzplot=1", "zs=12.5", "Conv_Source=0", "tstart=3.5", "xmin=100.0", "xbeg=3.0"]
INPUTS = ("run.par", "raymodel", "rec_file", "seis.u", "seis.v", "seis.w")


def write_inputs(d: str) -> None:
    """The case's par file, ray model and receiver file, and seeded seismograms."""
    c = synth.Case(nex=20, nez=8, eh=2.0, sdt=0.01, nst=101, layers=synth.layered_two(16.0, 5.0), p=0.04, f0=1.0,
                   ntrace=6, rec_dx=4.0, write_records=False)
    synth.write_case(c, d)
    rng = np.random.default_rng(4)
    for name in ("seis.u", "seis.v", "seis.w"):
        rng.normal(size=(c.nst, c.ntrace)).astype(np.float32).tofile(os.path.join(d, name))


def main() -> None:
    prog = os.path.join(ROOT, "oracle", "_ref", "uvw2sac")
    out = {}
    for get_rec in (0, 1):
        with tempfile.TemporaryDirectory() as d:
            write_inputs(d)
            before = set(os.listdir(d))
            if get_rec == 0:
                for f in INPUTS:
                    out[f"in/{f}"] = np.frombuffer(open(os.path.join(d, f), "rb").read(), np.uint8)
            r = subprocess.run([prog] + WORDS + [f"get_rec={get_rec}"], cwd=d, capture_output=True, text=True)
            if r.returncode != 0:
                raise SystemExit(f"uvw2sac failed: {r.stderr}")
            for f in sorted(set(os.listdir(d)) - before):
                out[f"get_rec{get_rec}/{f}"] = np.frombuffer(open(os.path.join(d, f), "rb").read(), np.uint8)
    np.savez_compressed(os.path.join(HERE, "uvw2sac.npz"), **out)
    print("wrote", len(out), "files")


if __name__ == "__main__":
    main()
