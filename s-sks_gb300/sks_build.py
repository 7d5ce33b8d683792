"""Build recipe of the library (no cmake): nvcc for the CUDA sources with one
-gencode for sm_103a, gcc for the host C, everything in s-sks_gb300/_build/.

    python s-sks_gb300/sks_build.py        # library + drop-in CLI
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
INC = os.path.join(ROOT, "include")
LIB = os.path.join(OUT, "libsks_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(INC, "sks.h")] + [os.path.join(CSRC, h) for h in (
        "sks_model.h", "sks_internal.h", "sks_kernels.cuh", "sks_aux_kernels.cuh", "sks_variants.cuh",
        "sks_step_inst.cuh", "sks_batch_inst.cuh")]
    units = [
        (os.path.join(CSRC, c + ".c"), os.path.join(OUT, c + ".o"),
         ["gcc", "-O2", "-std=gnu11", "-fPIC", "-Wall", "-I" + INC, "-c"]) for c in ("sks_model", "sks_elastic",
                                                                                    "sks_sac", "sks_layered")
    ]
    for cu in ("sks_solver", "sks_batch", "sks_server", "sks_step_f32", "sks_step_f64", "sks_batch_f32", "sks_batch_f64",
               "sks_step_f32_tp", "sks_step_f64_tp", "sks_batch_f32_tp", "sks_batch_f64_tp",
               "sks_step_f32_d5", "sks_step_f64_d5", "sks_batch_f32_d5", "sks_batch_f64_d5",
               "sks_step_f32_d3", "sks_step_f64_d3", "sks_step_f32_d6", "sks_step_f64_d6",
               "sks_batch_f32_d3", "sks_batch_f64_d3", "sks_batch_f32_d6", "sks_batch_f64_d6",
               "sks_noalloc", "sks_post", "sks_probe"):
        units.append((os.path.join(CSRC, cu + ".cu"), os.path.join(OUT, cu + ".o"),
                      [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INC, "-I" + CSRC,
                       "-c"]))
    jobs = []
    for src, obj, cmd in units:
        if _stale(obj, [src] + hdrs):
            jobs.append(cmd + [src, "-o", obj])
    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    objs = [u[1] for u in units]
    if _stale(LIB, objs):
        _run([nvcc, ARCH, "-shared", "-o", LIB] + objs + ["-lcudart_static", "-ldl", "-lpthread", "-lrt"])
    cli = os.path.join(OUT, "sem2d_psvsh_gb300")
    main_c = os.path.join(CSRC, "sem2d_psvsh_main.c")
    if _stale(cli, [main_c, LIB]):
        _run(["gcc", "-O2", "-std=gnu11", "-I" + INC, "-o", cli, main_c, "-L" + OUT, "-lsks_gb300",
              "-Wl,-rpath,$ORIGIN"])
        link = os.path.join(OUT, "sem2d_gb300")
        if os.path.lexists(link):
            os.remove(link)
        os.symlink("sem2d_psvsh_gb300", link)
    conv = os.path.join(OUT, "uvw2sac_gb300")
    conv_c = os.path.join(CSRC, "uvw2sac_main.c")
    if _stale(conv, [conv_c, LIB]):
        _run(["gcc", "-O2", "-std=gnu11", "-I" + INC, "-o", conv, conv_c, "-L" + OUT, "-lsks_gb300",
              "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
