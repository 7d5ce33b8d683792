"""Benchmark of the SEM time step on one GB300 (and N replicas under torchrun).

Workload: the anisotropic 3-component SKS case -- an 800 x 300 km box of
800 x 300 elements of 1 km, GLL degree 4 (3201 x 1201 = 3,844,401 points), a
35 km crust over a 100 km layer of 4 % hexagonal anisotropy (fast axis at
azimuth 45 deg, tilt 20 deg: full c_ij) over the mantle, an SV plane wave with
ray parameter 0.042 s/km and a 0.5 Hz Ricker pulse, dt = 5 ms, 201 surface
receivers.  Inputs are synthetic (the generator in s-sks_gb300/synth.py).

A step is one SEM time step over the whole mesh.  `value` is GLL-point
updates per second of the FP32-compensated form, device resident, timed with
CUDA events on the solver's stream; `e2e` is the same metric through the C ABI
with host buffers (boundary records uploaded from pinned memory and the
seismograms read back inside the timed region).  The FP64 form is measured
the same way and reported beside it.  The per-step working set (~190 MB) is
larger than the 129 MB L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "s-sks_gb300")
for _p in (PKG, ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

NEX, NEZ = 800, 300
FULL_STEPS = 24000
# Algorithmic bytes per GLL-point update of the anisotropic 3-component step:
# W x (3 u^n read + 3 u^(n-1) read + 3 u^(n+1) write + 1 inverse mass + 15 c_ij)
# plus, for the compensated FP32 form, 4 B x 3 compensation words read and
# written: 124 B (FP32C), 200 B (FP64).  The kernels move less than that (the
# material is a 2-byte index into a table, read only on element rows of more
# than one material, and the inverse mass is rebuilt from GLL weights): 72 B
# per point in both forms on this mesh's one-material rows, 74 B on the few
# others (LAYOUT_BYTES_PER_POINT: the former).
BYTES_PER_POINT = {"fp32c": 124, "fp64": 200, "fp64_iso": 96}
# flops per grid-point update of the FP64 step as the kernel computes it (an
# FMA is 2 flops, an n-term dot product 2n-1): per element row a GLL column
# does, for each of its 5 rows, the x derivatives of 3 components with the
# strain sum u_z,x + u_x,z folded into one of them (28), their z derivatives
# in even-odd form (16.2: 27 per component for all 5 rows), the 5x5 stress
# (45), the x-divergence with the row weight in its table (27) and the
# even-odd z-divergence scaled into the rows (22.2): 138.4 x 5 = 692, an
# element's 5 columns 3460, over its 16 unique points 216.25; plus assembly
# (1.5) and the 3-level update (15).  (Direct 5-term sums: 276.)
# isotropic: the 5x5 stress is 9 flops instead of 45: 102.4 x 25 / 16 + 16.5
FLOPS_PER_POINT = {"aniso": 232.75, "iso": 176.5}
LAYOUT_BYTES_PER_POINT = {"fp32c": 72, "fp64": 72}
WORKLOAD = ("anisotropic 3-component SKS solve: 800x300 elements of 1 km, GLL degree 4, "
            "3,844,401 points, 100 km hexagonal layer (4 %, azimuth 45, tilt 20), dt 5 ms, 201 receivers")


def _peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_case(d: str, nst: int) -> None:
    import synth
    c = synth.config_aniso_3c(nst=nst)
    synth.write_case(c, d)


class Clocks:
    """nvidia-smi clock/throttle sampling while the timed region runs."""

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            self.proc.wait()

    def summary(self) -> dict:
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    smax.append(float(f[2]))
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        except OSError:
            pass
        finally:
            if self.path and os.path.exists(self.path):
                os.remove(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def _pinned(n: int):
    import torch
    return torch.empty(n, dtype=torch.float32, pin_memory=True)


def run_fixed(d: str, precision: int, steps: int, warmup: int, gpu: int, tuning) -> dict:
    """Only the device-resident step loop with a given tuning (for profilers)."""
    import sks
    cwd = os.getcwd()
    os.chdir(d)
    try:
        s = sks.Solver(["par=run.par"], precision=precision, device=gpu)
        s.load_boundary_files()
        if tuning:
            s.set_tuning(*tuning)
        lib_run_noout(s, warmup)
        n = lib_run_noout(s, steps)
        ms = s.last_run_ms()
        info, t = s.info(), s.tuning()
        s.close()
    finally:
        os.chdir(cwd)
    npts = info["nx"] * info["nz"]
    return {"steps": n, "ms_per_step": ms / n, "updates_per_s": npts * n / (ms / 1e3), "tuning": t}


REF_MAX_STEPS = 30   # the reference arm's timed steps at most (about 0.3 s each per process)
REF_MAX_WARMUP = 5
REPEATS = 5          # repetitions of the timed window (median reported, spread beside it)


def _spread(rates: list) -> dict:
    return {"median": statistics.median(rates), "min": min(rates), "max": max(rates), "repeats": len(rates)}


def run_form(d: str, precision: int, steps: int, warmup: int, gpu: int, clocks: bool = False,
             repeats: int = REPEATS) -> dict:
    """Device-resident timing of one form.  Autotune (state restored), one
    warm-up pass, then R repetitions of the same window: steps 1..K of the
    solve (reset and the initialising step 0 before each, untimed), CUDA
    events on the solver's stream.  The median repetition is the value.  A
    last pass of the same window brackets every kernel launch with events (for
    the roofline)."""
    import sks
    cwd = os.getcwd()
    os.chdir(d)
    try:
        s = sks.Solver(["par=run.par"], precision=precision, device=gpu)
        s.load_boundary_files()
        info = s.info()
        lib_run_noout(s, warmup)
        tuning = s.autotune(16)
        s.reset()
        lib_run_noout(s, 1 + max(warmup, steps))       # warm-up pass over the window
        ck = Clocks(gpu) if clocks else None
        if ck:
            ck.__enter__()
        times, launches = [], 0
        for _ in range(repeats):
            s.reset()
            lib_run_noout(s, 1)
            l0 = s.launches()
            n = lib_run_noout(s, steps)
            times.append(s.last_run_ms())
            launches = s.launches() - l0
        if ck:
            ck.__exit__(None, None, None)
        # kernel-level pass over the same window: every launch bracketed by events
        s.reset()
        lib_run_noout(s, 1)
        s.enable_kernel_timing(True)
        lib_run_noout(s, steps)
        kt = s.kernel_timing()
        s.close()
    finally:
        os.chdir(cwd)
    npts = info["nx"] * info["nz"]
    ms = statistics.median(times)
    res = {"steps": n, "ms": ms, "ms_per_step": ms / n, "points": npts, "tuning": tuning,
           "updates_per_s": npts * n / (ms / 1e3), "launches": launches, "kernels": kt, "info": info,
           "spread": _spread([npts * n / (t / 1e3) for t in times])}
    if ck:
        res["clocks"] = ck.summary()
    return res


def lib_run_noout(s, steps: int) -> int:
    """sks_run with no seismogram buffers: nothing is copied back, no host sync per chunk."""
    import sks
    n = sks.lib().sks_run(s.h, steps, None, None, None)
    if n < 0:
        raise sks.SksError(n, sks.lib().sks_last_error().decode())
    return n


def run_e2e(d: str, precision: int, steps: int, warmup: int, gpu: int, tuning=None,
            repeats: int = REPEATS) -> dict:
    """Through the C ABI with host buffers, over the window of run_form from
    the solve's start: upload the boundary records from pinned memory, run
    steps 0..K (step 0 initialises; K updates are counted), read the
    seismograms back; wall-clock timed, one warm-up pass, then R repetitions
    (median reported).  The solver is opened (host set-up, device allocation)
    before the timed region.  The tuning found for the device-resident run is
    reused."""
    import ctypes as C
    import sks
    cwd = os.getcwd()
    os.chdir(d)
    try:
        s = sks.Solver(["par=run.par", f"nst={steps + 1}"], precision=precision, device=gpu)
        if tuning:
            s.set_tuning(tuning["warps_per_block"], tuning["band_rows"], tuning["zseam"], tuning["register_cap"],
                         tuning["waves"], tuning.get("pipeline", 0))
        info = s.info()
        npsv, nsh = info["nrec_psv"] * info["mtotal"], info["nrec_sh"] * info["shtotal"]
        psv, sh = _pinned(npsv), _pinned(nsh)
        psv.numpy()[:] = np.fromfile("greenfile", np.float32, count=npsv)
        sh.numpy()[:] = np.fromfile("shgreenfile", np.float32, count=nsh)
        nt = info["ntrace"]
        outs = [_pinned((steps + 1) * nt) for _ in range(3)]
        fp = C.POINTER(C.c_float)
        ptr = lambda t: C.cast(t.data_ptr(), fp)
        walls = []
        for rep in range(repeats + 1):                 # rep 0: warm-up
            s.reset()
            t0 = time.perf_counter()
            rc = sks.lib().sks_set_boundary(s.h, ptr(psv), info["nrec_psv"], ptr(sh), info["nrec_sh"])
            if rc < 0:
                raise sks.SksError(rc, sks.lib().sks_last_error().decode())
            n = sks.lib().sks_run(s.h, steps + 1, ptr(outs[0]), ptr(outs[1]), ptr(outs[2]))
            if n < 0:
                raise sks.SksError(n, sks.lib().sks_last_error().decode())
            n -= 1                                     # updates: step 0 only initialises
            if rep:
                walls.append(time.perf_counter() - t0)
        s.close()
    finally:
        os.chdir(cwd)
    npts = info["nx"] * info["nz"]
    wall = statistics.median(walls)
    return {"value": npts * n / wall, "wall_s": wall, "h2d_bytes_per_step": (npsv + nsh) * 4 // max(1, n),
            "d2h_bytes_per_step": 3 * nt * 4, "steps": n, "spread": _spread([npts * n / w for w in walls])}


def run_plain(gpu: int, steps: int, warmup: int) -> dict:
    """The plain isotropic P-SV case: 400 x 200 km as 200 x 100 elements of
    2 km (801 x 401 = 321,201 points), GLL degree 4, crust over mantle, SV
    plane wave p = 0.045 s/km, Ricker 0.2 Hz, dt 10 ms, 6000 steps, 101
    receivers, P-SV only.  The FP64 form device-resident over a window of K
    steps after autotuning (with its FP64 compute and HBM rooflines), then the
    whole 6000-step solve of each form through the C ABI from the par file:
    boundary files read, run, seismograms back in host memory, wall-clock;
    solves per hour of each form and their ratio."""
    import sks
    import synth
    c = synth.config_isotropic_psv()
    d = tempfile.mkdtemp(prefix="sks_plain_")
    out = {}
    try:
        synth.write_case(c, d)
        cwd = os.getcwd()
        os.chdir(d)
        try:
            for name, prec in (("fp64", sks.FP64), ("fp32c", sks.FP32C)):
                s = sks.Solver(["par=run.par"], precision=prec, device=gpu)
                s.load_boundary_files()
                info = s.info()
                lib_run_noout(s, warmup)
                tun = s.autotune(16)
                s.reset()
                lib_run_noout(s, 1 + max(warmup, steps))
                times = []
                for _ in range(REPEATS):
                    s.reset()
                    lib_run_noout(s, 1)
                    n = lib_run_noout(s, steps)
                    times.append(s.last_run_ms())
                s.reset()
                lib_run_noout(s, 1)
                s.enable_kernel_timing(True)
                lib_run_noout(s, steps)
                kt = s.kernel_timing()
                s.enable_kernel_timing(False)
                # the whole solve: records from the files, seismograms to host memory
                s.reset()
                t0 = time.perf_counter()
                s.load_boundary_files()
                seis = s.run(c.nst)
                wall = time.perf_counter() - t0
                s.close()
                npts = info["nx"] * info["nz"]
                ms = statistics.median(times)
                km = kt["element"][0] / n
                out[name] = {"updates_per_s": npts * n / (ms / 1e3), "ms_per_step": ms / n, "timed_steps": n,
                             "spread": _spread([npts * n / (t / 1e3) for t in times]), "tuning": tun,
                             "kernel_ms_per_step": km, "whole_solve_s": wall,
                             "whole_solve_updates_per_s": npts * c.nst / wall,
                             "solves_per_hour": 3600.0 / wall,
                             "seismograms_finite": bool(all(np.isfinite(x).all() for x in seis))}
        finally:
            os.chdir(cwd)
    finally:
        shutil.rmtree(d, ignore_errors=True)
    out["points"] = npts
    out["steps"] = c.nst
    out["solves_per_hour_ratio_fp32c_over_fp64"] = out["fp32c"]["solves_per_hour"] / out["fp64"]["solves_per_hour"]
    return out


# ---------------------------------------------------------------- CPU side
def _open_instances(inst, precision: int, gpu: int, base: str) -> list:
    """Solvers of the batched workload's instances; boundary records generated on the device."""
    import sks
    import synth
    sol = []
    for k, i in enumerate(inst):
        d = os.path.join(base, f"i{k:02d}")
        synth.write_case(i["case"], d)
        cwd = os.getcwd()
        os.chdir(d)
        try:
            s = sks.Solver(["par=run.par"], precision=precision, device=gpu)
        finally:
            os.chdir(cwd)
        s.set_boundary_plane_wave(i["vs_bottom"], i["p"], i["f0"], 1.0, 0.0)
        sol.append(s)
    return sol


def run_batch(gpu: int, steps: int, warmup: int, fp64_steps: int = 8, instances: int = 64,
              full: bool = True, tuning=None) -> dict:
    """The batched workload (64 seeded uneven instances, FP32C): autotuned
    batch, a timed window with every member active, then all 64 full solves
    from step 0 to the end with the seismograms read back, wall-clock timed.
    An FP64 batch of the same instances is timed over a short window."""
    import sks
    import synth
    inst = synth.config_batch(n=instances)
    base = tempfile.mkdtemp(prefix="sks_batch_")
    out = {}
    try:
        t0 = time.perf_counter()
        sol = _open_instances(inst, sks.FP32C, gpu, base)
        open_s = time.perf_counter() - t0
        infos = [s.info() for s in sol]
        pts = [i["nx"] * i["nz"] for i in infos]
        work = sum(p * i["nst"] for p, i in zip(pts, infos))
        b = sks.Batch(sks.FP32C, gpu)
        for s in sol:
            b.add(s)
        b.run(warmup, want=False)
        if tuning:
            b.set_tuning(*tuning)
            tun = b.tuning()
        else:
            tun = b.autotune(4)
        k = max(1, min(steps, min(i["nst"] for i in infos) - warmup - 8))
        l0 = b.launches()
        b.run(k, want=False)
        ms = b.last_run_ms()
        launches = b.launches() - l0
        rate = sum(pts) * k / (ms / 1e3)
        # the full solves, from step 0, seismograms into host arrays
        wall = full_dev_ms = float("nan")
        finite = None
        if full:
            for s in sol:
                s.reset()
            t0 = time.perf_counter()
            res = b.run(10 ** 7, want=True)
            wall = time.perf_counter() - t0
            full_dev_ms = b.last_run_ms()
            assert all(r[0].shape[0] == i["nst"] for r, i in zip(res, infos))
            finite = all(np.isfinite(r[c]).all() for r in res for c in range(3))
        b.close()
        for s in sol:
            s.close()
        mem = sum(i["device_bytes"] for i in infos)
        out["fp32c"] = {"updates_per_s": rate, "ms_per_batch_step": ms / k, "timed_steps": k,
                        "launches_in_window": launches, "tuning": tun,
                        "full_solves": {"solves": len(sol), "wall_s": wall, "device_s": full_dev_ms / 1e3,
                                        "updates_per_s": work / wall, "solves_per_hour": len(sol) * 3600.0 / wall,
                                        "seismograms_finite": finite}}
        # FP64: same instances, short timed window
        sol = _open_instances(inst, sks.FP64, gpu, base)
        b = sks.Batch(sks.FP64, gpu)
        for s in sol:
            b.add(s)
        b.set_tuning(4, 8, 1, 0)
        b.run(3, want=False)
        b.run(fp64_steps, want=False)
        ms64 = b.last_run_ms()
        b.close()
        for s in sol:
            s.close()
        rate64 = sum(pts) * fp64_steps / (ms64 / 1e3)
        out["fp64"] = {"updates_per_s": rate64, "ms_per_batch_step": ms64 / fp64_steps, "timed_steps": fp64_steps,
                       "solves_per_hour_at_this_rate": len(inst) * 3600.0 / (work / rate64),
                       "tuning": {"warps_per_block": 4, "band_rows": 8, "zseam": 1, "register_cap": 0}}
        out.update({"instances": len(inst), "points_per_step": sum(pts), "updates_per_full_batch": work,
                    "steps_min_max": [min(i["nst"] for i in infos), max(i["nst"] for i in infos)],
                    "open_s": open_s, "fp32c_device_bytes": mem})
    finally:
        shutil.rmtree(base, ignore_errors=True)
    return out


def run_serve(gpu: int, rate: float, nreq: int = 24, seed: int = 7, fp64_frac: float = 0.1,
              prep_threads: int = 8, quantum: int = 64, tuning32=(4, 12, 0, 1, 1)) -> dict:
    """The served workload: seeded Poisson arrivals of `nreq` SKS solve
    requests at `rate` per second (mesh sizes lognormal, median 400 x 200
    elements, clipped to 100 x 50 .. 2000 x 600, element 1-2 km; physics as in
    the batched workload; FP64 with probability fp64_frac).  Each request's
    host set-up is built at its arrival by a pool of threads and submitted;
    the main thread runs the serving loop.  Latency runs from the scheduled
    arrival to the moment the seismograms are in host memory."""
    import threading
    from concurrent.futures import ThreadPoolExecutor
    import sks
    import synth
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, nreq)
    arrivals = np.cumsum(gaps) - gaps[0]
    specs = []
    for _ in range(nreq):
        nex, nez = synth.draw_served_size(rng)
        eh = float(rng.uniform(1.0, 2.0))
        inst = synth.draw_instance(rng, nex, nez, eh)
        form = sks.FP64 if rng.random() < fp64_frac else sks.FP32C
        specs.append((inst, form))
    base = tempfile.mkdtemp(prefix="sks_serve_")
    srv = sks.Server(gpu, 0, quantum)
    srv.set_tuning(sks.FP32C, *tuning32)
    srv.set_tuning(sks.FP64, 4, 8, 1, 0)
    lock = threading.Lock()
    ids, errors = {}, []
    t_start = srv.clock() + 1.0

    def prepare(k):
        inst, form = specs[k]
        wait = t_start + arrivals[k] - srv.clock()
        if wait > 0:
            time.sleep(wait)
        try:
            d = os.path.join(base, f"r{k:03d}")
            synth.write_case(inst["case"], d, absolute=True)
            su = sks.Setup([f"par={os.path.join(d, 'run.par')}"])
            rid = srv.submit(su, form, (inst["vs_bottom"], inst["p"], inst["f0"], 1.0, 0.0))
            with lock:
                ids[k] = rid
        except Exception as e:  # reported in the result
            with lock:
                errors.append(f"request {k}: {e}")
                ids[k] = None

    done = {}
    work = {}
    try:
        with ThreadPoolExecutor(prep_threads) as pool:
            futs = [pool.submit(prepare, k) for k in range(nreq)]
            while len(done) < nreq:
                srv.step()
                with lock:
                    items = list(ids.items())
                for k, rid in items:
                    if k in done:
                        continue
                    if rid is None:
                        done[k] = None
                        continue
                    inf = srv.info(rid)
                    if inf["state"] in (sks.REQ_DONE, sks.REQ_FAILED):
                        out = srv.result(rid)
                        ok = inf["state"] == sks.REQ_DONE and all(np.isfinite(o).all() for o in out)
                        inf["finite"] = bool(ok)
                        done[k] = inf
                        c = specs[k][0]["case"]
                        work[k] = (c.nex * 4 + 1) * (c.nez * 4 + 1) * inf["nst"]
                        srv.release(rid)
            for f in futs:
                f.result()
    finally:
        srv.close()
        shutil.rmtree(base, ignore_errors=True)
    ok = {k: v for k, v in done.items() if v is not None and v["state"] == sks.REQ_DONE}
    lat = {k: v["done_s"] - (t_start + arrivals[k]) for k, v in ok.items()}
    def pct(xs, q):
        return float(np.percentile(np.array(xs), q)) if xs else None
    by_form = {}
    for name, f in (("fp32c", sks.FP32C), ("fp64", sks.FP64)):
        xs = [lat[k] for k in lat if specs[k][1] == f]
        by_form[name] = {"requests": sum(1 for s in specs if s[1] == f), "completed": len(xs),
                         "p50_s": pct(xs, 50), "p99_s": pct(xs, 99)}
    span = max(v["done_s"] for v in ok.values()) - t_start if ok else None
    return {"rate_per_s": rate, "requests": nreq, "completed": len(ok), "failed": nreq - len(ok),
            "errors": errors[:3], "fp64_fraction": fp64_frac,
            "latency_s": {"p50": pct(list(lat.values()), 50), "p99": pct(list(lat.values()), 99), **by_form},
            "queue_wait_s_p50": pct([v["admit_s"] - (t_start + arrivals[k]) for k, v in ok.items()], 50),
            "span_s": span, "solves_per_hour": len(ok) * 3600.0 / span if span else None,
            "updates_per_s": sum(work[k] for k in ok) / span if span else None,
            "all_finite": all(v["finite"] for v in ok.values()),
            "arrival_window_s": float(arrivals[-1]), "quantum_steps": quantum,
            "tuning_fp32c": dict(zip(("warps_per_block", "band_rows", "zseam", "register_cap", "pipeline"), tuning32))}


def run_accuracy(gpu: int, nst: int = FULL_STEPS) -> dict:
    """The whole anisotropic 3-component solve (24000 steps) in both forms:
    relative L2 of the FP32C seismograms against the FP64 ones, per
    component, and the Silver-Chan splitting of both at five interior
    receivers.  The FP64 form stands in for the FP64 oracle at this size (it
    matches the oracle to relative L2 <= 1e-10 on the parity cases; the CPU
    oracle would need hours here).  Boundary records are generated on the
    device."""
    import sks
    import splitting
    import synth
    c = synth.config_aniso_3c(nst=nst)
    c.write_records = False
    d = tempfile.mkdtemp(prefix="sks_acc_")
    out = {}
    try:
        summ = synth.write_case(c, d)
        seis = {}
        for name, prec in (("fp64", sks.FP64), ("fp32c", sks.FP32C)):
            cwd = os.getcwd()
            os.chdir(d)
            try:
                s = sks.Solver(["par=run.par"], precision=prec, device=gpu)
            finally:
                os.chdir(cwd)
            s.set_boundary_plane_wave(summ["vs"], c.p, c.f0, c.sv_amp, c.sh_amp)
            t0 = time.perf_counter()
            seis[name] = s.run(nst)
            out[f"{name}_solve_s"] = time.perf_counter() - t0
            s.close()
        a, b = seis["fp64"], seis["fp32c"]
        out["rel_l2"] = {k: float(np.linalg.norm(b[i].astype(np.float64) - a[i]) / max(np.linalg.norm(a[i]), 1e-300))
                         for i, k in enumerate(("u_x", "u_y", "minus_u_z"))}
        sp = []
        for r in (50, 75, 100, 125, 150):
            w = splitting.sks_window(a[0][:, r], c.sdt, 5.0)
            e64 = splitting.splitting(a[0][:, r], a[1][:, r], c.sdt, w, max_delay=3.0, dphi=0.25)
            e32 = splitting.splitting(b[0][:, r], b[1][:, r], c.sdt, w, max_delay=3.0, dphi=0.25)
            sp.append({"receiver": r, "x_km": c.rec_x0 + r * c.rec_dx,
                       "fp64_phi_deg": e64["phi_deg"], "fp64_delay_s": e64["delay_s"],
                       "dphi_deg": abs(e32["phi_deg"] - e64["phi_deg"]),
                       "ddelay_s": abs(e32["delay_s"] - e64["delay_s"])})
        out.update({"splitting": sp, "max_dphi_deg": max(x["dphi_deg"] for x in sp),
                    "max_ddelay_s": max(x["ddelay_s"] for x in sp), "steps": nst,
                    "reference_form": "the GPU FP64 form over the whole solve (the oracle would need hours here); "
                                      "against the FP64 oracle itself: oracle_window",
                    "splitting_grid": {"dphi_deg": 0.25, "ddelay_s": c.sdt}})
    finally:
        shutil.rmtree(d, ignore_errors=True)
    return out


WINDOW_STEPS = 240        # the anisotropic mesh's oracle window: 1.2 s
WINDOW_RECORD_T0 = 400    # its records start 2 s into the plane wave, so the pulse enters inside it
STATE_HDR = 88            # bytes of a saved solver state's header; int32 `cur` at byte 32


def _oracle_window_worker(d: str, steps: int, out: str) -> None:
    sys.path.insert(0, ROOT)
    from oracle.oracle import Oracle
    o = Oracle([f"par={os.path.join(d, 'run.par')}"], fp64=True)
    o.run(steps)
    np.save(out, o.field())
    o.close()


def _state_field(state, info, precision: int) -> np.ndarray:
    """u^n of a saved solver state as [nz][nx][3] float64 (x, y, z)."""
    import sks
    n = info["nx"] * info["nz"]
    cur = int(np.frombuffer(state[32:36].tobytes(), np.int32)[0])
    dt = np.float64 if precision == sks.FP64 else np.float32
    el = np.dtype(dt).itemsize
    o = STATE_HDR + cur * 3 * n * el
    buf = np.frombuffer(state[o:o + 3 * n * el].tobytes(), dt).astype(np.float64)
    pairs = buf[:2 * n].reshape(n, 2)
    return np.stack([pairs[:, 0], buf[2 * n:3 * n], pairs[:, 1]], axis=1).reshape(info["nz"], info["nx"], 3)


class OracleWindow:
    """Accuracy against the FP64 oracle on the anisotropic 3-component mesh
    itself (3,844,401 points), over a window of 240 steps whose boundary
    records start 2 s into the plane wave: the oracle (a checker) runs in a
    spawned process on one host core while the GPU legs run; compare() solves
    the same window in both GPU forms and returns the relative L2 of the whole
    displacement field u^n at the window's end."""

    def __init__(self):
        import synth
        self.d = tempfile.mkdtemp(prefix="sks_window_")
        c = synth.config_aniso_3c(nst=WINDOW_STEPS)
        c.record_t0 = WINDOW_RECORD_T0
        synth.write_case(c, self.d, absolute=True)
        self.out = os.path.join(self.d, "oracle_field.npy")
        self.t0 = time.perf_counter()
        self.proc = mp.get_context("spawn").Process(target=_oracle_window_worker,
                                                    args=(self.d, WINDOW_STEPS, self.out))
        self.proc.start()

    def compare(self, gpu: int) -> dict:
        import sks
        try:
            fields = {}
            for name, prec in (("fp64", sks.FP64), ("fp32c", sks.FP32C)):
                with sks.Solver([f"par={os.path.join(self.d, 'run.par')}"], precision=prec, device=gpu) as s:
                    s.load_boundary_files()
                    lib_run_noout(s, WINDOW_STEPS)
                    fields[name] = _state_field(s.save_state(), s.info(), prec)
            self.proc.join()
            wall = time.perf_counter() - self.t0
            if self.proc.exitcode != 0 or not os.path.exists(self.out):
                return {"error": f"oracle process exit code {self.proc.exitcode}"}
            ref = np.load(self.out)
            nr = np.linalg.norm(ref)
            out = {"steps": WINDOW_STEPS, "points": int(ref.shape[0] * ref.shape[1]),
                   "records_from_s": WINDOW_RECORD_T0 * 0.005, "oracle_wall_s": wall,
                   "what": "relative L2 of the 3-component displacement field u^n after the window, against "
                           "the FP64 oracle (C restatement of the reference's loop, FP64 build)"}
            for name, f in fields.items():
                out[name] = {"field_rel_l2": float(np.linalg.norm(f - ref) / nr),
                             "per_component": [float(np.linalg.norm(f[..., k] - ref[..., k]) /
                                                     max(np.linalg.norm(ref[..., k]), 1e-300)) for k in range(3)]}
            return out
        finally:
            if self.proc.is_alive():
                self.proc.terminate()
            shutil.rmtree(self.d, ignore_errors=True)


def run_large(gpu: int, steps: int, warmup: int) -> dict:
    """The single large solve: 1000 x 250 km as 4000 x 1000 elements of 250 m
    (64,020,001 points), the anisotropic layer of the 3-component case, SV
    plane wave p = 0.045 s/km, Ricker 2 Hz, dt 1.5 ms, 1001 receivers; FP32C,
    autotuned, device-resident, boundary records generated on the device.
    A timed window of `steps` steps (the whole solve is 40000)."""
    import sks
    import synth
    c = synth.config_large()
    c.write_records = False
    d = tempfile.mkdtemp(prefix="sks_large_")
    try:
        summ = synth.write_case(c, d)
        cwd = os.getcwd()
        os.chdir(d)
        try:
            t0 = time.perf_counter()
            s = sks.Solver(["par=run.par"], precision=sks.FP32C, device=gpu)
            open_s = time.perf_counter() - t0
        finally:
            os.chdir(cwd)
        s.set_boundary_plane_wave(summ["vs"], c.p, c.f0, c.sv_amp, c.sh_amp)
        info = s.info()
        lib_run_noout(s, warmup)
        tun = s.autotune(6)
        n = lib_run_noout(s, steps)
        ms = s.last_run_ms()
        s.reset()
        lib_run_noout(s, warmup)
        s.enable_kernel_timing(True)
        lib_run_noout(s, steps)
        kt = s.kernel_timing()
        s.close()
    finally:
        shutil.rmtree(d, ignore_errors=True)
    npts = info["nx"] * info["nz"]
    km, kc = kt["element"]
    t_launch = km / max(1, n) / 1e3
    return {"points": npts, "steps": n, "ms_per_step": ms / n, "updates_per_s": npts * n / (ms / 1e3),
            "kernel_ms_per_step": t_launch * 1e3,
            "kernel_gbs": npts * BYTES_PER_POINT["fp32c"] / t_launch / 1e9,
            "kernel_gbs_layout_bytes": npts * LAYOUT_BYTES_PER_POINT["fp32c"] / t_launch / 1e9,
            "tuning": tun, "device_bytes": info["device_bytes"], "open_s": open_s,
            "full_solve_s_at_this_rate": 40000 * ms / n / 1e3}


def _cpu_worker(args):
    d, nsteps, fp64, warm = args
    sys.path.insert(0, ROOT)
    from oracle.oracle import Oracle
    os.chdir(d)
    o = Oracle(["par=run.par"], fp64=fp64)
    o.run(1 + warm)               # step 0 (initialisation only), then the warm-up steps
    t0 = time.perf_counter()
    o.run(nsteps)
    dt = time.perf_counter() - t0
    pts = o.nx * o.nz
    o.close()
    return pts * nsteps, dt


def cpu_rate(d: str, nsteps: int, procs: int, warm: int = 0) -> dict:
    """The oracle's float build (the reference's arithmetic restated, bit-exact
    to the reference binary) on the host cores: `procs` independent
    single-threaded solves at once, each `warm` untimed steps then `nsteps`
    timed ones."""
    from oracle import oracle as orc
    orc.build(with_reference=False)
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        t0 = time.perf_counter()
        res = pool.map(_cpu_worker, [(d, nsteps, False, warm)] * procs)
        wall = time.perf_counter() - t0
    pts = sum(r[0] for r in res)
    per_proc = [r[0] / r[1] for r in res]
    step_s = [r[1] / nsteps for r in res]
    return {"value": sum(per_proc), "per_process": statistics.median(per_proc), "wall_s": wall, "procs": procs,
            "pts": pts, "s_per_step_median": statistics.median(step_s), "s_per_step_max": max(step_s)}


# ---------------------------------------------------------------- main
def _dist():
    """Replicas: one process per GPU under torchrun (NCCL), or gloo without GPUs."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        return dist, int(os.environ["RANK"]), ws, int(os.environ.get("LOCAL_RANK", "0"))
    return None, 0, 1, 0


def _max_over_ranks(dist, v: float) -> float:
    """The largest of the ranks' values (every rank gets it)."""
    if dist is None:
        return v
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(dist, world: int, units_per_rank: float, ms: float) -> tuple[float, float]:
    """Whole-job rate of N independent replicas (weak scaling): every rank did
    units_per_rank units; the job took the slowest rank's time.  Returns
    (max ms over ranks, units per second of the whole job)."""
    ms_max = _max_over_ranks(dist, ms)
    return ms_max, world * units_per_rank / (ms_max / 1e3)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--warmup", type=int, default=30)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=45,
                    help="time steps of the CPU baseline sample (45: about 10 s of one core)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--kernel-only", action="store_true",
                    help="only the device-resident step loop of one form (profiling)")
    ap.add_argument("--form", default="fp32c", choices=["fp32c", "fp64"])
    ap.add_argument("--tuning", default="", help="W,B,Z,C[,V[,P]]: warps per CTA, band rows, band seams, register cap, "
                    "waves, pipelined chunks")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched 64-instance workload")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain isotropic P-SV FP64 workload")
    ap.add_argument("--batch-only", action="store_true", help="only the batched workload (one JSON object)")
    ap.add_argument("--batch-instances", type=int, default=64,
                    help="with --batch-only: the first N instances of the seeded batch (profiling a smaller batch)")
    ap.add_argument("--batch-no-full", action="store_true", help="with --batch-only: skip the full solves")
    ap.add_argument("--batch-tuning", default="", help="with --batch-only: W,B,Z,C instead of autotuning")
    ap.add_argument("--no-serve", action="store_true", help="skip the served workload")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the whole-solve FP32C-vs-FP64 accuracy run")
    ap.add_argument("--accuracy-only", action="store_true")
    ap.add_argument("--no-large", action="store_true", help="skip the 64 M-point single solve")
    ap.add_argument("--large-only", action="store_true")
    ap.add_argument("--serve-rates", default="", help="only the served workload at these arrival rates (req/s), "
                    "one JSON object per rate, e.g. 2,5,10,20")
    ap.add_argument("--serve-requests", type=int, default=24)
    ap.add_argument("--serve-fp64-fraction", type=float, default=0.1)
    ap.add_argument("--serve-tuning", default="4,12,0,1,1",
                    help="with --serve-rates: W,B,Z,C,P of the FP32C batch (P: pipelined chunks)")
    a = ap.parse_args()
    warmup_requested = a.warmup
    a.warmup = max(3, a.warmup)
    dist, rank, world, local = _dist()

    if a.impl == "reference":
        # the reference's CPU path (float restatement, bit-exact to the
        # reference binary) on every host core, rank 0 only.  A step here is
        # one time step of the full mesh in each of the host's cores'
        # independent solves; the run is capped so it ends within a minute.
        if rank != 0:
            return
        ncpu = os.cpu_count() or 1
        ksteps = max(1, min(a.steps, REF_MAX_STEPS))
        kwarm = max(1, min(a.warmup, REF_MAX_WARMUP))
        d = tempfile.mkdtemp(prefix="sks_ref_")
        try:
            make_case(d, ksteps + kwarm + 8)
            r = cpu_rate(d, ksteps, ncpu, kwarm)
        finally:
            shutil.rmtree(d, ignore_errors=True)
        v = r["value"]
        line = {"impl": "reference", "metric": "GLL-pt updates/s", "value": v, "unit": "GLL-pt updates/s",
                "n_gpus": a.gpus, "steps": ksteps, "warmup": kwarm,
                "ms_per_step": r["s_per_step_median"] * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": WORKLOAD, "form": "reference float arithmetic",
                           "step": f"one time step of the 3,844,401-point mesh in each of {ncpu} independent "
                                   "single-threaded solves running at once",
                           "steps_requested": a.steps, "warmup_requested": warmup_requested},
                "cpu_baseline": {"value": v, "unit": "GLL-pt updates/s", "cores": ncpu, "kind": "port",
                                 "sample": f"{kwarm} untimed then {ksteps} timed time steps of the full mesh in "
                                           f"each of {ncpu} independent single-threaded processes (oracle float "
                                           "build, bit-exact to the reference binary; the reference sources are "
                                           "not on the GPU host, so its binary cannot be built there)",
                                 "per_process": r["per_process"], "s_per_step_max": r["s_per_step_max"]},
                "e2e": {"value": v, "unit": "GLL-pt updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    gpu = local if world > 1 else 0
    torch.cuda.set_device(gpu)
    if a.kernel_only:
        d = tempfile.mkdtemp(prefix="sks_prof_")
        try:
            make_case(d, a.warmup + a.steps + 8)
            tun = tuple(int(x) for x in a.tuning.split(",")) if a.tuning else None
            r = run_fixed(d, 1 if a.form == "fp32c" else 0, a.steps, a.warmup, gpu, tun)
        finally:
            shutil.rmtree(d, ignore_errors=True)
        print(json.dumps({"kernel_only": a.form, **r}))
        return
    if a.batch_only:
        bt = tuple(int(x) for x in a.batch_tuning.split(",")) if a.batch_tuning else None
        print(json.dumps({"batch": run_batch(gpu, min(a.steps, 200), a.warmup, instances=a.batch_instances,
                                             full=not a.batch_no_full, tuning=bt)}))
        return
    if a.accuracy_only:
        print(json.dumps({"accuracy": run_accuracy(gpu)}))
        return
    if a.large_only:
        print(json.dumps({"large": run_large(gpu, min(a.steps, 300), a.warmup)}))
        return
    if a.serve_rates:
        for r in a.serve_rates.split(","):
            t32 = tuple(int(x) for x in a.serve_tuning.split(","))
            print(json.dumps({"serve": run_serve(gpu, float(r), a.serve_requests, fp64_frac=a.serve_fp64_fraction,
                                                 tuning32=t32)}), flush=True)
        return
    orc_win = None
    if rank == 0 and world == 1 and not a.no_cpu and not a.no_accuracy:
        # part of the CPU-baseline leg: the FP64 oracle over the anisotropic
        # mesh's window runs on a host core while the GPU legs run, as the
        # checker of both forms (its result is only compared, never timed)
        orc_win = OracleWindow()
    d = tempfile.mkdtemp(prefix="sks_bench_")
    try:
        nst = a.warmup + a.steps + 8
        make_case(d, nst)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        r32 = run_form(d, 1, a.steps, a.warmup, gpu, clocks=True)
        r64 = run_form(d, 0, min(a.steps, 600), a.warmup, gpu)
        e2e = run_e2e(d, 1, a.steps, a.warmup, gpu, r32["tuning"])
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        ms32 = _max_over_ranks(dist, r32["ms"])
        ms64 = _max_over_ranks(dist, r64["ms"])
        e2e_wall = _max_over_ranks(dist, e2e["wall_s"])
        cpu = None
        if rank == 0 and world == 1 and not a.no_cpu:
            cpu = cpu_rate(d, a.cpu_steps, 1, warm=1)
    finally:
        shutil.rmtree(d, ignore_errors=True)
    plain = None
    if not a.no_plain:
        plain = run_plain(gpu, min(a.steps, 600), a.warmup)
    batch = None
    if not a.no_batch:
        batch = run_batch(gpu, min(a.steps, 200), a.warmup)
    serve = None
    serve_sat = None
    if not a.no_serve:
        serve = run_serve(gpu, 2.0, a.serve_requests)
        # FP32C requests only, arriving faster than they are served: the
        # served form at saturation (its roofline fraction is the served
        # form's target: 0.6 of the HBM bandwidth)
        serve_sat = run_serve(gpu, 20.0, 48, seed=11, fp64_frac=0.0)
    accuracy = None
    if not a.no_accuracy:
        accuracy = run_accuracy(gpu)
    large = None
    if not a.no_large:
        large = run_large(gpu, min(a.steps, 300), a.warmup)
    oracle_check = orc_win.compare(gpu) if orc_win else None
    if accuracy and oracle_check:
        accuracy["oracle_window"] = oracle_check
    if rank != 0:
        return
    npts = r32["points"]
    value = world * npts * r32["steps"] / (ms32 / 1e3)      # ms32: max over ranks (replica_rate)
    v64 = world * npts * r64["steps"] / (ms64 / 1e3)
    peak, peak_kind = _peaks()
    import sks
    fma_peaks = {"fp64": sks.probe_fma_peak(sks.FP64, gpu), "fp32": sks.probe_fma_peak(sks.FP32C, gpu)}
    # roofline of the dominant kernel (the fused step kernel): algorithmic
    # bytes per launch = points it updates x 124 B over its mean event-timed
    # duration; the same with the 72 B the layout actually moves beside it
    # step-kernel time per step (a pipelined chunk is one launch of many steps)
    km, kc = r32["kernels"]["element"]
    main_pts = npts
    t_launch = km / max(1, r32["steps"]) / 1e3
    achieved = main_pts * BYTES_PER_POINT["fp32c"] / t_launch / 1e9
    achieved_layout = main_pts * LAYOUT_BYTES_PER_POINT["fp32c"] / t_launch / 1e9
    traffic = _traffic_per_launch(main_pts)
    km64, kc64 = r64["kernels"]["element"]
    t64 = km64 / max(1, r64["steps"]) / 1e3
    total_k = sum(v[0] for v in r32["kernels"].values())
    # flops the FP64 kernel performs: element rows of isotropic materials take
    # the isotropic stress (FLOPS_PER_POINT["iso"]), the others the full one
    info = r32["info"]
    iso_frac = info.get("iso_rows", 0) / max(1, info["nez"])
    fp64_flops = iso_frac * FLOPS_PER_POINT["iso"] + (1.0 - iso_frac) * FLOPS_PER_POINT["aniso"]
    fp64_roof = npts * fp64_flops / t64 / 1e12
    line = {
        "metric": "GLL-pt updates/s", "value": value, "unit": "GLL-pt updates/s", "n_gpus": world,
        "steps": r32["steps"], "warmup": a.warmup, "ms_per_step": ms32 / r32["steps"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "form": "FP32 wavefield, Kahan-compensated leapfrog",
                   "points_updated_per_step": npts, "points": npts, "l2": "working set > L2 (no flush)",
                   "window": f"steps 1..{r32['steps']} of the solve, timed {REPEATS} times from a reset and "
                             "step 0 (median; spread in value_spread), after autotuning and a warm-up pass",
                   "parallelism": f"replicas x{world}"},
        "value_spread": r32["spread"],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": ("k_step_pipe (pipelined chunk of steps: " if r32["tuning"].get("pipeline") else
                                "k_step (one step: ") + "element force + assembly + update + receivers + injection)",
                     "kernel_ms_per_step": t_launch * 1e3, "kernel_share": km / max(total_k, 1e-12),
                     "bytes_per_point": BYTES_PER_POINT["fp32c"], "points_per_launch": main_pts,
                     "layout_bytes_per_point": LAYOUT_BYTES_PER_POINT["fp32c"],
                     "achieved_layout_bytes": achieved_layout, "frac_layout_bytes": achieved_layout / peak},
        "e2e": {"value": world * npts * e2e["steps"] / e2e_wall, "unit": "GLL-pt updates/s",
                "h2d_bytes_per_step": e2e["h2d_bytes_per_step"], "d2h_bytes_per_step": e2e["d2h_bytes_per_step"],
                "window": "steps 0..K from the solve's start, K updates counted (value's window plus the "
                          "initialising step 0); records uploaded from pinned memory and seismograms read back "
                          "inside the timed region; solver opened before it", "spread": e2e["spread"]},
        "gpu_launches": r32["launches"],
        "clocks": r32.get("clocks"),
        "fp64": {"value": v64, "unit": "GLL-pt updates/s", "ms_per_step": ms64 / r64["steps"],
                 "steps": r64["steps"], "spread": r64["spread"],
                 "roofline": {"bound": "fp64 pipe", "achieved": fp64_roof,
                              "peak": fma_peaks["fp64"], "unit": "TFLOP/s",
                              "frac": fp64_roof / fma_peaks["fp64"] if fma_peaks["fp64"] else None,
                              "peak_kind": "measured: FMA-chain probe of the FP64 pipe (sks_probe_fma_peak)",
                              "flops_per_point": fp64_flops, "isotropic_element_rows": iso_frac,
                              "kernel_ms_per_step": t64 * 1e3,
                              "achieved_gbs": npts * BYTES_PER_POINT["fp64"] / t64 / 1e9,
                              "bytes_per_point": BYTES_PER_POINT["fp64"], "peak_gbs": peak,
                              "fp32_fma_peak_tflops": fma_peaks["fp32"]}},
        "solves_per_hour": {"fp32c": 3600.0 / (FULL_STEPS * ms32 / r32["steps"] / 1e3) * world,
                            "fp64": 3600.0 / (FULL_STEPS * ms64 / r64["steps"] / 1e3) * world,
                            "solve_steps": FULL_STEPS},
        "kernel_ms": {k: v[0] for k, v in r32["kernels"].items()},
        "tuning": {"fp32c": r32["tuning"], "fp64": r64["tuning"]},
    }
    if plain:
        p64 = plain["fp64"]
        t = p64["kernel_ms_per_step"] / 1e3
        tf = plain["points"] * FLOPS_PER_POINT["iso"] / t / 1e12
        p64["roofline"] = {"bound": "fp64 pipe", "achieved": tf, "peak": fma_peaks["fp64"], "unit": "TFLOP/s",
                           "frac": tf / fma_peaks["fp64"] if fma_peaks["fp64"] else None,
                           "flops_per_point": FLOPS_PER_POINT["iso"],
                           "achieved_gbs": plain["points"] * BYTES_PER_POINT["fp64_iso"] / t / 1e9,
                           "bytes_per_point": BYTES_PER_POINT["fp64_iso"], "peak_gbs": peak,
                           "frac_hbm": plain["points"] * BYTES_PER_POINT["fp64_iso"] / t / 1e9 / peak}
        plain["workload"] = ("plain isotropic P-SV case: 200x100 elements of 2 km, 321,201 points, crust over mantle, "
                             "SV p 0.045 s/km, Ricker 0.2 Hz, dt 10 ms, 6000 steps, 101 receivers, P-SV only")
        line["plain_fp64"] = plain
    if batch:
        pb = batch["points_per_step"] * BYTES_PER_POINT["fp32c"] / (batch["fp32c"]["ms_per_batch_step"] / 1e3) / 1e9
        batch["workload"] = ("64 seeded instances: nex U{200..1000}, nez U{100..400}, element 1-2 km, GLL degree 4, "
                             "p U[0.038,0.052], anisotropy U[0,6]%, azimuth U[0,180), tilt U[0,30), Ricker "
                             "U[0.2,0.5] Hz, dt = 0.4 h_min/vp_max, 60 s simulated, SV plane wave generated on the device")
        batch["fp32c"]["roofline"] = {"achieved": pb, "peak": peak, "unit": "GB/s", "frac": pb / peak,
                                      "bytes_per_point": BYTES_PER_POINT["fp32c"]}
        batch["solves_per_hour_ratio_fp32c_full_over_fp64"] = (batch["fp32c"]["full_solves"]["solves_per_hour"] /
                                                                batch["fp64"]["solves_per_hour_at_this_rate"])
        line["batch"] = batch
    if serve:
        serve["workload"] = ("seeded Poisson arrivals of SKS solve requests; meshes lognormal, median 400x200 "
                             "elements, clipped 100x50..2000x600, element 1-2 km, GLL degree 4; physics drawn as "
                             "in the batched workload; 10 % FP64 requests; 60 s simulated each")
        line["serve"] = serve
    if serve_sat:
        u = serve_sat.get("updates_per_s") or 0.0
        serve_sat["roofline"] = {"achieved": u * BYTES_PER_POINT["fp32c"] / 1e9, "peak": peak, "unit": "GB/s",
                                 "frac": u * BYTES_PER_POINT["fp32c"] / 1e9 / peak,
                                 "bytes_per_point": BYTES_PER_POINT["fp32c"],
                                 "over": "the whole span from the first arrival to the last result (ramps "
                                         "included)"}
        line["serve_fp32c_saturated"] = serve_sat
    if accuracy:
        line["accuracy"] = accuracy
    if large:
        large["workload"] = ("single large solve: 4000x1000 elements of 250 m, 64,020,001 points, anisotropic layer "
                             "(4 %, azimuth 45, tilt 20), Ricker 2 Hz, dt 1.5 ms, 1001 receivers, FP32C")
        large["roofline"] = {"achieved": large["kernel_gbs"], "peak": peak, "unit": "GB/s",
                             "frac": large["kernel_gbs"] / peak, "bytes_per_point": BYTES_PER_POINT["fp32c"]}
        line["large"] = large
    if cpu:
        line["cpu_baseline"] = {"value": cpu["value"], "unit": "GLL-pt updates/s", "cores": 1, "kind": "port",
                                "sample": f"1 untimed then {a.cpu_steps} timed time steps of the same mesh, one thread, oracle float "
                                          "build (bit-exact to the reference binary)"}
        if oracle_check:
            line["cpu_baseline"]["oracle_check"] = "accuracy.oracle_window: both GPU forms against the FP64 oracle"
    line["summary"] = _summary(line)
    print(json.dumps(line))


def _summary(line: dict) -> dict:
    """The workloads' headline figures in a few hundred bytes, last in the line."""
    r = lambda x, n=4: None if x is None else float(f"{x:.{n}g}")
    out = {"c1_fp32c": {"value": r(line["value"]), "frac": r(line["roofline"]["frac"], 3),
                        "frac_layout_bytes": r(line["roofline"]["frac_layout_bytes"], 3),
                        "e2e": r(line["e2e"]["value"]), "solves_per_hour": r(line["solves_per_hour"]["fp32c"])},
           "c1_fp64": {"value": r(line["fp64"]["value"]), "frac_fp64_pipe": r(line["fp64"]["roofline"]["frac"], 3),
                       "solves_per_hour": r(line["solves_per_hour"]["fp64"])}}
    out["c1_solves_per_hour_ratio"] = r(line["solves_per_hour"]["fp32c"] / line["solves_per_hour"]["fp64"], 3)
    p = line.get("plain_fp64")
    if p:
        out["c0_plain"] = {"fp64_value": r(p["fp64"]["updates_per_s"]),
                           "fp64_frac_fp64_pipe": r(p["fp64"]["roofline"]["frac"], 3),
                           "fp64_solves_per_hour": r(p["fp64"]["solves_per_hour"]),
                           "fp32c_solves_per_hour": r(p["fp32c"]["solves_per_hour"]),
                           "ratio": r(p["solves_per_hour_ratio_fp32c_over_fp64"], 3)}
    b = line.get("batch")
    if b:
        out["c2_batch"] = {"fp32c_value": r(b["fp32c"]["updates_per_s"]), "frac": r(b["fp32c"]["roofline"]["frac"], 3),
                           "solves_per_hour": r(b["fp32c"]["full_solves"]["solves_per_hour"]),
                           "fp64_value": r(b["fp64"]["updates_per_s"]),
                           "ratio_fp32c_over_fp64": r(b["solves_per_hour_ratio_fp32c_full_over_fp64"], 3)}
    sv = line.get("serve")
    if sv:
        lat = sv["latency_s"]
        out["c3_serve"] = {"rate_per_s": sv["rate_per_s"], "completed": sv["completed"],
                           "p50_s": r(lat["p50"], 3), "p99_s": r(lat["p99"], 3),
                           "fp32c_p50_s": r(lat["fp32c"]["p50_s"], 3), "fp32c_p99_s": r(lat["fp32c"]["p99_s"], 3),
                           "solves_per_hour": r(sv["solves_per_hour"]), "value": r(sv["updates_per_s"])}
    ss = line.get("serve_fp32c_saturated")
    if ss:
        out["c3_serve_fp32c_saturated"] = {"rate_per_s": ss["rate_per_s"], "completed": ss["completed"],
                                           "solves_per_hour": r(ss["solves_per_hour"]),
                                           "value": r(ss["updates_per_s"]), "frac": r(ss["roofline"]["frac"], 3),
                                           "p50_s": r(ss["latency_s"]["p50"], 3),
                                           "p99_s": r(ss["latency_s"]["p99"], 3)}
    acc = line.get("accuracy")
    if acc:
        out["c1_accuracy"] = {"fp32c_vs_fp64_rel_l2": {k: r(v, 3) for k, v in acc["rel_l2"].items()},
                              "max_dphi_deg": acc["max_dphi_deg"], "max_ddelay_s": acc["max_ddelay_s"]}
        ow = acc.get("oracle_window")
        if ow:
            out["c1_accuracy"]["vs_fp64_oracle_window"] = {k: r(ow[k]["field_rel_l2"], 3) for k in ("fp64", "fp32c")}
    lg = line.get("large")
    if lg:
        out["c4_large"] = {"value": r(lg["updates_per_s"]), "frac": r(lg["roofline"]["frac"], 3)}
    return out


def _traffic_per_launch(points: int):
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        t = json.load(f)
    bpp = t.get("fp32c_dram_bytes_per_point")
    return None if bpp is None else bpp * points


if __name__ == "__main__":
    main()
