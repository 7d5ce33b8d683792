"""GPU: the serving loop (continuous batching).

Requests of both forms, uneven sizes and boundary sources arrive while others
run; each result equals the same request run alone with the batch's tuning,
bit for bit; admission never lets the running requests hold more device
memory than the budget; a request that can never fit fails cleanly.
"""
import numpy as np
import pytest

import sks
import synth
from util import chdir

pytestmark = pytest.mark.gpu

T32 = (4, 3, 0, 1)
T64 = (4, 4, 1, 0)


def _layers(H, aniso):
    mid = synth.hexagonal_cij(8.1, 4.5, 3.4, 0.05, 60.0, 20.0) if aniso else synth.iso_cij(8.0, 4.45, 3.35)
    return [synth.SemLayer(H - 6, synth.iso_cij(8.1, 4.5, 3.4), 3.4),
            synth.SemLayer(H - 3, mid, 3.4),
            synth.SemLayer(H + 1, synth.iso_cij(6.4, 3.6, 2.8), 2.8)]


REQS = [  # nex, nez, eh, dt, nst, p, f0, aniso, form, device records
    (31, 10, 1.0, 0.005, 850, 0.045, 1.5, True, sks.FP32C, True),
    (17, 6, 2.0, 0.01, 620, 0.05, 0.8, False, sks.FP64, False),
    (45, 12, 1.0, 0.004, 1100, 0.038, 1.2, True, sks.FP32C, False),
    (24, 10, 1.5, 0.006, 960, 0.042, 1.0, True, sks.FP64, True),
    (20, 8, 1.0, 0.005, 700, 0.048, 1.4, True, sks.FP32C, True),
    (38, 9, 1.0, 0.005, 800, 0.040, 1.1, False, sks.FP32C, False),
]


@pytest.fixture(scope="module")
def reqs(tmp_path_factory):
    out = []
    for i, (nex, nez, eh, dt, nst, p, f0, aniso, form, dev) in enumerate(REQS):
        d = str(tmp_path_factory.mktemp(f"req{i}"))
        H = nez * eh + 0.002
        layers = _layers(H, aniso)
        c = synth.Case(nex=nex, nez=nez, eh=eh, sdt=dt, nst=nst, layers=layers, p=p, f0=f0, sv_amp=1.0, sh_amp=0.3,
                       ntrace=7, rec_dx=nex * eh / 8, semmodel_full=True, write_records=not dev)
        synth.write_case(c, d)
        pw = (float(np.sqrt(layers[0].C[3, 3] / layers[0].rho)), p, f0, 1.0, 0.3) if dev else None
        out.append((d, form, pw, nst))
    return out


def _alone(d, form, pw, nst):
    with chdir(d):
        s = sks.Solver(["par=run.par"], precision=form)
        if pw is None:
            s.load_boundary_files()
    if pw is not None:
        s.set_boundary_plane_wave(*pw)
    s.set_tuning(*(T32 if form == sks.FP32C else T64), 0)
    out = s.run(nst)
    s.close()
    return out


def _setup(d):
    with chdir(d):
        return sks.Setup(["par=run.par"])


def _serve(reqs, budget, arrivals, check_budget=None):
    """arrivals[i]: scheduling round at which request i is submitted."""
    srv = sks.Server(0, budget, 64)
    srv.set_tuning(sks.FP32C, *T32)
    srv.set_tuning(sks.FP64, *T64)
    ids = {}
    rnd = 0
    saw_queue_while_running = False
    while True:
        for i, (d, form, pw, nst) in enumerate(reqs):
            if arrivals[i] == rnd:
                with chdir(d):                       # relative boundary file names resolve here
                    ids[i] = srv.submit(_setup(d), form, pw)
        left = srv.step()
        if check_budget is not None:
            assert srv.device_bytes() <= check_budget
            st = [srv.info(r)["state"] for r in ids.values()]
            if sks.REQ_QUEUED in st and sks.REQ_RUNNING in st:
                saw_queue_while_running = True
        rnd += 1
        if left == 0 and len(ids) == len(reqs):
            break
        assert rnd < 100000
    return srv, ids, saw_queue_while_running


def test_each_result_is_the_same_alone_and_in_the_mix(reqs):
    alone = [_alone(*r) for r in reqs]
    assert all(max(np.abs(x).max() for x in a) > 0.05 for a in alone)
    srv, ids, _ = _serve(reqs, 0, arrivals=[0, 0, 3, 5, 9, 14])
    for i, rid in ids.items():
        info = srv.info(rid)
        assert info["state"] == sks.REQ_DONE, info
        assert info["step"] == reqs[i][3]
        assert 0 <= info["submit_s"] <= info["admit_s"] <= info["done_s"]
        got = srv.result(rid)
        for c in range(3):
            assert np.array_equal(got[c], alone[i][c]), f"request {i} component {c}"
        srv.release(rid)
    assert srv.device_bytes() == 0
    srv.close()


def test_admission_respects_the_device_budget(reqs):
    # the server's own footprint estimates (reported while queued), then room
    # for about two requests at a time
    est = []
    with sks.Server(0, 1 << 40, 64) as probe:
        for d, form, pw, nst in reqs:
            with chdir(d):
                est.append(probe.info(probe.submit(_setup(d), form, pw))["device_bytes"])
    budget = int(2.2 * max(est))
    alone = [_alone(*r) for r in reqs]
    srv, ids, queued_while_running = _serve(reqs, budget, arrivals=[0] * len(reqs), check_budget=budget)
    assert queued_while_running
    for k, rid in ids.items():
        assert srv.info(rid)["state"] == sks.REQ_DONE
        got = srv.result(rid)
        for c in range(3):
            assert np.array_equal(got[c], alone[k][c])
    srv.close()


def test_request_larger_than_the_budget_fails(reqs):
    srv = sks.Server(0, 1 << 20, 64)
    d, form, pw, nst = reqs[2]
    rid = srv.submit(_setup(d), form, pw)
    assert srv.step() == 0
    info = srv.info(rid)
    assert info["state"] == sks.REQ_FAILED and info["status"] == -6
    srv.close()


def test_points_cap_runs_each_form_first_come_first_served(reqs):
    alone = [_alone(*r) for r in reqs]
    srv = sks.Server(0, 0, 64)
    srv.set_tuning(sks.FP32C, *T32)
    srv.set_tuning(sks.FP64, *T64)
    srv.set_active_points(sks.FP32C, 1)        # one request of a form at a time
    srv.set_active_points(sks.FP64, 1)
    ids = []
    for d, form, pw, nst in reqs:
        with chdir(d):
            ids.append(srv.submit(_setup(d), form, pw))
    while srv.step():
        running = [k for k, r in enumerate(ids) if srv.info(r)["state"] == sks.REQ_RUNNING]
        for f in (sks.FP32C, sks.FP64):
            assert sum(1 for k in running if reqs[k][1] == f) <= 1
    for f in (sks.FP32C, sks.FP64):
        ks = [k for k in range(len(reqs)) if reqs[k][1] == f]
        done = [srv.info(ids[k])["done_s"] for k in ks]
        assert done == sorted(done)            # completions in arrival order
    for k, rid in enumerate(ids):
        got = srv.result(rid)
        for c in range(3):
            assert np.array_equal(got[c], alone[k][c])
    srv.close()


def test_layered_requests_are_the_same_alone_and_served(tmp_path):
    """Requests whose boundary records come from a plane wave through a
    layered stack (sks_server_submit_layered) equal the same solve alone."""
    runs = []
    for k, form in enumerate((sks.FP32C, sks.FP64)):
        d = str(tmp_path / f"layered{k}")
        H = 10 * 1.0 + 0.002
        layers = _layers(H, True)
        c = synth.Case(nex=27 + 6 * k, nez=10, eh=1.0, sdt=0.005, nst=640, layers=layers, p=0.042, f0=1.2,
                       sv_amp=1.0, sh_amp=0.4, ntrace=6, rec_dx=3.0, semmodel_full=True, write_records=False)
        synth.write_case(c, d)
        stack = [(8.1, 4.5, 3.4), (6.9, 3.9, 3.0, 7.0 + k), (8.3, 4.6, 3.45)]
        runs.append((d, form, stack, c.nst))
    alone = []
    for d, form, stack, nst in runs:
        with chdir(d):
            s = sks.Solver(["par=run.par"], precision=form)
        s.set_boundary_layered_wave(stack, 0.042, 1.2, 0.0, 1.0, 0.4)
        s.set_tuning(*(T32 if form == sks.FP32C else T64), 0)
        alone.append(s.run(nst))
        s.close()
    assert all(max(np.abs(x).max() for x in a) > 0.05 for a in alone)
    srv = sks.Server(0, 0, 64)
    srv.set_tuning(sks.FP32C, *T32)
    srv.set_tuning(sks.FP64, *T64)
    ids = [srv.submit(_setup(d), form, layered=(stack, 0.042, 1.2, 0.0, 1.0, 0.4)) for d, form, stack, _ in runs]
    rnd = 0
    while srv.step() > 0:
        rnd += 1
        assert rnd < 100000
    for i, rid in enumerate(ids):
        assert srv.info(rid)["state"] == sks.REQ_DONE
        got = srv.result(rid)
        for c in range(3):
            assert np.array_equal(got[c], alone[i][c]), f"request {i} component {c}"
        srv.release(rid)
    srv.close()


@pytest.mark.parametrize("degs", [(4, 5, 4, 5), (3, 6, 4, 3)], ids=["4-5", "3-6-4"])
def test_mixed_degrees_are_served_in_turn(tmp_path, degs):
    """A form's batch runs one GLL degree at a time: requests of several
    degrees arriving mixed all complete, another degree waiting for the batch
    to drain, and each equals its solo run."""
    reqs = []
    for k, hpn in enumerate(degs):
        d = str(tmp_path / f"deg{k}")
        nez, eh = 8, 2.0
        H = nez * eh + 0.002
        c = synth.Case(nex=20 + 3 * k, nez=nez, eh=eh, sdt=0.008, nst=300 + 40 * k, layers=_layers(H, True),
                       p=0.045, f0=1.0, sv_amp=1.0, sh_amp=0.3, hpn=hpn, ntrace=5, rec_dx=4.0, semmodel_full=True,
                       write_records=False)
        synth.write_case(c, d)
        pw = (float(np.sqrt(c.layers[0].C[3, 3] / c.layers[0].rho)), c.p, c.f0, 1.0, 0.3)
        reqs.append((d, sks.FP32C, pw, c.nst))
    alone = [_alone(*r) for r in reqs]
    srv, ids, _ = _serve(reqs, 0, arrivals=[0, 0, 1, 1])
    for i, rid in ids.items():
        assert srv.info(rid)["state"] == sks.REQ_DONE, (i, srv.info(rid))
        got = srv.result(rid)
        for c in range(3):
            assert np.array_equal(got[c], alone[i][c]), f"request {i} component {c}"
        srv.release(rid)
    srv.close()


def test_tunings_that_cannot_run_a_degree_are_refused_early(tmp_path):
    """Degrees 3, 5 and 6 run with 4-warp CTAs and register cap 0 or 1: a
    form tuning outside that is refused while such a request waits, and such
    requests are refused at submission once it is set."""
    dirs = {}
    for hpn in (3, 6):
        d = str(tmp_path / f"deg{hpn}")
        H = 8 * 2.0 + 0.002
        c = synth.Case(nex=20, nez=8, eh=2.0, sdt=0.006 if hpn == 6 else 0.008, nst=200, layers=_layers(H, True),
                       p=0.045, f0=1.0, sv_amp=1.0, sh_amp=0.3, hpn=hpn, ntrace=5, rec_dx=4.0, semmodel_full=True,
                       write_records=False)
        synth.write_case(c, d)
        dirs[hpn] = (d, (float(np.sqrt(c.layers[0].C[3, 3] / c.layers[0].rho)), c.p, c.f0, 1.0, 0.3))
    srv = sks.Server(0, 0, 64)
    rid = srv.submit(_setup(dirs[3][0]), sks.FP32C, dirs[3][1])
    with pytest.raises(sks.SksError) as e:
        srv.set_tuning(sks.FP32C, 2, 4, 0, 1)
    assert e.value.code == -8
    while srv.step() > 0:
        pass
    assert srv.info(rid)["state"] == sks.REQ_DONE
    srv.set_tuning(sks.FP32C, 2, 4, 0, 1)
    for hpn in (3, 6):
        with pytest.raises(sks.SksError) as e:
            srv.submit(_setup(dirs[hpn][0]), sks.FP32C, dirs[hpn][1])
        assert e.value.code == -4
    srv.submit(_setup(dirs[6][0]), sks.FP64, dirs[6][1])       # the other form's tuning still runs it
    while srv.step() > 0:
        pass
    srv.close()
