"""GPU: boundary records generated on the device equal the host generator's.

sks_set_boundary_plane_wave() evaluates the plane-wave records of
synth.plane_wave_records() on the device, with explicitly rounded FP64
arithmetic; only exp may round differently, which moves a float32 record by
at most one unit in the last place.  Both record sets drive the same FP64
solve here: the interpolated boundary increments and the seismograms agree to
that rounding.
"""
import numpy as np
import pytest

import sks
import synth
from util import chdir

pytestmark = pytest.mark.gpu


def _case(tmp_path, psv_only=False, sh_amp=0.6, hpn=4):
    H = 12.002
    layers = [synth.SemLayer(H - 6, synth.iso_cij(8.1, 4.5, 3.4), 3.4),
              synth.SemLayer(H - 3, synth.hexagonal_cij(8.1, 4.5, 3.4, 0.05, 30.0, 15.0), 3.4),
              synth.SemLayer(H + 1, synth.iso_cij(6.4, 3.6, 2.8), 2.8)]
    # degree 6's closest GLL nodes are 85 m apart in a 1 km element: a shorter step keeps it stable
    sdt, nst = (0.0035, 900) if hpn == 6 else (0.005, 700)
    c = synth.Case(nex=29, nez=12, eh=1.0, sdt=sdt, nst=nst, layers=layers, p=0.044, f0=1.3, sv_amp=1.0,
                   sh_amp=sh_amp, ntrace=13, rec_dx=2.0, semmodel_full=True, write_records=False,
                   psv_only=psv_only, hpn=hpn)
    d = str(tmp_path)
    synth.write_case(c, d)
    return d, c, float(np.sqrt(layers[0].C[3, 3] / layers[0].rho))


@pytest.mark.parametrize("psv_only,hpn", [(False, 4), (True, 4), (False, 5), (False, 3), (False, 6)])
def test_device_records_match_host_generator(tmp_path, psv_only, hpn):
    d, c, vs = _case(tmp_path, psv_only, hpn=hpn)
    sh_amp = 0.0 if psv_only else c.sh_amp
    with chdir(d):
        host = sks.Solver(["par=run.par"], precision=sks.FP64)
        dev = sks.Solver(["par=run.par"], precision=sks.FP64)
    i = host.info()
    nbl = i["neh"] * i["hpn"]
    nrec = max(i["nrec_psv"], i["nrec_sh"])
    psv, sh = synth.plane_wave_records(i["nx"], i["nz"], i["h"], nbl, vs, c.p, c.f0, c.sdt, 0, nrec,
                                       c.sv_amp, sh_amp, eh=i["eh"], deg=hpn)
    host.set_boundary(psv[:i["nrec_psv"]], None if psv_only else sh[:i["nrec_sh"]])
    dev.set_boundary_plane_wave(vs, c.p, c.f0, c.sv_amp, sh_amp)
    # interpolated FP64 increments of the interface line: one float32 ulp of a record at most
    scale = float(np.abs(psv).max())
    a = host.line_increments(0, 400)
    b = dev.line_increments(0, 400)
    assert np.abs(a).max() > 1e-3 * scale
    assert np.abs(a - b).max() <= 4 * np.finfo(np.float32).eps * scale
    ua = host.run(c.nst)
    ub = dev.run(c.nst)
    assert np.linalg.norm(ua[0]) > 0 and np.linalg.norm(ua[2]) > 0
    for k in range(3):
        ref = np.linalg.norm(ua[k])
        if ref == 0.0:
            assert np.abs(ub[k]).max() == 0.0
        else:
            assert np.linalg.norm(ua[k] - ub[k]) <= 1e-6 * ref
    host.close()
    dev.close()


def test_plane_wave_rejects_bad_parameters(tmp_path):
    d, c, vs = _case(tmp_path)
    with chdir(d):
        s = sks.Solver(["par=run.par"], precision=sks.FP32C)
    for bad in ((0.0, 0.04, 1.0), (4.5, 0.04, 0.0), (4.5, -0.01, 1.0)):
        with pytest.raises(sks.SksError):
            s.set_boundary_plane_wave(*bad)
    with pytest.raises(sks.SksError):
        s.run(5)                                   # still no boundary records
    s.close()


def test_generated_records_hold_no_table(tmp_path):
    """The generators are evaluated where the interpolation reads a record, so
    a generated run holds no record table: its device memory is the table's
    size below that of the same run fed from caller memory, less the line's
    delays and amplitudes (two doubles per line value)."""
    d, c, vs = _case(tmp_path)
    with chdir(d):
        a = sks.Solver(["par=run.par"], precision=sks.FP32C)
        b = sks.Solver(["par=run.par"], precision=sks.FP32C)
    i = a.info()
    nbl = i["neh"] * i["hpn"]
    nrec = max(i["nrec_psv"], i["nrec_sh"])
    psv, sh = synth.plane_wave_records(i["nx"], i["nz"], i["h"], nbl, vs, c.p, c.f0, c.sdt, 0, nrec,
                                       c.sv_amp, c.sh_amp, eh=i["eh"])
    a.set_boundary(psv[:i["nrec_psv"]], sh[:i["nrec_sh"]])
    b.set_boundary_plane_wave(vs, c.p, c.f0, c.sv_amp, c.sh_amp)
    table = 4 * (i["nrec_psv"] * i["mtotal"] + i["nrec_sh"] * i["shtotal"])
    line = 16 * (i["mtotal"] + i["shtotal"])
    assert a.info()["device_bytes"] - b.info()["device_bytes"] == table - line
    # and back: records from memory replace the generator
    b.set_boundary(psv[:i["nrec_psv"]], sh[:i["nrec_sh"]])
    assert b.info()["device_bytes"] == a.info()["device_bytes"]
    ua, ub = a.run(c.nst), b.run(c.nst)
    for k in range(3):
        assert np.array_equal(ua[k], ub[k])
    a.close()
    b.close()
