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
