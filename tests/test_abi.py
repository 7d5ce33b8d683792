"""The C-ABI library loads and exports every entry point include/sks.h declares (CPU)."""
import ctypes
import os
import re
import subprocess

import pytest

import sks

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "sks.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(sks_[a-z_0-9]+)\s*\(", txt)))


def test_header_declares_the_api():
    names = _declared()
    for n in ("sks_open_par", "sks_run", "sks_set_boundary", "sks_load_boundary_files", "sks_destroy"):
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(sks.LIB_PATH)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_library_hides_internal_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", sks.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (sks_\w+)", out))
    assert exported == set(_declared()), exported ^ set(_declared())


def test_binding_covers_every_symbol():
    assert set(sks.EXPORTS) == set(_declared())


def test_cli_is_built():
    cli = os.path.join(os.path.dirname(sks.LIB_PATH), "sem2d_psvsh_gb300")
    assert os.access(cli, os.X_OK)
    assert os.path.islink(os.path.join(os.path.dirname(sks.LIB_PATH), "sem2d_gb300"))
    assert os.access(os.path.join(os.path.dirname(sks.LIB_PATH), "uvw2sac_gb300"), os.X_OK)


def test_error_string_after_failure():
    with pytest.raises(sks.SksError) as e:
        sks.Setup(["par=/nonexistent/run.par"])
    assert "cannot open par file" in str(e.value)


def test_no_device_is_an_error_not_a_crash(tmp_path):
    from conftest import have_gpu
    if have_gpu():
        pytest.skip("a GPU is present")
    import synth
    from util import chdir
    c = synth.Case(nex=6, nez=4, eh=2.0, sdt=0.01, nst=5, layers=synth.layered_two(8.0, 2.0), ntrace=3, rec_dx=2.0)
    synth.write_case(c, str(tmp_path))
    with chdir(str(tmp_path)):
        with pytest.raises(sks.SksError) as e:
            sks.Solver(["par=run.par"])
    assert e.value.code == -5


@pytest.mark.parametrize("words,msg", [
    (["sks_plane_wave=4.5,0.04"], "sks_plane_wave=vs,p,f0"),
    (["sks_plane_wave=4.5,x,1"], "sks_plane_wave=vs,p,f0"),
    (["sks_plane_wave=4.5,0.04,1", "sks_wave=0.04,1"], "exclude each other"),
    (["sks_wave=0.04,1"], "go together"),
    (["sks_stack=stack.txt", "sks_wave=0.04"], "sks_wave=p,f0"),
    (["sks_stack=missing.txt", "sks_wave=0.04,1"], "cannot read the stack file"),
    (["sks_stack=short.txt", "sks_wave=0.04,1"], "2 media at least"),
])
def test_program_refuses_malformed_generator_words(tmp_path, words, msg):
    """The device-generator words of the drop-in program are checked before
    any device work, so their refusals need no GPU."""
    (tmp_path / "stack.txt").write_text("# vp vs rho thickness\n7.6 4.3 3.3 0\n8.1 4.5 3.4 0\n")
    (tmp_path / "short.txt").write_text("7.6 4.3 3.3 0\n")
    cli = os.path.join(os.path.dirname(sks.LIB_PATH), "sem2d_psvsh_gb300")
    r = subprocess.run([cli, "par=run.par"] + words, cwd=str(tmp_path), capture_output=True, text=True)
    assert r.returncode == 1 and msg in r.stderr, r.stderr
