"""The C ABI library: it loads, exports every function the headers declare, and rejects
bad input with error codes (no device needed for these)."""
import ctypes as C
import re
from pathlib import Path

import pytest

import cases
import lgame_gpu as L
from conftest import has_gpu

INCLUDE = Path(__file__).resolve().parent.parent / "include"


def declared_functions():
    names = []
    for h in sorted(INCLUDE.glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"\b(lgame_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_function():
    lib = C.CDLL(str(L.LIB_PATH))
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_error_string():
    lib = L.load_library()
    assert b"sm_103a" in lib.lgame_gpu_version()
    assert isinstance(L.last_error(), str)


def _cfg(**kw):
    n = cases.small_case("schaer")
    c = L.config_from_namelist(n)
    for k, v in kw.items():
        setattr(c, k, v)
    return c


@pytest.mark.parametrize("field,value,code", [
    ("n_layers", 2, L.ERR_BAD_DIMS),
    ("n_layers", 200, L.ERR_BAD_DIMS),
    ("n_oro_layers", 0, L.ERR_BAD_DIMS),
    ("theta_adv_order", 5, L.ERR_BAD_CONFIG),
    ("dtime", -1.0, L.ERR_BAD_CONFIG),
    ("precision", 9, L.ERR_BAD_CONFIG),
    ("diff_coeff_scheme_h", 7, L.ERR_BAD_CONFIG),
    ("ltemp_diff_h", 1, L.ERR_UNSUPPORTED),
    ("lmass_diff_h", 1, L.ERR_UNSUPPORTED),
    ("lmom_diff_v", 1, L.ERR_UNSUPPORTED),
    ("lpbl", 1, L.ERR_BAD_CONFIG),                    # the PBL needs lmom_diff_h
    ("lsfc_sensible_heat_flux", 1, L.ERR_UNSUPPORTED),  # divides by a zero resistance without the soil
    ("nsoillays", 17, L.ERR_BAD_CONFIG),
    ("nsoillays", -1, L.ERR_BAD_CONFIG),
])
def test_create_rejects_bad_config(field, value, code):
    lib = L.load_library()
    h = C.c_void_p()
    rc = lib.lgame_gpu_create(C.byref(_cfg(**{field: value})), C.byref(h))
    assert rc == code and not h.value


@pytest.mark.parametrize("kw,code", [
    # non-periodic horizontal momentum diffusion needs lmom_diff_v or third-order theta
    (dict(lmom_diff_h=1, lperiodic=0, theta_adv_order=2), L.ERR_UNSUPPORTED),
    # the prognostic soil needs at least two soil layers
    (dict(lprog_soil_temp=1, nsoillays=1), L.ERR_BAD_CONFIG),
    # the surface layer needs positive karman and h_prandtl
    (dict(lmom_diff_h=1, lpbl=1, karman=0.0), L.ERR_BAD_CONFIG),
])
def test_create_rejects_unsupported_combinations(kw, code):
    lib = L.load_library()
    h = C.c_void_p()
    rc = lib.lgame_gpu_create(C.byref(_cfg(**kw)), C.byref(h))
    assert rc == code and not h.value


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_create_without_device_reports_no_device():
    lib = L.load_library()
    h = C.c_void_p()
    rc = lib.lgame_gpu_create(C.byref(_cfg()), C.byref(h))
    assert rc == L.ERR_NO_DEVICE and not h.value
    assert "device" in L.last_error()


def test_null_arguments_are_errors():
    lib = L.load_library()
    assert lib.lgame_gpu_create(None, None) == L.ERR_INVALID_ARG
    assert lib.lgame_gpu_pchevi(None, 0, 1, 0, 0, 0.0) == L.ERR_INVALID_ARG
    assert lib.lgame_gpu_set_grid(None, None, 0) == L.ERR_INVALID_ARG
    assert lib.lgame_gpu_output(None, 0, 1, 0.5, 0.5, None, 6, None) == L.ERR_INVALID_ARG
    assert lib.lgame_gpu_bc_setup(None, 5, 10800, 0.0, L.BC_LOADER(), None) == L.ERR_INVALID_ARG
    assert lib.lgame_gpu_set_bc(None, 1, None, None, None, None, None) == L.ERR_INVALID_ARG
    assert lib.lgame_gpu_update_boundaries(None, 0, 0.0) == L.ERR_INVALID_ARG
    assert lib.lgame_gpu_bc_state(None, None, None, None) == L.ERR_INVALID_ARG
    lib.lgame_gpu_destroy(None)


def test_c_driver(tmp_path):
    """The headers compile as C99 (-Wall -Werror) and a C program linked against the library
    uses the ABI: namelist, host set-up, snapshot round trip, file names, context creation."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    here = Path(__file__).resolve().parent
    lib = Path(L.LIB_PATH)
    exe = tmp_path / "c_driver"
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", str(INCLUDE), str(here / "c_driver.c"),
                    str(lib), f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
    nml = tmp_path / "namelist.nml"
    nml.write_text(cases.namelist_text(*cases.SMALL["hills_nonperiodic"][0:1], **cases.SMALL["hills_nonperiodic"][1]))
    out = subprocess.run([str(exe), str(nml), str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip().endswith("ok")


def _build_c_driver(tmp_path):
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    here = Path(__file__).resolve().parent
    lib = Path(L.LIB_PATH)
    exe = tmp_path / "c_driver"
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", str(INCLUDE), str(here / "c_driver.c"),
                    str(lib), f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
    return exe


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["jet", "hills"])
def test_c_driver_steps(tmp_path, key):
    """A C host steps the model: two lgame_gpu_pchevi calls against two lgame_gpu_pchevi_host
    calls, FP64 and split, finite and bit-equal (checked inside the C program)."""
    import subprocess
    exe = _build_c_driver(tmp_path)
    nml = tmp_path / "namelist.nml"
    nml.write_text(cases.namelist_text(*cases.SMALL[key][0:1], **cases.SMALL[key][1]))
    out = subprocess.run([str(exe), str(nml), str(tmp_path), "step"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert out.stdout.count("pchevi == pchevi_host") == 2, out.stdout
    assert out.stdout.strip().endswith("ok")

