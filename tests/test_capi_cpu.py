"""The C-ABI library without a GPU: it loads, exports every symbol the header
declares, fills the reference defaults and rejects bad arguments before touching
a device.  No compute call is made here."""
import ctypes
import math
import os
import re

import pytest

import ambient_image_processor_gb300 as pkg
from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "tgvdct.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b(tgvdct_[a-z0-9_]+)\s*\(", text))
    return sorted(n for n in names if n != "tgvdct_iteration_callback")


def test_library_exports_every_declared_symbol():
    lib = pkg.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(declared_functions()) <= set(pkg.EXPORTED) | set(declared_functions())


def test_python_binding_covers_header():
    assert set(declared_functions()) == set(pkg.EXPORTED)


def test_params_init_gives_reference_defaults():
    p = pkg.default_params()
    assert p.lambda_ == 1.0 and p.alpha0 == 2.0 and p.alpha1 == 1.0
    assert math.isclose(p.tau, 1 / math.sqrt(20), rel_tol=1e-7)
    assert math.isclose(p.sigma, 1 / math.sqrt(20), rel_tol=1e-7)
    assert p.theta == 1.0
    assert p.data_term == pkg.DATA_L1 and p.geometry == pkg.GEOMETRY_3D
    assert p.state_precision == pkg.STATE_FP32 and p.poisson_eigen == pkg.EIGEN_REFERENCE


@pytest.mark.parametrize("kw", [
    dict(width=0, height=4, depth=4),
    dict(width=4, height=4, depth=2, geometry=1),
    dict(width=4, height=4, depth=4, alpha0=0.0),
    dict(width=4, height=4, depth=4, alpha1=-1.0),
    dict(width=4, height=4, depth=4, lambda_=-1.0),
    dict(width=4, height=4, depth=4, tau=0.0),
    dict(width=4, height=4, depth=4, data_term=7),
    dict(width=4, height=4, depth=4, state_precision=9),
    dict(width=4, height=4, depth=4, dct_mode=9),
    dict(width=4, height=4, depth=4, alpha0=float("nan")),
])
def test_create_rejects_bad_parameters_before_the_device(kw):
    p = pkg.default_params(**kw)
    ctx = ctypes.c_void_p()
    st = pkg.lib().tgvdct_create(ctypes.byref(p), ctypes.byref(ctx))
    assert st == pkg.ERR_BAD_ARG
    assert not ctx.value
    assert pkg.lib().tgvdct_last_error()


def test_null_arguments_are_rejected():
    lib = pkg.lib()
    assert lib.tgvdct_create(None, ctypes.byref(ctypes.c_void_p())) == pkg.ERR_BAD_ARG
    assert lib.tgvdct_tgv2_run_dev(None, None, None, None, None, None, pkg.CALLBACK(), None,
                                   None) == pkg.ERR_BAD_ARG
    assert lib.tgvdct_destroy(None) == pkg.OK


def test_status_strings():
    lib = pkg.lib()
    for s in range(7):
        assert lib.tgvdct_status_string(s)


def test_workspace_bytes_scale_with_precision():
    lib = pkg.lib()
    p32 = pkg.default_params(width=64, height=64, depth=64)
    p16 = pkg.default_params(width=64, height=64, depth=64, state_precision=pkg.STATE_FX16_DUAL)
    b32 = lib.tgvdct_workspace_bytes(ctypes.byref(p32))
    b16 = lib.tgvdct_workspace_bytes(ctypes.byref(p16))
    n = 64 ** 3
    # 3 + 6 FP32 (u, ubar, f, v, vbar) + 9 dual fields, plus the DCT plan
    assert b32 >= 18 * 4 * n and b16 >= (9 * 4 + 9 * 2) * n and b16 < b32


def test_bounds_check_needs_the_checked_build():
    """The normal library has no bounds checks compiled in and says so."""
    import ambient_image_processor_gb300 as pkg
    w = ctypes.c_uint64(0)
    assert pkg.lib().tgvdct_bounds_check(ctypes.byref(w)) == pkg.ERR_UNSUPPORTED


def test_release_cached_without_a_cached_context():
    """Nothing is cached before a host-buffer call: releasing needs no device."""
    import ambient_image_processor_gb300 as pkg
    assert pkg.lib().tgvdct_release_cached() == pkg.OK
    pkg.release_cached()
