"""CPU tests of the host side: shapes, argument errors, and the C ABI surface.

The shape tests mirror the reference's test_calc_cape_shape_3d
(test/test_core.py:39-58), which drives the 'dummy' backend.  The ABI tests
load libxcape_gb300.so and check that every entry point declared in
include/xcape_gb300.h is exported; calls whose arguments are rejected return
before any CUDA work, so they run without a GPU.
"""
import ctypes
import os
import re

import numpy as np
import pytest

import xcape_gb300 as X
from xcape_gb300 import _lib
from xcape_gb300.core import calc_cape, calc_srh

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def p_t_td_3d():
    rng = np.random.default_rng(0)
    return tuple(rng.random((5, 10, 20)) for _ in range(3))


@pytest.fixture(scope="module")
def p_t_td_surface():
    rng = np.random.default_rng(1)
    return tuple(rng.random((5, 10)) for _ in range(3))


@pytest.mark.parametrize("sourcein,n_returns", [("surface", 2), ("most-unstable", 4)])
@pytest.mark.parametrize("vertical_levin", ["sigma", "pressure", "model"])
def test_calc_cape_shape_3d(p_t_td_3d, p_t_td_surface, sourcein, n_returns, vertical_levin):
    p, t, td = p_t_td_3d
    ps, ts, tds = p_t_td_surface
    if vertical_levin == "pressure":
        args = (np.ones(t.shape[-1]), t, td, ps, ts, tds)
    else:
        args = (p, t, td, ps, ts, tds)
    result = calc_cape(*args, source=sourcein, vertical_lev=vertical_levin, method="dummy")
    assert len(result) == n_returns
    for data in result:
        assert data.shape == p.shape[:-1]


def test_calc_cape_argument_errors(p_t_td_3d, p_t_td_surface):
    p, t, td = p_t_td_3d
    ps, ts, tds = p_t_td_surface
    with pytest.raises(ValueError, match="Too few"):
        calc_cape(p, t, td, ps, ts)
    with pytest.raises(ValueError, match="Too many"):
        calc_cape(p, t, td, ps, ts, tds, ps)
    with pytest.raises(ValueError, match="vertical_lev"):
        calc_cape(p, t, td, ps, ts, tds, vertical_lev="height")
    with pytest.raises(ValueError, match="P should be 1d"):
        calc_cape(p, t, td, ps, ts, tds, vertical_lev="pressure", method="dummy")
    with pytest.raises(ValueError, match="invalid method"):
        calc_cape(p, t, td, ps, ts, tds, vertical_lev="sigma", method="numba")
    with pytest.raises(ValueError, match="source"):
        calc_cape(p, t, td, ps, ts, tds, source="lifted", method="dummy")
    with pytest.raises(ValueError, match="adiabat"):
        calc_cape(p, t, td, ps, ts, tds, adiabat="dry", method="dummy")
    with pytest.raises(ValueError, match="same shape"):
        calc_cape(p[..., :5], t, td, ps, ts, tds, method="dummy")


def test_calc_srh_argument_errors(p_t_td_3d, p_t_td_surface):
    p, t, td = p_t_td_3d
    ps, ts, tds = p_t_td_surface
    with pytest.raises(ValueError, match="output_var"):
        calc_srh(p, t, td, t, td, ps, ts, tds, ps, ts, output_var="helicity")
    with pytest.raises(ValueError, match="P should be 1d"):
        calc_srh(p, t, td, t, td, ps, ts, tds, ps, ts, vertical_lev="pressure")


def test_fortran_method_needs_reference(p_t_td_3d, p_t_td_surface):
    p, t, td = p_t_td_3d
    ps, ts, tds = p_t_td_surface
    try:
        import xcape  # noqa: F401
        pytest.skip("reference xcape installed")
    except ImportError:
        pass
    with pytest.raises(ImportError, match="reference xcape"):
        calc_cape(p, t, td, ps, ts, tds, vertical_lev="sigma", method="fortran")


def _declared_entry_points():
    text = open(os.path.join(ROOT, "include", "xcape_gb300.h")).read()
    return sorted(set(re.findall(r"^(?:int|size_t|long long|const char \*)\s*(xc_\w+)\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    declared = _declared_entry_points()
    assert len(declared) >= 18
    for name in declared:
        assert hasattr(L, name), f"{name} declared in include/xcape_gb300.h but not exported"
    assert set(declared) == set(_lib.exported_symbols())
    assert "sm_103a" in X.version()


def test_invalid_arguments_return_status_without_gpu():
    L = _lib.lib()
    null = None
    # unknown source: the reference Fortran would `stop` (CAPE_CODE_model_lev.f90:343-351)
    rc = L.xc_loopcape_ml(null, null, null, null, null, null, 0, 500.0, 7, 500.0, 1, 10, 4,
                          null, null, null, null, null, null)
    assert rc == _lib.XC_ERR_INVALID
    assert b"source" in L.xc_last_error()
    # undefined adiabat (:492-497)
    rc = L.xc_loopcape_ml(null, null, null, null, null, null, 0, 500.0, 1, 500.0, 9, 10, 4,
                          null, null, null, null, null, null)
    assert rc == _lib.XC_ERR_INVALID and b"adiabat" in L.xc_last_error()
    # non-positive pressure increment
    rc = L.xc_loopcape_ml(null, null, null, null, null, null, 0, 0.0, 1, 500.0, 1, 10, 4,
                          null, null, null, null, null, null)
    assert rc == _lib.XC_ERR_INVALID
    # bad dtype / level count
    rc = L.xc_loopcape_ml(null, null, null, null, null, null, 5, 500.0, 1, 500.0, 1, 10, 4,
                          null, null, null, null, null, null)
    assert rc == _lib.XC_ERR_INVALID
    rc = L.xc_loopcape_ml(null, null, null, null, null, null, 0, 500.0, 1, 500.0, 1, 0, 4,
                          null, null, null, null, null, null)
    assert rc == _lib.XC_ERR_INVALID
    # grid 3 without start
    rc = L.xc_loopcape_pl(null, null, null, null, null, null, 0, 500.0, 1, 500.0, 1, null, 10, 4,
                          null, null, null, null, null, null)
    assert rc == _lib.XC_ERR_INVALID
    # zero columns is a no-op
    rc = L.xc_loopcape_ml(null, null, null, null, null, null, 0, 500.0, 1, 500.0, 1, 10, 0,
                          null, null, null, null, null, null)
    assert rc == _lib.XC_OK
    # rm/lm/mean6 must come together
    buf = ctypes.c_void_p(16)
    rc = L.xc_calc_srh(1, *([null] * 10), 0, null, 3000.0, 2.0, 10, 4, null, null, buf, null,
                       null, null)
    assert rc == _lib.XC_ERR_INVALID


def test_cape_srh_arguments_are_checked_before_any_cuda_call(p_t_td_3d, p_t_td_surface):
    """xc_cape_srh rejects what neither of its halves can run, with no GPU."""
    L = _lib.lib()
    null = None

    def call(grid=1, guess=0, precision=0, n2=4, rm=None, source=1):
        return L.xc_cape_srh(grid, *([null] * 10), 0, 500.0, source, 500.0, 1, null, 3000.0,
                             2.0, 10, n2, guess, precision, *([null] * 5), null, null, rm,
                             null, null, null, 0, null)
    assert call(grid=3) == _lib.XC_ERR_INVALID and b"grid" in L.xc_last_error()
    assert call(guess=_lib.XC_GUESS_EXTRAPOLATED) == _lib.XC_ERR_INVALID
    assert b"guess" in L.xc_last_error()
    assert call(precision=7) == _lib.XC_ERR_INVALID and b"precision" in L.xc_last_error()
    assert call(rm=ctypes.c_void_p(16)) == _lib.XC_ERR_INVALID
    assert call(source=5) == _lib.XC_ERR_INVALID and b"source" in L.xc_last_error()
    assert call(n2=0) == _lib.XC_OK
    assert call() == _lib.XC_ERR_INVALID and b"NULL" in L.xc_last_error()
    p, t, td = p_t_td_3d
    ps, ts, tds = p_t_td_surface
    with pytest.raises(ValueError, match="guess"):
        X.calc_cape_srh(p, t, td, t, td, ps, ts, tds, ps, ts, guess="secant")
    with pytest.raises(ValueError, match="P should be 1d"):
        X.calc_cape_srh(p, t, td, t, td, ps, ts, tds, ps, ts, vertical_lev="pressure")
    with pytest.raises(ValueError, match="precision"):
        X.calc_cape_srh(p, t, td, t, td, ps, ts, tds, ps, ts, precision="fp16")


def test_python_constants_match_the_header():
    """Every XC_* integer the Python layer mirrors has the header's value."""
    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                       "xcape_gb300.h")
    defines = dict(re.findall(r"^#define (XC_\w+) (-?\d+)", open(hdr).read(), re.M))
    mirrored = {k: getattr(_lib, k) for k in dir(_lib) if k.startswith("XC_") and
                isinstance(getattr(_lib, k), int)}
    assert len(mirrored) >= 10
    for k, v in mirrored.items():
        assert k in defines and int(defines[k]) == v, k
    for k in ("COL_NOCONV", "COL_BADSTART", "COL_TOOMANYSTEPS", "COL_FP64"):
        assert int(defines["XC_" + k]) == getattr(_lib, k), k


def test_empty_inputs_and_level_limit_without_gpu():
    """No columns: calc_cape / calc_srh return empty arrays of the right shape
    (the host entry points return before any CUDA call).  More levels than
    XC_MAX_LEVELS: the library refuses the call with a status, no work."""
    p = np.zeros((0, 37), np.float32)
    sf = np.zeros(0, np.float32)
    cape, cin, mulev, zmulev = calc_cape(p, p, p, sf, sf, sf, source="most-unstable")
    assert cape.shape == cin.shape == mulev.shape == zmulev.shape == (0,)
    srh_rm, srh_lm = calc_srh(p, p, p, p, p, sf, sf, sf, sf, sf)
    assert srh_rm.shape == srh_lm.shape == (0,)
    nk = _lib.XC_MAX_LEVELS + 1
    tall = np.zeros((2, nk), np.float32)
    with pytest.raises(_lib.XcapeError, match="nk="):
        calc_cape(tall, tall, tall, np.zeros(2, np.float32), np.ones(2, np.float32),
                  np.zeros(2, np.float32))


def test_python_raises_library_errors():
    with pytest.raises(_lib.XcapeError, match="status 1"):
        _lib.call("xc_loopcape_ml", None, None, None, None, None, None, 0, 500.0, 4, 500.0, 1,
                  10, 4, None, None, None, None, None, None)


def test_batch_arguments_are_checked_before_any_cuda_call():
    L = _lib.lib()
    h = ctypes.c_void_p()
    # capacity and solver checks come before the device is touched
    assert L.xc_batch_create(0, 1 << 20, 0, ctypes.byref(h)) == _lib.XC_ERR_INVALID
    assert L.xc_batch_create(16, 8, 0, ctypes.byref(h)) == _lib.XC_ERR_INVALID
    assert L.xc_batch_create(16, 1 << 20, _lib.XC_GUESS_SECANT, ctypes.byref(h)) == \
        _lib.XC_ERR_INVALID
    assert L.xc_batch_create(16, 1 << 20, 0, None) == _lib.XC_ERR_INVALID
    assert h.value is None
    assert L.xc_batch_run(None, None, 0, None) == _lib.XC_ERR_INVALID
    a, b = ctypes.c_longlong(), ctypes.c_longlong()
    assert L.xc_batch_work(None, ctypes.byref(a), ctypes.byref(b)) == _lib.XC_ERR_INVALID
    assert L.xc_batch_destroy(None) == _lib.XC_OK


def test_batch_request_descriptor_layout_matches_the_header():
    emul = pytest.importorskip("emul")
    if emul.nvcc() is None:
        pytest.skip("nvcc not available")
    out = (ctypes.c_longlong * 8)()
    emul.lib().emu_request_layout(out)
    R = _lib.CapeRequest
    assert list(out) == [ctypes.sizeof(R), R.n2.offset, R.ld.offset, R.p.offset, R.pinc.offset,
                         R.adiabat.offset, R.cape.offset, R.status.offset]


def test_plugin_stub_binds_the_library_without_a_gpu(monkeypatch):
    """The reference-side binding (xcape_gb300/plugin/cape_cuda.py, the file
    a maintainer copies into xcape) loads the library and declares the
    argument types of the two host entry points it calls; an argument the
    library rejects before any CUDA work comes back as RuntimeError."""
    import importlib.util
    from xcape_gb300 import _build
    monkeypatch.setenv("XCAPE_GB300_LIB", _build.build())
    spec = importlib.util.spec_from_file_location(
        "cape_cuda_stub", os.path.join(ROOT, "xcape_gb300", "plugin", "cape_cuda.py"))
    stub = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(stub)
    L = stub._lib()
    assert len(L.xc_loopcape_ex_host.argtypes) == len(_lib.SIGNATURES["xc_loopcape_ex_host"])
    assert len(L.xc_calc_srh_host.argtypes) == len(_lib.SIGNATURES["xc_calc_srh_host"])
    t2 = np.zeros((20, 4), np.float32)   # (nlev, ngrid), as the seam hands it over
    s1 = np.zeros(4, np.float32)
    with pytest.raises(RuntimeError, match="adiabat"):
        stub.cape(t2, t2, t2, s1, s1, s1, 0, 1, source=1, ml_depth=500.0, adiabat=7, pinc=500.0,
                  type_grid=1)
    with pytest.raises(ValueError, match="1-D pressure"):
        stub.cape(t2, t2, t2, s1, s1, s1, 0, 1, source=1, ml_depth=500.0, adiabat=1, pinc=500.0,
                  type_grid=2)
