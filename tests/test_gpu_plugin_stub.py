"""GPU tests of the reference-side binding ``xcape_gb300/plugin/cape_cuda.py``:
the module a maintainer drops into xcape as ``src/xcape/cape_cuda.py``.

The stub is fed exactly what xcape's own seams hand to its Fortran: the
arrays reshaped by ``_reshape_inputs`` / ``_reshape_surface_inputs``
(``src/xcape/core.py:31-50, 81-100``) into ``(nlev, ngrid)`` transposed views
and ``(ngrid,)`` vectors, ``p_2d`` of shape ``(nlev, 1)`` with the 1-based
``pres_lev_pos`` of ``core.py:286-289`` for pressure levels, the integer 1
for sigma levels, and the option codes of ``core.py:302-311``.  Its results,
reshaped back by the seam's ``_reshape_outputs`` rule (``core.py:52-63``),
are checked against the reference's golden vectors and the oracle.
"""
import importlib.util
import os
from functools import reduce

import numpy as np
import pytest

import oracle as O
from xcape_gb300 import _build
from xcape_gb300 import synthetic as S

from gpu_util import compare_cape, oracle_cols

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STUB = os.path.join(ROOT, "xcape_gb300", "plugin", "cape_cuda.py")

_SOURCE = {"surface": 1, "most-unstable": 2, "mixed-layer": 3}
_ADIABAT = {"pseudo-liquid": 1, "reversible-liquid": 2, "pseudo-ice": 3, "reversible-ice": 4}
_GRID = {"sigma": 1, "pressure": 2}


@pytest.fixture(scope="module")
def stub():
    """The stub imported from its file, bound to the in-tree library."""
    os.environ["XCAPE_GB300_LIB"] = _build.build()
    spec = importlib.util.spec_from_file_location("cape_cuda", STUB)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


# ---- the seam: what xcape's core.py hands to its compiled code ---------------

def _reshape_inputs(*args):
    """core.py:31-50: (..., nlev) -> (nlev, npoints) transposed views."""
    args = [np.atleast_2d(a) for a in args]
    shape = args[0].shape
    new = (reduce(lambda x, y: x * y, shape[:-1]), shape[-1])
    return [np.reshape(a, new).transpose() for a in args]


def _reshape_surface_inputs(*args):
    """core.py:81-100: (...) -> (npoints,)."""
    args = [np.atleast_1d(a) for a in args]
    n = reduce(lambda x, y: x * y, args[0].shape)
    return [np.reshape(a, (n,)) for a in args]


def _reshape_outputs(*args, shape):
    """core.py:52-63."""
    target = (1,) if len(shape) == 1 else shape[:-1]
    return [np.reshape(a.transpose(), target) for a in args]


def _seam(p, level_arrays, surface_arrays, vertical_lev):
    """core.py:278-300 / :489-506: the 2-D views, flag_1d and pres_lev_pos."""
    surf = _reshape_surface_inputs(*surface_arrays)
    if np.ndim(p) == 1:
        lev = _reshape_inputs(*level_arrays)
        p_2d = _reshape_inputs(p)[0]
        pres_lev_pos = np.ma.masked_less(surf[0] - p_2d, 0).argmin(axis=0) + 1
        return p_2d, lev, surf, 1, pres_lev_pos
    p_2d, *lev = _reshape_inputs(p, *level_arrays)
    return p_2d, lev, surf, 0, 1


def _cape_via_stub(stub, p, t, td, ps, ts, tds, source, ml_depth, adiabat, pinc, vertical_lev):
    p_2d, (t_2d, td_2d), (ps1, ts1, tds1), flag_1d, plp = _seam(p, (t, td), (ps, ts, tds),
                                                               vertical_lev)
    assert t_2d.shape == (np.shape(t)[-1], ps1.size)
    out = stub.cape(p_2d, t_2d, td_2d, ps1, ts1, tds1, flag_1d, plp, source=_SOURCE[source],
                    ml_depth=ml_depth, adiabat=_ADIABAT[adiabat], pinc=pinc,
                    type_grid=_GRID[vertical_lev])
    return _reshape_outputs(*out, shape=np.shape(t))


def _close(got, want):
    np.testing.assert_almost_equal(got, want, 0)
    w = np.asarray(want, np.float64)
    assert np.all(np.abs(np.asarray(got, np.float64) - w) <= np.maximum(1.0, 1e-3 * np.abs(w)))


@pytest.mark.parametrize("source,pinc,keys", [
    ("surface", 100, ("SB_CAPE_pinc100", "SB_CIN_pinc100")),
    ("mixed-layer", 1000, ("ML_CAPE_pinc1000_mldepth500", "ML_CIN_pinc1000_mldepth500")),
    ("most-unstable", 100, ("MU_CAPE_pinc100", "MU_CIN_pinc100", "MU_lv_pinc100",
                            "MU_z_pinc100")),
])
def test_stub_cape_sigma_golden(stub, soundings, source, pinc, keys):
    s = soundings
    P, T, TD = s["pressure"], s["temperature"], s["dewpoint"]
    res = _cape_via_stub(stub, P[:, 1:], T[:, 1:], TD[:, 1:], P[:, 0], T[:, 0], TD[:, 0],
                         source, 500.0, "pseudo-liquid", pinc, "sigma")
    for k, key in enumerate(keys):
        if key.startswith("MU_lv"):
            np.testing.assert_array_equal(res[2], s[key].astype(np.int32))
        elif key.startswith("MU_z"):
            np.testing.assert_almost_equal(res[3], s[key], 0)
        else:
            _close(res[k], s[key])


@pytest.mark.parametrize("source,keys", [
    ("surface", ("sfc_capesp500", "sfc_cinsp500")),
    ("mixed-layer", ("sfc_capeml300p500", "sfc_cinml300p500")),
    ("most-unstable", ("sfc_capemup500", "sfc_cinmup500")),
])
def test_stub_cape_pressure_golden(stub, era5, source, keys):
    e = era5
    res = _cape_via_stub(stub, e["lev_level"], e["lev_t"], e["lev_td"], e["sfc_p"], e["sfc_t"],
                         e["sfc_td"], source, 300.0, "pseudo-liquid", 500.0, "pressure")
    for k, key in enumerate(keys):
        _close(res[k], e[key])


@pytest.mark.parametrize("adiabat", ["pseudo-liquid", "reversible-ice"])
@pytest.mark.parametrize("source", ["surface", "most-unstable", "mixed-layer"])
def test_stub_cape_pressure_synthetic_vs_oracle(stub, source, adiabat):
    """A (64, 96) grid of the ragged 1000..100 hPa workload through the
    stub, against the oracle on the same columns."""
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(64, 96), seed=12)
    res = _cape_via_stub(stub, plev, t, td, ps, ts, tds, source, 500.0, adiabat, 500.0,
                         "pressure")
    assert res[0].shape == (64, 96)
    want = oracle_cols(2, plev, t, td, ps, ts, tds, source, adiabat, 500.0, 500.0)
    want64 = oracle_cols(2, plev, t, td, ps, ts, tds, source, adiabat, 500.0, 500.0,
                         precision="f64")
    # The stub returns what f2py returns, without a status.  A column the
    # reference's iteration gave up on returns CAPE = CIN = 0 (:471-473);
    # where the oracle's result is not that zero, the GPU's zero pair is
    # such a give-up, i.e. a convergence flip, which compare_cape counts.
    zero = (res[0].ravel() == 0) & (res[1].ravel() == 0)
    real_zero = ((want["status"] & O.COL_NOCONV) == 0) & (want["cape"] == 0) & (want["cin"] == 0)
    got = {"cape": res[0].ravel(), "cin": res[1].ravel(),
           "status": np.where(zero & ~real_zero, O.COL_NOCONV, 0)}
    compare_cape(got, want, want64, what=f"stub {source} {adiabat}")


@pytest.mark.parametrize("output", [1, 2])
def test_stub_srh_sigma_golden(stub, soundings, output):
    s = soundings
    P, T, TD, U, V = (s[k] for k in ("pressure", "temperature", "dewpoint", "u_wind_ms",
                                      "v_wind_ms"))
    p_2d, lev, surf, flag_1d, plp = _seam(P[:, 1:], (T[:, 1:], TD[:, 1:], U[:, 1:], V[:, 1:]),
                                         (P[:, 0], T[:, 0], TD[:, 0], U[:, 0], V[:, 0]),
                                         "sigma")
    out = stub.srh_chain(p_2d, *lev, *surf, flag_1d, plp, 3000, type_grid=1, output=output)
    srh_rm, srh_lm = _reshape_outputs(out[0], out[1], shape=T[:, 1:].shape)
    np.testing.assert_almost_equal(srh_rm, s["SRH03_model_lev_rm"], 5)
    np.testing.assert_almost_equal(srh_lm, s["SRH03_model_lev_lm"], 5)
    if output == 2:
        want = O.calc_srh(P[:, 1:], T[:, 1:], TD[:, 1:], U[:, 1:], V[:, 1:], P[:, 0], T[:, 0],
                          TD[:, 0], U[:, 0], V[:, 0], depth=3000, vertical_lev="sigma",
                          output_var="all")
        for vec, (wu, wv) in zip(out[2:], ((want[2], want[3]), (want[4], want[5]),
                                          (want[6], want[7]))):
            assert vec.shape == (2, T.shape[0])
            np.testing.assert_allclose(vec[0], wu, atol=1e-4)
            np.testing.assert_allclose(vec[1], wv, atol=1e-4)


def test_stub_srh_pressure_golden(stub, era5):
    e = era5
    p_2d, lev, surf, flag_1d, plp = _seam(
        e["lev_level"], (e["lev_t"], e["lev_td"], e["lev_u"], e["lev_v"]),
        (e["sfc_p"], e["sfc_t"], e["sfc_td"], e["sfc_u"], e["sfc_v"]), "pressure")
    srh_rm, srh_lm = stub.srh_chain(p_2d, *lev, *surf, flag_1d, plp, 3000, type_grid=2,
                                    output=1)
    np.testing.assert_almost_equal(srh_rm, e["sfc_srh_rm"], 5)
    np.testing.assert_almost_equal(srh_lm, e["sfc_srh_lm"], 5)


def test_stub_reports_library_errors(stub, soundings):
    s = soundings
    P, T, TD = s["pressure"], s["temperature"], s["dewpoint"]
    p_2d, (t_2d, td_2d), surf, flag_1d, plp = _seam(P[:, 1:], (T[:, 1:], TD[:, 1:]),
                                                   (P[:, 0], T[:, 0], TD[:, 0]), "sigma")
    with pytest.raises(RuntimeError, match="adiabat"):
        stub.cape(p_2d, t_2d, td_2d, *surf, flag_1d, plp, source=1, ml_depth=500.0, adiabat=9,
                  pinc=500.0, type_grid=1)
