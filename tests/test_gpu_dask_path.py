"""The dask paths of calc_cape / calc_srh (one library call per chunk of
columns, core.py _calc_*_gufunc) with a stand-in for dask.array: dask is not
installed here, so `dask.array` is a small module whose Array marks the
inputs and whose apply_gufunc applies the function to chunks of columns the
way dask's does (core dimensions last, one call per chunk, outputs
concatenated).  It checks the plumbing -- signature arity, the pressure-level
binding of p, keyword forwarding, output count and dtypes -- against the
numpy path on the same arrays."""
import re
import sys
import types

import numpy as np
import pytest

import xcape_gb300 as X
from xcape_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


class _Array(np.ndarray):
    pass


def _apply_gufunc(func, signature, *args, output_dtypes=None, vectorize=False, **kwargs):
    ins, outs = signature.split("->")
    in_core = re.findall(r"\(([^)]*)\)", ins)
    out_core = re.findall(r"\(([^)]*)\)", outs)
    assert len(in_core) == len(args), (signature, len(args))
    assert len(out_core) == len(output_dtypes)
    assert not vectorize
    arrs = [np.asarray(a) for a in args]
    loop_shape = arrs[-1].shape if not in_core[-1] else arrs[-1].shape[:-1]
    n = loop_shape[0]
    chunks = []
    for lo, hi in ((0, n // 3), (n // 3, n)):  # two chunks along the first loop axis
        chunks.append(func(*[a[lo:hi] for a in arrs], **kwargs))
    res = tuple(np.concatenate([c[k] for c in chunks]).astype(dt)
                for k, dt in enumerate(output_dtypes))
    return res


@pytest.fixture
def fake_dask(monkeypatch):
    da = types.ModuleType("dask.array")
    da.Array = _Array
    da.apply_gufunc = _apply_gufunc
    dask = types.ModuleType("dask")
    dask.array = da
    monkeypatch.setitem(sys.modules, "dask", dask)
    monkeypatch.setitem(sys.modules, "dask.array", da)
    return da


@pytest.mark.parametrize("vertical_lev", ["sigma", "pressure"])
@pytest.mark.parametrize("source", ["surface", "most-unstable"])
def test_calc_cape_dask_path(fake_dask, vertical_lev, source):
    if vertical_lev == "sigma":
        args = S.sigma_c0(shape=(6, 16), nlev=40, seed=3, dtype=np.float32)
    else:
        args = S.pressure_c1(shape=(6, 16), seed=3)
    want = X.calc_cape(*args, source=source, vertical_lev=vertical_lev)
    dargs = [np.asarray(a).view(_Array) if i > 0 or vertical_lev == "sigma" else np.asarray(a)
             for i, a in enumerate(args)]
    got = X.calc_cape(*dargs, source=source, vertical_lev=vertical_lev)
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert g.dtype == w.dtype
        np.testing.assert_array_equal(g, w)


@pytest.mark.parametrize("output_var", ["srh", "all"])
def test_calc_srh_dask_path(fake_dask, output_var):
    args = S.srh_c2(shape=(6, 16), nlev=50, seed=4)
    want = X.calc_srh(*args, depth=3000, vertical_lev="model", output_var=output_var)
    got = X.calc_srh(*[np.asarray(a).view(_Array) for a in args], depth=3000,
                     vertical_lev="model", output_var=output_var)
    assert len(got) == len(want)
    for g, w in zip(got, want):
        np.testing.assert_allclose(g, w, rtol=0, atol=0)
