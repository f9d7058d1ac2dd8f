"""The dask paths of calc_cape / calc_srh (one library call per chunk of
columns, core.py _calc_*_gufunc) with a stand-in for dask.array: dask is not
installed here, so `dask.array` is a small module whose Array marks the
inputs and whose apply_gufunc applies the function to chunks of columns the
way dask's does (core dimensions last, one call per chunk, outputs
concatenated).  It checks the plumbing -- signature arity, the pressure-level
binding of p, keyword forwarding, output count and dtypes -- against the
numpy path on the same arrays, and, with the chunks computed concurrently by
a pool of threads as dask's threaded scheduler computes them, the results
against the oracle: each concurrent chunk call takes its own host context
(streams, staging, workspace), so the chunks' copies and lifts overlap on
the GPU."""
import re
import sys
import types
from concurrent.futures import ThreadPoolExecutor

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


def _apply_gufunc_threaded(func, signature, *args, output_dtypes=None, vectorize=False,
                           **kwargs):
    """apply_gufunc with the chunks (8 along the first loop axis) computed
    by 4 threads at once, as dask's threaded scheduler does."""
    ins, outs = signature.split("->")
    in_core = re.findall(r"\(([^)]*)\)", ins)
    assert len(in_core) == len(args) and not vectorize
    arrs = [np.asarray(a) for a in args]
    n = arrs[-1].shape[0]
    bounds = np.linspace(0, n, 9).astype(int)
    with ThreadPoolExecutor(4) as pool:
        futs = [pool.submit(func, *[a[lo:hi] for a in arrs], **kwargs)
                for lo, hi in zip(bounds[:-1], bounds[1:]) if hi > lo]
        chunks = [f.result() for f in futs]
    return tuple(np.concatenate([c[k] for c in chunks]).astype(dt)
                 for k, dt in enumerate(output_dtypes))


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


@pytest.fixture
def threaded_dask(monkeypatch):
    da = types.ModuleType("dask.array")
    da.Array = _Array
    da.apply_gufunc = _apply_gufunc_threaded
    dask = types.ModuleType("dask")
    dask.array = da
    monkeypatch.setitem(sys.modules, "dask", dask)
    monkeypatch.setitem(sys.modules, "dask.array", da)
    return da


@pytest.mark.parametrize("source", ["most-unstable", "mixed-layer"])
def test_calc_cape_concurrent_chunks_match_oracle(threaded_dask, source):
    """8 chunks of a (64, 1024) pressure-level grid computed by 4 threads
    at once through the dask path: equal to the one-call numpy path bit for
    bit, and within the parity criteria of the oracle."""
    from gpu_util import compare_cape, oracle_cols
    args = S.pressure_c1(shape=(64, 1024), seed=11)
    want = X.calc_cape(*args, source=source, vertical_lev="pressure")
    dargs = [np.asarray(a).view(_Array) if i > 0 else np.asarray(a) for i, a in enumerate(args)]
    got = X.calc_cape(*dargs, source=source, vertical_lev="pressure")
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)
    ref = oracle_cols(2, *args, source, "pseudo-liquid", 500.0, 500.0)
    ref64 = oracle_cols(2, *args, source, "pseudo-liquid", 500.0, 500.0, precision="f64")
    g = {"cape": got[0].ravel(), "cin": got[1].ravel()}
    zero = (g["cape"] == 0) & (g["cin"] == 0)
    real_zero = ((ref["status"] & 1) == 0) & (ref["cape"] == 0) & (ref["cin"] == 0)
    g["status"] = np.where(zero & ~real_zero, 1, 0)  # the give-ups (no status on this path)
    compare_cape(g, ref, ref64, what=f"dask {source}")


def test_concurrent_host_calls_overlap_and_agree():
    """calc_cape on numpy arrays from 6 threads at once (more threads than
    host contexts, so some wait for one): every call's results equal the
    same call made alone, and the CAPE + SRH host paths interleave safely."""
    parts = [S.pressure_c1(shape=(32, 512), seed=40 + k) for k in range(6)]
    alone = [X.calc_cape(*a, source="most-unstable", vertical_lev="pressure") for a in parts]
    srh_args = S.srh_c2(shape=(32, 64), nlev=50, seed=5)
    srh_alone = X.calc_srh(*srh_args, depth=3000, vertical_lev="model")

    def work(k):
        if k == 6:
            return X.calc_srh(*srh_args, depth=3000, vertical_lev="model")
        return X.calc_cape(*parts[k], source="most-unstable", vertical_lev="pressure")
    with ThreadPoolExecutor(6) as pool:
        res = list(pool.map(work, range(7)))
    for got, want in zip(res[:6], alone):
        for g, w in zip(got, want):
            np.testing.assert_array_equal(g, w)
    for g, w in zip(res[6], srh_alone):
        np.testing.assert_array_equal(g, w)
