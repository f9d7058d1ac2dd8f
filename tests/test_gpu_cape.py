"""GPU parity tests of the CAPE/CIN kernels against the CPU oracle and the
reference's golden vectors.

Mirrors test/test_core.py:68-170 of the reference (sigma and pressure golden
tests) and extends them to every source x adiabat on seeded synthetic
soundings, the three grid kinds, the ragged pressure-level start, edge cases
and the full 1,038,240-column pressure-level workload (through size-
independent properties plus a random sample checked column by column).
"""
import numpy as np
import pytest

import oracle as O
import xcape_gb300 as X
from xcape_gb300 import _lib
from xcape_gb300 import synthetic as S

from gpu_util import (ADIABATS, SOURCES, cape_device, compare_cape, oracle_cols, thetae_f64,
                      to_dev, torch_cuda)

pytestmark = pytest.mark.gpu

SIGMA_GOLDEN = [
    ("surface", 100, ("SB_CAPE_pinc100", "SB_CIN_pinc100")),
    ("mixed-layer", 1000, ("ML_CAPE_pinc1000_mldepth500", "ML_CIN_pinc1000_mldepth500")),
    ("most-unstable", 100, ("MU_CAPE_pinc100", "MU_CIN_pinc100", "MU_lv_pinc100", "MU_z_pinc100")),
]
PRESSURE_GOLDEN = [
    ("surface", ("sfc_capesp500", "sfc_cinsp500")),
    ("mixed-layer", ("sfc_capeml300p500", "sfc_cinml300p500")),
    ("most-unstable", ("sfc_capemup500", "sfc_cinmup500")),
]


def _close(got, want):
    np.testing.assert_almost_equal(got, want, 0)
    w = np.asarray(want, np.float64)
    assert np.all(np.abs(np.asarray(got, np.float64) - w) <= np.maximum(1.0, 1e-3 * np.abs(w)))


@pytest.mark.parametrize("use_torch", [False, True])
@pytest.mark.parametrize("source,pinc,keys", SIGMA_GOLDEN)
def test_cape_sigma_golden(soundings, source, pinc, keys, use_torch):
    s = soundings
    P, T, TD = s["pressure"], s["temperature"], s["dewpoint"]
    args = (P[:, 1:], T[:, 1:], TD[:, 1:], P[:, 0], T[:, 0], TD[:, 0])
    if use_torch:
        args = to_dev(*args)
    res = X.calc_cape(*args, source=source, ml_depth=500.0, adiabat="pseudo-liquid", pinc=pinc,
                      method="cuda", vertical_lev="sigma")
    assert len(res) == len(keys)
    res = [r.cpu().numpy() if use_torch else r for r in res]
    for got, key in zip(res, keys):
        if key.startswith("MU_lv"):
            assert got.dtype == np.int32
            np.testing.assert_array_equal(got, s[key].astype(np.int32))
        elif key.startswith("MU_z"):
            np.testing.assert_almost_equal(got, s[key], 0)
        else:
            assert got.dtype == np.float32
            _close(got, s[key])


@pytest.mark.parametrize("use_torch", [False, True])
@pytest.mark.parametrize("source,keys", PRESSURE_GOLDEN)
def test_cape_pressure_golden(era5, source, keys, use_torch):
    e = era5
    args = (e["lev_level"], e["lev_t"], e["lev_td"], e["sfc_p"], e["sfc_t"], e["sfc_td"])
    if use_torch:
        args = to_dev(*args)
    res = X.calc_cape(*args, source=source, ml_depth=300, adiabat="pseudo-liquid", pinc=500,
                      method="cuda", vertical_lev="pressure")
    res = [r.cpu().numpy() if use_torch else r for r in res]
    for got, key in zip(res, keys):
        _close(got, e[key])


_oracle_cols = oracle_cols


def _check_mulvl(got, want, p, t, td, ps, ts, tds, grid, start=None):
    same = got["mulvl"] == want["mulvl"]
    flip = ((got["status"] ^ want["status"]) & _lib.COL_NOCONV) != 0
    bad = np.nonzero(~same & ~flip)[0]
    if bad.size == 0:
        return
    # Near-ties: theta-e of the two chosen levels within 1e-3 K.
    nk = np.shape(t)[-1]
    t2, td2 = np.reshape(t, (-1, nk)), np.reshape(td, (-1, nk))
    for c in bad:
        def level(j):
            if j == 1:
                return np.ravel(ps)[c], np.ravel(ts)[c], np.ravel(tds)[c]
            m = (start[c] if start is not None else 1) - 3 + j
            pj = p[m] if grid == 2 else np.reshape(p, (-1, nk))[c, m]
            return pj, t2[c, m], td2[c, m]
        a = thetae_f64(*level(got["mulvl"][c]))
        b = thetae_f64(*level(want["mulvl"][c]))
        assert abs(a - b) < 1e-3, f"column {c}: MU level {got['mulvl'][c]} vs {want['mulvl'][c]}"
    assert bad.size <= max(2, 1e-3 * same.size)


@pytest.mark.parametrize("adiabat", list(ADIABATS))
@pytest.mark.parametrize("source", list(SOURCES))
def test_cape_sigma_synthetic_vs_oracle(source, adiabat):
    """64x64 columns x 40 sigma levels, float64 input (the small CPU case)."""
    p, t, td, ps, ts, tds = S.sigma_c0()
    got = cape_device(1, p, t, td, ps, ts, tds, source, adiabat, pinc=500.0, ml_depth=500.0)
    want = _oracle_cols(1, p, t, td, ps, ts, tds, source, adiabat, 500.0, 500.0)
    want64 = _oracle_cols(1, p, t, td, ps, ts, tds, source, adiabat, 500.0, 500.0,
                          precision="f64")
    compare_cape(got, want, want64, what=f"sigma {source} {adiabat}")
    if source == "most-unstable":
        _check_mulvl(got, want, p, t, td, ps, ts, tds, 1)
    else:
        assert np.all(got["mulvl"][ts.ravel() > 0] == -999999)


@pytest.mark.parametrize("adiabat", ["pseudo-liquid", "reversible-ice"])
@pytest.mark.parametrize("source", list(SOURCES))
def test_cape_pressure_synthetic_vs_oracle(source, adiabat):
    """Ragged pressure levels: 128x128 columns of the 1000..100 hPa workload,
    start level derived on the GPU."""
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(128, 128))
    got = cape_device(2, plev, t, td, ps, ts, tds, source, adiabat, pinc=500.0, ml_depth=500.0)
    want = _oracle_cols(2, plev, t, td, ps, ts, tds, source, adiabat, 500.0, 500.0)
    want64 = _oracle_cols(2, plev, t, td, ps, ts, tds, source, adiabat, 500.0, 500.0,
                          precision="f64")
    compare_cape(got, want, want64, what=f"pressure {source} {adiabat}")
    if source == "most-unstable":
        st = O.pres_lev_pos(plev, ps.ravel())
        _check_mulvl(got, want, plev, t, td, ps, ts, tds, 2, start=st)


@pytest.mark.parametrize("adiabat", list(ADIABATS))
@pytest.mark.parametrize("source", list(SOURCES))
def test_extrapolated_solver_vs_fp64(source, adiabat):
    """guess=XC_GUESS_EXTRAPOLATED (extrapolated first guess + secant steps,
    the reference's stopping test) against the FP64 oracle: as accurate as
    the plain FP32 iteration, none of its FP32 limit cycles, under 40 % of
    its iterations."""
    from gpu_util import BUOYANCY_TIE
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(96, 128))
    fast = cape_device(2, plev, t, td, ps, ts, tds, source, adiabat, guess=2, counters=True)
    plain = cape_device(2, plev, t, td, ps, ts, tds, source, adiabat, guess=0, counters=True)
    ref = _oracle_cols(2, plev, t, td, ps, ts, tds, source, adiabat, 500.0, 500.0,
                       precision="f64")
    conv64 = (ref["status"] & _lib.COL_NOCONV) == 0
    assert not np.any((fast["status"] & _lib.COL_NOCONV).astype(bool) & conv64)
    ok = conv64 & (fast["mulvl"] == ref["mulvl"])  # MU near-ties choose another parcel
    assert ok.mean() > 0.99
    d = np.abs(fast["cape"][ok].astype(np.float64) - ref["cape"][ok])
    assert np.all(d <= np.maximum(1.0, 1e-3 * np.abs(ref["cape"][ok]))), d.max()
    okc = ok & (ref["bmin"] >= BUOYANCY_TIE)
    d = np.abs(fast["cin"][okc].astype(np.float64) - ref["cin"][okc])
    assert np.all(d <= np.maximum(1.0, 1e-3 * np.abs(ref["cin"][okc]))), d.max()
    assert fast["niter_total"] < 0.4 * plain["niter_total"]


def test_cape_pressure_3d_grid_vs_oracle():
    """loopcape_pl: per-column pressure plus a given start level."""
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(32, 64))
    n2 = 32 * 64
    p3 = np.broadcast_to(plev, (n2, plev.size)).copy() * np.float32(1.0)
    p3 += np.random.default_rng(3).normal(0, 0.5, p3.shape).astype(np.float32)
    st = O.pres_lev_pos(plev, ps.ravel())
    got = cape_device(3, p3, t, td, ps, ts, tds, "mixed-layer", "pseudo-liquid", start=st)
    want = _oracle_cols(3, p3, t, td, ps, ts, tds, "mixed-layer", "pseudo-liquid", 500.0, 500.0,
                        start=st)
    compare_cape(got, want, what="pressure 3-D")


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_pres_lev_pos_kernel_matches_numpy(dtype):
    torch = torch_cuda()
    rng = np.random.default_rng(11)
    plev = np.array([1000, 975, 950, 950, 900, 850, 700, 500, 300, 100], dtype)
    ps = rng.uniform(800, 1050, 4096).astype(dtype)
    ps[:4] = [1000, 950, 899.99, 80]  # exact hit, tie, between, every level masked
    ps[4] = np.nan
    want = O.pres_lev_pos(plev, ps)
    P, PS = to_dev(plev, ps)
    st = torch.empty(ps.size, dtype=torch.int32, device="cuda")
    _lib.call("xc_pres_lev_pos", P.data_ptr(), PS.data_ptr(),
              _lib.XC_F64 if dtype == np.float64 else _lib.XC_F32, plev.size, ps.size,
              st.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(st.cpu().numpy(), want)


def test_cape_edge_cases():
    """Cold surface gate, short columns, MU above 500 hPa, single level,
    bad start, NaN input, one column."""
    p, t, td, ps, ts, tds = (np.array(a) for a in S.sigma_c0(shape=(1, 12), nlev=40, seed=4))
    p, t, td = p[0], t[0], td[0]
    ps, ts, tds = ps[0], ts[0], tds[0]
    ts[0] = -1.0          # ts <= 0: zeros, MU level 0 (CAPE_CODE_model_lev.f90:77-88)
    ts[1] = 0.0
    p[2] *= 0.45          # whole column above 500 hPa
    ps[2] *= 0.45
    t[3, :] = np.nan      # NaN column must finish with some status, not fault
    for source in SOURCES:
        got = cape_device(1, p, t, td, ps, ts, tds, source, "pseudo-liquid")
        want = _oracle_cols(1, p, t, td, ps, ts, tds, source, "pseudo-liquid", 500.0, 500.0)
        ok = np.ones(12, bool)
        ok[3] = False
        for key in ("cape", "cin", "mulvl"):
            np.testing.assert_allclose(got[key][ok], want[key][ok], rtol=1e-3, atol=1.0)
        assert got["cape"][0] == 0 and got["mulvl"][0] == 0 and got["z_out"][0] == 0
        assert got["cape"][1] == 0 and got["mulvl"][1] == 0
        if source == "most-unstable":
            assert got["mulvl"][2] == -999999
    # mixed layer deeper than the column: ascent never starts, sentinels stay
    got = cape_device(1, p[4:6, :2], t[4:6, :2], td[4:6, :2], ps[4:6], ts[4:6], tds[4:6],
                      "mixed-layer", "pseudo-liquid", ml_depth=5000.0)
    want = _oracle_cols(1, p[4:6, :2], t[4:6, :2], td[4:6, :2], ps[4:6], ts[4:6], tds[4:6],
                        "mixed-layer", "pseudo-liquid", 500.0, 5000.0)
    np.testing.assert_array_equal(got["cape"], want["cape"])
    np.testing.assert_array_equal(got["z_out"], want["z_out"])
    assert np.all(got["z_out"] == -999999.0)
    # a single 3-D level
    got = cape_device(1, p[:, :1], t[:, :1], td[:, :1], ps, ts, tds, "surface", "pseudo-liquid")
    want = _oracle_cols(1, p[:, :1], t[:, :1], td[:, :1], ps, ts, tds, "surface",
                        "pseudo-liquid", 500.0, 500.0)
    np.testing.assert_allclose(got["cape"][ok], want["cape"][ok], atol=1.0)
    # start outside 1..nk on the 3-D pressure grid: flagged, zeros (the
    # ts > 0 gate comes first, so a cold column stays unflagged)
    st = np.array([0, 1, 1, 1, 0, 41] + [1] * 6, np.int32)
    got = cape_device(3, p, t, td, ps, ts, tds, "surface", "pseudo-liquid", start=st)
    assert got["status"][4] & _lib.COL_BADSTART and got["status"][5] & _lib.COL_BADSTART
    assert got["cape"][4] == 0 and got["cape"][5] == 0 and got["status"][0] == 0


def test_host_and_device_paths_agree():
    torch = torch_cuda()
    p, t, td, ps, ts, tds = S.pressure_c1(shape=(48, 48))
    host = X.calc_cape(p, t, td, ps, ts, tds, source="most-unstable", vertical_lev="pressure")
    dev = X.calc_cape(*to_dev(p, t, td, ps, ts, tds), source="most-unstable",
                      vertical_lev="pressure")
    torch.cuda.synchronize()
    for h, d in zip(host, dev):
        np.testing.assert_array_equal(h, d.cpu().numpy())
        assert h.shape == (48, 48)


def test_work_counters_match_oracle():
    p, t, td, ps, ts, tds = S.sigma_c0(shape=(16, 64))
    got = cape_device(1, p, t, td, ps, ts, tds, "surface", "pseudo-liquid", counters=True)
    want = _oracle_cols(1, p, t, td, ps, ts, tds, "surface", "pseudo-liquid", 500.0, 500.0)
    assert got["nsub_total"] == int(want["nsub"].sum())
    assert abs(got["niter_total"] - int(want["niter"].sum())) <= 0.01 * want["niter"].sum()


def test_cape_full_size_pressure_workload():
    """1,038,240 columns x 37 levels (the benchmark workload): determinism,
    column-permutation invariance, and a random sample against the oracle."""
    torch = torch_cuda()
    plev, t, td, ps, ts, tds = S.pressure_c1()
    n2 = ps.size
    a = cape_device(2, plev, t, td, ps, ts, tds, "most-unstable", "pseudo-liquid")
    b = cape_device(2, plev, t, td, ps, ts, tds, "most-unstable", "pseudo-liquid")
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
    # the column ordering changes which warp computes a column, never its result
    u = cape_device(2, plev, t, td, ps, ts, tds, "most-unstable", "pseudo-liquid", order=False)
    for k in a:
        np.testing.assert_array_equal(a[k], u[k])
    perm = np.random.default_rng(5).permutation(n2)
    t2, td2 = t.reshape(n2, -1)[perm], td.reshape(n2, -1)[perm]
    c = cape_device(2, plev, t2, td2, ps.ravel()[perm], ts.ravel()[perm], tds.ravel()[perm],
                    "most-unstable", "pseudo-liquid")
    for k in a:
        np.testing.assert_array_equal(a[k][perm], c[k])
    idx = np.sort(np.random.default_rng(6).choice(n2, 4096, replace=False))
    want = _oracle_cols(2, plev, t.reshape(n2, -1)[idx], td.reshape(n2, -1)[idx],
                        ps.ravel()[idx], ts.ravel()[idx], tds.ravel()[idx], "most-unstable",
                        "pseudo-liquid", 500.0, 500.0)
    compare_cape({k: v[idx] for k, v in a.items()}, want, what="full-size sample")
    assert np.all(a["cape"] >= 0) and np.all(a["cin"] >= 0)
    del torch


def test_nonfinite_inputs_match_oracle():
    """NaN and infinite inputs on the GPU: every launch ends, NaN appears
    where the oracle's NaN is, finite results agree, and the only columns
    flagged too-many-sub-steps (bit 4, zero outputs) are ones with a NaN
    pressure, whose sub-step count the reference leaves undefined."""
    from cases import with_nonfinite
    p, t, td, ps, ts, tds = with_nonfinite()
    for source in ("surface", "most-unstable", "mixed-layer"):
        got = cape_device(1, p, t, td, ps, ts, tds, source, "pseudo-liquid")
        n2 = ps.size
        want = O.loopcape(p.reshape(n2, -1), t.reshape(n2, -1), td.reshape(n2, -1), ps.ravel(),
                          ts.ravel(), tds.ravel(), 500.0, SOURCES[source], 500.0, 1, stats=True)
        flagged = (got["status"] & 4) != 0
        nan_p = np.isnan(p.reshape(n2, -1)).any(axis=1) | np.isnan(ps.ravel())
        assert np.all(nan_p[flagged])
        keep = ~flagged & ((want["status"] & 1) == 0) & ((got["status"] & 1) == 0)
        for k in ("cape", "cin"):
            g, w = got[k][keep], want[k][keep]
            assert np.array_equal(np.isnan(g), np.isnan(w)), k
            fin = ~np.isnan(w)
            assert np.all(np.abs(g[fin].astype(np.float64) - w[fin]) <=
                          np.maximum(1.0, 1e-3 * np.abs(w[fin]))), k


@pytest.mark.parametrize("guess", [0, 1])
def test_tall_columns(guess):
    """1,000 sigma levels per column (the 4,096-level limit's order of
    magnitude; ~2,000 sub-steps per column): plain solver against the FP32
    oracle, learned solver against FP64."""
    from xcape_gb300 import guess as G
    if guess == 1:
        G.ensure_loaded()
    p, t, td, ps, ts, tds = S.sigma_c0(shape=(4, 64), nlev=1000, seed=17, dtype=np.float32)
    got = cape_device(1, p, t, td, ps, ts, tds, "surface", "pseudo-liquid", guess=guess)
    n2 = ps.size
    want = O.loopcape(p.reshape(n2, -1), t.reshape(n2, -1), td.reshape(n2, -1), ps.ravel(),
                      ts.ravel(), tds.ravel(), 500.0, 1, 500.0, 1, stats=True,
                      precision="f32" if guess == 0 else "f64")
    ok = ((want["status"] & 1) == 0) & ((got["status"] & 1) == 0)
    assert ok.mean() > 0.95
    d = np.abs(got["cape"][ok].astype(np.float64) - want["cape"][ok])
    assert np.all(d <= np.maximum(1.0, 1e-3 * want["cape"][ok])), d.max()


@pytest.mark.parametrize("ring,chunks,streams,copies", [(None, None, None, None),
                                                         ("1", None, None, "0"),
                                                         (None, "2", "1", "3"),
                                                         ("1", "3", "3", "7")])
@pytest.mark.parametrize("guess", ["plain", "learned"])
def test_host_path_chunks_match_device_path(guess, ring, chunks, streams, copies, monkeypatch):
    """numpy inputs go through the pipelined host entry point (chunks of
    131,072+ columns, their inputs copied on one stream, their lifts on two
    in turn, their outputs moved into the caller's arrays by the copy
    threads); the results equal those of the device entry point on the same
    arrays, bit for bit, whatever the pipelining: with XC_HOST_RING_BYTES=1
    the three chunks share two device slots, so the third reuses the first's
    buffers and staging; XC_HOST_CHUNKS and XC_HOST_STREAMS change the chunk
    count and the compute streams, XC_HOST_COPY_THREADS the output copies'
    split (0: the calling thread copies)."""
    import torch
    for name, val in (("XC_HOST_RING_BYTES", ring), ("XC_HOST_CHUNKS", chunks),
                      ("XC_HOST_STREAMS", streams), ("XC_HOST_COPY_THREADS", copies)):
        if val is not None:
            monkeypatch.setenv(name, val)
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(216, 1440))  # 311,040 columns: 3 chunks
    host = X.calc_cape(plev, t, td, ps, ts, tds, source="most-unstable",
                       vertical_lev="pressure", guess=guess)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (plev, t, td, ps, ts, tds)]
    ref = X.calc_cape(*dev, source="most-unstable", vertical_lev="pressure", guess=guess)
    torch.cuda.synchronize()
    for h, d in zip(host, ref):
        np.testing.assert_array_equal(h, d.cpu().numpy())


@pytest.mark.parametrize("ring", [None, "1"])
@pytest.mark.parametrize("guess", ["plain", "learned"])
def test_calc_cape_sources_one_upload(guess, ring, monkeypatch):
    """calc_cape_sources (xc_loopcape_multi_host): the three sources of the
    same columns from one upload of the inputs.  Each source's results equal
    a calc_cape call of its own bit for bit (the same kernels on the same
    columns, one ordering shared by the sources), over three chunks, also
    when the chunks share two device slots (XC_HOST_RING_BYTES=1); the plain
    solver's results meet the parity criteria against the oracle."""
    if ring is not None:
        monkeypatch.setenv("XC_HOST_RING_BYTES", ring)
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(216, 1440), seed=4)  # 311,040 columns
    names = ["mixed-layer", "surface", "most-unstable"]
    got = X.calc_cape_sources(plev, t, td, ps, ts, tds, sources=names, vertical_lev="pressure",
                              guess=guess)
    assert list(got) == names
    for name in names:
        single = X.calc_cape(plev, t, td, ps, ts, tds, source=name, vertical_lev="pressure",
                             guess=guess)
        assert len(got[name]) == len(single) == (4 if name == "most-unstable" else 2)
        for a, b in zip(got[name], single):
            assert a.shape == (216, 1440)
            np.testing.assert_array_equal(a, b)
    if guess == "plain":
        n = 8192  # a strided sample of the grid against the oracle
        idx = np.arange(n) * (ps.size // n)
        sub = [np.reshape(a, (ps.size, -1))[idx] for a in (t, td)] + \
              [np.ravel(a)[idx] for a in (ps, ts, tds)]
        for name in names:
            want = oracle_cols(2, plev, *sub, name, "pseudo-liquid", 500.0, 500.0)
            g = {"cape": got[name][0].ravel()[idx], "cin": got[name][1].ravel()[idx]}
            # the host path returns no status: a zero pair where the oracle's
            # is not the reference's give-up is a convergence flip
            zero = (g["cape"] == 0) & (g["cin"] == 0)
            real_zero = ((want["status"] & 1) == 0) & (want["cape"] == 0) & (want["cin"] == 0)
            g["status"] = np.where(zero & ~real_zero, 1, 0)
            compare_cape(g, want, what=f"calc_cape_sources {name}")


@pytest.mark.parametrize("guess", ["plain", "learned"])
def test_loopcape_multi_device(guess):
    """xc_loopcape_multi on device arrays (calc_cape_sources with CUDA
    tensors): one ordering of the columns serves the three sources.  Each
    source's outputs equal an xc_loopcape_ex call of its own bit for bit, the
    work counters are the sum of the three calls' counters, and with
    XC_RETRY_FP64 the retries, which reuse the ordering workspace, follow all
    three lifts and give the single calls' results too."""
    import ctypes
    import torch
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(96, 512), seed=8)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (plev, t, td, ps, ts, tds)]
    names = ["mixed-layer", "surface", "most-unstable"]
    gs = {"plain": _lib.XC_GUESS_PLAIN, "learned": _lib.XC_GUESS_LEARNED}[guess]
    if guess == "learned":
        from xcape_gb300 import guess as G
        G.ensure_loaded()
    got = X.calc_cape_sources(*dev, sources=names, vertical_lev="pressure", guess=guess)
    for name in names:
        single = X.calc_cape(*dev, source=name, vertical_lev="pressure", guess=guess)
        for a, b in zip(got[name], single):
            np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())
    n2, nk = ps.size, t.shape[-1]
    codes = [SOURCES[n] for n in names]
    ws_bytes = _lib.workspace_bytes(n2)
    wsbuf = torch.empty(ws_bytes + 256, dtype=torch.uint8, device="cuda")
    ws = wsbuf.data_ptr() + (-wsbuf.data_ptr()) % 256
    stream = torch.cuda.current_stream().cuda_stream
    ptrs = [x.data_ptr() for x in dev]

    def outputs(n):
        return ([torch.empty(n, dtype=torch.float32, device="cuda") for _ in range(3)] +
                [torch.empty(n, dtype=torch.int32, device="cuda") for _ in range(2)])

    for g in (gs, gs | _lib.XC_RETRY_FP64):
        cape, cin, zout, mulvl, status = outputs(3 * n2)
        cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
        arr = (ctypes.c_int * 3)(*codes)
        _lib.call("xc_loopcape_multi", 2, *ptrs, _lib.XC_F32, 500.0, 3,
                  ctypes.cast(arr, ctypes.c_void_p), 500.0, 1, None, nk, n2, g, cape.data_ptr(),
                  cin.data_ptr(), mulvl.data_ptr(), zout.data_ptr(), status.data_ptr(),
                  cnt.data_ptr(), ws, ws_bytes, stream)
        total = torch.zeros(2, dtype=torch.int64, device="cuda")
        for j, code in enumerate(codes):
            o = outputs(n2)
            c1 = torch.zeros(2, dtype=torch.int64, device="cuda")
            _lib.call("xc_loopcape_ex", 2, *ptrs, _lib.XC_F32, 500.0, code, 500.0, 1, None, nk,
                      n2, g, o[0].data_ptr(), o[1].data_ptr(), o[3].data_ptr(), o[2].data_ptr(),
                      o[4].data_ptr(), c1.data_ptr(), ws, ws_bytes, stream)
            total += c1
            sl = slice(j * n2, (j + 1) * n2)
            for a, b in zip((cape, cin, zout, mulvl, status), o):
                np.testing.assert_array_equal(a[sl].cpu().numpy(), b.cpu().numpy())
        np.testing.assert_array_equal(cnt.cpu().numpy(), total.cpu().numpy())
    with pytest.raises(_lib.XcapeError, match="nsrc"):
        _lib.call("xc_loopcape_multi", 2, *ptrs, _lib.XC_F32, 500.0, 4,
                  ctypes.cast(arr, ctypes.c_void_p), 500.0, 1, None, nk, n2, gs, cape.data_ptr(),
                  cin.data_ptr(), mulvl.data_ptr(), zout.data_ptr(), None, None, ws, ws_bytes,
                  stream)


@pytest.mark.parametrize("adiabat", ["pseudo-liquid", "reversible-ice"])
def test_loopcape_multi_device_sigma_f64(adiabat):
    """xc_loopcape_multi on the sigma grid with float64 CUDA tensors (the
    small CPU case, 64 x 64 columns x 40 levels): every source equals its
    own calc_cape call bit for bit, with the plain and the learned solver."""
    import torch
    p, t, td, ps, ts, tds = S.sigma_c0()
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (p, t, td, ps, ts, tds)]
    names = ["most-unstable", "mixed-layer", "surface"]
    for guess in ("plain", "learned"):
        got = X.calc_cape_sources(*dev, sources=names, adiabat=adiabat, vertical_lev="sigma",
                                  guess=guess)
        for name in names:
            single = X.calc_cape(*dev, source=name, adiabat=adiabat, vertical_lev="sigma",
                                 guess=guess)
            assert len(got[name]) == len(single)
            for a, b in zip(got[name], single):
                np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())


def test_calc_cape_sources_arguments():
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(4, 8))
    with pytest.raises(ValueError, match="at most once"):
        X.calc_cape_sources(plev, t, td, ps, ts, tds, sources=["surface", "surface"],
                            vertical_lev="pressure")
    with pytest.raises(ValueError, match="source"):
        X.calc_cape_sources(plev, t, td, ps, ts, tds, sources=["lifted"], vertical_lev="pressure")


@pytest.mark.parametrize("source", ["surface", "most-unstable", "mixed-layer"])
@pytest.mark.parametrize("adiabat", ["pseudo-liquid", "reversible-ice"])
def test_fp64_retry_of_given_up_columns(source, adiabat):
    """XC_RETRY_FP64 with the plain solver (the reference's iteration) on the
    noisy pressure-level workload, where FP32 rounding makes the iteration
    give up on a few percent of the columns.  Exactly those columns are
    lifted again in double precision (XC_COL_FP64), and then match the FP64
    oracle within max(1 J/kg, 0.1 %); every other column is bit for bit what
    the lift without the retry gives.  With and without the ordering
    workspace (the retry then scans every column's status instead of a
    compacted list)."""
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(96, 128), seed=6)
    base = cape_device(2, plev, t, td, ps, ts, tds, source, adiabat, guess=0)
    gave_up = (base["status"] & _lib.COL_NOCONV) != 0
    assert gave_up.sum() >= 20  # the workload exercises the retry
    ref = oracle_cols(2, plev, t, td, ps, ts, tds, source, adiabat, 500.0, 500.0,
                      precision="f64")
    for order in (True, False):
        got = cape_device(2, plev, t, td, ps, ts, tds, source, adiabat,
                          guess=_lib.XC_GUESS_PLAIN | _lib.XC_RETRY_FP64, order=order)
        retried = (got["status"] & _lib.COL_FP64) != 0
        np.testing.assert_array_equal(retried, gave_up)
        for k in ("cape", "cin", "z_out", "mulvl", "status"):
            np.testing.assert_array_equal(got[k][~retried], base[k][~retried])
        conv64 = (ref["status"] & _lib.COL_NOCONV) == 0
        np.testing.assert_array_equal((got["status"][retried] & _lib.COL_NOCONV) != 0,
                                      ~conv64[retried])
        ok = retried & conv64
        assert ok.sum() >= 0.9 * retried.sum()  # FP64 converges on nearly all of them
        for k in ("cape", "cin"):
            w = ref[k][ok]
            d = np.abs(got[k][ok].astype(np.float64) - w)
            assert np.all(d <= np.maximum(1.0, 1e-3 * np.abs(w))), (k, d.max())
        np.testing.assert_array_equal(got["mulvl"][ok], ref["mulvl"][ok])


def test_fp64_retry_through_the_public_api():
    """calc_cape(..., fp64_retry=True) on numpy (the host pipeline, three
    chunks) and on CUDA tensors gives the same results, and no column is
    left at the reference's give-up zeros where FP64 converges."""
    import torch
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(216, 1440), seed=8)
    host = X.calc_cape(plev, t, td, ps, ts, tds, source="most-unstable", vertical_lev="pressure",
                       fp64_retry=True)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (plev, t, td, ps, ts, tds)]
    devr = X.calc_cape(*dev, source="most-unstable", vertical_lev="pressure", fp64_retry=True)
    torch.cuda.synchronize()
    for h, d in zip(host, devr):
        np.testing.assert_array_equal(h, d.cpu().numpy())
    plain = X.calc_cape(plev, t, td, ps, ts, tds, source="most-unstable", vertical_lev="pressure")
    changed = host[0] != plain[0]
    assert changed.sum() > 100
    assert np.all(plain[0][changed] == 0)  # only the give-ups changed
    n = 4096
    idx = np.flatnonzero(changed.ravel())[:n]
    sub = [np.reshape(a, (ps.size, -1))[idx] for a in (t, td)] + \
          [np.ravel(a)[idx] for a in (ps, ts, tds)]
    ref = oracle_cols(2, plev, *sub, "most-unstable", "pseudo-liquid", 500.0, 500.0,
                      precision="f64")
    d = np.abs(host[0].ravel()[idx].astype(np.float64) - ref["cape"])
    assert np.all(d <= np.maximum(1.0, 1e-3 * np.abs(ref["cape"])))
    srcs = X.calc_cape_sources(plev, t, td, ps, ts, tds, sources=["most-unstable"],
                               vertical_lev="pressure", fp64_retry=True)
    for a, b in zip(srcs["most-unstable"], host):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("guess", ["extrapolated", "learned"])
def test_surface_on_a_pressure_level(guess):
    """ps exactly on a pressure level (the first sub-step has no pressure
    drop): the accelerated solvers stay finite and within their FP64
    contract on every column."""
    from gpu_util import check_vs_fp64
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(64, 128), seed=17)
    ps = ps.copy().ravel()
    ps[::2] = plev[np.arange(ps.size // 2) % 12].astype(ps.dtype)
    code = {"extrapolated": _lib.XC_GUESS_EXTRAPOLATED, "learned": _lib.XC_GUESS_LEARNED}[guess]
    if code == _lib.XC_GUESS_LEARNED:
        from xcape_gb300 import guess as G
        G.ensure_loaded()
    for source in ("surface", "most-unstable", "mixed-layer"):
        got = cape_device(2, plev, t, td, ps, ts, tds, source, "pseudo-liquid", guess=code)
        assert np.all(np.isfinite(got["cape"])) and np.all(np.isfinite(got["cin"]))
        ref = oracle_cols(2, plev, t, td, ps, ts, tds, source, "pseudo-liquid", 500.0, 500.0,
                          precision="f64")
        check_vs_fp64(got, ref, what=f"{guess} {source}")
