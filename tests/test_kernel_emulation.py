"""CPU checks of the CUDA kernels' column routines.

tests/emul builds cape_column.cuh and srh_column.cuh -- the code every CUDA
thread runs -- as host code with glibc math and no FMA contraction.  Run that
way it must reproduce the oracle bit for bit: same operations, same order,
same rounding.  This pins the kernels' logic (level offsets, the one-pass
mixed layer, the upward Bunkers sweep, ragged start levels, edge cases) on
the CPU; the GPU tests then only have to account for CUDA's own expf/logf/
powf rounding and FMA contraction.
"""
import shutil

import numpy as np
import pytest

import oracle as O
from xcape_gb300 import synthetic as S

from cases import with_nonfinite

emul = pytest.importorskip("emul")
if emul.nvcc() is None:
    pytest.skip("nvcc not available", allow_module_level=True)

SOURCES = (1, 2, 3)
ADIABATS = (1, 2, 3, 4)


def _emu_cape(grid, p, t, td, ps, ts, tds, source, adiabat, pinc=500.0, ml_depth=500.0,
              start=None, guess=0, guess_w=None, diag=False):
    L = emul.lib()
    f64 = any(np.asarray(a).dtype == np.float64 for a in (p, t, td, ps, ts, tds))
    dt = np.float64 if f64 else np.float32
    t = np.ascontiguousarray(t, dt)
    nk = t.shape[-1]
    n2 = t.size // nk
    arrs = [np.ascontiguousarray(a, dt) for a in (p, t, td, ps, ts, tds)]
    st = None if start is None else np.ascontiguousarray(start, np.int32)
    out = dict(cape=np.empty(n2, np.float32), cin=np.empty(n2, np.float32),
               mulvl=np.empty(n2, np.int32), z_out=np.empty(n2, np.float32),
               status=np.empty(n2, np.int32))
    cnt = np.zeros(2, np.int64)
    gw = None if guess_w is None else np.ascontiguousarray(guess_w, np.float32)
    dg = np.zeros((n2, 6), np.float32) if diag else None
    L.emu_cape(grid, *[a.ctypes.data for a in arrs], int(f64), pinc, source, ml_depth, adiabat,
               None if st is None else st.ctypes.data, nk, n2, out["cape"].ctypes.data,
               out["cin"].ctypes.data, out["mulvl"].ctypes.data, out["z_out"].ctypes.data,
               out["status"].ctypes.data, cnt.ctypes.data, guess,
               None if gw is None else gw.ctypes.data, dg.ctypes.data if dg is not None else None)
    out["counters"] = cnt
    if dg is not None:
        out.update({k: dg[:, j] for j, k in enumerate(O.DIAG_FIELDS)})
    return out


def _oracle(grid, p, t, td, ps, ts, tds, source, adiabat, pinc=500.0, ml_depth=500.0, start=None,
            precision="f32"):
    nk = np.shape(t)[-1]
    t2, td2 = np.reshape(t, (-1, nk)), np.reshape(td, (-1, nk))
    sf = [np.ravel(a) for a in (ps, ts, tds)]
    kw = dict(stats=True, precision=precision)
    if grid == 1:
        return O.loopcape(np.reshape(p, (-1, nk)), t2, td2, *sf, pinc, source, ml_depth, adiabat,
                          **kw)
    if grid == 2:
        st = O.pres_lev_pos(p, sf[0]) if start is None else start
        return O.loopcape(np.ravel(p), t2, td2, *sf, pinc, source, ml_depth, adiabat, start=st,
                          p_is_1d=True, **kw)
    return O.loopcape(np.reshape(p, (-1, nk)), t2, td2, *sf, pinc, source, ml_depth, adiabat,
                      start=start, **kw)


@pytest.mark.parametrize("adiabat", ADIABATS)
@pytest.mark.parametrize("source", SOURCES)
def test_emulated_extrapolated_solver_vs_fp64(source, adiabat):
    """XC_GUESS_EXTRAPOLATED keeps the reference's map and stopping test, so
    its CAPE/CIN sit as close to the FP64 run as the plain FP32 iteration
    does -- with under 40 % of the iterations and without the FP32 limit
    cycles that make the plain iteration give up (cape = 0) on a few percent
    of these warm, moist columns."""
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(32, 64))
    fast = _emu_cape(2, plev, t, td, ps, ts, tds, source, adiabat, guess=2)
    plain = _emu_cape(2, plev, t, td, ps, ts, tds, source, adiabat, guess=0)
    ref = _oracle(2, plev, t, td, ps, ts, tds, source, adiabat, precision="f64")
    conv64 = (ref["status"] & 1) == 0
    assert not np.any((fast["status"] & 1) & conv64)
    assert (plain["status"] & 1).sum() > 0  # the limit cycles are present in this workload
    same_parcel = fast["mulvl"] == ref["mulvl"]  # MU-level near-ties pick another parcel
    ok = conv64 & same_parcel
    assert ok.mean() > 0.99
    for key in ("cape", "cin"):
        d = np.abs(fast[key][ok].astype(np.float64) - ref[key][ok])
        bad = d > np.maximum(1.0, 1e-3 * np.abs(ref[key][ok]))
        if key == "cin":
            # CIN is banked only when the buoyancy turns positive: where the
            # parcel grazes b = 0 (|b| < 1e-3 m/s^2 at some level) a last-bit
            # difference decides whether a negative area is banked
            tie = ref["bmin"][ok] < 1e-3
            assert bad[tie].sum() <= max(1, 0.005 * ok.sum())
            bad &= ~tie
        assert not np.any(bad), (key, d[bad].max())
    assert fast["counters"][1] < 0.4 * plain["counters"][1]


@pytest.mark.parametrize("adiabat", [1, 4])
def test_emulated_newton_point_ending(adiabat):
    """The extrapolated and learned solvers end a sub-step at their first
    Newton point when that step is below 0.01 K (newton_accept): about 1.1
    evaluations of the map per sub-step here (most-unstable parcels on
    pressure levels), against about 1.9 when every sub-step is evaluated
    again at the Newton point, with CAPE within 1 J/kg of the FP64 run."""
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(32, 64))
    fast = _emu_cape(2, plev, t, td, ps, ts, tds, 2, adiabat, guess=2)
    ref = _oracle(2, plev, t, td, ps, ts, tds, 2, adiabat, precision="f64")
    c = fast["counters"]
    assert c[1] < 1.2 * c[0], c
    ok = ((ref["status"] & 1) == 0) & (fast["mulvl"] == ref["mulvl"])
    assert ok.mean() > 0.99
    d = np.abs(fast["cape"][ok].astype(np.float64) - ref["cape"][ok])
    assert d.max() < 1.0, d.max()


def _qvs_ref(p, t):
    """getqvs (CAPE_CODE_model_lev.f90:570-581) in float64."""
    es = 611.2 * np.exp(17.67 * (t - 273.15) / (t - 29.65))
    return (287.04 / 461.5) * es / (p - es)


@pytest.mark.parametrize("reversible", [False, True])
@pytest.mark.parametrize("ice", [0, 1])
def test_emulated_map_slope_matches_finite_differences(ice, reversible):
    """The slope F'(x) that the accelerated solvers' first (Newton) step uses,
    differentiated analytically through qsat(T), the liquid/ice split and the
    exponent (accel_map), against a central difference of the map itself:
    saturated and unsaturated sub-steps from 215 to 305 K, on both sides of
    the ice ramp, away from the kinks of the map (saturation onset and the
    ramp's ends)."""
    L = emul.lib()
    rng = np.random.default_rng(11 + 2 * ice + int(reversible))
    o0, op, om = (np.zeros(9, np.float32) for _ in range(3))
    rddcp = 287.04 / 1005.7
    h = 0.05
    checked = sat_checked = 0
    for _ in range(600):
        p1 = rng.uniform(20000.0, 100000.0)
        dp = rng.uniform(100.0, 2000.0)
        p2 = p1 - dp
        t1 = rng.uniform(215.0, 305.0)
        qs1 = min(_qvs_ref(p1, t1), 0.04)
        sat = rng.random() < 0.7
        qv1 = qs1 if sat else qs1 * rng.uniform(0.3, 0.9)
        ql1 = rng.uniform(0.0, 2e-3) if (reversible and sat) else 0.0
        qt = qv1 + ql1
        th1 = t1 / (p1 / 1e5) ** rddcp
        pi2 = (p2 / 1e5) ** rddcp
        lp = np.log(p2 / p1)
        x = th1 + rng.uniform(-0.6, 0.1)
        args = (np.float32(p2), np.float32(pi2), np.float32(lp), np.float32(t1), np.float32(th1),
                np.float32(qv1), np.float32(ql1), np.float32(0.0), np.float32(qt))
        f0 = L.emu_accel_map(ice, np.float32(x), *args, o0.ctypes.data)
        fp = L.emu_accel_map(ice, np.float32(x + h), *args, op.ctypes.data)
        fm = L.emu_accel_map(ice, np.float32(x - h), *args, om.ctypes.data)
        cond = [o[3] + o[4] > 0.0 for o in (om, o0, op)]
        if len(set(cond)) > 1:
            continue  # the stencil straddles the saturation onset
        if ice and any(min(om[1], op[1]) - 0.1 <= tb <= max(om[1], op[1]) + 0.1
                       for tb in (233.15, 273.15)):
            continue  # the stencil straddles an end of the liquid/ice ramp
        fd = (np.float64(fp) - np.float64(fm)) / (2 * h)
        assert abs(o0[0] - fd) <= 3e-3 + 2e-2 * abs(fd), (o0[0], fd, t1, p1, sat)
        # the state's derivatives that the Newton point's state is built
        # from (d/dt2 of qv2, ql2, qi2; zero where unsaturated)
        dt = np.float64(op[1]) - np.float64(om[1])
        for j in (2, 3, 4):
            fdq = (np.float64(op[j]) - np.float64(om[j])) / dt
            scale = max(abs(fdq), 1e-6)
            assert abs(o0[j + 3] - fdq) <= 2e-7 + 2e-2 * scale, (j, o0[j + 3], fdq, t1, p1, sat)
        checked += 1
        sat_checked += cond[1]
    assert checked > 300 and sat_checked > 150, (checked, sat_checked)


def _same(a, b):
    for k in ("cape", "cin", "mulvl", "z_out", "status"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    assert a["counters"][0] == b["nsub"].sum()
    assert a["counters"][1] == b["niter"].sum()


@pytest.mark.parametrize("adiabat", ADIABATS)
@pytest.mark.parametrize("source", SOURCES)
def test_emulated_cape_sigma_bit_exact(source, adiabat):
    p, t, td, ps, ts, tds = S.sigma_c0(shape=(16, 24))
    _same(_emu_cape(1, p, t, td, ps, ts, tds, source, adiabat),
          _oracle(1, p, t, td, ps, ts, tds, source, adiabat))


@pytest.mark.parametrize("adiabat", (1, 4))
@pytest.mark.parametrize("source", SOURCES)
def test_emulated_cape_pressure_bit_exact(source, adiabat):
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(24, 24))
    _same(_emu_cape(2, plev, t, td, ps, ts, tds, source, adiabat),
          _oracle(2, plev, t, td, ps, ts, tds, source, adiabat))


def test_emulated_cape_goldens_bit_exact(soundings, era5):
    s = soundings
    P, T, TD = s["pressure"], s["temperature"], s["dewpoint"]
    for source, pinc in ((1, 100.0), (2, 100.0), (3, 1000.0)):
        args = (P[:, 1:], T[:, 1:], TD[:, 1:], P[:, 0], T[:, 0], TD[:, 0])
        _same(_emu_cape(1, *args, source, 1, pinc=pinc),
              _oracle(1, *args, source, 1, pinc=pinc))
    e = era5
    for source in SOURCES:
        args = (e["lev_level"], e["lev_t"], e["lev_td"], e["sfc_p"], e["sfc_t"], e["sfc_td"])
        _same(_emu_cape(2, *args, source, 1, ml_depth=300.0),
              _oracle(2, *args, source, 1, ml_depth=300.0))


def test_emulated_cape_3d_pressure_and_edges():
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(8, 16))
    n2 = 128
    p3 = np.broadcast_to(plev, (n2, plev.size)) + np.random.default_rng(3).normal(
        0, 0.5, (n2, plev.size)).astype(np.float32)
    st = O.pres_lev_pos(plev, ps.ravel())
    st[:3] = [1, 37, 5]
    for source in SOURCES:
        _same(_emu_cape(3, p3, t, td, ps, ts, tds, source, 1, start=st),
              _oracle(3, p3, t, td, ps, ts, tds, source, 1, start=st))
    # short columns, deep mixed layer, cold surface, MU above 500 hPa
    p, t, td, ps, ts, tds = (np.array(a) for a in S.sigma_c0(shape=(1, 12), nlev=40, seed=4))
    ts[0, 0] = -1.0
    p[0, 2] *= 0.45
    ps[0, 2] *= 0.45
    for nlev, mld in ((40, 500.0), (2, 5000.0), (1, 500.0)):
        for source in SOURCES:
            args = (p[..., :nlev], t[..., :nlev], td[..., :nlev], ps, ts, tds)
            _same(_emu_cape(1, *args, source, 1, ml_depth=mld),
                  _oracle(1, *args, source, 1, ml_depth=mld))


@pytest.mark.parametrize("dtype", (np.float32, np.float64))
def test_emulated_pres_lev_pos(dtype):
    L = emul.lib()
    plev = np.array([1000, 975, 950, 950, 900, 850, 700, 500, 300, 100], dtype)
    ps = np.random.default_rng(11).uniform(800, 1050, 512).astype(dtype)
    ps[:5] = [1000, 950, 899.99, 80, np.nan]
    st = np.empty(ps.size, np.int32)
    L.emu_pres_lev_pos(plev.ctypes.data, ps.ctypes.data, int(dtype == np.float64), plev.size,
                       ps.size, st.ctypes.data)
    np.testing.assert_array_equal(st, O.pres_lev_pos(plev, ps))


def _emu_srh(grid, p, t, td, u, v, ps, ts, tds, us, vs, depth, precision=0):
    L = emul.lib()
    f64 = any(np.asarray(a).dtype == np.float64 for a in (p, t, td, u, v, ps, ts, tds, us, vs))
    dt = np.float64 if f64 else np.float32
    nk = np.shape(t)[-1]
    n2 = np.size(t) // nk
    arrs = [np.ascontiguousarray(a, dt) for a in (p, t, td, u, v, ps, ts, tds, us, vs)]
    srm, slm = np.empty(n2), np.empty(n2)
    rm, lm, mean = (np.empty((n2, 2), np.float32) for _ in range(3))
    L.emu_srh(grid, *[a.ctypes.data for a in arrs], int(f64), None, float(depth), 2.0, nk, n2,
              srm.ctypes.data, slm.ctypes.data, rm.ctypes.data, lm.ctypes.data, mean.ctypes.data,
              precision)
    return (srm, slm, rm[:, 0], rm[:, 1], lm[:, 0], lm[:, 1], mean[:, 0], mean[:, 1])


def _srh_same(got, args, grid, depth):
    want = O.calc_srh(*args, depth=depth, vertical_lev="sigma" if grid == 1 else "pressure",
                      output_var="all")
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, np.ravel(w))


@pytest.mark.parametrize("depth", (1000, 3000))
def test_emulated_srh_bit_exact(soundings, era5, depth):
    s = soundings
    P, T, TD, U, V = s["pressure"], s["temperature"], s["dewpoint"], s["u_wind_ms"], s["v_wind_ms"]
    args = (P[:, 1:], T[:, 1:], TD[:, 1:], U[:, 1:], V[:, 1:], P[:, 0], T[:, 0], TD[:, 0],
            U[:, 0], V[:, 0])
    _srh_same(_emu_srh(1, *args, depth), args, 1, depth)
    e = era5
    args = (e["lev_level"], e["lev_t"], e["lev_td"], e["lev_u"], e["lev_v"], e["sfc_p"],
            e["sfc_t"], e["sfc_td"], e["sfc_u"], e["sfc_v"])
    _srh_same(_emu_srh(2, *args, depth), args, 2, depth)
    args = S.srh_c2(shape=(16, 16), nlev=50)
    _srh_same(_emu_srh(1, *args, depth), args, 1, depth)
    args = S.pressure_srh(shape=(16, 16))
    _srh_same(_emu_srh(2, *args, depth), args, 2, depth)


def test_emulated_srh_decreasing_heights():
    p, t, td, u, v, ps, ts, tds, us, vs = (np.array(a, np.float64) for a in
                                           S.srh_c2(shape=(4, 8), nlev=50, seed=9))
    p, t, td = (a[..., ::-1].copy() for a in (p, t, td))
    ps = p[..., 0] * 1.2
    args = (p, t, td, u, v, ps, ts, tds, us, vs)
    _srh_same(_emu_srh(1, *args, 3000), args, 1, 3000)


@pytest.mark.parametrize("depth", (1000, 3000))
def test_emulated_fp32_srh_vs_fp64_oracle(soundings, depth):
    """precision=XC_SRH_FP32 (FP32 height and helicity with compensated
    sums) against the oracle run in FP64 throughout: SRH within 0.05
    m^2/s^2 (the stated tolerance is 0.5), storm motion within 1e-3 m/s."""
    for args, grid in ((S.srh_c2(shape=(64, 64), nlev=50), 1),
                       (S.pressure_srh(shape=(48, 48)), 2)):
        got = _emu_srh(grid, *args, depth, precision=1)
        vl = "sigma" if grid == 1 else "pressure"
        want = O.calc_srh(*args, depth=depth, vertical_lev=vl, output_var="all", precision="f64")
        for g, w in zip(got[:2], want[:2]):
            np.testing.assert_allclose(g, np.ravel(w), rtol=0, atol=0.05)
        for g, w in zip(got[2:], want[2:]):
            np.testing.assert_allclose(g, np.ravel(w), rtol=0, atol=1e-3)


@pytest.mark.parametrize("adiabat", (1, 4))
@pytest.mark.parametrize("source", SOURCES)
def test_emulated_diagnostics_bit_exact(source, adiabat):
    """The LFC/EL/source diagnostics of the column code (DIAG) against the
    oracle's restatement of the same definitions, sigma and pressure grids."""
    p, t, td, ps, ts, tds = S.sigma_c0(shape=(12, 24))
    got = _emu_cape(1, p, t, td, ps, ts, tds, source, adiabat, diag=True)
    nk = t.shape[-1]
    want = O.loopcape_diag(np.reshape(p, (-1, nk)), np.reshape(t, (-1, nk)),
                           np.reshape(td, (-1, nk)), ps, ts, tds, 500.0, source, 500.0, adiabat)
    plev, t2, td2, ps2, ts2, tds2 = S.pressure_c1(shape=(16, 24))
    got2 = _emu_cape(2, plev, t2, td2, ps2, ts2, tds2, source, adiabat, diag=True)
    want2 = O.loopcape_diag(plev, np.reshape(t2, (-1, 37)), np.reshape(td2, (-1, 37)), ps2, ts2,
                            tds2, 500.0, source, 500.0, adiabat,
                            start=O.pres_lev_pos(plev, ps2.ravel()))
    for g, w in ((got, want), (got2, want2)):
        for k in ("cape", "cin", "mulvl", "z_out", "status") + O.DIAG_FIELDS:
            np.testing.assert_array_equal(g[k], w[k], err_msg=k)
        pos = g["cape"] > 0
        assert pos.any()
        # LFC below EL; undefined without positive area
        assert np.all(g["plfc"][pos] >= g["pel"][pos])
        assert np.all(g["zlfc"][pos] <= g["zel"][pos])
        assert np.all(g["plfc"][g["cape"] == 0] == -999999)


@pytest.mark.parametrize("source", SOURCES)
def test_emulated_nonfinite_inputs_bit_exact(source):
    """NaN and infinite inputs: the column code ends (the iteration and
    sub-step caps bound every loop) and reproduces the oracle bit for bit,
    NaN for NaN -- except where a pressure is NaN.  There the sub-step count
    1 + int(dp/pinc) (CAPE_CODE_model_lev.f90:410-415) converts NaN to an
    integer, which Fortran and C leave undefined (x86 gives INT_MIN and
    skips the sub-steps, aarch64 gives 0); the kernels flag such a column
    (status bit 4, too many sub-steps) and return zero."""
    p, t, td, ps, ts, tds = with_nonfinite()
    got = _emu_cape(1, p, t, td, ps, ts, tds, source, 1)
    want = _oracle(1, p, t, td, ps, ts, tds, source, 1)
    nan_p = np.isnan(p.reshape(64, -1)).any(axis=1) | np.isnan(ps.ravel())
    flagged = (got["status"] & 4) != 0
    assert np.all(nan_p[flagged]) and flagged.any()
    assert np.all(got["cape"][flagged] == 0) and np.all(got["cin"][flagged] == 0)
    for k in ("cape", "cin", "mulvl", "z_out"):
        np.testing.assert_array_equal(got[k][~flagged], want[k][~flagged], err_msg=k)


def _emu_cape64(grid, p, t, td, ps, ts, tds, source, adiabat, pinc=500.0, ml_depth=500.0,
                start=None):
    L = emul.lib()
    f64 = any(np.asarray(a).dtype == np.float64 for a in (p, t, td, ps, ts, tds))
    dt = np.float64 if f64 else np.float32
    t = np.ascontiguousarray(t, dt)
    nk = t.shape[-1]
    n2 = t.size // nk
    arrs = [np.ascontiguousarray(a, dt) for a in (p, t, td, ps, ts, tds)]
    st = None if start is None else np.ascontiguousarray(start, np.int32)
    out = dict(cape=np.empty(n2, np.float32), cin=np.empty(n2, np.float32),
               mulvl=np.empty(n2, np.int32), z_out=np.empty(n2, np.float32),
               status=np.empty(n2, np.int32))
    L.emu_cape64(grid, *[a.ctypes.data for a in arrs], int(f64), pinc, source, ml_depth, adiabat,
                 None if st is None else st.ctypes.data, nk, n2, out["cape"].ctypes.data,
                 out["cin"].ctypes.data, out["mulvl"].ctypes.data, out["z_out"].ctypes.data,
                 out["status"].ctypes.data)
    return out


@pytest.mark.parametrize("adiabat", ADIABATS)
@pytest.mark.parametrize("source", SOURCES)
def test_emulated_fp64_plain_solver_vs_fp64_oracle(source, adiabat):
    """The double-precision instance of the column routine (the FP64
    retry's) against the oracle's FP64 build: the same algorithm in double,
    differing only in the named physical constants, which the routine takes
    from the FP32 program widened to double (relative differences near
    1e-8).  Every column's give-up flag must agree, the parcel level too,
    and CAPE/CIN within 1e-3 J/kg (or 1e-5 relative)."""
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(24, 64), seed=13)
    got = _emu_cape64(2, plev, t, td, ps, ts, tds, source, adiabat)
    want = _oracle(2, plev, t, td, ps, ts, tds, source, adiabat, precision="f64")
    np.testing.assert_array_equal(got["status"] & 1, want["status"] & 1)
    np.testing.assert_array_equal(got["mulvl"], want["mulvl"])
    for k in ("cape", "cin", "z_out"):
        w = want[k].astype(np.float64)
        d = np.abs(got[k].astype(np.float64) - w)
        assert np.all(d <= np.maximum(1e-3, 1e-5 * np.abs(w))), (k, d.max())
    # in double precision the plain iteration converges where FP32 cycled
    f32 = _oracle(2, plev, t, td, ps, ts, tds, source, adiabat)
    assert (got["status"] & 1).sum() <= (f32["status"] & 1).sum()


@pytest.mark.parametrize("guess", [1, 2, 3])
@pytest.mark.parametrize("source", SOURCES)
def test_emulated_surface_on_a_pressure_level(source, guess):
    """ps exactly equal to a pressure level: the first sub-step above the
    surface has no pressure drop.  The accelerated solvers extrapolate the
    previous sub-step's increment per unit pressure, which such a step does
    not define; they must stay finite and agree with the FP64 oracle like
    every other column (the plain solver is pinned bit for bit elsewhere)."""
    from xcape_gb300 import guess as G
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(16, 48), seed=17)
    ps = ps.copy().ravel()
    ps[::2] = plev[np.arange(ps.size // 2) % 12].astype(ps.dtype)  # 1000..725 hPa
    w = G.bf16_round(G.init_weights(5, 0.3)) if guess == 1 else None
    got = _emu_cape(2, plev, t, td, ps, ts, tds, source, 1, guess=guess, guess_w=w)
    ref = _oracle(2, plev, t, td, ps, ts, tds, source, 1, precision="f64")
    assert np.all(np.isfinite(got["cape"])) and np.all(np.isfinite(got["cin"]))
    conv = ((ref["status"] & 1) == 0) & (got["mulvl"] == ref["mulvl"])
    d = np.abs(got["cape"][conv].astype(np.float64) - ref["cape"][conv])
    assert np.all(d <= np.maximum(1.0, 1e-3 * np.abs(ref["cape"][conv]))), d.max()
