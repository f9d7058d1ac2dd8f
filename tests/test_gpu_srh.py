"""GPU parity tests of storm-relative helicity and its stages.

Mirrors test/test_core.py:173-286 of the reference (sigma and pressure SRH
goldens, decimal=5) and checks the Bunkers vectors, the individual stage
entry points (stdheight, Bunkers, SREH) and seeded synthetic workloads
against the CPU oracle.  SRH is double precision in the reference and here,
so the bar is 1e-5 m^2/s^2 on the goldens and a relative 1e-9 on synthetic
columns; the FP32 Bunkers vectors must agree to 1e-4 m/s.
"""
import numpy as np
import pytest

import oracle as O
import xcape_gb300 as X
from xcape_gb300 import _lib
from xcape_gb300 import synthetic as S

from gpu_util import to_dev, torch_cuda

pytestmark = pytest.mark.gpu


def _snd_args(s):
    P, T, TD, U, V = s["pressure"], s["temperature"], s["dewpoint"], s["u_wind_ms"], s["v_wind_ms"]
    return (P[:, 1:], T[:, 1:], TD[:, 1:], U[:, 1:], V[:, 1:], P[:, 0], T[:, 0], TD[:, 0],
            U[:, 0], V[:, 0])


def _era_args(e):
    return (e["lev_level"], e["lev_t"], e["lev_td"], e["lev_u"], e["lev_v"], e["sfc_p"],
            e["sfc_t"], e["sfc_td"], e["sfc_u"], e["sfc_v"])


def _check_all(got, want, srh_atol):
    np.testing.assert_allclose(got[0], want[0], rtol=1e-9, atol=srh_atol)
    np.testing.assert_allclose(got[1], want[1], rtol=1e-9, atol=srh_atol)
    for g, w in zip(got[2:], want[2:]):
        assert g.dtype == np.float32
        np.testing.assert_allclose(g, w, rtol=0, atol=1e-4)


@pytest.mark.parametrize("use_torch", [False, True])
@pytest.mark.parametrize("output_var,n", [("srh", 2), ("all", 8)])
def test_srh_sigma_golden(soundings, output_var, n, use_torch):
    s = soundings
    args = _snd_args(s)
    if use_torch:
        args = to_dev(*args)
    res = X.calc_srh(*args, depth=3000, vertical_lev="sigma", output_var=output_var)
    assert len(res) == n
    res = [r.cpu().numpy() if use_torch else r for r in res]
    np.testing.assert_almost_equal(res[0], s["SRH03_model_lev_rm"], 5)
    np.testing.assert_almost_equal(res[1], s["SRH03_model_lev_lm"], 5)
    if output_var == "all":
        want = O.calc_srh(*_snd_args(s), depth=3000, vertical_lev="sigma", output_var="all")
        _check_all(res, want, 1e-6)


@pytest.mark.parametrize("output_var,n", [("srh", 2), ("all", 8)])
def test_srh_pressure_golden(era5, output_var, n):
    e = era5
    res = X.calc_srh(*_era_args(e), depth=3000, vertical_lev="pressure", output_var=output_var)
    assert len(res) == n
    np.testing.assert_almost_equal(res[0], e["sfc_srh_rm"], 5)
    np.testing.assert_almost_equal(res[1], e["sfc_srh_lm"], 5)
    if output_var == "all":
        want = O.calc_srh(*_era_args(e), depth=3000, vertical_lev="pressure", output_var="all")
        _check_all(res, want, 1e-6)


@pytest.mark.parametrize("depth", [1000, 3000])
def test_srh_model_levels_synthetic(depth):
    """256x256 columns x 50 model levels, float32, veering jet
    (vertical_lev='model' aliases 'sigma')."""
    args = S.srh_c2(shape=(256, 256))
    got = X.calc_srh(*args, depth=depth, vertical_lev="model", output_var="all")
    want = O.calc_srh(*args, depth=depth, vertical_lev="model", output_var="all")
    _check_all(got, want, 1e-6)
    assert np.mean(got[0]) > 0  # veering hodograph: positive right-mover helicity


def test_srh_pressure_synthetic():
    args = S.pressure_srh(shape=(96, 96))
    got = X.calc_srh(*args, depth=3000, vertical_lev="pressure", output_var="all")
    want = O.calc_srh(*args, depth=3000, vertical_lev="pressure", output_var="all")
    _check_all(got, want, 1e-6)


def test_srh_decreasing_height_columns():
    """Columns whose heights fall with level index take DINTERP2DZ's other
    scan rule (Bunkers_model_lev.f90:210-215)."""
    p, t, td, u, v, ps, ts, tds, us, vs = (np.array(a, np.float64) for a in
                                           S.srh_c2(shape=(4, 8), nlev=50, seed=9))
    p = p[..., ::-1].copy()
    t = t[..., ::-1].copy()
    td = td[..., ::-1].copy()
    ps = p[..., 0] * 1.2
    got = X.calc_srh(p, t, td, u, v, ps, ts, tds, us, vs, depth=3000, output_var="all")
    want = O.calc_srh(p, t, td, u, v, ps, ts, tds, us, vs, depth=3000, output_var="all")
    _check_all(got, want, 1e-6)


def test_srh_stage_entry_points(soundings):
    """loop_stdheight_ml, bunkers_loop_ml and loop_sreh_ml bound one by one."""
    torch = torch_cuda()
    P, T, TD, U, V, ps, ts, tds, us, vs = (np.ascontiguousarray(a, np.float64)
                                           for a in _snd_args(soundings))
    n2, nk = T.shape
    hin = np.full(n2, 2.0)
    H_w, Hs_w = O.loop_stdheight(P, T, TD, ps, ts, tds, hin)
    d = to_dev(P, T, TD, ps, ts, tds, hin)
    H = torch.empty((n2, nk), dtype=torch.float64, device="cuda")
    Hs = torch.empty(n2, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    _lib.call("xc_loop_stdheight_ml", *[x.data_ptr() for x in d], nk, n2, H.data_ptr(),
              Hs.data_ptr(), st)
    torch.cuda.synchronize()
    np.testing.assert_allclose(H.cpu().numpy(), H_w, rtol=1e-12)
    np.testing.assert_array_equal(Hs.cpu().numpy(), Hs_w)

    f32 = [np.ascontiguousarray(a, np.float32) for a in (U, V, H_w, us, vs, Hs_w)]
    rm_w, lm_w, mean_w = O.bunkers_loop(*f32)
    d = to_dev(*f32)
    RM, LM, MEAN = (torch.empty((n2, 2), dtype=torch.float32, device="cuda") for _ in range(3))
    _lib.call("xc_bunkers_loop_ml", *[x.data_ptr() for x in d], nk, n2, RM.data_ptr(),
              LM.data_ptr(), MEAN.data_ptr(), st)
    torch.cuda.synchronize()
    for g, w in ((RM, rm_w), (LM, lm_w), (MEAN, mean_w)):
        np.testing.assert_allclose(g.cpu().numpy(), w, rtol=0, atol=1e-5)

    srm_w, slm_w = O.loop_sreh(U, V, H_w, us, vs, Hs_w, rm_w[:, 0], rm_w[:, 1], lm_w[:, 0],
                               lm_w[:, 1], 3000.0)
    d = to_dev(U, V, H_w, us, vs, Hs_w, *(np.ascontiguousarray(a, np.float64) for a in
                                          (rm_w[:, 0], rm_w[:, 1], lm_w[:, 0], lm_w[:, 1])))
    SRM = torch.empty(n2, dtype=torch.float64, device="cuda")
    SLM = torch.empty_like(SRM)
    _lib.call("xc_loop_sreh_ml", *[x.data_ptr() for x in d], 3000.0, nk, n2, SRM.data_ptr(),
              SLM.data_ptr(), st)
    torch.cuda.synchronize()
    np.testing.assert_allclose(SRM.cpu().numpy(), srm_w, rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(SLM.cpu().numpy(), slm_w, rtol=1e-12, atol=1e-9)


def test_srh_pressure_stage_entry_points(era5):
    """loop_stdheight_pl1d, bunkers_loop_pl and loop_sreh_pl with start_3d."""
    torch = torch_cuda()
    e = era5
    plev = np.ascontiguousarray(e["lev_level"], np.float64)
    T, TD, U, V = (np.ascontiguousarray(e[k], np.float64) for k in ("lev_t", "lev_td", "lev_u",
                                                                      "lev_v"))
    ps, ts, tds, us, vs = (np.ascontiguousarray(e[k], np.float64) for k in
                           ("sfc_p", "sfc_t", "sfc_td", "sfc_u", "sfc_v"))
    n2, nk = T.shape
    start = O.pres_lev_pos(plev, ps)
    hin = np.full(n2, 2.0)
    H_w, Hs_w = O.loop_stdheight(plev, T, TD, ps, ts, tds, hin, start=start, p_is_1d=True)
    st = torch.cuda.current_stream().cuda_stream
    d = to_dev(T, TD, plev, ps, ts, tds, hin)
    S_ = to_dev(start)[0]
    H = torch.empty((n2, nk), dtype=torch.float64, device="cuda")
    Hs = torch.empty(n2, dtype=torch.float64, device="cuda")
    _lib.call("xc_loop_stdheight_pl1d", *[x.data_ptr() for x in d], S_.data_ptr(), nk, n2,
              H.data_ptr(), Hs.data_ptr(), st)
    torch.cuda.synchronize()
    np.testing.assert_allclose(H.cpu().numpy(), H_w, rtol=1e-12)
    f32 = [np.ascontiguousarray(a, np.float32) for a in (U, V, H_w, us, vs, Hs_w)]
    rm_w, lm_w, mean_w = O.bunkers_loop(*f32, start=start)
    d = to_dev(*f32)
    RM, LM, MEAN = (torch.empty((n2, 2), dtype=torch.float32, device="cuda") for _ in range(3))
    _lib.call("xc_bunkers_loop_pl", *[x.data_ptr() for x in d], S_.data_ptr(), nk, n2,
              RM.data_ptr(), LM.data_ptr(), MEAN.data_ptr(), st)
    torch.cuda.synchronize()
    np.testing.assert_allclose(RM.cpu().numpy(), rm_w, atol=1e-5)
    srm_w, _ = O.loop_sreh(U, V, H_w, us, vs, Hs_w, rm_w[:, 0], rm_w[:, 1], lm_w[:, 0],
                           lm_w[:, 1], 3000.0, start=start)
    d = to_dev(U, V, H_w, us, vs, Hs_w, *(np.ascontiguousarray(a, np.float64) for a in
                                          (rm_w[:, 0], rm_w[:, 1], lm_w[:, 0], lm_w[:, 1])))
    SRM = torch.empty(n2, dtype=torch.float64, device="cuda")
    SLM = torch.empty_like(SRM)
    _lib.call("xc_loop_sreh_pl", *[x.data_ptr() for x in d], 3000.0, S_.data_ptr(), nk, n2,
              SRM.data_ptr(), SLM.data_ptr(), st)
    torch.cuda.synchronize()
    np.testing.assert_allclose(SRM.cpu().numpy(), srm_w, rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("hin_m", [2.0, 0.0])
def test_stdheight_pressure_3d_entry_point(hin_m):
    """loop_stdheight_pl (stdheight_2D_pressure_lev.f90:5-47, :133-219): a
    pressure per column and level plus a per-column start level, against the
    oracle's restatement of the same routine.  The columns' pressures are the
    shared levels perturbed per column, ps is ragged so that the start level
    varies, and a few columns start at the first or the last level."""
    torch = torch_cuda()
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(24, 40), seed=9)
    n2, nk = ps.size, plev.size
    rng = np.random.default_rng(19)
    P = np.broadcast_to(plev.astype(np.float64), (n2, nk)).copy()
    P *= 1.0 + rng.normal(0.0, 2e-3, P.shape)
    T = np.ascontiguousarray(t.reshape(n2, nk), np.float64)
    TD = np.ascontiguousarray(td.reshape(n2, nk), np.float64)
    ps64, ts64, tds64 = (np.ascontiguousarray(np.ravel(a), np.float64) for a in (ps, ts, tds))
    start = np.array([O.pres_lev_pos(P[i], ps64[i:i + 1])[0] for i in range(n2)], np.int32)
    start[:3] = [1, nk, nk - 1]
    hin = np.full(n2, hin_m)
    H_w, Hs_w = O.loop_stdheight(P, T, TD, ps64, ts64, tds64, hin, start=start)
    d = to_dev(P, T, TD, ps64, ts64, tds64, hin)
    S_ = to_dev(start)[0]
    H = torch.empty((n2, nk), dtype=torch.float64, device="cuda")
    Hs = torch.empty(n2, dtype=torch.float64, device="cuda")
    _lib.call("xc_loop_stdheight_pl", *[x.data_ptr() for x in d], S_.data_ptr(), nk, n2,
              H.data_ptr(), Hs.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = H.cpu().numpy()
    # below-ground levels carry the reference's -999999 sentinel on both sides
    np.testing.assert_array_equal(got == -999999.0, H_w == -999999.0)
    np.testing.assert_allclose(got, H_w, rtol=1e-12, atol=1e-9)
    np.testing.assert_array_equal(Hs.cpu().numpy(), Hs_w)
    assert len(set(start.tolist())) > 3  # the start level really varies


def test_srh_full_size_workload():
    """1024x1024 columns x 50 levels: determinism and a sample vs the oracle."""
    torch = torch_cuda()
    args = S.srh_c2()
    dev = to_dev(*args)
    a = X.calc_srh(*dev, depth=3000, vertical_lev="model", output_var="all")
    b = X.calc_srh(*dev, depth=3000, vertical_lev="model", output_var="all")
    torch.cuda.synchronize()
    for x, y in zip(a, b):
        assert torch.equal(x, y)
    n2 = 1024 * 1024
    idx = np.sort(np.random.default_rng(8).choice(n2, 8192, replace=False))
    sub = [np.reshape(x, (n2, -1))[idx] for x in args[:5]] + [np.ravel(x)[idx] for x in args[5:]]
    want = O.calc_srh(*sub, depth=3000, vertical_lev="model", output_var="all")
    got = [x.reshape(-1).cpu().numpy()[idx] for x in a]
    _check_all(got, want, 1e-6)


@pytest.mark.parametrize("depth", [1000, 3000])
def test_srh_fp32_precision_vs_fp64(depth):
    """precision='fp32' (FP32 height and helicity stages, compensated sums)
    against the oracle run in FP64 throughout: SRH within 0.05 m^2/s^2 --
    the stated tolerance is 0.5 -- and storm motion within 1e-3 m/s."""
    for args, vl in ((S.srh_c2(shape=(128, 128)), "model"),
                     (S.pressure_srh(shape=(96, 96)), "pressure")):
        got = X.calc_srh(*args, depth=depth, vertical_lev=vl, output_var="all", precision="fp32")
        want = O.calc_srh(*args, depth=depth, vertical_lev=vl, output_var="all", precision="f64")
        for g, w in zip(got[:2], want[:2]):
            np.testing.assert_allclose(g, w, rtol=0, atol=0.05)
        for g, w in zip(got[2:], want[2:]):
            np.testing.assert_allclose(g, w, rtol=0, atol=1e-3)


@pytest.mark.parametrize("depth", [1000, 3000])
def test_srh_fp32_level_parallel_kernel_matches_column_path(depth):
    """float32 inputs take the level-parallel kernel (srh_seg_kernel: eight
    lanes per column, heights by a segmented scan, helicity from its
    storm-motion free part); the same values as float64 take the one-thread
    FP32 column path.  Both are FP32 forms of the same formulas with
    approximate transcendentals, but not the same forms (the kernel's
    virtual temperature takes one reciprocal, its log is of the pressure
    ratio taken the other way up) nor the same summation orders: SRH within
    0.01 m^2/s^2, storm motion within 5e-4 m/s (each is within 1e-3 m/s of
    the FP64 oracle, test_srh_fp32_precision_vs_fp64), for sigma and
    pressure grids, ragged starts and a partial last block."""
    for args, vl in ((S.srh_c2(shape=(37, 41)), "model"),
                     (S.pressure_srh(shape=(29, 33)), "pressure")):
        a32 = [np.asarray(x, np.float32) for x in args]
        a64 = [x.astype(np.float64) for x in a32]
        got = X.calc_srh(*a32, depth=depth, vertical_lev=vl, output_var="all", precision="fp32")
        want = X.calc_srh(*a64, depth=depth, vertical_lev=vl, output_var="all", precision="fp32")
        for g, w in zip(got[:2], want[:2]):
            np.testing.assert_allclose(g, w, rtol=0, atol=1e-2)
        for g, w in zip(got[2:], want[2:]):
            np.testing.assert_allclose(g, w, rtol=0, atol=5e-4)


@pytest.mark.parametrize("nlev", [137, 100])
def test_srh_fp32_level_parallel_kernel_several_rounds(nlev):
    """Columns deeper than one round of the level-parallel kernel (137 sigma
    levels: three rounds of 8 lanes x 6 levels; 100 pressure levels with
    ragged starts: three rounds of 8 x 5) against the FP64 oracle, at the
    FP32 path's tolerance."""
    cases = ((S.srh_c2(shape=(20, 24), nlev=nlev), "model") if nlev == 137 else
             (S.pressure_srh(shape=(20, 24), nlev=nlev), "pressure"))
    args, vl = cases
    args = [np.asarray(x, np.float32) for x in args]
    for depth in (1000, 3000):
        got = X.calc_srh(*args, depth=depth, vertical_lev=vl, output_var="all", precision="fp32")
        want = O.calc_srh(*[x.astype(np.float64) for x in args], depth=depth, vertical_lev=vl,
                          output_var="all", precision="f64")
        for g, w in zip(got[:2], want[:2]):
            np.testing.assert_allclose(g, w, rtol=0, atol=0.05)
        for g, w in zip(got[2:], want[2:]):
            np.testing.assert_allclose(g, w, rtol=0, atol=1e-3)


def test_srh_fp32_level_parallel_kernel_short_columns():
    """A coarse pressure grid (9 levels, 1000-100 hPa) with ragged starts:
    columns with fewer levels above the ground than one run of the
    level-parallel kernel (5 levels here) are taken by the column routine;
    all agree with the FP64 oracle at the FP32 path's tolerance."""
    args = [np.asarray(x, np.float32).copy() for x in S.pressure_srh(shape=(24, 30), nlev=9,
                                                                       seed=5)]
    args[5].reshape(-1)[::3] = 520.0   # high ground: 4 levels above it
    start = O.pres_lev_pos(args[0].astype(np.float64), np.ravel(args[5]).astype(np.float64))
    assert (9 - np.ravel(start) + 1 < 5).any() and (9 - np.ravel(start) + 1 >= 5).any()
    for depth in (1000, 3000):
        got = X.calc_srh(*args, depth=depth, vertical_lev="pressure", output_var="all",
                         precision="fp32")
        want = O.calc_srh(*[x.astype(np.float64) for x in args], depth=depth,
                          vertical_lev="pressure", output_var="all", precision="f64")
        for g, w in zip(got[:2], want[:2]):
            np.testing.assert_allclose(g, w, rtol=0, atol=0.05)
        for g, w in zip(got[2:], want[2:]):
            np.testing.assert_allclose(g, w, rtol=0, atol=1e-3)


def test_srh_fp32_staged_and_direct_loads_agree():
    """Float32 CUDA tensors on 16-byte boundaries take the level-parallel
    kernel with its rows staged in shared memory by bulk copies (all full
    blocks; the partial last block reads global memory); the same values one
    float off a 16-byte boundary take the direct-load kernel for every
    block.  Both run the same arithmetic on the same values: the same bits."""
    torch = torch_cuda()
    for args, vl in ((S.srh_c2(shape=(37, 41)), "model"), (S.pressure_srh(shape=(29, 33)), "pressure")):
        dev = to_dev(*[np.asarray(x, np.float32) for x in args])
        assert all(x.data_ptr() % 16 == 0 for x in dev)
        off = []
        for x in dev:
            buf = torch.empty(x.numel() + 1, dtype=x.dtype, device=x.device)
            y = buf[1:].view(x.shape)
            y.copy_(x)
            assert y.data_ptr() % 16 == 4
            off.append(y)
        a = X.calc_srh(*dev, depth=3000, vertical_lev=vl, output_var="all", precision="fp32")
        b = X.calc_srh(*off, depth=3000, vertical_lev=vl, output_var="all", precision="fp32")
        torch.cuda.synchronize()
        for x, y in zip(a, b):
            assert torch.equal(x, y)


def test_srh_fp32_level_parallel_kernel_falls_back_on_irregular_columns():
    """Columns whose heights do not increase with level -- pressure rising
    with level, a NaN, a level below the previous one -- are redone by the
    one-thread FP32 column path, which follows the reference's scan rules for
    any column: outputs equal that path's bit for bit (NaN where it has NaN),
    and the regular columns beside them stay within the FP64 tolerance."""
    args = [np.asarray(a, np.float32).copy() for a in S.srh_c2(shape=(16, 16), nlev=50, seed=8)]
    p, t, td, u, v, ps, ts, tds, us, vs = args
    p2 = p.reshape(256, 50)
    p2[0] = p2[0][::-1].copy()        # pressure rising with level: decreasing heights
    p2[1, 20] = np.nan                  # a non-finite input
    p2[2, 5] = p2[2, 4] * 1.01          # one level below the one under it
    t.reshape(256, 50)[3, 30] = np.nan
    a64 = [x.astype(np.float64) for x in args]
    got = X.calc_srh(*args, depth=3000, vertical_lev="model", output_var="all", precision="fp32")
    col = X.calc_srh(*a64, depth=3000, vertical_lev="model", output_var="all", precision="fp32")
    want = O.calc_srh(*a64, depth=3000, vertical_lev="model", output_var="all", precision="f64")
    for g, c in zip(got, col):
        g, c = np.ravel(g), np.ravel(c)
        np.testing.assert_array_equal(g[:4], c[:4])
    for g, w in zip(got[:2], want[:2]):
        np.testing.assert_allclose(np.ravel(g)[4:], np.ravel(w)[4:], rtol=0, atol=0.05)
