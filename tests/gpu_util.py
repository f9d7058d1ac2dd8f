"""Helpers for the GPU tests: direct C-ABI calls on torch device buffers and
the parity criteria shared by the tests.

Parity criteria (the tolerance the product states, tighter than the
reference's own ``decimal=0`` on CAPE/CIN):
  * CAPE, CIN: |diff| <= max(1 J/kg, 0.1 %);
  * MU level: equal, except near-ties where the two levels' theta-e differ by
    less than 1e-3 K (the argmax is then decided by rounding);
  * a column whose moist-adiabat iteration ends in the reference's
    100-iteration abort on one side only is a near-tie of the convergence
    test: FP32 rounding can leave the damped iteration in a two-value limit
    cycle whose step is just above the 2e-4 K threshold, and a one-ulp
    difference in expf decides whether that cycle is entered.  Such columns
    are counted and bounded (2 %); where only the GPU converged, its result
    must agree with the FP64 oracle;
  * CIN banks the accumulated negative area only at a negative-to-positive
    buoyancy crossing (CAPE_CODE_model_lev.f90:509-523), so where the
    parcel's buoyancy comes within 1e-3 m/s^2 of zero at some level, a
    rounding-level difference decides whether a whole layer is banked.  CIN
    may differ only in such columns (the oracle reports the smallest |b|),
    at most 0.5 % of them; CAPE is continuous there and is always compared.
"""
import numpy as np

from xcape_gb300 import _lib

SOURCES = {"surface": 1, "most-unstable": 2, "mixed-layer": 3}
ADIABATS = {"pseudo-liquid": 1, "reversible-liquid": 2, "pseudo-ice": 3, "reversible-ice": 4}


def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def to_dev(*arrays, dtype=None):
    torch = torch_cuda()
    out = []
    for a in arrays:
        a = np.ascontiguousarray(a if dtype is None else np.asarray(a, dtype=dtype))
        out.append(torch.from_numpy(a).cuda())
    return out


def cape_device(grid, p, t, td, ps, ts, tds, source, adiabat, pinc=500.0, ml_depth=500.0,
                start=None, guess=0, counters=False, order=True):
    """Runs xc_loopcape_ex on device copies; returns numpy outputs + status.
    order: pass a workspace so that the columns are ordered before the lift."""
    torch = torch_cuda()
    t = np.asarray(t)
    nk = t.shape[-1]
    n2 = int(np.prod(t.shape[:-1]))
    f64 = any(np.asarray(a).dtype == np.float64 for a in (p, t, td, ps, ts, tds))
    dt = np.float64 if f64 else np.float32
    P, T, TD, PS, TS, TDS = to_dev(p, t, td, ps, ts, tds, dtype=dt)
    ST = to_dev(np.asarray(start, np.int32))[0] if start is not None else None
    cape = torch.empty(n2, dtype=torch.float32, device="cuda")
    cin = torch.empty_like(cape)
    zout = torch.empty_like(cape)
    mulvl = torch.empty(n2, dtype=torch.int32, device="cuda")
    status = torch.empty(n2, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(2, dtype=torch.int64, device="cuda") if counters else None
    stream = torch.cuda.current_stream().cuda_stream
    ws, ws_bytes = None, 0
    if order:
        ws_bytes = _lib.workspace_bytes(n2)
        wsbuf = torch.empty(ws_bytes + 256, dtype=torch.uint8, device="cuda")
        ws = wsbuf.data_ptr() + (-wsbuf.data_ptr()) % 256
    _lib.call("xc_loopcape_ex", grid, P.data_ptr(), T.data_ptr(), TD.data_ptr(), PS.data_ptr(),
              TS.data_ptr(), TDS.data_ptr(), _lib.XC_F64 if f64 else _lib.XC_F32, float(pinc),
              SOURCES.get(source, source), float(ml_depth), ADIABATS.get(adiabat, adiabat),
              ST.data_ptr() if ST is not None else None, nk, n2, guess, cape.data_ptr(),
              cin.data_ptr(), mulvl.data_ptr(), zout.data_ptr(), status.data_ptr(),
              cnt.data_ptr() if cnt is not None else None, ws, ws_bytes, stream)
    torch.cuda.synchronize()
    out = dict(cape=cape.cpu().numpy(), cin=cin.cpu().numpy(), mulvl=mulvl.cpu().numpy(),
               z_out=zout.cpu().numpy(), status=status.cpu().numpy())
    if counters:
        c = cnt.cpu().numpy()
        out["nsub_total"], out["niter_total"] = int(c[0]), int(c[1])
    return out


def thetae_f64(p_hpa, t_c, td_c):
    """getthe (CAPE_CODE_model_lev.f90:604-620) in float64, for near-tie checks."""
    p = 100.0 * np.asarray(p_hpa, np.float64)
    t = 273.15 + np.asarray(t_c, np.float64)
    td = 273.15 + np.asarray(td_c, np.float64)
    es = 611.2 * np.exp(17.67 * (td - 273.15) / (td - 29.65))
    q = (287.04 / 461.5) * es / (p - es)
    tlcl = np.where((td - t) >= -0.1, t,
                    56.0 + 1.0 / (1.0 / (td - 56.0) + 0.00125 * np.log(t / td)))
    return t * (100000.0 / p) ** (0.2854 * (1.0 - 0.28 * q)) * np.exp(
        ((3376.0 / tlcl) - 2.54) * q * (1.0 + 0.81 * q))


BUOYANCY_TIE = 1e-3  # m/s^2: |b| below this at some level makes CIN's banking a near-tie


def _tol(w):
    return np.maximum(1.0, 1e-3 * np.abs(w))


def compare_cape(got, want, want64=None, max_status_flip=0.02, max_cin_ties=0.005, what=""):
    """Asserts the parity criteria above; returns a summary dict.

    got: GPU outputs with status; want: FP32 oracle with stats (status,
    bmin); want64: optional FP64 oracle, against which a column that only
    the GPU brought to convergence is checked.
    """
    n = got["cape"].size
    noconv_g = (got["status"] & _lib.COL_NOCONV) != 0
    noconv_w = (want["status"] & _lib.COL_NOCONV) != 0
    flip = noconv_g != noconv_w
    assert flip.sum() <= max(1, max_status_flip * n), (
        f"{what}: {flip.sum()} of {n} convergence flips")
    summary = {"n": n, "flips": int(flip.sum())}
    if want64 is not None:
        # the GPU converged where FP32 Fortran arithmetic cycled: FP64 agrees
        only_gpu = flip & ~noconv_g & ((want64["status"] & _lib.COL_NOCONV) == 0)
        d = np.abs(got["cape"][only_gpu] - want64["cape"][only_gpu])
        assert np.all(d <= _tol(want64["cape"][only_gpu])), f"{what}: converged flips vs FP64"
        summary["flips_checked_vs_f64"] = int(only_gpu.sum())
    keep = ~flip
    g, w = got["cape"][keep].astype(np.float64), want["cape"][keep].astype(np.float64)
    bad = np.abs(g - w) > _tol(w)
    summary["max_abs_cape"] = float(np.max(np.abs(g - w))) if g.size else 0.0
    assert not bad.any(), (f"{what}: cape differs in {bad.sum()} columns, worst "
                           f"{np.max(np.abs(g - w)):.4f} (got {g[bad][:5]} want {w[bad][:5]})")
    g, w = got["cin"][keep].astype(np.float64), want["cin"][keep].astype(np.float64)
    bad = np.abs(g - w) > _tol(w)
    tie = want["bmin"][keep] < BUOYANCY_TIE
    assert not (bad & ~tie).any(), (
        f"{what}: cin differs in {(bad & ~tie).sum()} columns without a buoyancy near-tie "
        f"(got {g[bad & ~tie][:5]} want {w[bad & ~tie][:5]})")
    assert bad.sum() <= max(2, max_cin_ties * n), f"{what}: {bad.sum()} CIN near-ties"
    summary["cin_ties"] = int(bad.sum())
    summary["max_abs_cin_nontie"] = float(np.max(np.abs(g - w)[~tie])) if (~tie).any() else 0.0
    return summary


def oracle_cols(grid, p, t, td, ps, ts, tds, source, adiabat, pinc, ml_depth, start=None,
                precision="f32"):
    """The oracle (loopcape_ml / _pl1d / _pl restated in C) on the same
    columns, with its per-column statistics (status, bmin)."""
    import oracle as O
    n2 = int(np.prod(np.shape(t)[:-1]))
    nk = np.shape(t)[-1]
    t2, td2 = np.reshape(t, (n2, nk)), np.reshape(td, (n2, nk))
    sf = [np.ravel(a) for a in (ps, ts, tds)]
    src, adi = SOURCES.get(source, source), ADIABATS.get(adiabat, adiabat)
    kw = dict(stats=True, precision=precision)
    if grid == 1:
        return O.loopcape(np.reshape(p, (n2, nk)), t2, td2, *sf, pinc, src, ml_depth, adi, **kw)
    if grid == 2:
        st = O.pres_lev_pos(p, sf[0]) if start is None else start
        return O.loopcape(np.ravel(p), t2, td2, *sf, pinc, src, ml_depth, adi, start=st,
                          p_is_1d=True, **kw)
    return O.loopcape(np.reshape(p, (n2, nk)), t2, td2, *sf, pinc, src, ml_depth, adi, start=start,
                      **kw)


def check_vs_fp64(got, ref, what="", min_same_parcel=0.99):
    """The accelerated solvers' contract against the FP64 oracle: no column
    gives up where FP64 converges; CAPE within max(1 J/kg, 0.1 %) wherever
    both lift the same parcel (a most-unstable theta-e near-tie can pick
    another level); CIN within the same bound outside buoyancy near-ties.
    Returns the largest |dCAPE|."""
    conv64 = (ref["status"] & _lib.COL_NOCONV) == 0
    gave_up = (got["status"] & _lib.COL_NOCONV) != 0
    assert not np.any(gave_up & conv64), f"{what}: {np.sum(gave_up & conv64)} columns gave up"
    ok = conv64 & (got["mulvl"] == ref["mulvl"])
    other = int(np.sum(conv64 & ~ok))
    assert other <= max(1, (1.0 - min_same_parcel) * ok.size), (
        f"{what}: {other} of {ok.size} columns lift another parcel")
    d = np.abs(got["cape"][ok].astype(np.float64) - ref["cape"][ok])
    assert np.all(d <= _tol(ref["cape"][ok])), f"{what}: |dCAPE| up to {d.max()}"
    okc = ok & (ref["bmin"] >= BUOYANCY_TIE)
    dc = np.abs(got["cin"][okc].astype(np.float64) - ref["cin"][okc])
    assert np.all(dc <= _tol(ref["cin"][okc])), f"{what}: |dCIN| up to {dc.max()}"
    return float(d.max()) if d.size else 0.0
