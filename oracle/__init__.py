"""CPU oracle for xcape's column kernels -- TEST INFRASTRUCTURE ONLY.

This package is the checker that the CUDA product path is measured against.
Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py``
import it; the ``xcape_gb300`` package never does.

* ``oracle/xcape_oracle.c`` restates the reference Fortran (file:line cited in
  that file) and is built as ``oracle/_build/liboracle.so`` by
  ``oracle/Makefile`` in two precisions: ``'f32'`` is the reference's own
  single-precision arithmetic, ``'f64'`` is the same algorithm in double
  precision (the FP64 comparator).
* This module binds it with ctypes and restates the reference's numpy glue
  (``src/xcape/core.py``: ``_reshape_inputs`` :31-50, ``_reshape_outputs``
  :52-63, ``_reshape_outputs_uv_components`` :65-79,
  ``_reshape_surface_inputs`` :81-100, ``_calc_cape_numpy`` :261-332,
  ``_calc_srh_numpy`` :473-542, ``stdheight.stdheight`` :5-38 and
  ``srh.srh`` :4-66) so that the oracle can be called like the reference.

Parity of the oracle itself is pinned against the reference's golden vectors
(``tests/golden/*.npz``, extracted from the reference's ``test/fixtures.py``
by ``tests/golden/make_golden.py``) in ``tests/test_oracle_golden.py``.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_vp = ctypes.c_void_p
_int = ctypes.c_int

COL_NOCONV = 1
COL_BADSTART = 2


def build(force=False):
    """Compile liboracle.so with the committed Makefile."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        for prec, rp, rt in (("f32", _f32p, ctypes.c_float), ("f64", _f64p, ctypes.c_double)):
            f = getattr(L, f"oc_loopcape_ml_{prec}")
            f.argtypes = [rp, rp, rp, rp, rp, rp, rt, _int, rt, _int, _int, _int,
                          rp, rp, _i32p, rp, _vp, _vp, _vp, _vp, _int]
            f.restype = None
            for name in (f"oc_loopcape_pl1d_{prec}", f"oc_loopcape_pl_{prec}"):
                f = getattr(L, name)
                f.argtypes = [rp, rp, rp, rp, rp, rp, rt, _int, rt, _int, _i32p, _int, _int,
                              rp, rp, _i32p, rp, _vp, _vp, _vp, _vp, _int]
                f.restype = None
            f = getattr(L, f"oc_loopcape_diag_ml_{prec}")
            f.argtypes = [rp, rp, rp, rp, rp, rp, rt, _int, rt, _int, _int, _int,
                          rp, rp, _i32p, rp, _vp, rp, _int]
            f.restype = None
            f = getattr(L, f"oc_loopcape_diag_pl1d_{prec}")
            f.argtypes = [rp, rp, rp, rp, rp, rp, rt, _int, rt, _int, _i32p, _int, _int,
                          rp, rp, _i32p, rp, _vp, rp, _int]
            f.restype = None
            f = getattr(L, f"oc_bunkers_loop_ml_{prec}")
            f.argtypes = [rp, rp, rp, rp, rp, rp, _int, _int, rp, rp, rp, _int]
            f.restype = None
            f = getattr(L, f"oc_bunkers_loop_pl_{prec}")
            f.argtypes = [rp, rp, rp, rp, rp, rp, _i32p, _int, _int, rp, rp, rp, _int]
            f.restype = None
        L.oc_loop_stdheight_ml.argtypes = [_f64p] * 7 + [_int, _int, _f64p, _f64p, _int]
        L.oc_loop_stdheight_pl1d.argtypes = [_f64p] * 7 + [_i32p, _int, _int, _f64p, _f64p, _int]
        L.oc_loop_stdheight_pl.argtypes = [_f64p] * 7 + [_i32p, _int, _int, _f64p, _f64p, _int]
        L.oc_loop_sreh_ml.argtypes = [_f64p] * 10 + [ctypes.c_double, _int, _int, _f64p, _f64p, _int]
        L.oc_loop_sreh_pl.argtypes = [_f64p] * 10 + [ctypes.c_double, _i32p, _int, _int, _f64p,
                                                     _f64p, _int]
        L.oc_max_threads.restype = _int
        _lib = L
    return _lib


def max_threads():
    return lib().oc_max_threads()


def _dt(precision):
    if precision not in ("f32", "f64"):
        raise ValueError("precision must be 'f32' or 'f64'")
    return np.float32 if precision == "f32" else np.float64


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


# ---------------------------------------------------------------------------
# Column-loop entry points.  2-D arrays are (n2, nk) C-contiguous, i.e. the
# memory layout of the Fortran (nk, n2) arrays of the f2py interfaces.

DIAG_FIELDS = ("plfc", "zlfc", "pel", "zel", "zsource", "thetae_source")


def loopcape_diag(p, t, td, ps, ts, tds, pinc, source, ml_depth, adiabat, start=None,
                  precision="f32", nthreads=0):
    """loopcape_ml (start None) or loopcape_pl1d (1-D p) with the diagnostics
    getcape computes and discards: a dict with cape, cin, mulvl, z_out,
    status and the DIAG_FIELDS arrays (LFC/EL pressure in hPa and height in
    m, source height, source theta-e; -999999 where undefined)."""
    dt = _dt(precision)
    t = _c(t, dt)
    n2, nk = t.shape
    td = _c(td, dt)
    ps, ts, tds = (_c(np.ravel(x), dt) for x in (ps, ts, tds))
    cape, cin, zout = (np.empty(n2, dt) for _ in range(3))
    mulvl = np.empty(n2, np.int32)
    status = np.zeros(n2, np.int32)
    diag = np.empty((n2, 6), dt)
    L = lib()
    if start is None:
        getattr(L, f"oc_loopcape_diag_ml_{precision}")(
            _c(p, dt), t, td, ps, ts, tds, pinc, source, ml_depth, adiabat, nk, n2, cape, cin,
            mulvl, zout, status.ctypes.data, diag, nthreads)
    else:
        getattr(L, f"oc_loopcape_diag_pl1d_{precision}")(
            t, td, _c(np.ravel(p), dt), ps, ts, tds, pinc, source, ml_depth, adiabat,
            _c(np.ravel(start), np.int32), nk, n2, cape, cin, mulvl, zout, status.ctypes.data,
            diag, nthreads)
    out = dict(cape=cape, cin=cin, mulvl=mulvl, z_out=zout, status=status)
    out.update({k: diag[:, j] for j, k in enumerate(DIAG_FIELDS)})
    return out


def loopcape(p, t, td, ps, ts, tds, pinc, source, ml_depth, adiabat, start=None, p_is_1d=False,
             precision="f32", nthreads=0, stats=False):
    """loopcape_ml (start is None), loopcape_pl1d (p_is_1d) or loopcape_pl."""
    dt = _dt(precision)
    t = _c(t, dt)
    n2, nk = t.shape
    td = _c(td, dt)
    p = _c(p, dt)
    ps, ts, tds = (_c(np.ravel(x), dt) for x in (ps, ts, tds))
    cape = np.empty(n2, dt)
    cin = np.empty(n2, dt)
    mulvl = np.empty(n2, np.int32)
    zout = np.empty(n2, dt)
    nsub = np.zeros(n2, np.int32) if stats else None
    niter = np.zeros(n2, np.int32) if stats else None
    status = np.zeros(n2, np.int32) if stats else None
    bmin = np.zeros(n2, np.float32) if stats else None
    ptr = lambda a: a.ctypes.data if a is not None else None
    L = lib()
    if start is None:
        getattr(L, f"oc_loopcape_ml_{precision}")(
            p, t, td, ps, ts, tds, pinc, source, ml_depth, adiabat, nk, n2,
            cape, cin, mulvl, zout, ptr(nsub), ptr(niter), ptr(status), ptr(bmin), nthreads)
    else:
        start = _c(np.ravel(start), np.int32)
        name = f"oc_loopcape_pl1d_{precision}" if p_is_1d else f"oc_loopcape_pl_{precision}"
        if p_is_1d:
            args = (t, td, _c(np.ravel(p), dt))
        else:
            args = (p, t, td)
        getattr(L, name)(*args, ps, ts, tds, pinc, source, ml_depth, adiabat, start, nk, n2,
                         cape, cin, mulvl, zout, ptr(nsub), ptr(niter), ptr(status), ptr(bmin), nthreads)
    out = dict(cape=cape, cin=cin, mulvl=mulvl, z_out=zout)
    if stats:
        out.update(nsub=nsub, niter=niter, status=status, bmin=bmin)
    return out


def loop_stdheight(p, t, td, ps, ts, tds, hin, start=None, p_is_1d=False, nthreads=0):
    t = _c(t, np.float64)
    n2, nk = t.shape
    td = _c(td, np.float64)
    ps, ts, tds, hin = (_c(np.ravel(x), np.float64) for x in (ps, ts, tds, hin))
    H = np.empty((n2, nk), np.float64)
    Hs = np.empty(n2, np.float64)
    L = lib()
    if start is None:
        L.oc_loop_stdheight_ml(_c(p, np.float64), t, td, ps, ts, tds, hin, nk, n2, H, Hs, nthreads)
    elif p_is_1d:
        L.oc_loop_stdheight_pl1d(t, td, _c(np.ravel(p), np.float64), ps, ts, tds, hin,
                                 _c(np.ravel(start), np.int32), nk, n2, H, Hs, nthreads)
    else:
        L.oc_loop_stdheight_pl(_c(p, np.float64), t, td, ps, ts, tds, hin,
                               _c(np.ravel(start), np.int32), nk, n2, H, Hs, nthreads)
    return H, Hs


def bunkers_loop(u, v, aglh, us, vs, aglhs, start=None, precision="f32", nthreads=0):
    dt = _dt(precision)
    u = _c(u, dt)
    n2, nk = u.shape
    v, aglh = _c(v, dt), _c(aglh, dt)
    us, vs, aglhs = (_c(np.ravel(x), dt) for x in (us, vs, aglhs))
    rm = np.zeros((n2, 2), dt)
    lm = np.zeros((n2, 2), dt)
    mean = np.zeros((n2, 2), dt)
    L = lib()
    if start is None:
        getattr(L, f"oc_bunkers_loop_ml_{precision}")(u, v, aglh, us, vs, aglhs, nk, n2, rm, lm,
                                                     mean, nthreads)
    else:
        getattr(L, f"oc_bunkers_loop_pl_{precision}")(u, v, aglh, us, vs, aglhs,
                                                     _c(np.ravel(start), np.int32), nk, n2, rm,
                                                     lm, mean, nthreads)
    return rm, lm, mean


def loop_sreh(u, v, aglh, us, vs, aglhs, cu_rm, cv_rm, cu_lm, cv_lm, top, start=None, nthreads=0):
    u = _c(u, np.float64)
    n2, nk = u.shape
    v, aglh = _c(v, np.float64), _c(aglh, np.float64)
    rest = [_c(np.ravel(x), np.float64) for x in (us, vs, aglhs, cu_rm, cv_rm, cu_lm, cv_lm)]
    srm = np.empty(n2, np.float64)
    slm = np.empty(n2, np.float64)
    L = lib()
    if start is None:
        L.oc_loop_sreh_ml(u, v, aglh, *rest, float(top), nk, n2, srm, slm, nthreads)
    else:
        L.oc_loop_sreh_pl(u, v, aglh, *rest, float(top), _c(np.ravel(start), np.int32), nk, n2,
                          srm, slm, nthreads)
    return srm, slm


# ---------------------------------------------------------------------------
# Restatement of the reference's numpy glue (src/xcape/core.py).

SOURCE = {"surface": 1, "most-unstable": 2, "mixed-layer": 3}
ADIABAT = {"pseudo-liquid": 1, "reversible-liquid": 2, "pseudo-ice": 3, "reversible-ice": 4}


def _columns(*arrays):
    """core.py:31-50 without the transpose: (..., nlev) -> (ncol, nlev)."""
    shape = arrays[0].shape
    for a in arrays:
        if a.shape != shape:
            raise ValueError("Input arrays must have the same shape.")
    a2 = [np.atleast_2d(a) for a in arrays]
    nlev = a2[0].shape[-1]
    return [np.reshape(a, (-1, nlev)) for a in a2]


def _surface(*arrays):
    """core.py:81-100."""
    shape = arrays[0].shape
    for a in arrays:
        if a.shape != shape:
            raise ValueError("Input arrays must have the same shape.")
    return [np.reshape(np.atleast_1d(a), (-1,)) for a in arrays]


def _out_shape(shape):
    """core.py:59-62."""
    return (1,) if len(shape) == 1 else shape[:-1]


def pres_lev_pos(p1d, ps1d):
    """core.py:286-289: masked argmin of ps - p over levels, Fortran 1-based."""
    p_2d = np.reshape(np.atleast_2d(p1d), (1, -1)).T  # (nlev, 1)
    temp_index = ps1d - p_2d
    return (np.ma.masked_less(temp_index, 0).argmin(axis=0) + 1).astype(np.int32)


def calc_cape(p, t, td, ps, ts, tds, source="surface", ml_depth=500.0, adiabat="pseudo-liquid",
              pinc=500.0, vertical_lev="sigma", precision="f32", nthreads=0, stats=False):
    """core.py:261-332 with the oracle in place of cape_fortran.cape."""
    if vertical_lev == "model":
        vertical_lev = "sigma"
    original_shape = t.shape
    ps1, ts1, tds1 = _surface(ps, ts, tds)
    if np.ndim(p) == 1:
        t2, td2 = _columns(t, td)
        start = pres_lev_pos(p, ps1)
        out = loopcape(np.ravel(p), t2, td2, ps1, ts1, tds1, pinc, SOURCE[source], ml_depth,
                       ADIABAT[adiabat], start=start, p_is_1d=True, precision=precision,
                       nthreads=nthreads, stats=stats)
    elif p.shape == t.shape and vertical_lev == "sigma":
        p2, t2, td2 = _columns(p, t, td)
        out = loopcape(p2, t2, td2, ps1, ts1, tds1, pinc, SOURCE[source], ml_depth,
                       ADIABAT[adiabat], precision=precision, nthreads=nthreads, stats=stats)
    else:
        raise ValueError("P should be 1d")
    shp = _out_shape(original_shape)
    res = [out["cape"].reshape(shp), out["cin"].reshape(shp)]
    if SOURCE[source] == 2:
        res += [out["mulvl"].reshape(shp), out["z_out"].reshape(shp)]
    if stats:
        return tuple(res), out
    return tuple(res)


def calc_srh(p, t, td, u, v, ps, ts, tds, us, vs, depth=3000, vertical_lev="sigma",
             output_var="srh", precision="f32", nthreads=0):
    """core.py:473-542 + stdheight.py:5-38 + srh.py:4-66 with the oracle."""
    if vertical_lev == "model":
        vertical_lev = "sigma"
    original_shape = t.shape
    ps1, ts1, tds1, us1, vs1 = _surface(ps, ts, tds, us, vs)
    if np.ndim(p) == 1:
        t2, td2, u2, v2 = _columns(t, td, u, v)
        start = pres_lev_pos(p, ps1)
        p1 = np.ravel(p)
        hin = np.ones(t2.shape[0]) * 2.0
        H, Hs = loop_stdheight(p1, t2, td2, ps1, ts1, tds1, hin, start=start, p_is_1d=True,
                               nthreads=nthreads)
    elif p.shape == t.shape and vertical_lev == "sigma":
        p2, t2, td2, u2, v2 = _columns(p, t, td, u, v)
        start = None
        hin = np.ones(t2.shape[0]) * 2.0
        H, Hs = loop_stdheight(p2, t2, td2, ps1, ts1, tds1, hin, nthreads=nthreads)
    else:
        raise ValueError("P should be 1d")
    rm, lm, mean = bunkers_loop(u2, v2, H, us1, vs1, Hs, start=start, precision=precision,
                                nthreads=nthreads)
    srm, slm = loop_sreh(u2, v2, H, us1, vs1, Hs, rm[:, 0], rm[:, 1], lm[:, 0], lm[:, 1], depth,
                         start=start, nthreads=nthreads)
    shp = _out_shape(original_shape)
    if output_var == "srh":
        return srm.reshape(shp), slm.reshape(shp)
    uvshape = (2,) if len(original_shape) == 1 else (2,) + tuple(original_shape[:-1])
    rm2, lm2, mean2 = (np.reshape(np.ascontiguousarray(a.T), uvshape) for a in (rm, lm, mean))
    return (srm.reshape(shp), slm.reshape(shp), rm2[0], rm2[1], lm2[0], lm2[1], mean2[0],
            mean2[1])
