"""calc_cape / calc_srh with the reference's signatures, computed on the GPU.

Mirrors ``src/xcape/core.py`` of xcape:

* ``calc_cape(p, t, td, ps, ts, tds, source='surface', ml_depth=500.,
  adiabat='pseudo-liquid', pinc=500., method='cuda', vertical_lev='sigma')``
  (core.py:130-235, 261-332) returns ``(cape, cin)`` or, for
  ``source='most-unstable'``, ``(cape, cin, mulev, zmulev)``;
* ``calc_srh(p, t, td, u, v, ps, ts, tds, us, vs, depth=3000,
  vertical_lev='sigma', output_var='srh', method='cuda')`` (core.py:335-447,
  473-542) returns ``(srh_rm, srh_lm)`` or, for ``output_var='all'``, eight
  arrays ``srh_rm, srh_lm, rm_u, rm_v, lm_u, lm_v, mean_6km_u, mean_6km_v``.

The vertical axis is the LAST axis of the 3-D inputs, as in the reference's
tests (test/test_core.py:22-26, 77-82).  ``vertical_lev`` accepts
``'sigma'``, ``'model'`` (an alias of ``'sigma'``) and ``'pressure'`` (1-D
``p`` shared by all columns; levels below the surface are skipped per column
with the reference's ``pres_lev_pos`` rule, evaluated on the GPU).

``calc_cape_srh`` computes both for the same columns in one pass.

Methods:

* ``'cuda'`` -- the GB300 kernels of ``libxcape_gb300.so``.  numpy inputs go
  through the library's host entry points (the arrays are staged to the
  device and back inside the call); torch CUDA tensors are used in place and
  the results are returned as CUDA tensors on the caller's current stream.
* ``'dummy'`` -- the reference's shape-test backend (core.py:107-121).
* ``'fortran'`` -- delegates to an installed reference ``xcape`` package (its
  compiled Fortran); raises ImportError when that is not installed.

Differences from the reference that a caller can observe are deliberate and
limited to error handling: unknown option strings raise ``ValueError``
instead of ``KeyError``, ``vertical_lev`` defaults to ``'sigma'`` instead of
raising ``KeyError`` when omitted, and option codes the Fortran would
``stop`` on are rejected before any work is done.
"""
from functools import reduce

import numpy as np

from . import _lib

_SOURCE = {"surface": 1, "most-unstable": 2, "mixed-layer": 3}
_ADIABAT = {"pseudo-liquid": 1, "reversible-liquid": 2, "pseudo-ice": 3, "reversible-ice": 4}
_VERTICAL = {"sigma": 1, "model": 1, "pressure": 2}
_OUTPUT = {"srh": 1, "all": 2}
_GUESS = {"plain": _lib.XC_GUESS_PLAIN, "learned": _lib.XC_GUESS_LEARNED,
          "extrapolated": _lib.XC_GUESS_EXTRAPOLATED, "secant": _lib.XC_GUESS_SECANT,
          "learned-every": _lib.XC_GUESS_LEARNED_EVERY, "learned-warp": _lib.XC_GUESS_LEARNED_WARP}


def _is_torch(a):
    return type(a).__module__.startswith("torch") and hasattr(a, "data_ptr")


def _prod(v):
    return reduce(lambda x, y: x * y, v, 1)


def _option(table, value, name):
    try:
        return table[value]
    except (KeyError, TypeError):
        raise ValueError(f"`{name}` must be one of: {list(table)}") from None


def _out_shape(shape):
    """core.py:59-62: the input shape without its vertical axis."""
    return (1,) if len(shape) == 1 else tuple(shape[:-1])


def _check_same(arrays):
    shape = tuple(arrays[0].shape)
    for a in arrays:
        if tuple(a.shape) != shape:
            raise ValueError("Input arrays must have the same shape.")


def _any_dask_array(*args):
    try:
        import dask.array as da
    except ImportError:
        return False
    return any(isinstance(a, da.Array) for a in args)


# ---------------------------------------------------------------------------
# numpy / torch marshalling


class _Batch:
    """Inputs of one call in the layout the library binds: 3-D arrays as
    contiguous (ncol, nlev), surface arrays as (ncol,), one dtype."""

    def __init__(self, level_arrays, surface_arrays, p, grid):
        self.torch = any(_is_torch(a) for a in (p, *level_arrays, *surface_arrays))
        allx = (p, *level_arrays, *surface_arrays)
        if self.torch:
            import torch
            dev = None
            for a in allx:
                if not _is_torch(a) or not a.is_cuda:
                    raise ValueError("torch inputs must all be CUDA tensors")
                dev = a.device if dev is None else dev
                if a.device != dev:
                    raise ValueError("torch inputs must be on one device")
            f64 = any(a.dtype == torch.float64 for a in allx)
            self.tdtype = torch.float64 if f64 else torch.float32
            self.device = dev
            conv = lambda a: a.to(self.tdtype).contiguous()
            self.stream = torch.cuda.current_stream(dev).cuda_stream
        else:
            allx = [np.asarray(a) for a in allx]
            f64 = any(a.dtype != np.float32 for a in allx)
            self.ndtype = np.float64 if f64 else np.float32
            conv = lambda a: np.ascontiguousarray(np.asarray(a), dtype=self.ndtype)
            self.stream = None
        self.dtype = _lib.XC_F64 if f64 else _lib.XC_F32
        nlev = level_arrays[0].shape[-1]
        ncol = _prod(tuple(level_arrays[0].shape[:-1]))
        self.nk, self.n2 = int(nlev), int(ncol)
        self.levels = [conv(a).reshape(self.n2, self.nk) for a in level_arrays]
        self.surface = [conv(a).reshape(self.n2) for a in surface_arrays]
        if grid == _lib.GRID_SIGMA:
            self.p = conv(p).reshape(self.n2, self.nk)
        else:
            self.p = conv(p).reshape(self.nk)

    def ptr(self, a):
        if a is None:
            return None
        return a.data_ptr() if self.torch else a.ctypes.data

    def workspace(self, nbytes):
        """A 256-byte aligned device scratch buffer (torch's caching
        allocator), kept alive on the batch until the call returns."""
        import torch
        buf = torch.empty(nbytes + 256, dtype=torch.uint8, device=self.device)
        self._ws = buf
        ptr = buf.data_ptr()
        return ptr + (-ptr) % 256, nbytes

    def empty(self, n, kind):
        if self.torch:
            import torch
            dt = {"f4": torch.float32, "f8": torch.float64, "i4": torch.int32}[kind]
            return torch.empty(n, dtype=dt, device=self.device)
        return np.empty(n, dtype=kind)


# ---------------------------------------------------------------------------
# CAPE


def _cape_dummy(p, t, td, ps, ts, tds, **kwargs):
    """core.py:107-121: a fake backend returning ones, for shape tests."""
    assert p.ndim == 2
    shape = t.shape
    one = np.ones((1, shape[1]))
    return one, one.copy(), one.copy(), one.copy()


def calc_cape(*args, **kwargs):
    """Convective Available Potential Energy (CAPE) and Convective Inhibition
    (CIN) of every column (reference: src/xcape/core.py:130-235).

    Parameters follow the reference: ``p`` (hPa; same shape as ``t`` for
    ``vertical_lev='sigma'``/``'model'``, 1-D for ``'pressure'``), ``t``, ``td``
    (degC, vertical axis last), ``ps`` (hPa), ``ts``, ``tds`` (degC).
    Keywords: ``source``, ``ml_depth`` (m), ``adiabat``, ``pinc`` (Pa),
    ``method`` (``'cuda'``, ``'dummy'``, ``'fortran'``), ``vertical_lev``, and
    ``guess``: the moist-adiabat solver. ``'plain'`` is the reference's
    iteration.  ``fp64_retry=True`` lifts again, in double precision with the
    reference's iteration, the columns whose FP32 iteration gave up after 100
    steps (the reference then returns CAPE = CIN = 0; FP32 rounding causes
    that on a few percent of warm, noisy columns where FP64 converges).  The others keep its stopping test and take secant steps:
    ``'extrapolated'`` (first guess from the previous sub-step's increment),
    ``'learned'`` (as extrapolated, with the trained guess network's guess on
    the first saturated sub-step), ``'secant'`` (the reference's first
    guess), ``'learned-every'`` (the network's guess on every saturated
    sub-step).

    Returns ``(cape, cin)`` (J/kg, float32) or ``(cape, cin, mulev, zmulev)``
    for ``source='most-unstable'`` (int32 level index counted with the
    surface as 1; float32 height in m).
    """
    if len(args) < 6:
        raise ValueError("Too few arguments.")
    if len(args) > 6:
        raise ValueError("Too many arguments.")
    vertical_lev = kwargs.get("vertical_lev", "sigma")
    if vertical_lev not in _VERTICAL:
        raise ValueError(f"`vertical_lev` must be one of: {list(_VERTICAL)}")
    if _any_dask_array(*args):
        return _calc_cape_gufunc(*args, **kwargs)
    return _calc_cape_numpy(*args, **kwargs)


def _calc_cape_gufunc(*args, **kwargs):
    """dask arrays: one library call per chunk of columns (core.py:237-258).
    The 1-D ``p`` of pressure levels is bound to every chunk's call rather
    than passed as a gufunc argument (the reference's pressure signature
    lists seven inputs for six arrays, core.py:245-247); the level axis is
    the trailing core dimension, so no ``axis`` argument is passed."""
    import dask.array as da
    vertical_lev = kwargs.get("vertical_lev", "sigma")
    signature = "(i),(i),(i),(),(),()->(),()"
    output_dtypes = ("f4", "f4")
    if kwargs.get("source", "surface") == "most-unstable":
        signature += ",(),()"
        output_dtypes = output_dtypes + ("i4", "f4")
    if vertical_lev == "pressure":
        p, rest = args[0], args[1:]
        p_np = np.asarray(p)

        def f(t, td, ps, ts, tds, **kw):
            return _calc_cape_numpy(p_np, t, td, ps, ts, tds, **kw)
        sig = signature.replace("(i),(i),(i)", "(i),(i)", 1)
        return da.apply_gufunc(f, sig, *rest, output_dtypes=output_dtypes,
                               vectorize=False, **kwargs)
    return da.apply_gufunc(_calc_cape_numpy, signature, *args, output_dtypes=output_dtypes,
                           vectorize=False, **kwargs)


def _cape_grid(p, t, td, ps, ts, tds, vl):
    """The grid kind and the 3-D shape of one calc_cape call, with the
    reference's shape checks (core.py:278-300)."""
    original_shape = tuple(t.shape)
    _check_same([t, td])
    _check_same([ps, ts, tds])
    if len(p.shape) == 1 and vl == _lib.GRID_PRESSURE_1D:
        grid = _lib.GRID_PRESSURE_1D
        if p.shape[0] != t.shape[-1]:
            raise ValueError("1-D p must have one value per level of t")
    elif tuple(p.shape) == original_shape and vl == _lib.GRID_SIGMA:
        grid = _lib.GRID_SIGMA
    elif tuple(p.shape) == original_shape and vl == _lib.GRID_PRESSURE_1D:
        raise ValueError("P should be 1d")
    else:
        raise ValueError("Input arrays must have the same shape.")
    if _prod(tuple(ps.shape)) != _prod(original_shape[:-1]):
        raise ValueError("Surface arrays must have one value per column.")
    return grid, original_shape


def _calc_cape_numpy(*args, source="surface", ml_depth=500.0, adiabat="pseudo-liquid",
                     pinc=500.0, method="cuda", vertical_lev="sigma", guess="plain",
                     fp64_retry=False):
    p, t, td, ps, ts, tds = args
    src = _option(_SOURCE, source, "source")
    adi = _option(_ADIABAT, adiabat, "adiabat")
    vl = _option(_VERTICAL, vertical_lev, "vertical_lev")
    gs = _option(_GUESS, guess, "guess")
    grid, original_shape = _cape_grid(p, t, td, ps, ts, tds, vl)

    if method == "dummy":
        p2 = np.reshape(np.atleast_2d(np.asarray(p)), (-1, np.asarray(p).shape[-1])).T
        t2 = np.reshape(np.atleast_2d(np.asarray(t)), (-1, original_shape[-1])).T
        outs = _cape_dummy(p2, t2, None, None, None, None)
        shp = _out_shape(original_shape)
        res = [np.reshape(o.T, shp) for o in outs]
        return tuple(res) if src == 2 else tuple(res[:2])
    if method == "fortran":
        return _reference_fortran_cape(p, t, td, ps, ts, tds, source=source, ml_depth=ml_depth,
                                       adiabat=adiabat, pinc=pinc, vertical_lev=vertical_lev)
    if method != "cuda":
        raise ValueError("invalid method")

    if gs in (_lib.XC_GUESS_LEARNED, _lib.XC_GUESS_LEARNED_EVERY, _lib.XC_GUESS_LEARNED_WARP):
        from . import guess as _guess
        _guess.ensure_loaded()
    b = _Batch([t, td], [ps, ts, tds], p, grid)
    cape, cin, zout = (b.empty(b.n2, "f4") for _ in range(3))
    mulvl = b.empty(b.n2, "i4")
    status = None
    if fp64_retry:
        gs |= _lib.XC_RETRY_FP64
        if b.torch:
            status = b.empty(b.n2, "i4")  # the device path carries the flags in it
    args_ = (grid, b.ptr(b.p), b.ptr(b.levels[0]), b.ptr(b.levels[1]), b.ptr(b.surface[0]),
             b.ptr(b.surface[1]), b.ptr(b.surface[2]), b.dtype, float(pinc), src,
             float(ml_depth), adi, None, b.nk, b.n2, gs, b.ptr(cape), b.ptr(cin), b.ptr(mulvl),
             b.ptr(zout), b.ptr(status))
    if b.torch:
        ws, ws_bytes = b.workspace(_lib.workspace_bytes(b.n2))
        _lib.call("xc_loopcape_ex", *args_, None, ws, ws_bytes, b.stream)
    else:
        _lib.call("xc_loopcape_ex_host", *args_, None)
    shp = _out_shape(original_shape)
    res = [cape.reshape(shp), cin.reshape(shp)]
    if src == 2:
        res += [mulvl.reshape(shp), zout.reshape(shp)]
    return tuple(res)


def calc_cape_sources(p, t, td, ps, ts, tds, sources=("most-unstable", "mixed-layer"),
                      ml_depth=500.0, adiabat="pseudo-liquid", pinc=500.0, vertical_lev="sigma",
                      guess="plain", fp64_retry=False):
    """``calc_cape`` for several parcel sources of the same columns in one
    call: ``{source: calc_cape(p, t, td, ps, ts, tds, source=source, ...)}``
    for each entry of ``sources`` (each of ``'surface'``, ``'most-unstable'``,
    ``'mixed-layer'`` at most once), with the same values.

    The reference computes each source with its own ``calc_cape`` call
    (src/xcape/core.py:130-235), so numpy inputs would cross to the device
    once per source; here they cross once (``xc_loopcape_multi_host``), and
    the columns are ordered once for all the sources.  CUDA tensors are used
    in place (``xc_loopcape_multi``: one ordering, one launch per source).
    ``guess`` and ``fp64_retry`` as in ``calc_cape``.
    """
    names = list(sources)
    if not names or len(set(names)) != len(names):
        raise ValueError("sources must name each source at most once")
    codes = [_option(_SOURCE, src, "source") for src in names]
    adi = _option(_ADIABAT, adiabat, "adiabat")
    vl = _option(_VERTICAL, vertical_lev, "vertical_lev")
    gs = _option(_GUESS, guess, "guess")
    grid, original_shape = _cape_grid(p, t, td, ps, ts, tds, vl)
    if gs in (_lib.XC_GUESS_LEARNED, _lib.XC_GUESS_LEARNED_EVERY, _lib.XC_GUESS_LEARNED_WARP):
        from . import guess as _guess
        _guess.ensure_loaded()
    b = _Batch([t, td], [ps, ts, tds], p, grid)
    ns = len(codes)
    cape, cin, zout = (b.empty(ns * b.n2, "f4") for _ in range(3))
    mulvl = b.empty(ns * b.n2, "i4")
    status = None
    if fp64_retry:
        gs |= _lib.XC_RETRY_FP64
        if b.torch:
            status = b.empty(ns * b.n2, "i4")
    common = (grid, b.ptr(b.p), b.ptr(b.levels[0]), b.ptr(b.levels[1]), b.ptr(b.surface[0]),
              b.ptr(b.surface[1]), b.ptr(b.surface[2]), b.dtype, float(pinc))
    import ctypes
    arr = (ctypes.c_int * ns)(*codes)
    if b.torch:
        ws, ws_bytes = b.workspace(_lib.workspace_bytes(b.n2))
        _lib.call("xc_loopcape_multi", *common, ns, ctypes.cast(arr, ctypes.c_void_p),
                  float(ml_depth), adi, None, b.nk, b.n2, gs, b.ptr(cape), b.ptr(cin),
                  b.ptr(mulvl), b.ptr(zout), None if status is None else b.ptr(status), None, ws,
                  ws_bytes, b.stream)
    else:
        _lib.call("xc_loopcape_multi_host", *common, ns, ctypes.cast(arr, ctypes.c_void_p),
                  float(ml_depth), adi, None, b.nk, b.n2, gs, b.ptr(cape), b.ptr(cin),
                  b.ptr(mulvl), b.ptr(zout), None, None)
    shp = _out_shape(original_shape)
    out = {}
    for j, (name, code) in enumerate(zip(names, codes)):
        sl = slice(j * b.n2, (j + 1) * b.n2)
        res = [cape[sl].reshape(shp), cin[sl].reshape(shp)]
        if code == 2:
            res += [mulvl[sl].reshape(shp), zout[sl].reshape(shp)]
        out[name] = tuple(res)
    return out


DIAG_FIELDS = ("plfc", "zlfc", "pel", "zel", "zsource", "thetae_source")


def calc_cape_diagnostics(p, t, td, ps, ts, tds, source="surface", ml_depth=500.0,
                          adiabat="pseudo-liquid", pinc=500.0, vertical_lev="sigma",
                          guess="plain"):
    """calc_cape with the diagnostics the reference's getcape computes and
    discards (CAPE_CODE_model_lev.f90:505, :511, :526), in one pass on the GPU.

    Arguments as ``calc_cape`` (numpy arrays, or CUDA tensors used in place);
    ``guess`` is ``'plain'`` or ``'learned'``.  Returns a dict of arrays shaped
    like ``ps``: ``cape``, ``cin``, ``mulev``, ``zmulev`` (as calc_cape), and
    ``plfc``, ``zlfc`` (level of free convection: the lowest point of the first
    layer with positive area, hPa and m), ``pel``, ``zel`` (equilibrium level:
    the highest positive-to-negative crossing, or the last level reached while
    still buoyant), ``zsource`` and ``thetae_source`` (height and theta-e of the
    lifted parcel's source).  -999999 where undefined.
    """
    src = _option(_SOURCE, source, "source")
    adi = _option(_ADIABAT, adiabat, "adiabat")
    vl = _option(_VERTICAL, vertical_lev, "vertical_lev")
    gs = _option(_GUESS, guess, "guess")
    if gs not in (_lib.XC_GUESS_PLAIN, _lib.XC_GUESS_LEARNED):
        raise ValueError("calc_cape_diagnostics: guess must be 'plain' or 'learned'")
    if gs == _lib.XC_GUESS_LEARNED:
        from . import guess as _guess
        _guess.ensure_loaded()
    _check_same([t, td])
    _check_same([ps, ts, tds])
    shape = tuple(t.shape)
    if len(p.shape) == 1 and vl == _lib.GRID_PRESSURE_1D:
        grid = _lib.GRID_PRESSURE_1D
        if p.shape[0] != shape[-1]:
            raise ValueError("1-D p must have one value per level of t")
    elif tuple(p.shape) == shape and vl == _lib.GRID_SIGMA:
        grid = _lib.GRID_SIGMA
    else:
        raise ValueError("Input arrays must have the same shape.")
    import torch
    host = not any(_is_torch(a) for a in (p, t, td, ps, ts, tds))
    if host:
        p, t, td, ps, ts, tds = (torch.from_numpy(np.ascontiguousarray(a)).cuda()
                                 for a in (p, t, td, ps, ts, tds))
    b = _Batch([t, td], [ps, ts, tds], p, grid)
    cape, cin, zout = (b.empty(b.n2, "f4") for _ in range(3))
    mulvl = b.empty(b.n2, "i4")
    diag = b.empty(6 * b.n2, "f4")
    _lib.call("xc_loopcape_diag", grid, b.ptr(b.p), b.ptr(b.levels[0]), b.ptr(b.levels[1]),
              b.ptr(b.surface[0]), b.ptr(b.surface[1]), b.ptr(b.surface[2]), b.dtype,
              float(pinc), src, float(ml_depth), adi, None, b.nk, b.n2, gs, b.ptr(cape),
              b.ptr(cin), b.ptr(mulvl), b.ptr(zout), None, b.ptr(diag), b.stream)
    shp = _out_shape(shape)
    out = {"cape": cape, "cin": cin, "mulev": mulvl, "zmulev": zout}
    d = diag.reshape(b.n2, 6)
    out.update({k: d[:, j] for j, k in enumerate(DIAG_FIELDS)})
    out = {k: v.reshape(shp) for k, v in out.items()}
    if host:
        out = {k: v.cpu().numpy() for k, v in out.items()}
    return out


# ---------------------------------------------------------------------------
# SRH


def calc_srh(*args, **kwargs):
    """Storm-relative helicity with Bunkers storm motion (reference:
    src/xcape/core.py:335-447).

    Parameters follow the reference: ``p, t, td, u, v`` (hPa, degC, degC, m/s,
    m/s; vertical axis last; ``p`` 1-D for ``vertical_lev='pressure'``),
    ``ps, ts, tds, us, vs`` (surface), ``depth`` (m), ``vertical_lev``,
    ``output_var`` (``'srh'`` or ``'all'``), ``method`` (``'cuda'`` or
    ``'fortran'``) and ``precision``: ``'reference'`` keeps the reference's
    FP64 height and helicity stages; ``'fp32'`` runs them in FP32 with
    compensated sums (tens of times faster on this GPU, whose FP64 rate is a
    small fraction of its FP32 rate; differences from the reference far inside
    0.5 m^2/s^2).
    """
    if len(args) != 10:
        raise ValueError("calc_srh takes 10 positional arrays.")
    if _any_dask_array(*args):
        return _calc_srh_gufunc(*args, **kwargs)
    return _calc_srh_numpy(*args, **kwargs)


def _calc_srh_gufunc(*args, **kwargs):
    """dask arrays (core.py:449-470), one library call per chunk."""
    import dask.array as da
    signature = "(i),(i),(i),(i),(i),(),(),(),(),()->(),()"
    output_dtypes = ("f8", "f8")
    if kwargs.get("output_var", "srh") == "all":
        signature += ",(),(),(),(),(),()"
        output_dtypes = output_dtypes + ("f4",) * 6
    if kwargs.get("vertical_lev", "sigma") == "pressure":
        p_np = np.asarray(args[0])

        def f(*a, **kw):
            return _calc_srh_numpy(p_np, *a, **kw)
        return da.apply_gufunc(f, signature.replace("(i),", "", 1), *args[1:],
                               output_dtypes=output_dtypes, vectorize=False, **kwargs)
    return da.apply_gufunc(_calc_srh_numpy, signature, *args, output_dtypes=output_dtypes,
                           vectorize=False, **kwargs)


_SRH_PRECISION = {"reference": 0, "fp32": 1}


def _calc_srh_numpy(*args, depth=3000, vertical_lev="sigma", output_var="srh", method="cuda",
                    precision="reference"):
    p, t, td, u, v, ps, ts, tds, us, vs = args
    vl = _option(_VERTICAL, vertical_lev, "vertical_lev")
    out = _option(_OUTPUT, output_var, "output_var")
    prec = _option(_SRH_PRECISION, precision, "precision")
    original_shape = tuple(t.shape)
    _check_same([t, td, u, v])
    _check_same([ps, ts, tds, us, vs])
    if len(p.shape) == 1 and vl == _lib.GRID_PRESSURE_1D:
        grid = _lib.GRID_PRESSURE_1D
        if p.shape[0] != t.shape[-1]:
            raise ValueError("1-D p must have one value per level of t")
    elif tuple(p.shape) == original_shape and vl == _lib.GRID_SIGMA:
        grid = _lib.GRID_SIGMA
    elif tuple(p.shape) == original_shape and vl == _lib.GRID_PRESSURE_1D:
        raise ValueError("P should be 1d")
    else:
        raise ValueError("Input arrays must have the same shape.")
    if method == "fortran":
        return _reference_fortran_srh(p, t, td, u, v, ps, ts, tds, us, vs, depth=depth,
                                      vertical_lev=vertical_lev, output_var=output_var)
    if method != "cuda":
        raise ValueError("invalid method")

    b = _Batch([t, td, u, v], [ps, ts, tds, us, vs], p, grid)
    srm, slm = b.empty(b.n2, "f8"), b.empty(b.n2, "f8")
    if out == 2:
        rm, lm, mean = (b.empty(2 * b.n2, "f4") for _ in range(3))
    else:
        rm = lm = mean = None
    lv = b.levels
    sf = b.surface
    args_ = (grid, b.ptr(b.p), b.ptr(lv[0]), b.ptr(lv[1]), b.ptr(lv[2]), b.ptr(lv[3]),
             b.ptr(sf[0]), b.ptr(sf[1]), b.ptr(sf[2]), b.ptr(sf[3]), b.ptr(sf[4]), b.dtype,
             None, float(depth), 2.0, b.nk, b.n2, prec, b.ptr(srm), b.ptr(slm), b.ptr(rm),
             b.ptr(lm), b.ptr(mean), b.stream)
    _lib.call("xc_calc_srh_ex" if b.torch else "xc_calc_srh_host", *args_)
    shp = _out_shape(original_shape)
    if out == 1:
        return srm.reshape(shp), slm.reshape(shp)
    res = [srm.reshape(shp), slm.reshape(shp)]
    for a in (rm, lm, mean):
        a2 = a.reshape(b.n2, 2)
        res += [a2[:, 0].reshape(shp), a2[:, 1].reshape(shp)]
    if not b.torch:
        res = [np.ascontiguousarray(r) for r in res]
    return tuple(res)


# ---------------------------------------------------------------------------
# CAPE and SRH of the same columns


def calc_cape_srh(p, t, td, u, v, ps, ts, tds, us, vs, source="surface", ml_depth=500.0,
                  adiabat="pseudo-liquid", pinc=500.0, depth=3000, vertical_lev="sigma",
                  output_var="srh", guess="plain", precision="reference"):
    """``calc_cape(p, t, td, ps, ts, tds, ...)`` and ``calc_srh(p, t, td, u, v,
    ps, ts, tds, us, vs, ...)`` on the same columns in one kernel on the GPU:
    the FP32 lift and the SRH chain's FP64 stages run on different pipes at
    once, so with ``precision='reference'`` the pair takes about as long as
    calc_srh alone.  The reference computes the two separately
    (src/xcape/core.py:261-332, :473-542); the results are those of the two
    calls.

    Arguments as the two functions (numpy arrays, or CUDA tensors used in
    place); ``guess`` is ``'plain'`` or ``'learned'``; ``vertical_lev`` is
    ``'sigma'``/``'model'`` or ``'pressure'``.  Returns ``(cape_result,
    srh_result)``: the tuples ``calc_cape`` and ``calc_srh`` return.
    """
    src = _option(_SOURCE, source, "source")
    adi = _option(_ADIABAT, adiabat, "adiabat")
    vl = _option(_VERTICAL, vertical_lev, "vertical_lev")
    out = _option(_OUTPUT, output_var, "output_var")
    prec = _option(_SRH_PRECISION, precision, "precision")
    gs = _option(_GUESS, guess, "guess")
    if gs not in (_lib.XC_GUESS_PLAIN, _lib.XC_GUESS_LEARNED):
        raise ValueError("calc_cape_srh: guess must be 'plain' or 'learned'")
    shape = tuple(t.shape)
    _check_same([t, td, u, v])
    _check_same([ps, ts, tds, us, vs])
    if len(p.shape) == 1 and vl == _lib.GRID_PRESSURE_1D:
        grid = _lib.GRID_PRESSURE_1D
        if p.shape[0] != shape[-1]:
            raise ValueError("1-D p must have one value per level of t")
    elif tuple(p.shape) == shape and vl == _lib.GRID_SIGMA:
        grid = _lib.GRID_SIGMA
    elif tuple(p.shape) == shape and vl == _lib.GRID_PRESSURE_1D:
        raise ValueError("P should be 1d")
    else:
        raise ValueError("Input arrays must have the same shape.")
    if _prod(tuple(ps.shape)) != _prod(shape[:-1]):
        raise ValueError("Surface arrays must have one value per column.")
    if gs == _lib.XC_GUESS_LEARNED:
        from . import guess as _guess
        _guess.ensure_loaded()
    import torch
    host = not any(_is_torch(a) for a in (p, t, td, u, v, ps, ts, tds, us, vs))
    if host:
        p, t, td, u, v, ps, ts, tds, us, vs = (
            torch.from_numpy(np.ascontiguousarray(a)).cuda()
            for a in (p, t, td, u, v, ps, ts, tds, us, vs))
    b = _Batch([t, td, u, v], [ps, ts, tds, us, vs], p, grid)
    cape, cin, zout = (b.empty(b.n2, "f4") for _ in range(3))
    mulvl = b.empty(b.n2, "i4")
    srm, slm = b.empty(b.n2, "f8"), b.empty(b.n2, "f8")
    if out == 2:
        rm, lm, mean = (b.empty(2 * b.n2, "f4") for _ in range(3))
    else:
        rm = lm = mean = None
    lv, sf = b.levels, b.surface
    ws, ws_bytes = b.workspace(_lib.workspace_bytes(b.n2))
    _lib.call("xc_cape_srh", grid, b.ptr(b.p), b.ptr(lv[0]), b.ptr(lv[1]), b.ptr(lv[2]),
              b.ptr(lv[3]), b.ptr(sf[0]), b.ptr(sf[1]), b.ptr(sf[2]), b.ptr(sf[3]),
              b.ptr(sf[4]), b.dtype, float(pinc), src, float(ml_depth), adi, None,
              float(depth), 2.0, b.nk, b.n2, gs, prec, b.ptr(cape), b.ptr(cin), b.ptr(mulvl),
              b.ptr(zout), None, b.ptr(srm), b.ptr(slm), b.ptr(rm), b.ptr(lm), b.ptr(mean),
              ws, ws_bytes, b.stream)
    shp = _out_shape(shape)
    cape_res = [cape.reshape(shp), cin.reshape(shp)]
    if src == 2:
        cape_res += [mulvl.reshape(shp), zout.reshape(shp)]
    srh_res = [srm.reshape(shp), slm.reshape(shp)]
    if out == 2:
        for a in (rm, lm, mean):
            a2 = a.reshape(b.n2, 2)
            srh_res += [a2[:, 0].reshape(shp), a2[:, 1].reshape(shp)]
    if host:
        cape_res = [r.cpu().numpy() for r in cape_res]
        srh_res = [np.ascontiguousarray(r.cpu().numpy()) for r in srh_res]
    return tuple(cape_res), tuple(srh_res)


# ---------------------------------------------------------------------------
# method='fortran': the installed reference, if any.


def _reference_core():
    try:
        from xcape import core as ref_core  # the reference package, if installed
    except Exception as exc:
        raise ImportError("method='fortran' needs the reference xcape package with its compiled "
                          "Fortran extensions; it is not installed") from exc
    return ref_core


def _reference_fortran_cape(*args, **kwargs):
    vl = kwargs.get("vertical_lev", "sigma")
    kwargs["vertical_lev"] = "sigma" if vl == "model" else vl
    return _reference_core().calc_cape(*args, method="fortran", **kwargs)


def _reference_fortran_srh(*args, **kwargs):
    vl = kwargs.get("vertical_lev", "sigma")
    kwargs["vertical_lev"] = "sigma" if vl == "model" else vl
    return _reference_core().calc_srh(*args, **kwargs)
