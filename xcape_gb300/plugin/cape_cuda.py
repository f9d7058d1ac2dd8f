"""method='cuda' for xcape itself: a drop-in module for xcape's source tree.

A maintainer of xcape copies this file to ``src/xcape/cape_cuda.py`` and adds
a ``method == 'cuda'`` branch at the two seams where xcape enters its
compiled Fortran.  It depends on numpy and ctypes only (no torch): it binds
``libxcape_gb300.so`` by its C ABI (``include/xcape_gb300.h``), found through
the environment variable ``XCAPE_GB300_LIB`` or the dynamic loader's search
path.

* CAPE, ``src/xcape/core.py:313-324`` (``_calc_cape_numpy``), beside the
  ``method == 'fortran'`` branch::

      elif method == 'cuda':
          from .cape_cuda import cape as _cape_cuda
          cape_2d, cin_2d, mulev, zmulev = _cape_cuda(p_2d, t_2d, td_2d,
                                                      p_s1d, t_s1d, td_s1d,
                                                      flag_1d, pres_lev_pos,
                                                      **kwargs)

  ``cape`` takes exactly the arguments of ``cape_fortran.cape``
  (``src/xcape/cape_fortran.py:3``) and returns what it returns.

* SRH, ``src/xcape/core.py:516-542`` (``_calc_srh_numpy``): the two calls
  ``_stdheight`` then ``_srh`` become one::

      if method == 'cuda':
          from .cape_cuda import srh_chain
          out = srh_chain(p_2d, t_2d, td_2d, u_2d, v_2d, p_s1d, t_s1d, td_s1d,
                          u_s1d, v_s1d, flag_1d, pres_lev_pos, depth, **kwargs)

  ``srh_chain`` returns what ``srh.srh`` (``src/xcape/srh.py:4-66``) returns
  for the heights ``stdheight.stdheight`` would have produced with
  ``aglh0 = 2`` (``core.py:519``): ``(srh_rm, srh_lm)`` for ``output == 1``,
  else ``(srh_rm, srh_lm, rm, lm, mean_6km)`` with the vectors shaped
  ``(2, ngrid)`` like the f2py outputs.

What the seams hand over (``core.py:31-50, 81-100, 278-300``): the 3-D
fields as ``(nlev, ngrid)`` views -- the transposes of the caller's
C-contiguous ``(ngrid, nlev)`` data -- and the surface fields as
``(ngrid,)``.  For pressure levels ``p_2d`` is ``(nlev, 1)`` and
``pres_lev_pos`` the 1-based first level at or above the ground per column;
for sigma levels ``pres_lev_pos`` is the integer 1.  ``.T`` of each view is
the C-contiguous ``(ngrid, nlev)`` array the library binds, so nothing is
transposed or copied when the data are already contiguous float32.

Errors: the library returns a status instead of executing Fortran ``stop``;
a non-zero status raises ``RuntimeError`` with the library's message.
"""
import ctypes
import os

import numpy as np

_vp, _i, _f, _d = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double

_XC_F32, _XC_F64 = 0, 1
_XC_GUESS_PLAIN = 0
_XC_SRH_REFERENCE = 0

_L = None


def _lib():
    global _L
    if _L is None:
        L = ctypes.CDLL(os.environ.get("XCAPE_GB300_LIB", "libxcape_gb300.so"))
        L.xc_loopcape_ex_host.argtypes = ([_i] + [_vp] * 6 + [_i, _f, _i, _f, _i, _vp, _i, _i, _i]
                                          + [_vp] * 5 + [_vp])
        L.xc_loopcape_ex_host.restype = _i
        L.xc_calc_srh_host.argtypes = ([_i] + [_vp] * 10 + [_i, _vp, _d, _d, _i, _i, _i]
                                       + [_vp] * 5 + [_vp])
        L.xc_calc_srh_host.restype = _i
        L.xc_last_error.restype = ctypes.c_char_p
        _L = L
    return _L


def _check(rc):
    if rc != 0:
        raise RuntimeError(_lib().xc_last_error().decode(errors="replace"))


def _columns(a, dtype):
    """(nlev, ngrid) view from the seam -> C-contiguous (ngrid, nlev)."""
    return np.ascontiguousarray(np.asarray(a).T, dtype)


def _flat(a, dtype):
    return np.ascontiguousarray(np.ravel(a), dtype)


def _ptr(a):
    return None if a is None else a.ctypes.data


def cape(p_2d, t_2d, td_2d, p_s, t_s, td_s, flag_1d, pres_lev_pos, source, ml_depth, adiabat,
         pinc, type_grid):
    """CAPE, CIN, MU level and zMU of every column, as ``cape_fortran.cape``.

    Like f2py for the Fortran's ``real`` arguments, the inputs are taken as
    float32; the outputs are ``(ngrid,)`` float32 (mulev int32)."""
    nlev, ngrid = np.shape(t_2d)
    t, td = _columns(t_2d, np.float32), _columns(td_2d, np.float32)
    ps, ts, tds = (_flat(a, np.float32) for a in (p_s, t_s, td_s))
    if type_grid == 2 and flag_1d == 1:      # loopcape_pl1d: shared levels, ragged start
        grid, p = 2, _flat(p_2d, np.float32)
        start = _flat(pres_lev_pos, np.int32)
    elif type_grid == 1:                     # loopcape_ml
        grid, p, start = 1, _columns(p_2d, np.float32), None
    else:
        raise ValueError("type_grid 2 needs a 1-D pressure axis (flag_1d == 1)")
    out = [np.empty(ngrid, np.float32), np.empty(ngrid, np.float32),
           np.empty(ngrid, np.int32), np.empty(ngrid, np.float32)]
    cape_, cin_, mulev, zmulev = out
    _check(_lib().xc_loopcape_ex_host(
        grid, _ptr(p), _ptr(t), _ptr(td), _ptr(ps), _ptr(ts), _ptr(tds), _XC_F32, float(pinc),
        int(source), float(ml_depth), int(adiabat), _ptr(start), int(nlev), int(ngrid),
        _XC_GUESS_PLAIN, _ptr(cape_), _ptr(cin_), _ptr(mulev), _ptr(zmulev), None, None))
    return cape_, cin_, mulev, zmulev


def srh_chain(p_2d, t_2d, td_2d, u_2d, v_2d, p_s, t_s, td_s, u_s, v_s, flag_1d, pres_lev_pos,
              depth, type_grid, output):
    """``stdheight.stdheight`` (aglh0 = 2 m) followed by ``srh.srh``, in one
    call.  The heights and helicity are double precision as in the
    reference; float64 inputs are used as given, float32 ones widened on
    the device (as f2py widens them for the double-precision routines)."""
    nlev, ngrid = np.shape(t_2d)
    arrays = (p_2d, t_2d, td_2d, u_2d, v_2d, p_s, t_s, td_s, u_s, v_s)
    f64 = any(np.asarray(a).dtype != np.float32 for a in arrays)
    dt = np.float64 if f64 else np.float32
    t, td, u, v = (_columns(a, dt) for a in (t_2d, td_2d, u_2d, v_2d))
    ps, ts, tds, us, vs = (_flat(a, dt) for a in (p_s, t_s, td_s, u_s, v_s))
    if type_grid == 2 and flag_1d == 1:
        grid, p = 2, _flat(p_2d, dt)
        start = _flat(pres_lev_pos, np.int32)
    elif type_grid == 1:
        grid, p, start = 1, _columns(p_2d, dt), None
    else:
        raise ValueError("type_grid 2 needs a 1-D pressure axis (flag_1d == 1)")
    srh_rm, srh_lm = np.empty(ngrid, np.float64), np.empty(ngrid, np.float64)
    vec = [np.empty((ngrid, 2), np.float32) for _ in range(3)] if output != 1 else [None] * 3
    _check(_lib().xc_calc_srh_host(
        grid, _ptr(p), _ptr(t), _ptr(td), _ptr(u), _ptr(v), _ptr(ps), _ptr(ts), _ptr(tds),
        _ptr(us), _ptr(vs), _XC_F64 if f64 else _XC_F32, _ptr(start), float(depth), 2.0,
        int(nlev), int(ngrid), _XC_SRH_REFERENCE, _ptr(srh_rm), _ptr(srh_lm),
        *[_ptr(x) for x in vec], None))
    if output == 1:
        return srh_rm, srh_lm
    rm, lm, mean_6km = (np.ascontiguousarray(x.T) for x in vec)   # (2, ngrid) like f2py
    return srh_rm, srh_lm, rm, lm, mean_6km
