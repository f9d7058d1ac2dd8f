"""Ragged batches of calc_cape requests in one graph-launched persistent kernel.

``CapeBatch`` wraps the library's batch executor (``xc_batch_*`` in
``include/xcape_gb300.h``): many requests, each with its own column count,
level count, vertical coordinate, source, adiabat, pinc and ml_depth, run in
one launch of a CUDA graph (table upload, counter reset, the persistent
kernel).  Inputs are float32 CUDA tensors in the units of ``calc_cape`` (hPa,
degC); a request may be a view of the first ``nk`` levels of a wider array
(row stride >= nk, unit stride along the levels).

    b = CapeBatch(max_requests=256, max_columns=1 << 22, guess="learned")
    r1 = b.request(p, t, td, ps, ts, tds, source="surface", vertical_lev="sigma")
    r2 = b.request(plev, t2, td2, ps2, ts2, tds2, source="most-unstable",
                   vertical_lev="pressure")
    b.run([r1, r2])            # asynchronous on the current stream
    cape, cin = r1.cape, r1.cin
"""
import ctypes

from . import _lib

_SOURCES = {"surface": 1, "most-unstable": 2, "mixed-layer": 3}
_ADIABATS = {"pseudo-liquid": 1, "reversible-liquid": 2, "pseudo-ice": 3, "reversible-ice": 4}
_GRIDS = {"sigma": 1, "model": 1, "pressure": 2}
_GUESS = {"plain": _lib.XC_GUESS_PLAIN, "learned": _lib.XC_GUESS_LEARNED,
          "extrapolated": _lib.XC_GUESS_EXTRAPOLATED}


class Request:
    """One request of a batch: its descriptor, its inputs (kept alive until
    the batch has run) and its output tensors."""

    def __init__(self, desc, keep, cape, cin, mulvl, z_out, status):
        self.desc = desc
        self._keep = keep
        self.cape, self.cin, self.mulvl, self.z_out, self.status = cape, cin, mulvl, z_out, status


def _torch():
    import torch
    return torch


def _check_2d(x, name):
    torch = _torch()
    if not (isinstance(x, torch.Tensor) and x.is_cuda and x.dtype == torch.float32):
        raise TypeError(f"{name} must be a float32 CUDA tensor")
    if x.dim() != 2 or x.stride(1) != 1:
        raise ValueError(f"{name} must be 2-D (columns, levels) with unit stride along levels")


def _check_1d(x, name, n):
    torch = _torch()
    if not (isinstance(x, torch.Tensor) and x.is_cuda and x.dtype == torch.float32):
        raise TypeError(f"{name} must be a float32 CUDA tensor")
    if x.dim() != 1 or x.shape[0] != n or (n > 1 and x.stride(0) != 1):
        raise ValueError(f"{name} must be contiguous with {n} elements")


class CapeBatch:
    """Executor of ragged calc_cape batches on the current CUDA device."""

    def __init__(self, max_requests=1024, max_columns=1 << 22, guess="learned"):
        if guess not in _GUESS:
            raise ValueError(f"guess must be one of {sorted(_GUESS)}")
        if guess == "learned":
            from . import guess as _guess
            _guess.ensure_loaded()
        self.max_requests = int(max_requests)
        self.max_columns = int(max_columns)
        self.guess = guess
        h = ctypes.c_void_p()
        _lib.call("xc_batch_create", self.max_requests, self.max_columns, _GUESS[guess],
                  ctypes.byref(h))
        self._h = h

    def request(self, p, t, td, ps, ts, tds, source="surface", adiabat="pseudo-liquid",
                vertical_lev="sigma", pinc=500.0, ml_depth=500.0, outputs=None):
        """Describes one calc_cape call and allocates its outputs, or uses
        `outputs` = [cape, cin, mulvl, z_out] (contiguous CUDA tensors of n2
        float32, float32, int32, float32; no status output then)."""
        torch = _torch()
        if source not in _SOURCES:
            raise ValueError(f"source must be one of {sorted(_SOURCES)}")
        if adiabat not in _ADIABATS:
            raise ValueError(f"adiabat must be one of {sorted(_ADIABATS)}")
        if vertical_lev not in _GRIDS:
            raise ValueError(f"vertical_lev must be one of {sorted(_GRIDS)}")
        grid = _GRIDS[vertical_lev]
        _check_2d(t, "t")
        _check_2d(td, "td")
        n2, nk = t.shape
        if td.shape != t.shape or td.stride() != t.stride():
            raise ValueError("t and td must have the same shape and strides")
        ld = t.stride(0) if n2 > 1 else nk
        if grid == 1:
            _check_2d(p, "p")
            if p.shape != t.shape or p.stride() != t.stride():
                raise ValueError("sigma/model p must have the shape and strides of t")
        else:
            _check_1d(p, "p", nk)
        for x, name in ((ps, "ps"), (ts, "ts"), (tds, "tds")):
            _check_1d(x, name, n2)
        dev = t.device
        if outputs is None:
            cape = torch.empty(n2, dtype=torch.float32, device=dev)
            cin = torch.empty_like(cape)
            z_out = torch.empty_like(cape)
            mulvl = torch.empty(n2, dtype=torch.int32, device=dev)
            status = torch.empty_like(mulvl)
        else:
            cape, cin, mulvl, z_out = outputs
            for x, name in ((cape, "cape"), (cin, "cin"), (z_out, "z_out")):
                _check_1d(x, name, n2)
            if not (isinstance(mulvl, torch.Tensor) and mulvl.is_cuda and
                    mulvl.dtype == torch.int32 and mulvl.shape == (n2,) and mulvl.is_contiguous()):
                raise TypeError("mulvl must be a contiguous int32 CUDA tensor of n2 elements")
            status = None
        d = _lib.CapeRequest(grid=grid, nk=nk, n2=n2, ld=ld, p=p.data_ptr(), t3d=t.data_ptr(),
                             td3d=td.data_ptr(), ps=ps.data_ptr(), ts=ts.data_ptr(),
                             tds=tds.data_ptr(), pinc=float(pinc), source=_SOURCES[source],
                             ml_depth=float(ml_depth), adiabat=_ADIABATS[adiabat],
                             cape=cape.data_ptr(), cin=cin.data_ptr(), mulvl=mulvl.data_ptr(),
                             z_out=z_out.data_ptr(),
                             status=status.data_ptr() if status is not None else None)
        return Request(d, (p, t, td, ps, ts, tds), cape, cin, mulvl, z_out, status)

    def run(self, requests, stream=None):
        """Launches one batch on `stream` (default: the current stream)."""
        torch = _torch()
        reqs = list(requests)
        arr = (_lib.CapeRequest * max(1, len(reqs)))(*[r.desc for r in reqs])
        s = stream if stream is not None else torch.cuda.current_stream()
        _lib.call("xc_batch_run", self._h, ctypes.cast(arr, ctypes.c_void_p), len(reqs),
                  s.cuda_stream)

    def work(self):
        """(sub-steps, iterations) of the last run; waits for it."""
        a, b = ctypes.c_longlong(), ctypes.c_longlong()
        _lib.call("xc_batch_work", self._h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def close(self):
        if self._h is not None and self._h.value:
            _lib.call("xc_batch_destroy", self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
