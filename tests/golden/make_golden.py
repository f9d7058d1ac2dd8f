"""Extract the reference's own golden vectors into small .npz fixtures.

The reference keeps its parity data as two pytest fixtures in
``test/fixtures.py`` (``dataset_soundings``, fixtures.py:1166-3441, and
``dataset_ERA5pressurelevel``, fixtures.py:29-1162).  They are built with
``xarray.Dataset.from_dict`` and depend on xarray/dask, neither of which is
installed.  This script executes that file with small stand-in modules for
``xarray``/``dask``/``pytest`` so that ``Dataset.from_dict`` only keeps the
raw arrays, then writes every variable of both fixtures to

* ``tests/golden/soundings.npz``        (13 soundings x 108 levels, level 0 = surface)
* ``tests/golden/era5_pressure.npz``    (17 ERA5 columns x 37 pressure levels)

The values are read from the reference file; nothing is typed in by hand.
The tests in this repository only read the .npz files, so they run where the
reference tree is absent.

Usage::

    python tests/golden/make_golden.py [path/to/reference/test/fixtures.py]
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_FIXTURES = "/root/reference/test/fixtures.py"


class _Var:
    def __init__(self, data, dims):
        self.data = np.asarray(data, dtype=np.float64) if not _is_int(data) else np.asarray(data)
        self.dims = tuple(dims)

    @property
    def values(self):
        return self.data


def _is_int(data):
    arr = np.asarray(data)
    return arr.dtype.kind in "iu"


class _Dataset:
    """Keeps ``data_vars`` and ``coords`` of an xarray dict as numpy arrays."""

    def __init__(self, d):
        self.vars = {}
        for name, v in d.get("coords", {}).items():
            self.vars[name] = _Var(v["data"], v["dims"])
        for name, v in d.get("data_vars", {}).items():
            self.vars[name] = _Var(v["data"], v["dims"])

    @classmethod
    def from_dict(cls, d):
        return cls(d)

    def transpose(self):
        # xarray's Dataset.transpose() with no arguments reverses every
        # variable's dimension order.
        out = _Dataset({})
        for name, v in self.vars.items():
            nv = _Var(v.data.T if v.data.ndim > 1 else v.data, v.dims[::-1])
            out.vars[name] = nv
        return out

    def __getattr__(self, name):
        try:
            return self.__dict__["vars"][name]
        except KeyError as exc:
            raise AttributeError(name) from exc


def _load_fixtures(path):
    xr = types.ModuleType("xarray")
    xr.Dataset = _Dataset
    dask = types.ModuleType("dask")
    dask.delayed = lambda f: f
    dsa = types.ModuleType("dask.array")
    dask.array = dsa
    pytest = types.ModuleType("pytest")
    pytest.fixture = lambda *a, **k: (lambda f: f)
    saved = {k: sys.modules.get(k) for k in ("xarray", "dask", "dask.array", "pytest")}
    sys.modules.update({"xarray": xr, "dask": dask, "dask.array": dsa, "pytest": pytest})
    try:
        src = open(path).read()
        ns = {"__name__": "reference_fixtures", "np": np}
        exec(compile(src, path, "exec"), ns)
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    return ns


def main(argv):
    path = argv[1] if len(argv) > 1 else DEFAULT_FIXTURES
    ns = _load_fixtures(path)

    snd = ns["dataset_soundings"]()  # already transposed: (n2, level)
    out = {name: v.data for name, v in snd.vars.items()}
    np.savez_compressed(os.path.join(HERE, "soundings.npz"), **out)
    print("soundings:", {k: v.shape for k, v in out.items()})

    ds3d, dssurf = ns["dataset_ERA5pressurelevel"]()
    out = {}
    for name, v in ds3d.vars.items():
        out["lev_" + name] = v.data
    for name, v in dssurf.vars.items():
        out["sfc_" + name] = v.data
    np.savez_compressed(os.path.join(HERE, "era5_pressure.npz"), **out)
    print("era5:", {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main(sys.argv)
