"""The allocation-free CAPE entry point, xc_loopcape_ex_noalloc.

Some callers cannot call cudaMalloc while they work: a host framework that
owns every byte of the device's memory, a serving process under a fixed
memory budget, a real-time loop that forbids allocation after start-up.
xc_loopcape_ex orders the columns in a workspace the caller allocates;
xc_loopcape_ex_noalloc uses a static device array inside the library
instead.  These tests call it through the C ABI, twice in a row, and check
each result against xc_loopcape_ex with a caller-provided workspace (within
the CAPE/CIN tolerance the other GPU tests use; the two run the same
kernels), also at exactly XC_NOALLOC_MAX_COLUMNS columns, and one result
directly against the oracle under the parity criteria of gpu_util.  They check that
the calls make no allocation -- neither the library's own (its allocation
counter, xc_alloc_count) nor torch's -- including in a fresh process under
lazy module loading, and that a batch above the limit is refused with a
message.  This file is collected last, so that a run stopping at the first
failure has run every other test before it.
"""
import ctypes
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from xcape_gb300 import _lib
from xcape_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MAX_COLUMNS = _lib.XC_NOALLOC_MAX_COLUMNS  # the header's value (checked by test_host_api)


def _device_inputs(shape, seed=1):
    import torch
    assert torch.cuda.is_available()
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=shape, seed=seed)
    d = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (plev, t, td, ps, ts, tds)]
    return d, ps.size


@pytest.fixture(scope="module")
def dev_inputs():
    return _device_inputs((256, 512))


def _outputs(n2):
    import torch
    f = [torch.empty(n2, dtype=torch.float32, device="cuda") for _ in range(3)]
    i = [torch.empty(n2, dtype=torch.int32, device="cuda") for _ in range(2)]
    return f + i  # cape, cin, z_out, mulvl, status


def _args(d, n2, guess, outs):
    cape, cin, zout, mulvl, status = outs
    return (2, *[x.data_ptr() for x in d], _lib.XC_F32, 500.0, 2, 500.0, 1, None, 37, n2, guess,
            cape.data_ptr(), cin.data_ptr(), mulvl.data_ptr(), zout.data_ptr(), status.data_ptr(),
            None)


def _numpy(outs):
    return [o.cpu().numpy() for o in outs]


def _close(a, b):
    cape_a, cin_a, z_a, mu_a, st_a = a
    cape_b, cin_b, z_b, mu_b, st_b = b
    for x, y in ((cape_a, cape_b), (cin_a, cin_b), (z_a, z_b)):
        y = y.astype(np.float64)
        np.testing.assert_array_equal(np.isnan(x), np.isnan(y))
        ok = ~np.isnan(y)
        assert np.all(np.abs(x[ok] - y[ok]) <= np.maximum(1.0, 1e-3 * np.abs(y[ok])))
    np.testing.assert_array_equal(mu_a, mu_b)
    np.testing.assert_array_equal(st_a, st_b)


def _with_workspace(d, n2, guess):
    """The existing entry point, xc_loopcape_ex, with a caller workspace."""
    import torch
    L = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    ws_bytes = _lib.workspace_bytes(n2)
    wsbuf = torch.empty(ws_bytes + 256, dtype=torch.uint8, device="cuda")
    ws = wsbuf.data_ptr() + (-wsbuf.data_ptr()) % 256
    ref = _outputs(n2)
    _lib.check(L.xc_loopcape_ex(*_args(d, n2, guess, ref), ws, ws_bytes, stream))
    torch.cuda.synchronize()
    return _numpy(ref)


def _check_two_calls(d, n2, guess):
    import torch
    L = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    want = _with_workspace(d, n2, guess)
    for _ in range(2):  # two calls in a row share the static scratch
        outs = _outputs(n2)
        _lib.check(L.xc_loopcape_ex_noalloc(*_args(d, n2, guess, outs), stream))
        torch.cuda.synchronize()
        _close(_numpy(outs), want)


@pytest.mark.parametrize("guess", [_lib.XC_GUESS_PLAIN, _lib.XC_GUESS_EXTRAPOLATED])
def test_noalloc_matches_workspace_entry_point(dev_inputs, guess):
    d, n2 = dev_inputs
    _check_two_calls(d, n2, guess)


def test_noalloc_against_the_oracle():
    """The allocation-free entry point pinned to the oracle directly, not only
    through xc_loopcape_ex: the plain solver against the FP32 oracle with the
    parity criteria of the single-call tests, on 4,096 columns of pressure
    levels, most-unstable parcels."""
    import torch
    from gpu_util import compare_cape, oracle_cols
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(64, 64), seed=12)
    d = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (plev, t, td, ps, ts, tds)]
    n2 = ps.size
    L = _lib.lib()
    outs = _outputs(n2)
    _lib.check(L.xc_loopcape_ex_noalloc(*_args(d, n2, _lib.XC_GUESS_PLAIN, outs),
                                        torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    cape, cin, zout, mulvl, status = _numpy(outs)
    args = (2, plev, t, td, ps, ts, tds, "most-unstable", "pseudo-liquid", 500.0, 500.0)
    compare_cape({"cape": cape, "cin": cin, "mulvl": mulvl, "z_out": zout, "status": status},
                 oracle_cols(*args), oracle_cols(*args, precision="f64"),
                 what="noalloc vs oracle")


def test_noalloc_at_the_column_limit():
    """Exactly XC_NOALLOC_MAX_COLUMNS columns: the ordering scratch fills the
    static array."""
    assert MAX_COLUMNS == 1024 * 1024
    d, n2 = _device_inputs((1024, 1024), seed=5)
    assert n2 == MAX_COLUMNS
    _check_two_calls(d, n2, _lib.XC_GUESS_EXTRAPOLATED)


def test_noalloc_allocates_nothing(dev_inputs):
    """Neither the library (its allocation counter) nor torch's allocator
    allocates during the calls -- a measure that, unlike the device's free
    memory, other processes on the GPU cannot move."""
    import torch
    d, n2 = dev_inputs
    L = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    outs = _outputs(n2)
    torch.cuda.synchronize()
    lib_before = L.xc_alloc_count()
    torch_before = torch.cuda.memory_allocated()
    for guess in (_lib.XC_GUESS_PLAIN, _lib.XC_GUESS_EXTRAPOLATED, _lib.XC_GUESS_PLAIN):
        _lib.check(L.xc_loopcape_ex_noalloc(*_args(d, n2, guess, outs), stream))
    torch.cuda.synchronize()
    assert L.xc_alloc_count() == lib_before
    assert torch.cuda.memory_allocated() == torch_before
    # the counter does count: the host entry point allocates its workspace
    # (or reuses it), and the batch executor allocates its tables
    from xcape_gb300.batch import CapeBatch
    with CapeBatch(max_requests=2, max_columns=64, guess="plain"):
        pass
    assert L.xc_alloc_count() > lib_before


FRESH = textwrap.dedent("""
    import os, sys
    sys.path.insert(0, {root!r})
    sys.path.insert(0, os.path.join({root!r}, "tests"))
    import torch
    import test_zz_no_alloc as T
    from xcape_gb300 import _lib
    L = _lib.lib()
    torch.cuda.init()
    stream = torch.cuda.current_stream().cuda_stream
    d, n2 = T._device_inputs((64, 128), seed=3)
    want = T._with_workspace(d, n2, _lib.XC_GUESS_PLAIN)
    # the start-up call: n2 == 0 loads the array on this device
    _lib.check(L.xc_loopcape_ex_noalloc(2, *([None] * 6), _lib.XC_F32, 500.0, 2, 500.0, 1, None,
                                        37, 0, 0, *([None] * 6), stream))
    outs = [T._outputs(n2) for _ in range(2)]
    torch.cuda.synchronize()
    lib0, torch0 = L.xc_alloc_count(), torch.cuda.memory_allocated()
    for o in outs:
        _lib.check(L.xc_loopcape_ex_noalloc(*T._args(d, n2, _lib.XC_GUESS_PLAIN, o), stream))
    torch.cuda.synchronize()
    assert L.xc_alloc_count() == lib0 and torch.cuda.memory_allocated() == torch0
    for o in outs:
        T._close(T._numpy(o), want)
    print("fresh-process noalloc ok")
""")


def test_noalloc_in_a_fresh_process_with_lazy_loading():
    env = dict(os.environ, CUDA_MODULE_LOADING="LAZY")
    r = subprocess.run([sys.executable, "-c", FRESH.format(root=ROOT)], env=env, cwd=ROOT,
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, timeout=600)
    out = r.stdout.decode(errors="replace")
    assert r.returncode == 0, out[-3000:]
    assert "fresh-process noalloc ok" in out


def test_noalloc_rejects_oversized_batch():
    L = _lib.lib()
    n2 = MAX_COLUMNS + 1
    null = ctypes.c_void_p(None)
    rc = L.xc_loopcape_ex_noalloc(2, *([None] * 6), _lib.XC_F32, 500.0, 2, 500.0, 1, None, 37, n2,
                                  0, *([None] * 6), null)
    assert rc == _lib.XC_ERR_INVALID
    assert b"at most" in L.xc_last_error()
