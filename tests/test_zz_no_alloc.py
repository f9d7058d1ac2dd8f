"""The allocation-free CAPE entry point, xc_loopcape_ex_noalloc.

Some callers cannot call cudaMalloc while they work: a host framework that
owns every byte of the device's memory, a serving process under a fixed
memory budget, a real-time loop that forbids allocation after start-up.
xc_loopcape_ex orders the columns in a workspace the caller allocates;
xc_loopcape_ex_noalloc uses a static device array inside the library
instead.  These tests call it through the C ABI, twice in a row, and check
each result against xc_loopcape_ex with a caller-provided workspace (within
the CAPE/CIN tolerance the other GPU tests use; the two run the same
kernels), check that repeated calls leave the free device memory unchanged,
and that a batch above XC_NOALLOC_MAX_COLUMNS is refused with a message.
"""
import ctypes

import numpy as np
import pytest

from xcape_gb300 import _lib
from xcape_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

NOALLOC_MAX_COLUMNS = 1048576


@pytest.fixture(scope="module")
def dev_inputs():
    import torch
    assert torch.cuda.is_available()
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(256, 512))
    d = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (plev, t, td, ps, ts, tds)]
    return d, ps.size


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
        assert np.all(np.abs(x - y) <= np.maximum(1.0, 1e-3 * np.abs(y)))
    np.testing.assert_array_equal(mu_a, mu_b)
    np.testing.assert_array_equal(st_a, st_b)


@pytest.mark.parametrize("guess", [_lib.XC_GUESS_PLAIN, _lib.XC_GUESS_EXTRAPOLATED])
def test_noalloc_matches_workspace_entry_point(dev_inputs, guess):
    import torch
    d, n2 = dev_inputs
    L = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    ws_bytes = _lib.workspace_bytes(n2)
    wsbuf = torch.empty(ws_bytes + 256, dtype=torch.uint8, device="cuda")
    ws = wsbuf.data_ptr() + (-wsbuf.data_ptr()) % 256
    ref = _outputs(n2)
    _lib.check(L.xc_loopcape_ex(*_args(d, n2, guess, ref), ws, ws_bytes, stream))
    torch.cuda.synchronize()
    want = _numpy(ref)
    for _ in range(2):  # two calls in a row share the static scratch
        outs = _outputs(n2)
        _lib.check(L.xc_loopcape_ex_noalloc(*_args(d, n2, guess, outs), stream))
        torch.cuda.synchronize()
        _close(_numpy(outs), want)


def test_noalloc_allocates_nothing(dev_inputs):
    import torch
    d, n2 = dev_inputs
    L = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    outs = _outputs(n2)
    for guess in (_lib.XC_GUESS_PLAIN, _lib.XC_GUESS_EXTRAPOLATED):
        _lib.check(L.xc_loopcape_ex_noalloc(*_args(d, n2, guess, outs), stream))
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for guess in (_lib.XC_GUESS_PLAIN, _lib.XC_GUESS_EXTRAPOLATED):
        _lib.check(L.xc_loopcape_ex_noalloc(*_args(d, n2, guess, outs), stream))
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before


def test_noalloc_rejects_oversized_batch():
    L = _lib.lib()
    n2 = NOALLOC_MAX_COLUMNS + 1
    null = ctypes.c_void_p(None)
    rc = L.xc_loopcape_ex_noalloc(2, *([None] * 6), _lib.XC_F32, 500.0, 2, 500.0, 1, None, 37, n2,
                                  0, *([None] * 6), null)
    assert rc == _lib.XC_ERR_INVALID
    assert b"at most" in L.xc_last_error()
