"""GPU tests of the service loop (xcape_gb300.serve.CapeServer): requests
with host inputs, admitted by device-memory budget into one of two arenas,
copied, batched and returned, with batch k + 1 launched before batch k is
finished.  Every request's results are checked against the oracle on its
own columns: the plain solver against the FP32 oracle with the parity
criteria of the single-call tests, the learned solver against the FP64
oracle within its contract."""
import numpy as np
import pytest

from xcape_gb300 import synthetic as S

from gpu_util import check_vs_fp64, compare_cape, oracle_cols, torch_cuda

pytestmark = pytest.mark.gpu


def _requests(seed=3):
    from xcape_gb300.serve import Request
    rng = np.random.default_rng(seed)
    out = []
    for k in range(14):
        n2 = int(rng.integers(1, 3000))
        nk = int(rng.integers(20, 138))
        grid = ("sigma", "pressure")[k % 2]
        source = ("surface", "most-unstable", "mixed-layer")[k % 3]
        adiabat = ("pseudo-liquid", "reversible-liquid", "pseudo-ice", "reversible-ice")[k % 4]
        if grid == "sigma":
            p, t, td, ps, ts, tds = S.sigma_c0(shape=(n2,), nlev=nk, seed=100 + k,
                                               dtype=np.float32)
            p = np.reshape(p, (n2, nk))
        else:
            p, t, td, ps, ts, tds = S.pressure_c1(shape=(n2,), nlev=nk, seed=100 + k)
        out.append(Request(p, np.reshape(t, (n2, nk)), np.reshape(td, (n2, nk)), ps, ts, tds,
                           source=source, adiabat=adiabat, vertical_lev=grid, tag=k))
    return out


def _check(req, res, guess):
    cape, cin, mulvl, z_out = res
    g = 1 if req.vertical_lev == "sigma" else 2
    args = (req.p, req.t, req.td, req.ps, req.ts, req.tds)
    what = f"request {req.tag} {req.vertical_lev} {req.source} {req.adiabat} n2={req.n2}"
    ref64 = oracle_cols(g, *args, req.source, req.adiabat, 500.0, 500.0, precision="f64")
    # the service returns no status: a zero pair where the oracle's result is
    # not the reference's give-up is a give-up (a convergence flip)
    got = {"cape": cape, "cin": cin, "mulvl": mulvl}
    if guess == "plain":
        ref = oracle_cols(g, *args, req.source, req.adiabat, 500.0, 500.0)
        zero = (cape == 0) & (cin == 0)
        real_zero = ((ref["status"] & 1) == 0) & (ref["cape"] == 0) & (ref["cin"] == 0)
        got["status"] = np.where(zero & ~real_zero, 1, 0)
        compare_cape(got, ref, ref64, what=what)
    else:
        got["status"] = np.zeros(req.n2, np.int32)
        check_vs_fp64(got, ref64, what=what, min_same_parcel=0.98)


@pytest.mark.parametrize("guess", ["plain", "learned"])
def test_server_batches_match_oracle(guess):
    """A small memory budget splits the requests over several batches; each
    batch is launched before the previous one is finished."""
    torch_cuda()
    from xcape_gb300.serve import CapeServer
    reqs = _requests()
    pending = list(reqs)
    total = sum(r.device_bytes() for r in reqs)
    done = {}
    with CapeServer(memory_budget=total // 2, guess=guess) as srv:
        inflight, batches = None, 0
        while pending or inflight is not None:
            batch = None
            if pending:
                take = srv.admit(pending)
                assert take and sum(r.device_bytes() for r in take) <= srv.arena_bytes
                batch = srv.launch(take)
                batches += 1
            if inflight is not None:
                for r, res in srv.finish(inflight):
                    done[r.tag] = (r, res)
            inflight = batch
    assert batches >= 3
    assert sorted(done) == list(range(len(reqs)))
    for r, res in done.values():
        assert all(a.shape == (r.n2,) for a in res)
        _check(r, res, guess)


def test_server_refuses_a_request_larger_than_its_arena():
    torch_cuda()
    from xcape_gb300.serve import CapeServer
    reqs = _requests()
    with CapeServer(memory_budget=1 << 20, guess="plain") as srv:
        big = max(reqs, key=lambda r: r.device_bytes())
        assert big.device_bytes() > srv.arena_bytes
        with pytest.raises(ValueError, match="arena"):
            srv.admit([big])


def test_server_pinned_row_views_with_a_leading_dimension():
    """Requests whose arrays are blocks of rows of wider pinned pools (137
    values per row, the first nk of them the column's levels), as a service
    whose clients write into registered buffers hands them over: copied to
    the device without staging, and the results match the same requests
    given as dense pageable arrays."""
    torch = torch_cuda()
    from xcape_gb300.serve import CapeServer, Request
    ld, n = 137, 4096
    p, t, td, ps, ts, tds = S.pressure_c1(shape=(n,), nlev=ld, seed=77)

    def pinned(a):
        out = torch.empty(a.shape, dtype=torch.float32).pin_memory().numpy()
        out[...] = a
        return out
    P, T, TD, PS, TS, TDS = (pinned(np.asarray(a, np.float32)) for a in (p, t, td, ps, ts, tds))
    specs = [(0, 1000, 37), (1000, 77, 90), (2048, 2048, 137)]
    views = [Request(P, T[c0:c0 + m], TD[c0:c0 + m], PS[c0:c0 + m], TS[c0:c0 + m],
                     TDS[c0:c0 + m], source="most-unstable", vertical_lev="pressure", nk=nk)
             for c0, m, nk in specs]
    dense = [Request(np.ascontiguousarray(P[:nk]), np.ascontiguousarray(T[c0:c0 + m, :nk]),
                     np.ascontiguousarray(TD[c0:c0 + m, :nk]), PS[c0:c0 + m].copy(),
                     TS[c0:c0 + m].copy(), TDS[c0:c0 + m].copy(), source="most-unstable",
                     vertical_lev="pressure") for c0, m, nk in specs]
    with CapeServer(memory_budget=1 << 30, guess="plain") as srv:
        a = srv.finish(srv.launch(srv.admit(list(views))))
        b = srv.finish(srv.launch(srv.admit(list(dense))))
    for (ra, xa), (rb, xb) in zip(a, b):
        for u, v in zip(xa, xb):
            np.testing.assert_array_equal(u, v)


def test_copy_list_round_trip():
    """xc_copy_list: pinned and pageable host arrays to the device and back
    in one call each, zero-byte entries skipped, a NULL pointer refused."""
    torch = torch_cuda()
    from xcape_gb300 import _lib
    L = _lib.lib()
    rng = np.random.default_rng(1)
    sizes = [0, 4, 1000, 1 << 20, 3 << 20]
    pinned = [torch.from_numpy(rng.integers(0, 255, n, dtype=np.uint8)).pin_memory()
              for n in sizes]
    host = [rng.integers(0, 255, n, dtype=np.uint8) for n in sizes]
    dev = [torch.empty(2 * n, dtype=torch.uint8, device="cuda") for n in sizes]
    s = torch.cuda.current_stream()
    ptrs = []
    for p, h, d, n in zip(pinned, host, dev, sizes):
        ptrs.append((d.data_ptr(), p.data_ptr(), n))
        ptrs.append((d.data_ptr() + n, h.ctypes.data, n))
    c = np.array(ptrs, dtype=np.uint64)
    dst, src, nb = (np.ascontiguousarray(c[:, k]) for k in range(3))
    _lib.check(L.xc_copy_list(len(ptrs), dst.ctypes.data, src.ctypes.data, nb.ctypes.data,
                              s.cuda_stream))
    back = [torch.empty(2 * n, dtype=torch.uint8).pin_memory() for n in sizes]
    c = np.array([(b.data_ptr(), d.data_ptr(), 2 * n) for b, d, n in zip(back, dev, sizes)],
                 dtype=np.uint64)
    dst, src, nb = (np.ascontiguousarray(c[:, k]) for k in range(3))
    _lib.check(L.xc_copy_list(len(sizes), dst.ctypes.data, src.ctypes.data, nb.ctypes.data,
                              s.cuda_stream))
    s.synchronize()
    for p, h, b, n in zip(pinned, host, back, sizes):
        np.testing.assert_array_equal(b.numpy()[:n], p.numpy())
        np.testing.assert_array_equal(b.numpy()[n:], h)
    bad = np.array([0], dtype=np.uint64)
    one = np.array([4], dtype=np.uint64)
    assert L.xc_copy_list(1, bad.ctypes.data, bad.ctypes.data, one.ctypes.data,
                          s.cuda_stream) != 0
