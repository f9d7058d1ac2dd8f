"""A calc_cape service loop on one GPU: requests arrive with their inputs in
host memory, are admitted by device-memory budget, and run in ragged
batches on the batch executor (``xcape_gb300.batch.CapeBatch``, one graph
launch per batch).

``CapeServer`` keeps two device arenas and two pinned staging areas.  A
batch is admitted into the free arena (requests are taken in arrival order
while their inputs and outputs fit), its inputs are copied host -> pinned ->
device on a copy stream (one library call queues all of a batch's copies,
xc_copy_list), the executor runs it on a compute stream once the
copies are in, and its outputs (cape, cin, mulvl, z_out) go back to pinned
memory on the same stream.  ``launch`` only queues that work; ``finish``
waits for a batch and hands out each request's results.  A loop that
launches batch k + 1 before finishing batch k therefore prepares and copies
the next batch while the current one runs, and the two executor slots
(tables and graphs) alternate in step with the arenas.

    server = CapeServer(memory_budget=4 << 30, guess="learned")
    pending = [...]                               # Request objects
    inflight = None
    while pending or inflight:
        batch = server.launch(server.admit(pending)) if pending else None
        if inflight:
            for req, result in server.finish(inflight): ...
        inflight = batch

The reference has no serving loop: its unit of work is one ``calc_cape``
call on one array (src/xcape/core.py:130-235); each request here is such a
call, with the same options and results.
"""
import numpy as np

from .batch import CapeBatch

_ALIGN = 256


def _nbytes(n):
    return (int(n) + _ALIGN - 1) // _ALIGN * _ALIGN


class Request:
    """One calc_cape call, its inputs in host memory in the units of
    calc_cape (hPa, degC): t and td [n2][ld] float32 (the first nk of every
    ld values are a column's levels; ld = nk for a dense array), p the same
    (sigma/model levels) or [>= nk] (pressure levels), ps, ts and tds [n2];
    and its options.  Arrays in pinned memory are copied to the device
    directly; others go through the server's pinned staging first."""

    def __init__(self, p, t, td, ps, ts, tds, source="surface", adiabat="pseudo-liquid",
                 vertical_lev="sigma", pinc=500.0, ml_depth=500.0, nk=None, tag=None):
        def arr(a, ndim):
            a = np.asarray(a)
            if a.dtype != np.float32 or a.ndim != ndim or not a.flags.c_contiguous:
                raise ValueError("request arrays must be C-contiguous float32 "
                                 f"({ndim}-D here)")
            return a
        self.t, self.td = arr(t, 2), arr(td, 2)
        self.n2, self.ld = self.t.shape
        self.nk = self.ld if nk is None else int(nk)
        if not 1 <= self.nk <= self.ld or self.td.shape != self.t.shape:
            raise ValueError("inconsistent request shapes")
        self.p = arr(p, 2 if vertical_lev in ("sigma", "model") else 1)
        if (self.p.ndim == 2 and self.p.shape != self.t.shape) or \
                (self.p.ndim == 1 and self.p.shape[0] < self.nk):
            raise ValueError("p does not match t")
        self.ps, self.ts, self.tds = (arr(x, 1) for x in (ps, ts, tds))
        if any(x.shape != (self.n2,) for x in (self.ps, self.ts, self.tds)):
            raise ValueError("surface arrays must have one value per column")
        self.source, self.adiabat, self.vertical_lev = source, adiabat, vertical_lev
        self.pinc, self.ml_depth, self.tag = pinc, ml_depth, tag
        self.pinned = tuple(_pinned(a) for a in self.inputs())

    def inputs(self):
        return (self.p, self.t, self.td, self.ps, self.ts, self.tds)

    def device_bytes(self):
        """Arena bytes of the request: inputs and the four outputs."""
        return sum(_nbytes(a.nbytes) for a in self.inputs()) + 4 * _nbytes(4 * self.n2)

    def staging_bytes(self):
        """Pinned staging bytes of the request: its pageable inputs and the
        four outputs."""
        return sum(_nbytes(a.nbytes) for a, pin in zip(self.inputs(), self.pinned) if not pin) + \
            4 * _nbytes(4 * self.n2)


def _pinned(a):
    import torch
    return torch.from_numpy(a.reshape(-1).view(np.uint8)).is_pinned()


def _copy_list(copies, stream):
    """Queues [(dst pointer, src pointer, bytes)] on `stream` with one
    library call (xc_copy_list: one cudaMemcpyAsync per entry)."""
    from . import _lib
    if not copies:
        return
    c = np.array(copies, dtype=np.uint64).reshape(-1, 3)
    dst, src, nb = (np.ascontiguousarray(c[:, k]) for k in range(3))
    _lib.check(_lib.lib().xc_copy_list(len(copies), dst.ctypes.data, src.ctypes.data,
                                       nb.ctypes.data, stream.cuda_stream))


class _Batch:
    def __init__(self, slot, reqs, views, events):
        self.slot, self.reqs, self.views = slot, reqs, views
        self.events = events  # copies start, copies in, run done, results out
        self.done = events[-1]
        self.h2d_bytes = 0


class CapeServer:
    """The service loop's device side (see the module docstring)."""

    def __init__(self, memory_budget=4 << 30, max_requests=4096, guess="learned",
                 staging_bytes=None, device=None):
        import torch
        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else device)
        self.arena_bytes = int(memory_budget) // 2 // _ALIGN * _ALIGN
        self.staging_bytes = (self.arena_bytes if staging_bytes is None
                              else int(staging_bytes) // _ALIGN * _ALIGN)
        self.arena = [torch.empty(self.arena_bytes, dtype=torch.uint8, device=self.device)
                      for _ in range(2)]
        self.staging = [torch.empty(self.staging_bytes, dtype=torch.uint8).pin_memory()
                        for _ in range(2)]
        self.copy_stream = torch.cuda.Stream(self.device)
        self.compute_stream = torch.cuda.Stream(self.device)
        # columns of one batch: a column takes at least 36 arena bytes (one
        # level of t and td, three surface values, four outputs), and every
        # request rounds up to 32 columns
        self.executor = CapeBatch(max_requests=max_requests,
                                  max_columns=self.arena_bytes // 36 + 32 * max_requests,
                                  guess=guess)
        self.max_requests = max_requests
        self.slot = 0
        self.busy = [None, None]
        # per finished batch: host-to-device copies, executor run and
        # device-to-host copies (ms, CUDA events) and bytes copied in
        self.stats = {"batches": 0, "h2d_ms": 0.0, "run_ms": 0.0, "d2h_ms": 0.0,
                      "h2d_bytes": 0, "per_batch": []}

    def admit(self, pending):
        """Takes requests from the front of `pending` (a list, consumed) while
        they fit in one arena (and their pageable inputs and outputs in one
        staging area), at most max_requests; returns them.  A request larger
        than an arena or a staging area is refused with ValueError."""
        take, used, staged = [], 0, 0
        while pending and len(take) < self.max_requests:
            need, stage = pending[0].device_bytes(), pending[0].staging_bytes()
            if need > self.arena_bytes or stage > self.staging_bytes:
                raise ValueError(f"request of {need} device bytes ({stage} staged) exceeds the "
                                 f"{self.arena_bytes}-byte arena or the {self.staging_bytes}-byte "
                                 "staging; raise memory_budget or staging_bytes")
            if used + need > self.arena_bytes or staged + stage > self.staging_bytes:
                break
            take.append(pending.pop(0))
            used += need
            staged += stage
        return take

    def launch(self, reqs):
        """Queues one batch: host-to-device copies of the inputs (pinned ones
        directly, others through the pinned staging), the executor run and
        the device-to-host copies of the outputs.  Returns a handle for
        finish().  The arena it takes must not hold an unfinished batch."""
        torch = self.torch
        k = self.slot
        self.slot ^= 1
        if self.busy[k] is not None:
            raise RuntimeError("the arena still holds an unfinished batch: finish it first")
        arena, stage = self.arena[k], self.staging[k]
        st = stage.numpy()
        arena_ptr, stage_ptr = arena.data_ptr(), stage.data_ptr()
        off = soff = 0  # arena and staging offsets
        views = []
        copies = []  # (device pointer, host pointer, bytes) of the inputs

        def place(a, pinned):
            nonlocal off, soff
            n = a.nbytes
            if pinned:
                src = a.ctypes.data
            else:  # pageable: through the staging
                st[soff:soff + n] = a.reshape(-1).view(np.uint8)
                src = stage_ptr + soff
                soff += _nbytes(n)
            copies.append((arena_ptr + off, src, n))
            v = (off, n)
            off += _nbytes(n)
            return v

        def alloc(n):
            nonlocal off, soff
            v = (off, n, soff)  # arena offset, bytes, staging offset of the result
            off += _nbytes(n)
            soff += _nbytes(n)
            return v
        for r in reqs:
            v = dict(zip(("p", "t", "td", "ps", "ts", "tds"),
                         (place(a, pin) for a, pin in zip(r.inputs(), r.pinned))))
            for name in ("cape", "cin", "mulvl", "z_out"):
                v[name] = alloc(4 * r.n2)
            views.append(v)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        copied = ev[1]
        ev[0].record(self.copy_stream)
        _copy_list(copies, self.copy_stream)
        copied.record(self.copy_stream)

        def dev(view, dtype, shape):
            o, n = view[0], view[1]
            return arena[o:o + n].view(dtype).view(shape)
        descs = []
        f32, i32 = torch.float32, torch.int32
        for r, v in zip(reqs, views):
            t2 = (r.n2, r.ld)
            p = dev(v["p"], f32, r.p.shape)
            if p.dim() == 2:
                p = p[:, :r.nk]
            else:
                p = p[:r.nk]
            q = self.executor.request(p, dev(v["t"], f32, t2)[:, :r.nk],
                                      dev(v["td"], f32, t2)[:, :r.nk],
                                      dev(v["ps"], f32, (r.n2,)), dev(v["ts"], f32, (r.n2,)),
                                      dev(v["tds"], f32, (r.n2,)), source=r.source,
                                      adiabat=r.adiabat, vertical_lev=r.vertical_lev,
                                      pinc=r.pinc, ml_depth=r.ml_depth,
                                      outputs=[dev(v[n], i32 if n == "mulvl" else f32, (r.n2,))
                                               for n in ("cape", "cin", "mulvl", "z_out")])
            descs.append(q)
        self.compute_stream.wait_event(copied)
        done = ev[3]
        with torch.cuda.stream(self.compute_stream):
            if descs:
                self.executor.run(descs, stream=self.compute_stream)
            ev[2].record(self.compute_stream)
            # the outputs back into the staging (the inputs staged there have
            # been copied: the compute stream waited for the copies)
            _copy_list([(stage_ptr + v[name][2], arena_ptr + v[name][0], v[name][1])
                        for v in views for name in ("cape", "cin", "mulvl", "z_out")],
                       self.compute_stream)
            done.record(self.compute_stream)
        b = _Batch(k, reqs, views, ev)
        b.h2d_bytes = sum(n for _, _, n in copies)
        self.busy[k] = b
        return b

    def finish(self, batch):
        """Waits for `batch`; returns [(request, (cape, cin, mulvl, z_out))]
        with the results as numpy arrays (copies)."""
        batch.done.synchronize()
        e = batch.events
        self.stats["batches"] += 1
        self.stats["h2d_ms"] += e[0].elapsed_time(e[1])
        self.stats["run_ms"] += e[1].elapsed_time(e[2])
        self.stats["d2h_ms"] += e[2].elapsed_time(e[3])
        self.stats["h2d_bytes"] += batch.h2d_bytes
        self.stats["per_batch"].append((batch.h2d_bytes, e[0].elapsed_time(e[1]),
                                        e[1].elapsed_time(e[2])))
        st = self.staging[batch.slot].numpy()
        out = []
        for r, v in zip(batch.reqs, batch.views):
            res = []
            for name, dt in (("cape", np.float32), ("cin", np.float32), ("mulvl", np.int32),
                             ("z_out", np.float32)):
                _, n, so = v[name]
                res.append(st[so:so + n].view(dt).copy())
            out.append((r, tuple(res)))
        self.busy[batch.slot] = None
        return out

    def close(self):
        self.executor.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
