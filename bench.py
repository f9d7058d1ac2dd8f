"""Benchmark of the CAPE/CIN hot path on the pressure-level workload.

Workload (one "step"): calc_cape on 721 x 1440 = 1,038,240 columns x 37
pressure levels (1000..100 hPa, float32, ps ~ U(700, 1030) hPa so the valid
level count is ragged), once with source='most-unstable' and once with
source='mixed-layer' (ml_depth 500 m), pseudo-liquid adiabat, pinc 500 Pa.
value = columns per second (both sources computed for every column).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--guess learned|plain|extrapolated|secant|learned-every]
                    [--workload cape|srh]

The headline is the learned-guess solver (guess='learned'); the same run times
the plain solver (the reference's iteration) on the same launches for the
"learned-guess vs plain" ratio, and surface-based parcels for both.

--impl reference times the reference algorithm on the host cores (the CPU
restatement of the Fortran in oracle/, all host threads, a bounded sample of
the same workload per step).  Under torchrun every rank processes its own
equal share of columns (weak scaling, no collective on the data path).
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GRID_SHAPE = (721, 1440)
NLEV = 37
SOURCES = (("most-unstable", 2), ("mixed-layer", 3))
PINC = 500.0
ML_DEPTH = 500.0
ADIABAT = 1
METRIC = "CAPE/CIN columns/s at 1M×37 lev: learned-guess vs plain CUDA, |ΔCAPE|≤1 J/kg"
SRH_METRIC = "SRH columns/s at 1M×50 lev (calc_srh, depth 1000+3000 m)"
CPU_SAMPLE = 131072      # columns per CPU-baseline measurement
# Recorded values, not measurements of the run that prints them: DRAM bytes
# (read + write) of one most-unstable launch of the lift on this workload, and
# the issue-slot activity (smsp__issue_active over active cycles), tensor-pipe
# share and active threads per warp instruction, from `ncu --set full`
# captures of `bench.py --profile` (profiles/cape_kernel_pressure_1M.md).
NCU_RECORDED = "ncu --set full of bench.py --profile, profiles/cape_kernel_pressure_1M.md"
NCU_TRAFFIC = {"learned": 689_983_744, "plain": 728_342_784}
NCU_ISSUE = {"learned": {"issue_active": 0.811, "tensor_pipe_active": 0.0131,
                         "threads_per_warp_instruction": 28.65},
             "plain": {"issue_active": 0.879, "tensor_pipe_active": 0.0,
                       "threads_per_warp_instruction": 27.11}}
ACC_SAMPLE = 8192        # columns checked against the FP64 oracle in the CPU leg (strided)
CPU_SAMPLE_1T = 8192     # columns per single-core CPU-baseline measurement
REF_SAMPLE = 32768       # columns per --impl reference step


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--guess", default="learned",
                    choices=["plain", "extrapolated", "learned", "secant", "learned-every",
                             "learned-warp"])
    ap.add_argument("--workload", default="cape",
                    choices=["cape", "srh", "serve", "adiabats", "cape_srh", "dask"])
    ap.add_argument("--serve-seconds", type=float, default=10.0,
                    help="length of the request trace of --workload serve")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-order", action="store_true",
                    help="launch the lift in natural column order (no ordering workspace)")
    ap.add_argument("--profile", action="store_true",
                    help="one launch per source and exit (for ncu captures)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# distributed plumbing (one process per GPU)

def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def shard(n, world, rank):
    """Contiguous, near-equal share [lo, hi) of n columns for `rank`."""
    base, rem = divmod(n, world)
    lo = rank * base + min(rank, rem)
    return lo, lo + base + (1 if rank < rem else 0)


def init_dist(world, backend):
    if world <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group(backend=backend)
    return dist


def max_over_ranks(dist, value, device=None):
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# clocks during the timed region

# NVML's clock-event reason bits (nvml.h, nvmlClocksEventReason*), under the
# names nvidia-smi prints for them.
NVML_REASONS = ((0x4, "sw_power_cap"), (0x8, "hw_slowdown"), (0x20, "sw_thermal_slowdown"),
                (0x40, "hw_thermal_slowdown"), (0x80, "hw_power_brake_slowdown"))


class NvmlReader:
    """Read-only NVML queries (SM clock, its maximum, clock-event reasons,
    power) for the GPU behind one CUDA device, through ctypes.

    The GPU is found by the CUDA device's UUID, else its PCI bus id, because
    CUDA's device numbering (CUDA_VISIBLE_DEVICES) need not be NVML's.  It
    only reads: no clock, power or mode setting is touched."""

    def __init__(self, device_index, lib=None, props=None):
        import ctypes
        self.ct = ctypes
        if lib is None:
            lib = ctypes.CDLL("libnvidia-ml.so.1")
        if props is None:
            import torch
            props = torch.cuda.get_device_properties(device_index)
        rc = lib.nvmlInit_v2()
        if rc:
            raise OSError(f"nvmlInit_v2 returned {rc}")
        self.lib = lib
        self.h = ctypes.c_void_p()
        found = False
        uuid = getattr(props, "uuid", None)
        if uuid is not None:
            u = str(uuid)
            u = u if u.startswith(("GPU-", "MIG-")) else "GPU-" + u
            found = lib.nvmlDeviceGetHandleByUUID(u.encode(), ctypes.byref(self.h)) == 0
        if not found and hasattr(props, "pci_bus_id"):
            bus = f"{props.pci_domain_id:08x}:{props.pci_bus_id:02x}:{props.pci_device_id:02x}.0"
            found = lib.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(self.h)) == 0
        if not found:
            lib.nvmlShutdown()
            raise OSError("no NVML device for this CUDA device")
        self._reasons = (getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None)
                         or lib.nvmlDeviceGetCurrentClocksThrottleReasons)
        mx = ctypes.c_uint(0)
        self.max_mhz = (float(mx.value)
                        if lib.nvmlDeviceGetMaxClockInfo(self.h, 1, ctypes.byref(mx)) == 0 else None)

    def sample(self):
        """(SM MHz, reason bits, watts or None), or None if a query failed."""
        ct = self.ct
        mhz, bits, mw = ct.c_uint(0), ct.c_ulonglong(0), ct.c_uint(0)
        if self.lib.nvmlDeviceGetClockInfo(self.h, 1, ct.byref(mhz)) != 0:  # NVML_CLOCK_SM
            return None
        if self._reasons(self.h, ct.byref(bits)) != 0:
            return None
        watts = mw.value / 1e3 if self.lib.nvmlDeviceGetPowerUsage(self.h, ct.byref(mw)) == 0 else None
        return float(mhz.value), int(bits.value), watts

    def close(self):
        self.lib.nvmlShutdown()


class ClockSampler:
    """SM clocks and clock-event reasons of this process's GPU while the
    timed region runs (the `with` block holds exactly that region).

    NVML is polled every 2 ms from a thread, and once on entry and once on
    exit, so a timed region of a few tens of milliseconds still holds many
    samples.  Without NVML it falls back to an `nvidia-smi -lms 200` loop
    (started before the region, so at least one sample falls near it)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    PERIOD_S = 0.002

    def __init__(self, index, reader=None):
        self.index = index
        self.reader = reader
        self.source = None
        self.proc = None
        self.lines = []
        self.samples = []  # (SM MHz, reason bits, watts) from NVML
        self._stop = threading.Event()
        self.thread = None

    def __enter__(self):
        if self.reader is None:
            try:
                self.reader = NvmlReader(self.index)
            except Exception:
                self.reader = None
        if self.reader is not None:
            self.source = "nvml"
            self._take()
            self.thread = threading.Thread(target=self._poll, daemon=True)
            self.thread.start()
            return self
        try:
            sel = str(self.index)
            try:
                import torch
                u = str(torch.cuda.get_device_properties(self.index).uuid)
                sel = u if u.startswith("GPU-") else "GPU-" + u
            except Exception:
                pass
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", sel, f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            self.source = "nvidia-smi"
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 3.0:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def _take(self):
        s = self.reader.sample()
        if s is not None:
            self.samples.append(s)

    def _poll(self):
        while not self._stop.wait(self.PERIOD_S):
            self._take()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.reader is not None:
            self._stop.set()
            if self.thread is not None:
                self.thread.join(timeout=5)
            self._take()
            self.reader.close()
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, power, reasons = [], [], [], set()
        if self.samples:
            for mhz, bits, watts in self.samples:
                sm.append(mhz)
                if watts is not None:
                    power.append(watts)
                reasons.update(name for bit, name in NVML_REASONS if bits & bit)
            if self.reader.max_mhz is not None:
                mx.append(self.reader.max_mhz)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            try:
                power.append(float(f[3]))
            except ValueError:
                pass
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        loaded = [s for s in sm if s > 0.5 * max(sm)] or sm
        out = {"sm_mhz": float(np.median(loaded)), "sm_max_mhz": float(max(mx)) if mx else None,
               "reasons": sorted(reasons), "samples": len(sm), "source": self.source}
        if power:
            out["power_w_median"] = float(np.median(power))
        return out


# ---------------------------------------------------------------------------
# workloads

def cape_inputs(lo, hi):
    from xcape_gb300 import synthetic as S
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=GRID_SHAPE, nlev=NLEV)
    n2 = ps.size
    t, td = t.reshape(n2, NLEV)[lo:hi], td.reshape(n2, NLEV)[lo:hi]
    ps, ts, tds = (a.reshape(n2)[lo:hi] for a in (ps, ts, tds))
    return plev, t, td, ps, ts, tds


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_cape(sample, nthreads):
    """Times the oracle (FP32 restatement of the Fortran) on `sample` columns
    per source with `nthreads` OpenMP threads; returns columns/s."""
    import oracle as O
    plev, t, td, ps, ts, tds = cape_inputs(0, sample)
    start = O.pres_lev_pos(plev, ps)
    O.loopcape(plev, t[:64], td[:64], ps[:64], ts[:64], tds[:64], PINC, 2, ML_DEPTH, ADIABAT,
               start=start[:64], p_is_1d=True, nthreads=nthreads)
    t0 = time.perf_counter()
    for _, src in SOURCES:
        O.loopcape(plev, t, td, ps, ts, tds, PINC, src, ML_DEPTH, ADIABAT, start=start,
                   p_is_1d=True, nthreads=nthreads)
    return sample / (time.perf_counter() - t0)


def accuracy_vs_fp64(outs, nthreads, host):
    """|dCAPE|, |dCIN| of the timed launches' outputs on ACC_SAMPLE columns
    taken with a constant stride over the whole 721 x 1440 grid (every
    latitude band of the synthetic field, hence the whole ps range) against
    the FP64 oracle (the checker), over the columns whose FP64 iteration
    converges and, for most-unstable parcels, whose source level is the same
    (theta-e near-ties pick another parcel)."""
    import oracle as O
    import torch
    plev, t, td, ps, ts, tds = host
    n2 = ps.shape[0]
    idx = np.arange(ACC_SAMPLE, dtype=np.int64) * (n2 // ACC_SAMPLE)
    t, td, ps, ts, tds = (np.ascontiguousarray(a[idx]) for a in (t, td, ps, ts, tds))
    start = O.pres_lev_pos(plev, ps)
    res = {"columns": ACC_SAMPLE, "sample": f"every {n2 // ACC_SAMPLE}th column of {n2}"}
    for src, code in SOURCES:
        ref = O.loopcape(plev, t, td, ps, ts, tds, PINC, code, ML_DEPTH, ADIABAT, start=start,
                         p_is_1d=True, nthreads=nthreads, precision="f64", stats=True)
        sel = torch.from_numpy(idx).to(outs[src][0].device)
        cape, cin, _, mulvl = (x.index_select(0, sel).cpu().numpy() for x in outs[src])
        ok = (ref["status"] & 1) == 0
        if code == 2:
            ok &= mulvl == ref["mulvl"]
        dc = np.abs(cape[ok].astype(np.float64) - ref["cape"][ok])
        dn = np.abs(cin[ok].astype(np.float64) - ref["cin"][ok])
        res[src] = {"compared": int(ok.sum()), "max_abs_dcape": float(dc.max()),
                    "frac_dcape_le_1": float(np.mean(dc <= 1.0)),
                    "frac_dcin_le_1_or_0.1pct": float(np.mean(
                        dn <= np.maximum(1.0, 1e-3 * np.abs(ref["cin"][ok]))))}
    return res


def column_levels(plev, ps, ts):
    """Per-column work units of the lift, from the inputs: the levels each
    column's passes walk (surface included: nk - start + 2, for columns with
    ts > 0, CAPE_CODE_model_lev.f90:77), and of them the levels at or below
    500 hPa that the most-unstable search evaluates theta-e on (:261-281).
    start is the reference's masked-argmin rule (src/xcape/core.py:286-289)."""
    nk = plev.shape[0]
    d = ps[None, :].astype(np.float64) - plev[:, None].astype(np.float64)
    start = np.ma.masked_less(d, 0).argmin(axis=0).astype(np.int64) + 1
    live = ts > 0
    ncl = np.where(live, nk - start + 2, 0)
    ge500 = np.cumsum((plev >= 500.0)[::-1])[::-1]           # levels >= 500 hPa from k on
    nmu = np.where(live, 1 + ge500[start - 1], 0)             # + the surface
    return {"columns": int(live.sum()), "levels": int(ncl.sum()), "levels_mu": int(nmu.sum())}


# XU (transcendental unit) lane operations of the accelerated solvers per unit
# of work, counted from the column code (cape_column.cuh, xc_common.cuh): each
# approximate exp (ex2), log (lg2) and reciprocal (rcp) is one XU operation.
#   environment of a level (make_env<true>): pi = 2^(k log2 p) 2, qsat_fast
#     3, theta and theta_v 2                                          -> 7
#   ascent level: the environment, the two buoyancy divides, 1/dp and
#     1/nloop                                                         -> 11
#   most-unstable level (p >= 500 hPa): qsat_fast 3 + getthe_fast 8    -> 11
#   mixed-layer pass level: the environment                           -> 7
#   sub-step: log2 p2, pi2, the Newton step's reciprocal               -> 3
#   iteration (accel_map, liquid): qsat 3, exponent 1, exp 1          -> 5
#   step between iterations (secant quotient, root step)             -> 2
XU_MODEL = {"ascent_level": 11, "mu_level": 11, "ml_level": 7, "substep": 3, "iteration": 5,
            "step": 2}
# FP32 lane operations (FFMA, FADD, FMUL, FMNMX, FSETP, FSEL and the
# multiplies of the approximate functions) of the same code, per unit:
#   iteration (accel_map, liquid, without the slope): t2, qsat 7, the clamps
#     5, the sums 3, lhv/rm/cpm 5, the exponent's quotient 5, the exp 3    -> 29
#   sub-step: p2, log p, pi2 4; the guess 1; the convergence test 2; the
#     Newton step 8; the Newton-point ending 16; the rate 3; the network's
#     onset test 2; the slope of the first evaluation (saturated) 16       -> 52
#   step between iterations: secant quotient 3, root step 6, test 2      -> 12
#   ascent level: the environment 16, height 5, sub-step count and dp 13,
#     buoyancy 9, areas and sums 20                                        -> 63
#   most-unstable level: the level 4, qsat 7, getthe_fast 18, the maximum
#     4                                                                    -> 33
#   mixed-layer pass level: the environment 16, the averages 9             -> 25
FP32_MODEL = {"ascent_level": 63, "mu_level": 33, "ml_level": 25, "substep": 52,
              "iteration": 29, "step": 12}


def model_ops(model, work, lev, source_code):
    """Operations of `model` for one launch: work = (sub-steps, iterations)
    from the kernel's counters, lev = column_levels()."""
    nsub, niter = work
    ops = model["ascent_level"] * lev["levels"] + model["substep"] * nsub \
        + model["iteration"] * niter + model["step"] * max(0, niter - nsub)
    if source_code == 2:
        ops += model["mu_level"] * lev["levels_mu"]
    elif source_code == 3:
        ops += model["ml_level"] * lev["levels"]
    return float(ops)


def pipe_peaks(L, stream_ptr):
    """FP32 and XU lane-operation rates of this GPU (xc_measure_pipe_peaks),
    best of three."""
    import ctypes
    best = [0.0, 0.0]
    for _ in range(3):
        a, b = ctypes.c_double(), ctypes.c_double()
        rc = L.xc_measure_pipe_peaks(ctypes.byref(a), ctypes.byref(b), stream_ptr)
        if rc != 0:
            return None
        best = [max(best[0], a.value), max(best[1], b.value)]
    return {"fp32_gops": best[0], "xu_gops": best[1],
            "how": "xc_measure_pipe_peaks: 8 independent FFMA chains / 8 independent "
                   "ex2.approx chains per thread, 8 x 256 threads per SM, CUDA events, best of 3"}


def run_reference(args):
    """--impl reference: the reference algorithm on the host cores."""
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    import oracle as O
    nthreads = os.cpu_count() or 1
    plev, t, td, ps, ts, tds = cape_inputs(0, REF_SAMPLE)
    start = O.pres_lev_pos(plev, ps)

    def step():
        for _, src in SOURCES:
            O.loopcape(plev, t, td, ps, ts, tds, PINC, src, ML_DEPTH, ADIABAT, start=start,
                       p_is_1d=True, nthreads=nthreads)
    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = (time.perf_counter() - t0) / args.steps
    value = REF_SAMPLE / dt
    line = {
        "metric": METRIC, "value": value, "unit": "columns/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "impl": "reference",
        "config": {"workload": "calc_cape pressure levels 721x1440 cols x 37 lev, sources "
                   "most-unstable + mixed-layer(500 m), pseudo-liquid, pinc 500 Pa",
                   "columns": GRID_SHAPE[0] * GRID_SHAPE[1], "levels": NLEV},
        "cpu_baseline": {"value": value, "unit": "columns/s", "cores": nthreads, "kind": "port",
                         "sample": f"{REF_SAMPLE} of the 1,038,240 columns per step, both "
                                   "sources, OpenMP over columns"},
        "e2e": {"value": value, "unit": "columns/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = init_dist(world, "nccl")
    dev = torch.device("cuda", local)
    from xcape_gb300 import _lib
    L = _lib.lib()
    guess = {"plain": _lib.XC_GUESS_PLAIN, "learned": _lib.XC_GUESS_LEARNED,
             "extrapolated": _lib.XC_GUESS_EXTRAPOLATED, "secant": _lib.XC_GUESS_SECANT,
             "learned-every": _lib.XC_GUESS_LEARNED_EVERY,
             "learned-warp": _lib.XC_GUESS_LEARNED_WARP}[args.guess]
    # the network serves the headline and the lockstep variant timed beside it
    from xcape_gb300 import guess as guess_net
    guess_net.ensure_loaded()

    n_total = GRID_SHAPE[0] * GRID_SHAPE[1]
    lo, hi = shard(n_total, world, rank)
    plev, t, td, ps, ts, tds = cape_inputs(lo, hi)
    n2 = hi - lo
    P, T, TD, PS, TS, TDS = (torch.from_numpy(np.ascontiguousarray(a)).to(dev)
                             for a in (plev, t, td, ps, ts, tds))
    # outputs [source][n2] in one array each, as xc_loopcape_multi writes them
    nsrc = len(SOURCES)
    out_all = [torch.empty(nsrc * n2, dtype=torch.float32, device=dev) for _ in range(3)] + \
        [torch.empty(nsrc * n2, dtype=torch.int32, device=dev)]
    outs = {src: [x[j * n2:(j + 1) * n2] for x in out_all] for j, (src, _) in enumerate(SOURCES)}
    src_codes = (ctypes.c_int * nsrc)(*[code for _, code in SOURCES])
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream
    ws_bytes = _lib.workspace_bytes(n2)
    wsbuf = torch.empty(ws_bytes + 256, dtype=torch.uint8, device=dev)
    ws = wsbuf.data_ptr() + (-wsbuf.data_ptr()) % 256
    order = not args.no_order
    # per step: the 3 ordering kernels once, then one lift per source
    launches_per_step = (3 if order else 0) + nsrc

    def launch(src_code, o, counters=None, g=None):
        cape, cin, zout, mulvl = o
        _lib.check(L.xc_loopcape_ex(2, P.data_ptr(), T.data_ptr(), TD.data_ptr(), PS.data_ptr(),
                                    TS.data_ptr(), TDS.data_ptr(), _lib.XC_F32, PINC, src_code,
                                    ML_DEPTH, ADIABAT, None, NLEV, n2,
                                    guess if g is None else g, cape.data_ptr(),
                                    cin.data_ptr(), mulvl.data_ptr(), zout.data_ptr(), None,
                                    counters, ws if order else None, ws_bytes if order else 0,
                                    sptr))

    def step():
        # both sources in one call: the columns are ordered once for both
        cape, cin, zout, mulvl = out_all
        _lib.check(L.xc_loopcape_multi(2, P.data_ptr(), T.data_ptr(), TD.data_ptr(), PS.data_ptr(),
                                       TS.data_ptr(), TDS.data_ptr(), _lib.XC_F32, PINC, nsrc,
                                       ctypes.cast(src_codes, ctypes.c_void_p), ML_DEPTH, ADIABAT,
                                       None, NLEV, n2, guess, cape.data_ptr(), cin.data_ptr(),
                                       mulvl.data_ptr(), zout.data_ptr(), None, None,
                                       ws if order else None, ws_bytes if order else 0, sptr))

    if args.profile:
        step()
        torch.cuda.synchronize()
        return 0

    # work accounting (untimed): sub-steps and iterations per source
    cnt = torch.zeros(2, dtype=torch.int64, device=dev)
    work = {}
    for src, code in SOURCES:
        cnt.zero_()
        launch(code, outs[src], cnt.data_ptr())
        torch.cuda.synchronize()
        work[src] = [int(x) for x in cnt.cpu()]

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = ev0.elapsed_time(ev1) / args.steps
    ms_max = max_over_ranks(dist, ms, dev)

    # per-kernel (per-source) average durations, for the roofline
    def time_source(code, o, g=None):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            launch(code, o, g=g)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    per_src_ms = {src: time_source(code, outs[src]) for src, code in SOURCES}

    # the same launches with the plain solver (the reference's iteration), and
    # surface-based parcels with both, into scratch outputs
    scratch = [torch.empty_like(x) for x in outs[SOURCES[0][0]]]
    plain_ms = {}
    compare = guess != _lib.XC_GUESS_PLAIN
    if compare:
        for _ in range(2):
            launch(SOURCES[0][1], scratch, g=_lib.XC_GUESS_PLAIN)
        plain_ms = {src: time_source(code, scratch, _lib.XC_GUESS_PLAIN) for src, code in SOURCES}
    sb_ms = {args.guess: time_source(1, scratch)}
    if compare:
        sb_ms["plain"] = time_source(1, scratch, _lib.XC_GUESS_PLAIN)
    # the learned solver against the method without the network
    # (extrapolated), and the network evaluated by each warp at every
    # saturated sub-step on the tensor cores (learned-warp): the same launches
    variant_ms, variant_work = {}, {}
    for vname, vcode in (("extrapolated", _lib.XC_GUESS_EXTRAPOLATED),
                         ("learned-warp", _lib.XC_GUESS_LEARNED_WARP)):
        if vcode == guess:
            continue
        launch(SOURCES[0][1], scratch, g=vcode)
        variant_ms[vname] = {src: time_source(code, scratch, vcode) for src, code in SOURCES}
        cnt.zero_()
        launch(SOURCES[0][1], scratch, cnt.data_ptr(), g=vcode)
        torch.cuda.synchronize()
        variant_work[vname] = [int(x) for x in cnt.cpu()]
    # every rank times its own shard: the job's time is the slowest rank's
    per_src_ms = {k: max_over_ranks(dist, v, dev) for k, v in per_src_ms.items()}
    plain_ms = {k: max_over_ranks(dist, v, dev) for k, v in plain_ms.items()}
    sb_ms = {k: max_over_ranks(dist, v, dev) for k, v in sb_ms.items()}
    variant_ms = {k: {s_: max_over_ranks(dist, v, dev) for s_, v in d.items()}
                  for k, d in variant_ms.items()}

    # end to end through the public API from pinned host memory
    import xcape_gb300 as X
    pinned = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in
              (plev, t, td, ps, ts, tds)]
    host = [x.numpy() for x in pinned]
    # both sources from one upload of the inputs (calc_cape_sources); the
    # outputs of both come back
    h2d = sum(a.nbytes for a in host)
    d2h = 4 * 4 * n2 * len(SOURCES)

    def e2e_step():
        return X.calc_cape_sources(*host, sources=[src for src, _ in SOURCES], ml_depth=ML_DEPTH,
                                   adiabat="pseudo-liquid", pinc=PINC, vertical_lev="pressure",
                                   guess=args.guess)
    e2e_step()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    e2e_steps = max(5, min(args.steps, 10))
    for _ in range(e2e_steps):
        e2e_step()
    e2e_dt = max_over_ranks(dist, (time.perf_counter() - t0) / e2e_steps, dev)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    cols_all = n_total if world > 1 else n2
    value = cols_all / (ms_max / 1e3)
    hbm_peak, peak_kind = measured_peaks()
    # algorithmic bytes of one launch: t, td (nk per column) + ps, ts, tds
    # in, cape/cin/z_out/mulvl out, p1d once.
    bytes_per_launch = n2 * (2 * NLEV * 4 + 3 * 4 + 4 * 4) + NLEV * 4
    top = max(per_src_ms, key=per_src_ms.get)
    top_code = dict(SOURCES)[top]
    top_s = per_src_ms[top] / 1e3
    clocks = clk.summary()
    roof = {"hbm": {"achieved": bytes_per_launch / top_s / 1e9, "peak": hbm_peak, "unit": "GB/s",
                    "peak_kind": peak_kind, "algorithmic_bytes": bytes_per_launch}}
    peaks = pipe_peaks(L, sptr)
    lev = column_levels(plev, ps, ts)
    if peaks and guess != _lib.XC_GUESS_PLAIN:
        # the compute side: FP32 and XU lane operations of the launch (the
        # op model above, on the kernel's own sub-step and iteration
        # counters) against the rates measured on this GPU
        for key, model, pk in (("fp32", FP32_MODEL, peaks["fp32_gops"]),
                               ("xu", XU_MODEL, peaks["xu_gops"])):
            ops = model_ops(model, work[top], lev, top_code)
            roof[key] = {"achieved": ops / top_s / 1e9, "peak": pk, "unit": "Gop/s",
                         "peak_kind": "measured (xc_measure_pipe_peaks)", "ops": ops}
    for v in roof.values():
        v["frac"] = v["achieved"] / v["peak"]
    bound = max(roof, key=lambda k: roof[k]["frac"])
    kernel = (f"cape_learned_kernel ({top})" if args.guess == "learned"
              else f"cape_kernel ({top})")
    roofline = {"bound": bound, "achieved": roof[bound]["achieved"], "peak": roof[bound]["peak"],
                "unit": roof[bound]["unit"], "frac": roof[bound]["frac"],
                "traffic": NCU_TRAFFIC.get(args.guess), "kernel": kernel,
                "traffic_source": f"recorded: {NCU_RECORDED}" if args.guess in NCU_TRAFFIC
                else None,
                "components": roof,
                "work": {"substeps": work[top][0], "iterations": work[top][1], **lev}}
    line = {
        "metric": METRIC, "value": value, "unit": "columns/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms_max,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "calc_cape pressure levels 721x1440 cols x 37 lev (1000..100 hPa), "
                               "ps~U(700,1030) ragged, sources most-unstable + mixed-layer(500 m), "
                               "pseudo-liquid, pinc 500 Pa",
                   "columns": cols_all, "levels": NLEV, "guess": args.guess,
                   "column_order": "start level x surface dewpoint" if order else "natural",
                   "l2": "inputs (307 MB) larger than L2 (129 MB), no flush"},
        "roofline": roofline,
        "pipe_peaks": peaks,
        "issue_roofline": dict(NCU_ISSUE.get(args.guess, {}), source=f"recorded: {NCU_RECORDED}")
        if args.guess in NCU_ISSUE else None,
        "per_source_ms": per_src_ms,
        "per_source_note": "one xc_loopcape_ex call per source, each ordering the columns itself; "
                           "the timed step orders them once for both (xc_loopcape_multi)",
        "vs_plain": ({"plain_value": cols_all / (sum(plain_ms.values()) / 1e3),
                      "plain_per_source_ms": plain_ms,
                      "speedup": sum(plain_ms.values()) / sum(per_src_ms.values()),
                      "surface_based_ms": sb_ms,
                      "surface_based_speedup": sb_ms["plain"] / sb_ms[args.guess]}
                     if compare else {"surface_based_ms": sb_ms}),
        "work": {k: {"substeps": v[0], "iterations": v[1]} for k, v in work.items()},
        "vs_extrapolated": {
            "per_source_ms": {args.guess: per_src_ms, **variant_ms},
            "speedup_over_extrapolated": {
                k: sum(variant_ms["extrapolated"].values()) / sum(v.values())
                for k, v in {args.guess: per_src_ms, **variant_ms}.items()}
            if "extrapolated" in variant_ms else None,
            "iterations_per_substep_most_unstable": {
                args.guess: work[SOURCES[0][0]][1] / max(1, work[SOURCES[0][0]][0]),
                **{k: v[1] / max(1, v[0]) for k, v in variant_work.items()}},
            "note": "extrapolated: the same Newton/secant solver without the network; "
                    "learned-warp: the network evaluated by every warp at every saturated "
                    "sub-step, in lockstep, on the tensor cores"},
        "e2e": {"value": cols_all / e2e_dt, "unit": "columns/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "api": "xcape_gb300.calc_cape_sources(numpy, pinned), both sources in one call"},
        "gpu_launches": args.steps * launches_per_step,
        "clocks": clocks,
    }
    if not args.no_cpu_baseline and world == 1:
        import oracle  # noqa: F401
        nth = os.cpu_count() or 1
        v = cpu_cape(CPU_SAMPLE, nth)
        v1 = cpu_cape(CPU_SAMPLE_1T, 1)
        line["cpu_baseline"] = {"value": v, "unit": "columns/s", "cores": nth, "kind": "port",
                                "sample": f"first {CPU_SAMPLE} columns, both sources, FP32 "
                                          "oracle (C restatement of the Fortran), OpenMP",
                                "single_core": {"value": v1, "cores": 1,
                                                "sample": f"first {CPU_SAMPLE_1T} columns"}}
        line["accuracy_vs_fp64"] = accuracy_vs_fp64(outs, nth, (plev, t, td, ps, ts, tds))
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def run_srh(args):
    """Secondary workload: calc_srh on 1024x1024 columns x 50 model levels."""
    import torch
    from xcape_gb300 import _lib
    from xcape_gb300 import synthetic as S
    L = _lib.lib()
    a = S.srh_c2()
    n2 = 1024 * 1024
    d = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in a]
    srm, slm = (torch.empty(n2, dtype=torch.float64, device="cuda") for _ in range(2))
    rm, lm, mean = (torch.empty(2 * n2, dtype=torch.float32, device="cuda") for _ in range(3))
    s = torch.cuda.current_stream().cuda_stream
    ref_out = None  # the reference precision's outputs at depth 3000 m

    for prec, prec_name, dt in ((0, "reference", "f64+f32"), (1, "fp32", "f32")):
        def step():
            for depth in (1000.0, 3000.0):
                _lib.check(L.xc_calc_srh_ex(1, *[x.data_ptr() for x in d], _lib.XC_F32, None,
                                            depth, 2.0, 50, n2, prec, srm.data_ptr(),
                                            slm.data_ptr(), rm.data_ptr(), lm.data_ptr(),
                                            mean.data_ptr(), s))
        for _ in range(max(3, args.warmup)):
            step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(0) as clk:
            e0.record()
            for _ in range(args.steps):
                step()
            e1.record()
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        outs = (srm, slm, rm, lm, mean)  # those of the last launch, depth 3000 m
        agree = None
        if ref_out is None:
            ref_out = [x.clone() for x in outs]
        else:
            # every column of the FP32 path against the reference precision
            agree = {"columns": n2, "depth_m": 3000.0,
                     "srh_max_abs_m2s2": max(float((x - y).abs().max())
                                             for x, y in zip(outs[:2], ref_out[:2])),
                     "storm_motion_max_abs_ms": max(float((x - y).abs().max())
                                                    for x, y in zip(outs[2:], ref_out[2:]))}
        hbm_peak, kind = measured_peaks()
        # algorithmic bytes of one launch: p, t, td, u, v (50 levels) and five
        # surface fields in, two f64 helicities and three f32 pairs out
        bytes_launch = n2 * (5 * 50 * 4 + 5 * 4 + 2 * 8 + 6 * 4)
        ach = bytes_launch / (ms / 2 / 1e3) / 1e9
        print(json.dumps({"metric": SRH_METRIC, "value": n2 / (ms / 1e3), "unit": "columns/s",
                          "n_gpus": 1, "steps": args.steps, "ms_per_step": ms, "dtype": dt,
                          "higher_is_better": True, "data": "synthetic",
                          "config": {"workload": "calc_srh 1024x1024 cols x 50 model levels, "
                                                 "depth 1000 and 3000 m, output_var='all'",
                                     "precision": prec_name},
                          "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm_peak,
                                       "unit": "GB/s", "frac": ach / hbm_peak,
                                       "peak_kind": kind},
                          "gpu_launches": 2 * args.steps,
                          **({"agreement_vs_reference_precision": agree} if agree else {}),
                          "clocks": clk.summary()}), flush=True)
    return 0


CAPE_SRH_METRIC = "calc_cape + calc_srh columns/s at 1M×50 lev: xc_cape_srh vs two calls"


def run_cape_srh(args):
    """--workload cape_srh: CAPE (most-unstable, pseudo-liquid) and SRH (depth
    3000 m, output_var='all') of the same 1024x1024 columns x 50 model levels,
    device-resident: xc_cape_srh (one kernel) against xc_loopcape_ex followed
    by xc_calc_srh_ex, for the plain and learned solvers and both SRH
    precisions.  Both paths order the columns for the lift."""
    import torch
    from xcape_gb300 import _lib, guess as G
    from xcape_gb300 import synthetic as S
    L = _lib.lib()
    G.ensure_loaded()
    a = S.srh_c2()
    n2, nk = 1024 * 1024, 50
    p, t, td, u, v, ps, ts, tds, us, vs = (torch.from_numpy(np.ascontiguousarray(x)).cuda()
                                           for x in a)
    cape, cin, zo = (torch.empty(n2, device="cuda") for _ in range(3))
    mul = torch.empty(n2, dtype=torch.int32, device="cuda")
    srm, slm = (torch.empty(n2, dtype=torch.float64, device="cuda") for _ in range(2))
    rm, lm, mean = (torch.empty(2 * n2, dtype=torch.float32, device="cuda") for _ in range(3))
    wsb = _lib.workspace_bytes(n2)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    lev = [x.data_ptr() for x in (p, t, td)]
    sfc = [x.data_ptr() for x in (ps, ts, tds)]
    outs_c = [x.data_ptr() for x in (cape, cin, mul, zo)]
    outs_s = [x.data_ptr() for x in (srm, slm, rm, lm, mean)]
    src, adi, depth = 2, 1, 3000.0

    def separate(g, prec):
        _lib.check(L.xc_loopcape_ex(1, *lev, *sfc, _lib.XC_F32, PINC, src, ML_DEPTH, adi, None, nk,
                                    n2, g, *outs_c, None, None, ws.data_ptr(), wsb, st))
        _lib.check(L.xc_calc_srh_ex(1, *lev, u.data_ptr(), v.data_ptr(), *sfc, us.data_ptr(),
                                    vs.data_ptr(), _lib.XC_F32, None, depth, 2.0, nk, n2, prec,
                                    *outs_s, st))

    def fused(g, prec):
        _lib.check(L.xc_cape_srh(1, *lev, u.data_ptr(), v.data_ptr(), *sfc, us.data_ptr(),
                                 vs.data_ptr(), _lib.XC_F32, PINC, src, ML_DEPTH, adi, None,
                                 depth, 2.0, nk, n2, g, prec, *outs_c, None, *outs_s,
                                 ws.data_ptr(), wsb, st))

    def timed(fn, g, prec):
        for _ in range(max(3, args.warmup)):
            fn(g, prec)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            fn(g, prec)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    if args.profile:
        # one launch of each schedule, plain solver and reference SRH stages
        # (the fused kernel's case), for ncu
        separate(_lib.XC_GUESS_PLAIN, 0)
        fused(_lib.XC_GUESS_PLAIN, 0)
        torch.cuda.synchronize()
        return 0
    res = {}
    with ClockSampler(0) as clk:
        for gname, g in (("learned", _lib.XC_GUESS_LEARNED), ("plain", _lib.XC_GUESS_PLAIN)):
            for pname, prec in (("fp32", 1), ("reference", 0)):
                ms_s = timed(separate, g, prec)
                ms_f = timed(fused, g, prec)
                res[f"{gname}/{pname}"] = {
                    "separate_ms": ms_s, "xc_cape_srh_ms": ms_f, "speedup": ms_s / ms_f,
                    # xc_cape_srh runs the lift and the level-parallel SRH
                    # kernel back to back for FP32 SRH stages on f32 inputs
                    "schedule": "two kernels" if pname == "fp32" else "fused kernel"}
    head = res["learned/reference"]
    line = {"metric": CAPE_SRH_METRIC, "value": n2 / (head["xc_cape_srh_ms"] / 1e3),
            "unit": "columns/s", "n_gpus": 1, "steps": args.steps,
            "ms_per_step": head["xc_cape_srh_ms"], "dtype": "f32 (SRH stages f64)",
            "higher_is_better": True, "data": "synthetic", "workload": "cape_srh",
            "config": {"workload": "calc_cape (most-unstable, pseudo-liquid, pinc 500 Pa) and "
                                   "calc_srh (depth 3000 m, output_var='all') of 1024x1024 cols "
                                   "x 50 model levels, device-resident, columns ordered",
                       "headline": "learned solver, SRH precision 'reference' (calc_srh's "
                                   "default)"},
            "per_mode": res, "gpu_launches": 4 * args.steps, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


SERVE_METRIC = "calc_cape serving loop: p50/p99 latency and columns/s, learned vs plain"
SERVE_RATE = 200.0        # requests per second (Poisson)
SERVE_POOL = 1 << 20      # columns of each device-resident input pool
SERVE_BASE = 1 << 17      # distinct synthetic columns tiled into a pool


def serve_trace(seconds, seed=4):
    """The request trace: Poisson arrivals, log-uniform column counts
    (1e3..1e6), uniform level counts (20..137), mixed grids, sources and
    adiabats, and where each request's columns sit in the input pools."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / SERVE_RATE)
        if t >= seconds:
            return out
        n2 = int(10 ** rng.uniform(3, 6))
        out.append({"arrival": t, "n2": n2, "nk": int(rng.integers(20, 138)),
                    "grid": ("sigma", "pressure")[int(rng.integers(2))],
                    "source": ("surface", "most-unstable", "mixed-layer")[int(rng.integers(3))],
                    "adiabat": ("pseudo-liquid", "reversible-liquid", "pseudo-ice",
                                "reversible-ice")[int(rng.integers(4))],
                    "c0": int(rng.integers(0, SERVE_POOL - n2 + 1))})


def run_serve(args):
    """--workload serve: calc_cape requests arriving at 200/s with their
    inputs in host memory, served by xcape_gb300.serve.CapeServer: admitted
    by device-memory budget, copied to the device and batched (one graph
    launch per batch), with batch k + 1 prepared and launched while batch k
    runs; for the learned and the plain solver on the same trace."""
    import torch
    from xcape_gb300 import synthetic as S
    from xcape_gb300.serve import CapeServer, Request
    world, rank, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    nl = 137
    reps = SERVE_POOL // SERVE_BASE

    def pinned_pool(a):
        # SERVE_BASE synthetic columns tiled to SERVE_POOL, in pinned host
        # memory: the buffers a service's clients write their requests into
        a = np.ascontiguousarray(a, np.float32)
        shape = (SERVE_POOL, nl) if a.ndim == 2 else (SERVE_POOL,)
        out = torch.empty(shape, dtype=torch.float32).pin_memory().numpy()
        out[...] = np.tile(a, (reps, 1) if a.ndim == 2 else reps)
        return out
    sig = S.sigma_c0(shape=(SERVE_BASE,), nlev=nl, seed=31, dtype=np.float32)
    sig_h = [pinned_pool(a) for a in sig]
    prs = S.pressure_c1(shape=(SERVE_BASE,), nlev=nl, seed=32)
    plev = np.ascontiguousarray(prs[0], np.float32)
    prs_h = [plev] + [pinned_pool(a) for a in prs[1:]]
    trace = serve_trace(args.serve_seconds)

    def request(r):
        c0, n2, nk = r["c0"], r["n2"], r["nk"]
        src = sig_h if r["grid"] == "sigma" else prs_h
        p = src[0][c0:c0 + n2] if r["grid"] == "sigma" else src[0]
        return Request(p, *[x[c0:c0 + n2] for x in src[1:]], source=r["source"],
                       adiabat=r["adiabat"], vertical_lev=r["grid"], nk=nk, tag=r)

    def serve(guess):
        with CapeServer(memory_budget=8 << 30, guess=guess, staging_bytes=512 << 20) as srv:
            # warm-up: one batch of the first requests
            srv.finish(srv.launch(srv.admit([request(r) for r in trace[:8]])))
            torch.cuda.synchronize()
            srv.stats = {k: [] if isinstance(v, list) else 0 for k, v in srv.stats.items()}
            lat, batches, cols, nxt = [], [], 0, 0
            pending, inflight = [], None
            busy, t_busy = 0.0, None
            t0 = time.perf_counter()
            while nxt < len(trace) or pending or inflight is not None:
                now = time.perf_counter() - t0
                while nxt < len(trace) and trace[nxt]["arrival"] <= now:
                    pending.append(request(trace[nxt]))
                    nxt += 1
                if not pending and inflight is None:
                    time.sleep(max(0.0, trace[nxt]["arrival"] - now))
                    continue
                batch = None
                if pending:
                    take = srv.admit(pending)
                    if t_busy is None:
                        t_busy = time.perf_counter()
                    batch = srv.launch(take)
                    batches.append(len(take))
                if inflight is not None:
                    results = srv.finish(inflight)
                    done = time.perf_counter() - t0
                    for q, _ in results:
                        lat.append(done - q.tag["arrival"])
                        cols += q.n2
                    if batch is None:  # the device goes idle
                        busy += time.perf_counter() - t_busy
                        t_busy = None
                inflight = batch
            wall = time.perf_counter() - t0
            st = dict(srv.stats)
        lat_ms = np.array(lat) * 1e3
        # host-to-device rate of the batches by their input volume
        pb = np.array(st.pop("per_batch"), dtype=np.float64).reshape(-1, 3)
        st["h2d_by_batch_size"] = {}
        for name, lo, hi in (("<64MB", 0, 64e6), ("64MB-1GB", 64e6, 1e9), (">1GB", 1e9, 1e30)):
            sel = (pb[:, 0] >= lo) & (pb[:, 0] < hi)
            if sel.any():
                st["h2d_by_batch_size"][name] = {
                    "batches": int(sel.sum()), "gbs": float(pb[sel, 0].sum() /
                                                           (pb[sel, 1].sum() * 1e-3) / 1e9),
                    "run_ms_mean": float(pb[sel, 2].mean())}
        st["h2d_gbs"] = st["h2d_bytes"] / (st["h2d_ms"] * 1e-3) / 1e9 if st["h2d_ms"] else None
        return {"requests": len(lat), "columns": cols, "wall_s": wall, "device_time": st,
                "columns_per_s": cols / wall, "busy_fraction": busy / wall,
                "columns_per_busy_s": cols / busy if busy else None,
                "p50_ms": float(np.percentile(lat_ms, 50)),
                "p99_ms": float(np.percentile(lat_ms, 99)),
                "max_ms": float(lat_ms.max()), "batches": len(batches),
                "mean_requests_per_batch": float(np.mean(batches)),
                "graph_launches": len(batches)}

    res = {g: serve(g) for g in ("learned", "plain")}
    line = {"metric": SERVE_METRIC, "impl": "ours", "n_gpus": 1, "workload": "serve",
            "config": {"rate_per_s": SERVE_RATE, "seconds": args.serve_seconds,
                       "requests": len(trace), "columns": "log-uniform 1e3..1e6",
                       "levels": "uniform 20..137", "grids": "sigma, pressure (ragged)",
                       "sources": "surface, most-unstable, mixed-layer",
                       "adiabats": "all four",
                       "inputs": "host memory (pinned client buffers, rows of 137 values), "
                                 "copied to the device inside the loop",
                       "admission": "device-memory budget 8 GiB (two 4 GiB arenas)",
                       "results": "cape, cin, mulvl, z_out back to host memory"},
            "learned": res["learned"], "plain": res["plain"],
            "p99_speedup": res["plain"]["p99_ms"] / res["learned"]["p99_ms"]}
    print(json.dumps(line), flush=True)
    return 0


ADIABAT_METRIC = ("CAPE/CIN columns/s at 4M×60 model levels per adiabat: learned-guess vs "
                  "plain CUDA; iterations saved by the network vs the plain first guess")
ADIABAT_COLUMNS = 1 << 22   # 4,194,304 columns
ADIABAT_BASE = 1 << 18      # distinct synthetic columns tiled to ADIABAT_COLUMNS
ADIABAT_LEVELS = 60
ADIABAT_NAMES = ("pseudo-liquid", "reversible-liquid", "pseudo-ice", "reversible-ice")


def run_adiabats(args):
    """--workload adiabats: surface-based calc_cape on 4M columns x 60 sigma
    levels for each adiabat, with the plain solver (the reference's
    iteration), the learned solver, and, for the network's own contribution,
    the secant solver from the plain first guess against the same solver from
    the network's guess on every saturated sub-step (equal stopping test)."""
    import torch
    from xcape_gb300 import _lib
    from xcape_gb300 import guess as G
    from xcape_gb300 import synthetic as S
    world, rank, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    G.ensure_loaded()
    L = _lib.lib()
    reps = ADIABAT_COLUMNS // ADIABAT_BASE
    base = S.sigma_c0(shape=(ADIABAT_BASE,), nlev=ADIABAT_LEVELS, seed=3, dtype=np.float32)
    d = [torch.from_numpy(np.ascontiguousarray(a)).to(dev).repeat((reps, 1) if a.ndim == 2
                                                                  else (reps,)) for a in base]
    n2 = ADIABAT_COLUMNS
    cape, cin, zout = (torch.empty(n2, dtype=torch.float32, device=dev) for _ in range(3))
    mulvl = torch.empty(n2, dtype=torch.int32, device=dev)
    ws_bytes = _lib.workspace_bytes(n2)
    wsbuf = torch.empty(ws_bytes + 256, dtype=torch.uint8, device=dev)
    ws = wsbuf.data_ptr() + (-wsbuf.data_ptr()) % 256
    stream = torch.cuda.current_stream(dev)
    cnt = torch.zeros(2, dtype=torch.int64, device=dev)

    def launch(adiabat, guess, counters=None):
        _lib.check(L.xc_loopcape_ex(1, *[x.data_ptr() for x in d], _lib.XC_F32, PINC, 1, ML_DEPTH,
                                    adiabat, None, ADIABAT_LEVELS, n2, guess, cape.data_ptr(),
                                    cin.data_ptr(), mulvl.data_ptr(), zout.data_ptr(), None,
                                    counters, ws, ws_bytes, stream.cuda_stream))

    def measure(adiabat, guess, steps):
        cnt.zero_()
        launch(adiabat, guess, cnt.data_ptr())
        torch.cuda.synchronize()
        work = [int(x) for x in cnt.cpu()]
        for _ in range(2):
            launch(adiabat, guess)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            launch(adiabat, guess)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps, work

    out = {}
    with ClockSampler(local) as clk:
        for code, name in enumerate(ADIABAT_NAMES, start=1):
            r = {}
            for g, gname, steps in ((_lib.XC_GUESS_PLAIN, "plain", args.steps),
                                    (_lib.XC_GUESS_LEARNED, "learned", args.steps),
                                    (_lib.XC_GUESS_SECANT, "secant", 2),
                                    (_lib.XC_GUESS_LEARNED_EVERY, "learned-every", 1)):
                ms, work = measure(code, g, steps)
                r[gname] = {"ms": ms, "substeps": work[0], "iterations": work[1]}
            r["learned_speedup_vs_plain"] = r["plain"]["ms"] / r["learned"]["ms"]
            r["network_iterations_saved_vs_plain_guess"] = \
                1.0 - r["learned-every"]["iterations"] / r["secant"]["iterations"]
            if not args.no_cpu_baseline:
                # the learned solver's CAPE on the first columns against FP64 (the checker)
                launch(code, _lib.XC_GUESS_LEARNED)
                torch.cuda.synchronize()
                r["accuracy_vs_fp64"] = _adiabat_accuracy(base, cape, code)
            out[name] = r
    line = {"metric": ADIABAT_METRIC, "impl": "ours", "n_gpus": 1, "workload": "adiabats",
            "unit": "columns/s", "dtype": "f32", "data": "synthetic",
            "config": {"columns": n2, "levels": ADIABAT_LEVELS, "grid": "sigma 0.995..0.1",
                       "source": "surface", "pinc": PINC, "distinct_columns": ADIABAT_BASE,
                       "steps": args.steps},
            "per_adiabat": out,
            "learned_value": {k: n2 / (v["learned"]["ms"] / 1e3) for k, v in out.items()},
            "plain_value": {k: n2 / (v["plain"]["ms"] / 1e3) for k, v in out.items()},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


def _adiabat_accuracy(base, cape, code, n=4096):
    import oracle as O
    p, t, td, ps, ts, tds = (np.asarray(a)[:n] for a in base)
    ref = O.loopcape(p, t, td, ps, ts, tds, PINC, 1, ML_DEPTH, code, precision="f64",
                     nthreads=os.cpu_count() or 1, stats=True)
    got = cape[:n].cpu().numpy().astype(np.float64)
    ok = (ref["status"] & 1) == 0
    dc = np.abs(got[ok] - ref["cape"][ok])
    return {"columns": n, "compared": int(ok.sum()), "max_abs_dcape": float(dc.max()),
            "frac_dcape_le_1": float(np.mean(dc <= 1.0))}


DASK_METRIC = "calc_cape columns/s on numpy chunks of the 1M x 37 grid (dask-style, threads)"


def run_dask(args):
    """calc_cape on the 721 x 1440 x 37 pressure-level grid split into 16
    chunks of columns, as dask's apply_gufunc hands them over (one numpy call
    per chunk, pageable host memory), computed one after another and by 4
    threads at once as dask's threaded scheduler does; beside one call over
    the whole grid.  Each concurrent call takes its own host context
    (streams, pinned staging, device workspace), so chunk k + 1's copies
    overlap chunk k's lift.  most-unstable parcels, learned guess."""
    import torch
    from concurrent.futures import ThreadPoolExecutor
    import xcape_gb300 as X
    from xcape_gb300 import guess as guess_net
    torch.cuda.set_device(0)
    guess_net.ensure_loaded()
    plev, t, td, ps, ts, tds = cape_inputs(0, GRID_SHAPE[0] * GRID_SHAPE[1])
    n2 = ps.shape[0]
    nch = 16
    bounds = np.linspace(0, n2, nch + 1).astype(int)
    chunks = [(plev, t[lo:hi], td[lo:hi], ps[lo:hi], ts[lo:hi], tds[lo:hi])
              for lo, hi in zip(bounds[:-1], bounds[1:])]
    kw = dict(source="most-unstable", vertical_lev="pressure", guess=args.guess)

    def one(c):
        return X.calc_cape(*c, **kw)

    def timed(fn):
        for _ in range(max(args.warmup, 2)):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / args.steps

    whole = timed(lambda: one((plev, t, td, ps, ts, tds)))
    seq = timed(lambda: [one(c) for c in chunks])
    with ThreadPoolExecutor(4) as pool:
        par = timed(lambda: list(pool.map(one, chunks)))
    line = {"metric": DASK_METRIC, "value": n2 / par, "unit": "columns/s", "n_gpus": 1,
            "steps": args.steps, "warmup": max(args.warmup, 2), "ms_per_step": par * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "calc_cape most-unstable, 721x1440 cols x 37 pressure levels, "
                                   f"{nch} numpy chunks of columns, guess {args.guess}"},
            "threads_4": {"columns_per_s": n2 / par, "ms": par * 1e3},
            "sequential_chunks": {"columns_per_s": n2 / seq, "ms": seq * 1e3},
            "one_call": {"columns_per_s": n2 / whole, "ms": whole * 1e3},
            "overlap_gain": seq / par}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "srh":
        return run_srh(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "adiabats":
        return run_adiabats(args)
    if args.workload == "cape_srh":
        return run_cape_srh(args)
    if args.workload == "dask":
        return run_dask(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
