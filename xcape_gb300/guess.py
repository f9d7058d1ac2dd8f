"""The learned first guess of the moist-adiabat iteration.

A 3 -> 64 -> 64 -> 1 ReLU network (``xcape_gb300/csrc/guess_mlp.cuh``) maps a
saturated parcel's (target pressure, theta-e, total water) to the increment
of its potential temperature over a sub-step, per unit log-pressure:
theta2 = theta1 + 50 K * y * ln(p1 / p2).  ``calc_cape(..., guess='learned')``
starts the first saturated sub-step's iteration there (the later ones
extrapolate the previous sub-step's increment); ``guess='learned-every'``
starts every saturated sub-step there.  Both take secant steps; the stopping
test and the result are the reference's.

Everything runs on the GPU through the library:
  * ``xc_guess_pairs``  -- training pairs, solved by the plain (reference)
    iteration;
  * ``xc_guess_grad_tc`` -- forward and backward pass of the squared error
    with the three 64-wide products on the 5th-generation tensor cores
    (tcgen05.mma, BF16 operands, FP32 accumulators in tensor memory);
    ``xc_guess_grad`` the same with mma.sync;
  * ``xc_guess_adam``   -- Adam on FP32 master weights;
  * ``xc_guess_eval``   -- batched inference.
The trained weights are stored rounded to BF16 in
``xcape_gb300/data/guess_mlp.npz`` with their training metadata, and
``ensure_loaded()`` hands them to the library (``xc_guess_set_weights``).

    python -m xcape_gb300.guess train [--pairs N] [--epochs E] [--out PATH]
"""
import argparse
import json
import os
import time

import numpy as np

from . import _lib

NPARAM = _lib.XC_GUESS_NPARAM
H = 64
OFF_W1, OFF_B1, OFF_W2, OFF_B2, OFF_W3, OFF_B3 = 0, 192, 256, 4352, 4416, 4480
SLOPE_SCALE = 50.0  # K per unit ln p of the output
FORMAT_VERSION = 2  # the increment target; version 1 predicted the temperature
DEFAULT_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "guess_mlp.npz")

_loaded = set()


def bf16_round(w):
    """Round float32 values to the nearest BF16 value (ties to even)."""
    u = np.ascontiguousarray(w, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def init_weights(seed=0, target_mean=0.0):
    rng = np.random.default_rng(seed)
    w = np.zeros(NPARAM, np.float32)
    w[OFF_W1:OFF_B1] = rng.normal(0, np.sqrt(2.0 / 3), 3 * H)
    w[OFF_B1:OFF_W2] = 0.1
    w[OFF_W2:OFF_B2] = rng.normal(0, np.sqrt(2.0 / H), H * H)
    w[OFF_B2:OFF_W3] = 0.1
    w[OFF_W3:OFF_B3] = rng.normal(0, np.sqrt(1.0 / H), H)
    w[OFF_B3] = target_mean
    return w


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("the guess network is trained and evaluated on the GPU")
    return torch


def make_pairs(n, seed=1):
    """n training pairs as CUDA tensors (feats [n,3], targets [n], iters [n]).

    iters is the plain iteration's count, negative where it gave up."""
    torch = _torch()
    f = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    t = torch.empty(n, dtype=torch.float32, device="cuda")
    it = torch.empty(n, dtype=torch.int32, device="cuda")
    _lib.call("xc_guess_pairs", n, seed, f.data_ptr(), t.data_ptr(), it.data_ptr(),
              torch.cuda.current_stream().cuda_stream)
    return f, t, it


# training kernels: the products on tcgen05 (5th-generation tensor cores,
# accumulators in tensor memory) or on mma.sync
KERNELS = ("tcgen05", "mma")


def _grad_call(kernel, w, f, t, n, g, loss, status, stream):
    if kernel == "tcgen05":
        _lib.call("xc_guess_grad_tc", w, f, t, n, g, loss, status, stream)
    elif kernel == "mma":
        _lib.call("xc_guess_grad", w, f, t, n, g, loss, stream)
    else:
        raise ValueError(f"kernel must be one of {KERNELS}")


def gradient(weights, feats, targets, kernel="tcgen05"):
    """(grad [NPARAM], loss) of the mean squared error, on the GPU."""
    torch = _torch()
    w = torch.as_tensor(np.asarray(weights, np.float32)).cuda()
    f = torch.as_tensor(np.asarray(feats, np.float32)).cuda().contiguous()
    t = torch.as_tensor(np.asarray(targets, np.float32)).cuda().contiguous()
    g = torch.zeros(NPARAM, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    _grad_call(kernel, w.data_ptr(), f.data_ptr(), t.data_ptr(), t.numel(), g.data_ptr(),
               loss.data_ptr(), status.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    if int(status.item()):
        raise RuntimeError("the tensor-core training kernel gave up waiting for its products")
    return g.cpu().numpy(), float(loss.item())


def evaluate(weights, feats):
    """Network outputs for feats [n, 3] (normalised increments y)."""
    torch = _torch()
    w = torch.as_tensor(np.asarray(weights, np.float32)).cuda()
    f = torch.as_tensor(feats).cuda().contiguous() if not hasattr(feats, "data_ptr") else feats
    out = torch.empty(f.shape[0], dtype=torch.float32, device="cuda")
    _lib.call("xc_guess_eval", w.data_ptr(), f.data_ptr(), f.shape[0], out.data_ptr(),
              torch.cuda.current_stream().cuda_stream)
    return out


# outputs outside this range are not used by the solvers (guess_mlp.cuh)
Y_MIN, Y_MAX = -0.2, 2.0


def train(n_pairs=10_000_000, epochs=12, batch=16384, lr=2e-3, seed=7, log=print,
          kernel="tcgen05"):
    """Trains the network on the GPU; returns (weights rounded to BF16, meta).
    ``kernel`` is the gradient kernel, one of KERNELS.

    The pairs cover the four adiabats over p 100..1050 hPa and T -80..40 degC
    (xc_guess_pairs); those the plain iteration could not solve, and those
    whose increment lies outside the range the solvers accept from the
    network, are left out."""
    torch = _torch()
    t0 = time.time()
    feats, targets, iters = make_pairs(n_pairs, seed)
    keep = (iters > 0) & (targets >= Y_MIN) & (targets <= Y_MAX)
    kept = int(keep.sum().item())
    feats, targets = feats[keep].contiguous(), targets[keep].contiguous()
    n_val = kept // 32
    n_tr = kept - n_val
    fv, tv = feats[n_tr:], targets[n_tr:]
    w = torch.as_tensor(init_weights(seed, float(targets[:n_tr].mean().item()))).cuda()
    m = torch.zeros_like(w)
    v = torch.zeros_like(w)
    grad = torch.zeros_like(w)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    step = 0
    curve = []
    n_batches = n_tr // batch
    for ep in range(epochs):
        perm = torch.randperm(n_tr, device="cuda", generator=gen)
        fe, te = feats[perm].contiguous(), targets[perm].contiguous()
        lr_ep = lr * (0.5 * (1 + np.cos(np.pi * ep / epochs)))
        loss.zero_()
        for b in range(n_batches):
            step += 1
            _grad_call(kernel, w.data_ptr(), fe[b * batch:].data_ptr(), te[b * batch:].data_ptr(),
                       batch, grad.data_ptr(), loss.data_ptr(), status.data_ptr(), stream)
            _lib.call("xc_guess_adam", w.data_ptr(), grad.data_ptr(), m.data_ptr(), v.data_ptr(),
                      float(lr_ep), step, stream)
        if int(status.item()):
            raise RuntimeError("the tensor-core training kernel gave up waiting for its products")
        rms = float(np.sqrt(loss.item() / n_batches))
        curve.append(rms)
        if log:
            log(f"epoch {ep + 1}/{epochs}: train RMS error of y {rms:.5f}")
    w_bf = bf16_round(w.cpu().numpy())
    pred = evaluate(w_bf, fv)
    val_rms = float(torch.sqrt(torch.mean((pred - tv) ** 2)).item())
    val_rel = float((torch.sqrt(torch.mean((pred - tv) ** 2)) /
                     torch.sqrt(torch.mean(tv ** 2))).item())
    it = iters.cpu().numpy()
    meta = {"version": FORMAT_VERSION, "target": "y = (theta2 - theta1) / (50 K ln(p1/p2))",
            "pairs": n_pairs, "pairs_kept": kept,
            "pair_box": "four adiabats, p 100..1050 hPa, T -80..40 degC (saturation mixing "
                        "ratio <= 40 g/kg), reversible condensate 0..10 g/kg, dp 50..2000 Pa",
            "epochs": epochs, "batch": batch, "lr": lr, "seed": seed, "kernel": kernel,
            "train_rms_y": curve, "val_rms_y_bf16": val_rms, "val_rel_rms_bf16": val_rel,
            "plain_iterations_mean": float(np.abs(it).mean()),
            "plain_gave_up": int((it < 0).sum()), "seconds": time.time() - t0}
    if log:
        log(f"validation RMS error of y with BF16 weights: {val_rms:.5f} "
            f"({100 * val_rel:.2f}% of the RMS target)")
    return w_bf, meta


def save(path, weights, meta):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez_compressed(path, weights=np.asarray(weights, np.float32),
                        meta=np.frombuffer(json.dumps(meta).encode(), np.uint8))


def read(path=DEFAULT_PATH):
    with np.load(path) as z:
        w, meta = z["weights"], json.loads(bytes(z["meta"]).decode())
    if meta.get("version") != FORMAT_VERSION:
        raise ValueError(f"{path} holds a guess network of format {meta.get('version')}, "
                         f"expected {FORMAT_VERSION}; retrain it")
    return w, meta


def set_weights(weights):
    """Makes `weights` the network XC_GUESS_LEARNED uses on the current device."""
    w = np.ascontiguousarray(weights, np.float32)
    if w.size != NPARAM:
        raise ValueError(f"expected {NPARAM} parameters, got {w.size}")
    _lib.call("xc_guess_set_weights", w.ctypes.data, 0, None)
    try:
        import torch
        _loaded.add(torch.cuda.current_device())
    except Exception:
        pass


def ensure_loaded(path=DEFAULT_PATH):
    """Loads the stored network on the current device once."""
    try:
        import torch
        dev = torch.cuda.current_device() if torch.cuda.is_available() else None
    except ImportError:
        dev = None
    if dev is not None and dev in _loaded:
        return
    if not os.path.exists(path):
        raise FileNotFoundError(f"guess='learned' needs the trained network ({path}); "
                                "train it with `python -m xcape_gb300.guess train`")
    set_weights(read(path)[0])


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m xcape_gb300.guess")
    sub = ap.add_subparsers(dest="cmd", required=True)
    tr = sub.add_parser("train")
    tr.add_argument("--pairs", type=int, default=10_000_000)
    tr.add_argument("--epochs", type=int, default=12)
    tr.add_argument("--out", default=DEFAULT_PATH)
    tr.add_argument("--kernel", choices=KERNELS, default="tcgen05")
    args = ap.parse_args(argv)
    w, meta = train(n_pairs=args.pairs, epochs=args.epochs, kernel=args.kernel)
    save(args.out, w, meta)
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
