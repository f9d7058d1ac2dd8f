"""GPU tests of the learned first guess (xcape_gb300.guess).

* the training kernel's gradient against a numpy FP64 reference that rounds
  the hidden layer's operands to BF16 as the tensor cores see them;
* the batched (tensor-core) inference against the same reference;
* a short training run that cuts the error of the untrained network;
* what the trained network gains over the method without it: with the same
  secant solver and the reference's stopping test, the network's first guess
  against the plain first guess (th1), on the ragged pressure-level workload,
  counting iterations on the device and checking CAPE against the FP64
  oracle.
"""
import os

import numpy as np
import pytest

import oracle as O
from xcape_gb300 import _lib
from xcape_gb300 import guess as G
from xcape_gb300 import synthetic as S

from gpu_util import cape_device, torch_cuda
from guess_ref import forward, loss_and_grad

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pairs():
    torch_cuda()
    f, t, it = G.make_pairs(4096, seed=123)
    return f.cpu().numpy(), t.cpu().numpy(), it.cpu().numpy()


def test_pairs_are_solved_by_the_plain_iteration(pairs):
    f, t, it = pairs
    assert np.all(np.isfinite(f)) and np.all(np.isfinite(t))
    assert np.mean(np.abs(it)) > 2 and np.all(np.abs(it) >= 1)
    temps = G.T_MID + G.T_SCALE * t
    assert temps.min() > 150 and temps.max() < 330


def test_training_gradient_matches_fp64_reference(pairs):
    f, t, _ = pairs
    n = 300  # two full blocks and a partial one
    w = G.init_weights(11, float(t[:n].mean()))
    g_gpu, loss_gpu = G.gradient(w, f[:n], t[:n])
    loss_ref, g_ref = loss_and_grad(w, f[:n], t[:n])
    assert abs(loss_gpu - loss_ref) <= 1e-4 * loss_ref + 1e-7
    scale = np.max(np.abs(g_ref))
    np.testing.assert_allclose(g_gpu, g_ref, rtol=2e-3, atol=2e-4 * scale)
    # and the direction is right: a small step along -grad lowers the loss
    w2 = w - 1e-3 * g_gpu / np.linalg.norm(g_gpu)
    assert loss_and_grad(w2, f[:n], t[:n])[0] < loss_ref


def test_tensor_core_inference_matches_reference(pairs):
    f, _, _ = pairs
    w = G.bf16_round(G.init_weights(4, 0.3))
    got = G.evaluate(w, f).cpu().numpy()
    want = forward(w, f)[0]
    np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-4)


def test_short_training_reduces_error():
    w, meta = G.train(n_pairs=1 << 16, epochs=3, batch=4096, log=None)
    assert meta["train_rms_K"][-1] < 0.5 * meta["train_rms_K"][0]
    assert meta["val_rms_K_bf16"] < 3.0


def _network():
    if os.path.exists(G.DEFAULT_PATH):
        return G.read()[0]
    return G.train(n_pairs=1 << 19, epochs=6, log=None)[0]


def test_learned_guess_saves_iterations_over_plain_first_guess():
    w = _network()
    G.set_weights(w)
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(96, 128))
    base = cape_device(2, plev, t, td, ps, ts, tds, "surface", "pseudo-liquid",
                       guess=_lib.XC_GUESS_SECANT, counters=True)
    lrn = cape_device(2, plev, t, td, ps, ts, tds, "surface", "pseudo-liquid",
                      guess=_lib.XC_GUESS_LEARNED, counters=True)
    n2 = ps.size
    ref = O.loopcape(plev, t.reshape(n2, -1), td.reshape(n2, -1), ps.ravel(), ts.ravel(),
                     tds.ravel(), 500.0, 1, 500.0, 1, start=O.pres_lev_pos(plev, ps.ravel()),
                     p_is_1d=True, precision="f64", stats=True)
    conv = (ref["status"] & 1) == 0
    for got in (base, lrn):
        assert not np.any((got["status"] & 1).astype(bool) & conv)
        d = np.abs(got["cape"][conv].astype(np.float64) - ref["cape"][conv])
        assert np.all(d <= np.maximum(1.0, 1e-3 * ref["cape"][conv])), d.max()
    assert lrn["nsub_total"] == base["nsub_total"]
    assert lrn["niter_total"] < base["niter_total"], (lrn["niter_total"], base["niter_total"])
