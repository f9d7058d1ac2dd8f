"""GPU tests of the learned first guess (xcape_gb300.guess).

* the training kernel's gradient against a numpy FP64 reference that rounds
  the hidden layer's operands to BF16 as the tensor cores see them;
* the batched (tensor-core) inference against the same reference;
* the GPU's training pairs against the host build of the same code;
* a short training run that cuts the error of the untrained network;
* what the trained network gains over the method without it, on the ragged
  pressure-level workload, counting iterations on the device and checking
  CAPE against the FP64 oracle: with the same secant solver and the
  reference's stopping test, the network's guess on every saturated
  sub-step against the plain first guess (th1); and the learned mode
  against the extrapolated mode it extends.
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


@pytest.fixture(scope="module")
def many_pairs():
    torch_cuda()
    f, t, it = G.make_pairs(65536, seed=321)
    return f.cpu().numpy(), t.cpu().numpy(), it.cpu().numpy()


def test_pairs_over_the_state_box(pairs):
    """The GPU's pairs (four adiabats, p 100..1050 hPa, T -80..40 degC):
    the plain iteration solves every atmospheric one (theta-e below 380 K)
    and gives up only in hot, moist corners of the box, which training
    leaves out."""
    f, y, it = pairs
    assert np.all(np.isfinite(f))
    the = 320.0 + 40.0 * f[:, 1]
    assert np.all(it[the < 380.0] >= 1)
    assert np.mean(it >= 1) > 0.8 and np.mean(np.abs(it)) > 2
    ok = (it >= 1) & (the < 380.0)
    assert np.all(np.isfinite(y[ok])) and y[ok].min() > -0.05 and y[ok].max() < 2.0


def test_pairs_match_host_build(pairs):
    emul = pytest.importorskip("emul")
    if emul.nvcc() is None:
        pytest.skip("nvcc not available")
    f, y, it = pairs
    n = len(y)
    fh, yh, ith = (np.zeros((n, 3), np.float32), np.zeros(n, np.float32), np.zeros(n, np.int32))
    emul.lib().emu_guess_pairs(n, 123, fh.ctypes.data, yh.ctypes.data, ith.ctypes.data, None)
    # same draws; CUDA's and glibc's expf/powf/logf differ by an ulp or two,
    # and the iteration stops anywhere within its 2e-4 K tolerance
    np.testing.assert_allclose(f, fh, rtol=1e-5, atol=1e-5)
    both = (it >= 1) & (ith >= 1)  # where the iteration gave up, y is wherever it stopped
    assert np.mean(both) > 0.8
    np.testing.assert_allclose(y[both], yh[both], rtol=0, atol=5e-3)
    # an ulp can move the stop of the damped iteration by a step either way
    assert np.mean(it[both] == ith[both]) > 0.8
    assert np.mean(np.abs(it[both] - ith[both]) <= 1) > 0.98


@pytest.mark.parametrize("kernel", G.KERNELS)
@pytest.mark.parametrize("n", [300, 50_000])
def test_training_gradient_matches_fp64_reference(many_pairs, kernel, n):
    """300 pairs: two full tiles of 128 and a partial one; 50,000: 391
    tiles over one block per SM, so each block of the tcgen05 kernel adds
    two or three tiles' dW2 in its tensor memory before writing it out."""
    f, t, _ = many_pairs
    assert len(t) >= n
    w = G.init_weights(11, float(t[:n].mean()))
    g_gpu, loss_gpu = G.gradient(w, f[:n], t[:n], kernel=kernel)
    loss_ref, g_ref = loss_and_grad(w, f[:n], t[:n])
    assert abs(loss_gpu - loss_ref) <= 1e-4 * loss_ref + 1e-7
    scale = np.max(np.abs(g_ref))
    np.testing.assert_allclose(g_gpu, g_ref, rtol=2e-3, atol=2e-4 * scale)
    # and the direction is right: a small step along -grad lowers the loss
    w2 = w - 1e-3 * g_gpu / np.linalg.norm(g_gpu)
    assert loss_and_grad(w2, f[:n], t[:n])[0] < loss_ref


def test_training_kernels_agree(many_pairs):
    """The tcgen05 and mma.sync gradients of the same batch: the same BF16
    operands with FP32 accumulation, summed in other orders."""
    f, t, _ = many_pairs
    w = G.init_weights(5, float(t[:20000].mean()))
    g_tc, l_tc = G.gradient(w, f[:20000], t[:20000], kernel="tcgen05")
    g_mma, l_mma = G.gradient(w, f[:20000], t[:20000], kernel="mma")
    assert abs(l_tc - l_mma) <= 1e-5 * l_mma
    np.testing.assert_allclose(g_tc, g_mma, rtol=1e-3, atol=1e-5 * np.max(np.abs(g_mma)))


def test_tensor_core_inference_matches_reference(pairs):
    f, _, _ = pairs
    w = G.bf16_round(G.init_weights(4, 0.3))
    got = G.evaluate(w, f).cpu().numpy()
    want = forward(w, f)[0]
    # FP32 accumulation of the BF16 products can move a pre-activation across
    # zero where the FP64 sum does not; that bounds the few worst elements
    np.testing.assert_allclose(got, want, rtol=1e-3, atol=1e-3)
    assert np.mean(np.abs(got - want) < 1e-4) > 0.99


def test_short_training_reduces_error():
    w, meta = G.train(n_pairs=1 << 17, epochs=4, batch=4096, log=None)
    assert meta["train_rms_y"][-1] < 0.5 * meta["train_rms_y"][0]
    assert meta["val_rel_rms_bf16"] < 0.3


_trained = []


def _network():
    """The stored network, or one trained here when none is stored."""
    if os.path.exists(G.DEFAULT_PATH):
        return G.read()[0]
    if not _trained:
        _trained.append(G.train(n_pairs=1 << 20, epochs=8, log=None)[0])
    return _trained[0]


def _run(guess, shape=(96, 128)):
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=shape)
    got = cape_device(2, plev, t, td, ps, ts, tds, "surface", "pseudo-liquid", guess=guess,
                      counters=True)
    n2 = ps.size
    ref = O.loopcape(plev, t.reshape(n2, -1), td.reshape(n2, -1), ps.ravel(), ts.ravel(),
                     tds.ravel(), 500.0, 1, 500.0, 1, start=O.pres_lev_pos(plev, ps.ravel()),
                     p_is_1d=True, precision="f64", stats=True)
    conv = (ref["status"] & 1) == 0
    assert not np.any((got["status"] & 1).astype(bool) & conv)
    d = np.abs(got["cape"][conv].astype(np.float64) - ref["cape"][conv])
    assert np.all(d <= np.maximum(1.0, 1e-3 * ref["cape"][conv])), d.max()
    return got


def test_network_guess_saves_iterations_over_plain_first_guess():
    G.set_weights(_network())
    base = _run(_lib.XC_GUESS_SECANT)
    lrn = _run(_lib.XC_GUESS_LEARNED_EVERY)
    assert lrn["nsub_total"] == base["nsub_total"]
    # a few percent of relative error on the increment against th1's 100 %
    assert lrn["niter_total"] < 0.9 * base["niter_total"], (lrn["niter_total"], base["niter_total"])


def test_learned_mode_against_extrapolated_mode():
    G.set_weights(_network())
    ext = _run(_lib.XC_GUESS_EXTRAPOLATED)
    lrn = _run(_lib.XC_GUESS_LEARNED)
    assert lrn["nsub_total"] == ext["nsub_total"]
    # the network replaces the extrapolation only on the first saturated
    # sub-step of a column, where the increment of the sub-step that crossed
    # saturation is a poor predictor
    assert lrn["niter_total"] < ext["niter_total"], (lrn["niter_total"], ext["niter_total"])


@pytest.mark.parametrize("bad", ["nan", "large"])
def test_learned_mode_without_a_usable_network_falls_back_to_extrapolation(bad):
    """NaN weights, or an output bias of 1000 (far outside the output range):
    the tensor-core evaluation's output is rejected for every column and the
    learned kernel runs the extrapolated solver's ascent -- same levels,
    sources and work within the solver tolerance (the two are compiled into
    different kernels)."""
    w = np.array(G.read()[0] if os.path.exists(G.DEFAULT_PATH) else _network(), np.float32)
    if bad == "nan":
        w[:] = np.nan
    else:
        w[G.OFF_B3] = 1000.0
    try:
        G.set_weights(w)
        lrn = _run(_lib.XC_GUESS_LEARNED)
        ext = _run(_lib.XC_GUESS_EXTRAPOLATED)
    finally:
        G.set_weights(_network())
    for k in ("mulvl", "status"):
        np.testing.assert_array_equal(lrn[k], ext[k], err_msg=k)
    for k in ("cape", "cin", "z_out"):
        np.testing.assert_allclose(lrn[k], ext[k], rtol=2e-4, atol=0.5, err_msg=k)
    assert lrn["nsub_total"] == ext["nsub_total"]
    assert abs(lrn["niter_total"] - ext["niter_total"]) <= 1e-3 * ext["niter_total"]


@pytest.mark.parametrize("adiabat", ["pseudo-liquid", "reversible-liquid", "pseudo-ice",
                                     "reversible-ice"])
def test_network_saves_iterations_on_every_adiabat(adiabat):
    """Sigma levels (60), surface parcels, every adiabat: the network's guess
    (trained on pseudo-liquid sub-steps) on every saturated sub-step needs
    fewer iterations than the plain first guess with the same secant steps,
    and the learned solver stays within the CAPE tolerance of FP64."""
    G.set_weights(_network())
    p, t, td, ps, ts, tds = S.sigma_c0(shape=(48, 64), nlev=60, seed=9, dtype=np.float32)
    runs = {g: cape_device(1, p, t, td, ps, ts, tds, "surface", adiabat, guess=g, counters=True)
            for g in (_lib.XC_GUESS_SECANT, _lib.XC_GUESS_LEARNED_EVERY, _lib.XC_GUESS_LEARNED)}
    n2 = ps.size
    code = {"pseudo-liquid": 1, "reversible-liquid": 2, "pseudo-ice": 3, "reversible-ice": 4}
    ref = O.loopcape(p.reshape(n2, -1), t.reshape(n2, -1), td.reshape(n2, -1), ps.ravel(),
                     ts.ravel(), tds.ravel(), 500.0, 1, 500.0, code[adiabat], precision="f64",
                     stats=True)
    conv = (ref["status"] & 1) == 0
    for got in runs.values():
        assert not np.any((got["status"] & 1).astype(bool) & conv)
        d = np.abs(got["cape"][conv].astype(np.float64) - ref["cape"][conv])
        assert np.all(d <= np.maximum(1.0, 1e-3 * ref["cape"][conv])), d.max()
    sec = runs[_lib.XC_GUESS_SECANT]["niter_total"]
    every = runs[_lib.XC_GUESS_LEARNED_EVERY]["niter_total"]
    assert every < 0.95 * sec, (adiabat, every, sec)


def test_lockstep_network_solver_meets_the_fp64_contract():
    """XC_GUESS_LEARNED_WARP: the warp evaluates the network for its 32
    columns at every sub-step, in lockstep, on the tensor cores; the first
    guess of each saturated sub-step is the network's.  Same sub-steps as
    the extrapolated solver, CAPE within the FP64 contract (checked in
    _run).  Its guesses take no fewer evaluations than the extrapolation's:
    a first Newton step below 0.01 K ends a sub-step (newton_accept), which
    the extrapolated guess reaches on more sub-steps than the network's
    (1.08 against 1.26 evaluations per sub-step on the bench workload); at
    most 30 % more evaluations here."""
    G.set_weights(_network())
    ext = _run(_lib.XC_GUESS_EXTRAPOLATED)
    warp = _run(_lib.XC_GUESS_LEARNED_WARP)
    assert warp["nsub_total"] == ext["nsub_total"]
    assert warp["niter_total"] < 1.3 * ext["niter_total"], (warp["niter_total"],
                                                           ext["niter_total"])
