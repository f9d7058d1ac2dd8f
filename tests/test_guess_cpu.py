"""CPU checks of the learned-guess machinery: BF16 rounding, the network's
per-thread evaluation (the code the CAPE kernel runs, built for the host),
and the learned / secant solver modes of the column routine against the FP64
oracle.  A first guess only changes where the iteration starts: whatever the
network says, the stopping test is the reference's, so the results must stay
as close to FP64 as the plain FP32 iteration -- checked here with an
untrained (random) network, the worst case."""
import numpy as np
import pytest

import oracle as O
from xcape_gb300 import guess as G
from xcape_gb300 import synthetic as S

from guess_ref import forward

G_P_MID, G_P_SCALE = 55000.0, 45000.0  # guess_mlp.cuh feature scaling

emul = pytest.importorskip("emul")
if emul.nvcc() is None:
    pytest.skip("nvcc not available", allow_module_level=True)


def test_bf16_round_matches_torch():
    torch = pytest.importorskip("torch")
    x = np.random.default_rng(0).normal(0, 3, 10000).astype(np.float32)
    x[:4] = [0.0, -0.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9]  # exact ties round to even
    want = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    np.testing.assert_array_equal(G.bf16_round(x), want)


def test_host_guess_eval_matches_numpy():
    L = emul.lib()
    w = G.bf16_round(G.init_weights(3, 0.5))
    x = np.random.default_rng(1).uniform(-1, 1, (64, 3)).astype(np.float32)
    want = forward(w, x, bf16_hidden=False)[0]
    got = np.array([L.emu_guess_eval(w.ctypes.data, *map(float, r)) for r in x])
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-5)
    # the packed copy the CAPE kernel reads gives the same sums in the same order
    packed = np.array([L.emu_guess_eval_packed(w.ctypes.data, *map(float, r)) for r in x])
    np.testing.assert_array_equal(packed, got)


def emulated_pairs(n, seed, with_adiabat=False):
    L = emul.lib()
    f = np.zeros((n, 3), np.float32)
    y = np.zeros(n, np.float32)
    it = np.zeros(n, np.int32)
    adi = np.zeros(n, np.int32)
    L.emu_guess_pairs(n, seed, f.ctypes.data, y.ctypes.data, it.ctypes.data, adi.ctypes.data)
    return (f, y, it, adi) if with_adiabat else (f, y, it)


def test_training_pairs_cover_the_state_box():
    """Pairs over the four adiabats, p 100..1050 hPa and T -80..40 degC
    (saturation mixing ratio capped at 40 g/kg; the reversible adiabats
    carry up to 10 g/kg of condensate).  Within atmospheric states
    (theta-e below 380 K) the plain iteration solves every pair, and below
    400 K all but a few hot, moist ones near the ground, where FP32 rounding
    locks it into a cycle (as in real columns); it gives up mostly in the
    hot, moist corners of the box at low pressure.  Training leaves the
    unsolved pairs out."""
    f, y, it, adi = emulated_pairs(40000, 3, with_adiabat=True)
    p2 = G_P_MID + G_P_SCALE * f[:, 0]
    assert p2.min() > 9000 and p2.max() < 105000
    qt = (f[:, 2] + 0.5) / 50.0
    assert np.all(qt <= 0.05 + 1e-6)
    assert sorted(set(adi.tolist())) == [1, 2, 3, 4]
    for a in (1, 2, 3, 4):
        assert abs(np.mean(adi == a) - 0.25) < 0.02
    the = 320.0 + 40.0 * f[:, 1]
    assert np.all(it[the < 380.0] > 0), "the plain iteration solves every atmospheric pair"
    atm = the < 400.0
    assert np.mean(it[atm] > 0) > 0.999
    assert np.mean(it > 0) > 0.8
    # the moist-adiabat increment of solved atmospheric pairs: non-negative,
    # largest for warm moist parcels
    ok = atm & (it > 0)
    assert y[ok].min() > -0.05 and y[ok].max() < 2.0
    warm = ok & (qt > 0.01)
    assert y[warm].mean() > 2 * y[ok & (qt <= 0.01)].mean()


def test_pairs_are_deterministic():
    a = emulated_pairs(512, 9)
    b = emulated_pairs(512, 9)
    for x, z in zip(a, b):
        np.testing.assert_array_equal(x, z)


@pytest.mark.parametrize("guess", [1, 3, 4])
def test_emulated_learned_and_secant_modes_vs_fp64(guess):
    from test_kernel_emulation import _emu_cape, _oracle
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(16, 48))
    w = G.bf16_round(G.init_weights(5, 0.3))
    got = _emu_cape(2, plev, t, td, ps, ts, tds, 1, 1, guess=guess, guess_w=w)
    ref = _oracle(2, plev, t, td, ps, ts, tds, 1, 1, precision="f64")
    conv = (ref["status"] & 1) == 0
    assert not np.any((got["status"] & 1) & conv)
    d = np.abs(got["cape"][conv].astype(np.float64) - ref["cape"][conv])
    assert np.all(d <= np.maximum(1.0, 1e-3 * ref["cape"][conv])), d.max()


@pytest.mark.parametrize("bad", ["nan", "large"])
def test_emulated_learned_mode_without_a_usable_network_is_the_extrapolated_mode(bad):
    """A network whose output is not finite or outside its range (here: NaN
    weights, or an output bias of 1000) leaves the learned solver with the
    extrapolated guess everywhere: the host build gives the extrapolated
    solver's results and work counts exactly."""
    from test_kernel_emulation import _emu_cape
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(16, 48))
    w = G.bf16_round(G.init_weights(5, 0.3))
    if bad == "nan":
        w[:] = np.nan
    else:
        w[G.OFF_B3] = 1000.0
    for source in (1, 2, 3):
        lrn = _emu_cape(2, plev, t, td, ps, ts, tds, source, 1, guess=1, guess_w=w)
        ext = _emu_cape(2, plev, t, td, ps, ts, tds, source, 1, guess=2)
        for k in ("cape", "cin", "mulvl", "z_out", "status", "counters"):
            np.testing.assert_array_equal(lrn[k], ext[k], err_msg=f"{k}, source {source}")

