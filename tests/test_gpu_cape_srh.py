"""GPU tests of calc_cape_srh: CAPE and SRH of the same columns in one kernel.

The fused kernel must return what the two separate calls (calc_cape,
calc_srh) return on the same inputs: bit for bit for SRH, whose routines
round every product on their own in any kernel that inlines them, and for
the plain CAPE solver; for the learned solver within the accelerated
solvers' tolerance, because the lift compiled into another kernel can stop
its iteration at another point inside the 2e-4 K test.  The SRH half is
also checked against the oracle.
"""
import numpy as np
import pytest

import oracle as O
import xcape_gb300 as X
from xcape_gb300 import synthetic as S

from gpu_util import to_dev, torch_cuda

pytestmark = pytest.mark.gpu

CASES = [("most-unstable", "pseudo-liquid"), ("mixed-layer", "reversible-ice"),
         ("surface", "pseudo-ice"), ("most-unstable", "reversible-liquid")]


def _inputs(grid):
    if grid == "model":
        return S.srh_c2(shape=(48, 64))
    return S.pressure_srh(shape=(40, 52))


def _same_cape(got, want, exact):
    assert len(got) == len(want)
    for k, (g, w) in enumerate(zip(got, want)):
        g, w = np.asarray(g), np.asarray(w)
        if exact or g.dtype.kind == "i":
            np.testing.assert_array_equal(g, w, err_msg=f"output {k}")
        else:
            np.testing.assert_allclose(g, w, rtol=2e-4, atol=0.5, err_msg=f"output {k}")


@pytest.mark.parametrize("precision", ["reference", "fp32"])
@pytest.mark.parametrize("guess", ["plain", "learned"])
@pytest.mark.parametrize("grid", ["model", "pressure"])
def test_fused_matches_the_two_separate_calls(grid, guess, precision):
    args = _inputs(grid)
    p, t, td, u, v, ps, ts, tds, us, vs = args
    srh_s = X.calc_srh(*args, depth=3000, vertical_lev=grid, output_var="all",
                       precision=precision)
    for source, adiabat in CASES:
        cape_f, srh_f = X.calc_cape_srh(*args, source=source, adiabat=adiabat, vertical_lev=grid,
                                        depth=3000, output_var="all", guess=guess,
                                        precision=precision)
        cape_s = X.calc_cape(p, t, td, ps, ts, tds, source=source, adiabat=adiabat,
                             vertical_lev=grid, guess=guess)
        assert len(srh_f) == 8
        for k, (g, w) in enumerate(zip(srh_f, srh_s)):
            np.testing.assert_array_equal(g, w, err_msg=f"srh output {k}, {source} {adiabat}")
        _same_cape(cape_f, cape_s, exact=guess == "plain")


@pytest.mark.parametrize("grid", ["model", "pressure"])
def test_fused_kernel_on_f64_inputs(grid):
    """f64 inputs: the learned solver with the FP32 SRH stages runs the fused
    kernel (f32 inputs run the two kernels back to back there)."""
    args = [np.asarray(a, np.float64) for a in _inputs(grid)]
    p, t, td, u, v, ps, ts, tds, us, vs = args
    for guess in ("learned", "plain"):
        cape_f, srh_f = X.calc_cape_srh(*args, source="most-unstable", vertical_lev=grid,
                                        output_var="all", guess=guess, precision="fp32")
        cape_s = X.calc_cape(p, t, td, ps, ts, tds, source="most-unstable", vertical_lev=grid,
                             guess=guess)
        srh_s = X.calc_srh(*args, vertical_lev=grid, output_var="all", precision="fp32")
        for g, w in zip(srh_f, srh_s):
            np.testing.assert_array_equal(g, w)
        _same_cape(cape_f, cape_s, exact=guess == "plain")


@pytest.mark.parametrize("guess", ["plain", "learned"])
def test_fused_partial_warps(guess):
    """1,517 columns (a partial last warp and block), pressure levels with
    ragged starts: the lanes past the last column take part in the guess
    network's evaluation and write nothing."""
    args = S.pressure_srh(shape=(37, 41), seed=8)
    p, t, td, u, v, ps, ts, tds, us, vs = args
    cape_f, srh_f = X.calc_cape_srh(*args, source="most-unstable", vertical_lev="pressure",
                                    output_var="all", guess=guess, precision="reference")
    cape_s = X.calc_cape(p, t, td, ps, ts, tds, source="most-unstable", vertical_lev="pressure",
                         guess=guess)
    srh_s = X.calc_srh(*args, vertical_lev="pressure", output_var="all", precision="reference")
    for g, w in zip(srh_f, srh_s):
        np.testing.assert_array_equal(g, w)
    _same_cape(cape_f, cape_s, exact=guess == "plain")


@pytest.mark.parametrize("grid", ["model", "pressure"])
def test_fused_srh_against_the_oracle(grid):
    """SRH at the reference precision against the oracle's calc_srh (the CAPE
    half equals calc_cape, whose parity with the oracle the CAPE tests pin)."""
    args = _inputs(grid)
    _, srh_f = X.calc_cape_srh(*args, source="most-unstable", vertical_lev=grid, depth=1000,
                               output_var="all")
    want = O.calc_srh(*args, depth=1000, vertical_lev=grid, output_var="all")
    np.testing.assert_allclose(srh_f[0], want[0], rtol=1e-9, atol=1e-6)
    np.testing.assert_allclose(srh_f[1], want[1], rtol=1e-9, atol=1e-6)
    for g, w in zip(srh_f[2:], want[2:]):
        np.testing.assert_allclose(g, w, rtol=0, atol=1e-4)


def test_fused_on_device_tensors_and_srh_only_outputs():
    """CUDA tensors in, CUDA tensors out on the caller's stream; the SRH
    tuple of output_var='srh' is the first two arrays of 'all'."""
    torch = torch_cuda()
    args = _inputs("pressure")
    dev = to_dev(*args)
    cape_d, srh_d = X.calc_cape_srh(*dev, source="mixed-layer", vertical_lev="pressure",
                                    guess="learned", precision="fp32")
    assert all(isinstance(x, torch.Tensor) and x.is_cuda for x in (*cape_d, *srh_d))
    assert len(cape_d) == 2 and len(srh_d) == 2
    cape_h, srh_h = X.calc_cape_srh(*args, source="mixed-layer", vertical_lev="pressure",
                                    guess="learned", precision="fp32", output_var="all")
    for g, w in zip(srh_d, srh_h[:2]):
        np.testing.assert_array_equal(g.cpu().numpy(), w)
    for g, w in zip(cape_d, cape_h):
        np.testing.assert_array_equal(g.cpu().numpy(), w)
