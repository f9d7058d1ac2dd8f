"""Pin the CPU oracle to the reference's own golden vectors.

Mirrors the reference's parity tests (test/test_core.py:68-116 sigma CAPE,
:120-170 pressure CAPE, :173-229 sigma SRH, :231-286 pressure SRH) with the
oracle in place of the Fortran.  The reference's tolerances are
``assert_almost_equal(decimal=0)`` for CAPE/CIN/MU level/MU height and
``decimal=5`` for SRH; the FP32 oracle is in fact much closer (bit-exact on
the soundings), which is also asserted so that a drift in the restatement
cannot hide under the loose bar.
"""
import numpy as np
import pytest

import oracle as O

SIGMA_CASES = [
    ("surface", 100, ("SB_CAPE_pinc100", "SB_CIN_pinc100")),
    ("mixed-layer", 1000, ("ML_CAPE_pinc1000_mldepth500", "ML_CIN_pinc1000_mldepth500")),
    ("most-unstable", 100, ("MU_CAPE_pinc100", "MU_CIN_pinc100", "MU_lv_pinc100", "MU_z_pinc100")),
]

PRESSURE_CASES = [
    ("surface", ("sfc_capesp500", "sfc_cinsp500")),
    ("mixed-layer", ("sfc_capeml300p500", "sfc_cinml300p500")),
    ("most-unstable", ("sfc_capemup500", "sfc_cinmup500")),
]


def _sigma_args(s):
    P, T, TD = s["pressure"], s["temperature"], s["dewpoint"]
    return (P[:, 1:], T[:, 1:], TD[:, 1:], P[:, 0], T[:, 0], TD[:, 0])


@pytest.mark.parametrize("source,pinc,keys", SIGMA_CASES)
def test_oracle_cape_sigma_golden(soundings, source, pinc, keys):
    res = O.calc_cape(*_sigma_args(soundings), source=source, ml_depth=500.0,
                      adiabat="pseudo-liquid", pinc=pinc, vertical_lev="sigma")
    assert len(res) == len(keys)
    for got, key in zip(res, keys):
        want = soundings[key]
        if key.startswith("MU_lv"):
            np.testing.assert_array_equal(got, want.astype(np.int32))
        else:
            np.testing.assert_almost_equal(got, want, 0)
            np.testing.assert_allclose(got, want, rtol=0, atol=1e-2)


@pytest.mark.parametrize("source,keys", PRESSURE_CASES)
def test_oracle_cape_pressure_golden(era5, source, keys):
    e = era5
    res = O.calc_cape(e["lev_level"], e["lev_t"], e["lev_td"], e["sfc_p"], e["sfc_t"], e["sfc_td"],
                      source=source, ml_depth=300, adiabat="pseudo-liquid", pinc=500,
                      vertical_lev="pressure")
    for got, key in zip(res, keys):
        np.testing.assert_almost_equal(got, e[key], 0)
        np.testing.assert_allclose(got, e[key], rtol=0, atol=1e-2)


def test_oracle_pres_lev_pos(era5):
    # The fixture stores the 0-based form of core.py:286-289.
    got = O.pres_lev_pos(era5["lev_level"], era5["sfc_p"])
    np.testing.assert_array_equal(got - 1, era5["sfc_start3d"])


@pytest.mark.parametrize("output_var,n", [("srh", 2), ("all", 8)])
def test_oracle_srh_sigma_golden(soundings, output_var, n):
    s = soundings
    P, T, TD, U, V = s["pressure"], s["temperature"], s["dewpoint"], s["u_wind_ms"], s["v_wind_ms"]
    res = O.calc_srh(P[:, 1:], T[:, 1:], TD[:, 1:], U[:, 1:], V[:, 1:], P[:, 0], T[:, 0],
                     TD[:, 0], U[:, 0], V[:, 0], depth=3000, vertical_lev="sigma",
                     output_var=output_var)
    assert len(res) == n
    np.testing.assert_almost_equal(res[0], s["SRH03_model_lev_rm"], 5)
    np.testing.assert_almost_equal(res[1], s["SRH03_model_lev_lm"], 5)


@pytest.mark.parametrize("output_var,n", [("srh", 2), ("all", 8)])
def test_oracle_srh_pressure_golden(era5, output_var, n):
    e = era5
    res = O.calc_srh(e["lev_level"], e["lev_t"], e["lev_td"], e["lev_u"], e["lev_v"], e["sfc_p"],
                     e["sfc_t"], e["sfc_td"], e["sfc_u"], e["sfc_v"], depth=3000,
                     vertical_lev="pressure", output_var=output_var)
    assert len(res) == n
    np.testing.assert_almost_equal(res[0], e["sfc_srh_rm"], 5)
    np.testing.assert_almost_equal(res[1], e["sfc_srh_lm"], 5)


def test_oracle_stdheight_matches_fixture_aglh(soundings):
    s = soundings
    P, T, TD = s["pressure"], s["temperature"], s["dewpoint"]
    H, Hs = O.loop_stdheight(P[:, 1:], T[:, 1:], TD[:, 1:], P[:, 0], T[:, 0], TD[:, 0],
                             np.full(P.shape[0], 2.0))
    np.testing.assert_allclose(Hs, s["AGLH_model_lev"][:, 0])
    np.testing.assert_allclose(H, s["AGLH_model_lev"][:, 1:], rtol=0, atol=1e-9)


def test_oracle_f64_close_to_f32(soundings):
    """The FP64 build runs the same algorithm: it must agree with FP32 to
    within the reference's own CAPE tolerance on the goldens."""
    args = _sigma_args(soundings)
    a = O.calc_cape(*args, source="surface", pinc=100, vertical_lev="sigma", precision="f32")
    b = O.calc_cape(*args, source="surface", pinc=100, vertical_lev="sigma", precision="f64")
    np.testing.assert_allclose(a[0], b[0], atol=1.0)
    np.testing.assert_allclose(a[1], b[1], atol=1.0)


def test_oracle_cold_surface_gate(soundings):
    """CAPE_CODE_model_lev.f90:77-88: ts <= 0 gives zeros and MU level 0."""
    s = soundings
    res = O.calc_cape(*_sigma_args(s), source="most-unstable", pinc=100, vertical_lev="sigma")
    cold = s["temperature"][:, 0] <= 0
    assert cold.any()
    for r in res:
        assert np.all(r[cold] == 0)
