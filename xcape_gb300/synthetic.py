"""Seeded synthetic soundings with the shapes and value ranges of the
benchmark workloads (there is no public dataset for this path; the reference
only ships 30 test columns).

Profile of one column:
  * ps ~ U(ps_lo, ps_hi) hPa, Ts ~ U(12, 32) degC, RH0 ~ U(0.6, 0.95);
  * T(z) = Ts - 6.5 K/km * min(z, 12 km), isothermal above;
  * RH(z) = RH0 * exp(-z / 3 km), dewpoint from the Magnus form
    (17.67, 243.5 degC) inverted, clipped to T;
  * z(p) from the hypsometric relation of that temperature profile;
  * winds (SRH workload): speed 5 + 25 tanh(z / 4 km) m/s, direction veering
    from southerly to westerly over the lowest 6 km, plus N(0, 2 m/s) noise;
    the surface wind is the lowest level's.

Workloads:
  * ``sigma_c0``   64 x 64 columns x 40 sigma levels (0.995 .. 0.1), float64,
                   ps ~ U(950, 1020)   -- the small CPU-runnable case;
  * ``pressure_c1`` 721 x 1440 columns x 37 pressure levels (1000 .. 100 hPa),
                   float32, ps ~ U(700, 1030) so that below-ground levels are
                   masked, T + N(0, 2 K) noise;
  * ``srh_c2``     1024 x 1024 columns x 50 sigma levels, float32, with winds.
Every generator takes a ``shape`` override so tests can draw small batches
from the same distributions.
"""
import numpy as np

G = 9.80665
RD = 287.04
LAPSE = 6.5e-3
Z_TROP = 12000.0


def sigma_levels(n):
    k = np.arange(n, dtype=np.float64)
    return 0.995 * (0.1 / 0.995) ** (k / (n - 1))


def _z_of_p(p, ps, ts_k):
    """Height (m) of pressure p (hPa) above a surface at ps (hPa), ts_k (K),
    for the 6.5 K/km troposphere capped by an isothermal layer at 12 km."""
    expo = RD * LAPSE / G
    t_trop = ts_k - LAPSE * Z_TROP
    p_trop = ps * (t_trop / ts_k) ** (1.0 / expo)
    z_lo = ts_k / LAPSE * (1.0 - (p / ps) ** expo)
    z_hi = Z_TROP + RD * t_trop / G * np.log(p_trop / p)
    return np.where(p >= p_trop, z_lo, z_hi)


def _thermo(z, ts_c, rh0):
    t = ts_c - LAPSE * 1000.0 * np.minimum(z, Z_TROP) / 1000.0
    rh = rh0 * np.exp(-np.maximum(z, 0.0) / 3000.0)
    es = 6.112 * np.exp(17.67 * t / (t + 243.5))
    lne = np.log(np.maximum(rh * es, 1e-12) / 6.112)
    td = 243.5 * lne / (17.67 - lne)
    return t, np.minimum(td, t)


def _surface(rng, n, ps_lo, ps_hi):
    ps = rng.uniform(ps_lo, ps_hi, n)
    ts = rng.uniform(12.0, 32.0, n)
    rh0 = rng.uniform(0.6, 0.95, n)
    return ps, ts, rh0


def sigma_c0(shape=(64, 64), nlev=40, seed=0, dtype=np.float64, ps_range=(950.0, 1020.0)):
    """Returns (p, t, td, ps, ts, tds) for calc_cape(vertical_lev='sigma')."""
    rng = np.random.default_rng(seed)
    n = int(np.prod(shape))
    ps, ts, rh0 = _surface(rng, n, *ps_range)
    sig = sigma_levels(nlev)
    p = ps[:, None] * sig[None, :]
    z = _z_of_p(p, ps[:, None], ts[:, None] + 273.15)
    t, td = _thermo(z, ts[:, None], rh0[:, None])
    tds = _thermo(np.zeros(n), ts, rh0)[1]
    out = [p, t, td, ps, ts, tds]
    full = tuple(shape) + (nlev,)
    return tuple(a.reshape(full if a.ndim == 2 else tuple(shape)).astype(dtype) for a in out)


def pressure_levels(nlev=37):
    return np.linspace(1000.0, 100.0, nlev)


def pressure_c1(shape=(721, 1440), nlev=37, seed=1, dtype=np.float32, noise_k=2.0,
                ps_range=(700.0, 1030.0)):
    """Returns (p1d, t, td, ps, ts, tds) for calc_cape(vertical_lev='pressure')."""
    rng = np.random.default_rng(seed)
    n = int(np.prod(shape))
    ps, ts, rh0 = _surface(rng, n, *ps_range)
    plev = pressure_levels(nlev)
    z = _z_of_p(plev[None, :], ps[:, None], ts[:, None] + 273.15)
    t, td = _thermo(z, ts[:, None], rh0[:, None])
    t = t + rng.normal(0.0, noise_k, t.shape)
    td = np.minimum(td, t)
    tds = _thermo(np.zeros(n), ts, rh0)[1]
    full = tuple(shape) + (nlev,)
    return (plev.astype(dtype), t.reshape(full).astype(dtype), td.reshape(full).astype(dtype),
            ps.reshape(shape).astype(dtype), ts.reshape(shape).astype(dtype),
            tds.reshape(shape).astype(dtype))


def _winds(rng, z):
    speed = 5.0 + 25.0 * np.tanh(z / 4000.0)
    phi = np.deg2rad(180.0 + 90.0 * np.clip(z / 6000.0, 0.0, 1.0))
    u = -speed * np.sin(phi) + rng.normal(0.0, 2.0, z.shape)
    v = -speed * np.cos(phi) + rng.normal(0.0, 2.0, z.shape)
    return u, v


def srh_c2(shape=(1024, 1024), nlev=50, seed=2, dtype=np.float32):
    """Returns (p, t, td, u, v, ps, ts, tds, us, vs) for
    calc_srh(vertical_lev='model')."""
    rng = np.random.default_rng(seed)
    n = int(np.prod(shape))
    ps, ts, rh0 = _surface(rng, n, 950.0, 1020.0)
    sig = sigma_levels(nlev)
    p = ps[:, None] * sig[None, :]
    z = _z_of_p(p, ps[:, None], ts[:, None] + 273.15)
    t, td = _thermo(z, ts[:, None], rh0[:, None])
    u, v = _winds(rng, z)
    tds = _thermo(np.zeros(n), ts, rh0)[1]
    us, vs = u[:, 0].copy(), v[:, 0].copy()
    full = tuple(shape) + (nlev,)
    lv = [a.reshape(full).astype(dtype) for a in (p, t, td, u, v)]
    sf = [a.reshape(shape).astype(dtype) for a in (ps, ts, tds, us, vs)]
    return tuple(lv + sf)


def pressure_srh(shape=(64, 64), nlev=37, seed=3, dtype=np.float32):
    """calc_srh inputs on pressure levels (1-D p), for tests."""
    rng = np.random.default_rng(seed)
    n = int(np.prod(shape))
    ps, ts, rh0 = _surface(rng, n, 700.0, 1030.0)
    plev = pressure_levels(nlev)
    z = _z_of_p(plev[None, :], ps[:, None], ts[:, None] + 273.15)
    t, td = _thermo(z, ts[:, None], rh0[:, None])
    u, v = _winds(rng, np.maximum(z, 0.0))
    tds = _thermo(np.zeros(n), ts, rh0)[1]
    us, vs = rng.normal(0.0, 2.0, n), 5.0 + rng.normal(0.0, 2.0, n)
    full = tuple(shape) + (nlev,)
    return (plev.astype(dtype), *(a.reshape(full).astype(dtype) for a in (t, td, u, v)),
            *(a.reshape(shape).astype(dtype) for a in (ps, ts, tds, us, vs)))
