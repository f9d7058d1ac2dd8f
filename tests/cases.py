"""Shared test inputs."""
import numpy as np

from xcape_gb300 import synthetic as S


def with_nonfinite(seed=13):
    """64 sigma columns x 40 levels with NaN and infinite values planted in
    levels, whole pressure columns and surface fields."""
    p, t, td, ps, ts, tds = (np.array(a) for a in S.sigma_c0(shape=(4, 16), nlev=40, seed=seed,
                                                             dtype=np.float32))
    t[0, 1, 5] = np.nan          # a level temperature
    td[0, 2, 30] = np.nan        # a dewpoint high up
    p[0, 3, :] = np.nan          # a whole pressure column
    ps[0, 4] = np.nan            # surface pressure
    tds[0, 5] = np.inf           # surface dewpoint
    t[0, 6, 10:] = -np.inf       # a cold-infinite upper column
    ts[0, 7] = np.nan            # the ts > 0 gate with NaN
    return p, t, td, ps, ts, tds
