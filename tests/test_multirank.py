"""Multi-rank host logic of bench.py on CPU (gloo, world_size 2).

Columns are independent, so N ranks each take an equal contiguous share of
the columns and never exchange data; the only collectives are the barrier
and the max-over-ranks of the step time.  This test runs that logic with
two gloo ranks and the CPU oracle as the per-rank compute, and checks that
the union of the shards is the whole grid and equals a single-rank run.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_covers_all_columns():
    for n in (1, 7, 1038240):
        for world in (1, 2, 3, 8):
            spans = [bench.shard(n, world, r) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            for (a, b), (c, d) in zip(spans, spans[1:]):
                assert b == c
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


def _worker(rank, world, port, out_path):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import oracle as O
    from xcape_gb300 import synthetic as S
    d = bench.init_dist(world, "gloo")
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(8, 16), nlev=37)
    n = ps.size
    lo, hi = bench.shard(n, world, rank)
    t2, td2 = t.reshape(n, -1)[lo:hi], td.reshape(n, -1)[lo:hi]
    sf = [a.ravel()[lo:hi] for a in (ps, ts, tds)]
    st = O.pres_lev_pos(plev, sf[0])
    r = O.loopcape(plev, t2, td2, *sf, 500.0, 2, 500.0, 1, start=st, p_is_1d=True, nthreads=1)
    tmax = bench.max_over_ranks(d, float(rank + 1))
    np.save(f"{out_path}.{rank}.npy", np.concatenate([[lo, hi, tmax], r["cape"]]))
    d.barrier()
    d.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_gloo_ranks_match_single_rank(tmp_path):
    world = 2
    port = _free_port()
    out = str(tmp_path / "r")
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, start_method="spawn")
    parts = [np.load(f"{out}.{r}.npy") for r in range(world)]
    for p in parts:
        assert p[2] == world  # max over ranks of (rank + 1)
    cape = np.concatenate([p[3:] for p in parts])
    import oracle as O
    from xcape_gb300 import synthetic as S
    plev, t, td, ps, ts, tds = S.pressure_c1(shape=(8, 16), nlev=37)
    want = O.calc_cape(plev, t, td, ps, ts, tds, source="most-unstable", vertical_lev="pressure")
    np.testing.assert_array_equal(cape.astype(np.float32), want[0].ravel())
