"""Host-side multi-rank logic with world_size 2 over gloo on the CPU: the
slowest-rank timing, whole-job rate, rank-ordered partial sums of a state
sharded by bands or by G' rows (checked against the oracle), and a failing
rank surfacing as an error on its peer instead of a hang."""
import datetime
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import PKG_ROOT, REPO


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, mode, out):
    sys.path.insert(0, PKG_ROOT)
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import torch.distributed as dist
    from gppsigma import dist as gd, workload as W
    import oracle_py

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world, timeout=datetime.timedelta(seconds=20))
    try:
        if mode == "timing":
            ms = 10.0 * (rank + 1)
            out[rank] = (gd.max_over_ranks(ms, dist), gd.job_rate(1e9, ms * 1e-3, dist))
        elif mode == "shard":
            # One state, bands split across ranks; partial sums added on rank 0.
            inp = W.make_inputs(W.Shape(8, 2, 300, 9, 3), 5)
            a, b = (0, 4) if rank == 0 else (4, 8)
            part = oracle_py.run(inp, band_begin=a, band_end=b)["achtemp"]
            total = gd.sum_in_rank_order(part, dist)
            if rank == 0:
                out[0] = total
        elif mode == "rows":
            # One state, G' rows split across ranks as the reference's MPI
            # version splits my_igp; partial sums added on rank 0.
            inp = W.make_inputs(W.Shape(8, 2, 300, 11, 3), 6)
            r0, r1 = gd.row_range(11, rank, world)
            part = oracle_py.run(inp.rows(r0, r1))
            total = [gd.sum_in_rank_order(part[k], dist) for k in ("achtemp", "asxtemp", "achstemp")]
            if rank == 0:
                out[0] = total
        elif mode == "rows_bench":
            # bench.py --shard rows: each rank generates and holds only its
            # rows (gd.rank_rows_inputs, here on the CPU), sums them (the
            # oracle standing in for the GPU call) and the partials are added
            # on rank 0 in rank order.
            shape = W.Shape(8, 2, 300, 11, 3, near_pole=0.03)
            d, (r0, r1) = gd.rank_rows_inputs(shape, 6, rank, world, device="cpu")
            assert d.ngpown == r1 - r0 == d.I_eps_array.shape[0] == d.wtilde_array.shape[0]
            inp = W.Inputs(W.Shape(8, 2, 300, r1 - r0, 3, near_pole=0.03), 6,
                           d.aqsmtemp.numpy(), d.aqsntemp.numpy(), d.I_eps_array.numpy(),
                           d.wtilde_array.numpy(), d.vcoul.numpy(), d.inv_igp_index.numpy(),
                           d.indinv.numpy(), d.wx_array.numpy())
            part = oracle_py.run(inp)
            total = [gd.sum_in_rank_order(part[k], dist) for k in ("achtemp", "asxtemp", "achstemp")]
            if rank == 0:
                out[0] = total
            out[("rows", rank)] = (r0, r1)
        elif mode == "rank_fails":
            if rank == 1:
                raise RuntimeError("rank 1 fails before the collective")
            try:
                gd.max_over_ranks(1.0, dist)
                out[0] = "no error"
            except Exception as e:  # the peer's failure must surface, not hang
                out[0] = type(e).__name__
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def _run(mode):
    mgr = mp.Manager()
    out = mgr.dict()
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_worker, args=(r, 2, port, mode, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        if p.is_alive():
            p.kill()
            pytest.fail("worker did not finish")
    return dict(out), [p.exitcode for p in procs]


def test_slowest_rank_sets_the_job_time():
    out, codes = _run("timing")
    assert codes == [0, 0]
    for r in (0, 1):
        slowest, rate = out[r]
        assert slowest == 20.0
        assert rate == pytest.approx(2 * 1e9 / 0.020)


def test_sharded_state_partials_add_up_in_rank_order():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_py
    from gppsigma import workload as W
    out, codes = _run("shard")
    assert codes == [0, 0]
    want = oracle_py.run(W.make_inputs(W.Shape(8, 2, 300, 9, 3), 5))["achtemp"]
    np.testing.assert_allclose(out[0], want, rtol=1e-12)


def test_row_sharded_state_adds_up_to_the_full_sums():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_py
    from gppsigma import dist as gd, workload as W
    assert [gd.row_range(11, r, 2) for r in (0, 1)] == [(0, 6), (6, 11)]
    assert [gd.row_range(7, r, 3) for r in range(3)] == [(0, 2), (2, 4), (4, 7)]
    out, codes = _run("rows")
    assert codes == [0, 0]
    want = oracle_py.run(W.make_inputs(W.Shape(8, 2, 300, 11, 3), 6))
    for got, key in zip(out[0], ("achtemp", "asxtemp", "achstemp")):
        np.testing.assert_allclose(got, want[key], rtol=1e-12)


def test_failing_rank_surfaces_on_its_peer():
    out, codes = _run("rank_fails")
    assert codes[1] != 0
    assert out[0] != "no error"


def test_bench_row_sharding_holds_only_its_rows_and_adds_up():
    """The code path of bench.py --shard rows (gppsigma.dist.rank_rows_inputs
    + sum_in_rank_order), world size 2 over gloo: each rank holds only its
    G' rows, and the rank-ordered sum of the ranks' partials equals the
    oracle's sums over the whole state."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_py
    from gppsigma import workload as W
    out, codes = _run("rows_bench")
    assert codes == [0, 0]
    assert out[("rows", 0)] == (0, 6) and out[("rows", 1)] == (6, 11)
    want = oracle_py.run(W.make_inputs(W.Shape(8, 2, 300, 11, 3, near_pole=0.03), 6))
    for got, key in zip(out[0], ("achtemp", "asxtemp", "achstemp")):
        np.testing.assert_allclose(got, want[key], rtol=1e-12)
