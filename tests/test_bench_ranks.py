"""The benchmark's host logic on the CPU: the replica path on two gloo ranks
(the barrier, the max-over-ranks timing and the whole-job aggregate that
`bench.py --gpus N` reports when torchrun starts one replica per GPU), and the
clock record parsed from nvidia-smi samples."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, results):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        bench.barrier(world)
        # the second rank is the slower one in the timed region, the first in the end-to-end leg
        ms, e2e = bench.max_over_ranks([10.0 + rank, 3.0 - rank], world)
        bench.barrier(world)
        results[rank] = (ms, e2e, bench.job_mlups(1000, 20, world, ms))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        results = m.dict()
        mp.start_processes(_rank_main, args=(2, _free_port(), results), nprocs=2, join=True,
                           start_method="spawn")
        got = dict(results)
    assert got[0] == got[1]
    ms, e2e, mlups = got[0]
    assert ms == 11.0 and e2e == 3.0
    # both replicas' cells over the slowest replica's time
    assert mlups == pytest.approx(1000 * 20 * 2 / (11.0 * 1e3))


def test_one_rank_needs_no_process_group():
    import bench
    bench.barrier(1)
    assert bench.max_over_ranks([2, 5.5], 1) == [2.0, 5.5]
    assert bench.job_mlups(33554432, 100, 1, 50.0) == pytest.approx(67108.864)


def test_clock_rows_report_median_clock_and_throttle_reasons():
    """The clocks record that rejects a throttled run: median SM clock under load,
    the maximum clock, and every throttle reason that was active in any sample."""
    import bench
    text = "\n".join([
        "0, 2070, 2070, 950.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 1980, 2070, 1390.5, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1200.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
        "0, 1400, 2070, 1000.0, 0x0000000000000008, Active, Not Active, Not Active, Not Active",
    ])
    got = bench.parse_clock_rows(text)
    assert got == {"sm_mhz": 2025.0, "sm_max_mhz": 2070.0, "reasons": ["hw_slowdown", "sw_power_cap"],
                   "samples": 4}
    assert bench.parse_clock_rows("") is None
    assert bench.parse_clock_rows("not,a,number") is None
