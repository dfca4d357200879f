"""bench.py's multi-GPU mode runs independent replicas: two gloo ranks on CPU
check the max-over-ranks timing, the whole-job value and the barrier, and
that the reference arm does no work on ranks other than 0."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    bench.init_dist(world, "gloo")
    ms_local = 100.0 * (rank + 1)  # rank 1 is the slower replica
    value = bench.replica_value(ms_local, 4, world)
    bench.barrier(world)
    args = bench.parse_args(["--impl", "reference", "--steps", "1", "--warmup", "0", "--grid", "32"])
    ref, _ = bench.run_reference(args, rank, world)
    ok = ref is None
    if ref is not None:
        # the reference arm's line: the contract's keys, its own CPU baseline and an e2e with no copies
        want = {"impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"}
        ok = (want <= set(ref) and ref["impl"] == "reference" and ref["metric"] == bench.METRIC
              and ref["higher_is_better"] is False and ref["value"] > 0
              and ref["cpu_baseline"]["value"] == ref["value"] and ref["cpu_baseline"]["kind"] == "port"
              and ref["e2e"]["h2d_bytes_per_step"] == 0 and ref["e2e"]["d2h_bytes_per_step"] == 0)
    out.put((rank, value, ok))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_two_replicas_report_slowest_rank_over_all_snapshots():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # max over ranks = 200 ms for 4 snapshots on each of 2 replicas
    assert [v for _, v, _ in res] == [25.0, 25.0]
    # only rank 0 runs the reference arm, and its line keeps the contract
    assert res[0][2] is True and res[1][2] is True
