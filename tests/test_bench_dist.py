"""The bench's N>1 path on CPU: world_size-2 gloo ranks aggregate whole-job
throughput as (sum of units) / (max of elapsed times), and the reference arm
runs on rank 0 only."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    dist = bench.dist_init(world, "gloo")
    elapsed = [2.0, 3.0][rank]
    units = [100.0, 150.0][rank]
    tmax, total = bench.aggregate(elapsed, units, world, dist, "cpu")
    q.put((rank, tmax, total))
    dist.barrier()
    dist.destroy_process_group()


def test_aggregate_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, tmax, total in res:
        assert tmax == 3.0 and total == 250.0


def test_single_rank_aggregate_is_identity():
    import bench

    assert bench.aggregate(1.5, 10.0, 1) == (1.5, 10.0)


def _ref_worker(rank, world, port, q):
    import contextlib
    import io

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.main(["--impl", "reference", "--workload", "d1", "--steps", "1", "--warmup", "0",
                    "--cpu-seconds", "0.5"])
    q.put((rank, buf.getvalue()))


@pytest.mark.timeout(600)
def test_reference_arm_prints_on_rank0_only():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_ref_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=600) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert '"impl": "reference"' in out[0]
    assert out[1].strip() == ""


def test_reference_arm_without_cpu_sample_says_unavailable():
    """The one-matrix Cholesky has no CPU sample: its reference is the cuSOLVER
    call on the GPU, reported in our own line."""
    import contextlib
    import io
    import json

    import bench

    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.main(["--impl", "reference", "--workload", "large", "--steps", "1", "--warmup", "0"])
    line = json.loads(buf.getvalue().strip().splitlines()[-1])
    assert line["impl"] == "reference" and "unavailable" in line
