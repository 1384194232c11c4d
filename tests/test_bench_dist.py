"""The multi-rank plumbing of bench.py on CPU, world size 2 over gloo (the
step path does not shard: N GPUs run N replicas, so the ranks only meet in
the barrier around the timed region and the max-over-ranks of the time).

Two spawned ranks check that max_over_ranks returns the slowest rank's
time on every rank, that the barrier releases both, and that the reference
arm runs on rank 0 only: rank 0 prints one JSON line with the
impl="reference" keys, rank 1 returns without output."""
import contextlib
import io
import json
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench

    dist = bench.init_dist(world, "gloo")
    t = bench.max_over_ranks(1.0 + rank, world, "cpu")
    bench.barrier(world)
    sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0", "--mx", "256"]
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(bench.parse_args())
    dist.destroy_process_group()
    with open(os.path.join(outdir, f"rank{rank}.json"), "w") as f:
        json.dump({"max": t, "stdout": buf.getvalue()}, f)


@pytest.mark.timeout(300)
def test_two_ranks_gloo(tmp_path):
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    r0 = json.load(open(tmp_path / "rank0.json"))
    r1 = json.load(open(tmp_path / "rank1.json"))
    assert r0["max"] == r1["max"] == 2.0
    assert r1["stdout"] == ""
    lines = [ln for ln in r0["stdout"].splitlines() if ln.strip()]
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["n_gpus"] == 2 and out["value"] > 0
    assert out["e2e"]["h2d_bytes_per_step"] == 0 and out["cpu_baseline"]["kind"] == "port"
