"""Multi-process paths on CPU (gloo, world_size 2): the pulse sharding
driver (every pulse on exactly one rank, balanced steps, metadata gathered
on rank 0, no data-path collective) with a stand-in for the GPU runner, and
bench.py's max-over-ranks timing of replicas."""
import json
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _init(rank, world, port):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)


def _shard_worker(rank, world, port, outdir):
    sys.path.insert(0, ROOT)
    from dirac_hydrogen_code_gb300 import shard
    from dirac_hydrogen_code_gb300.gen.pulses import draw_pulses
    _init(rank, world, port)
    pulses = draw_pulses(9, 5)

    def fake_runner(ids):
        for k in ids:
            with open(os.path.join(outdir, f"pulse{k}.json"), "w") as f:
                json.dump({"rank": rank}, f)
        return {"pulses": ids, "pulse_steps": sum(pulses[k]["ntime"] for k in ids), "wall_s": 1.0 + rank}

    shard.worker(rank, world, pulses, outdir, fake_runner)
    dist.barrier()
    dist.destroy_process_group()


def test_shard_driver_two_ranks(tmp_path):
    from dirac_hydrogen_code_gb300 import shard
    from dirac_hydrogen_code_gb300.gen.pulses import draw_pulses
    pulses = draw_pulses(9, 5)
    a = shard.assign(pulses, 2)
    assert sorted(a[0] + a[1]) == list(range(9)) and not set(a[0]) & set(a[1])
    loads = [sum(pulses[k]["ntime"] for k in r) for r in a]
    assert abs(loads[0] - loads[1]) <= max(p["ntime"] for p in pulses)
    mp.spawn(_shard_worker, args=(2, _port(), str(tmp_path)), nprocs=2, join=True)
    summary = json.load(open(tmp_path / "summary.json"))
    assert sorted(k for r in summary["ranks"] for k in r["pulses"]) == list(range(9))
    assert summary["wall_s"] == 2.0 and summary["pulse_steps"] == sum(p["ntime"] for p in pulses)
    for k in range(9):
        owner = json.load(open(tmp_path / f"pulse{k}.json"))["rank"]
        assert k in a[owner]


def _bench_worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import bench
    _init(rank, world, port)
    t = bench.max_over_ranks(0.5 + rank, dist, "cpu")
    q.put((rank, t))
    dist.destroy_process_group()


def test_bench_replica_timing_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    ps = [ctx.Process(target=_bench_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    got = dict(q.get() for _ in range(2))
    assert got == {0: 1.5, 1: 1.5}
