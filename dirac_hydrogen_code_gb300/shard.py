"""Pulses sharded over GPUs: one process per GPU (launched by torchrun),
each rank advances its own pulses as one batch on its own GPU.  Pulses are
independent, so nothing but metadata crosses ranks: there is no collective on
the data path (the reference's multi-rank path partitions one pulse with
METIS and needs halo exchanges; that does not apply to independent pulses).

Outputs per pulse k: ``pulse<k>.out`` (final state, the x<iter>.out format)
and ``pulse<k>.json`` (steps, iterations, populations when asked); rank 0
writes ``summary.json`` after gathering the per-rank metadata.

    python -m torch.distributed.run --nnodes=1 --nproc-per-node N --master-addr 127.0.0.1 \\
        -m dirac_hydrogen_code_gb300.shard --workdir D --params params.json --pulses pulses.json --out OUT
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

from .cn import step_times


def assign(pulses: list[dict], world: int) -> list[list[int]]:
    """Longest-first greedy assignment by step count: every pulse on exactly
    one rank, total steps per rank balanced; deterministic."""
    lengths = []
    for k, p in enumerate(pulses):
        maxtime = p.get("maxtime", p["cycles"] * 2 * np.pi / p["omega"])
        lengths.append((len(step_times(maxtime, p["ntime"])[1]), k))
    load = [0] * world
    out = [[] for _ in range(world)]
    for n, k in sorted(lengths, key=lambda t: (-t[0], t[1])):
        r = min(range(world), key=lambda i: (load[i], i))
        out[r].append(k)
        load[r] += n
    return [sorted(o) for o in out]


def gpu_runner(workdir: str, params: dict, pulses: list[dict], ids: list[int], outdir: str, device: int,
               precision: str, tol: float, with_populations: bool) -> dict:
    """Runs pulses ``ids`` as one batch on ``device`` and writes their outputs."""
    import torch
    from .cn import run_batch
    from .formats import out_write
    from .gen.pulses import pulse_tables_many
    from .native import Problem
    torch.cuda.set_device(device)
    lmax = params["Nl"] if params["Nl"] else 2 * params["Nkappa"] + 1
    prob = Problem(workdir, lmax)
    mine = [pulses[k] for k in ids]
    tables = pulse_tables_many(params, mine)
    t0 = time.perf_counter()
    xs, recs, b = run_batch(prob, mine, tables, tol=tol, precision=precision, device=device)
    wall = time.perf_counter() - t0
    _, xperm = prob.psi0()
    pops = None
    if with_populations:
        from .populations import Eigenbasis
        kap, _ = prob.blocks()
        eb = Eigenbasis(workdir, kap)
        pops = [eb.populations(x) for x in xs]
    steps = 0
    for j, k in enumerate(ids):
        xorig = np.empty_like(xs[j])
        xorig[xperm] = xs[j]
        out_write(os.path.join(outdir, f"pulse{k}.out"), xorig)
        rec = {"pulse": pulses[k], "steps": len(recs[j]), "iters": [r["iters"] for r in recs[j]]}
        if pops is not None:
            rec["populations"] = pops[j]
        with open(os.path.join(outdir, f"pulse{k}.json"), "w") as f:
            json.dump(rec, f)
        steps += len(recs[j])
    b.close()
    return {"pulses": ids, "pulse_steps": steps, "wall_s": wall}


def worker(rank: int, world: int, pulses: list[dict], outdir: str, runner) -> dict | None:
    """One rank: its share of the pulses, then a metadata gather to rank 0."""
    import torch.distributed as dist
    ids = assign(pulses, world)[rank]
    meta = runner(ids) if ids else {"pulses": [], "pulse_steps": 0, "wall_s": 0.0}
    meta["rank"] = rank
    gathered = [None] * world
    if world > 1:
        dist.all_gather_object(gathered, meta)
    else:
        gathered = [meta]
    if rank != 0:
        return None
    done = sorted(k for m in gathered for k in m["pulses"])
    if done != list(range(len(pulses))):
        raise RuntimeError(f"pulses processed {done} != all {len(pulses)}")
    wall = max(m["wall_s"] for m in gathered)
    summary = {"ranks": gathered, "pulse_steps": sum(m["pulse_steps"] for m in gathered), "wall_s": wall,
               "pulse_steps_per_s": sum(m["pulse_steps"] for m in gathered) / wall if wall > 0 else None}
    with open(os.path.join(outdir, "summary.json"), "w") as f:
        json.dump(summary, f)
    return summary


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m dirac_hydrogen_code_gb300.shard")
    ap.add_argument("--workdir", required=True, help="problem directory (generator outputs)")
    ap.add_argument("--params", required=True, help="generator JSON (Nsplines, Nkappa, Nmu, Nl, rBox, ...)")
    ap.add_argument("--pulses", required=True, help="JSON list of {E0, omega, cycles, ntime[, maxtime]}")
    ap.add_argument("--out", required=True)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--tol", type=float, default=1e-12)
    ap.add_argument("--populations", action="store_true")
    args = ap.parse_args(argv)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    with open(args.params) as f:
        params = json.load(f)
    with open(args.pulses) as f:
        pulses = json.load(f)
    os.makedirs(args.out, exist_ok=True)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")          # metadata only
    runner = lambda ids: gpu_runner(args.workdir, params, pulses, ids, args.out, local,  # noqa: E731
                                    args.precision, args.tol, args.populations)
    s = worker(rank, world, pulses, args.out, runner)
    if s is not None:
        print(json.dumps({k: v for k, v in s.items() if k != "ranks"}))
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
