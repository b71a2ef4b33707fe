"""Multi-GPU runs: independent replicas of one mesh, or a batch of meshes
sharded over the ranks; the job figures reduce over ranks (slowest time,
summed units) and rank 0 gathers the per-mesh rows.  Exercised here with
two gloo ranks on the CPU."""
import json
import os
import socket
import subprocess
import sys
import textwrap

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

WORKER = textwrap.dedent("""
    import json, os, sys
    sys.path.insert(0, %r)
    import torch.distributed as dist
    from bookleaf_f90_gb300.replicas import gather_to_root, job_rate, max_over_ranks, shard
    rank = int(os.environ["RANK"])
    dist.init_process_group("gloo", init_method="env://")
    ms = [10.0, 20.0][rank]
    units = [100, 300][rank]
    rate, t_max, total = job_rate(ms, units)
    e2e_t = max_over_ranks([1.5, 0.5][rank])
    # the ensemble's shards: each rank computes its own share, rank 0
    # gathers them (and the ranks' rows)
    w = [(7 * i) %% 11 + 1 for i in range(40)]
    mine = shard(w, 2, rank)
    got = gather_to_root({"rank": rank, "mine": mine})
    dist.destroy_process_group()
    print(json.dumps({"rank": rank, "rate": rate, "t_max": t_max, "total": total, "e2e_t": e2e_t,
                      "gathered": got}))
""") % ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_job_rate_two_gloo_ranks():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", WORKER], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for o in outs:
        assert o["t_max"] == 20.0
        assert o["total"] == 400.0
        assert abs(o["rate"] - 400 / 20e-3) < 1e-6
        assert o["e2e_t"] == 1.5
    g = {o["rank"]: o["gathered"] for o in outs}
    assert g[1] is None
    assert [q["rank"] for q in g[0]] == [0, 1]
    a, b = g[0][0]["mine"], g[0][1]["mine"]
    assert not set(a) & set(b) and sorted(a + b) == list(range(40))


def test_job_rate_single_process():
    from bookleaf_f90_gb300.replicas import job_rate
    rate, t, z = job_rate(4.0, 2000)
    assert (rate, t, z) == (2000 / 4e-3, 4.0, 2000.0)


def test_shard_covers_once_and_balances():
    """Every item on exactly one rank, each rank's list in increasing order,
    the same answer on every call, and the loads within the largest item
    of one another (the longest-processing-time rule)."""
    import random
    from bookleaf_f90_gb300.replicas import shard
    rng = random.Random(5)
    w = [rng.uniform(1.0, 100.0) ** 1.5 for _ in range(512)]
    assert shard(w, 1, 0) == list(range(512))
    for world in (2, 3, 4, 8):
        parts = [shard(w, world, r) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(512))
        assert all(p == sorted(p) for p in parts)
        assert parts == [shard(w, world, r) for r in range(world)]
        loads = [sum(w[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(w)
