"""Multi-GPU path = replicas: world size 2 over gloo on CPU, each rank advances
its own bed (oracle on the CPU stands in for the device), timings reduced as in
bench.py (max elapsed, summed particles)."""
import json
import os
import socket
import sys
import time

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as tmp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle.oracle import OracleSystem
    from sdem_gb300 import beds, replicas
    ws, r, _ = replicas.world()
    case = beds.lattice_cloud_case(150 + 50 * r, seed=replicas.rank_seed(40, r))
    o = OracleSystem(case)
    dist.barrier()
    t0 = time.perf_counter()
    o.step(3)
    el = time.perf_counter() - t0
    dist.barrier()
    value, tmax, ntot = replicas.aggregate(el, case.particles.n, 3)
    json.dump({"rank": r, "value": value, "tmax": tmax, "ntot": ntot, "el": el, "n": case.particles.n,
               "x0": float(case.particles.posR[0, 0])}, open(f"{out}.{r}", "w"))
    dist.destroy_process_group()


def test_two_replicas_gloo(tmp_path):
    port = _free_port()
    out = str(tmp_path / "res")
    tmp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    r = [json.load(open(f"{out}.{k}")) for k in range(2)]
    assert r[0]["ntot"] == r[1]["ntot"] == r[0]["n"] + r[1]["n"] == 350
    assert r[0]["tmax"] == r[1]["tmax"] == max(r[0]["el"], r[1]["el"])
    assert r[0]["value"] == pytest.approx(350 * 3 / r[0]["tmax"])
    assert r[0]["x0"] != r[1]["x0"]   # independent beds (seeds 40, 41)
