"""The bench's multi-rank path on the host: two gloo ranks (one replica per rank on a GPU machine).

Each rank of a torchrun launch runs its own replica; the ranks meet only at the
barriers around the timed region and in the max-over-ranks of the elapsed
time.  This runs those pieces with world size 2 over gloo on 127.0.0.1, and
checks that under two ranks the reference arm prints exactly one line, from
rank 0.
"""

import io
import json
import os
import socket
import sys
from contextlib import redirect_stdout
from types import SimpleNamespace

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update({"WORLD_SIZE": "2", "RANK": str(rank), "LOCAL_RANK": str(rank), "MASTER_ADDR": "127.0.0.1",
                       "MASTER_PORT": str(port), "ASTREA_DIST_BACKEND": "gloo"})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    ws, r, _ = bench.dist_init()
    bench.barrier(ws)
    m = bench.allmax(1.0 + 1.5 * r, ws)
    buf = io.StringIO()
    args = SimpleNamespace(cpu_n=16, steps=1, warmup=0, gpus=2)
    with redirect_stdout(buf):
        rc = bench.reference_arm(args)
    bench.barrier(ws)
    dist.destroy_process_group()
    q.put((r, ws, m, rc, buf.getvalue()))


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [x[1] for x in res] == [2, 2]
    assert [x[2] for x in res] == [2.5, 2.5]  # the max over ranks, on every rank
    assert [x[3] for x in res] == [0, 0]
    lines0 = [l for l in res[0][4].splitlines() if l.strip()]
    assert len(lines0) == 1 and res[1][4].strip() == ""
    line = json.loads(lines0[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
