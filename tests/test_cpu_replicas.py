"""The replica path of bench.py under torch.distributed (gloo, world size 2,
CPU only): barrier, max over ranks and whole-job sums as the JSON line uses
them, and the reference arm leaving every rank but 0 without work."""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, out_dir):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    D = bench.Dist()
    D.barrier()
    res = {"rank": D.rank, "ws": D.ws, "max": D.max(float(rank + 1)),
           "sum": D.sum(10.0 * (rank + 1))}
    # work of both replicas over the slower one's time, as `value` is formed
    res["value"] = D.sum(100.0) / D.max(2.0 + rank)
    if rank == 1:
        # the reference arm runs on rank 0 only: other ranks return at once
        sys.argv = ["bench.py", "--impl", "reference"]
        res["ref_returned"] = bench.run_reference(bench.parse(), D) is None
    D.barrier()
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump(res, f)
    D.td.destroy_process_group()


def test_two_replicas_over_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    mp.start_processes(_worker, args=(_free_port(), str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    r = [json.loads((tmp_path / f"r{i}.json").read_text()) for i in range(2)]
    for i in range(2):
        assert r[i]["ws"] == 2 and r[i]["rank"] == i
        assert r[i]["max"] == 2.0
        assert r[i]["sum"] == 30.0
        assert r[i]["value"] == pytest.approx(200.0 / 3.0)
    assert r[1]["ref_returned"] is True
