"""The N > 1 bench path on CPU: world_size-2 `gloo` process groups standing in
for the one-process-per-GPU launch.  The path does not shard (replicas only),
so what is checked is what the replicas share: the whole-job value is all
ranks' units over the slowest rank's time, every rank builds the same work
(the seeded generator and the host stream give identical hypergraphs and
initial partitions in every process), and the reference arm prints from rank
0 alone."""
import contextlib
import hashlib
import io
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out_dir):
    import torch
    import torch.distributed as tdist
    import bench
    import fastpartitioner_gb300 as fp
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # aggregation: rank r took 1 + r seconds for 1000 units
        value, secs, n = bench.whole_job(1000, 1.0 + rank)
        # the replicas' work: the workload at a small scale, streamed on the host
        w = bench.WORKLOADS["zipf4m"]
        hg = fp.generate(bench.spec_for(fp, w, 1024))
        s = fp.stream_partition(hg, w["K"], "TV", w["eps"])
        h = hashlib.sha256()
        for a in (hg.nptr, hg.npins, s["part_vec"], s["ep_parts"]):
            h.update(np.ascontiguousarray(a).tobytes())
        digests = [None] * world
        tdist.all_gather_object(digests, (hg.pins, h.hexdigest()))
        np.save(Path(out_dir) / f"rank{rank}.npy",
                np.array([value, secs, n, int(len(set(digests)) == 1), digests[0][0]], np.float64))
        tdist.barrier()
    finally:
        tdist.destroy_process_group()


def test_whole_job_and_identical_replicas_over_gloo(tmp_path):
    world = 2
    mp.spawn(rank_main, args=(world, free_port(), str(tmp_path)), nprocs=world, join=True)
    rows = [np.load(tmp_path / f"rank{r}.npy") for r in range(world)]
    for r in rows:
        value, secs, n, same, pins = r
        assert n == world
        assert secs == 2.0                       # the slowest rank's time
        assert value == 1000 * world / 2.0       # all ranks' units over it
        assert same == 1 and pins > 0            # every replica built the same work


def test_whole_job_without_a_process_group():
    import bench
    assert bench.whole_job(500, 2.0) == (250.0, 2.0, 1)


def test_reference_arm_prints_from_rank_zero_only(monkeypatch):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference_arm(None)            # returns before reading any argument
    assert buf.getvalue() == ""
