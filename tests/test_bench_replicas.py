"""bench.py's replica plumbing on the CPU (gloo, world size 2): the process-group
set-up, the max over ranks of the timed region, the barrier, and the launcher
that `bench.py --gpus N` uses when it is not started by torchrun. A training
step does not shard (one view against one global parameter set), so N GPUs run
N independent replicas; no GPU is needed to check how they are started and how
their times are combined."""

from __future__ import annotations

import os
import subprocess
import sys
import textwrap
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

RANK_SCRIPT = textwrap.dedent("""
    import os, sys
    sys.path.insert(0, {root!r})
    import bench

    class Args:
        gpus = 2
    rank, world, local, group = bench.dist_setup(Args())
    assert world == 2 and local == rank and group is not None
    slowest = bench.reduce_max(group, 1.5 + rank)   # each rank's own time
    bench.barrier(group)
    assert slowest == 2.5, slowest
    if rank == 0:
        print(f"world={{world}} max={{slowest}}", flush=True)
    group.destroy_process_group()
""")


@pytest.fixture()
def rank_script(tmp_path):
    path = tmp_path / "rank.py"
    path.write_text(RANK_SCRIPT.format(root=str(ROOT)))
    return path


def test_two_gloo_ranks_take_the_max_time(rank_script):
    pytest.importorskip("torch")
    sys.path.insert(0, str(ROOT))
    import bench

    port = bench.free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, str(rank_script)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    assert [p.returncode for p in procs] == [0, 0], outs
    assert "world=2 max=2.5" in outs[0][0]


def test_launcher_starts_one_replica_per_gpu(rank_script, capfd):
    pytest.importorskip("torch")
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.launch_replicas(2, [], script=str(rank_script)) == 0
    assert "world=2 max=2.5" in capfd.readouterr().out


def test_launcher_reports_a_failing_replica(tmp_path):
    sys.path.insert(0, str(ROOT))
    import bench

    failing = tmp_path / "fail.py"
    failing.write_text("import os, sys\nsys.exit(3 if os.environ['RANK'] == '1' else 0)\n")
    assert bench.launch_replicas(2, [], script=str(failing)) == 3
