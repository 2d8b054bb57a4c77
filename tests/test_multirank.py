"""The N > 1 path of bench.py on CPU with the gloo backend (world size 2):
every rank solves its own K-sector (J = rank mod Nphi) with no data exchange;
the only collectives are the barrier around the timed region and the max of
the per-rank times. Run as two processes on 127.0.0.1."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    w, r, local, pg = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank) and pg is not None
    bench.barrier(pg)
    m = bench.max_over_ranks(pg, 1.5 + rank)  # per-rank step times: the job's time is the max
    with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as f:
        f.write(repr(m))
    pg.destroy_process_group()


def test_barrier_and_max_over_ranks_gloo(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    vals = [float((tmp_path / f"r{r}.txt").read_text()) for r in range(2)]
    assert vals == [2.5, 2.5]


def test_rank_sector_assignment_is_disjoint():
    sys.path.insert(0, ROOT)
    import bench

    for world in (2, 4, 8):
        Js = [bench.rank_sector(r, bench.NPHI) for r in range(world)]
        assert len(set(Js)) == world  # weak scaling: one K-sector per rank, all different


def test_reference_arm_under_torchrun():
    """torchrun with 2 ranks: rank 0 times the CPU implementation and prints one
    JSON line, rank 1 exits 0 without work."""
    env = dict(os.environ)
    env.pop("CUDA_VISIBLE_DEVICES", None)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] in ("port", "reference")
