"""The N > 1 path of bench.py on CPU ranks (gloo, world size 2): the path runs
independent replicas, so its only cross-rank steps are the barriers around the
timed region and the max-over-ranks of the timing, and under torchrun only
rank 0 prints the reference arm's line."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    w, r, _ = bench.dist_setup()
    assert (w, r) == (world, rank) and dist.get_backend() == "gloo"
    bench.barrier(w)
    m = bench.max_over_ranks(10.0 * (rank + 1), w)
    bench.barrier(w)
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"max": m}, f)
    dist.destroy_process_group()


def test_barrier_and_max_over_ranks_on_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    got = [json.load(open(tmp_path / f"rank{r}.json"))["max"] for r in range(2)]
    assert got == [20.0, 20.0]


@pytest.mark.timeout(600)
def test_reference_arm_under_torchrun_prints_once():
    """`bench.py --impl reference` launched as a multi-GPU run launches it (torchrun, 127.0.0.1): rank 0 times
    the CPU oracle and prints one JSON line, rank 1 exits 0 without output."""
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "0", "--resolution", "24", "--npz", "8", "--nq", "4"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
