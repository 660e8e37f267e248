"""The N > 1 host logic of bench.py on CPU: every rank runs its own replica
(the path has no exchange), the ranks meet at a barrier around the timed
steps, the slowest rank's time is taken with a max-reduce, and the value is
the units of all ranks over that time.  Run as two gloo ranks, as torchrun
would start them; the reference arm's other ranks exit without work."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    w, r, local = bench._dist()
    grp = bench._Group(w, local)
    try:
        grp.barrier()
        slowest = grp.max(times[r])
        grp.barrier()
        out.put((r, w, slowest, bench.aggregate_value(1000, 20, w, slowest)))
    finally:
        grp.close()


def test_two_gloo_ranks_take_the_slowest_time_and_sum_the_replicas():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    times = [12.5, 20.0]   # ms of each rank's timed steps
    procs = [mp.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, world, slowest, value) in enumerate(got):
        assert (rank, world) == (r, 2)
        assert slowest == 20.0
        # 1000 cells x 20 steps on each of 2 replicas in 20 ms
        assert value == pytest.approx(2 * 1000 * 20 / 20e-3 / 1e6)


def test_one_rank_needs_no_process_group():
    grp = bench._Group(1, 0)
    grp.barrier()
    assert grp.max(3.5) == 3.5
    grp.close()


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun the reference arm's other ranks exit 0 at once,
    printing nothing and touching no process group."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1",
               MASTER_PORT=str(_free_port()))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "2", "--warmup", "3"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
