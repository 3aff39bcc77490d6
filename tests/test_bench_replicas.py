"""bench.py's N>1 path on CPU: world_size-2 gloo ranks take the max time over
ranks and report the whole job's units; under --impl reference only rank 0
measures and prints (no GPU needed)."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _rank(rank, ws, port, out):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        own = 1.0 + rank  # rank 1 is the slower one
        t = bench.replica_elapsed(own, ws, "cpu")
        out.put((rank, t, bench.replica_value(100.0, ws, t)))
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_max_time_over_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = 29600 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(out.get(timeout=10) for _ in range(2))
    # both ranks see the slower rank's 2.0 s; 2 ranks x 100 units in 2.0 s
    assert [r[1] for r in res] == [2.0, 2.0]
    assert [r[2] for r in res] == [100.0, 100.0]


def test_single_rank_is_unchanged():
    import bench

    assert bench.replica_elapsed(3.5, 1, "cpu") == 3.5
    assert bench.replica_value(70.0, 1, 3.5) == 20.0


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "1"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_reference_arm_loads_no_product_code():
    # the reference arm's workload generator and CPU pass must not import the
    # product package (whose __init__ loads its native library)
    code = ("import sys; sys.path.insert(0, %r); import bench; "
            "s = bench.synth_module(); rows, root, _ = s.alignment(40, 300, seed=3, dup_frac=0.3); "
            "fa = s.to_fasta(rows); lt, idx, rd, sec = bench.oracle_pass(fa, root.tobytes()); "
            "assert len(idx) == 40 and len(rd) == 40 and lt.size > 0; "
            "bad = [m for m in sys.modules if m.startswith('hammingdist')]; "
            "assert not bad, bad" % ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
