"""The bench's N>1 host logic as two gloo ranks on the CPU.

The contact path does not exchange data between GPUs: each rank is a replica
that evaluates its own block of the direction sweep, and the only collectives
are the timing ones (barriers and the max over ranks).  These tests run that
host logic with world size 2 over gloo: the split of the sweep into disjoint
per-rank blocks, the max-over-ranks aggregate, and the reference arm's
"rank 0 alone works" rule.
"""
import json
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as tmp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank), "SDFC_BENCH_BACKEND": "gloo"})
    sys.path.insert(0, ROOT)
    import io
    import contextlib

    import torch.distributed as dist

    import bench

    w, r = bench.dist_setup()
    assert (w, r) == (world, rank) and dist.get_backend() == "gloo"
    n = 16
    EA, phiA, EB, phiB = bench.instance_states(n, r, w)
    dirs = phiA[:, 3:] / 0.01
    gathered = [None] * w
    dist.all_gather_object(gathered, dirs.tolist())
    # the sharded legs: each rank's block of a shared workload, its per-instance results gathered
    # in rank order on every rank, sums over ranks
    blk = bench.rank_block(np.arange(8 * w), 8, r, w)
    rows = bench.gather_rows(np.stack([blk, 10 * blk], 1), w)
    total = bench.dist_sum(r + 1, w)
    c4_dirs = bench.rank_block(bench.W.cone_directions(4 * w, 30.0, seed=4), 4, r, w)
    c4_all = bench.gather_rows(c4_dirs, w)
    # max over ranks of a per-rank time, and the weak-scaling aggregate built on it
    t_max = bench.dist_max(0.5 + r, w)
    rate, t_job = bench.whole_job_rate(1000, 0.5 + r, w)
    bench.dist_barrier(w)
    # the reference arm: ranks other than 0 return without work and print nothing
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        ret = bench.run_reference(None, w, r) if r != 0 else None
    res = {"rank": r, "gathered": gathered, "t_max": t_max, "rate": rate, "t_job": t_job,
           "blk": blk.tolist(), "rows": rows.tolist(), "total": total, "c4_all": c4_all.tolist(),
           "ref_stdout": buf.getvalue(), "ref_ret": ret, "EB_eye": bool(np.allclose(EB, np.eye(4))),
           "phiB_zero": bool(not phiB.any()), "EA_rot_ok": bool(np.allclose(EA[:, 3], [0, 0, 0, 1]))}
    with open(os.path.join(out_dir, f"rank{r}.json"), "w") as f:
        json.dump(res, f)
    dist.barrier()
    dist.destroy_process_group()


@pytest.fixture(scope="module")
def two_ranks(tmp_path_factory):
    out = tmp_path_factory.mktemp("gloo")
    tmp.spawn(_rank_main, args=(2, _free_port(), str(out)), nprocs=2, join=True)
    return [json.load(open(out / f"rank{r}.json")) for r in range(2)]


def test_ranks_take_disjoint_blocks_of_one_sweep(two_ranks, workloads):
    g = two_ranks[0]["gathered"]
    assert g == two_ranks[1]["gathered"]
    d0, d1 = np.array(g[0]), np.array(g[1])
    full = workloads.fibonacci_directions(32)
    np.testing.assert_allclose(np.concatenate([d0, d1]), full, atol=1e-12)
    # no direction is evaluated twice
    assert np.min(np.linalg.norm(d0[:, None] - d1[None], axis=-1)) > 1e-3
    # world 1 keeps the single-GPU sweep
    _, phiA, _, _ = workloads.direction_sweep_states(16)
    np.testing.assert_allclose(phiA[:, 3:] / 0.01, workloads.fibonacci_directions(16), atol=1e-12)
    for r in two_ranks:
        assert r["EB_eye"] and r["phiB_zero"] and r["EA_rot_ok"]


def test_sharded_legs_split_and_gather(two_ranks, workloads):
    """Simulation, rollout and multi-part legs: disjoint blocks of one workload per rank, per-instance
    results gathered in rank order (the whole workload), counts summed over ranks."""
    assert two_ranks[0]["blk"] == list(range(8)) and two_ranks[1]["blk"] == list(range(8, 16))
    for r in two_ranks:
        assert r["rows"] == [[k, 10 * k] for k in range(16)]
        assert r["total"] == 3.0
        np.testing.assert_allclose(r["c4_all"], workloads.cone_directions(8, 30.0, seed=4), atol=0)


def test_max_over_ranks_and_whole_job_rate(two_ranks):
    for r in two_ranks:
        assert r["t_max"] == 1.5
        assert r["t_job"] == 1.5
        assert r["rate"] == pytest.approx(2 * 1000 / 1.5)


def test_reference_arm_runs_on_rank0_only(two_ranks):
    r1 = two_ranks[1]
    assert r1["ref_stdout"] == "" and r1["ref_ret"] is None


def test_rank_outside_world_is_rejected(workloads):
    with pytest.raises(ValueError):
        workloads.direction_sweep_states(4, rank=2, world=2)


def test_reference_arm_under_torchrun_prints_one_line():
    """`bench.py --impl reference` launched as the multi-GPU bench is (torchrun, 2 ranks, gloo
    here): exactly one JSON line, from rank 0, on a tiny workload."""
    import subprocess
    env = dict(os.environ, SDFC_BENCH_BACKEND="gloo")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--instances", "16", "--points", "500", "--grid", "32",
           "--cpu-sample", "8", "--steps", "1", "--warmup", "3", "--sim-steps", "0"]
    p = subprocess.run(cmd, env=env, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [json.loads(x) for x in p.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["scaling"] == "weak"
    # the reference's own Force where its library builds from staged sources, else the C port
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] in ("reference", "port")
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
