"""Multi-GPU is replicas only: the one cross-rank step of bench.py is the whole-job rate (particles summed
over ranks, time of the slowest rank).  Checked here with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r ran 100 (r+1) particles for 5 steps in 1 + r seconds
    rate, slowest = bench.replica_rate(100 * (rank + 1), 5, 1.0 + rank, dist, "cpu")
    out.put((rank, rate, slowest))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_rate_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, rate, slowest in res:
        assert slowest == 2.0
        assert rate == pytest.approx((100 + 200) * 5 / 2.0)


def test_replica_rate_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_rate(1000, 4, 2.0) == (2000.0, 2.0)


def test_reference_arm_reports_the_gpu_arms_config():
    """bench.py --impl reference prints the config of the GPU arm for the same flags (full workload sizes)."""
    import argparse
    import bench
    from piclas_gb300 import workloads
    from piclas_gb300.mesh import build_box_mesh
    from piclas_gb300.mesh import p_adaption_degrees
    cases = (("curved", 32, 16_000_000, 1, None, False, None, 0.0), ("plasma_wave", 8, 200_000, 1, None, False, None, 0.0),
             ("curved", 32, 16_000_000, 2, None, True, None, 0.0), ("curved", 32, 16_000_000, 1, "random", False, None, 0.0),
             ("curved", 32, 16_000_000, 2, None, False, "reflective", 0.2))
    for name, cells, n, ngeo, padapt, ptrace, walls, bulge in cases:
        args = argparse.Namespace(workload=name, precision="fp64", gpus=1, ngeo=ngeo, p_adaption=padapt,
                                  periodic_tracing=ptrace, walls=walls, wall_bulge=bulge)
        ref = bench.reference_config(args)
        mesh = build_box_mesh(2, 2, 2, 3)
        stand_in = workloads.Workload(**{**workloads.plasma_wave(mesh=mesh, n_particles=10).__dict__})
        n_loc = p_adaption_degrees(cells, cells, cells, padapt, 1, 3, seed=0) if padapt else None
        n_dofs = cells ** 3 * 64 if n_loc is None else int(((n_loc + 1) ** 3).sum())
        stand_in.mesh = type("M", (), {"n_elems": cells ** 3, "N": 3, "n_geo": ngeo, "n_loc": n_loc,
                                       "n_dofs": n_dofs})()
        stand_in.part_state = type("P", (), {"shape": (n, 6)})()
        stand_in.periodic_tracing = ptrace
        stand_in.walls, stand_in.wall_bulge = walls, bulge
        gpu = dict(bench.workload_config(stand_in, name), precision="fp64", parallelism="replicas x1")
        assert ref == gpu


def test_bench_reads_the_committed_ncu_figures():
    """The bench line's roofline takes DRAM traffic, issue and FP64-pipe figures from the committed ncu summary:
    the keys it builds must be present there (a renamed kernel or row would silently drop them)."""
    import bench
    assert bench.read_traffic("k_sf_gather5<3,0,0,1> @ curved") > 1e9
    assert bench.read_traffic("k_sf_gather7<1> @ curved") > 1e8
    assert bench.read_ncu_summary("k_sf_gather7<1> @ 16^3 curved, 2M particles")["inst_per_hit"] > 0
    fp64 = bench.read_ncu_fp64("k_sf_gather5<3,0,0,1> @ 16^3 curved, 2M particles")
    assert 0 < fp64["fp64_pipe_busy_pct"] <= 100 and 0 < fp64["lanes_active_of_32"] <= 32
