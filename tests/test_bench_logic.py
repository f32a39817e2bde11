"""Host logic of bench.py without a GPU: the roofline of the dominant class
launch from per-launch records, and the caller-side Boys values used to
prepare the generated-library inputs (against the oracle)."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_kernel_roofline_picks_dominant_launch():
    import bench
    launches = [
        {"class": (0, 0, 1, 0), "fp32": 0, "kernel": "register", "ms_avg": 30.0,
         "flops": 1.5e10, "prim_quartets": 10, "quartets": 5},
        {"class": (1, 0, 1, 0), "fp32": 1, "kernel": "register", "ms_avg": 10.0,
         "flops": 2.0e11, "prim_quartets": 20, "quartets": 7},
    ]
    peaks = {"fp64": 1.1, "fp32": 70.0}
    r = bench.kernel_roofline(launches, peaks, "h2o32_cc-pvdz", "mixed")
    assert r["kernel"] == "rk_kernel<double,0,0,1,0,J/K>"
    assert abs(r["achieved"] - 1.5e10 / 0.030 / 1e12) < 1e-12
    assert abs(r["frac"] - r["achieved"] / 1.1) < 1e-12
    assert abs(r["share_of_pass"] - 0.75) < 1e-12 and r["bound"] == "fp64-pipe"
    assert bench.kernel_roofline([], peaks, "x", "mixed") is None


def test_primitive_inputs_boys_match_oracle():
    # the scipy Boys values bench.py uses for --primitive-api inputs
    import bench
    import libint_gb300 as lg
    from oracle import oracle
    oracle.build()
    rng = np.random.default_rng(3)
    sh, prims, AB, CD = bench._prim_inputs(rng, (1, 0, 2, 1), 2, 1, lg._lgx.PRIM_DTYPE)
    assert len(prims) == 16
    for r in prims[:4]:
        # ss[m] / ss[0] = F_m(T) / F_0(T); recover T from the records
        P_Q = (r["PA"] + sh[0][3]) - (r["QC"] + sh[2][3])
        rho = r["roz"] / (2.0 * r["oo2z"])
        T = rho * float(np.dot(P_Q, P_Q))
        F = np.asarray(oracle.boys(T, 5))
        got = r["ss"][:6] / r["ss"][0]
        assert np.allclose(got, F / F[0], rtol=1e-12, atol=0)


def _max_rank_worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    q.put((rank, bench.max_over_ranks(1.5 + rank, world, device="cpu")))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo_two_processes():
    # the N > 1 reduction of bench.py (slowest rank's time) on two gloo ranks
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_max_rank_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert got == [(0, 2.5), (1, 2.5)]
    import bench
    assert bench.max_over_ranks(3.25, 1) == 3.25


def test_reference_arm_other_ranks_exit_without_work(monkeypatch):
    # under torchrun only rank 0 times the CPU reference; the others exit 0
    import bench
    monkeypatch.setenv("RANK", "1")
    args = bench.argparse.Namespace(workload="h2o32_cc-pvdz", steps=1, warmup=1, gpus=2)
    assert bench.run_reference(args) == 0


def test_kernel_roofline_blends_peaks_for_fp64_boys_launch():
    # an FP32 launch of the mixed scheme does part of its work (the Boys
    # function and its argument) in FP64: its peak is the time at peak of
    # both shares
    import bench
    launches = [{"class": (1, 0, 1, 0), "fp32": 1, "kernel": "register", "ms_avg": 10.0,
                 "flops": 1.0e11, "flops_fp64": 1.0e9, "prim_quartets": 1, "quartets": 1}]
    peaks = {"fp64": 1.0, "fp32": 64.0}
    r = bench.kernel_roofline(launches, peaks, "w", "mixed")
    t_min = 1.0e9 / 1.0e12 + 0.99e11 / 64.0e12
    assert r["bound"] == "fp64+fp32 pipes"
    assert abs(r["peak"] - 1.0e11 / t_min / 1e12) < 1e-12
    assert abs(r["frac"] - (1.0e11 / 0.010 / 1e12) / r["peak"]) < 1e-12
