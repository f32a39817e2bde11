"""Benchmark of the GB300 Coulomb ERI path: screened ERIs/s of one J/K build
(one "step" = one Schwarz-screened J/K pass over all unique shell quartets
of a synthetic water cluster), FP64 and mixed FP32/FP64, on 1 GPU.

Prints ONE JSON line (rank 0).  `value` = mixed-precision ERIs/s with D, J,
K resident in HBM (device time of the whole pass from CUDA events on the
launching stream, L2 flushed between steps); `e2e` = the same metric
through the host-buffer API (lgx_jk: host D in, host J/K out, copies
timed); `fp64` = the plain FP64 path; `cpu_baseline` = the CPU oracle
(FP64 restatement of libint's algorithm) on a bounded sample of the same
screened quartet space, all host threads.

--impl reference times that CPU implementation alone (the reference libint
library cannot be built here, so its algorithm restated in C++ stands in).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (grid, basis, schwarz threshold, description)
    "h2o64_cc-pvtz": ((4, 4, 4), "cc-pVTZ", 1e-12, "(H2O)64 cc-pVTZ 4x4x4 grid, Schwarz 1e-12"),
    "h2o32_cc-pvdz": ((4, 4, 2), "cc-pVDZ", 1e-12, "(H2O)32 cc-pVDZ 4x4x2 grid, Schwarz 1e-12"),
    "h2o16_cc-pvdz": ((4, 2, 2), "cc-pVDZ", 1e-12, "(H2O)16 cc-pVDZ 4x2x2 grid, Schwarz 1e-12"),
    "h2o4_cc-pvdz": ((2, 2, 1), "cc-pVDZ", 0.0, "(H2O)4 cc-pVDZ 2x2x1 grid, no screening"),
    "h2o8_cc-pvtz": ((2, 2, 2), "cc-pVTZ", 1e-12, "(H2O)8 cc-pVTZ 2x2x2 grid, Schwarz 1e-12"),
}
MIXED_THRESH = 1e-4
SEED = 2024


def build_inputs(name):
    import libint_gb300 as lg
    grid, basis, thresh, desc = WORKLOADS[name]
    atoms = lg.water_cluster(*grid, spacing=3.0, jitter=0.2, seed=SEED)
    bs = lg.BasisSet(basis, atoms)
    nwater = grid[0] * grid[1] * grid[2]
    D = lg.random_density(bs.nbf, 5 * nwater, seed=SEED + 1)
    return atoms, bs, D, thresh, desc


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=5)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                mx = float(p[1])
            except ValueError:
                continue
            for n, v in zip(names, p[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measure_peaks(torch):
    """FP64 and FP32 (no TF32) CUDA-core peaks, measured live with cuBLAS
    DGEMM / SGEMM (best of a few 8192^3 products)."""
    out = {}
    torch.backends.cuda.matmul.allow_tf32 = False
    for name, dt, n in (("fp64", torch.float64, 8192), ("fp32", torch.float32, 8192)):
        a = torch.randn(n, n, device="cuda", dtype=dt)
        b = torch.randn(n, n, device="cuda", dtype=dt)
        torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 0.0
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
        out[name] = best
        del a, b
    torch.cuda.empty_cache()
    return out


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per launch of
# a class kernel in the timed pass, from an ncu launch list of this same
# bench command on the full workload (one-pass metrics; the summary and the
# command line are in profiles/launches_dram_jk_h2o32_cc-pvdz.md).  Keyed by
# (workload, pass precision mode, kernel).  The traffic does not grow with
# the primitive quartets (it is the cold read of the pair records, the
# density and the Boys table), so it is not scaled to other workloads.
NCU_TRAFFIC_BYTES = {
    ("h2o32_cc-pvdz", "mixed", "rk_kernel<double,0,0,1,0,J/K>"): 11.6e6,
    ("h2o32_cc-pvdz", "fp64", "rk_kernel<double,0,0,1,0,J/K>"): 29.9e6,
    ("h2o32_cc-pvdz", "mixed", "rk_kernel<double,0,0,0,0,J/K>"): 8.2e6,
    ("h2o32_cc-pvdz", "fp64", "rk_kernel<double,0,0,0,0,J/K>"): 19.1e6,
}


def kernel_name(r):
    t = "float" if r["fp32"] else "double"
    la, lb, lc, ld = r["class"]
    if r["kernel"] == "register":
        return "rk_kernel<%s,%d,%d,%d,%d,J/K>" % (t, la, lb, lc, ld)
    post = "generated post (%d%d|%d%d)" % (la, lb, lc, ld) if "generated" in r["kernel"] \
        else "interpreted post"
    return "eri_warp_kernel<%s,J/K,%s>" % (t, post)


def kernel_roofline(launches, peaks, workload, mode):
    """Roofline of the dominant class launch of a pass (largest average
    device time over the timed steps): its algorithmic FLOPs per launch over
    its average duration, against the FP64 or FP32 pipe peak measured live
    (cuBLAS DGEMM / SGEMM without TF32)."""
    if not launches:
        return None
    r = max(launches, key=lambda x: x["ms_avg"])
    total = sum(x["ms_avg"] for x in launches)
    pipe = "fp32" if r["fp32"] else "fp64"
    ach = r["flops"] / (r["ms_avg"] * 1e-3) / 1e12
    name = kernel_name(r)
    return {"bound": pipe + "-pipe", "kernel": name, "achieved": ach, "peak": peaks[pipe],
            "unit": "TFLOP/s", "frac": ach / peaks[pipe],
            "traffic": NCU_TRAFFIC_BYTES.get((workload, mode, name)),
            "launch_ms": r["ms_avg"], "share_of_pass": r["ms_avg"] / total if total else None,
            "flops_per_launch": r["flops"], "prim_quartets": r["prim_quartets"],
            "quartets": r["quartets"],
            "peak_source": "cuBLAS %s measured live in this run (MEASURED_PEAKS.json holds "
                           "only HBM and bf16 figures)" % ("SGEMM, no TF32" if r["fp32"]
                                                           else "DGEMM")}


def cpu_baseline(bs, D, Kq, thresh, budget_s, nthreads=0):
    """Oracle J/K over bounded samples of bra shell pairs spread across the
    canonical quartet enumeration; returns ERIs/s and the sample size."""
    from oracle import oracle
    ob = oracle.OracleBasis.from_basis(bs)
    ns = len(bs)
    npairs = ns * (ns + 1) // 2
    # chunks at 8 positions of the pair range, grown until the budget is used
    chunk = 1
    nint_tot, t_tot, npair_tot = 0, 0.0, 0
    positions = [int(npairs * f) for f in (0.05, 0.2, 0.35, 0.5, 0.65, 0.8, 0.9, 0.97)]
    while t_tot < budget_s and chunk < npairs:
        for p0 in positions:
            p1 = min(npairs, p0 + chunk)
            t0 = time.perf_counter()
            _, _, nq, nint = oracle.jk_sample(ob, D, Kq, thresh, p0, p1, nthreads)
            t_tot += time.perf_counter() - t0
            nint_tot += nint
            npair_tot += p1 - p0
        chunk *= 2
    return nint_tot / t_tot, nint_tot, t_tot, npair_tot


def run_reference(args):
    """--impl reference: the CPU implementation of the path (oracle port of
    libint's Engine + compute_2body_fock digestion), all host threads."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import libint_gb300 as lg
    from oracle import oracle
    oracle.build()
    atoms, bs, D, thresh, desc = build_inputs(args.workload)
    ctx = lg.Context(int(os.environ.get("LOCAL_RANK", "0")))
    ctx.set_basis(bs)
    Kq = ctx.schwarz()  # the screening list input, shared with the GPU arm
    ctx.close()
    cores = os.cpu_count()
    per_step = max(2.0, args.ref_budget / max(1, args.steps + args.warmup))
    vals = []
    for i in range(args.warmup + args.steps):
        v, nint, t, npair = cpu_baseline(bs, D, Kq, thresh, per_step)
        if i >= args.warmup:
            vals.append(v)
    value = float(np.mean(vals))
    line = {
        "impl": "reference", "metric": "screened ERIs/s per J/K build", "value": value,
        "unit": "ERI/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": desc, "basis": bs.name, "nbf": bs.nbf, "nshell": len(bs),
                   "schwarz_thresh": thresh},
        "cpu_baseline": {"value": value, "unit": "ERI/s", "cores": cores, "kind": "port",
                         "sample": "oracle J/K over bra-pair chunks at 8 positions of the "
                                   "canonical quartet enumeration, %.1f s per step" % per_step},
        "e2e": {"value": value, "unit": "ERI/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def max_over_ranks(value, world, device="cuda"):
    """The slowest rank's value: an all-reduce MAX over the process group
    when world > 1 (one process per GPU; the ranks' timed regions are
    bracketed by barriers), the value itself otherwise."""
    if world <= 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def run_gpu(args):
    import torch
    import libint_gb300 as lg
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    atoms, bs, D, thresh, desc = build_inputs(args.workload)
    nbf = bs.nbf
    ctx = lg.Context(local)
    ctx.set_basis(bs)
    dD = torch.tensor(D, device="cuda")
    dJ = torch.empty_like(dD)
    dK = torch.empty_like(dD)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    def timed(mode):
        for _ in range(args.warmup):
            ctx.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), thresh, mode, MIXED_THRESH)
        barrier()
        ms, last, launches = [], None, None
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            last = ctx.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), thresh, mode,
                                 MIXED_THRESH)
            ms.append(last.pass_ms)
            # per-launch device times of this step (events between launches,
            # recorded by the replayed pass graph itself)
            rec = ctx.last_pass_launches()
            if launches is None:
                launches = rec
                for r in launches:
                    r["ms_sum"] = r["ms"]
            else:
                for r, x in zip(launches, rec):
                    r["ms_sum"] += x["ms"]
        barrier()
        wall = time.perf_counter() - t0
        for r in launches or []:
            r["ms_avg"] = r.pop("ms_sum") / args.steps
        return ms, last, wall, launches

    peaks = measure_peaks(torch)
    with ClockSampler(local) as clk:
        ms64, st64, wall64, lau64 = timed(lg._lgx.LGX_FP64)
        J64, K64 = dJ.cpu().numpy(), dK.cpu().numpy()
        msmx, stmx, wallmx, laumx = timed(lg._lgx.LGX_MIXED)
        Jmx, Kmx = dJ.cpu().numpy(), dK.cpu().numpy()
    clocks = clk.summary()

    def agg(ms):
        return max_over_ranks(float(np.sum(ms)), world)

    t64 = agg(ms64) / 1e3
    tmx = agg(msmx) / 1e3
    v64 = world * st64.integrals * args.steps / t64
    vmx = world * stmx.integrals * args.steps / tmx
    e64 = lg.jk_energies(D, J64, K64)
    emx = lg.jk_energies(D, Jmx, Kmx)

    # e2e: host buffers through the public API, copies inside the timed region
    J_h = np.zeros((nbf, nbf)); K_h = np.zeros((nbf, nbf))
    for _ in range(max(1, args.warmup // 2)):
        ctx.jk(D, thresh, lg._lgx.LGX_MIXED, MIXED_THRESH)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        J_h, K_h, st_e = ctx.jk(D, thresh, lg._lgx.LGX_MIXED, MIXED_THRESH)
    barrier()
    te2e = time.perf_counter() - t0
    # remove the flush time, measured separately
    f0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
    te2e -= time.perf_counter() - f0
    te2e = max_over_ranks(te2e, world)
    ve2e = world * st_e.integrals * args.steps / te2e

    # roofline of the whole mixed pass: time at peak for its FP64 and FP32 work
    fl64, fl32 = stmx.flops_fp64, stmx.flops_fp32
    t_min = fl64 / (peaks["fp64"] * 1e12) + fl32 / (peaks["fp32"] * 1e12)
    t_step = tmx / args.steps
    achieved = (fl64 + fl32) / t_step / 1e12
    peak_blend = (fl64 + fl32) / t_min / 1e12
    roof64 = st64.flops_fp64 / (t64 / args.steps) / 1e12
    dom = kernel_roofline(laumx, peaks, args.workload, "mixed")
    dom64 = kernel_roofline(lau64, peaks, args.workload, "fp64")
    # the timed passes run class launches on parallel branches, so a launch
    # shares the GPU; one more mixed pass on a context without branches
    # gives each kernel's time on its own (the ncu launch list is serial too)
    os.environ["LGX_OVERLAP"] = "0"
    ser = lg.Context(local)
    del os.environ["LGX_OVERLAP"]
    ser.set_basis(bs)
    for _ in range(2):
        ser.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), thresh, lg._lgx.LGX_MIXED,
                      MIXED_THRESH)
    flush.zero_()
    torch.cuda.synchronize()
    ser.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), thresh, lg._lgx.LGX_MIXED,
                  MIXED_THRESH)
    lau_ser = ser.last_pass_launches()
    for r in lau_ser:
        r["ms_avg"] = r["ms"]
    dom_ser = kernel_roofline(lau_ser, peaks, args.workload, "mixed")
    dom64_ser = None
    if t64 / args.steps < 5.0:  # the FP64 pass too, when it is short
        ser.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), thresh, lg._lgx.LGX_FP64,
                      MIXED_THRESH)
        flush.zero_()
        torch.cuda.synchronize()
        ser.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), thresh, lg._lgx.LGX_FP64,
                      MIXED_THRESH)
        l64 = ser.last_pass_launches()
        for r in l64:
            r["ms_avg"] = r["ms"]
        dom64_ser = kernel_roofline(l64, peaks, args.workload, "fp64")
    ser.close()
    for r in (dom, dom64):
        if r:
            r["note"] = ("launch times inside the timed passes, whose class launches run "
                         "concurrently on parallel branches")
    for r in (dom_ser, dom64_ser):
        if r:
            r["note"] = ("dominant class launch of one extra pass with serial launches, "
                         "so that its time is its own (CUDA events on its stream)")

    if rank != 0:
        return 0
    cpu = None
    if not args.no_cpu:
        Kq = ctx.schwarz()
        v, nint, t, npair = cpu_baseline(bs, D, Kq, thresh, args.cpu_budget)
        cpu = {"value": v, "unit": "ERI/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "%d integrals from %d bra shell pairs at 8 positions of the "
                         "screened quartet enumeration, %.1f s" % (nint, npair, t)}
    line = {
        "metric": "screened ERIs/s per J/K build",
        "value": vmx, "unit": "ERI/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": tmx / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64 (mixed)", "data": "synthetic",
        "config": {"workload": desc, "basis": bs.name, "nbf": nbf, "nshell": len(bs),
                   "schwarz_thresh": thresh, "mixed_thresh": MIXED_THRESH,
                   "l2": "flushed between steps (256 MiB write)",
                   "quartets_fp64": stmx.quartets_fp64, "quartets_fp32": stmx.quartets_fp32,
                   "integrals_per_step": stmx.integrals,
                   "prim_quartets_per_step": stmx.prim_quartets},
        "fp64": {"value": v64, "unit": "ERI/s", "ms_per_step": t64 / args.steps * 1e3,
                 "quartets": st64.quartets_fp64, "E_J": e64[0], "E_K": e64[1],
                 "roofline": dom64_ser or dom64,
                 "roofline_concurrent": dom64,
                 "roofline_pass": {"bound": "fp64-pipe", "achieved": roof64,
                                   "peak": peaks["fp64"], "unit": "TFLOP/s",
                                   "frac": roof64 / peaks["fp64"]}},
        "mixed_error": {"dE_J": abs(emx[0] - e64[0]), "dE_K": abs(emx[1] - e64[1]),
                        "max_abs_dJ": float(np.max(np.abs(Jmx - J64))),
                        "max_abs_dK": float(np.max(np.abs(Kmx - K64)))},
        "speedup_mixed_vs_fp64": vmx / v64,
        "roofline": dom_ser,
        "roofline_concurrent": dom,
        "roofline_pass": {"bound": "fp64+fp32 pipes", "achieved": achieved, "peak": peak_blend,
                          "unit": "TFLOP/s", "frac": achieved / peak_blend,
                          "peak_source": "cuBLAS DGEMM %.2f / SGEMM(no TF32) %.1f TFLOP/s "
                                         "measured live; blended by the pass's FP64/FP32 work"
                                         % (peaks["fp64"], peaks["fp32"]),
                          "flops_fp64": fl64, "flops_fp32": fl32},
        "e2e": {"value": ve2e, "unit": "ERI/s", "h2d_bytes_per_step": nbf * nbf * 8,
                "d2h_bytes_per_step": 2 * nbf * nbf * 8},
        "gpu_launches": int(stmx.launches) * args.steps + int(st64.launches) * args.steps,
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    ctx.close()
    return 0


def _prim_inputs(rng, ls, depth, deriv, dtype):
    """Caller-side Libint_t prefactors of random raw shells (what a libint
    caller computes before libint2_build_eri*), Boys values from scipy."""
    from scipy.special import gamma, gammainc
    sh = []
    for l in ls:
        a = np.sort(rng.uniform(0.3, 3.0, depth))[::-1].copy()
        sh.append((l, a, rng.uniform(0.4, 1.2, depth), rng.uniform(-1.2, 1.2, 3)))
    (_, a1s, c1s, A), (_, a2s, c2s, B), (_, a3s, c3s, C), (_, a4s, c4s, D) = sh
    mmax = sum(ls) + deriv
    m = np.arange(mmax + 1) + 0.5
    recs = []
    for a1, c1 in zip(a1s, c1s):
        for a2, c2 in zip(a2s, c2s):
            for a3, c3 in zip(a3s, c3s):
                for a4, c4 in zip(a4s, c4s):
                    z, e = a1 + a2, a3 + a4
                    P, Q = (a1 * A + a2 * B) / z, (a3 * C + a4 * D) / e
                    rho = z * e / (z + e)
                    W = (z * P + e * Q) / (z + e)
                    T = rho * np.dot(P - Q, P - Q)
                    F = (gammainc(m, T) * gamma(m) / (2 * T ** m) if T > 1e-12
                         else 1.0 / (2 * m))
                    pfac = (2 * np.pi ** 2.5 * np.exp(-a1 * a2 / z * np.dot(A - B, A - B))
                            * np.exp(-a3 * a4 / e * np.dot(C - D, C - D))
                            / (z * e * np.sqrt(z + e)) * c1 * c2 * c3 * c4)
                    r = np.zeros((), dtype)
                    r["PA"], r["QC"], r["WP"], r["WQ"] = P - A, Q - C, W - P, W - Q
                    r["oo2z"], r["oo2e"], r["oo2ze"] = 0.5 / z, 0.5 / e, 0.5 / (z + e)
                    r["roz"], r["roe"] = rho / z, rho / e
                    r["two_alpha"] = [2 * a1, 2 * a2, 2 * a3, 2 * a4]
                    ss = np.zeros(dtype["ss"].shape)
                    ss[:mmax + 1] = pfac * F
                    r["ss"] = ss
                    recs.append(r)
    return sh, np.array(recs, dtype=dtype), A - B, C - D


def run_primitive_api(args):
    """--primitive-api: latency of the generated-library entry
    (lgx_compute_primitive_set, behind libint2_build_eri*): one synchronous
    call per contracted shell set, host records in, host sets out, through
    the Python binding; the oracle's contracted quartet of the same shells
    (one host thread) beside it."""
    import libint_gb300 as lg
    from oracle import oracle
    oracle.build()
    ctx = lg.Context(int(os.environ.get("LOCAL_RANK", "0")))
    rng = np.random.default_rng(2024)
    rows = []
    for ls, depth, deriv in (((1, 1, 1, 1), 3, 0), ((2, 2, 2, 2), 1, 0), ((3, 3, 3, 3), 1, 0),
                             ((2, 1, 2, 1), 2, 1), ((1, 1, 1, 1), 1, 2)):
        sh, prims, AB, CD = _prim_inputs(rng, ls, depth, deriv, lg._lgx.PRIM_DTYPE)
        n = 200
        for _ in range(5):
            ctx.compute_primitive_set(ls, prims, AB, CD, deriv)
        t0 = time.perf_counter()
        for _ in range(n):
            out = ctx.compute_primitive_set(ls, prims, AB, CD, deriv)
        t_gpu = (time.perf_counter() - t0) / n
        ob = oracle.OracleBasis(np.array(ls, np.int32), np.zeros(4, np.int32),
                                np.full(4, depth, np.int32), np.concatenate([s[3] for s in sh]),
                                np.concatenate([s[1] for s in sh]),
                                np.concatenate([s[2] for s in sh]))
        t0 = time.perf_counter()
        for _ in range(n):
            oracle.compute_quartet(ob, 0, 1, 2, 3, deriv=deriv, precision=0.0)
        t_cpu = (time.perf_counter() - t0) / n
        nint = sum(x.size for x in out)
        rows.append({"class": "(%d%d|%d%d)" % ls, "deriv": deriv, "prim_quartets": len(prims),
                     "integrals": nint, "us_per_call": 1e6 * t_gpu,
                     "eri_per_s": nint / t_gpu, "oracle_us_per_call": 1e6 * t_cpu})
    ctx.close()
    print(json.dumps({"metric": "generated-library entry latency (libint2_build_eri*)",
                      "unit": "us/call", "data": "synthetic", "calls": 200,
                      "note": "synchronous: host records -> GPU -> host sets, Python binding",
                      "classes": rows}))
    return 0


def run_rows(args):
    """--rows: the widened rows of the path, each timed end to end through
    the public API on the GPU with the oracle beside it on the host cores:
    density-fitting tensors (BraKet xs_xx / xs_xs through lgx_compute_batch),
    second-derivative shell sets (deriv_order 2, per call) and a
    range-separated J/K pass (erfc, omega = 0.4)."""
    import torch
    import libint_gb300 as lg
    from oracle import oracle
    oracle.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    rows = {}
    cores = os.cpu_count()

    # density fitting: (P|ab) and (P|Q) of (H2O)8 cc-pVDZ / cc-pVDZ-jkfit
    atoms = lg.water_cluster(2, 2, 2, spacing=3.0, jitter=0.2, seed=SEED)
    obs = lg.BasisSet("cc-pVDZ", atoms)
    dfbs = lg.BasisSet("cc-pVDZ-jkfit", atoms)
    full = lg.BasisSet(list(obs) + list(dfbs) + [lg.Shell.unit()])
    full.atom_of_shell = obs.atom_of_shell + dfbs.atom_of_shell + [0]
    ns, na, u = len(obs), len(dfbs), len(obs) + len(dfbs)
    a, b = np.tril_indices(ns)
    P = np.arange(ns, ns + na)
    q3 = np.stack(np.broadcast_arrays(P[:, None], u, a[None, :], b[None, :]), -1).reshape(-1, 4)
    r1, r2 = np.tril_indices(na)
    q2 = np.stack([P[r1], np.full_like(r1, u), P[r2], np.full_like(r1, u)], -1)
    q = np.ascontiguousarray(np.concatenate([q3, q2]), np.int32)
    ctx = lg.Context(local)
    ctx.set_basis(full)
    ctx.compute_batch(q)
    torch.cuda.synchronize()
    reps = 5
    t0 = time.perf_counter()
    for _ in range(reps):
        out, offs, _ = ctx.compute_batch(q)
    t_gpu = (time.perf_counter() - t0) / reps
    sz = np.array([sh.size() for sh in full], np.int64)
    nint = int((sz[q[:, 0]] * sz[q[:, 2]] * sz[q[:, 3]]).sum())
    # the same tensors left in HBM (lgx_compute_batch_device)
    dout = torch.empty(int(offs[-1]) + nint, dtype=torch.float64, device="cuda")
    ctx.compute_batch_device(q, dout.data_ptr(), dout.numel(), offsets=offs)
    t0 = time.perf_counter()
    for _ in range(reps):
        ctx.compute_batch_device(q, dout.data_ptr(), dout.numel(), offsets=offs)
    t_dev = (time.perf_counter() - t0) / reps
    ob = oracle.OracleBasis.from_basis(full)
    t0 = time.perf_counter()
    oracle.compute_batch(ob, q, offs, int(offs[-1] + nint), nthreads=0)
    t_cpu = time.perf_counter() - t0
    rows["f2_df_tensors"] = {
        "workload": "(H2O)8 cc-pVDZ / cc-pVDZ-jkfit: every (P|ab) and (P|Q)",
        "quartets": len(q), "integrals": nint, "ms": 1e3 * t_gpu, "eri_per_s": nint / t_gpu,
        "device_ms": 1e3 * t_dev, "device_eri_per_s": nint / t_dev,
        "oracle_ms": 1e3 * t_cpu, "oracle_eri_per_s": nint / t_cpu, "oracle_cores": cores,
        "note": "lgx_compute_batch, FP64: ms with the host output buffer (copy timed), "
                "device_ms with the tensors left in HBM (lgx_compute_batch_device); "
                "oracle output in host memory"}
    ctx.close()

    # second derivatives: per-call shell sets through the Engine entry
    rng = np.random.default_rng(SEED)
    d2 = []
    ctx = lg.Context(local)
    for ls in ((1, 1, 1, 1), (2, 1, 2, 0), (2, 2, 2, 2), (3, 2, 1, 0)):
        sh = [lg.Shell(l, [(float(x), 1.0) for x in np.sort(rng.uniform(0.3, 3.0, 2))[::-1]],
                       tuple(rng.uniform(-1.2, 1.2, 3)), pure=l >= 2) for l in ls]
        for _ in range(3):
            ctx.compute_shellset(sh, deriv=2)
        n = 50
        t0 = time.perf_counter()
        for _ in range(n):
            r = ctx.compute_shellset(sh, deriv=2)
        tg = (time.perf_counter() - t0) / n
        ob = oracle.OracleBasis.from_basis(lg.BasisSet(sh))
        t0 = time.perf_counter()
        for _ in range(n):
            oracle.compute_quartet(ob, 0, 1, 2, 3, deriv=2)
        tc = (time.perf_counter() - t0) / n
        nint = sum(x.size for x in r)
        d2.append({"class": "(%d%d|%d%d)" % ls, "integrals": nint, "us_per_call": 1e6 * tg,
                   "oracle_us_per_call": 1e6 * tc})
    rows["f3_deriv2_shellsets"] = {"classes": d2, "note": "78 sets per call, 2 primitives per "
                                   "shell, pure d/f; oracle on one host core"}
    ctx.close()

    # range-separated J/K: erfc(0.4 r)/r pass vs the Coulomb pass, (H2O)16 cc-pVDZ
    atoms, bs, D, thresh, _ = build_inputs("h2o16_cc-pvdz")
    peaks = measure_peaks(torch)
    res = {}
    for name, op in (("coulomb", lg.Operator.coulomb), ("erfc", lg.Operator.erfc_coulomb)):
        ctx = lg.Context(local)
        ctx.set_basis(bs)
        ctx.set_operator(op, 0.4)
        dD = torch.tensor(D, device="cuda")
        dJ, dK = torch.empty_like(dD), torch.empty_like(dD)
        for _ in range(2):
            ctx.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), thresh, lg._lgx.LGX_FP64)
        ms = []
        for _ in range(3):
            st = ctx.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), thresh,
                               lg._lgx.LGX_FP64)
            ms.append(st.pass_ms)
        launches = ctx.last_pass_launches()
        for r in launches:
            r["ms_avg"] = r["ms"]
        roof = kernel_roofline(launches, peaks, "h2o16_cc-pvdz", "fp64")
        if roof:
            roof["note"] = ("dominant class launch of the last pass (concurrent branches: its "
                            "time includes sharing the GPU); FLOPs counted as for the Coulomb "
                            "operator (the attenuation's second Boys evaluation not included)")
        Kq = ctx.schwarz()
        oracle.set_operator(oracle.OP_ERFC_COULOMB if name == "erfc" else oracle.OP_COULOMB, 0.4)
        v, nsamp, tsamp, npair = cpu_baseline(bs, D, Kq, thresh, 8.0)
        res[name] = {"pass_ms": statistics.median(ms), "integrals": int(st.integrals),
                     "eri_per_s": st.integrals / (statistics.median(ms) * 1e-3),
                     "roofline_pass": {"bound": "fp64-pipe", "unit": "TFLOP/s",
                                       "achieved": st.flops_fp64 / (st.pass_ms * 1e-3) / 1e12,
                                       "peak": peaks["fp64"],
                                       "frac": st.flops_fp64 / (st.pass_ms * 1e-3) / 1e12
                                       / peaks["fp64"]},
                     "roofline": roof,
                     "oracle_eri_per_s": v, "oracle_sample_integrals": int(nsamp)}
        ctx.close()
    oracle.set_operator(oracle.OP_COULOMB, 0.0)
    rows["f4_erfc_jk"] = dict(res, workload="(H2O)16 cc-pVDZ, Schwarz 1e-12, FP64, omega 0.4",
                             note="device-resident D/J/K, pass time from CUDA events; oracle "
                                  "on a bounded sample of bra pairs, all host threads")
    print(json.dumps({"metric": "widened rows: GPU vs oracle", "data": "synthetic",
                      "cores": cores, "rows": rows}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="lgx", choices=["lgx", "reference"])
    ap.add_argument("--workload", default="h2o32_cc-pvdz", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--ref-budget", type=float, default=60.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--primitive-api", action="store_true",
                    help="time the generated-library entry (libint2_build_eri*) instead")
    ap.add_argument("--rows", action="store_true",
                    help="time the widened rows (DF tensors, deriv 2, erfc J/K) instead")
    args = ap.parse_args()
    if args.primitive_api:
        return run_primitive_api(args)
    if args.rows:
        return run_rows(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
