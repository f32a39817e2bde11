"""Benchmark of the GB300 Coulomb ERI path: screened ERIs/s of one J/K build
(one "step" = one Schwarz-screened J/K pass over all unique shell quartets
of a synthetic water cluster), FP64 and mixed FP32/FP64, on 1 GPU.

Default workload: (H2O)64 / cc-pVTZ on a 4x4x4 grid, Schwarz 1e-12 (3712
basis functions, 1.95e10 screened quartets, 5.4e11 integrals per pass).

Prints ONE JSON line (rank 0).  `value` = mixed-precision ERIs/s with D, J,
K resident in HBM (device time of the whole pass from CUDA events on the
launching stream, L2 flushed between steps, over --steps passes); `e2e` =
the same metric through the host-buffer API (lgx_jk: host D in, host J/K
out, copies inside each step's timed interval, the L2 flush outside it);
`fp64` = the plain FP64 path over its own, smaller step count
(--fp64-steps); `cpu_baseline` = the CPU oracle (FP64 restatement of
libint's Engine and of compute_2body_fock's digestion) on a fixed sample
of the same screened pass, all host threads.

--impl reference times that CPU implementation alone, built from the
oracle's own inputs (its G94 reader, cluster construction and Schwarz
factors), so it loads no part of the GPU library.  The reference libint
library itself cannot be built here (its generated integral code needs
Boost.MPL and GMP, its Engine Eigen), so its algorithm restated in C++
stands in for it.
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
    "h2o16_cc-pvtz": ((4, 2, 2), "cc-pVTZ", 1e-12, "(H2O)16 cc-pVTZ 4x2x2 grid, Schwarz 1e-12"),
}
DEFAULT_WORKLOAD = "h2o64_cc-pvtz"
MIXED_THRESH = 1e-4
SEED = 2024
# CPU sample: this many bra shell pairs (a fixed, seeded, class-stratified
# draw from the significant pairs), whatever the time budget or core count
CPU_SAMPLE_PAIRS = 1024
# pair subset of the oracle comparison of the full J/K kernels
CHECK_SUBSET_PAIRS = 3000


def build_inputs(name):
    """GPU arm: atoms, basis (the product's loader), density."""
    import libint_gb300 as lg
    grid, basis, thresh, desc = WORKLOADS[name]
    atoms = lg.water_cluster(*grid, spacing=3.0, jitter=0.2, seed=SEED)
    bs = lg.BasisSet(basis, atoms)
    nwater = grid[0] * grid[1] * grid[2]
    D = lg.random_density(bs.nbf, 5 * nwater, seed=SEED + 1)
    return atoms, bs, D, thresh, desc


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


class CpuArm:
    """The CPU implementation of the path (the oracle: libint's Engine
    algorithm and compute_2body_fock's digestion restated in C++, OpenMP over
    bra shell pairs) on the workload, with inputs from the oracle's own
    loaders and its own Schwarz factors (compute_schwarz_ints,
    hartree-fock++.cc:1231-1298), so nothing of the GPU library is loaded.

    A step is the fixed sample of CPU_SAMPLE_PAIRS bra shell pairs with all
    their kets of the screened pass; ERIs/s = the sample's integrals over its
    time, which estimates the full pass's rate (every significant pair is
    drawn with the same probability, stratified by pair class).  The full
    pass's time is extrapolated from the sample plus the one reduction of
    the per-thread accumulators that a full pass makes."""

    def __init__(self, workload, nthreads=0, npairs=CPU_SAMPLE_PAIRS):
        from oracle import inputs, oracle
        oracle.build()
        self.oracle = oracle
        grid, basis, self.thresh, self.desc = WORKLOADS[workload]
        atoms = inputs.water_cluster(*grid, spacing=3.0, jitter=0.2, seed=SEED)
        self.ob = inputs.load_basis(basis, atoms)
        self.basis_name = basis
        nwater = grid[0] * grid[1] * grid[2]
        self.D = inputs.random_density(self.ob.nbf, 5 * nwater, seed=SEED + 1)
        self.nthreads = nthreads or cpu_threads()
        t0 = time.perf_counter()
        self.K = oracle.schwarz(self.ob, self.nthreads)
        self.t_schwarz = time.perf_counter() - t0
        self.total_quartets, self.total_integrals = oracle.count_screened(self.ob, self.K,
                                                                          self.thresh)
        self.pairs = sample_pairs(self.ob, self.K, self.thresh, npairs, SEED + 7)
        self.acc = oracle.JKAccumulator(self.ob.nbf, self.nthreads)

    def step(self):
        t0 = time.perf_counter()
        nq, nint = self.acc.add_pairs(self.ob, self.D, self.K, self.thresh, self.pairs)
        return nint, time.perf_counter() - t0

    def reduce_seconds(self):
        t0 = time.perf_counter()
        self.acc.reduce()
        return time.perf_counter() - t0

    def describe(self, nint, seconds):
        return ("%d bra shell pairs (seeded draw of the significant pairs, stratified by pair "
                "class), all their kets: %d integrals, %.1f s per step; the full pass has %d "
                "integrals" % (len(self.pairs), nint, seconds, self.total_integrals))

    def close(self):
        self.acc.close()


def sample_pairs(ob, K, thresh, npairs, seed):
    """A fixed draw of bra shell pairs (canonical indices s1 (s1+1)/2 + s2)
    among the significant ones (K12 max K >= thresh), stratified by pair
    class (l1, l2) in proportion to the class sizes."""
    ns = ob.nshell
    s1, s2 = np.tril_indices(ns)
    kp = K[s1, s2]
    sig = kp * K.max() >= thresh
    l = ob.l
    cls = np.maximum(l[s1], l[s2]) * 8 + np.minimum(l[s1], l[s2])
    idx = s1.astype(np.int64) * (s1 + 1) // 2 + s2
    rng = np.random.default_rng(seed)
    n_sig = int(sig.sum())
    take = []
    for c in np.unique(cls[sig]):
        members = idx[sig & (cls == c)]
        k = max(1, int(round(npairs * len(members) / n_sig)))
        take.append(rng.choice(members, min(k, len(members)), replace=False))
    return np.sort(np.concatenate(take))


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


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of one launch
# of the dominant class kernel, from a one-pass ncu capture of that launch
# in this benchmark's workload (the command and figures are in the profiles/
# summary named beside each entry).  Not measured in the run that prints it.
NCU_TRAFFIC = {
    # (workload, pass mode, kernel): (bytes per launch, profiles/ summary)
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
    device time): its algorithmic FLOPs per launch (the class's operation
    counts from the equations, see lgx_api.cu prologue_flops) over its
    average duration, against the FP64 or FP32 pipe peak measured live
    (cuBLAS DGEMM / SGEMM without TF32)."""
    if not launches:
        return None
    r = max(launches, key=lambda x: x["ms_avg"])
    total = sum(x["ms_avg"] for x in launches)
    pipe = "fp32" if r["fp32"] else "fp64"
    ach = r["flops"] / (r["ms_avg"] * 1e-3) / 1e12
    name = kernel_name(r)
    f64 = r.get("flops_fp64", 0.0 if r["fp32"] else r["flops"])
    peak = peaks[pipe]
    bound = pipe + "-pipe"
    if r["fp32"] and f64 > 0:
        # FP32 launch of the mixed scheme with its Boys function in FP64: the
        # time at peak is the FP64 share at the FP64 peak plus the rest at
        # the FP32 peak
        peak = r["flops"] / (f64 / peaks["fp64"] + (r["flops"] - f64) / peaks["fp32"])
        bound = "fp64+fp32 pipes"
    tr = NCU_TRAFFIC.get((workload, mode, name))
    out = {"bound": bound, "kernel": name, "achieved": ach, "peak": peak,
           "unit": "TFLOP/s", "frac": ach / peak, "flops_fp64_per_launch": f64,
           "traffic": tr[0] if tr else None,
           "launch_ms": r["ms_avg"], "share_of_pass": r["ms_avg"] / total if total else None,
           "flops_per_launch": r["flops"], "prim_quartets": r["prim_quartets"],
           "quartets": r["quartets"],
           "peak_source": "cuBLAS %s measured live in this run (MEASURED_PEAKS.json holds "
                          "no FP64/FP32 CUDA-core figure)" % (
                              "DGEMM %.2f / SGEMM (no TF32) %.1f TFLOP/s, blended by the "
                              "launch's FP64 / FP32 operations" % (peaks["fp64"], peaks["fp32"])
                              if bound.startswith("fp64+") else
                              ("SGEMM, no TF32" if r["fp32"] else "DGEMM"))}
    if tr:
        out["traffic_source"] = "ncu capture of this workload's launch, not this run: " + tr[1]
    return out


def run_reference(args):
    """--impl reference: the CPU implementation of the path (oracle port of
    libint's Engine + compute_2body_fock digestion) on all host threads,
    rank 0 only; each step is the same fixed sample of the screened pass."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    arm = CpuArm(args.workload)
    per = []
    for i in range(args.warmup + args.steps):
        nint, t = arm.step()
        if i >= args.warmup:
            per.append((nint, t))
    t_red = arm.reduce_seconds()
    nint = per[0][0]
    tsum = sum(t for _, t in per)
    value = nint * len(per) / tsum
    t_step = tsum / len(per)
    full_s = t_step * arm.total_integrals / nint + t_red
    line = {
        "impl": "reference", "metric": "screened ERIs/s per J/K build", "value": value,
        "unit": "ERI/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": arm.desc, "basis": arm.basis_name, "nbf": arm.ob.nbf,
                   "nshell": arm.ob.nshell, "schwarz_thresh": arm.thresh,
                   "integrals_per_pass": arm.total_integrals,
                   "quartets_per_pass": arm.total_quartets},
        "cpu_baseline": {"value": value, "unit": "ERI/s", "cores": arm.nthreads, "kind": "port",
                         "sample": arm.describe(nint, t_step),
                         "full_pass_s_extrapolated": full_s,
                         "schwarz_s": arm.t_schwarz},
        "e2e": {"value": value, "unit": "ERI/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    arm.close()
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


def oracle_subset_check(lg, bs, D, thresh, local, modes, npairs=CHECK_SUBSET_PAIRS):
    """J/K of the GPU pass restricted to a pair subset (lgx_set_pair_subset:
    every quartet whose bra and ket pairs are both in the subset) against the
    oracle's J/K over the same quartets: energy and element errors per
    precision mode, with the oracle as the FP64 reference."""
    import torch
    from oracle import oracle
    ob = oracle.OracleBasis.from_basis(bs)
    K = oracle.schwarz(ob, cpu_threads())
    pairs = sample_pairs(ob, K, thresh, npairs, SEED + 11)
    acc = oracle.JKAccumulator(ob.nbf, cpu_threads())
    nq, nint = acc.add_pairs(ob, D, K, thresh, pairs, ket_subset=True)
    Jo, Ko = acc.reduce()
    acc.close()
    EJo, EKo = lg.jk_energies(D, Jo, Ko)
    s1 = (np.sqrt(8.0 * pairs + 1) - 1).astype(np.int64) // 2
    s1 = np.where(s1 * (s1 + 1) // 2 > pairs, s1 - 1, s1)
    s1 = np.where((s1 + 1) * (s1 + 2) // 2 <= pairs, s1 + 1, s1)
    s2 = pairs - s1 * (s1 + 1) // 2
    os.environ["LGX_TUNE"] = "0"
    ctx = lg.Context(local)
    del os.environ["LGX_TUNE"]
    ctx.set_basis(bs)
    ctx.set_pair_subset(np.stack([s1, s2], 1))
    dD = torch.tensor(D, device="cuda")
    dJ, dK = torch.empty_like(dD), torch.empty_like(dD)
    out = {"pairs": int(len(pairs)), "quartets": int(nq), "integrals": int(nint),
           "E_J_oracle": EJo, "E_K_oracle": EKo}
    for name, mode in modes:
        st = ctx.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), thresh, mode,
                           MIXED_THRESH)
        J, Kx = dJ.cpu().numpy(), dK.cpu().numpy()
        EJ, EK = lg.jk_energies(D, J, Kx)
        out[name] = {"dE_J": abs(EJ - EJo), "dE_K": abs(EK - EKo),
                     "max_abs_dJ": float(np.max(np.abs(J - Jo))),
                     "max_abs_dK": float(np.max(np.abs(Kx - Ko))),
                     "gpu_quartets": int(st.quartets_fp64 + st.quartets_fp32)}
    ctx.close()
    return out


def mixed_integral_error(lg, bs, thresh, local, modes, n=20000):
    """Maximum integral error of each mixed mode against the FP64 oracle on
    quartets sampled from the FP32 space of the screened pass (thresh <=
    K12 K34 < MIXED_THRESH), through the batched entry, which runs the same
    FP32 kernel family as the J/K pass in store mode."""
    from oracle import oracle
    ob = oracle.OracleBasis.from_basis(bs)
    K = oracle.schwarz(ob, cpu_threads())
    ns = ob.nshell
    a, b = np.tril_indices(ns)
    kp = K[a, b]
    sig = kp * K.max() >= thresh
    a, b, kp = a[sig], b[sig], kp[sig]
    rng = np.random.default_rng(SEED + 13)
    got = []
    for _ in range(50):
        i = rng.integers(0, len(a), 20 * n)
        j = rng.integers(0, len(a), 20 * n)
        w = kp[i] * kp[j]
        ok = (w >= thresh) & (w < MIXED_THRESH)
        got.append(np.stack([i[ok], j[ok]], 1))
        if sum(len(g) for g in got) >= n:
            break
    p = np.concatenate(got)[:n]
    q = np.stack([a[p[:, 0]], b[p[:, 0]], a[p[:, 1]], b[p[:, 1]]], 1).astype(np.int32)
    ctx = lg.Context(local)
    ctx.set_basis(bs)
    out = {"quartets": int(len(q)), "integrals": None}
    ref = None
    for name, mode in modes:
        v, offs, _ = ctx.compute_batch(q, mode=mode, mixed_thresh=MIXED_THRESH)
        if ref is None:
            ref, _ = oracle.compute_batch(ob, q, offs, len(v), nthreads=cpu_threads())
            out["integrals"] = int(len(v))
            out["max_abs_integral"] = float(np.max(np.abs(ref)))
        out[name] = float(np.max(np.abs(v - ref)))
    ctx.close()
    return out


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

    def timed(mode, warmup, steps):
        for _ in range(warmup):
            ctx.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), thresh, mode, MIXED_THRESH)
        barrier()
        ms, last, launches = [], None, None
        for _ in range(steps):
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
        for r in launches or []:
            r["ms_avg"] = r.pop("ms_sum") / steps
        return ms, last, launches

    peaks = measure_peaks(torch)
    with ClockSampler(local) as clk:
        ms64, st64, lau64 = timed(lg._lgx.LGX_FP64, args.fp64_warmup, args.fp64_steps)
        J64, K64 = dJ.cpu().numpy(), dK.cpu().numpy()
        msmx, stmx, laumx = timed(lg._lgx.LGX_MIXED, args.warmup, args.steps)
        Jmx, Kmx = dJ.cpu().numpy(), dK.cpu().numpy()
        # the faster, less exact variant (Boys function of the FP32 quartets
        # in FP32 too), over its own step count
        msfb, stfb, laufb = timed(lg._lgx.LGX_MIXED_FP32_BOYS, 1, args.alt_steps)
        Jfb, Kfb = dJ.cpu().numpy(), dK.cpu().numpy()

        # e2e: host buffers through the public API (lgx_jk: D copied in, the
        # pass, J and K copied out); each step's interval brackets that call
        # alone, the L2 flush before it stays outside
        for _ in range(1):
            ctx.jk(D, thresh, lg._lgx.LGX_MIXED, MIXED_THRESH)
        barrier()
        te2e = 0.0
        dev_e2e = 0.0  # device time of the same passes (CUDA events)
        for _ in range(args.e2e_steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            J_h, K_h, st_e = ctx.jk(D, thresh, lg._lgx.LGX_MIXED, MIXED_THRESH)
            te2e += time.perf_counter() - t0
            dev_e2e += st_e.pass_ms * 1e-3
        barrier()
    clocks = clk.summary()

    def agg(ms):
        return max_over_ranks(float(np.sum(ms)), world)

    t64 = agg(ms64) / 1e3
    tmx = agg(msmx) / 1e3
    te2e = max_over_ranks(te2e, world)
    v64 = world * st64.integrals * args.fp64_steps / t64
    vmx = world * stmx.integrals * args.steps / tmx
    tfb = agg(msfb) / 1e3
    vfb = world * stfb.integrals * args.alt_steps / tfb
    efb = lg.jk_energies(D, Jfb, Kfb)
    ve2e = world * st_e.integrals * args.e2e_steps / te2e
    e64 = lg.jk_energies(D, J64, K64)
    emx = lg.jk_energies(D, Jmx, Kmx)

    # roofline of the whole mixed pass: time at peak for its FP64 and FP32 work
    fl64, fl32 = stmx.flops_fp64, stmx.flops_fp32
    t_min = fl64 / (peaks["fp64"] * 1e12) + fl32 / (peaks["fp32"] * 1e12)
    t_step = tmx / args.steps
    achieved = (fl64 + fl32) / t_step / 1e12
    peak_blend = (fl64 + fl32) / t_min / 1e12
    roof64 = st64.flops_fp64 / (t64 / args.fp64_steps) / 1e12
    dom = kernel_roofline(laumx, peaks, args.workload, "mixed")
    dom64 = kernel_roofline(lau64, peaks, args.workload, "fp64")
    # the timed passes run class launches on parallel branches, so a launch
    # shares the GPU; one more mixed pass on a context without branches
    # gives each kernel's time on its own (the ncu launch list is serial too)
    os.environ["LGX_OVERLAP"] = "0"
    ser = lg.Context(local)
    del os.environ["LGX_OVERLAP"]
    ser.set_basis(bs)
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
    if t64 / args.fp64_steps < 5.0:  # the FP64 pass too, when it is short
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
    subset = None
    if not args.no_check:
        subset = oracle_subset_check(lg, bs, D, thresh, local,
                                     (("fp64", lg._lgx.LGX_FP64), ("mixed", lg._lgx.LGX_MIXED),
                                      ("mixed_fp32_boys", lg._lgx.LGX_MIXED_FP32_BOYS)))
        ierr = mixed_integral_error(lg, bs, thresh, local,
                                    (("mixed", lg._lgx.LGX_MIXED),
                                     ("mixed_fp32_boys", lg._lgx.LGX_MIXED_FP32_BOYS)))
    else:
        ierr = None
    cpu = None
    if not args.no_cpu:
        arm = CpuArm(args.workload)
        arm.step()  # first touch of the sample's code and data
        nint, tc = arm.step()
        t_red = arm.reduce_seconds()
        cpu = {"value": nint / tc, "unit": "ERI/s", "cores": arm.nthreads, "kind": "port",
               "sample": arm.describe(nint, tc),
               "full_pass_s_extrapolated": tc * arm.total_integrals / nint + t_red}
        arm.close()
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
        "quartets_per_s": world * float(stmx.quartets_fp64 + stmx.quartets_fp32) * args.steps
                          / tmx,
        "fp64": {"value": v64, "unit": "ERI/s", "dtype": "f64", "steps": args.fp64_steps,
                 "warmup": args.fp64_warmup, "ms_per_step": t64 / args.fp64_steps * 1e3,
                 "quartets": st64.quartets_fp64,
                 "quartets_per_s": world * float(st64.quartets_fp64) * args.fp64_steps / t64,
                 "E_J": e64[0], "E_K": e64[1],
                 "roofline": dom64_ser or dom64,
                 "roofline_concurrent": dom64,
                 "roofline_pass": {"bound": "fp64-pipe", "achieved": roof64,
                                   "peak": peaks["fp64"], "unit": "TFLOP/s",
                                   "frac": roof64 / peaks["fp64"]}},
        "mixed_scheme": "FP32 VRR/HRR/contraction/transform for quartets with K12 K34 < "
                        "%g; the Boys function of those quartets (Taylor or asymptotic "
                        "branch, e^-T, downward recursion) in FP64 with its argument T in "
                        "double-float arithmetic (~1e-13 relative), rounded to FP32; all "
                        "other quartets in FP64; J/K accumulated in FP64" % MIXED_THRESH,
        "mixed_error": {"vs": "GPU FP64 pass of the same step (full pass)",
                        "dE_J": abs(emx[0] - e64[0]), "dE_K": abs(emx[1] - e64[1]),
                        "max_abs_dJ": float(np.max(np.abs(Jmx - J64))),
                        "max_abs_dK": float(np.max(np.abs(Kmx - K64)))},
        "max_integral_error_vs_oracle": ierr,
        "mixed_fp32_boys": {
            "scheme": "as mixed, with the Boys function of the FP32 quartets in FP32",
            "value": vfb, "unit": "ERI/s", "steps": args.alt_steps, "warmup": 1,
            "ms_per_step": tfb / args.alt_steps * 1e3, "speedup_vs_fp64": vfb / v64,
            "mixed_error": {"vs": "GPU FP64 pass (full pass)",
                            "dE_J": abs(efb[0] - e64[0]), "dE_K": abs(efb[1] - e64[1]),
                            "max_abs_dJ": float(np.max(np.abs(Jfb - J64))),
                            "max_abs_dK": float(np.max(np.abs(Kfb - K64)))},
            "roofline_concurrent": kernel_roofline(laufb, peaks, args.workload,
                                                   "mixed_fp32_boys")},
        "oracle_subset": subset,
        "speedup_mixed_vs_fp64": vmx / v64,
        "roofline": dom_ser,
        "roofline_concurrent": dom,
        "roofline_pass": {"bound": "fp64+fp32 pipes", "achieved": achieved, "peak": peak_blend,
                          "unit": "TFLOP/s", "frac": achieved / peak_blend,
                          "peak_source": "cuBLAS DGEMM %.2f / SGEMM(no TF32) %.1f TFLOP/s "
                                         "measured live; blended by the pass's FP64/FP32 work"
                                         % (peaks["fp64"], peaks["fp32"]),
                          "flops_fp64": fl64, "flops_fp32": fl32},
        "e2e": {"value": ve2e, "unit": "ERI/s", "steps": args.e2e_steps,
                "h2d_bytes_per_step": nbf * nbf * 8, "d2h_bytes_per_step": 2 * nbf * nbf * 8,
                "wall_over_device_same_steps": te2e / dev_e2e if dev_e2e > 0 else None,
                "note": "host D in, host J/K out through lgx_jk, wall clock per call; "
                        "the copies add milliseconds to a pass of seconds, so across "
                        "different steps e2e and value differ by pass-to-pass noise"},
        "gpu_launches": int(stmx.launches) * args.steps + int(st64.launches) * args.fp64_steps
        + int(stfb.launches) * args.alt_steps + int(st_e.launches) * args.e2e_steps,
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
        oracle.set_operator(oracle.OP_ERFC_COULOMB if name == "erfc" else oracle.OP_COULOMB, 0.4)
        ob = oracle.OracleBasis.from_basis(bs)
        Kq = oracle.schwarz(ob, cpu_threads())
        acc = oracle.JKAccumulator(ob.nbf, cpu_threads())
        pairs = sample_pairs(ob, Kq, thresh, CPU_SAMPLE_PAIRS, SEED + 7)
        t0 = time.perf_counter()
        _, nsamp = acc.add_pairs(ob, D, Kq, thresh, pairs)
        v = nsamp / (time.perf_counter() - t0)
        acc.close()
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


def run_profile_pass(args):
    """--profile-pass MODES: one J/K pass of the workload per precision mode
    (0 FP64, 1 mixed, 2 mixed with FP32 Boys), with default launch shapes
    (no tuning), serial class launches and no pass graph, so that each class
    kernel is launched once per mode and a profiler can pick one launch by
    name; prints every launch's device time."""
    os.environ["LGX_TUNE"] = "0"
    os.environ["LGX_OVERLAP"] = "0"
    os.environ["LGX_GRAPHS"] = "0"
    import torch
    import libint_gb300 as lg
    atoms, bs, D, thresh, desc = build_inputs(args.workload)
    ctx = lg.Context(int(os.environ.get("LOCAL_RANK", "0")))
    ctx.set_basis(bs)
    dD = torch.tensor(D, device="cuda")
    dJ, dK = torch.empty_like(dD), torch.empty_like(dD)
    out = {"workload": desc, "nbf": bs.nbf, "passes": []}
    for mode in [int(x) for x in args.profile_pass.split(",")]:
        st = ctx.jk_device(dD.data_ptr(), dJ.data_ptr(), dK.data_ptr(), thresh, mode, MIXED_THRESH)
        out["passes"].append({"mode": mode, "pass_ms": st.pass_ms,
                              "launches": [{k: r[k] for k in ("class", "fp32", "kernel", "ms",
                                                              "quartets", "prim_quartets")}
                                           for r in ctx.last_pass_launches()]})
    ctx.close()
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--fp64-steps", type=int, default=2,
                    help="timed passes of the FP64 comparison (default 2)")
    ap.add_argument("--fp64-warmup", type=int, default=1)
    ap.add_argument("--alt-steps", type=int, default=2,
                    help="timed passes of the FP32-Boys mixed variant (default 2)")
    ap.add_argument("--e2e-steps", type=int, default=3,
                    help="timed host-buffer passes of the e2e figure (default 3)")
    ap.add_argument("--impl", default="lgx", choices=["lgx", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-check", action="store_true",
                    help="skip the pair-subset comparison with the oracle")
    ap.add_argument("--primitive-api", action="store_true",
                    help="time the generated-library entry (libint2_build_eri*) instead")
    ap.add_argument("--profile-pass", default=None, metavar="MODES",
                    help="one untuned, serial J/K pass per listed precision mode (profiling)")
    ap.add_argument("--rows", action="store_true",
                    help="time the widened rows (DF tensors, deriv 2, erfc J/K) instead")
    args = ap.parse_args()
    if args.primitive_api:
        return run_primitive_api(args)
    if args.rows:
        return run_rows(args)
    if args.profile_pass:
        return run_profile_pass(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
