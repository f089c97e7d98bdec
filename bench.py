"""Benchmark: two-site H_eff matvec GFLOP/s at chi=1024 on the U(1) XXZ chain's mid bond.

The workload is the local problem of the plain FP64 U(1) DMRG of the XXZ chain N=64, J=1,
Delta=1, chi=1024 (2 S^z sectors -8..8 of dims 2, 29, 113, 231, 291, 228, 104, 24, 2 on both
bonds of the two-site block, the converged chain's mid bond), with seeded random environments
and block. One step = one H_eff matvec (the call Lanczos makes hundreds of times per bond).

  value   GFLOP/s of the device matvec, FLOPs = 2 x the reference's algorithmic MAC count
          (sum over its four block tensordots of R*K*C, tnkit/blocks.py:1089-1090)
  e2e     the same through the C ABI tnk_apply_two_site_f64 with theta in pinned host memory:
          host->device copy of theta, matvec, device->host copy of the result, every step
  roofline  the dominant kernel (gemm_f64_kernel, the two grouped-GEMM stages) against the
          FP64 peak measured in this run (cuBLAS DGEMM 8192^3 through torch)
  cpu_baseline  the oracle's numpy restatement of the reference's block matvec on the host
  sweep   the whole DMRG the matvec serves -- XXZ N=64 chi=1024, 6 sweeps, seed 1 -- in FP64 and
          in the mixed mode (tensor-core opening sweeps, one float-float polished sweep): sweep
          seconds, phase times and |dE| against the reference's own energy (run by default at
          N=1; --no-sweep skips it)

L2 is flushed (a 256 MiB write) before every timed step, outside the step's CUDA events.
--impl reference times the oracle port (the reference's algorithm, numpy) on the host cores.
Multi-GPU: replicas only (one independent matvec stream per rank, no collective).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "DMRG sweep s & H_eff GFLOP/s at chi=1024; mixed-TC vs FP64 GPU at |dE|<=1e-10"
WORKLOAD = ("U(1) XXZ chain N=64, J=1, Delta=1, chi=1024: two-site H_eff matvec at the mid bond "
            "(sectors 2Sz=-8..8, dims 2,29,113,231,291,228,104,24,2), FP64")


def _env_rank():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def _clock_sampler(path):
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    try:
        f = open(path, "w")
        p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                              "-lms", "200"], stdout=f, stderr=subprocess.DEVNULL)
        return p, f
    except (OSError, FileNotFoundError):
        return None, None


def _clock_summary(path, gpu_index):
    sm, mx, reasons = [], None, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    try:
        for line in open(path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9 or parts[0] != str(gpu_index):
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
    except OSError:
        pass
    return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
            "reasons": sorted(reasons), "samples": len(sm)}


def cpu_matvec_baseline(th, L, W1, W2, R, budget_s=15.0, max_reps=40):
    """Oracle (numpy) block matvec on the host: GFLOP/s over a bounded number of repetitions."""
    from oracle.blocks_np import BT, Leg as OL
    from oracle import dmrg_np as O

    def ob(t):
        return BT.from_flat([OL(tuple(l.charges), tuple(l.dims), l.sign) for l in t.legs],
                            t.charge, t.numpy())
    a = [ob(t) for t in (th, L, W1, W2, R)]
    O.apply_two_site(*a)                       # warm (BLAS threads up)
    reps, t0 = 0, time.perf_counter()
    while reps < max_reps and (time.perf_counter() - t0 < budget_s or reps < 2):
        O.apply_two_site(*a)
        reps += 1
    dt = (time.perf_counter() - t0) / reps
    return dt, reps


def host_threads():
    for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS"):
        if os.environ.get(k):
            return int(os.environ[k])
    return os.cpu_count() or 1


def run_reference(args, rank, world):
    """--impl reference: the oracle port of the reference's block matvec on the host cores."""
    if rank != 0:
        return
    from tnkit_gb300 import workloads, plan as P
    th, L, W1, W2, R = workloads.mid_bond_problem(seed=3, device="cpu")
    macs = P.two_site_ref_macs(th.layout, L.layout, W1.layout, W2.layout, R.layout)
    from oracle.blocks_np import BT, Leg as OL
    from oracle import dmrg_np as O

    def ob(t):
        return BT.from_flat([OL(tuple(l.charges), tuple(l.dims), l.sign) for l in t.legs],
                            t.charge, t.numpy())
    a = [ob(t) for t in (th, L, W1, W2, R)]
    for _ in range(args.warmup):
        O.apply_two_site(*a)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.apply_two_site(*a)
    dt = (time.perf_counter() - t0) / args.steps
    v = 2 * macs / dt / 1e9
    cores = host_threads()
    line = {"metric": METRIC, "value": v, "unit": "GFLOP/s", "impl": "reference",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "parallelism": "replicas only (host rank 0)"},
            "cpu_baseline": {"value": v, "unit": "GFLOP/s", "cores": cores, "kind": "port",
                             "sample": f"{args.steps} full chi=1024 block matvecs (numpy oracle "
                                       f"of tnkit apply_two_site)"},
            "e2e": {"value": v, "unit": "GFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def reduce_max(values, device="cpu"):
    """Elementwise max of per-rank values over the process group (identity without one)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor(values, dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t]


def measure_dgemm_peak(torch, dev):
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    return 2 * n ** 3 / best / 1e12


def measure_tf32_peak(torch, dev):
    """cuBLAS's dense TF32 rate on this GPU (an 8192^3 FP32 GEMM with TF32 tensor cores
    allowed), the denominator of the tensor-core kernel's roofline."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        n = 8192
        a = torch.randn(n, n, dtype=torch.float32, device=dev)
        b = torch.randn(n, n, dtype=torch.float32, device=dev)
        torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 1e30
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1) / 1e3)
        del a, b
        return 2 * n ** 3 / best / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--sweep", action="store_true",
                    help="run the whole chi=1024 DMRG leg even under torchrun (it runs by default "
                         "at N=1)")
    ap.add_argument("--no-sweep", action="store_true",
                    help="skip the whole chi=1024 DMRG leg (FP64 against mixed-ff, ~2 minutes)")
    ap.add_argument("--no-sweep-exact", action="store_true",
                    help="skip the second sweep record (the exact truncation, FP64 and mixed)")
    ap.add_argument("--no-trunc", action="store_true",
                    help="skip the truncation leg (the chi=1024 mid-bond cut on each route)")
    ap.add_argument("--trunc-only", action="store_true",
                    help="run only the truncation leg and print its record")
    ap.add_argument("--trunc-routes", default="gram,svd",
                    help="routes of the truncation leg: 'gram' (device, cuSOLVER, host LAPACK), "
                         "'svd' (exact: device, torch), 'gram-device', 'svd-device'")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the 64-chain batched local problems (sequential, batched, "
                         "graph-captured; a few seconds, run by default at N=1)")
    ap.add_argument("--batch-dmrg", action="store_true",
                    help="also run the 16-chain batched DMRG against one chain after another: "
                         "minutes")
    ap.add_argument("--batch-sweeps", type=int, default=2)
    ap.add_argument("--batch-chains", type=int, default=16,
                    help="chains of the batched-DMRG leg: the first half Ising and half XXZ of "
                         "the 64 seed-2 draws (64: all of them)")
    ap.add_argument("--c5", action="store_true",
                    help="also run the differentiated configuration: disordered XXZ N=48 chi=512 "
                         "DMRG, dE/dJ_i by Hellmann-Feynman, central differences at three bonds; "
                         "and its TDVP half (--c5-tdvp)")
    ap.add_argument("--c5-tdvp", action="store_true",
                    help="also run the TDVP half of the differentiated configuration: d<Z_24(t)>/dJ_i "
                         "after 20 TDVP2 steps of dt=0.05 from the Neel state, by the continuous "
                         "adjoint, central differences at one bond: several minutes")
    ap.add_argument("--batch-pipeline", action="store_true",
                    help="batched DMRG with the two chain groups' phases overlapped")
    ap.add_argument("--sweep-chi", type=int, default=1024)
    ap.add_argument("--sweep-n", type=int, default=64)
    ap.add_argument("--sweep-model", default="xxz", choices=["xxz", "hubbard"])
    ap.add_argument("--sweeps", type=int, default=6)
    ap.add_argument("--svd-method", default="gram", choices=["svd", "gram"])
    ap.add_argument("--svd-host", default="auto", choices=["auto", "device", "never", "always"],
                    help="with --svd-method gram: where the sectors factor (device: reduction "
                         "and back-transformation on the GPU, tridiagonal eigenproblems on the "
                         "host)")
    ap.add_argument("--sweep-precisions", default="f64,mixed,mixed-ff",
                    help="comma-separated among f64, ff, mixed, mixed-ff")
    ap.add_argument("--mixed-schedule", default="sweep", choices=["bond", "sweep"],
                    help="mixed modes: polish every bond, or tensor-core-only opening sweeps")
    ap.add_argument("--polish-sweeps", type=int, default=1)
    ap.add_argument("--polish-mode", default="refine", choices=["lanczos", "refine"],
                    help="mixed modes' polish: high-precision Lanczos, or defect correction "
                         "with tensor-core correction solves")
    ap.add_argument("--sweep-warmup-chi", type=int, default=256,
                    help="untimed 2-sweep DMRG at this chi before each timed precision (0: none)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = _env_rank()

    if args.impl == "reference":
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
        run_reference(args, rank, world)
        return

    import torch
    import ctypes as C
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    from tnkit_gb300 import build, ops, workloads, _lib, plan as P
    build.build()
    _lib.load()
    if args.trunc_only:
        if rank == 0:
            print(json.dumps({"truncation": trunc_leg(torch, dev, measure_dgemm_peak(torch, dev),
                                                      max(args.steps // 2, 5),
                                                      args.trunc_routes)}), flush=True)
        return
    th, L, W1, W2, R = workloads.mid_bond_problem(seed=3 + rank, device=dev)
    # the schedule (FP64 inner product, stage-3 split-K, tile order) picked by the autotuner on
    # this problem; every FP64 launch of the legs below uses its inner product
    op = ops.TwoSiteOperator(th.layout, L, W1, W2, R, tune=True)
    _lib.lib().tnk_gemm_f64_variant(op.inner)
    p = op.plan
    hp = p.host
    ref_macs = P.two_site_ref_macs(th.layout, L.layout, W1.layout, W2.layout, R.layout)
    flops_ref = 2 * ref_macs
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device=dev)
    x = th.data
    y = torch.empty_like(x)

    for _ in range(args.warmup):
        op(x, y)
    torch.cuda.synchronize()

    # --- device-resident timed region: K matvecs, L2 flushed before each ---
    clk_path = os.path.join(tempfile.gettempdir(), f"tnk_bench_clocks_rank{rank}.csv")
    sampler, fh = _clock_sampler(clk_path)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    for i in range(args.steps):
        flush.fill_(float(i))
        evs[i][0].record(stream)
        op(x, y)
        evs[i][1].record(stream)
    torch.cuda.synchronize()
    t_steps = [a.elapsed_time(b) / 1e3 for a, b in evs]
    t_dev = float(sum(t_steps))
    # kernels one matvec launches: the stages of the plan that have work
    per_step = sum(1 for k in (len(hp.g1[2]), len(hp.c2[2]), len(hp.g3[2]), len(hp.c4[2]))
                   if k > 0)

    # --- per-stage kernel timing (same stream, CUDA events around each launch) ---
    lib = _lib.lib()
    ws = op.ws
    cplan = p.c
    sp = _lib.stream_ptr()
    t_g1 = t_c2 = t_g3 = 0.0
    nrep = max(5, args.steps // 2)
    import ctypes
    for i in range(nrep):
        flush.fill_(float(i))
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        slots = (ctypes.c_void_p * 4)()
        e[0].record(stream)
        _lib.check(lib.tnk_grouped_gemm_f64(cplan.t1, cplan.s1, cplan.tiles1, cplan.n_tiles1,
                                            L.data.data_ptr(), x.data_ptr(), R.data.data_ptr(),
                                            ws.data_ptr(), ws.data_ptr(), sp), "gemm1")
        e[1].record(stream)
        _lib.check(lib.tnk_combine_f64(cplan.t2, cplan.c2, cplan.items2, cplan.n_items2,
                                       ws.data_ptr(), ws.data_ptr(), sp), "comb")
        e[2].record(stream)
        _lib.check(lib.tnk_grouped_gemm_f64(cplan.t3, cplan.s3, cplan.tiles3, cplan.n_tiles3,
                                            L.data.data_ptr(), x.data_ptr(), R.data.data_ptr(),
                                            ws.data_ptr(), y.data_ptr(), sp), "gemm3")
        e[3].record(stream)
        torch.cuda.synchronize()
        t_g1 += e[0].elapsed_time(e[1]) / 1e3
        t_c2 += e[1].elapsed_time(e[2]) / 1e3
        t_g3 += e[2].elapsed_time(e[3]) / 1e3
    t_g1, t_c2, t_g3 = t_g1 / nrep, t_c2 / nrep, t_g3 / nrep

    # --- the other inner product of the FP64 grouped GEMM (tnk_gemm_f64_variant), same
    # problem, same timing: the default variant is the headline above ---
    var0 = lib.tnk_gemm_f64_variant(-1)
    var1 = 1 - var0
    lib.tnk_gemm_f64_variant(var1)
    op.inner = var1                      # the tuned operator sets its variant around each call
    y_alt = torch.empty_like(x)
    for _ in range(3):
        op(x, y_alt)
    torch.cuda.synchronize()
    t_alt = 0.0
    t_alt_g = 0.0
    for i in range(args.steps):
        flush.fill_(float(i))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        op(x, y_alt)
        b.record(stream)
        torch.cuda.synchronize()
        t_alt += a.elapsed_time(b) / 1e3
    for i in range(nrep):
        flush.fill_(float(i))
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        e[0].record(stream)
        _lib.check(lib.tnk_grouped_gemm_f64(cplan.t1, cplan.s1, cplan.tiles1, cplan.n_tiles1,
                                            L.data.data_ptr(), x.data_ptr(), R.data.data_ptr(),
                                            ws.data_ptr(), ws.data_ptr(), sp), "gemm1")
        e[1].record(stream)
        _lib.check(lib.tnk_combine_f64(cplan.t2, cplan.c2, cplan.items2, cplan.n_items2,
                                       ws.data_ptr(), ws.data_ptr(), sp), "comb")
        e[2].record(stream)
        _lib.check(lib.tnk_grouped_gemm_f64(cplan.t3, cplan.s3, cplan.tiles3, cplan.n_tiles3,
                                            L.data.data_ptr(), x.data_ptr(), R.data.data_ptr(),
                                            ws.data_ptr(), y_alt.data_ptr(), sp), "gemm3")
        e[3].record(stream)
        torch.cuda.synchronize()
        t_alt_g += (e[0].elapsed_time(e[1]) + e[2].elapsed_time(e[3])) / 1e3
    t_alt_g /= nrep
    op(x, y_alt)                          # the result of the alternative, checked below
    lib.tnk_gemm_f64_variant(var0)
    op.inner = var0
    torch.cuda.synchronize()
    alt_err = float((y_alt - y).abs().max() / y.abs().max())

    # --- end to end through the C ABI: pinned host theta in, pinned host result out ---
    h_in = torch.empty(x.numel(), dtype=torch.float64, pin_memory=True)
    h_in.copy_(x.cpu())
    h_out = torch.empty_like(h_in, pin_memory=True)
    d_in = torch.empty_like(x)
    d_out = torch.empty_like(x)
    for _ in range(2):
        d_in.copy_(h_in, non_blocking=True)
        _lib.check(lib.tnk_apply_two_site_f64(C.byref(cplan), L.data.data_ptr(), d_in.data_ptr(),
                                              R.data.data_ptr(), d_out.data_ptr(), ws.data_ptr(),
                                              ws.numel(), sp), "e2e")
        h_out.copy_(d_out, non_blocking=True)
    torch.cuda.synchronize()
    t_e2e = 0.0
    for i in range(args.steps):
        flush.fill_(float(i))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        d_in.copy_(h_in, non_blocking=True)
        _lib.check(lib.tnk_apply_two_site_f64(C.byref(cplan), L.data.data_ptr(), d_in.data_ptr(),
                                              R.data.data_ptr(), d_out.data_ptr(), ws.data_ptr(),
                                              ws.numel(), sp), "e2e")
        h_out.copy_(d_out, non_blocking=True)
        b.record(stream)
        torch.cuda.synchronize()
        t_e2e += a.elapsed_time(b) / 1e3
    if sampler is not None:
        sampler.terminate()
        sampler.wait()
        fh.close()
    err_e2e = float((h_out.to(dev) - y).abs().max() / y.abs().max())

    # max over ranks
    t_dev, t_e2e = reduce_max([t_dev, t_e2e], dev)
    if rank != 0:
        dist.barrier()
        return

    dgemm = measure_dgemm_peak(torch, dev)
    ms = t_dev / args.steps * 1e3
    value = world * flops_ref * args.steps / t_dev / 1e9
    e2e = world * flops_ref * args.steps / t_e2e / 1e9
    # dominant kernel: the grouped FP64 GEMM (stages 1 and 3); its algorithmic FLOPs are the
    # reference's L.theta and R.x3 tensordots
    parts = P.two_site_ref_macs(th.layout, L.layout, W1.layout, W2.layout, R.layout,
                                parts=True)
    gemm_flops = 2 * (parts[0] + parts[3])
    t_gemm = t_g1 + t_g3
    achieved = gemm_flops / t_gemm / 1e12
    clocks = _clock_summary(clk_path, local)
    line = {"metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded random environments and block, chi=1024 sector dims)",
            "config": {"workload": WORKLOAD, "l2": "flushed (256 MiB write) before every step",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "ref_gflop_per_matvec": flops_ref / 1e9,
                       "exec_gflop_per_matvec": 2 * hp.macs / 1e9,
                       "theta_entries": x.numel()},
            "roofline": {"bound": "fp64", "kernel": "gemm_f64_kernel (stages 1+3)",
                         "achieved": achieved, "peak": dgemm, "unit": "TFLOP/s",
                         "frac": achieved / dgemm,
                         "peak_source": "cuBLAS DGEMM 8192^3 measured in this run (torch.matmul "
                                        "float64); MEASURED_PEAKS.json has no FP64 figure",
                         # DRAM bytes read + written by the two gemm_f64_kernel launches of
                         # one matvec, from `ncu --set full --clock-control none -k
                         # regex:gemm_f64 -s 2 -c 3 python bench.py --steps 2 --warmup 1
                         # --no-cpu --no-sweep` (14.73 MB + 34.15 MB): the operands L, theta, R once; the
                         # intermediates stay in the 129 MB L2
                         "traffic": 48.88e6,
                         "traffic_unit": "bytes per matvec (stages 1+3)",
                         "stage_ms": {"gemm1": t_g1 * 1e3, "comb": t_c2 * 1e3,
                                      "gemm3": t_g3 * 1e3}},
            "e2e": {"value": e2e, "unit": "GFLOP/s", "h2d_bytes_per_step": x.numel() * 8,
                    "d2h_bytes_per_step": x.numel() * 8, "max_rel_err_vs_device": err_e2e},
            "gpu_launches": per_step * args.steps,
            "clocks": clocks}
    line["autotune"] = {"choice": op.tuned.schedule.label(), "ms": op.tuned.ms,
                        "candidates_ms": op.tuned.table,
                        "how": "each candidate schedule once untimed, then 3 matvecs between "
                               "CUDA events on the launching stream (L2 not flushed)"}
    names = {0: "fp64 FMA tile (4 x 4 per thread)", 1: "DMMA tile (mma.sync m8n8k4 f64)"}
    line["fp64_variants"] = {
        "headline": names[var0],
        "headline_gemm_ms": t_gemm * 1e3,
        "headline_executed_tflops": 2 * hp.macs / t_gemm / 1e12,
        "other": names[var1],
        "other_ms_per_step": t_alt / args.steps * 1e3,
        "other_value": flops_ref * args.steps / t_alt / 1e9,
        "other_gemm_ms": t_alt_g * 1e3,
        "other_credited_tflops": gemm_flops / t_alt_g / 1e12,
        "other_executed_tflops": 2 * hp.macs / t_alt_g / 1e12,
        "other_max_rel_diff": alt_err,
        "note": "executed = the FLOPs the plan runs (skipped unused intermediate blocks "
                "excluded); credited = the reference's algorithmic FLOPs of the two GEMM stages"}
    line["mixed"] = mixed_leg(torch, dev, th, L, W1, W2, R, y, flush, flops_ref, parts,
                              args.steps, ms)
    line["float_float"] = ff_leg(torch, th, L, W1, W2, R, y, flush, flops_ref, parts,
                                 args.steps, ms, dgemm)
    # launches of this library's kernels per step in each timed leg (the headline region is the
    # device-resident FP64 matvec); the mixed leg: staging, two tcgen05 GEMMs, FP32 combination;
    # the float-float leg: theta split, two GEMMs, combination, split-K sum when present
    line["gpu_launches_per_step"] = {"fp64": per_step, "e2e": per_step, "mixed": 4,
                                     "float_float": per_step + 1}
    if world == 1 and not args.no_trunc:
        line["truncation"] = trunc_leg(torch, dev, dgemm, max(args.steps // 2, 5),
                                       args.trunc_routes)
    if args.sweep or (world == 1 and not args.no_sweep):
        line["sweep"] = sweep_leg(torch, args)
        if not args.no_sweep_exact and args.svd_method == "gram" and args.sweep_model == "xxz":
            # the same DMRG with the reference's default exact truncation, FP64 and mixed
            ex = argparse.Namespace(**vars(args))
            ex.svd_method, ex.sweep_precisions = "svd", "f64,mixed"
            line["sweep_exact"] = sweep_leg(torch, ex)
    if world == 1 and not args.no_batch:
        line["batch"] = batch_leg(torch, dev, flush, max(args.steps, 5))
    if args.batch_dmrg:
        line["batch_dmrg"] = batch_dmrg_leg(torch, args)
    if args.c5:
        line["c5_gradient"] = c5_leg(torch, args)
    if args.c5 or args.c5_tdvp:
        line["c5_tdvp_gradient"] = c5_tdvp_leg(torch, args)
    if not args.no_cpu:
        dt, reps = cpu_matvec_baseline(th, L, W1, W2, R)
        line["cpu_baseline"] = {"value": flops_ref / dt / 1e9, "unit": "GFLOP/s",
                                "cores": host_threads(), "kind": "port",
                                "sample": f"{reps} full chi=1024 block matvecs (numpy oracle of "
                                          f"tnkit apply_two_site), {dt * 1e3:.1f} ms each"}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()


def trunc_block(torch, dev, seed=0):
    """The chi=1024 mid-bond two-site block (U(1) XXZ N=64 sector dimensions) fused to a matrix,
    with a DMRG-like spectrum: sigma_i = exp(-i / 40) over all 2048 values, dealt to the sectors
    at random, unit norm (synthetic data of the workload's shapes)."""
    from tnkit_gb300 import linalg as LA, workloads
    from tnkit_gb300.tensor import BlockTensor
    th, *_ = workloads.mid_bond_problem(seed=3, device=dev)
    mat, _ = LA.fuse_matrix(th, 2)
    lay = mat.layout
    rng = np.random.default_rng(seed)
    ks = [min(lay.shape(j)) for j in range(lay.nblocks)]
    sig = np.exp(-np.arange(sum(ks)) / 40.0)
    owner = np.concatenate([[j] * k for j, k in enumerate(ks)])
    rng.shuffle(owner)
    data = np.zeros(lay.size)
    for j in range(lay.nblocks):
        R, Cc = lay.shape(j)
        k = ks[j]
        sj = np.sort(sig[owner == j])[::-1]
        U, _ = np.linalg.qr(rng.standard_normal((R, k)))
        V, _ = np.linalg.qr(rng.standard_normal((Cc, k)))
        o = int(lay.offsets[j])
        data[o:o + R * Cc] = ((U * sj) @ V.T).reshape(-1)
    data /= np.linalg.norm(data)
    return BlockTensor(lay, torch.as_tensor(data, device=dev))


def trunc_leg(torch, dev, dgemm, reps, routes_arg="gram,svd"):
    """The truncation of the chi=1024 mid bond (keep 1024 of 2048 values, scale 'right', as the
    left-to-right sweep cuts) on each Gram route: 'device' (the sectors' reductions and the
    back-transformation of the kept vectors on the GPU, tridiagonal problems on host threads),
    'never' (each sector's eigh on cuSOLVER), 'always' (each sector's eigh on host LAPACK,
    sectors over host threads); and the exact route (method='svd', the reference's default) on
    the device against torch.linalg.svd per sector. The spectra are compared sorted: below ~1e-8 of the largest
    value the Gram route resolves nothing, so which sector a value that small lands in is
    rounding, and the routes' bonds may differ there."""
    from tnkit_gb300 import linalg as LA
    m = trunc_block(torch, dev)
    out = {"workload": "chi=1024 mid-bond truncation, U(1) XXZ N=64 sector dims (2 .. 522 "
                       "rows), keep 1024 of 2048, sigma_i = exp(-i/40) dealt to sectors "
                       "(synthetic), scale 'right'",
           "sectors": [list(m.layout.shape(j)) for j in range(m.layout.nblocks)]}
    res = {}
    want = set(routes_arg.split(","))
    routes = []
    if want & {"gram", "gram-device"} and LA.device_gram_available():
        routes.append("device")
    if "gram" in want:
        routes += ["never", "always"]
    for host in routes:
        for _ in range(2):
            r = LA.truncated_svd(m, 1024, scale="right", method="gram", host=host)
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            r = LA.truncated_svd(m, 1024, scale="right", method="gram", host=host)
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        res[host] = r
        out[host] = {"ms_median": float(np.median(ts)) * 1e3, "ms_min": float(min(ts)) * 1e3}
    if "never" in res:
        S0 = torch.sort(res["never"][1], descending=True).values
        for host in routes:
            S = torch.sort(res[host][1], descending=True).values
            out[host]["max_abs_dsigma2_vs_never"] = float((S ** 2 - S0 ** 2).abs().max())
            out[host]["discarded"] = res[host][3]
    # the exact route (method='svd', the reference's default): device bidiagonalisation against
    # torch.linalg.svd per sector
    if want & {"svd", "svd-device"} and LA.device_svd_available():
        ex = {}
        for host in (("device", "never") if "svd" in want else ("device",)):
            for _ in range(2):
                r = LA.truncated_svd(m, 1024, scale="right", method="svd", host=host)
            torch.cuda.synchronize()
            ts = []
            for _ in range(max(3, reps // 3) if host == "never" else reps):
                t0 = time.perf_counter()
                r = LA.truncated_svd(m, 1024, scale="right", method="svd", host=host)
                torch.cuda.synchronize()
                ts.append(time.perf_counter() - t0)
            ex[host] = r
            out[f"svd_{host}"] = {"ms_median": float(np.median(ts)) * 1e3,
                                  "ms_min": float(min(ts)) * 1e3, "discarded": r[3]}
        if "never" in ex:
            Sa = torch.sort(ex["device"][1], descending=True).values
            Sb = torch.sort(ex["never"][1], descending=True).values
            out["svd_device"]["max_abs_dsigma_vs_torch"] = float((Sa - Sb).abs().max())
        tm = {}
        for _ in range(reps):
            blocks = list(LA._blocks(m))
            LA._svd_device_many([(m, blocks, 1024, "right", True)], timing=tm)
        out["svd_device_phases_ms"] = {k: v / reps for k, v in tm.items() if k.endswith("_ms")}
    if "device" in res:
        tm = {}
        for _ in range(reps):
            blocks = list(LA._blocks(m))
            LA._gram_device_many([(m, blocks, 1024, "right", True)], timing=tm)
        ph = {k: v / reps for k, v in tm.items() if k.endswith("_ms") or k == "reduce_flops"}
        out["device_phases_ms"] = {k: v for k, v in ph.items() if k.endswith("_ms")}
        achieved = ph["reduce_flops"] / (ph["reduce_ms"] * 1e-3) / 1e12
        n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
        cls = LA._sytrd_clusters(sorted((min(s) for s in out["sectors"]), reverse=True), n_sm)
        out["roofline"] = {
            "bound": "fp64", "kernel": "sytrd_cluster_kernel (all sectors, one launch per "
                                       "cluster size)",
            "achieved": achieved, "peak": dgemm, "unit": "TFLOP/s", "frac": achieved / dgemm,
            "flops": "4/3 n^3 per sector (LAPACK dsytrd's count)",
            "sms_used": int(sum(cls)), "clusters": cls,
            "peak_source": "cuBLAS DGEMM 8192^3 measured in this run over all SMs"}
    return out


def _peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["bf16_tflops"]), "measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback"


def mixed_leg(torch, dev, th, L, W1, W2, R, y64, flush, flops_ref, parts, steps, ms64):
    """The same matvec on the tensor cores (tcgen05, split TF32, FP32 accumulation) in each
    form: TF32 hi/lo parts staged (passes 3) under both GEMM schedules (tnk_tc_schedule: one CTA
    per tile, or persistent CTAs with two TMEM accumulators for stages with more tiles than
    SMs), and the parts formed in shared memory by the GEMM (passes 4, one CTA per tile); the
    fastest form is the leg's result."""
    from tnkit_gb300 import _lib
    from tnkit_gb300.mixed import TwoSiteOperatorTC
    lib = _lib.lib()
    ops_tc = {p: TwoSiteOperatorTC(th.layout, L, W1, W2, R, passes=p) for p in (3, 4)}
    x = th.data
    y = torch.empty_like(x)
    stream = torch.cuda.current_stream()
    sp = _lib.stream_ptr()
    nrep = max(5, steps // 2)

    def measure(op, sched):
        c = op.c
        prev = lib.tnk_tc_schedule(sched)
        try:
            for _ in range(3):
                op(x, y)
            torch.cuda.synchronize()
            err = float((y - y64).abs().max() / y64.abs().max())
            t = 0.0
            for i in range(steps):
                flush.fill_(float(i))
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                op(x, y)
                b.record(stream)
                torch.cuda.synchronize()
                t += a.elapsed_time(b) / 1e3
            # the two tcgen05 GEMM stages alone, same stream, CUDA events around each launch
            tg = t1 = 0.0
            for i in range(nrep):
                flush.fill_(float(i))
                e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
                e[0].record(stream)
                _lib.check(lib.tnk_grouped_gemm_tc(c.t1, c.s1, c.tiles1, c.n_tiles1, c.maps,
                                                   c.y32, c.err, op.passes, sp), "tc1")
                e[1].record(stream)
                _lib.check(lib.tnk_combine_f32(c.t2, c.c2, c.items2, c.n_items2, c.y32,
                                               c.stage, c.lo_off, 1 if op.passes == 3 else 0,
                                               sp), "comb32")
                e[2].record(stream)
                _lib.check(lib.tnk_grouped_gemm_tc_bn(c.t3, c.s3, c.tiles3, c.n_tiles3, c.maps,
                                                      y.data_ptr(), c.err, op.passes,
                                                      c.bn3 or 128, sp), "tc3")
                e[3].record(stream)
                torch.cuda.synchronize()
                t1 += e[0].elapsed_time(e[1]) / 1e3
                tg += (e[0].elapsed_time(e[1]) + e[2].elapsed_time(e[3])) / 1e3
            op(x, y)
            torch.cuda.synchronize()
            op.check_device_error()
            return t / steps, tg / nrep, t1 / nrep, err
        finally:
            lib.tnk_tc_schedule(prev)
    forms = {"staged_one_tile_per_cta": (3, 0), "staged_persistent": (3, 1),
             "smem_split_one_tile_per_cta": (4, 0)}
    runs = {name: measure(ops_tc[p], k) for name, (p, k) in forms.items()}
    best = min(runs, key=lambda k: runs[k][0])     # the fastest whole matvec
    t, tg, _, err = runs[best]
    c = ops_tc[forms[best][0]].c
    bf16, src = _peaks()
    tf32_meas = measure_tf32_peak(torch, dev)
    tf32_peak = tf32_meas
    alg = 2 * (parts[0] + parts[3]) / tg / 1e12
    mms = t * 1e3
    return {"value": flops_ref / t / 1e9, "unit": "GFLOP/s", "ms_per_step": mms,
            "speedup_vs_fp64": ms64 / mms, "max_rel_err_vs_fp64": err, "dtype": "tf32x3/f32",
            "form": best,
            "forms": {k: {"ms_per_step": v[0] * 1e3, "gemm_ms": v[1] * 1e3,
                          "stage1_ms": v[2] * 1e3, "max_rel_err_vs_fp64": v[3]}
                      for k, v in runs.items()},
            "tiles": {"stage1": int(c.n_tiles1), "stage3": int(c.n_tiles3),
                      "stage3_tile": f"128x{c.bn3 or 128}"},
            "roofline": {"bound": "tensor", "kernel": "gemm_tc_kernel (tcgen05 kind::tf32, "
                                                      "stages 1+3)",
                         "achieved": alg, "mma_issued": 3 * alg, "peak": tf32_peak,
                         "unit": "TFLOP/s", "frac": alg / tf32_peak,
                         "peak_source": "cuBLAS TF32 GEMM 8192^3 measured in this run "
                                        f"(bf16 {src} {bf16:.0f} TFLOP/s; half of it "
                                        f"{bf16 / 2:.0f} would give frac "
                                        f"{alg / (bf16 / 2):.3f})",
                         "traffic": None, "gemm_ms": tg * 1e3}}


def ff_leg(torch, th, L, W1, W2, R, y64, flush, flops_ref, parts, steps, ms64, dgemm):
    """The same matvec with the float-float grouped GEMM (double-FP32 on the FP32 cores)."""
    from tnkit_gb300 import ops
    op = ops.TwoSiteOperator(th.layout, L, W1, W2, R, precision="ff")
    x = th.data
    y = torch.empty_like(x)
    for _ in range(3):
        op(x, y)
    torch.cuda.synchronize()
    err = float((y - y64).abs().max() / y64.abs().max())
    stream = torch.cuda.current_stream()
    t = 0.0
    for i in range(steps):
        flush.fill_(float(i))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        op(x, y)
        b.record(stream)
        torch.cuda.synchronize()
        t += a.elapsed_time(b) / 1e3
    mms = t / steps * 1e3
    gf = flops_ref * steps / t / 1e9
    return {"value": gf, "unit": "GFLOP/s", "ms_per_step": mms, "speedup_vs_fp64": ms64 / mms,
            "max_rel_err_vs_fp64": err, "dtype": "f32x2 (float-float, 48-bit)",
            "vs_measured_dgemm_peak": gf / 1e3 / dgemm}


def batch_leg(torch, dev, flush, steps):
    """The batched-solve workload: the mid-bond local problems of 64 chains (half dense
    transverse-field Ising, half U(1) XXZ; N in {16, ..., 64}, chi in {64, 128, 256}; seed 2)
    applied one operator per chain (a launch sequence each), as one batched operator (one
    launch per stage for all 64), and as that operator captured in a CUDA graph, FP64 and
    float-float. L2 flushed before every timed step; CUDA events on the launching stream."""
    from tnkit_gb300 import batch as B, ops
    probs = B.batch_problems(64, seed=2, device=dev)
    singles = [ops.TwoSiteOperator(th, L, W1, W2, R) for th, L, W1, W2, R in probs]
    op = B.BatchedTwoSiteOperator(probs, tune=True)
    opf = B.BatchedTwoSiteOperator(probs, precision="ff", tune=True)
    opt = B.BatchedTwoSiteOperator(probs, precision="tc")
    flops = 2 * op.ref_macs
    x = torch.randn(op.n, dtype=torch.float64, device=dev)
    y, yf, yg, yt = (torch.empty_like(x) for _ in range(4))
    xs, ys = op.split(x), [torch.empty_like(v) for v in op.split(x)]
    stream = torch.cuda.current_stream()

    def run_seq():
        for o, a, b in zip(singles, xs, ys):
            o(a, b)
    for _ in range(3):
        run_seq()
        op(x, y)
        opf(x, yf)
        opt(x, yt)
    torch.cuda.synchronize()
    opt.tc.check_device_error()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        op(x, yg)
    graph.replay()
    torch.cuda.synchronize()
    ref = torch.cat(ys)
    err = float((y - ref).abs().max() / ref.abs().max())
    errf = float((yf - ref).abs().max() / ref.abs().max())
    errg = float((yg - y).abs().max())
    errt = float((yt - ref).abs().max() / ref.abs().max())

    def timed(fn):
        t = 0.0
        for i in range(steps):
            flush.fill_(float(i))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            t += a.elapsed_time(b) / 1e3
        ms = t / steps * 1e3
        return {"ms_per_step": ms, "value": flops / (ms / 1e3) / 1e9, "unit": "GFLOP/s"}
    seq = timed(run_seq)
    bat = timed(lambda: op(x, y))
    gra = timed(graph.replay)
    bff = timed(lambda: opf(x, yf))
    btc = timed(lambda: opt(x, yt))
    draws = B.chain_draws(64, 2)

    def launches(hp):      # stages with work (an empty stage launches nothing)
        return sum(len(t) > 0 for t in (hp.g1[2], hp.c2[2], hp.g3[2], hp.c4[2]))
    n_seq, n_bat = sum(launches(o.plan.host) for o in singles), launches(op.host)
    return {"workload": "mid-bond two-site H_eff of 64 chains: 32 dense transverse-field Ising "
                        "(g in [0.5, 1.5]), 32 U(1) XXZ (Delta in [0, 2]), N in {16, 24, 32, 48, "
                        "64}, chi in {64, 128, 256}, seed 2; random environments",
            "chains": len(probs), "entries": op.n,
            "chi_counts": {str(c): sum(1 for *_, ch in draws if ch == c) for c in (64, 128, 256)},
            "gflop_per_step": flops / 1e9,
            "sequential_f64": dict(seq, launches=n_seq),
            "batched_f64": dict(bat, launches=n_bat, speedup_vs_sequential=seq["ms_per_step"] /
                                bat["ms_per_step"], max_rel_err_vs_sequential=err,
                                autotune=op.tuned.schedule.label(),
                                autotune_candidates_ms=op.tuned.table),
            "graph_f64": dict(gra, launches=n_bat, speedup_vs_sequential=seq["ms_per_step"] /
                              gra["ms_per_step"], max_abs_diff_vs_batched=errg),
            "batched_ff": dict(bff, launches=n_bat + 1, max_rel_err_vs_sequential_f64=errf,
                               autotune=opf.tuned.schedule.label()),
            "batched_tc": dict(btc, launches=4, max_rel_err_vs_sequential_f64=errt,
                               note="split-TF32 tcgen05 grouped GEMMs of the same batched plan "
                                    "(theta staging, two GEMM stages, FP32 combination)")}


def batch_dmrg_leg(torch, args):
    """Whole DMRG of the 64-chain workload or a sample of it -- the first `--batch-chains` / 2
    Ising and as many XXZ chains of the seed-2 draws (all 64 with --batch-chains 64),
    `--batch-sweeps` sweeps each, seeds 0..K-1 -- run one chain after another with `dmrg` (FP64)
    and as one lockstep batch (`dmrg_batch`, FP64 and float-float); after an untimed warm-up of
    both drivers. Wall-clock seconds and the largest energy difference between the batched and
    the one-by-one runs."""
    from tnkit_gb300 import batch as B, workloads
    from tnkit_gb300.batch_dmrg import dmrg_batch
    from tnkit_gb300.dmrg import dmrg
    from tnkit_gb300.mpo import to_block_mpo
    draws = B.chain_draws(64, 2)
    half = max(1, args.batch_chains // 2)
    sel = [d for d in draws if d[0] == "tfim"][:half] + [d for d in draws if d[0] == "xxz"][:half]

    def mk(m, g, N):
        return workloads.tfim_mpo(N, g) if m == "tfim" else \
            to_block_mpo(workloads.xxz_mpo(N, g), [[1, -1]] * N)[0]
    kw = dict(n_sweeps=args.batch_sweeps, tol=0, rtol=0, expand=0, svd_method=args.svd_method,
              svd_host=args.svd_host)
    dmrg_batch([mk("tfim", 1.0, 8), mk("xxz", 1.0, 8)], [16, 16], charges=[None, 0],
               **dict(kw, n_sweeps=1))
    dmrg(mk("xxz", 1.0, 8), 16, charge=0, **dict(kw, n_sweeps=1))
    torch.cuda.synchronize()
    out = {"workload": f"DMRG of {len(sel)} chains (the first {half} transverse-field Ising and "
                       f"first {half} U(1) XXZ chains of the 64-chain seed-2 draws), "
                       f"{args.batch_sweeps} sweeps each, seeds 0..{len(sel) - 1}, "
                       f"truncation '{args.svd_method}' (host '{args.svd_host}')",
           "chains": [list(d) for d in sel]}
    for prec in ("f64", "ff", "mixed"):
        t0 = time.perf_counter()
        Eb, _, info = dmrg_batch([mk(m, g, N) for m, g, N, _ in sel],
                                 [chi for *_, chi in sel],
                                 charges=[None if m == "tfim" else 0 for m, *_ in sel],
                                 seeds=list(range(len(sel))), precision=prec,
                                 pipeline=args.batch_pipeline, **kw)
        torch.cuda.synchronize()
        out[f"batched_{prec}"] = {"s": time.perf_counter() - t0, "phase_time": info["phase_time"],
                                  "rounds": info["rounds"], "batched_iterations": info["matvecs"],
                                  "batched_iterations_tc": info["matvecs_lo"],
                                  "pipeline": info["pipeline"], "E": Eb}
    t0 = time.perf_counter()
    Es, ph = [], {"eig": 0.0, "trunc": 0.0, "env": 0.0}
    for q, (m, g, N, chi) in enumerate(sel):
        ckw = dict(kw, seed=q, **({"charge": 0} if m == "xxz" else {}))
        E, _, inf = dmrg(mk(m, g, N), chi, **ckw)
        Es.append(E)
        for k in ph:
            ph[k] += inf["phase_time"][k]
    torch.cuda.synchronize()
    out["sequential_f64"] = {"s": time.perf_counter() - t0, "phase_time": ph, "E": Es}
    for prec in ("f64", "ff", "mixed"):
        b = out[f"batched_{prec}"]
        b["speedup_vs_sequential_f64"] = out["sequential_f64"]["s"] / b["s"]
        b["max_abs_dE_vs_sequential"] = float(np.max(np.abs(np.array(b["E"]) - np.array(Es))))
    return out


def sweep_leg(torch, args):
    """The whole DMRG at chi (seed 1, expand 0) in each precision: the U(1) XXZ chain, with the
    reference's own FP64 result (tests/golden/c2_xxz_n64_chi1024.json) as the oracle at N=64
    chi=1024, or the half-filled Fermi-Hubbard chain (t=1, U=4) under U(1) x U(1) (N_up, N_dn)
    blocks, compared with the FP64 run."""
    from tnkit_gb300 import ops, workloads
    from tnkit_gb300.dmrg import dmrg
    from tnkit_gb300.mpo import to_block_mpo
    N, chi = args.sweep_n, args.sweep_chi
    if args.sweep_model == "hubbard":
        name = f"Fermi-Hubbard t=1 U=4 half filling, U(1)xU(1), N={N} chi={chi}"
        make = lambda: to_block_mpo(workloads.hubbard_mpo(N, 1.0, 4.0),
                                    [workloads.HUBBARD_SITE_CHARGES] * N)[0]
        charge = (N // 2, N // 2)
    else:
        name = f"U(1) XXZ N={N} chi={chi}"
        make = lambda: to_block_mpo(workloads.xxz_mpo(N), [[1, -1]] * N)[0]
        charge = 0
    out = {"workload": f"{name}, {args.sweeps} sweeps, seed 1, expand 0, "
                       f"truncation '{args.svd_method}' (host '{args.svd_host}'), "
                       f"mixed schedule '{args.mixed_schedule}', "
                       f"polish '{args.polish_mode}'"
                       + (f" ({args.polish_sweeps} polished sweeps)"
                          if args.mixed_schedule == "sweep" else ""),
           "warmup": (f"each precision after an untimed 2-sweep DMRG at chi="
                      f"{min(chi, args.sweep_warmup_chi)} (first-use library and kernel loading), "
                      if args.sweep_warmup_chi > 0 else "no warm-up DMRG, ")
                     + "plan caches cleared before each timed run"}
    ref = None
    gp = os.path.join(HERE, "tests", "golden", "c2_xxz_n64_chi1024.json")
    if args.sweep_model == "xxz" and N == 64 and chi == 1024 and os.path.exists(gp):
        ref = json.load(open(gp))
        out["reference_E"] = ref["E"]
        out["reference_sweep_s"] = ref["sweep_s"]
    precs = [p for p in args.sweep_precisions.split(",") if p]
    for prec in precs:
        if args.sweep_warmup_chi > 0:
            dmrg(make(), min(chi, args.sweep_warmup_chi), charge=charge, seed=2, n_sweeps=2,
                 tol=0, rtol=0, expand=0, precision=prec, svd_method=args.svd_method,
                 svd_host=args.svd_host, mixed_schedule=args.mixed_schedule, polish_sweeps=1,
                 polish_mode=args.polish_mode)
        ops._PLANS.clear()
        Wb = make()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        E, M, info = dmrg(Wb, chi, charge=charge, seed=1, n_sweeps=args.sweeps, tol=0, rtol=0,
                          expand=0, precision=prec, svd_method=args.svd_method,
                          svd_host=args.svd_host, mixed_schedule=args.mixed_schedule,
                          polish_sweeps=args.polish_sweeps,
                          polish_mode=args.polish_mode)
        torch.cuda.synchronize()
        rec = {"E": E, "energies": info["energies"], "sweep_s": info["sweep_s"],
               "total_s": time.perf_counter() - t0, "phase_time": info["phase_time"],
               "matvecs": info["mixed_counts"], "discarded_weight": info["discarded_weight"],
               "discarded_per_sweep": info["discarded_per_sweep"],
               "mid_bond": {"sectors": len(M[N // 2].legs[0].dims),
                            "dim": int(sum(M[N // 2].legs[0].dims)),
                            "largest_sector": int(max(M[N // 2].legs[0].dims))}}
        if ref is not None:
            rec["abs_dE_vs_reference"] = abs(E - ref["E"])
            rec["discarded_weight_reference"] = ref["discarded_weight"]
            rec["abs_discarded_weight_diff"] = abs(info["discarded_weight"] -
                                                   ref["discarded_weight"])
            if "entropies" in ref:
                # the final state's Schmidt spectra (exact per-sector SVD sweep, after the timed
                # run) against the reference's own (its all_entropies of to_dense_mps)
                from tnkit_gb300.observables import _entropy, schmidt_spectra
                sp = schmidt_spectra(M)
                S = np.array([_entropy(x) for x in sp])
                Sr = np.asarray(ref["entropies"])
                mid = sp[N // 2 - 1]
                mr = np.asarray(ref["mid_bond_spectrum"])
                k = min(len(mid), len(mr))
                rec["entropy_max_rel_err_vs_reference"] = float(np.max(np.abs(S - Sr) /
                                                                       np.abs(Sr)))
                rec["mid_entropy"] = float(S[N // 2 - 1])
                rec["mid_spectrum_max_abs_err_vs_reference"] = float(np.max(np.abs(mid[:k] -
                                                                                   mr[:k])))
        out[prec] = rec
    if "f64" in out:
        for p in precs:
            if p != "f64":
                out[p]["abs_dE_vs_f64"] = abs(out[p]["E"] - out["f64"]["E"])
                out[p]["speedup_total_vs_f64"] = out["f64"]["total_s"] / out[p]["total_s"]
    return out


def c5_leg(torch, args):
    """The differentiated configuration: the disordered XXZ chain N=48 (J_i uniform in
    [0.5, 1.5] from seed 2, Delta=1) under U(1) at chi=512. The ground state by DMRG in FP64 (the
    Hamiltonian is real, so its ground state is real: the reference's complex128 run reaches
    the same state times a phase), then dE/dJ_i of every bond by Hellmann-Feynman
    (grad.energy_gradient_xxz: each bond's two-site operator applied by the matvec kernel at the
    bond's orthogonality centre), checked by sum_i J_i dE/dJ_i = E and by central differences
    (h = 1e-5) of DMRG energies restarted from the ground state at three bonds."""
    from tnkit_gb300 import workloads
    from tnkit_gb300.dmrg import dmrg
    from tnkit_gb300.grad import energy_gradient_xxz
    from tnkit_gb300.mpo import to_block_mpo
    N, chi, delta, h = 48, 512, 1.0, 1e-5
    J = np.random.default_rng(2).uniform(0.5, 1.5, N - 1)

    def run(Jv, init=None, sweeps=10):
        Wb = to_block_mpo(workloads.xxz_disordered_mpo(Jv, delta), [[1, -1]] * N)[0]
        kw = dict(charge=0) if init is None else dict(init_mps=init)
        return dmrg(Wb, chi, seed=1, n_sweeps=sweeps, tol=1e-13, rtol=0, expand=0,
                    eig_tol=1e-12, **kw)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    E, M, info = run(J)
    torch.cuda.synchronize()
    t_dmrg = time.perf_counter() - t0
    t0 = time.perf_counter()
    g = energy_gradient_xxz(M, delta)
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0
    fd = {}
    t0 = time.perf_counter()
    for i in (0, N // 2 - 1, N - 2):
        Jp, Jm = J.copy(), J.copy()
        Jp[i] += h
        Jm[i] -= h
        ep = run(Jp, init=M, sweeps=4)[0]
        em = run(Jm, init=M, sweeps=4)[0]
        d = (ep - em) / (2 * h)
        fd[str(i)] = {"fd": d, "hf": float(g[i]), "rel_err": abs(d - g[i]) / abs(g[i])}
    t_fd = time.perf_counter() - t0
    return {"workload": "disordered XXZ N=48, J_i uniform in [0.5, 1.5] (seed 2), Delta=1, "
                        "U(1), chi=512; DMRG seed 1, tol 1e-13, eig_tol 1e-12; FP64",
            "E": E, "sweeps": info["sweeps"], "dmrg_s": t_dmrg, "gradient_s": t_grad,
            "gradient": [float(x) for x in g],
            "sum_J_dE_dJ_minus_E": float(J @ g - E),
            "central_differences": dict(fd, h=h, seconds=t_fd),
            "max_rel_err_vs_central_differences": max(v["rel_err"] for k, v in fd.items())}


def c5_tdvp_leg(torch, args):
    """The TDVP half of the differentiated configuration: the disordered XXZ chain N=48 (J_i
    uniform in [0.5, 1.5] from seed 2, Delta=1, U(1), chi=512, complex128) quenched from the Neel
    state; <Z_24(t)> after 20 TDVP2 steps of dt=0.05 and its derivative with respect to every
    J_i by the continuous adjoint (grad.tdvp_observable_gradient: forward TDVP of psi, backward
    TDVP of Z psi(t), Im <lam|h_i|psi> at every step, Boole's rule), checked by central
    differences (h = 1e-5) of tdvp2_evolve at the bond left of the measured site (four TDVP
    runs of the chain in all; several minutes). The first sweep from a product state
    projects onto bonds still growing (two-site TDVP is exact only once every bond has its full
    dimension), so the adjoint of the exact evolution and the differences of the TDVP map differ
    by that projection's effect (~1e-6 relative at N=8)."""
    from tnkit_gb300 import workloads
    from tnkit_gb300.grad import tdvp_observable_gradient, xxz_bond_operator, z_expectation
    from tnkit_gb300.mpo import product_block_mps, to_block_mpo
    from tnkit_gb300.tdvp import tdvp2_evolve
    N, chi, delta, h, dt, steps, site = 48, 512, 1.0, 1e-5, 0.05, 20, 24
    J = np.random.default_rng(2).uniform(0.5, 1.5, N - 1)
    mpo = lambda Jv: to_block_mpo(workloads.xxz_disordered_mpo(Jv, delta), [[1, -1]] * N)[0]
    W = mpo(J)
    B = to_block_mpo(xxz_bond_operator(delta), [[1, -1]] * 2)[0]
    neel = product_block_mps(W, [1 if n % 2 == 0 else -1 for n in range(N)])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    value, g, info = tdvp_observable_gradient(neel, W, B, chi, dt, steps, site)
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0

    def z_of(Jv):
        out, _ = tdvp2_evolve(list(neel), mpo(Jv), chi, dt, steps)
        return z_expectation(out, W, site)
    t0 = time.perf_counter()
    fd = {}
    for i in (site - 1,):
        e = np.zeros(N - 1)
        e[i] = h
        d = (z_of(J + e) - z_of(J - e)) / (2 * h)
        fd[str(i)] = {"fd": d, "adjoint": float(g[i]),
                      "rel_err_vs_max": abs(d - g[i]) / float(np.abs(g).max())}
    t_fd = time.perf_counter() - t0
    return {"workload": "disordered XXZ N=48, J_i uniform in [0.5, 1.5] (seed 2), Delta=1, U(1), "
                        "chi=512, complex128; Neel state, 20 TDVP2 steps of dt=0.05, Z_24 = 2 S^z",
            "Z_t": value, "gradient": [float(x) for x in g], "gradient_s": t_grad,
            "max_bond": max(info["bond_dims"]),
            "central_differences": dict(fd, h=h, seconds=t_fd),
            "max_rel_err_vs_central_differences":
                max(v["rel_err_vs_max"] for v in fd.values())}


if __name__ == "__main__":
    main()
