#!/usr/bin/env python
"""Benchmark of the GB300 dense LU path (PDGESV on a 1x1 grid).

Workload (one "step"): plain FP64 PDGESV, N=16384, NB=256, NRHS=16, A and B iid
uniform[-0.5,0.5] from a seeded generator -- the configuration the headline
metric "LU solve TFLOP/s (2N^3/3)" is quoted on.

  value  device-resident: inputs already in HBM; each step restores A and B
         from pristine device copies and calls sl1x1_dgesv_dev. 2N^3/3 flops
         per step; whole-job TFLOP/s summed over ranks (max time over ranks).
  e2e    the same solve through the Fortran-ABI entry point pdgesv_ with A and
         B in pinned host memory: H2D of A and B, factor, solve, D2H of the
         factors, IPIV and X are all inside the timed region.
  roofline  the trailing update (PDGEMM step), timed live with the library's
         phase events on its launching stream: by default the sliced FP64
         product on the BF16 tensor cores (ozgemm_kernel: 36 BF16 slice
         products per FP64 product, against the measured sustained BF16 peak
         of MEASURED_PEAKS.json); with --f64-update dmma the FP64 DMMA kernel
         against the FP64 tensor peak measured live by a register-only DMMA
         loop. Both FP64-equivalent rates are reported.
  cpu_baseline  the CPU restatement of the reference (oracle/, OpenBLAS, all
         host cores) on a bounded sample of the same workload, rank 0 only.

--impl reference times that CPU implementation alone (rank 0; other ranks exit).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = ("LU solve TFLOP/s (2N³/3) plain FP64 vs mixed-IR at matched residual; "
          "batched solve/s")


def measured_peaks():
    """The machine's measured copy bandwidth and BF16 GEMM rates; the recipe's
    fallback figures when the file is absent."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        d["source"] = "measured"
        return d
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
                "source": "fallback"}


def phase_table(phases, steps, hbm_gbs):
    """Per-step phase figures from the library's phase timers: launches, device
    ms, algorithmic TFLOP/s and GB/s, and the GB/s as a fraction of the
    measured HBM copy bandwidth (the roofline of the memory-bound phases)."""
    out = {}
    for k, (launches, ms, flops, nbytes) in phases.items():
        if launches <= 0:
            continue
        gbs = (nbytes / (ms * 1e-3) / 1e9) if ms > 0 and nbytes > 0 else None
        out[k] = {"launches": launches, "ms_per_step": ms / steps,
                  "tflops": (flops / (ms * 1e-3) / 1e12) if ms > 0 and flops > 0 else None,
                  "gbs": gbs,
                  "hbm_frac": (gbs / hbm_gbs) if (gbs and hbm_gbs) else None}
    return out


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    p.add_argument("--n", type=int, default=16384)
    p.add_argument("--nb", type=int, default=256)
    p.add_argument("--nrhs", type=int, default=16)
    p.add_argument("--seed", type=int, default=2024)
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--f64-update", default="sliced", choices=["sliced", "dmma"],
                   help="trailing-update arithmetic of the FP64 factorization")
    p.add_argument("--ozgemm", default="",
                   help="M,N,K: time only the sliced FP64 product C += -A*B at that size "
                        "(the kernel the profiles capture) and exit")
    p.add_argument("--mixed-n", type=int, default=32768,
                   help="size of the mixed-precision LU-IR comparison (0 disables it)")
    p.add_argument("--mixed-fmts", default="bf16x3,fp16,bf16")
    p.add_argument("--cond-n", type=int, default=8192,
                   help="size of the conditioned-matrix sweep of the mixed solver (0 disables it)")
    p.add_argument("--batch", type=int, default=4096,
                   help="systems in the batched-solver comparison (0 disables it)")
    return p.parse_args()


def make_inputs(n, nrhs, seed):
    rng = np.random.default_rng(seed)
    A = np.asfortranarray(rng.uniform(-0.5, 0.5, size=(n, n)))
    B = np.asfortranarray(rng.uniform(-0.5, 0.5, size=(n, nrhs)))
    return A, B


def flops_lu(n):
    return 2.0 * n ** 3 / 3.0


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_time_estimate(A, B, nb):
    """Seconds the oracle's PDGESV restatement (all host cores) takes on the
    full workload, extrapolated (n^3) from a 2048 block."""
    from oracle import oracle as orc

    orc.lib()
    orc.set_threads(os.cpu_count() or 1)
    n0 = min(2048, A.shape[0])
    a0 = np.asfortranarray(A[:n0, :n0].copy())
    b0 = np.asfortranarray(B[:n0, :].copy())
    orc.solve_reference(a0, b0, nb=nb)  # first call: threads, page-in
    t = time.perf_counter()
    orc.solve_reference(a0, b0, nb=nb)
    return (time.perf_counter() - t) * (A.shape[0] / n0) ** 3


def cpu_solve_sample(A, B, nb, budget_s=30.0):
    """Time the oracle's PDGESV restatement (host BLAS, all cores) on a bounded
    sample of the workload: the full matrix when its estimated time fits the
    budget, else the leading n x n block with n scaled down to fit."""
    from oracle import oracle as orc

    orc.lib()
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    n_full = A.shape[0]
    n0 = min(2048, n_full)
    a0 = np.asfortranarray(A[:n0, :n0].copy())
    b0 = np.asfortranarray(B[:n0, :].copy())
    t = time.perf_counter()
    orc.solve_reference(a0, b0, nb=nb)
    t0 = time.perf_counter() - t
    est = t0 * (n_full / n0) ** 3
    n = n_full if est <= budget_s else int(n0 * (budget_s / t0) ** (1 / 3)) // nb * nb
    n = max(min(n, n_full), n0)
    a = np.asfortranarray(A[:n, :n].copy())
    b = np.asfortranarray(B[:n, :].copy())
    t = time.perf_counter()
    LU, ipiv, X, info = orc.solve_reference(a, b, nb=nb)
    dt = time.perf_counter() - t
    # second CPU reference: the host LAPACK's own dgetrf + dgetrs on the same sample
    a = np.asfortranarray(A[:n, :n].copy())
    b = np.asfortranarray(B[:n, :].copy())
    t = time.perf_counter()
    orc.lapack_dgesv(a, b)
    dl = time.perf_counter() - t
    return {"value": flops_lu(n) / dt / 1e12, "unit": "TFLOP/s", "cores": cores, "kind": "port",
            "sample": f"oracle PDGESV restatement (OpenBLAS, {cores} threads), N={n} NB={nb} "
                      f"NRHS={B.shape[1]}, one solve of {dt:.2f} s",
            "blas_loaded": orc.blas_loaded(), "seconds": dt, "n": n,
            "host_lapack": {"value": flops_lu(n) / dl / 1e12, "unit": "TFLOP/s", "seconds": dl,
                            "sample": f"host LAPACK dgetrf + dgetrs (OpenBLAS, {cores} threads) "
                                      f"on the same N={n} sample"}}


def torch_sresid(torch, A, B, X):
    """Tester scaled residual max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf N eps), FP64."""
    n = A.shape[0]
    R = B - A @ X
    anorm = A.abs().sum(dim=1).max()
    return float((R.abs().amax(dim=0) / (X.abs().amax(dim=0) * anorm * 2.0 ** -53 * n)).max())


def mixed_section(sl, torch, dev, args, stream):
    """Config: mixed-precision LU-IR at N=mixed_n, NRHS=1, A and B iid U[-0.5,0.5] FP64,
    against the plain FP64 GPU solve of the same system (time-to-solution, device-resident)."""
    n = args.mixed_n
    g = torch.Generator(device=dev).manual_seed(args.seed + 17)
    At = torch.rand((n, n), dtype=torch.float64, device=dev, generator=g) - 0.5  # column-major A^T view
    Bt = torch.rand((1, n), dtype=torch.float64, device=dev, generator=g) - 0.5
    A, B = At.T, Bt.T
    out = {"workload": f"mixed-precision LU-IR N={n} NRHS=1, A,B iid U[-0.5,0.5] FP64 "
                       "(torch Philox seed), tol: scaled residual <= 1", "n": n, "runs": {}}
    piv = torch.zeros(n, dtype=torch.int32, device=dev)
    Xt = torch.zeros_like(Bt)
    # small warm-up so that workspace growth and first-launch costs are outside the timings
    w = n
    sl.dgesv_ir_dev(w, 1, At.data_ptr(), n, piv.data_ptr(), Bt.data_ptr(), n, Xt.data_ptr(), n,
                    fmt="bf16x3", keep_a=True, stream=stream.cuda_stream)
    peaks = measured_peaks()
    for fmt in [f for f in args.mixed_fmts.split(",") if f]:
        Xt.zero_()
        torch.cuda.synchronize(dev)
        sl.prof_enable(True)
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        info, it, st = sl.dgesv_ir_dev(n, 1, At.data_ptr(), n, piv.data_ptr(), Bt.data_ptr(), n,
                                       Xt.data_ptr(), n, fmt=fmt, nb=256, tol=1.0, keep_a=True,
                                       stream=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1)
        ph = sl.prof_read()
        sl.prof_enable(False)
        g_launch, g_ms, g_flops, _ = ph["mixed_gemm"]
        kmul = 3.0 if fmt == "bf16x3" else 1.0  # BF16x3: three 16-bit products along K
        ach = kmul * g_flops / (g_ms * 1e-3) / 1e12 if g_ms > 0 else None
        pk = peaks.get("bf16_tflops_sustained", 1700.0)
        roof = {"bound": "tensor", "kernel": "lowp_gemm_kernel (tcgen05 kind::f16 trailing update)",
                "achieved": ach, "peak": pk, "unit": "TFLOP/s",
                "frac": (ach / pk) if ach else None,
                "peak_source": f"bf16_tflops_sustained ({'of measured' if peaks.get('source') == 'measured' else 'of fallback'})",
                "achieved_def": f"{'3 x ' if kmul > 1 else ''}sum 2*m*n*k of the update calls / their phase time (operand packing + tcgen05 GEMM)",
                "update_ms": g_ms, "launches": g_launch,
                "panel_ms": ph["mixed_panel"][1]}
        out["runs"][fmt] = {"info": info, "iter": it, "time_to_solution_ms": ms,
                            "factor_ms": st["factor_ms"], "refine_ms": st["refine_ms"],
                            "classical_steps": int(st["classical"]),
                            "gmres_outer": int(st["gmres_outer"]),
                            "gmres_inner": int(st["gmres_inner"]),
                            "fell_back_to_fp64": bool(st["fell_back"]),
                            "sresid": torch_sresid(torch, A, B, Xt.T),
                            "tflops_2n3_3": 2.0 * n ** 3 / 3.0 / (ms * 1e-3) / 1e12,
                            "roofline": roof}
    # plain FP64 GPU solve of the same system
    Ac = At.clone()
    Bc = Bt.clone()
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    info = sl.dgesv_dev(n, 1, Ac.data_ptr(), n, piv.data_ptr(), Bc.data_ptr(), n, 256,
                        stream=stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms64 = e0.elapsed_time(e1)
    out["fp64"] = {"info": info, "time_to_solution_ms": ms64, "sresid": torch_sresid(torch, A, B, Bc.T),
                   "tflops_2n3_3": 2.0 * n ** 3 / 3.0 / (ms64 * 1e-3) / 1e12}
    for fmt, r in out["runs"].items():
        r["time_ratio_vs_fp64"] = r["time_to_solution_ms"] / ms64
        r["meets_target"] = bool(r["sresid"] < 16.0 and r["time_ratio_vs_fp64"] <= 1.0 / 3.0)
    del Ac, Bc, At, Bt
    torch.cuda.empty_cache()
    return out


def conditioned_section(sl, torch, dev, args, stream):
    """Config: N=cond_n, A = (H_1 ... H_64) diag(s) (G_1 ... G_64)^T with Householder
    reflectors from seeded U[-0.5,0.5] vectors and s geometric from 1 to 1/kappa
    (the pattern of TOOLS/LAPACK/dlagge.f), kappa in {1e2, 1e4, 1e6, 1e8}, NRHS=4,
    B iid U[-1,1]: mixed LU-IR (BF16x3) against the plain FP64 GPU solve."""
    n, nrhs = args.cond_n, 4
    g = torch.Generator(device=dev).manual_seed(args.seed + 31)
    out = {"workload": f"conditioned N={n} NRHS={nrhs}, 64+64 Householder reflectors around "
                       "diag(s), s geometric 1..1/kappa (torch Philox seed), tol: scaled "
                       "residual <= 1", "n": n, "nrhs": nrhs, "runs": {}}
    piv = torch.zeros(n, dtype=torch.int32, device=dev)
    for kappa in (1e2, 1e4, 1e6, 1e8):
        s = torch.logspace(0.0, -float(np.log10(kappa)), n, dtype=torch.float64, device=dev)
        A = torch.diag(s)
        for side in (0, 1):
            for _ in range(64):
                v = torch.rand(n, dtype=torch.float64, device=dev, generator=g) - 0.5
                tau = 2.0 / float(v @ v)
                if side == 0:
                    A -= tau * torch.outer(v, v @ A)
                else:
                    A -= tau * torch.outer(A @ v, v)
        At = A.T.contiguous()  # column-major storage of A
        Bt = (torch.rand((nrhs, n), dtype=torch.float64, device=dev, generator=g) * 2.0 - 1.0)
        Xt = torch.zeros_like(Bt)
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        info, it, st = sl.dgesv_ir_dev(n, nrhs, At.data_ptr(), n, piv.data_ptr(), Bt.data_ptr(), n,
                                       Xt.data_ptr(), n, fmt="bf16x3", nb=256, tol=1.0,
                                       keep_a=True, stream=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1)
        Ac, Bc = At.clone(), Bt.clone()
        torch.cuda.synchronize(dev)
        e0.record(stream)
        info64 = sl.dgesv_dev(n, nrhs, Ac.data_ptr(), n, piv.data_ptr(), Bc.data_ptr(), n, 256,
                              stream=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms64 = e0.elapsed_time(e1)
        out["runs"][f"{kappa:.0e}"] = {
            "info": info, "iter": it, "time_to_solution_ms": ms, "fp64_ms": ms64,
            "time_ratio_vs_fp64": ms / ms64, "classical_steps": int(st["classical"]),
            "gmres_outer": int(st["gmres_outer"]), "gmres_inner": int(st["gmres_inner"]),
            "fell_back_to_fp64": bool(st["fell_back"]),
            "sresid": torch_sresid(torch, A, Bt.T, Xt.T),
            "sresid_fp64": torch_sresid(torch, A, Bt.T, Bc.T), "info_fp64": info64}
        del A, At, Ac, Bc, Bt, Xt
    torch.cuda.empty_cache()
    return out


def batched_cpu_baseline(dA, dB, budget_s=10.0):
    """Host LAPACK dgesv (OpenBLAS, all cores) on the batch's systems in order,
    as many as fit the budget: solves per second."""
    from oracle import oracle as orc

    orc.lib()
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    done, t_total = 0, 0.0
    for a, b in zip(dA, dB):
        A = np.asfortranarray(a.cpu().numpy().T)
        B = np.asfortranarray(b.cpu().numpy().T)
        t = time.perf_counter()
        orc.lapack_dgesv(A, B)
        t_total += time.perf_counter() - t
        done += 1
        if t_total > budget_s:
            break
    return {"value": done / t_total, "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": f"host LAPACK dgesv (OpenBLAS, {cores} threads) on the first {done} systems "
                      f"of the batch, one at a time ({t_total:.1f} s)"}


def batched_section(sl, torch, dev, args, stream):
    """Config: 4096 independent FP64 systems, N ~ U{16..512}, NRHS ~ U{1..8}, entries
    U[-0.5,0.5] plus a diagonal shift N/4 on half the batch; FP64 and FP32-factor +
    FP64-IR plans, each executed as one CUDA graph of persistent launches."""
    rng = np.random.default_rng(args.seed + 5)
    count = args.batch
    ns = rng.integers(16, 513, size=count)
    rs = rng.integers(1, 9, size=count)
    g = torch.Generator(device=dev).manual_seed(args.seed + 5)
    dA, dB, dX = [], [], []
    for i in range(count):
        n, r = int(ns[i]), int(rs[i])
        a = torch.rand((n, n), dtype=torch.float64, device=dev, generator=g) - 0.5
        if i % 2 == 0:
            a.diagonal().add_(n / 4.0)
        dA.append(a)
        dB.append(torch.rand((r, n), dtype=torch.float64, device=dev, generator=g) - 0.5)
        dX.append(torch.zeros((r, n), dtype=torch.float64, device=dev))
    systems = [(dA[i].data_ptr(), int(ns[i]), int(ns[i]), dB[i].data_ptr(), int(ns[i]), int(rs[i]),
                dX[i].data_ptr(), int(ns[i])) for i in range(count)]
    flops = float(sum(2.0 * int(n) ** 3 / 3.0 for n in ns))
    out = {"workload": f"{count} systems, N~U{{16..512}}, NRHS~U{{1..8}}, U[-0.5,0.5] "
                       "+ N/4 diagonal shift on half (torch Philox seed)",
           "systems": count, "sum_2n3_3_gflop": flops / 1e9, "modes": {}}
    for mode, name in ((0, "fp64"), (1, "fp32_factor_fp64_ir")):
        t0 = time.perf_counter()
        plan = sl.BatchPlan(systems, mode=mode, tol=1.0, autotune=True, stream=stream.cuda_stream)
        plan_s = time.perf_counter() - t0
        for _ in range(2):
            plan.execute()
        reps = 5
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            plan.execute()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / reps
        info, its, sr = plan.results()
        srv = np.array(sr)
        itv = np.array(its)
        out["modes"][name] = {
            "solves_per_s": count / (ms * 1e-3), "ms_per_batch": ms,
            "tflops_2n3_3": flops / (ms * 1e-3) / 1e12, "plan_create_s": plan_s,
            "shape": plan.shape(), "nonzero_info": int(np.count_nonzero(info)),
            "sresid_max": float(srv.max()), "sresid_median": float(np.median(srv)),
            "refine_steps_mean": float(itv[itv >= 0].mean()) if mode == 1 else 0.0,
            "fp64_pass_systems": int(np.count_nonzero(itv == -1)) if mode == 1 else 0}
        if mode == 0 and args.dmma_peak:
            # SIMT FP64 factor + solve: against the FP64 peak measured live
            ach = flops / (ms * 1e-3) / 1e12
            out["modes"][name]["roofline"] = {
                "bound": "fp64 pipe", "kernel": "batched persistent FP64 kernel",
                "achieved": ach, "peak": args.dmma_peak, "unit": "TFLOP/s",
                "frac": ach / args.dmma_peak,
                "peak_source": "register-only FP64 DMMA loop measured in this run (sl1x1_dmma_peak_tflops)",
                "achieved_def": "sum over systems of 2n^3/3 / batch time"}
        plan.close()
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = batched_cpu_baseline(dA, dB)
    del dA, dB, dX
    torch.cuda.empty_cache()
    return out


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if ws > 1:
        import torch.distributed as dist  # noqa: F811

        backend = "nccl" if args.impl == "gpu" else "gloo"
        dist.init_process_group(backend=backend)
    return ws, rank, local, dist


def run_reference(args):
    ws, rank, local, dist = dist_init(args)
    if rank != 0:
        return 0
    A, B = make_inputs(args.n, args.nrhs, args.seed)
    from oracle import oracle as orc

    orc.lib()
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    # Each timed step solves the full workload when the K steps fit about six
    # minutes, else a bounded leading block; the W warm-up steps (threads,
    # page-in) run on a 2048 block. The probe also times the host LAPACK.
    est = cpu_time_estimate(A, B, args.nb)
    n = args.n if est * args.steps <= 360.0 else \
        max(2048, int(args.n * (360.0 / (est * args.steps)) ** (1 / 3)) // args.nb * args.nb)
    probe = cpu_solve_sample(A, B, args.nb, budget_s=est * (n / args.n) ** 3 * 1.05 + 1.0)
    n = probe["n"]
    a0 = np.asfortranarray(A[:n, :n].copy())
    b0 = np.asfortranarray(B[:n, :].copy())
    w0 = min(2048, n)
    aw = np.asfortranarray(A[:w0, :w0].copy())
    bw = np.asfortranarray(B[:w0, :].copy())
    for _ in range(args.warmup):
        orc.solve_reference(aw, bw, nb=args.nb)
    t = time.perf_counter()
    for _ in range(args.steps):
        orc.solve_reference(a0, b0, nb=args.nb)
    dt = (time.perf_counter() - t) / args.steps
    val = flops_lu(n) / dt / 1e12
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "TFLOP/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": f"synthetic: A, B iid U[-0.5,0.5] (numpy PCG64 seed {args.seed})",
        "config": {"workload": f"plain FP64 PDGESV (1x1 grid) N={args.n} NB={args.nb} "
                               f"NRHS={args.nrhs}" + ("" if n == args.n else f"; CPU sample N={n}"),
                   "n": args.n, "nb": args.nb, "nrhs": args.nrhs, "sample_n": n,
                   "same_config": n == args.n, "warmup_n": w0},
        "cpu_baseline": {"value": val, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                         "sample": f"oracle PDGESV restatement on host BLAS (OpenBLAS, {cores} "
                                   f"threads), N={n} NB={args.nb} NRHS={args.nrhs} per step; the "
                                   "Fortran/MPI reference cannot be compiled here",
                         "host_lapack": probe.get("host_lapack")},
        "e2e": {"value": val, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    import torch

    ws, rank, local, dist = dist_init(args)
    torch.cuda.set_device(local)
    import scalapack_gb300 as sl

    L = sl.lib(build_if_missing=True)
    if L.sl1x1_device_ok() != 1:
        raise SystemExit("sl1x1: no usable sm_103 GPU")
    n, nb, nrhs = args.n, args.nb, args.nrhs
    sliced = args.f64_update == "sliced"
    sl.set_f64_update(1 if sliced else 0)
    A, B = make_inputs(n, nrhs, args.seed + rank)
    dev = torch.device("cuda", local)
    # column-major device copies: torch row-major (cols, rows) == Fortran (rows, cols)
    dA0 = torch.from_numpy(A.T).to(dev)  # contiguous (n, n) holding A column-major
    dB0 = torch.from_numpy(B.T).to(dev)
    dA = torch.empty_like(dA0)
    dB = torch.empty_like(dB0)
    dpiv = torch.empty(n, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    def step():
        dA.copy_(dA0)
        dB.copy_(dB0)
        info = sl.dgesv_dev(n, nrhs, dA.data_ptr(), n, dpiv.data_ptr(), dB.data_ptr(), n, nb,
                            stream=sptr)
        if info != 0:
            raise RuntimeError(f"sl1x1_dgesv_dev INFO={info}")

    def barrier():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)

    for _ in range(max(3, args.warmup)):
        step()
    peak = float(L.sl1x1_dmma_peak_tflops())
    args.dmma_peak = peak
    sl.prof_enable(True)
    launches0 = sl.launch_count()
    routes0 = int(L.sl1x1_ozgemm_fp64_routes())
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        barrier()
    ms = e0.elapsed_time(e1) / args.steps
    launches = sl.launch_count() - launches0
    fp64_routes = int(L.sl1x1_ozgemm_fp64_routes()) - routes0
    phases = sl.prof_read()
    sl.prof_enable(False)
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * flops_lu(n) / (ms * 1e-3) / 1e12

    # accuracy of the last device solve (tester residual, computed with torch FP64)
    X = dB.T  # (n, nrhs) view in row-major numpy sense after .cpu()
    Ad = dA0.T
    R = torch.from_numpy(B).to(dev) - Ad @ X
    anorm = Ad.abs().sum(dim=1).max()
    eps = 2.0 ** -53
    sresid = float((R.abs().amax(dim=0) / (X.abs().amax(dim=0) * anorm * eps * n)).max())

    # roofline of the dominant kernel: the trailing update
    g_launch, g_ms, g_flops, g_bytes = phases["gemm"]
    fp64_rate = g_flops / (g_ms * 1e-3) / 1e12 if g_ms > 0 else None
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    tkey = "ozgemm_trailing" if sliced else "dgemm_dmma_trailing"
    if os.path.exists(tp):
        try:
            traffic = json.load(open(tp)).get(tkey, {}).get("bytes_per_launch")
        except Exception:
            traffic = None
    if sliced:
        mp = measured_peaks()
        bf_peak = mp.get("bf16_tflops_sustained") or mp.get("bf16_tflops")
        achieved = 36.0 * fp64_rate if fp64_rate else None
        roofline = {"bound": "tensor", "achieved": achieved, "peak": bf_peak, "unit": "TFLOP/s",
                    "frac": (achieved / bf_peak) if (achieved and bf_peak) else None,
                    "traffic": traffic,
                    "kernel": "ozgemm_kernel + slice kernels (PDGEMM trailing update: FP64 "
                              "product from 36 exact BF16 slice products, tcgen05 kind::f16)",
                    "achieved_def": "36 x 2*m*n*k BF16 flops per trailing update / its phase time",
                    "peak_source": f"bf16_tflops_sustained (of {mp['source']})",
                    "fp64_equivalent_tflops": fp64_rate, "fp64_dmma_peak_tflops": peak,
                    "launches": g_launch, "avg_launch_ms": g_ms / max(1, g_launch),
                    "algorithmic_bytes_per_launch": g_bytes / max(1, g_launch)}
    else:
        roofline = {"bound": "tensor", "achieved": fp64_rate, "peak": peak, "unit": "TFLOP/s",
                    "frac": (fp64_rate / peak) if (fp64_rate and peak) else None,
                    "traffic": traffic,
                    "kernel": "dgemm_dmma_kernel (PDGEMM trailing update, FP64 DMMA m16n8k4)",
                    "peak_source": "measured live: register-only DMMA loop "
                                   "(sl1x1_dmma_peak_tflops); MEASURED_PEAKS.json has no FP64 figure",
                    "launches": g_launch, "avg_launch_ms": g_ms / max(1, g_launch),
                    "algorithmic_bytes_per_launch": g_bytes / max(1, g_launch)}
    phase_summary = phase_table(phases, args.steps, measured_peaks().get("hbm_gbs"))

    # end to end through the Fortran-ABI entry point with pinned host buffers
    e2e = None
    if args.e2e_steps > 0:
        ctxt = sl.blacs_gridinit(1, 1)
        hA0 = torch.from_numpy(A.T).pin_memory()
        hB0 = torch.from_numpy(B.T).pin_memory()
        hA = torch.empty_like(hA0).pin_memory()
        hB = torch.empty_like(hB0).pin_memory()
        ipiv = np.zeros(n + nb, dtype=np.int32)
        desca = np.array([1, ctxt, n, n, nb, nb, 0, 0, n], dtype=np.int32)
        descb = np.array([1, ctxt, n, nrhs, nb, nb, 0, 0, n], dtype=np.int32)
        an = hA.numpy().T  # Fortran-ordered view of pinned memory
        bn = hB.numpy().T
        tt = []
        for it in range(args.e2e_steps + 1):
            hA.copy_(hA0)
            hB.copy_(hB0)
            if dist is not None:
                dist.barrier()
            t = time.perf_counter()
            info = sl.pdgesv(n, nrhs, an, 1, 1, desca, ipiv, bn, 1, 1, descb)
            dt = time.perf_counter() - t
            if info != 0:
                raise RuntimeError(f"pdgesv_ INFO={info}")
            if it > 0:
                tt.append(dt)
        e2e_s = float(np.mean(tt))
        if dist is not None:
            t = torch.tensor([e2e_s], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e2e_s = float(t.item())
        e2e = {"value": ws * flops_lu(n) / e2e_s / 1e12, "unit": "TFLOP/s",
               "h2d_bytes_per_step": 8 * n * n + 8 * n * nrhs,
               "d2h_bytes_per_step": 8 * n * n + 4 * n + 8 * n * nrhs,
               "ms_per_step": e2e_s * 1e3, "steps": len(tt),
               "path": "pdgesv_ (Fortran ABI) from pinned host memory"}
        # the same call on ordinary (pageable) arrays, as a Fortran caller passes them
        del hA, hB, an, bn
        pa0 = np.asfortranarray(A)
        pb0 = np.asfortranarray(B)
        pa = np.empty_like(pa0, order="F")
        pb = np.empty_like(pb0, order="F")
        tp = []
        for it in range(args.e2e_steps + 1):
            np.copyto(pa, pa0)
            np.copyto(pb, pb0)
            if dist is not None:
                dist.barrier()
            t = time.perf_counter()
            info = sl.pdgesv(n, nrhs, pa, 1, 1, desca, ipiv, pb, 1, 1, descb)
            dt = time.perf_counter() - t
            if info != 0:
                raise RuntimeError(f"pdgesv_ INFO={info}")
            if it > 0:
                tp.append(dt)
        pg_s = float(np.mean(tp))
        if dist is not None:
            t = torch.tensor([pg_s], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            pg_s = float(t.item())
        e2e["pageable"] = {"value": ws * flops_lu(n) / pg_s / 1e12, "unit": "TFLOP/s",
                           "ms_per_step": pg_s * 1e3, "steps": len(tp),
                           "path": "pdgesv_ from ordinary (pageable) numpy arrays"}
        del pa, pb, pa0, pb0

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_solve_sample(A, B, nb)
        cpu.pop("n", None)

    mixed = None
    if args.mixed_n > 0:
        mixed = mixed_section(sl, torch, dev, args, stream)
    conditioned = None
    if args.cond_n > 0:
        conditioned = conditioned_section(sl, torch, dev, args, stream)
    batched = None
    if args.batch > 0:
        batched = batched_section(sl, torch, dev, args, stream)

    # cuBLAS DGEMM yardstick (run and timed only, never on the product path)
    yard = None
    try:
        x = torch.rand(4096, 4096, dtype=torch.float64, device=dev)
        y = torch.rand(4096, 4096, dtype=torch.float64, device=dev)
        x @ y
        torch.cuda.synchronize(dev)
        f0 = torch.cuda.Event(enable_timing=True); f1 = torch.cuda.Event(enable_timing=True)
        f0.record(); x @ y; f1.record(); torch.cuda.synchronize(dev)
        yard = 2 * 4096 ** 3 / (f0.elapsed_time(f1) * 1e-3) / 1e12
    except Exception:
        pass

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": f"synthetic: A, B iid U[-0.5,0.5] (numpy PCG64 seed {args.seed}+rank)",
            "config": {"workload": f"plain FP64 PDGESV (1x1 grid) N={n} NB={nb} NRHS={nrhs}",
                       "n": n, "nb": nb, "nrhs": nrhs,
                       "f64_update": "sliced FP64 on BF16 tensor cores" if sliced else "FP64 DMMA",
                       "parallelism": "replicas" if ws > 1 else "1 GPU",
                       "l2": "inputs (8N^2 = %.1f GiB) larger than L2; no flush" % (8 * n * n / 2**30)},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": clk.summary(),
            "gpu_launches": launches,
            "sliced_fp64_routes_per_step": fp64_routes / args.steps,
            "accuracy": {"sresid": sresid, "threshold": 16.0},
            "phases": phase_summary,
            "mixed_ir": mixed,
            "conditioned": conditioned,
            "batched": batched,
            "yardstick_cublas_dgemm_tflops": yard,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def run_ozgemm(args):
    """The sliced FP64 product alone at one size: 3 untimed and `steps` timed
    calls of sl1x1_ozgemm_dev on device-resident U[-0.5,0.5] operands."""
    import torch

    import scalapack_gb300 as sl

    m, n, k = (int(v) for v in args.ozgemm.split(","))
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev).manual_seed(args.seed)
    A = torch.rand((k, m), dtype=torch.float64, device=dev, generator=g) - 0.5
    B = torch.rand((n, k), dtype=torch.float64, device=dev, generator=g) - 0.5
    C = torch.rand((n, m), dtype=torch.float64, device=dev, generator=g) - 0.5
    call = lambda: sl.ozgemm_dev(m, n, k, -1.0, A.data_ptr(), m, B.data_ptr(), k, C.data_ptr(), m)
    for _ in range(3):
        assert call() == 0
    torch.cuda.synchronize()
    ts = []
    for _ in range(max(1, args.steps)):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        assert call() == 0
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    ms = float(np.median(ts))
    print(json.dumps({"ozgemm": [m, n, k], "ms": ms, "fp64_equivalent_tflops": 2 * m * n * k / ms / 1e9,
                      "bf16_slice_tflops": 36 * 2 * m * n * k / ms / 1e9}), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.ozgemm:
        return run_ozgemm(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
