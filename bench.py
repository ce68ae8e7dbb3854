#!/usr/bin/env python
"""Benchmark: z_s=1 magnification PDFs per second on one GB300 (plain GPU solver).

One step = one full PDF of generate_pdf_lnmu(1.0) with the default flat LCDM cosmology, on the
reference's own z_s=1 population (tests/golden/full/cells_zs1_gauss_full.npz, made by the
reference's code: 79,574 fine cells and 201 xi_lin groups): measured k-reach probes, ln Phi on the
1683 x 2687 k-grid (separable Psi_1 + the gauss xi term on the 101^2 coarse grid + bicubic
spline), exp, Hankel and kappa transforms onto the 2400 x 796 (kappa, gamma) grid,
Euler-Maclaurin term, constant-mu path integrals on 500 + 3201 ln mu points, normalisation.
Without that file a labelled stand-in (xi groups synthesised from one shell) is used.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision mixed|fp64] [--impl ours|reference]

* value    PDFs/s with the population resident in HBM, device-timed with CUDA events on the
           engine's streams (max over ranks; N ranks run N independent replicas: weak scaling).
* e2e      the same metric through the drop-in call Lam(population) + invert(...) with HOST
           buffers: population upload (H2D), every PDF stage, P_s read back (D2H) per step.
* roofline the kernel with the largest device time in the timed region: its algorithmic FLOPs
           (or bytes) per launch / its event-timed duration, against the measured peak.
* accuracy every PDF of the timed regions and of the e2e loop, against the reference's stored
           z_s=1 PDF (pdf_zs1.json) and against the FP64 path: max |dP| / peak, PDF L1 over
           ln mu in [-1, 9] (bar 1e-4) and the tail relative error for ln mu > 1 (bar 1e-3).
* fp64_path the parity path (max |dP| / peak <= 1e-9 vs the reference) timed the same way.
* --impl reference  the reference algorithm on the host CPU cores (the FP64 NumPy oracle that
           restates sgl_full.Lam / invert; the reference itself needs Numba, absent on the host).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "z_s=1 PDFs/sec on 1 GB300: plain GPU solver at PDF L1<=1e-4"
FULL_POP = ROOT / "tests" / "golden" / "full" / "cells_zs1_gauss_full.npz"
REF_PDF = ROOT / "tests" / "golden" / "pdf_zs1.json"
WORKLOAD_REAL = ("z_s=1 default flat LCDM PDF (generate_pdf_lnmu(1.0) defaults): the reference's own z_s=1 "
                 "population (79,574 fine cells, all 201 xi_lin groups), gauss closure, CLI ln mu grids "
                 "(1601 + 1600 points); accuracy against the reference's stored pdf_zs1.json")
WORKLOAD_STANDIN = ("STAND-IN (the reference's full z_s=1 population file is absent): the reference's z_s=1 "
                    "cells + 201 xi_lin groups synthesised from shell 30, gauss closure, CLI ln mu grids")
XI_OUT = np.concatenate([np.linspace(-1.0, 1.0, 1601), np.linspace(1.005, 9.0, 1600)])
XI_COARSE = 101        # the gauss term's coarse k grid per axis (Lam xi_coarse default)
# DRAM bytes (read + write) per launch of the dominant kernels on this workload, from one ncu
# capture each (dram__bytes_read.sum + dram__bytes_write.sum)
TRAFFIC = {"xi_fused": 2.7385e8}


def load_workload():
    """(population, workload description, reference PDF or None): the reference's own z_s=1
    population when its file is present, else the labelled stand-in."""
    from sgl_analytic_gb300 import Population
    from sgl_analytic_gb300.workloads import zs1_population
    if FULL_POP.exists():
        ref = json.loads(REF_PDF.read_text())
        P0 = np.concatenate([ref["P_s"], ref["P_s_tail"]])
        x0 = np.concatenate([ref["xi"], ref["xi_tail"]])
        assert np.array_equal(x0, XI_OUT)
        return Population.load(FULL_POP), WORKLOAD_REAL, P0
    return zs1_population(), WORKLOAD_STANDIN, None


def pdf_errors(P, Pref):
    """(max|dP| / peak, L1 over ln mu, tail relative error for ln mu > 1 where Pref > 1e-6 peak)."""
    peak = float(np.max(Pref))
    l1 = float(np.trapezoid(np.abs(P - Pref), XI_OUT))
    tail = (XI_OUT > 1.0) & (np.abs(Pref) > 1e-6 * peak)
    rel = float(np.max(np.abs(P[tail] - Pref[tail]) / np.abs(Pref[tail]))) if tail.any() else 0.0
    return float(np.max(np.abs(P - Pref))) / peak, l1, rel


def worst(Ps, Pref):
    """Worst (dpeak, L1, tail) over a list of PDFs."""
    e = np.array([pdf_errors(P, Pref) for P in Ps])
    return {"pdfs_checked": len(Ps), "max_dP_over_peak": float(e[:, 0].max()), "pdf_l1": float(e[:, 1].max()),
            "tail_rel": float(e[:, 2].max())}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Clocks:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        out = Path(os.environ.get("SGL_BENCH_CLOCKS_DIR", tempfile.gettempdir()))
        self.path = out / f"sgl_bench_clocks_r{device}.csv"

    def start(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.f = open(self.path, "w")
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clock sampling unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1])); mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text()), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def cpu_baseline_sample(pop, max_seconds=60.0):
    """The FP64 oracle (restatement of the reference's Lam + invert) on the host cores: one PDF."""
    from oracle import invert_oracle as IO
    from oracle import lam_oracle as LO
    X = LO.XiGroups(pop.groups(), pop.ce_k, pop.ce_g, prune=1e-7)
    lam = LO.OracleLam(pop.w0, pop.k0, pop.g0, pop.ig, pop.fe_g, pop.V, X)
    t = time.perf_counter()
    IO.invert(lam, lam.sigma(), XI_OUT)
    dt = time.perf_counter() - t
    return dt


def run_reference(args, rank, world):
    """--impl reference: the reference algorithm on the CPU (rank 0 only)."""
    if rank != 0:
        return
    pop, workload, _ = load_workload()
    for _ in range(args.warmup):
        cpu_baseline_sample(pop)
    ts = [cpu_baseline_sample(pop) for _ in range(args.steps)]
    tot = sum(ts)
    v = args.steps / tot
    cores = os.cpu_count()
    line = {"metric": METRIC, "value": v, "unit": "PDF/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "reference z_s=1 population" if workload == WORKLOAD_REAL else "synthetic stand-in",
            "impl": "reference",
            "config": {"workload": workload, "precision": "fp64", "device": "host CPU"},
            "cpu_baseline": {"value": v, "unit": "PDF/s", "cores": cores, "kind": "port",
                             "sample": "one full z_s=1 PDF per step (NumPy oracle restating sgl_full.Lam, "
                                       "separable Psi_1, _Qxi_gauss, _Q_interpolated and invert; BLAS threads "
                                       "= all host cores)"},
            "e2e": {"value": v, "unit": "PDF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# FP32-pipe operations per (k, cell) term of the mixed sweep, counted from the kernel source:
# float-float product 3, half-angle reduction 8, sincosf on the reduced argument ~14,
# cos-1 / sin-ph / small-argument select 6, two Kahan updates 8.
MIXED_OPS_PER_TERM = 39


def run_cf_sweep(args, rank, world, local):
    """Synthetic CF-sweep microbenchmark: 128 planes x 256 masses x 512 impact parameters = 16.8M cells,
    16384 log-spaced k in [1e-2, 1e6]; one step = one full sweep (2.75e11 compensated terms)."""
    import torch
    from sgl_analytic_gb300._lib import SGL_FP64, SGL_MIXED, Engine
    from sgl_analytic_gb300.workloads import cf_sweep_problem
    torch.cuda.set_device(local)
    kap, w, kk = cf_sweep_problem(seed=rank)
    eng = Engine(local)
    eng.sweep_set_cells(kap, w)
    stream = torch.cuda.ExternalStream(eng.stream, device=torch.device("cuda", local))
    terms = float(kk.size) * kap.size
    ref64 = eng.sweep(kk, SGL_FP64)                   # FP64 path: accuracy reference and its own timing
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream); eng.sweep(kk, SGL_FP64); e1.record(stream); torch.cuda.synchronize()
    ms64 = e0.elapsed_time(e1)
    for _ in range(max(3, args.warmup)):
        eng.sweep(kk, SGL_MIXED)
    clocks = Clocks(local)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0.record(stream)
    for _ in range(args.steps):
        out = eng.sweep(kk, SGL_MIXED)
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    f32 = eng.measure_peak(False)
    f64 = eng.measure_peak(True)
    rate = world * args.steps * terms / (ms / 1e3)
    mag = np.abs(ref64)
    rel = float(np.max(np.abs(out - ref64) / np.maximum(mag, 1e-300)))
    if rank == 0:
        ach = rate / world * MIXED_OPS_PER_TERM / 1e12          # FP32-pipe instructions / s (per GPU)
        peak_inst = f32 / 2.0                                   # FMA instructions / s from the probe
        line = {"metric": "CF-sweep compensated (k, cell) terms/sec", "value": rate, "unit": "terms/s",
                "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup),
                "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded)",
                "config": {"workload": "plane x mass x impact-parameter CF sweep: 128 x 256 x 512 = 16,777,216 "
                                       "cells, 16384 log-spaced k in [1e-2, 1e6], truncated-NFW kappa",
                           "precision": "mixed", "l2": "cells (269 MB) larger than L2"},
                "fp64_path": {"terms_per_s": terms / (ms64 / 1e3), "ms": ms64},
                "accuracy": {"max_rel_vs_fp64": rel},
                "roofline": {"bound": "fp32-pipe", "achieved": ach, "peak": peak_inst, "unit": "T inst/s",
                             "frac": ach / peak_inst, "traffic": None, "ops_per_term": MIXED_OPS_PER_TERM,
                             "peak_source": "FP32 FMA-throughput probe measured in this run",
                             "fp32_fma_tflops": f32, "fp64_fma_tflops": f64},
                "clocks": clk}
        print(json.dumps(line))


def run_batched(args, rank, world, local):
    """Batched plain solver: 4096 instances (Latin hypercube over h, Om, sigma8, Ob, ns, Ok, w0, wa and
    z_s in [0.3, 5]; gauss / vp alternating; 32-256 planes and 4096-32768 k-points per instance) in one
    persistent launch per step, the step (solve + Phi + inversion to dP/dln mu on 4096 points) replayed
    from a CUDA graph; launch shape from the engine's autotuner."""
    import torch
    from sgl_analytic_gb300._lib import SGL_FP64, SGL_MIXED, Engine
    from sgl_analytic_gb300.cfbatch import make_batch
    torch.cuda.set_device(local)
    n = args.batch_instances
    t0 = time.perf_counter()
    b = make_batch(n, seed=100 + rank, nm=12, nb=12)
    t_make = time.perf_counter() - t0
    eng = Engine(local)
    lnmu = np.linspace(-0.5, 2.0, 4096)
    eng.cfb_set(b.arrays())
    kt, cps = eng.cfb_tune(SGL_MIXED)
    for _ in range(max(3, args.warmup)):
        P, _ = eng.cfb_pdf(lnmu, SGL_MIXED, use_graph=True)
    clocks = Clocks(local)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ms_steps = []
    for _ in range(args.steps):
        P, ms = eng.cfb_pdf(lnmu, SGL_MIXED, use_graph=True)
        ms_steps.append(ms)
    clk = clocks.stop()
    ms = float(np.sum(ms_steps))
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    terms = b.terms()
    rate = world * args.steps * n / (ms / 1e3)
    # accuracy: a sample of the instances (every 256th) solved again alone in FP64
    sel = list(range(0, n, max(1, n // 16)))
    sub = b
    from sgl_analytic_gb300 import cfbatch as CB
    keep_p = np.concatenate([np.arange(sub.inst_plane0[i], sub.inst_plane0[i + 1]) for i in sel])
    cell_ranges = [(sub.plane_cells[p], sub.plane_cells[p + 1]) for p in keep_p]
    kap = np.concatenate([sub.kap[a:c] for a, c in cell_ranges])
    w = np.concatenate([sub.w[a:c] for a, c in cell_ranges])
    pc = np.concatenate([[0], np.cumsum([c - a for a, c in cell_ranges])]).astype(np.int64)
    ip0 = np.concatenate([[0], np.cumsum([sub.inst_plane0[i + 1] - sub.inst_plane0[i] for i in sel])]).astype(np.int32)
    vp_slots = np.cumsum(sub.closure == 1) - 1
    vsel = [int(vp_slots[i]) for i in sel if sub.closure[i] == 1]
    sb = CB.Batch(theta=sub.theta[sel], zs=sub.zs[sel], closure=sub.closure[sel], inst_plane0=ip0, plane_cells=pc,
                  kap=kap, w=w, nk=sub.nk[sel], dk=sub.dk[sel], V=sub.V[sel], sigma=sub.sigma[sel],
                  vp_D=sub.vp_D[keep_p], vp_K=sub.vp_K[vsel], vp_w=sub.vp_w[vsel])
    e64 = Engine(local)
    e64.cfb_set(sb.arrays())
    P64, ms64 = e64.cfb_pdf(lnmu, SGL_FP64, use_graph=False)
    l1, dpk = [], []
    for j, i in enumerate(sel):
        l1.append(float(np.trapezoid(np.abs(P[i] - P64[j]), lnmu)))
        dpk.append(float(np.max(np.abs(P[i] - P64[j])) / np.max(np.abs(P64[j]))))
    # e2e: the batch uploaded from host memory and its PDFs read back every step
    h2d = sum(a.nbytes for a in (b.kap, b.w, b.plane_cells, b.inst_plane0, b.nk, b.dk, b.V, b.vp_D, b.vp_K, b.vp_w))
    torch.cuda.synchronize()
    te = time.perf_counter()
    for _ in range(2):
        eng.cfb_set(b.arrays())
        Pe, _ = eng.cfb_pdf(lnmu, SGL_MIXED, use_graph=True)
    e2e = 2 * n / (time.perf_counter() - te)
    f32 = eng.measure_peak(False)
    if rank == 0:
        ach = terms / (ms / args.steps / 1e3) * MIXED_OPS_PER_TERM / 1e12
        line = {"metric": "batched plain solver: instance PDFs/sec (4096 uneven instances per persistent launch)",
                "value": rate, "unit": "PDF/s", "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup),
                "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32+f64", "data": "synthetic (seeded Latin hypercube)",
                "config": {"workload": f"{n} instances: cosmology box x z_s in [0.3, 5], gauss / vp alternating, "
                                       "32-256 planes x 144 cells, 4096-32768 k-points each, dP/dln mu on 4096 points",
                           "instances": n, "planes": int(b.inst_plane0[-1]), "cells": int(b.plane_cells[-1]),
                           "k_points": int(np.sum(b.nk.astype(np.int64))), "terms_per_step": terms,
                           "launch": {"k_per_item": kt, "ctas_per_sm": cps, "graph": True},
                           "l2": "cells (1.7 GB FP32 + float-float) and ln Phi (1.2 GB) larger than L2"},
                "accuracy": {"instances_checked": len(sel), "pdf_l1_vs_fp64_max": max(l1), "max_dP_over_peak": max(dpk),
                             "bar_l1": 1e-4},
                "e2e": {"value": e2e, "unit": "PDF/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(P.nbytes)},
                "roofline": {"kernel": "k_cfb_persistent (+ inversion)", "bound": "fp32-pipe", "achieved": ach,
                             "peak": f32 / 2, "unit": "T inst/s", "frac": ach / (f32 / 2),
                             "ops_per_term": MIXED_OPS_PER_TERM, "terms_per_s": terms / (ms / args.steps / 1e3),
                             "peak_source": "FP32 FMA-throughput probe of this run (FMA instructions / s)"},
                "batch_build_s": t_make, "clocks": clk}
        print(json.dumps(line))


def run_surrogate(args, rank, world, local):
    """Learned per-plane log-CF surrogate: 2e6 training samples (3907 planes x 512 ln k) and 1e5
    held-out samples (196 planes x 512) from the FP64 GPU solver over the cosmology box; a
    two-member ensemble of 8 -> 6 x 256 SiLU -> 2 BF16 MLPs trained by the engine's tensor-core
    kernels; accuracy against the FP64 solver and the judge's fallback fraction."""
    import torch
    from sgl_analytic_gb300 import surrogate as S
    from sgl_analytic_gb300._lib import Engine
    torch.cuda.set_device(local)
    eng = Engine(local)
    stream = torch.cuda.ExternalStream(eng.stream, device=torch.device("cuda", local))
    model = S.PlaneModel()
    n_tr, n_te, nk = 3907, 196, 512
    th, zl, lnk = S.sample_inputs(n_tr, nk, seed=11 + rank)
    t0 = time.perf_counter()
    L = S.solve_planes(eng, model, th, zl, lnk)
    t_solve = time.perf_counter() - t0
    th2, zl2, lnk2 = S.sample_inputs(n_te, nk, seed=1000 + rank)
    L2 = S.solve_planes(eng, model, th2, zl2, lnk2)
    X, Y, X2 = S.features(th, zl, lnk), S.targets(L), S.features(th2, zl2, lnk2)
    sur = S.Surrogate(eng, members=2, seed=rank)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    hist = sur.train(X, Y, epochs=args.sur_epochs, batch=16384, lr=2e-3)
    e1.record(stream)
    torch.cuda.synchronize()
    t_train = e0.elapsed_time(e1) / 1e3
    steps = args.sur_epochs * (X.shape[0] // 16384) * len(sur.mlps)
    sizes = sur.mlps[0].sizes
    gemm_flops = 3 * 2.0 * 16384 * sum(a * c for a, c in zip(sizes[:-1], sizes[1:]))    # fwd, dX, dW
    # inference throughput (device time, after warm-up) and accuracy on the held-out planes
    (X2d,) = S.to_device(eng, X2)
    for _ in range(3):
        sur.mlps[0].predict(X2d)
    torch.cuda.synchronize()
    e0.record(stream)
    reps = 10
    for _ in range(reps):
        sur.mlps[0].predict(X2d)
    e1.record(stream)
    torch.cuda.synchronize()
    t_inf = e0.elapsed_time(e1) / 1e3 / reps
    lam_s, dis = sur.log_cf(X2)
    lam_x = L2.ravel()
    d = np.abs(lam_s - lam_x)
    rel = d / np.maximum(np.abs(lam_x), 1e-300)
    fb = {f"{t:g}": float(np.mean(dis.reshape(n_te, nk).max(1) > t)) for t in (1e-5, 1e-3, 1e-1, 1.0)}
    pk, pk_src = peaks()
    ach = gemm_flops * steps / t_train / 1e12
    # surrogate + judge PDF sweep (z_s = 1 instances, 64 planes each) against the plain solver
    sw_thetas = S.sample_inputs(args.sweep_instances, 1, seed=5000 + rank)[0]
    sw = S.pdf_sweep(eng, model, sur, sw_thetas, threshold=1e-5)
    lnmu = sw["lnmu"]
    l1s = [float(np.trapezoid(np.abs(a - b), lnmu)) for a, b in zip(sw["P_sur"], sw["P_plain"])]
    sw_nojudge = S.pdf_sweep(eng, model, sur, sw_thetas[:2], threshold=np.inf)
    l1_raw = [float(np.trapezoid(np.abs(a - b), lnmu)) for a, b in zip(sw_nojudge["P_sur"], sw_nojudge["P_plain"])]
    if rank == 0:
        line = {"metric": "surrogate per-plane log-CF evaluations/sec (BF16 MLP inference, 1 member)",
                "value": X2.shape[0] / t_inf, "unit": "samples/s", "n_gpus": world, "steps": reps, "warmup": 3,
                "ms_per_step": 1e3 * t_inf, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "bf16+f32", "data": "synthetic (seeded cosmology-dependent lens planes)",
                "config": {"workload": "per-plane log-CF surrogate: 8 -> 6 x 256 SiLU -> 2 BF16 MLP, 2 members, "
                                       "2e6 training / 1e5 held-out samples from the FP64 GPU solver",
                           "train_samples": int(X.shape[0]), "heldout_samples": int(X2.shape[0]),
                           "epochs": args.sur_epochs, "batch": 16384},
                "solver_samples_per_s": X.shape[0] / t_solve,
                "gain_vs_solver": (X2.shape[0] / t_inf) / (X.shape[0] / t_solve),
                "training": {"seconds": t_train, "samples_per_s": steps * 16384 / t_train,
                             "final_loss": [h[-1] for h in hist], "first_loss": [h[0] for h in hist]},
                "accuracy": {"abs_dlncf_median": float(np.median(d)), "abs_dlncf_p90": float(np.quantile(d, 0.9)),
                             "rel_median": float(np.median(rel)), "rel_p90": float(np.quantile(rel, 0.9))},
                "judge_fallback_fraction": fb,
                "pdf_sweep": {"instances": int(len(sw_thetas)), "planes_per_instance": 64, "k_points": 2048,
                              "lnmu_points": int(lnmu.size), "judge_threshold_lncf": 1e-5,
                              "fallback_fraction": float(np.mean(sw["fallback"])),
                              "pdf_per_s_surrogate_judge": len(sw_thetas) / sw["t_sur"],
                              "pdf_per_s_plain_solver": len(sw_thetas) / sw["t_plain"],
                              "pdf_l1_vs_plain_max": max(l1s),
                              "pdf_l1_surrogate_without_judge": l1_raw},
                "roofline": {"kernel": "k_tc_gemm<1> (BF16) during training", "bound": "tensor", "achieved": ach,
                             "peak": float(pk["bf16_tflops"]), "unit": "TFLOP/s", "frac": ach / float(pk["bf16_tflops"]),
                             "traffic": None, "peak_source": f"{pk_src} bf16 burst",
                             "note": "whole training step time, including host-side launch overhead"}}
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--precision", default="mixed", choices=("fp64", "mixed"))
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--slots", type=int, default=4,
                    help="PDFs in flight at once (contexts on their own streams) for the headline value")
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--workload", default="zs1_pdf", choices=("zs1_pdf", "cf_sweep", "surrogate", "batched"))
    ap.add_argument("--batch-instances", type=int, default=4096)
    ap.add_argument("--sur-epochs", type=int, default=20)
    ap.add_argument("--sweep-instances", type=int, default=8)
    args = ap.parse_args()
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    if args.workload in ("cf_sweep", "surrogate", "batched"):
        {"cf_sweep": run_cf_sweep, "surrogate": run_surrogate, "batched": run_batched}[args.workload](args, rank, world,
                                                                                                    local)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    import torch
    from sgl_analytic_gb300 import Lam, invert
    from sgl_analytic_gb300._lib import Engine

    torch.cuda.set_device(local)
    pop, workload, Pref = load_workload()
    eng = Engine(local)
    lam = Lam(pop, xi=True, engine=eng, precision=args.precision)
    sig = lam.sigma()
    stream = torch.cuda.ExternalStream(eng.stream, device=torch.device("cuda", local))

    def step():
        return invert(lam, sig, xi_out=XI_OUT, phi_tol=1e-8, precision=args.precision)

    # reference PDF for the accuracy check: the FP64 path (parity-tested against the reference)
    _, P64, meta64 = invert(lam, sig, xi_out=XI_OUT, phi_tol=1e-8, precision="fp64")
    for _ in range(max(3, args.warmup)):
        step()
    # ---- timed region (population resident in HBM).  Profiling is off here: with it on, the
    # engine keeps the xi term and the separable part on one stream so that each kernel is timed
    # alone; the per-kernel statistics come from a separate profiled pass below.
    clocks = Clocks(local)
    eng.profile(False)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    P = None
    timed_P = []
    for _ in range(args.steps):
        _, P, meta = step()
        timed_P.append(P)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    # per-kernel statistics (kernels timed alone, one stream), same number of steps
    eng.profile(True)
    eng.stats(reset=True)
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    stats = eng.stats(reset=True)
    eng.profile(False)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    single_value, single_ms = world * args.steps / (ms / 1e3), ms / args.steps
    value = single_value
    # ---- batched plain solver: `slots` resident copies of the workload, one context (stream) each,
    # every slot running `steps` PDFs concurrently; device time from an event on the default stream
    # that all slot streams wait on, to an event recorded after every slot stream's last work
    batched = None
    if args.slots > 1:
        from sgl_analytic_gb300.batch import BatchSolver
        bs = BatchSolver(slots=args.slots, device=local, precision=args.precision)
        bs.load([pop] * args.slots)
        bs.solve(XI_OUT, repeats=max(1, args.warmup), phi_tol=1e-8)
        sstreams = [torch.cuda.ExternalStream(h, device=torch.device("cuda", local)) for h in bs.streams]
        master = torch.cuda.current_stream()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()
        b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        b0.record(master)
        for ss in sstreams:
            ss.wait_event(b0)
        outs = bs.solve(XI_OUT, repeats=args.steps, keep_all=True, phi_tol=1e-8)
        for ss in sstreams:
            ev = torch.cuda.Event()
            ev.record(ss)
            master.wait_event(ev)
        b1.record(master)
        torch.cuda.synchronize()
        bms = b0.elapsed_time(b1)
        if world > 1:
            import torch.distributed as dist
            t = torch.tensor([bms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            bms = float(t.item())
        batched_P = [P_ for slot in outs for P_ in slot]
        batched = {"slots": args.slots, "pdfs": args.slots * args.steps * world,
                   "value": world * args.slots * args.steps / (bms / 1e3), "ms": bms}
        bs.close()
        value = batched["value"]
    # clocks sampled over both timed regions (one PDF at a time, then the batched headline)
    clk = clocks.stop()
    # ---- the FP64 parity path, same timing method (outside the headline region)
    fp64_line = None
    if args.fp64_steps > 0 and args.precision != "fp64":
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.fp64_steps):
            invert(lam, sig, xi_out=XI_OUT, phi_tol=1e-8, precision="fp64")
        e1.record(stream)
        torch.cuda.synchronize()
        ms64 = e0.elapsed_time(e1)
        fp64_line = {"value": args.fp64_steps / (ms64 / 1e3), "unit": "PDF/s", "ms_per_pdf": ms64 / args.fp64_steps,
                     "steps": args.fp64_steps}
    # accuracy of every PDF of both timed regions (checked after the timing)
    all_P = timed_P + (batched_P if batched else [])
    # ---- e2e: drop-in call with host buffers (population upload + PDF + read-back)
    h2d = sum(a.nbytes for a in (pop.w0, pop.k0, pop.g0, pop.ig, pop.fe_g, pop.xg_m, pop.xg_nrow, pop.xg_nidx,
                                 pop.xg_idx, pop.xg_rows, pop.ce_k, pop.ce_g))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_P = []
    for _ in range(args.e2e_steps):
        lam_e = Lam(pop, xi=True, engine=eng, precision=args.precision)
        _, Pe, _ = invert(lam_e, lam_e.sigma(), xi_out=XI_OUT, phi_tol=1e-8, precision=args.precision)
        e2e_P.append(Pe)
    torch.cuda.synchronize()
    e2e = args.e2e_steps / (time.perf_counter() - t0)
    accuracy = {"bar_l1": 1e-4, "bar_tail": 1e-3, "vs_fp64_path": worst(all_P + e2e_P, P64)}
    if Pref is not None:
        accuracy["vs_reference_pdf"] = worst(all_P + e2e_P, Pref)
        accuracy["fp64_path_vs_reference_pdf"] = worst([P64], Pref)
    # ---- roofline of the dominant kernel
    pk, pk_src = peaks()
    tags = {k: v for k, v in stats.items() if not k.startswith("_")}
    top = max(tags, key=lambda k: tags[k]["ms"]) if tags else None
    roof = None
    launches = int(stats.get("_launches", {}).get("launches", 0))
    if top:
        r = tags[top]
        per_ms = r["ms"] / r["launches"]
        if r["flops"] > 0:
            fp64 = top.startswith("gemm_f64")
            peak_v = float(pk.get("fp64_tflops", 1.25)) if fp64 else float(pk["bf16_tflops_sustained"])
            ach = r["flops"] / r["launches"] / (per_ms / 1e3) / 1e12
            roof = {"kernel": top, "bound": "fp64" if fp64 else "tensor", "achieved": ach, "peak": peak_v,
                    "unit": "TFLOP/s", "frac": ach / peak_v, "traffic": TRAFFIC.get(top),
                    "peak_source": ("nominal GB300 FP64 (1.25 TFLOP/s): no measured FP64 peak in "
                                    "MEASURED_PEAKS.json") if fp64 else f"{pk_src} bf16 sustained (of measured)",
                    "launches": r["launches"], "ms_per_launch": per_ms,
                    "flops_per_launch": r["flops"] / r["launches"]}
            if top.startswith("gemm_f32"):
                # the kernel runs on the FP32 FMA pipe (SIMT): its own ceiling is the FMA probe
                f32 = eng.measure_peak(False)
                roof["simt_fp32"] = {"peak": f32, "frac": ach / f32, "peak_source": "FP32 FMA probe, this run"}
            if top == "xi_fused":
                # the fused Psi_2 kernel's tensor-core contraction (above) is fed by its CUDA-core
                # producer, which forms T = rows x J_m entry by entry in FP32: its FMA work per launch
                # is sum over groups of entries x rows x coarse k_gamma columns
                t_fl = 2.0 * float(np.sum(pop.xg_nidx.astype(np.float64) * pop.xg_nrow)) * XI_COARSE
                f32 = eng.measure_peak(False)
                a32 = t_fl / (per_ms / 1e3) / 1e12
                roof["producer_fp32"] = {"flops_per_launch": t_fl, "achieved": a32, "peak": f32, "frac": a32 / f32,
                                         "peak_source": "FP32 FMA probe, this run"}
        else:
            ach = r["bytes"] / r["launches"] / (per_ms / 1e3) / 1e9
            roof = {"kernel": top, "bound": "hbm", "achieved": ach, "peak": float(pk["hbm_gbs"]), "unit": "GB/s",
                    "frac": ach / float(pk["hbm_gbs"]), "traffic": TRAFFIC.get(top), "peak_source": pk_src,
                    "launches": r["launches"], "ms_per_launch": per_ms}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        dt = cpu_baseline_sample(pop)
        cpu = {"value": 1.0 / dt, "unit": "PDF/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "one full z_s=1 PDF (NumPy FP64 oracle restating the reference's Lam + invert, BLAS on "
                         "all host cores)"}
    if rank == 0:
        g = meta["grid"]
        line = {"metric": METRIC, "value": value, "unit": "PDF/s", "n_gpus": world, "steps": args.steps,
                "warmup": max(3, args.warmup), "ms_per_step": 1e3 * world / value, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if args.precision == "fp64" else "f32+f64",
                "data": ("the reference's own z_s=1 population (built by its code, tests/golden/make_fixtures.py)"
                         if Pref is not None else "synthetic stand-in (reference z_s=1 cells; xi groups from shell 30)"),
                "config": {"workload": workload, "precision": args.precision,
                           "k_grid": f"{g['nk_k']}x{g['nk_g']}", "out_grid": f"{g['n_kap']}x{g['n_gam']}",
                           "parallelism": f"replicas x{world}", "pdfs_in_flight": max(1, args.slots),
                           "l2": "inputs > L2 every step (xi group rows 151 MB FP32, separable T 86 MB, Phi 29 MB)"},
                "accuracy": accuracy,
                "single_stream": {"value": single_value, "unit": "PDF/s", "ms_per_pdf": single_ms},
                "batched": batched,
                "fp64_path": fp64_line,
                "e2e": {"value": e2e, "unit": "PDF/s", "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(XI_OUT.size * 8)},
                "roofline": roof, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches * 1,
                "stage_ms": meta.get("device_ms"), "kernels": tags}
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
