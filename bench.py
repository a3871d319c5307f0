#!/usr/bin/env python
"""Design iterations per second of the SIMP compliance loop on one GB300.

Workload: 3-D hex8 cantilever, 160 x 80 x 80 elements (1,024,000 elements,
3,168,963 DOFs), E=1, nu=0.3, volfrac 0.12, penal 3, rmin 1.5, density
filter, OC; boundary conditions of the reference's cantilever_3d callable
(x=0 face clamped, z=0 symmetry plane, linearly varying tip line load).
Every design iteration solves K u = f to an FP64 relative residual of 1e-8.

A step is one design iteration (solve, compliance + sensitivities, filter,
OC, density filter).  The headline arm is the mixed-precision solver (FP32
V-cycle and K.u with BF16 densities in the smoother, FP64 residual /
refinement / dots / compliance / coarsest solve); the plain FP64 GMG-PCG arm
runs the same iterations for the ratio.  Inputs are synthetic (the reference
publishes no dataset); the per-iteration working set (~1 GB) exceeds L2, so
no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm's CPU path (the oracle port of
assembly + SciPy SuperLU direct solve + filter + OC) on the host cores on a
bounded sample grid and scales it to the workload.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "design iters/s, 3D hex8 1M elems: learned+mixed vs plain GMG-PCG at res 1e-8"
UNIT = "design iters/s"
SIZE = (160, 80, 80)
VOLFRAC, RMIN, PENAL = 0.12, 1.5, 3.0
# V-cycle smoothing of both GPU arms (learned+mixed and plain FP64): one
# damped-Jacobi sweep (omega 0.6) before and after the coarse correction, and
# none on level 1 (its right-hand side restricted straight on to level 2,
# bit 1 of tg_problem.unsmoothed).  Measured on GB300 at 160x80x80 against
# the library default (2 sweeps on every level): one sweep, 21 % more PCG
# iterations but 15 % less time per design iteration (mixed), 22 % less
# (FP64); level 1 unsmoothed on top, 7 % more iterations and 13 % less time.
# Leaving level 2 or 3 unsmoothed costs more iterations than it saves; omega
# 0.65 was 1.5 % faster here but stalls the FP32 PCG on a random-density
# 32x16x16 design once level 1 is unsmoothed (omega 0.6 converges there).
# Two sweeps on the small coarse levels (2-3) cut the PCG iterations by 17 %
# for 2.4 % less time per design iteration (three: no further gain).
NSMOOTH, OMEGA, UNSMOOTHED, NSMOOTH_COARSE = 1, 0.6, 1 << 1, 2
CPU_SAMPLE = (24, 12, 12)
# grids of the reference arm: one design iteration of one grid per step, in
# turn; the seconds per iteration are fitted as a * nel^b
REF_LADDER = [(16, 8, 8), (24, 12, 12), (32, 16, 16)]


def _host_info():
    """Logical CPUs of this host and the CPU model (lscpu)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"cpu_count": os.cpu_count(), "cpu_model": model}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1, 0
    import torch
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend=backend)
    return dist, rank, ws, local


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def _max_over_ranks(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = tempfile.mktemp(suffix=".csv")

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for name, val in zip(names, p[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def _problem(precision, device, size=None, volfrac=None):
    size = size or SIZE
    from topoptlab_gb300.context import GpuProblem
    from topoptlab_gb300.elements import lk_linear_elast_3d
    from topoptlab_gb300.example_bc import cantilever_3d
    nx, ny, nz = size
    ndof = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    _, f, fixed, _, _ = cantilever_3d(nx, ny, nz, ndof)
    return GpuProblem(nx, ny, nz, lk_linear_elast_3d(), fixed, f[:, 0], volfrac or VOLFRAC, RMIN, ft=1,
                      penal=PENAL, precision=precision, rtol=1e-8, device=device,
                      nsmooth=NSMOOTH, omega=OMEGA, unsmoothed=UNSMOOTHED,
                      nsmooth_coarse=NSMOOTH_COARSE)


# kernel families timed one at a time with CUDA events (library profiling kinds)
FAMILIES = [(1, "fine_f64_residual"), (2, "fine_f32_kmul"), (3, "fine_bf16_jacobi"),
            (8, "stencil_level1_f32"), (4, "stencil_levels2plus_f32"), (5, "stencil_f64"),
            (6, "filter"), (7, "oc"), (9, "coarse_build"), (10, "coarse_inverse"),
            (11, "vector"), (12, "transfer"), (13, "compliance"), (14, "learned_warm_start"),
            (15, "coarse_tail")]
ROOFLINE_KERNEL = {1: "k_fine_zstream FP64 residual b - K u",
                   2: "k_fine_zpair FP32 K.u (inner PCG)",
                   3: "k_fine_zpair FP32 fine sweep (BF16 densities): damped Jacobi and the "
                      "V-cycle residual",
                   8: "k_stencil_apply FP32 level 1 (3 Jacobi sweeps + 1 residual per V-cycle)"}

# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum of one
# ncu --set full capture of the k_fine_zpair Jacobi sweep on this bench's
# 160x80x80 workload: 41.16 MB read, 0.02 MB written)
NCU_TRAFFIC = {(3, (160, 80, 80)): 41180000}


def _fine_bytes(kind, size=None):
    """Algorithmic HBM bytes of one launch of a kernel family."""
    nx, ny, nz = size or SIZE
    if kind == 8:    # level-1 stencil: 14 stored 3x3 FP32 blocks per node + vectors
        nn1 = (nx // 2 + 1) * (ny // 2 + 1) * (nz // 2 + 1)
        jac = 14 * 9 * 4 * nn1 + 4 * 4 * 3 * nn1     # A, u, b, dinv in; x out
        res = 14 * 9 * 4 * nn1 + 3 * 4 * 3 * nn1     # A, u, b in; r out
        return (3 * jac + res) // 4
    nel = nx * ny * nz
    nnodes = (nx + 1) * (ny + 1) * (nz + 1)
    ndof = 3 * nnodes
    if kind == 3:    # FP32 V-cycle smoother sweep, BF16 densities: u, b, dinv in, y out
        return 4 * 4 * ndof + 2 * nel + nnodes
    if kind == 2:    # FP32 K.u of the inner PCG: u in, y out, FP32 densities
        return 2 * 4 * ndof + 4 * nel + nnodes
    if kind == 1:    # FP64 residual b - K u: u, b in, y out, FP64 densities
        return 3 * 8 * ndof + 8 * nel + nnodes
    raise ValueError(kind)


# uniform-start runs of the same cantilever at other volume fractions than
# the timed one: training data of the benchmark family that never contains
# the timed trajectory itself
TRAIN_VOLFRACS = (0.10, 0.14)


def _train_network(device, args):
    """Train the warm-start network on solver-generated pairs: an optimisation
    run of the same cantilever started from seeded random densities uniform in
    [0.05, 1] smoothed once by the rmin=1.5 filter (--train-iters design
    iterations), plus uniform-start runs at volume fractions 0.10 and 0.14
    (--train-uniform iterations each); one (features, displacement change)
    pair per design iteration, then Adam at lr 1e-3."""
    from topoptlab_gb300 import _lib
    from topoptlab_gb300.learned import LearnedWarmStart
    if args.train_iters <= 0:
        return None, {"trained": False}
    owner = _problem("mixed", device)
    npairs = args.train_iters + len(TRAIN_VOLFRACS) * max(args.train_uniform, 0)
    net = LearnedWarmStart(owner, capacity=npairs, seed=0)
    try:
        gen = _problem("mixed", device)
        rng = np.random.default_rng(0)
        x = rng.uniform(0.05, 1.0, gen.nel)
        xs = gen.filter(x, 0)                      # (H x) / Hs
        gen.set(_lib.TG_FIELD_X, xs)
        gen.set(_lib.TG_FIELD_XPHYS, gen.filter(xs, 0))
        for _ in range(args.train_iters):
            net.record_step(gen)
        gen.close()
        for vf in TRAIN_VOLFRACS if args.train_uniform > 0 else ():
            gen = _problem("mixed", device, volfrac=vf)
            for _ in range(args.train_uniform):
                net.record_step(gen)
            gen.close()
        loss = net.train(epochs=args.train_epochs, lr=1e-3, seed=0)
        params = net.params()
    finally:
        net.close()
        owner.close()
    return params, {"trained": True, "pairs": npairs, "epochs": args.train_epochs,
                    "final_loss": loss, "optimizer": "Adam lr 1e-3",
                    "data": f"{args.train_iters} design iterations from seeded random densities "
                            f"U[0.05,1] smoothed by the rmin=1.5 filter, and {args.train_uniform} "
                            f"from uniform starts at each volume fraction {TRAIN_VOLFRACS} "
                            f"(the timed trajectory, volume fraction {VOLFRAC}, is not in it)"}


def _run_heat_batch(device, steps=3, warmup=2):
    """Heat-plate batch: 64 heat plates, nelx = nely uniform in [64, 512] (seed 0), stepped
    concurrently (tg_step_many), mixed precision and plain FP64, each to an
    FP64 relative residual of 1e-8; wall time of whole batch iterations."""
    from topoptlab_gb300.batch import heat_plate_batch, heat_plate_sizes
    sizes = heat_plate_sizes(64, seed=0, nmin=64, nmax=512)
    out = {"workload": "64 heat plates, nelx=nely ~ U{64..512} (seed 0), kmin 1e-3, penal 3, "
                       "volfrac 0.4, rmin 1.5, ft=1, source 0.01 per element, T=0 sink on the "
                       "middle 10% of the left edge, FP64 relative residual 1e-8",
           "elements": int(sum(n * n for n in sizes)), "sizes_min_max": [min(sizes), max(sizes)],
           "odd_sizes_padded": int(sum(n % 2 for n in sizes)), "steps": steps, "warmup": warmup,
           "execution": "one context per design on its own CUDA stream, stepped concurrently "
                        "by a host thread pool (tg_step_many); no learned warm start (the network "
                        "is built for 3-D elasticity)"}
    objs = {}
    for prec in ("mixed", "fp64"):
        batch = heat_plate_batch(sizes, precision=prec, device=device)
        try:
            for _ in range(warmup):
                batch.step()
            t0 = time.perf_counter()
            res = [batch.step() for _ in range(steps)]
            t = time.perf_counter() - t0
        finally:
            batch.close()
        objs[prec] = [[r.obj for r in it] for it in res]
        out[prec] = {"design_iters_per_s": len(sizes) * steps / t,
                     "batch_iteration_ms": 1000.0 * t / steps,
                     "max_rel_res": max(r.rel_res for it in res for r in it),
                     "pcg_iters_mean": float(np.mean([r.pcg_iters for it in res for r in it]))}
    out["ratio_mixed_vs_fp64"] = (out["mixed"]["design_iters_per_s"] /
                                  out["fp64"]["design_iters_per_s"])
    out["compliance_max_rel_diff_vs_fp64"] = max(
        abs(a - b) / abs(b) for ia, ib in zip(objs["mixed"], objs["fp64"]) for a, b in zip(ia, ib))
    return out


def run_ours(args, dist, rank, ws, local):
    from topoptlab_gb300 import _lib
    import ctypes as C
    lib = _lib.load()
    device = local
    prof_kind = int(os.environ.get("TG_BENCH_PROF_KIND", "3"))
    from topoptlab_gb300.learned import LearnedWarmStart

    # ---------------- learned warm start: training (set-up, not timed) ----------------
    t_train0 = time.perf_counter()
    net_params, train_info = _train_network(device, args)
    train_info["seconds"] = time.perf_counter() - t_train0

    # ---------------- learned + mixed precision (headline) ----------------
    prob = _problem("mixed", device)
    net = None
    if net_params is not None:
        net = LearnedWarmStart(prob, capacity=0, seed=0)
        net.set_params(net_params)
        net.attach(prob)
    steps_info = []
    for _ in range(args.warmup):
        prob.step()
    lib.tg_stats(1, None, None, None)
    _barrier(dist)
    with ClockSampler(device) as clk:
        lib.tg_timer(prob._h, 0, None)
        for _ in range(args.steps):
            steps_info.append(prob.step())
        ms = C.c_double()
        lib.tg_timer(prob._h, 1, C.byref(ms))
    t_mixed = ms.value / 1000.0
    launches = C.c_int64()
    lib.tg_stats(1, C.byref(launches), None, None)
    t_max = _max_over_ranks(dist, t_mixed)
    value = args.steps * ws / t_max

    # the roofline kernel: CUDA events around each of its launches on the
    # library's stream, over further design iterations launched directly
    # (CUDA-graph replay is switched off while a kernel family is timed)
    pms, pcount = C.c_double(), C.c_int64()
    lib.tg_profile_kernel(prof_kind)
    for _ in range(max(1, min(args.steps, 3))):
        steps_info.append(prob.step())
    lib.tg_stats(1, None, C.byref(pms), C.byref(pcount))
    lib.tg_profile_kernel(0)

    # device time per kernel family, one further design iteration per family
    families = {}
    tms = C.c_double()
    step_ms = []
    for kind, name in ([] if args.no_breakdown else FAMILIES):
        fms, fcount = C.c_double(), C.c_int64()
        lib.tg_profile_kernel(kind)
        lib.tg_timer(prob._h, 0, None)
        steps_info.append(prob.step())
        lib.tg_timer(prob._h, 1, C.byref(tms))
        lib.tg_stats(1, None, C.byref(fms), C.byref(fcount))
        lib.tg_profile_kernel(0)
        step_ms.append(tms.value)
        families[name] = {"ms": round(fms.value, 4), "launches": int(fcount.value)}
    breakdown = {"method": "CUDA events around each family's launches on the library stream "
                           "(event nodes inside the captured PCG-iteration graphs), one design "
                           "iteration per family; learned_warm_start includes its own FP32 K.u "
                           "launches (also in fine_f32_kmul)",
                 "step_ms_profiled": round(float(np.mean(step_ms)), 3) if step_ms else None,
                 "families": families}

    obj_mixed = [s.obj for s in steps_info]
    if net is not None:
        net.close()
    prob.close()

    # ---------------- end to end through the public API, host buffers ----------------
    # a fresh problem with the same network replays the timed window (the same
    # warm-up, then the same design iterations as `value`, bit for bit), each
    # step with the design copied in from pinned host memory and the densities
    # and the new design copied back
    prob = _problem("mixed", device)
    net = None
    if net_params is not None:
        net = LearnedWarmStart(prob, capacity=0, seed=0)
        net.set_params(net_params)
        net.attach(prob)
    for _ in range(args.warmup):
        prob.step()
    try:
        import torch
        xh = torch.empty(prob.nel, dtype=torch.float64, pin_memory=True).numpy()
        xp = torch.empty(prob.nel, dtype=torch.float64, pin_memory=True).numpy()
    except Exception:
        xh = np.empty(prob.nel)
        xp = np.empty(prob.nel)
    xh[:] = prob.get(_lib.TG_FIELD_X)
    nsteps_e2e = args.steps
    _barrier(dist)
    t0 = time.perf_counter()
    for _ in range(nsteps_e2e):
        prob.set(_lib.TG_FIELD_X, xh)                 # H2D: the design
        prob.step()
        prob.get(_lib.TG_FIELD_XPHYS, out=xp)         # D2H: the physical densities
        prob.get(_lib.TG_FIELD_X, out=xh)             # D2H: the updated design
    t_e2e = _max_over_ranks(dist, time.perf_counter() - t0)
    # the state after design iteration warmup + steps, for the errors against FP64
    fields_mixed = {"x": xh.copy(), "xPhys": xp.copy(), "dc": prob.get(_lib.TG_FIELD_DC),
                    "u": prob.get(_lib.TG_FIELD_U)}
    e2e = {"value": nsteps_e2e * ws / t_e2e, "unit": UNIT,
           "h2d_bytes_per_step": 8 * prob.nel, "d2h_bytes_per_step": 16 * prob.nel,
           "api": "GpuProblem.set/step/get over the C ABI (tg_set, tg_step, tg_get), "
                  "host buffers page-locked, get into them with out=",
           "design_iterations": f"{args.warmup + 1}..{args.warmup + args.steps}, as value"}
    if net is not None:
        net.close()
    prob.close()
    if os.environ.get("TG_BENCH_VERBOSE"):
        for s in steps_info:
            print("learned+mixed", s, file=sys.stderr)

    # ---------------- mixed precision without the network, same iterations ----------------
    probm = _problem("mixed", device)
    for _ in range(args.warmup):
        probm.step()
    lib.tg_timer(probm._h, 0, None)
    minfo = [probm.step() for _ in range(args.steps)]
    ms3 = C.c_double()
    lib.tg_timer(probm._h, 1, C.byref(ms3))
    probm.close()
    t_nolearn = _max_over_ranks(dist, ms3.value / 1000.0)
    value_nolearn = args.steps * ws / t_nolearn

    # ---------------- plain FP64 GMG-PCG, same iterations ----------------
    nplain = 0 if args.no_plain else args.steps
    plain = _problem("fp64", device)
    for _ in range(args.warmup if nplain else 0):
        plain.step()
    lib.tg_timer(plain._h, 0, None)
    pinfo = [plain.step() for _ in range(nplain)] or [steps_info[0]]
    ms2 = C.c_double()
    lib.tg_timer(plain._h, 1, C.byref(ms2))
    fields_plain = {"x": plain.get(_lib.TG_FIELD_X), "xPhys": plain.get(_lib.TG_FIELD_XPHYS),
                    "dc": plain.get(_lib.TG_FIELD_DC), "u": plain.get(_lib.TG_FIELD_U)}
    plain.close()
    if os.environ.get("TG_BENCH_VERBOSE"):
        for s in pinfo:
            print("plain", s, file=sys.stderr)
    t_plain = _max_over_ranks(dist, ms2.value / 1000.0)
    value_plain = (nplain * ws / t_plain) if nplain else float("nan")
    obj_plain = [s.obj for s in pinfo]
    obj_diff = max(abs(a - b) / abs(b) for a, b in zip(obj_mixed, obj_plain))
    # each quantity of the learned+mixed run against the plain FP64 run after
    # the same design iterations: max |a - b| / max |b|
    errors = {"compliance_per_iteration": obj_diff}
    if nplain:
        for k in ("x", "xPhys", "dc", "u"):
            a, b = fields_mixed[k], fields_plain[k]
            errors[k] = float(np.abs(a - b).max() / np.abs(b).max())
    errors["measure"] = ("max |a - b| / max |b| between the learned+mixed run and the plain "
                         f"FP64 run after design iteration {args.warmup + args.steps}; "
                         "compliance: max relative difference over the timed iterations")

    # ---------------- roofline of the dominant kernel ----------------
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    peak_hbm = peaks.get("hbm_gbs", 6800.0)
    avg_s = (pms.value / 1000.0 / pcount.value) if pcount.value else float("nan")
    nbytes = _fine_bytes(prof_kind)
    achieved = nbytes / avg_s / 1e9 if pcount.value else None
    roofline = {"kernel": ROOFLINE_KERNEL.get(prof_kind),
                "bound": "hbm", "achieved": achieved, "peak": peak_hbm, "unit": "GB/s",
                "frac": (achieved / peak_hbm) if achieved else None,
                "traffic": NCU_TRAFFIC.get((prof_kind, tuple(SIZE))),
                "traffic_note": "DRAM bytes of one ncu capture; the 12.7 MB of writes of a "
                                "launch stay in L2 when it ends" if prof_kind == 3 else None,
                "launches": pcount.value,
                "avg_launch_us": avg_s * 1e6 if pcount.value else None,
                "algorithmic_bytes_per_launch": nbytes,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if peaks else "fallback"}

    heat = None if args.no_heat_batch else _run_heat_batch(device)

    if rank != 0:
        return None
    mean = lambda k, L: float(np.mean([getattr(s, k) for s in L]))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64+f32+bf16", "data": "synthetic",
        "config": {"workload": "3-D hex8 cantilever 160x80x80 (1,024,000 elements, "
                               "3,168,963 DOFs), volfrac 0.12, rmin 1.5, ft=1, OC, "
                               "FP64 relative residual 1e-8",
                   "solver": "mixed-precision GMG-PCG (FP32 V-cycle, BF16 smoother densities, "
                             f"FP64 refinement), 5 levels, {NSMOOTH} damped-Jacobi sweep(s) "
                             f"omega {OMEGA} before and after on the fine level, "
                             f"{NSMOOTH_COARSE} on levels 2-3, level 1 unsmoothed, "
                             "FP32-screened OC, "
                             "learned warm start (3-level 16/32/64 conv encoder-decoder, FP32, "
                             "on its own stream beside the hierarchy build)",
                   "learned_warm_start": train_info,
                   "design_iterations_timed": f"{args.warmup + 1}..{args.warmup + args.steps}",
                   "l2": "working set > L2 (126 MB); no flush",
                   "parallelism": f"replicas x{ws}",
                   "host": _host_info()},
        "e2e": e2e,
        "gpu_launches": int(launches.value),
        "roofline": roofline,
        "plain_fp64": {"value": value_plain, "ms_per_step": 1000.0 * t_plain / args.steps,
                       "pcg_iters_per_step": mean("pcg_iters", pinfo),
                       "max_rel_res": max(s.rel_res for s in pinfo)},
        "learned_mixed": {"pcg_iters_per_step": mean("pcg_iters", steps_info[:args.steps]),
                          "refinements_per_step": mean("refinements", steps_info[:args.steps]),
                          "fallbacks": int(sum(s.fallback for s in steps_info[:args.steps])),
                          "warm_start_residual_ratio_mean": mean("warm_ratio",
                                                                 steps_info[:args.steps]),
                          "max_rel_res": max(s.rel_res for s in steps_info),
                          "solve_ms_per_step": mean("t_solve_ms", steps_info[:args.steps])},
        "mixed_without_network": {"value": value_nolearn,
                                  "ms_per_step": 1000.0 * t_nolearn / args.steps,
                                  "pcg_iters_per_step": mean("pcg_iters", minfo),
                                  "max_rel_res": max(s.rel_res for s in minfo)},
        "ratio_vs_plain_fp64": value / value_plain,
        "compliance_max_rel_diff_vs_fp64": obj_diff,
        "errors_vs_fp64": errors,
        "clocks": clk.summary(),
        "time_breakdown": breakdown,
    }
    if heat is not None:
        line["heat_plate_batch"] = heat
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(steps=2, warmup=1)
    return line


def _cpu_step_factory(size=CPU_SAMPLE):
    """One design iteration of the reference algorithm on the CPU (oracle port:
    COO->CSR assembly, Dirichlet slicing, SciPy SuperLU spsolve, compliance,
    sensitivity / density filter, OC), state carried between calls."""
    from oracle import topopt as O
    nx, ny, nz = size
    KE = O.ke_elast(3)
    fixed, f = O.bc_cantilever_3d(nx, ny, nz)
    edof = O.edofmat_vec(nx, ny, nz, 3)
    H, Hs = O.filter_matrix_vec(nx, ny, nz, RMIN)
    ndof = f.shape[0]
    nel = nx * ny * nz
    free = np.setdiff1d(np.arange(ndof), fixed)
    st = {"x": np.full(nel, VOLFRAC), "xPhys": np.full(nel, VOLFRAC), "g": 0.0}
    dv = np.asarray(H @ (np.ones(nel) / Hs))

    def step():
        K = O.assemble(KE, edof, O.simp(st["xPhys"]), ndof)
        u = O.solve_direct(K, f, free)
        obj, dc, _ = O.compliance_sens(st["xPhys"], u, KE, edof)
        dc = np.asarray(H @ (dc / Hs))
        st["x"], st["g"], _ = O.oc_top88(st["x"], dc, dv, st["g"])
        st["xPhys"] = np.asarray(H @ st["x"]) / Hs
        return obj
    return step, nel


def cpu_baseline(steps=2, warmup=1):
    """The workload itself on the host cores: design iterations of the same
    160x80x80 cantilever with our CPU FP64 GMG-PCG restatement (the GPU
    solver's algorithm, C/OpenMP kernels of oracle/cgmg.c on every host
    thread) and NumPy compliance, filter and OC; the first `warmup` design
    iterations untimed, the next `steps` timed."""
    from oracle import topopt as O
    from oracle import cpu_gmg as CG
    from topoptlab_gb300.example_bc import cantilever_3d
    nx, ny, nz = SIZE
    ndof = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    _, f, fixed, _, _ = cantilever_3d(nx, ny, nz, ndof)
    loop = CG.CpuDesignLoop(nx, ny, nz, O.ke_elast(3), fixed, f[:, 0], VOLFRAC, RMIN)
    for _ in range(warmup):
        loop.step()
    res, times = [], []
    for _ in range(steps):
        t0 = time.perf_counter()
        res.append(loop.step())
        times.append(time.perf_counter() - t0)
    t = float(np.mean(times))
    pcg = float(np.mean([r["pcg_iters"] for r in res]))
    nth = CG.threads()
    return {"value": 1.0 / t, "unit": UNIT, "cores": nth, "kind": "port",
            "sample": f"design iterations {warmup + 1}..{warmup + steps} of the same "
                      f"{nx}x{ny}x{nz} cantilever (uniform start) with our CPU FP64 GMG-PCG "
                      f"restatement (C/OpenMP on {nth} threads, 5 levels, the GPU solver's "
                      f"algorithm) and NumPy compliance / filter / OC: {t:.2f} s per design "
                      f"iteration, {pcg:.1f} PCG iterations per design iteration",
            "seconds_per_design_iteration": t, "pcg_iters_per_step": pcg,
            "seconds_per_pcg_iteration_incl_setup": t / max(pcg, 1.0),
            "max_rel_res": max(float(r["rel_res"]) for r in res),
            "host": _host_info()}


def _ref_nonsolve_at_workload(size=None):
    """The reference algorithm's functions of one design iteration other than
    the solve, each timed once at the full grid on the host (oracle port,
    single-threaded NumPy / SciPy like the reference): edofMat
    (trilinear_hexahedron.py:7-58), COO assembly + CSR conversion
    (fem.py:141-178), Dirichlet slicing K[free][:, free] (fem.py:208-237),
    compliance + sensitivities (objectives.py:51-55,
    topology_optimization.py:491-500), the distance-filter matrix
    (matrix_filter.py:101-232), the sensitivity filter, the OC bisection
    (optimality_criterion.py:59-79) and the density filter, at the uniform
    start with a seeded random displacement (the solve's output is not
    needed for timing)."""
    from oracle import topopt as O
    nx, ny, nz = size or SIZE
    nel = nx * ny * nz
    KE = O.ke_elast(3)
    fixed, f = O.bc_cantilever_3d(nx, ny, nz)
    ndof = f.shape[0]
    free = np.setdiff1d(np.arange(ndof), fixed)
    x = np.full(nel, VOLFRAC)
    t = {}

    def timed(key, fn):
        t0 = time.perf_counter()
        r = fn()
        t[key] = time.perf_counter() - t0
        return r
    edof = timed("edofmat", lambda: O.edofmat_vec(nx, ny, nz, 3))
    K = timed("assembly", lambda: O.assemble(KE, edof, O.simp(x), ndof))
    timed("dirichlet_slicing", lambda: K[free][:, free])
    del K
    u = np.random.default_rng(0).standard_normal(ndof)
    _, dc, _ = timed("compliance_and_sensitivities", lambda: O.compliance_sens(x, u, KE, edof))
    H, Hs = timed("filter_matrix", lambda: O.filter_matrix_vec(nx, ny, nz, RMIN))
    dv = np.ones(nel)
    dcf, dvf = timed("sensitivity_filter", lambda: (np.asarray(H @ (dc / Hs)),
                                                   np.asarray(H @ (dv / Hs))))
    xn, _, nsteps = timed("oc_bisection", lambda: O.oc_top88(x, dcf, dvf, 0.0))
    timed("density_filter", lambda: np.asarray(H @ xn) / Hs)
    per_iter = (t["assembly"] + t["dirichlet_slicing"] + t["compliance_and_sensitivities"]
                + t["sensitivity_filter"] + t["oc_bisection"] + t["density_filter"])
    return {"grid": f"{nx}x{ny}x{nz}", "seconds": t, "oc_steps": nsteps, "cores": 1,
            "seconds_per_design_iteration_without_solve": per_iter,
            "set_up_once": ["edofmat", "filter_matrix"]}


def run_reference(args, rank):
    """The reference algorithm's CPU path (oracle port: COO assembly, SciPy
    SuperLU, compliance, filter, OC) on the host cores.  The 160x80x80
    workload is out of reach of the direct solve (fill grows like nel^~2), so
    each step is one design iteration of one grid of a ladder (16x8x8,
    24x12x12, 32x16x16, in turn); the seconds per iteration of each grid are
    fitted as a * nel^b and `value` is that fit at 1,024,000 elements -- an
    extrapolation, labelled as such.  ms_per_step is the measured mean time of
    the steps run here."""
    if rank != 0:
        return None
    t_setup = time.perf_counter()
    steps = {s: _cpu_step_factory(s) for s in REF_LADDER}
    t_setup = time.perf_counter() - t_setup
    per = {s: [] for s in REF_LADDER}
    t_timed = 0.0
    t_run0 = time.perf_counter()
    for i in range(args.warmup + args.steps):
        s = REF_LADDER[i % len(REF_LADDER)]
        t0 = time.perf_counter()
        steps[s][0]()
        t = time.perf_counter() - t0
        if i >= args.warmup:
            per[s].append(t)
            t_timed += t
    t_run = time.perf_counter() - t_run0
    nonsolve = None
    if not args.no_ref_nonsolve:
        try:
            nonsolve = _ref_nonsolve_at_workload()
        except (MemoryError, ValueError, RuntimeError) as e:   # the ladder line stands
            nonsolve = {"unavailable": f"{type(e).__name__}: {e}"}
    nel = np.array([float(np.prod(s)) for s in REF_LADDER])
    sec = np.array([statistics.median(per[s]) if per[s] else float("nan") for s in REF_LADDER])
    ok = np.isfinite(sec)
    b, loga = np.polyfit(np.log(nel[ok]), np.log(sec[ok]), 1)
    full = float(np.prod(SIZE))
    t_full = float(np.exp(loga) * full ** b)
    value = 1.0 / t_full
    ms = 1000.0 * t_timed / max(args.steps, 1)
    ladder = {"x".join(map(str, s)): {"elements": int(np.prod(s)), "steps": len(per[s]),
                                      "seconds_per_iteration": float(sec[k])}
              for k, s in enumerate(REF_LADDER)}
    sample = (f"each step one design iteration of the reference algorithm on one grid of the "
              f"ladder {', '.join('x'.join(map(str, s)) for s in REF_LADDER)} in turn; seconds "
              f"per iteration fitted as {np.exp(loga):.3e} * nel^{b:.3f} and evaluated at "
              f"{int(full)} elements ({t_full:.0f} s per design iteration, extrapolated)")
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "3-D hex8 cantilever 160x80x80 (1,024,000 elements), "
                               "volfrac 0.12, rmin 1.5, ft=1, OC",
                   "solver": "SciPy SuperLU direct solve (reference default scipy-direct)",
                   "value_is": "extrapolated from the measured ladder (the direct solve at "
                               "160x80x80 does not fit a bench run)",
                   "ladder": ladder, "fit_exponent": float(b),
                   "fit_seconds_at_workload": t_full,
                   "ms_per_step_is": "measured mean wall time of the timed ladder steps",
                   "timed_seconds": t_timed, "run_seconds": t_run, "setup_seconds": t_setup,
                   "nonsolve_at_workload": nonsolve,
                   "host": _host_info()},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ref-nonsolve", action="store_true",
                    help="reference arm: skip timing the non-solve functions at 160x80x80")
    ap.add_argument("--train-iters", type=int, default=200,
                    help="design iterations recorded to train the warm-start network")
    ap.add_argument("--train-uniform", type=int, default=40,
                    help="design iterations recorded from each uniform-start training run")
    ap.add_argument("--train-epochs", type=int, default=10)
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain FP64 arm (profiling runs only)")
    ap.add_argument("--no-heat-batch", action="store_true",
                    help="skip the batched heat-plate measurement")
    ap.add_argument("--no-breakdown", action="store_true",
                    help="skip the per-family time breakdown (profiling runs only)")
    ap.add_argument("--size", default=None,
                    help="override the grid, e.g. 80,40,40 (profiling runs only)")
    args = ap.parse_args()
    if args.size:
        global SIZE
        SIZE = tuple(int(v) for v in args.size.split(","))
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else max(args.warmup, 1)
    dist, rank, ws, local = _dist()
    if args.impl == "reference":
        line = run_reference(args, rank)
    else:
        line = run_ours(args, dist, rank, ws, local)
    if line is not None:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
