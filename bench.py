"""Benchmark: particle-steps/s of the MPM step on the 2d slump at nel=[640,160].

Workload (the scaled-up 2d slump): L=[64.1584,16.0396] m, nel=[640,160],
3x3 points per cell -> 365,024 points, 103,201 nodes; cubic B-spline, finite
strain, FLIP (C_pf=1) with mUSL, F-bar locking fix, damping 0.1, non-associated
Drucker-Prager with softening; nonlocal averaging off (stated explicitly: the
reference's threaded nonlocal pass races, nonlocal.jl:29-35).  Cohesion: the
seeded random field when epgpu.grf is available, else uniform 20 kPa (said in
the JSON line).  A step = one elastoplastic MPM cycle over all points
(worflow.jl:80-82), dt from the reference's CFL rule.

Arms:
  default            the CUDA library through the C ABI (`--precision` mixed_df (default),
                     mixed or fp64); the plain FP64 step is timed beside it and the
                     stress error of the timed run against it is stated
  --impl reference   the reference path on the host cores: the FP64 restatement
                     (oracle/) with all threads (Julia is not installed)
"""
from __future__ import annotations

import argparse
import copy
import json
import math
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "elastoplasm.jl_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "particle-steps/s on GB300: mixed+learned vs plain FP64, at stated stress error"
WORKLOAD = "2d slump nel=[640,160], 3x3 points/cell (365,024 points), elastoplastic step"


def oracle_cohesion(X, cmpr, instr, mesh):
    """The same seeded cohesion field from the CPU restatement (oracle/grf_oracle.py), for the
    reference arm, which runs none of the library's kernels."""
    import grf_oracle
    p = dict(instr["grf"].get("param", {}))
    mean = float(p.get("mean", cmpr["c0"]))
    dim = mesh.dim
    return grf_oracle.field(X, dim, instr["grf"].get("covariance", "gaussian"), list(p.get("Ix", [2.5] * 3))[:dim],
                            mean, float(p.get("cov", 0.3)) * mean, float(p.get("min", cmpr["cr"])),
                            int(p.get("Nh", 5000)), int(p.get("seed", 1234)))


def make_workload(grf_fn=None):
    from epgpu import ic_slump
    fw = {"deform": "finite", "trsfr": "std", "C_pf": 1.0, "musl": True, "locking": True, "damping": 0.1}
    kw = dict(fwrk=fw, nonloc={"status": False, "ls": 0.5})
    field = "uniform 20 kPa"
    try:
        from epgpu import grf  # noqa: F401
        kw["grf"] = {"status": True, "covariance": "exponential",
                     "param": {"Ix": [5.0, 5.0], "mean": 2.0e4, "cov": 0.3, "min": 1.0e3, "seed": 1234}}
        field = "seeded exponential-covariance random field (mean 20 kPa, CoV 0.3, 5 m, >= 1 kPa)"
    except ImportError:
        pass
    ic, cfg = ic_slump([64.1584, 16.0396], [640, 160], ni=3, grf_fn=grf_fn, **kw)
    return ic, cfg, field


def cfl_dt(mesh, cmpr, vmax):
    # get_dt (physics.jl:21-26) without the checkpoint clip
    return 0.5 * max(mesh.h[i] / (vmax[i] + cmpr["c"]) for i in range(mesh.dim))


def profiled(engine, k, seq, vm, steps=10, flush=None):
    """Per-kernel device times over min(k, steps) more steps: the one-step graph captured with a CUDA
    event after every kernel (epgpu_profile), L2 flushed before each step as in the timed steps."""
    import torch
    mesh_dim = len(vm)
    g = [0.0] * (mesh_dim - 1) + [-9.81]
    engine.profile(True)
    for _ in range(min(k, steps)):
        if flush is not None:
            flush.fill_(1.0)
        torch.cuda.synchronize()
        seq.append(cfl_dt(engine.mesh, engine.cmpr, vm))
        vm = engine.step(1, seq[-1], g)
    kt = engine.kernel_times()
    engine.profile(False)
    return kt, vm


# algorithmic bytes (unique reads + writes) per launch of each kernel, 2d, as
# (bytes per point, bytes per node), from the arrays each kernel must touch once.
# FP64 oracle-order step:
ALG_BYTES_FP64_2D = {
    "bin64": (8 * (2 + 3 + 1) + 8 * 2 + 4 + 8 * 3 + 8 * 16, 0),
    "p2g64": (8 * 16 + 8 * 7 + 4 + 4 * 16, 4 + 8 * 5),
    "solve64": (0, 8 * 5 + 2 + 8 * 6),
    "g2p64": (8 * 16 + 4 + 8 * 4, 8 * 4),
    "augm64": (8 * 16 + 4 + 8 * 4 + 4 * 16, 4 + 8 * 5),
    "deform64": (8 * 16 + 4 + 8 * (4 + 1 + 2) + 8 * (4 * 3 + 5), 8 * 2),
    "dJ64": (8 * 16 + 4 + 8 * 3 + 4 * 16, 4 + 8 * 2),
    "elast64": (8 * 16 + 4 + 8 * (4 + 4 + 1 + 6) + 8 * (4 + 4 + 4 + 3 + 3), 8),
    "segsort_nodes": (8 * 16, 4),
    "node_lists": (4 + 4 * 16, 8 * 2),
}
# mixed step (FP32 point streams; F, b_e, accumulated plastic strain as FP64 or as
# FP32 pairs, the same bytes), finite strain, std transfer, mUSL, F-bar, DP, in the fused forms the
# 2d step launches (six kernels: zero, p2g, g2p, vmusl_scan, fbar, cons):
#   p2g   read list dx2 mp v2 Om0 tau3 (10 x 4 B)            nodes: m p2 f2 (atomics)
#   g2p   the grid update inside the tile, then G2P and the mUSL momentum scatter:
#         read list cell dx2 v2 mp; write v2 dx2(next) cell + count   nodes: read m p2 f2 + Dirichlet word;
#                                                                     pm2 (atomics)
#   vmusl_scan  next-step counts -> starts per cell (the mUSL velocity is formed in the F-bar tile)
#   fbar  the mUSL velocity inside the tile, then ∇v, δJ, placement: read list cell dx2 mp; write
#         the slot's ∇v (float4, read back by cons) and the next list + cell   nodes: read m pm2 +
#         Dirichlet word; dJacc (atomic)
#   cons  read list cell dx2 ∇v4 F4 b3 ep1 c0 cr tanphi (8-byte F, b, ep1); write F4 b3 ep1 tau3 dlam
#         nodes: read m dJacc (the nodal δJ formed in the gather)
ALG_BYTES_MIXED_2D = {
    "zero": (0, 20 + 12),                          # m p2 f2 per node, counts (2 parities) + cursor per cell
    "p2g": (40, 20),
    "solve": (0, 22 + 36),
    "g2p": (8 + 8 + 8 + 4 + 8 + 8 + 4, 24 + 8),
    "musl": (8 + 8 + 4 + 8, 8),                    # (separate mUSL scatter) list+cell, offsets, ρΩ, v read
    "vmusl": (0, 22),
    "vmusl_scan": (0, 8),
    "fbar": (20 + 16 + 8, 16 + 4),
    "dJn": (0, 12),
    "cons": (4 + 4 + 8 + 16 + 32 + 24 + 8 + 12 + 32 + 24 + 8 + 12 + 4, 8),
}
# DRAM bytes (read + write) per launch of the mixed_df step kernels on this workload, from one ncu
# capture of an exact-map step (dram__bytes_read.sum + dram__bytes_write.sum, cold caches; command in
# the profile summary of these kernels): the "traffic" of the roofline entry
NCU_DRAM_BYTES_MIXED_DF = {"p2g": 17523968, "g2p": 13693440, "vmusl_scan": 422656, "fbar": 11959040,
                           "cons": 40310272}
# the whole step by the per-point state S and per-node G rule: S = 35 values read or written once
# (x2 v2 F4 b3 tau3 epII dlam c0 phi Om0 read; x2 v2 F4 b3 tau3 epII dlam written), G = 30 values
STEP_BYTES = {"fp64": (35 * 8, 30 * 8), "mixed": (35 * 4, 30 * 4), "mixed_df": (35 * 4, 30 * 4)}


def bf16_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["bf16_tflops"]), "measured bf16_tflops"
    except Exception:
        return 1900.0, "fallback"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    out_dir = None          # --clocks-out; a temporary folder when not given

    def __init__(self, gpu: int):
        import tempfile
        d = Clocks.out_dir or tempfile.gettempdir()
        self.path = os.path.join(d, f"clocks_gpu{gpu}_{os.getpid()}.csv")
        os.makedirs(d, exist_ok=True)
        self.proc = None
        self.gpu = gpu

    def _once(self):
        # one synchronous sample, appended to the file
        try:
            with open(self.path, "a") as f:
                subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                "--format=csv,noheader,nounits"], stdout=f, stderr=subprocess.DEVNULL, timeout=10)
        except Exception:
            pass

    def __enter__(self):
        # a timed region of a few milliseconds is shorter than the sampling period: one sample right
        # before it and one right after it bracket it, the 200 ms sampler covers longer regions
        open(self.path, "w").close()
        self._once()
        try:
            self.f = open(self.path, "a")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        try:
            self.f.close()
        except Exception:
            pass
        self._once()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                c = [x.strip() for x in line.split(",")]
                if len(c) < 9:
                    continue
                try:
                    sm.append(float(c[1]))
                    mx = max(mx, float(c[2]))
                except ValueError:
                    continue
                for n, v in zip(names, c[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo" if os.environ.get("EP_BENCH_GLOO") else "nccl")
    return rank, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_sample(ic, cfg, seconds_budget=20.0, threads=None):
    """The FP64 restatement on the host cores: a bounded number of steps of the same workload."""
    import oracle
    threads = threads or os.cpu_count() or 1
    o = oracle.Oracle(ic, cfg["instr"], threads=threads)
    vmax = ic["mpts"].vmax.copy()
    g = [0.0] * (ic["mesh"].dim - 1) + [-9.81]
    steps, t0 = 0, time.perf_counter()
    while True:
        dt = cfl_dt(ic["mesh"], ic["cmpr"], vmax)
        vmax = o.step(1, dt, g)
        steps += 1
        el = time.perf_counter() - t0
        if el > seconds_budget or steps >= 50:
            break
    o.close()
    return ic["mpts"].nmp * steps / el, threads, steps, el


def run_reference(args, rank, ws):
    if rank != 0:
        return
    ic, cfg, field = make_workload(grf_fn=oracle_cohesion)
    if args.settle > 0:
        import oracle
        o = oracle.Oracle(ic, cfg["instr"], threads=os.cpu_count() or 1)
        o.run(1, args.settle, 10.0, 0.0)
        ic["mpts"] = o.download()
        o.close()
    # W untimed and K timed steps of the whole workload on all host threads (one CPU step is ~40 ms
    # on 16 Grace cores at nel=[640,160])
    import oracle
    threads = os.cpu_count() or 1
    o = oracle.Oracle(ic, cfg["instr"], threads=threads)
    vmax = ic["mpts"].vmax.copy()
    g = [0.0] * (ic["mesh"].dim - 1) + [-9.81]
    for _ in range(args.warmup):
        vmax = o.step(1, cfl_dt(ic["mesh"], ic["cmpr"], vmax), g)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vmax = o.step(1, cfl_dt(ic["mesh"], ic["cmpr"], vmax), g)
    el = time.perf_counter() - t0
    o.close()
    steps = args.steps
    val = ic["mpts"].nmp * steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "particle-steps/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": f"synthetic ({field})",
        "config": {"workload": WORKLOAD, "points": ic["mpts"].nmp, "nodes": ic["mesh"].nnodes},
        "cpu_baseline": {"value": val, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{steps} elastoplastic steps of the full workload on {threads} threads "
                                   "(Julia is not installed; the FP64 C++ restatement of the reference path)"},
        "e2e": {"value": val, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def batch_bench(args, rank, ws, emit=True):
    """The batched ensemble (256 uneven slumps): particle-steps/s of one batch window."""
    import torch
    from epgpu.batch import Batch, slump_ensemble
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    t0 = time.perf_counter()
    ics, instrs, desc = slump_ensemble(n=args.instances, seed=0)
    b = Batch(ics, instrs)
    setup_s = time.perf_counter() - t0
    np_i = np.array([d[3] for d in desc], dtype=np.float64)
    # plastic phase from t = 0 (as the single-slump workload), then the tile autotuner
    b.run(1, args.settle)
    tile, tms = b.autotune(phase=1)
    tuning = b.tuning()
    scheme = b.scheme()
    T = args.settle
    b.run(1, T + 0.01)                                      # warm-up window (the chosen scheme and tile)
    T += 0.01
    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        t, ns = b.run(1, T + args.window)
    st = b.stats()
    ps = float((np_i * ns).sum())
    value = ps / (st["device_ms"] * 1e-3)
    T += args.window
    # the other schemes over the next windows of the same length, for the record
    other = []
    if tuning["kernels_available"]:
        for oth in ("phases", "persistent", "graphs"):
            if oth == scheme:
                continue
            b.set_scheme(oth)
            b.run(1, T + 0.01)
            T += 0.01
            _, ns2 = b.run(1, T + args.window)
            T += args.window
            st2 = b.stats()
            other.append({"scheme": oth, "value": float((np_i * ns2).sum()) / (st2["device_ms"] * 1e-3),
                          "unit": "particle-steps/s"})
    line = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": ws, "steps": int(ns.max()),
        "warmup": 1, "ms_per_step": st["device_ms"] / max(float(ns.mean()), 1.0), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (+f32 pairs)",
        "data": "synthetic slump geometry, seeded exponential-covariance cohesion field per instance",
        "config": {"workload": f"batched ensemble of {args.instances} 2d slumps, nel_x ~ U(40..320), nel_y = nel_x/4, "
                               "2-3 points/cell/direction, friction ~ U(15..35 deg)",
                   "instances": args.instances, "points": int(np_i.sum()), "window_s": args.window,
                   "meshes_drawn_again": int(sum(d[4] for d in desc)),
                   "steps_per_instance": [int(ns.min()), int(ns.max())], "p2g_tile": tile,
                   "autotune_ms_per_batch_step": tms, "scheme": scheme,
                   "autotune_ms_by_scheme": {k: ({str(t): v for t, v in d.items()} if isinstance(d, dict) else d)
                                             for k, d in tuning.items()},
                   "other_schemes": other, "setup_s": setup_s,
                   "l2": "working set > L2 (129 MB)", "precision": "mixed_df", "return_map": "exact"},
        "gpu_launches": None, "batch_graph_launches": st["graph_launches"], "clocks": clk.summary(),
    }
    b.close()
    if rank == 0 and emit:
        print(json.dumps(line))
    return line


def c4_summary(args, rank, ws):
    """A reduced batched ensemble (config 4's draw of uneven 2d slumps, fewer instances) reported beside
    the 2d headline: the rate of the autotuned scheme, the scheme and tile it chose, and the others."""
    a = copy.copy(args)
    a.instances = args.c4_instances
    a.settle = 0.1
    a.window = 0.05
    line = batch_bench(a, rank, ws, emit=False)
    c = line["config"]
    return {"workload": c["workload"], "instances": c["instances"], "points": c["points"],
            "value": line["value"], "unit": "particle-steps/s", "ms_per_batch_step": line["ms_per_step"],
            "scheme": c["scheme"], "p2g_tile": c["p2g_tile"], "other_schemes": c["other_schemes"],
            "steps_per_instance": c["steps_per_instance"], "window_s": a.window}


def c3_bench(args, rank, ws):
    """The 3d slump (nel=[320,80,80], 2x2x2 points per cell): particle-steps/s of the mixed 3d step."""
    import torch
    from epgpu import Engine, ic_slump
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    kw = {"basis": {"which": "gimpm", "how": "undeformed", "ghost": True},
          "fwrk": {"deform": "infinitesimal", "trsfr": "tpic", "C_pf": 0.0, "musl": False, "locking": False,
                   "damping": 0.1},
          "plast": {"status": True, "constitutive": "J2"}, "nonloc": {"status": False, "ls": 0.5}}
    nel = [int(v) for v in args.nel_3d.split(",")]
    ic, cfg = ic_slump([64.1584, 16.0396, 16.0396], nel, ni=2,
                       cmpr_over={"E": 1.0e7, "rho0": 2000.0, "c0": 5.0e4, "Hp": 1.0e5}, **kw)
    setup_s = time.perf_counter() - t0
    mesh, mpts, cmpr = ic["mesh"], ic["mpts"], ic["cmpr"]
    np_ = mpts.nmp
    g = [0.0, 0.0, -9.81]
    instr = dict(cfg["instr"])
    instr["gpu"] = {"precision": args.precision if args.precision != "fp64" else "mixed_df", "jaumann": False,
                    "deterministic": args.deterministic}
    e = Engine(ic, instr)
    e.run(1, args.settle, 10.0, 0.0)
    host0 = e.download()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(engine, k, w, clk=None):
        engine.upload(host0)
        vm = host0.vmax.copy()
        seq = []
        for _ in range(w):
            seq.append(cfl_dt(mesh, cmpr, vm))
            vm = engine.step(1, seq[-1], g)
        ms = 0.0
        if clk:
            clk.__enter__()
        for _ in range(k):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            seq.append(cfl_dt(mesh, cmpr, vm))
            vm = engine.step(1, seq[-1], g)
            ms += engine.stats()["device_ms"]
        if clk:
            clk.__exit__(None, None, None)
        kt, vm = profiled(engine, k, seq, vm, flush=flush)
        return ms, seq, kt

    clk = Clocks(local)
    ms, dts, kt = timed(e, args.steps, args.warmup, clk)
    final = e.download()
    e.close()
    value = np_ * args.steps / (ms * 1e-3)
    tot = sum(v[1] for v in kt.values())
    # the FP64 step beside it (and the error of the timed run against it, same dt sequence)
    instr64 = dict(cfg["instr"])
    instr64["gpu"] = {"precision": "fp64", "jaumann": False}
    e64 = Engine({"mesh": mesh, "mpts": host0.copy(), "cmpr": cmpr}, instr64)
    t64 = 0.0
    for dt in dts:
        e64.step(1, dt, g)
        t64 += e64.stats()["device_ms"]
    b = e64.download()
    e64.close()
    x0 = host0.x
    line = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (+f32 pairs)" if instr["gpu"]["precision"] == "mixed_df" else "f32+f64",
        "data": "synthetic 3d slump geometry, uniform cohesion 50 kPa",
        "config": {"workload": f"3d slump L=[64.1584,16.0396,16.0396], nel={nel}, 2x2x2 points/cell, GIMP "
                               "(ghost), TPIC (PIC), USL, infinitesimal J2 (E=1e7, rho=2000, c0=50 kPa, H=1e5)",
                   "points": np_, "nodes": mesh.nnodes, "setup_s": setup_s, "settle_s": args.settle,
                   "precision": instr["gpu"]["precision"], "deterministic": args.deterministic,
                   "l2": "flushed between timed steps (256 MB write)"},
        "kernel_share": {k: round(v[1] / tot, 4) for k, v in kt.items()},
        "fp64_step": {"ms_per_step": t64 / len(dts), "value": np_ * len(dts) / (t64 * 1e-3),
                      "unit": "particle-steps/s"},
        "speedup_vs_fp64_step": (value / (np_ * len(dts) / (t64 * 1e-3))) if t64 > 0 else None,
        "error_vs_fp64": {"steps": len(dts),
                          "stress_rel_l2": float(np.linalg.norm(final.sig - b.sig) / np.linalg.norm(b.sig)),
                          "displacement_rel_l2": float(np.linalg.norm(final.x - b.x) / max(np.linalg.norm(b.x - x0), 1e-300))},
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line))


def c5_bench(args, rank, ws, emit=True):
    """The 3d slump of config 3 with finite-strain Drucker-Prager (phi = 25 deg) and a seeded cohesion
    field: particle-steps/s of the mixed 3d step with the learned return map (pairs of the exact map
    recorded during the settle, the network trained on the GPU), the exact-map step and the FP64 step
    beside it, and the error of the learned run against the FP64 step replayed with the same dt."""
    import torch
    from epgpu import Engine, ic_slump
    from epgpu.mlp import MLP, lambda_over_2G
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    kw = {"basis": {"which": "gimpm", "how": "undeformed", "ghost": True},
          "fwrk": {"deform": "finite", "trsfr": "tpic", "C_pf": 0.0, "musl": False, "locking": False, "damping": 0.1},
          "nonloc": {"status": False, "ls": 0.5},
          "grf": {"status": True, "covariance": "exponential",
                  "param": {"Ix": [5.0, 5.0, 5.0], "mean": 2.0e4, "cov": 0.3, "min": 1.0e3, "seed": 1234}}}
    phi = 25.0 * np.pi / 180.0
    nel = [int(v) for v in args.nel_3d.split(",")]
    ic, cfg = ic_slump([64.1584, 16.0396, 16.0396], nel, ni=2,
                       cmpr_over={"E": 1.0e7, "rho0": 2000.0, "phi0": phi, "phir": phi}, **kw)
    setup_s = time.perf_counter() - t0
    mesh, mpts, cmpr = ic["mesh"], ic["mpts"], ic["cmpr"]
    np_ = mpts.nmp
    g = [0.0, 0.0, -9.81]
    instr = dict(cfg["instr"])
    prec = args.precision if args.precision != "fp64" else "mixed_df"
    instr["gpu"] = {"precision": prec, "jaumann": False}
    e = Engine(ic, instr)
    learned = args.rmap == "learned"
    net, train = None, None
    if learned:
        net = MLP(seed=args.seed, l2g=lambda_over_2G(cmpr))
        net.record_buffer(args.pairs)
        e.set_return_map(net, "record")
    e.run(1, args.settle, 10.0, 0.0)
    host0 = e.download()
    if learned:
        nrec = e.return_map_stats()["recorded"]
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        it = args.train_iters
        losses = [net.train(iters=it, batch=16384, lr=1e-3, seed=1),
                  net.train(iters=it // 2, batch=16384, lr=2e-4, seed=2),
                  net.train(iters=it // 2, batch=16384, lr=4e-5, seed=3)]
        torch.cuda.synchronize()
        train = {"pairs_recorded": int(nrec), "pairs_kept": int(min(nrec, args.pairs)), "iterations": 2 * it,
                 "batch": 16384, "seconds": time.perf_counter() - t1, "loss": losses}
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(engine, k, w, clk=None):
        engine.upload(host0)
        vm = host0.vmax.copy()
        seq = []
        for _ in range(w):
            seq.append(cfl_dt(mesh, cmpr, vm))
            vm = engine.step(1, seq[-1], g)
        l0 = engine.stats()["launches"]
        ms = 0.0
        if clk:
            clk.__enter__()
        for _ in range(k):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            seq.append(cfl_dt(mesh, cmpr, vm))
            vm = engine.step(1, seq[-1], g)
            ms += engine.stats()["device_ms"]
        if clk:
            clk.__exit__(None, None, None)
        launches = engine.stats()["launches"] - l0
        kt, vm = profiled(engine, k, seq, vm, flush=flush)
        return ms, seq, kt, launches

    clk = Clocks(local)
    if learned:
        e.set_return_map(net, "learned")
    ms, dts, kt, launches = timed(e, args.steps, args.warmup, clk)
    rstats = e.return_map_stats() if learned else None
    final = e.download()
    value = np_ * args.steps / (ms * 1e-3)
    tot = sum(v[1] for v in kt.values())
    exact = final_x = dts_x = None
    if learned:
        e.set_return_map(None, "exact")
        ms_x, dts_x, _, _ = timed(e, args.steps, args.warmup)
        final_x = e.download()
        exact = {"value": np_ * args.steps / (ms_x * 1e-3), "unit": "particle-steps/s", "ms_per_step": ms_x / args.steps}
    e.close()
    instr64 = dict(cfg["instr"])
    instr64["gpu"] = {"precision": "fp64", "jaumann": False}

    def fp64_replay(seq):
        """The FP64 step from the same start state with the same dt sequence."""
        e64 = Engine({"mesh": mesh, "mpts": host0.copy(), "cmpr": cmpr}, instr64)
        tt = 0.0
        for dt in seq:
            e64.step(1, dt, g)
            tt += e64.stats()["device_ms"]
        out = e64.download()
        e64.close()
        return out, tt

    b, t64 = fp64_replay(dts)
    if exact is not None:
        # the exact-map mixed run against the FP64 step: what the lattice's conditioning leaves to any
        # FP32 arithmetic, beside the learned run's error
        bx, _ = fp64_replay(dts_x)
        exact["error_vs_fp64"] = {
            "steps": len(dts_x),
            "stress_rel_l2": float(np.linalg.norm(final_x.tau - bx.tau) / np.linalg.norm(bx.tau)),
            "displacement_rel_l2": float(np.linalg.norm(final_x.x - bx.x) / max(np.linalg.norm(bx.x - host0.x), 1e-300))}
    v64 = np_ * len(dts) / (t64 * 1e-3)
    bf = bf16_peak()
    mlp = None
    if learned and "mlp" in kt:
        nl_, tot_ = kt["mlp"]
        slots = (rstats["learned"] + rstats["fallback"]) / max(args.steps + args.warmup, 1)
        tf = 100608.0 * slots / (tot_ / nl_ * 1e-3) / 1e12
        mlp = {"bound": "tensor", "points_per_launch": slots, "avg_launch_ms": tot_ / nl_, "achieved": tf,
               "unit": "TFLOP/s", "peak": bf[0], "frac": tf / bf[0], "peak_source": bf[1]}
    line = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (+f32 pairs)" if prec == "mixed_df" else "f32+f64",
        "data": "synthetic 3d slump geometry, seeded exponential-covariance cohesion field (mean 20 kPa, CoV 0.3, "
                "5 m, >= 1 kPa)",
        "config": {"workload": f"3d slump L=[64.1584,16.0396,16.0396], nel={nel}, 2x2x2 points/cell, GIMP "
                               "(ghost), TPIC (PIC), USL, finite-strain DP (phi=25 deg, E=1e7, rho=2000), "
                               + ("learned return map" if learned else "exact return map"),
                   "points": np_, "nodes": mesh.nnodes, "setup_s": setup_s, "settle_s": args.settle,
                   "precision": prec, "l2": "flushed between timed steps (256 MB write)"},
        "gpu_launches": launches,
        "kernel_share": {k: round(v[1] / tot, 4) for k, v in kt.items()},
        "learned_return_map": ({"train": train, "stats": rstats,
                                "fallback_rate": rstats["fallback"] / max(rstats["learned"] + rstats["fallback"], 1),
                                "mlp_roofline": mlp} if learned else None),
        "exact_map_step": exact,
        "fp64_step": {"ms_per_step": t64 / len(dts), "value": v64, "unit": "particle-steps/s"},
        "speedup_vs_fp64_step": value / v64 if t64 > 0 else None,
        "error_vs_fp64": {"steps": len(dts),
                          "stress_rel_l2": float(np.linalg.norm(final.tau - b.tau) / np.linalg.norm(b.tau)),
                          "displacement_rel_l2": float(np.linalg.norm(final.x - b.x) /
                                                       max(np.linalg.norm(b.x - host0.x), 1e-300))},
        "clocks": clk.summary(),
    }
    if rank == 0 and emit:
        print(json.dumps(line))
    return line


def c5_summary(args, rank, ws):
    """The learned return map on a reduced config-5 slump (3d finite-strain DP, where the exact return
    needs an eigen decomposition per point), reported beside the 2d headline: learned, exact-map and
    FP64 step rates, the fallback rate and the error against the FP64 step."""
    a = copy.copy(args)
    a.nel_3d = args.c5_nel
    a.rmap = "learned"
    a.steps = min(args.steps, 20)
    a.warmup = max(min(args.warmup, 5), 3)
    a.pairs = 8_000_000
    line = c5_bench(a, rank, ws, emit=False)
    lr = line["learned_return_map"] or {}
    return {"workload": line["config"]["workload"], "points": line["config"]["points"],
            "learned_step": {"value": line["value"], "unit": "particle-steps/s", "ms_per_step": line["ms_per_step"]},
            "exact_map_step": line["exact_map_step"], "fp64_step": line["fp64_step"],
            "speedup_vs_exact_map": line["value"] / line["exact_map_step"]["value"] if line["exact_map_step"] else None,
            "fallback_rate": lr.get("fallback_rate"), "mlp_roofline": lr.get("mlp_roofline"),
            "error_vs_fp64": line["error_vs_fp64"], "steps": a.steps}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed_df", choices=["fp64", "mixed", "mixed_df"])
    ap.add_argument("--fp64-steps", type=int, default=10,
                    help="steps of the plain FP64 step timed beside the headline (0: skip)")
    ap.add_argument("--no-check", action="store_true",
                    help="skip the stress error of the timed run against the FP64 step")
    ap.add_argument("--rmap", default="learned", choices=["learned", "exact"],
                    help="return map of the mixed step: the learned one (pairs recorded during the settle, "
                         "trained on the GPU) or the exact one")
    ap.add_argument("--pairs", type=int, default=52_000_000, help="record buffer capacity (pairs)")
    ap.add_argument("--pairs-target", type=int, default=50_000_000,
                    help="training-set size: after the settle the exact map keeps recording (from a copy of the "
                         "run past the timed state) until this many pairs exist or --record-limit is reached")
    ap.add_argument("--record-limit", type=float, default=5.0, help="simulated seconds the recording may run to")
    ap.add_argument("--train-iters", type=int, default=3000)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--deterministic", action="store_true",
                    help="mixed step without floating-point atomics (bitwise reproducible)")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "c4", "c5"],
                    help="c2: the nel=[640,160] slump (headline); c3: the 3d slump; c4: the batched ensemble; "
                         "c5: the 3d slump with finite-strain DP and the learned return map")
    ap.add_argument("--nel-3d", default="320,80,80", help="cells of the 3d workloads (c3, c5)")
    ap.add_argument("--instances", type=int, default=256)
    ap.add_argument("--window", type=float, default=0.05, help="simulated seconds timed in the c4 workload")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--settle", type=float, default=0.5,
                    help="simulated seconds of elastoplastic flow run before timing (plastic points appear)")
    ap.add_argument("--no-other-precision", dest="other_precision", action="store_false",
                    help="skip the exact-map 'mixed' (FP64 islands) step timed beside a mixed_df headline")
    ap.add_argument("--c5-nel", default="160,40,40",
                    help="cells of the reduced config-5 slump whose learned-map step is reported beside the 2d "
                         "headline ('' to skip)")
    ap.add_argument("--c4-instances", type=int, default=48,
                    help="instances of the reduced batched ensemble reported beside the 2d headline (0 to skip)")
    ap.add_argument("--clocks-out", default=None,
                    help="folder for the nvidia-smi clock samples (default: a temporary folder)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    Clocks.out_dir = args.clocks_out
    rank, ws = dist_init()
    if args.impl == "reference":
        run_reference(args, rank, ws)
        return
    if args.workload == "c4":
        batch_bench(args, rank, ws)
        return
    if args.workload == "c3":
        c3_bench(args, rank, ws)
        return
    if args.workload == "c5":
        c5_bench(args, rank, ws)
        return
    import torch
    from epgpu import Engine
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ic, cfg, field = make_workload()
    cfg["instr"]["gpu"] = {"precision": args.precision, "jaumann": False, "deterministic": args.deterministic}
    mesh, mpts, cmpr = ic["mesh"], ic["mpts"], ic["cmpr"]
    np_, dim = mpts.nmp, mesh.dim
    g = [0.0] * (dim - 1) + [-9.81]
    learned = args.rmap == "learned" and args.precision != "fp64"
    host0 = mpts.copy()
    x_init = mpts.x.copy()
    e = Engine(ic, cfg["instr"])
    net, train = None, None
    if learned:
        # pairs of the exact return recorded during the settle, then training on the GPU
        from epgpu.mlp import MLP, lambda_over_2G
        net = MLP(seed=args.seed, l2g=lambda_over_2G(cmpr))
        net.record_buffer(args.pairs)
        e.set_return_map(net, "record")
    if args.settle > 0:
        e.run(1, args.settle, 10.0, 0.0)          # the device time loop (epgpu_run) up to t = settle
        host0 = e.download()
    t_rec = args.settle
    if learned:
        # the training set: pairs of the exact FP64 return recorded during the settle and, past the
        # state the timed steps start from (host0, uploaded again before timing), until the configured
        # number of pairs is reached
        while e.return_map_stats()["recorded"] < args.pairs_target and t_rec < args.record_limit:
            t_rec, _ = e.run(1, min(t_rec + 0.25, args.record_limit), 10.0, t_rec)
        nrec = e.return_map_stats()["recorded"]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        l1 = net.train(iters=args.train_iters, batch=16384, lr=1e-3, seed=1)
        l2 = net.train(iters=args.train_iters // 2, batch=16384, lr=2e-4, seed=2)
        l3 = net.train(iters=args.train_iters // 2, batch=16384, lr=4e-5, seed=3)
        torch.cuda.synchronize()
        train = {"pairs_recorded": int(nrec), "pairs_kept": int(min(nrec, args.pairs)),
                 "recorded_from_t_s": 0.0, "recorded_to_t_s": t_rec,
                 "iterations": 2 * args.train_iters, "batch": 16384,
                 "seconds": time.perf_counter() - t0, "loss": [l1, l2, l3]}
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")   # 256 MB > 129 MB L2

    def timed(engine, k, w, clk=None):
        """Upload host0, w warm-up and k timed steps (L2 flushed before each); device ms via CUDA events."""
        engine.upload(host0)
        vm = host0.vmax.copy()
        seq = []
        for _ in range(w):
            seq.append(cfl_dt(mesh, cmpr, vm))
            vm = engine.step(1, seq[-1], g)
        l0 = engine.stats()["launches"]
        ms = 0.0
        barrier(ws)
        torch.cuda.synchronize()
        if clk:
            clk.__enter__()
        try:
            for _ in range(k):
                flush.fill_(1.0)
                torch.cuda.synchronize()
                seq.append(cfl_dt(mesh, cmpr, vm))
                vm = engine.step(1, seq[-1], g)
                ms += engine.stats()["device_ms"]
        finally:
            if clk:
                clk.__exit__(None, None, None)
        torch.cuda.synchronize()
        barrier(ws)
        launches = engine.stats()["launches"] - l0
        kt, vm = profiled(engine, k, seq, vm, flush=flush)
        return ms, seq, launches, kt

    clk = Clocks(local)
    if learned:
        e.set_return_map(net, "learned")
    dev_ms, dts, launches, ktimes = timed(e, args.steps, args.warmup, clk)
    rstats = e.return_map_stats() if learned else None
    tmax = allmax(dev_ms, ws)
    value = ws * np_ * args.steps / (tmax * 1e-3)
    plastic = e.stats()["plastic"]
    final = e.download()
    # dominant kernel and its roofline
    # dominant memory-bound kernel (the network's tensor-core roofline is reported under "mlp")
    table = ALG_BYTES_FP64_2D if args.precision == "fp64" else ALG_BYTES_MIXED_2D
    dom = max(((k, v) for k, v in ktimes.items() if k in table), key=lambda kv: kv[1][1])
    name, (nl, tot) = dom
    avg_ms = tot / max(nl, 1)
    ppt, pnode = table.get(name, (0, 0))
    alg = ppt * np_ + pnode * mesh.nnodes
    peak, peak_kind = peaks()
    achieved = alg / (avg_ms * 1e-3) / 1e9 if alg else None
    sp, sn = STEP_BYTES[args.precision]
    step_bytes = sp * np_ + sn * mesh.nnodes
    step_gbs = step_bytes / (tmax / args.steps * 1e-3) / 1e9
    traffic = NCU_DRAM_BYTES_MIXED_DF.get(name) if args.precision == "mixed_df" else None
    roof = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "traffic": traffic,
            "traffic_note": "DRAM bytes per launch from an ncu capture (cold caches); the working set fits the "
                            "129 MB L2, so traffic can sit below the algorithmic bytes" if traffic else None,
            "peak_source": f"{peak_kind} hbm_gbs", "alg_bytes_per_launch": alg,
            "avg_launch_ms": avg_ms,
            "kernel_share": {k: round(v[1] / sum(x[1] for x in ktimes.values()), 4) for k, v in ktimes.items()},
            "step": {"alg_bytes": step_bytes, "achieved_gbs": step_gbs, "frac": step_gbs / peak}}
    if learned and "mlp" in ktimes:
        # the network on the tensor cores: 2 (6*128 + 3*128^2 + 128*3) flop per evaluated point; the
        # kernel timed alone on the step's row count (CUDA events over 20 launches), and its span in the
        # step between the events of the profiled step graph (which adds the kernel boundaries)
        nl_, tot_ = ktimes["mlp"]
        slots = (rstats["learned"] + rstats["fallback"]) / max(args.steps + args.warmup, 1)
        alone = net.time_forward(max(int(round(slots)), 1), 20)
        tf = 100608.0 * slots / (alone * 1e-3) / 1e12
        bf = bf16_peak()
        roof["mlp"] = {"bound": "tensor", "points_per_launch": slots, "avg_launch_ms": alone,
                       "achieved": tf, "unit": "TFLOP/s", "peak": bf[0], "frac": tf / bf[0],
                       "peak_source": bf[1], "timing": "the forward kernel alone on the step's rows",
                       "in_step_span_ms": tot_ / nl_,
                       "in_step_frac": 100608.0 * slots / (tot_ / nl_ * 1e-3) / 1e12 / bf[0]}
    # the headline run's FP64 conservation sums at its start (host0) and end
    cons_end = e.conservation()
    e.upload(host0)
    cons_start = e.conservation()
    # the exact-map mixed step beside the learned one
    exact = None
    exact_final, exact_dts = None, None
    if learned:
        e.set_return_map(None, "exact")
        ms_x, exact_dts, _, _ = timed(e, args.steps, args.warmup)
        exact_final = e.download()
        exact = {"value": ws * np_ * args.steps / (allmax(ms_x, ws) * 1e-3), "unit": "particle-steps/s",
                 "ms_per_step": ms_x / args.steps}
    # the benchmark spec-conforming precision beside the headline: FP64 islands (F, b_e, plastic strain,
    # isotropic log/exp in FP64), exact return map
    other = None
    if args.precision == "mixed_df" and args.other_precision:
        cfg_m = copy.deepcopy(cfg)
        cfg_m["instr"]["gpu"] = {"precision": "mixed", "jaumann": False, "deterministic": args.deterministic}
        em = Engine({"mesh": mesh, "mpts": host0.copy(), "cmpr": cmpr}, cfg_m["instr"])
        ms_m, mixed_dts, _, _ = timed(em, args.steps, args.warmup)
        other = {"precision": "mixed", "return_map": "exact",
                 "value": ws * np_ * args.steps / (allmax(ms_m, ws) * 1e-3), "unit": "particle-steps/s",
                 "ms_per_step": ms_m / args.steps, "final": em.download(), "dts": mixed_dts}
        em.close()
    # the plain FP64 step beside it, and the error of these runs against the FP64 step replayed with the
    # same dt sequence from the same state (the FP64 step matches the FP64 oracle bit for bit)
    fp64 = None
    check = None
    if args.precision != "fp64" and (args.fp64_steps > 0 or not args.no_check):
        ic64, cfg64, _ = make_workload()
        ic64["mpts"] = host0.copy()
        cfg64["instr"]["gpu"] = {"precision": "fp64", "jaumann": False}
        e64 = Engine(ic64, cfg64["instr"])

        def against_fp64(a, seq):
            """Errors of the final state a of a run with dt sequence seq against the FP64 replay, and the
            relative differences of their FP64 conservation sums."""
            e64.upload(host0)
            for dt in seq:
                e64.step(1, dt, g)
            b = e64.download()
            x0 = x_init                      # displacement and runout since t = 0 (the slump's own geometry)
            c64 = e64.conservation()
            return {
                "steps": len(seq),
                "stress_rel_l2": float(np.linalg.norm(a.tau - b.tau) / np.linalg.norm(b.tau)),
                "displacement_rel_l2": float(np.linalg.norm(a.x - b.x) / max(np.linalg.norm(b.x - x0), 1e-300)),
                "runout_rel": float(abs((a.x[0].max() - x0[0].max()) - (b.x[0].max() - x0[0].max()))
                                    / max(abs(b.x[0].max() - x0[0].max()), 1e-300)),
            }, c64

        if not args.no_check:
            check, c64 = against_fp64(final, dts)
            check["conservation_vs_fp64"] = {
                k: abs(cons_end[k] - c64[k]) / abs(c64[k]) for k in ("mass", "kinetic", "elastic")}
            if exact_final is not None:
                check["exact_map"], _ = against_fp64(exact_final, exact_dts)
            if other is not None:
                other["error_vs_fp64"], _ = against_fp64(other.pop("final"), other.pop("dts"))
        if args.fp64_steps > 0:
            ms64, _, _, _ = timed(e64, args.fp64_steps, 3)
            fp64 = {"value": np_ * args.fp64_steps / (ms64 * 1e-3), "unit": "particle-steps/s",
                    "steps": args.fp64_steps, "ms_per_step": ms64 / args.fp64_steps}
        e64.close()
    if other is not None:
        other.pop("final", None)
        other.pop("dts", None)
    conservation = {
        "sums_end": {k: cons_end[k] for k in ("mass", "kinetic", "elastic")},
        "mass_drift_rel": abs(cons_end["mass"] - cons_start["mass"]) / cons_start["mass"],
        "note": "FP64 fixed-order sums (epgpu_conservation) of the timed run's start and end state; "
                "mass = sum rho*Omega, kinetic = 1/2 sum m |v|^2, elastic = sum 1/2 tau.Del^-1 tau Omega0",
    }
    # end to end through the C ABI with host buffers, every step: the state the step reads and changes up
    # (epgpu_upload_fields), the step, the same arrays down (epgpu_download_fields); the constants
    # (c0, cr, phi, rho0, Omega0, ...) are uploaded once before the timed region
    e2e = None
    if not args.no_e2e:
        import ctypes as C
        from epgpu import abi
        pinned = []

        def pin(a):
            t = torch.from_numpy(np.ascontiguousarray(a.reshape(-1, order="F"))).pin_memory()
            pinned.append(t)
            return t.numpy().reshape(a.shape, order="F")

        hp = host0.copy()
        for k, v in list(hp.__dict__.items()):
            if isinstance(v, np.ndarray) and v.dtype == np.float64:
                setattr(hp, k, pin(v))
        view = abi.mpts_view(hp)
        vm = np.zeros(dim)
        e2 = Engine({"mesh": mesh, "mpts": hp, "cmpr": cmpr}, cfg["instr"])      # the full first upload
        if learned:
            e2.set_return_map(net, "learned")
        moved = sorted(set(e2.fields_read()) & set(e2.fields_changed()))
        mask = abi.mask_of(moved)
        up = down = sum(getattr(hp, f).nbytes for f in moved)
        tot = 0.0
        gv = np.zeros(3)
        gv[:dim] = g
        vbuf = np.zeros(3)
        gp, vp = gv.ctypes.data_as(C.POINTER(C.c_double)), vbuf.ctypes.data_as(C.POINTER(C.c_double))
        for k in range(args.warmup + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            # one host-loop step through the C ABI: the moved arrays in, the step, the moved arrays out
            e2._check(e2.lib.epgpu_step_fields(e2.h, C.byref(view), mask, 1, cfl_dt(mesh, cmpr, vm), gp, mask, vp))
            vm = vbuf[:dim].copy()
            if k >= args.warmup:
                tot += time.perf_counter() - t0
        tot = allmax(tot, ws)
        e2.close()
        e2e = {"value": ws * np_ * args.steps / tot, "unit": "particle-steps/s", "h2d_bytes_per_step": up,
               "d2h_bytes_per_step": down, "fields_moved": moved, "copies_declared": True,
               "api": "epgpu_step_fields (upload of the moved arrays, the step, their download; one call per step)",
               "host_memory": "page-locked (pinned) numpy arrays"}
    cpu = None
    if rank == 0 and ws == 1 and args.cpu_seconds > 0:
        ic2, cfg2, _ = make_workload()
        ic2["mpts"] = host0.copy()
        val, threads, steps, el = cpu_sample(ic2, cfg2, seconds_budget=args.cpu_seconds)
        cpu = {"value": val, "unit": "particle-steps/s", "cores": threads, "kind": "port",
               "sample": f"{steps} elastoplastic steps of the same workload, FP64 restatement on {threads} threads"}
    c5 = c4 = None
    if learned and args.c5_nel and args.workload == "c2":
        e.close()
        c5 = c5_summary(args, rank, ws)
    if args.c4_instances > 0 and args.workload == "c2":
        c4 = c4_summary(args, rank, ws)
    if rank == 0:
        rm = None
        if learned:
            n_eval = rstats["learned"] + rstats["fallback"]
            rm = {"return_map": "learned (BF16 tensor-core MLP, exact-return fallback)",
                  "fallback_rate": rstats["fallback"] / max(n_eval, 1), "points_evaluated": n_eval,
                  "training": train, "exact_map_step": exact,
                  "speedup_vs_exact_map": value / exact["value"] if exact else None}
        line = {
            "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tmax / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp64": "f64", "mixed": "f32+f64", "mixed_df": "f32 (+f32 pairs)"}[args.precision]
            + (" + bf16 MLP" if learned else ""),
            "data": f"synthetic slump geometry ({field})",
            "config": {"workload": WORKLOAD, "precision": args.precision,
                       "return_map": "learned" if learned else "exact", "deterministic": args.deterministic,
                       "points": np_,
                       "nodes": mesh.nnodes, "l2": "flushed between timed steps (256 MB write)",
                       "parallelism": f"replicas x{ws}", "plastic_points_last_step": plastic,
                       "settle_s": args.settle},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
            "error_vs_fp64": check, "fp64_step": fp64, "other_precision": other, "conservation": conservation,
            "speedup_vs_fp64_step": (value / fp64["value"]) if fp64 else None,
            "learned_return_map": rm, "c5_learned_reduced": c5, "c4_batch_reduced": c4,
            "clocks": clk.summary(),
        }
        print(json.dumps(line))


if __name__ == "__main__":
    main()
