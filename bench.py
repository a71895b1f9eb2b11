"""Benchmark: MLUPS of the chemical-potential multiphase D3Q19 MRT step.

Default workload (N=1): the 512^3 precision configuration -- RKS EOS at
T/Tc = 0.75, z walls, droplet radius 100, FUSED scheme with FP16 population
storage (the headline configuration; its 5.9 GB state is far larger than
the 129 MB L2, so no L2 flush is needed between steps).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload c3|c2|c1|c4|c3ref] [--storage f16|bf16|f32] [--scheme fused|plain]
                    [--tile ty,tz,xl[,np[,form]]] [--profile-case X,Y,Z]

Under torchrun (N > 1) every rank runs an independent replica (the step does
not shard on one GPU per box); value is the sum over ranks, time the max.
``--impl reference`` times the reference's own kernels compiled for the host
(oracle/_ref, FP64, OpenMP over every host core) -- or the FP64 oracle port
when that build is absent -- on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import importlib
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

METRIC = "MLUPS (lattice updates/s / 1e6), FP16-storage fused step"


def metric_name(args) -> str:
    """The headline metric for the default scheme and storage; the same unit
    named after the scheme and storage actually run otherwise."""
    if args.scheme == "fused" and args.storage == "f16":
        return METRIC
    names = {"f16": "FP16", "bf16": "BF16", "f32": "FP32", "f64": "FP64"}
    return f"MLUPS (lattice updates/s / 1e6), {names[args.storage]}-storage {args.scheme} step"
Q = 19

WORKLOADS = {
    # configs of the benchmark set; sizes and physics as stated
    "c3": dict(name="precision_512cube_rks_fp16", dx=512, dy=512, dz=512, model=205, tr=0.75,
               radius=100.0, width=10.0, wall_mode=1, base_pt=-0.04, k=0.2, ka=0.001, tau=0.8),
    "c2": dict(name="wetting_128x128x96_prw", dx=128, dy=128, dz=96, model=202, tr=0.7,
               radius=30.0, width=10.0, wall_mode=1, base_pt=-0.04, k=0.2, ka=0.001, tau=0.8,
               centre=(64.0, 64.0, 3.0)),
    "c4": dict(name="batched_96_boxes_48to112cube_fp16", batch=96, seed=0),
    # the reference's own defaults (CP-PRW, T/Tc 0.7) on the largest cube its
    # 32-bit population index allows (19 N < 2^31): the grid on which the
    # reference's CUDA step is timed on this GPU as well
    "c3ref": dict(name="reference_defaults_480cube_prw", dx=480, dy=480, dz=480, model=202, tr=0.7,
                  radius=100.0, width=10.0, wall_mode=1, base_pt=-0.04, k=0.2, ka=0.001, tau=0.8),
    "c1": dict(name="periodic_64cube_cs", dx=64, dy=64, dz=64, model=206, tr=0.85, eos_a=0.5,
               eos_b=4.0, radius=16.0, width=2.0, wall_mode=0, base_pt=0.0, k=0.2, ka=0.01,
               tau=1.0, centre=(32.0, 32.0, 32.0)),
}


def storage_bytes(storage: str) -> int:
    return {"f16": 2, "bf16": 2, "f32": 4, "f64": 8}[storage]


def algorithmic_bytes(scheme: str, storage: str, form: int = 0, kterm: bool = False) -> dict:
    """Algorithmic bytes per lattice update.

    B_LU = 2*19*s + 8 is the step-level unit (every population read and
    written once, one FP32 density written and read once).  Per kernel of the
    FUSED scheme: the fused collide reads and writes 18 moving populations of
    s bytes plus the FP32 rest population, and reads the density (4 B);
    the density pass reads the populations and writes the density.  In the
    two-pass form (form 1) the force pass reads the density and writes the
    FP32 force (12 B; 24 B with grad(rho) for the K1/K2 term), which the
    collide pass reads back."""
    s = storage_bytes(storage)
    b_lu = 2 * Q * s + 8
    if scheme == "fused":
        collide = 2 * (18 * s + 4) + 4
        d = {"step": b_lu, "fused_collide": collide, "density": 18 * s + 4 + 4}
        if form == 1:
            fb = 24 if kterm else 12
            d["fused_collide"] = collide + fb
            d["force"] = 4 + fb
        return d
    r = 8 if storage == "f64" else 4
    return {"step": b_lu, "collide_stream": 2 * Q * r + 12 * r + 1, "macro": Q * r + 4 * r + 1}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_solver(cp, wl: dict, scheme: str, storage: str, device: int):
    kw = {k: v for k, v in wl.items() if k not in ("name", "radius", "width", "centre")}
    s = cp.Solver(scheme=cp.SCHEME[scheme], storage=cp.STORE[storage], device=device, **kw)
    s.set_flow_field(radius=wl["radius"], width=wl["width"], centre=wl.get("centre"))
    return s


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(v: float, ws: int, device: str = "cuda") -> float:
    """The largest of every rank's value (the whole job waits for the
    slowest replica); identity for one rank."""
    if ws <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_mlups(nodes_per_rank: int, steps: int, seconds_max: float, ws: int) -> float:
    """Replicas only: every rank updates its own box of nodes_per_rank nodes,
    so the job's throughput is ws times one rank's, timed by the slowest."""
    return nodes_per_rank * steps / seconds_max / 1e6 * ws


def run_ours(args) -> None:
    import importlib

    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    importlib.import_module("3dcpmpmodel_gb300.build").build()
    cp = importlib.import_module("3dcpmpmodel_gb300")
    wl = WORKLOADS[args.workload]
    if "batch" in wl:
        run_batch(args, wl, cp, torch)
        return
    s = make_solver(cp, wl, args.scheme, args.storage, local)
    n = s.n
    stream = torch.cuda.ExternalStream(s.stream)

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    tile = None
    if args.scheme == "fused":
        if args.tile:
            s.set_tile(*(int(v) for v in args.tile.split(",")))
            tile = s.tile()
        else:
            tile = s.autotune()
    # warm-up (includes graph capture)
    s.step(args.warmup)
    s.sync()
    # ---- timed region: device-resident state, CUDA events on the solver's stream
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    l0 = s.launch_count
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.step(args.steps)
    e1.record(stream)
    e1.synchronize()
    s.sync()
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    launches = s.launch_count - l0
    ms_max = max_over_ranks(ms, ws)
    value = whole_job_mlups(n, args.steps, ms_max / 1e3, ws)

    # ---- per-kernel timing pass (same workload, events around each launch)
    s.kernel_timing(True)
    s.step(args.steps)
    s.sync()
    kt = s.kernel_times()
    s.kernel_timing(False)
    bytes_per = algorithmic_bytes(args.scheme, args.storage, (tile or {}).get("form", 0))
    dom = max(kt.items(), key=lambda kv: kv[1][1])
    dom_name, (dom_launches, dom_ms) = dom
    per_launch_s = dom_ms / dom_launches / 1e3
    units_per_launch = n  # one launch updates every node once
    alg = bytes_per.get(dom_name, bytes_per["step"])
    achieved = alg * units_per_launch / per_launch_s / 1e9
    peaks = measured_peaks()
    traffic, traffic_source = None, None
    tp = os.path.join(ROOT, "profiles", f"{dom_name}_traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            tj = json.load(f)
        key = f"{args.workload}_{args.storage}" + ("_twopass" if (tile or {}).get("form", 0) == 1 else "")
        if key in tj:
            traffic = tj[key]
            traffic_source = ("not measured in this run: " + tj.get("_note", "ncu capture")).strip()
    roofline = {"bound": "hbm", "kernel": dom_name, "achieved": round(achieved, 1),
                "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": round(achieved / peaks["hbm_gbs"], 4),
                "peak_source": peaks["source"], "traffic": traffic, "traffic_source": traffic_source,
                "alg_bytes_per_lu": alg,
                "kernels_ms_per_step": {k: round(v[1] / max(1, v[0]) * (v[0] / args.steps), 4)
                                        for k, v in kt.items()}}

    # ---- end to end through the public API with host buffers:
    # upload a state (DIST, FP32, pinned host) -> K x (step + device
    # diagnostics read back) -> density read back to pinned host.
    e2e = None
    if not args.no_e2e:
        host_f = torch.empty(Q * n, dtype=torch.float32, pin_memory=True).numpy()
        host_r = torch.empty(n, dtype=torch.float32, pin_memory=True).numpy()
        cpl = cp.lib()
        import ctypes as C
        cp._abi.check(cpl.cpmp_get_field(s._h, cp.FIELD["dist"], cp._abi.CPMP_F32,
                                         host_f.ctypes.data_as(C.c_void_p), C.c_size_t(host_f.nbytes)))
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        cp._abi.check(cpl.cpmp_set_field(s._h, cp.FIELD["dist"], cp._abi.CPMP_F32,
                                         host_f.ctypes.data_as(C.c_void_p), C.c_size_t(host_f.nbytes)))
        diag = cp.Diag()
        for _ in range(args.steps):
            cp._abi.check(cpl.cpmp_step(s._h, 1))
            rc = cpl.cpmp_reduce(s._h, C.byref(diag))
            if rc not in (0, cp._abi.CPMP_ERR_NONFINITE):
                cp._abi.check(rc)
        cp._abi.check(cpl.cpmp_get_field(s._h, cp.FIELD["rho"], cp._abi.CPMP_F32,
                                         host_r.ctypes.data_as(C.c_void_p), C.c_size_t(host_r.nbytes)))
        t1 = time.perf_counter()
        dt = max_over_ranks(t1 - t0, ws)
        e2e = {"value": round(whole_job_mlups(n, args.steps, dt, ws), 1), "unit": "MLUPS",
               "h2d_bytes_per_step": int(host_f.nbytes / args.steps),
               "d2h_bytes_per_step": int((host_r.nbytes + args.steps * C.sizeof(cp.Diag)) / args.steps),
               "what": "cpmp_set_field(DIST, pinned FP32) + K x (cpmp_step(1) + cpmp_reduce) + "
                       "cpmp_get_field(RHO, pinned FP32)"}

    # ---- CPU baseline on rank 0 (bounded sample)
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_sample(args, wl)
    s.close()
    # ---- the targets' other terms, measured in the same run outside the timed
    # region (one GPU, the default FUSED FP16 line only)
    targets = None
    if ws == 1 and not args.no_targets and args.scheme == "fused" and args.storage == "f16":
        targets = target_terms(args, wl, cp, torch, local, value)
    if rank == 0:
        line = {
            "metric": metric_name(args), "value": round(value, 1), "unit": "MLUPS", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 arithmetic, " + args.storage + " population storage",
            "data": "synthetic (seeded droplet initial field, no dataset)",
            "config": {"workload": wl["name"], "grid": [wl["dx"], wl["dy"], wl["dz"]],
                       "scheme": args.scheme, "storage": args.storage, "model": wl["model"],
                       "tr": wl["tr"], "tile": tile, "parallelism": f"replicas{ws}",
                       "l2": "state larger than L2 (no flush needed)" if n * 44 > 129e6
                             else "state fits in L2; numbers are L2-resident"},
            "gpu_launches": launches, "clocks": clk, "roofline": roofline, "e2e": e2e,
            "cpu_baseline": cpu, "targets": targets,
        }
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def target_terms(args, wl: dict, cp, torch, device: int, fused_mlups: float) -> dict:
    """The other terms of the benchmark's targets, each on its own workload:
    the PLAIN FP32 form of the same box (the FP16-storage fused solver's
    target is >= 2x its MLUPS), the adjoint-over-forward time of the
    wall-field inversion set-up (96^3 CS box, FP32; target <= 3x) against both
    the PLAIN forward it differentiates and the FUSED FP32 forward, and the
    aggregate MLUPS of the 96-box batch (one persistent launch per step)."""
    out = {}
    s = make_solver(cp, wl, "plain", "f32", device)
    stream = torch.cuda.ExternalStream(s.stream)
    s.step(3)
    s.sync()
    k = max(5, min(args.steps, 20))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.step(k)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / k
    plain = s.n / (ms / 1e3) / 1e6
    s.close()
    out["plain_f32"] = {"value": round(plain, 1), "unit": "MLUPS", "ms_per_step": round(ms, 4), "steps": k,
                        "workload": wl["name"]}
    out["fused_f16_over_plain_f32"] = round(fused_mlups / plain, 3)
    ab = importlib.import_module("3dcpmpmodel_gb300.adjoint_bench")
    steps = 400
    r = ab.measure(steps=steps, size=96)
    out["adjoint"] = {"workload": "wall-field inversion, 96^3 CS T/Tc 0.8, FP32", "steps": steps,
                      "checkpoint_every": int(np.ceil(np.sqrt(steps))),
                      "adjoint_s": r["adjoint_s"], "forward_plain_f32_s": r["forward_s"],
                      "forward_fused_f32_s": r["forward_fused_f32_s"],
                      "adjoint_over_plain_forward": r["value"],
                      "adjoint_over_fused_forward": r["adjoint_over_fused_forward"]}
    wb = WORKLOADS["c4"]
    params, drops = c4_params(cp, "f16", wb["seed"], wb["batch"])
    b = cp.Batch(params)
    for bs, d in zip(b.boxes, drops):
        bs.set_flow_field(**d)
    tile = b.autotune()
    stream = torch.cuda.ExternalStream(b.stream)
    b.step(3)
    b.sync()
    k = 20
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.step(k)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / k
    bv = b.nodes / (ms / 1e3) / 1e6
    out["batch"] = {"workload": wb["name"], "boxes": len(params), "total_nodes": b.nodes, "value": round(bv, 1),
                    "unit": "MLUPS", "ms_per_step": round(ms, 4), "steps": k, "tile": tile,
                    "per_node_rate_over_single_box": round(bv / fused_mlups, 3)}
    b.close()
    return out


def c4_params(cp, storage: str, seed: int = 0, count: int = 96):
    """96 droplet-on-wall boxes: cube edge uniform in 48..112, EOS drawn from
    VdW / CS / PR, T/Tc uniform in 0.6-0.9 snapped to the 0.005 table grid,
    wall potential in the range the reference calibrates to 30-150 degrees
    (FluidCuda.cu:128), FP16 storage; seeded."""
    rng = np.random.default_rng(seed)
    out, drops = [], []
    for _ in range(count):
        L = int(rng.integers(48, 113))
        model = int(rng.choice([201, 206, 202]))
        tr = round(float(rng.uniform(0.6, 0.9)) / 0.005) * 0.005
        base_pt = float(rng.uniform(-0.06, 0.15))
        p = cp.default_params(dx=L, dy=L, dz=L, model=model, tr=tr, base_pt=base_pt,
                              scheme=cp.SCHEME["fused"], storage=cp.STORE[storage])
        out.append(p)
        drops.append(dict(radius=L / 4, width=5.0, centre=(L / 2, L / 2, 3.0)))
    return out, drops


def run_batch(args, wl: dict, cp, torch) -> None:
    params, drops = c4_params(cp, args.storage, wl["seed"], wl["batch"])
    b = cp.Batch(params)
    for s, d in zip(b.boxes, drops):
        s.set_flow_field(**d)
    tile = b.autotune()
    stream = torch.cuda.ExternalStream(b.stream)
    b.step(args.warmup)
    b.sync()
    clocks = ClockSampler(0)
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    l0 = b.launch_count
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.step(args.steps)
    e1.record(stream)
    e1.synchronize()
    b.sync()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    launches = b.launch_count - l0
    value = b.nodes * args.steps / (ms / 1e3) / 1e6
    b.kernel_timing(True)
    b.step(args.steps)
    b.sync()
    kt = b.kernel_times()
    b.kernel_timing(False)
    bytes_per = algorithmic_bytes("fused", args.storage)
    dom_name, (dom_launches, dom_ms) = max(kt.items(), key=lambda kv: kv[1][1])
    alg = bytes_per.get(dom_name, bytes_per["step"])
    achieved = alg * b.nodes / (dom_ms / dom_launches / 1e3) / 1e9
    peaks = measured_peaks()
    bad = sum(1 for d in b.reduce(allow_nonfinite=True) if d["nonfinite"])

    # ---- end to end through the public API with host buffers: every box's
    # populations uploaded from pinned host memory (FP32), K x (one batch step
    # + the device diagnostics of every box read back), every box's density read
    # back to pinned host memory
    e2e = None
    if not args.no_e2e:
        import ctypes as C
        cpl = cp.lib()
        host_f = [torch.empty(Q * s.n, dtype=torch.float32, pin_memory=True).numpy() for s in b.boxes]
        host_r = [torch.empty(s.n, dtype=torch.float32, pin_memory=True).numpy() for s in b.boxes]
        for s, hf in zip(b.boxes, host_f):
            cp._abi.check(cpl.cpmp_get_field(s._h, cp.FIELD["dist"], cp._abi.CPMP_F32,
                                             hf.ctypes.data_as(C.c_void_p), C.c_size_t(hf.nbytes)))
        torch.cuda.synchronize()
        diags = (cp.Diag * len(b.boxes))()
        t0 = time.perf_counter()
        for s, hf in zip(b.boxes, host_f):
            cp._abi.check(cpl.cpmp_set_field(s._h, cp.FIELD["dist"], cp._abi.CPMP_F32,
                                             hf.ctypes.data_as(C.c_void_p), C.c_size_t(hf.nbytes)))
        for _ in range(args.steps):
            b.step(1)
            rc = cpl.cpmp_batch_reduce(b._b, diags, len(b.boxes))
            if rc not in (0, cp._abi.CPMP_ERR_NONFINITE):
                cp._abi.check(rc)
        for s, hr in zip(b.boxes, host_r):
            cp._abi.check(cpl.cpmp_get_field(s._h, cp.FIELD["rho"], cp._abi.CPMP_F32,
                                             hr.ctypes.data_as(C.c_void_p), C.c_size_t(hr.nbytes)))
        dt = time.perf_counter() - t0
        e2e = {"value": round(b.nodes * args.steps / dt / 1e6, 1), "unit": "MLUPS",
               "h2d_bytes_per_step": int(sum(h.nbytes for h in host_f) / args.steps),
               "d2h_bytes_per_step": int((sum(h.nbytes for h in host_r) + args.steps * len(b.boxes) *
                                          C.sizeof(cp.Diag)) / args.steps),
               "what": "cpmp_set_field(DIST, pinned FP32) of every box + K x (cpmp_batch_step(1) + "
                       "cpmp_batch_reduce: every box's diagnostics) + cpmp_get_field(RHO, pinned FP32) of every box"}
    cpu = None if args.no_cpu else cpu_sample(args, batch_sample_workload(wl))
    line = {
        "metric": metric_name(args) + " (aggregate over a batch)", "value": round(value, 1), "unit": "MLUPS",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 arithmetic, " + args.storage + " population storage",
        "data": "synthetic (seeded droplet initial fields, no dataset)",
        "config": {"workload": wl["name"], "boxes": len(params), "total_nodes": b.nodes,
                   "tile": tile, "parallelism": "one persistent launch per step",
                   "l2": "state larger than L2" if b.nodes * 44 > 129e6 else "state fits in L2",
                   "boxes_nonfinite": bad},
        "gpu_launches": launches, "clocks": clk,
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": round(achieved, 1),
                     "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 4),
                     "peak_source": peaks["source"], "traffic": None, "alg_bytes_per_lu": alg,
                     "kernels_ms_per_step": {k: round(v[1] / args.steps, 4) for k, v in kt.items()}},
        "e2e": e2e, "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    b.close()


def ref_state(args, wl: dict):
    """The CPU reference on a bounded sample of the workload: the reference's
    own kernels compiled for the host (oracle/_ref, FP64, OpenMP over every
    host core) where that build exists and the workload has the reference's
    z walls, else the oracle port; the grid is halved along its longest axis
    until it holds at most --cpu-nodes nodes.  Returns (state, kind, grid)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    kind = "reference"
    try:
        if O.build_ref() is None:
            kind = "port"
    except Exception:
        kind = "port"
    if wl["wall_mode"] != 1:
        kind = "port"  # the reference step always has z walls
    dx, dy, dz = wl["dx"], wl["dy"], wl["dz"]
    cap = args.cpu_nodes
    while dx * dy * dz > cap:
        if dx >= dy and dx >= dz:
            dx //= 2
        elif dy >= dz:
            dy //= 2
        else:
            dz //= 2
    model = wl["model"]
    tr = wl["tr"]
    kw = dict(dx=dx, dy=dy, dz=dz, model=model, tr=tr, K=wl["k"], Ka=wl["ka"], tau=wl["tau"],
              base_pt=wl["base_pt"], radius=min(wl["radius"], dz / 3), width=wl["width"],
              wall_mode=wl["wall_mode"])
    if "eos_a" in wl:
        kw["eos_a"], kw["eos_b"] = wl["eos_a"], wl["eos_b"]
    if wl.get("centre") is not None and kind != "reference":
        # the reference's own initialiser always places the droplet at
        # (DX/2, DY/2, R+2); placement does not change the work per update
        kw["centre"] = (dx / 2, dy / 2, min(wl["centre"][2], dz / 2))
    s = O.Setup(**kw)
    g, l = O.coexistence(model, tr, s.eos_a, s.eos_b)
    st = O.State(s, g, l, "ref" if kind == "reference" else "oracle").init()
    return st, kind, (dx, dy, dz)


def host_cores() -> int:
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def cpu_model() -> str:
    """The host CPU's model name as lscpu reports it ("" if unavailable)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
    except (OSError, subprocess.SubprocessError):
        return ""
    for line in out.splitlines():
        if line.startswith("Model name:"):
            return line.split(":", 1)[1].strip()
    return ""


def cpu_sample(args, wl: dict) -> dict:
    """cpu_baseline: the CPU reference (ref_state) stepped for about
    --cpu-seconds after one warm-up step."""
    st, kind, (dx, dy, dz) = ref_state(args, wl)
    st.step(1)
    steps = 0
    t0 = time.perf_counter()
    while True:
        st.step(1)
        steps += 1
        if time.perf_counter() - t0 > args.cpu_seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": round(dx * dy * dz * steps / dt / 1e6, 3), "unit": "MLUPS", "cores": host_cores(),
            "cpu": cpu_model(), "kind": kind,
            "sample": f"{steps} steps of a {dx}x{dy}x{dz} box, same EOS/T/walls, FP64"}


def batch_sample_workload(wl: dict) -> dict:
    """The first box of a batched workload, as a single-box workload (the CPU
    legs time the reference on one box; MLUPS is per lattice update)."""
    rng = np.random.default_rng(wl["seed"])
    L = int(rng.integers(48, 113))
    model = int(rng.choice([201, 206, 202]))
    tr = round(float(rng.uniform(0.6, 0.9)) / 0.005) * 0.005
    base_pt = float(rng.uniform(-0.06, 0.15))
    return dict(name=wl["name"] + "_box0", dx=L, dy=L, dz=L, model=model, tr=tr, radius=L / 4, width=5.0,
                wall_mode=1, base_pt=base_pt, k=0.2, ka=0.001, tau=0.8, centre=(L / 2, L / 2, 3.0))


def run_reference(args) -> None:
    """The reference arm: the CPU reference (ref_state) on every host core,
    W untimed warm-up steps, then K timed steps of the bounded sample."""
    ws, rank, local = dist_env()
    if rank != 0:
        return
    wl = WORKLOADS[args.workload]
    if "batch" in wl:
        wl = batch_sample_workload(wl)
    st, kind, (dx, dy, dz) = ref_state(args, wl)
    st.step(args.warmup)
    t0 = time.perf_counter()
    st.step(args.steps)
    dt = time.perf_counter() - t0
    v = round(dx * dy * dz * args.steps / dt / 1e6, 3)
    cpu = {"value": v, "unit": "MLUPS", "cores": host_cores(), "cpu": cpu_model(), "kind": kind,
           "sample": f"{args.steps} steps of a {dx}x{dy}x{dz} box, same EOS/T/walls, FP64"}
    line = {"metric": metric_name(args), "value": v, "unit": "MLUPS", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded droplet initial field, no dataset)",
            "config": {"workload": wl["name"], "grid": [wl["dx"], wl["dy"], wl["dz"]],
                       "sample_grid": [dx, dy, dz], "parallelism": "host cores"},
            "impl": "reference", "cpu_baseline": cpu,
            "e2e": {"value": v, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_profile_case(args) -> None:
    """A few steps of one box with the workload's physics on a grid of
    --profile-case, for profilers (no timing, no CPU leg); prints the mass."""
    import importlib
    importlib.import_module("3dcpmpmodel_gb300.build").build()
    cp = importlib.import_module("3dcpmpmodel_gb300")
    wl = dict(WORKLOADS[args.workload])
    wl["dx"], wl["dy"], wl["dz"] = (int(v) for v in args.profile_case.split(","))
    wl["radius"] = min(wl["radius"], wl["dz"] / 3)
    wl.pop("centre", None)
    s = make_solver(cp, wl, args.scheme, args.storage, 0)
    if args.tile and args.scheme == "fused":
        s.set_tile(*(int(v) for v in args.tile.split(",")))
    s.step(args.steps)
    s.sync()
    print(json.dumps({"profile_case": [wl["dx"], wl["dy"], wl["dz"]], "steps": args.steps,
                      "tile": s.tile() if args.scheme == "fused" else None, "mass": s.reduce()["mass"]}))
    s.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="c3")
    ap.add_argument("--scheme", choices=["fused", "plain"], default="fused")
    ap.add_argument("--storage", choices=["f16", "bf16", "f32", "f64"], default="f16")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--cpu-nodes", type=int, default=2_000_000)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-targets", action="store_true",
                    help="skip the PLAIN FP32 and adjoint sub-measurements of the default line")
    ap.add_argument("--tile", default="",
                    help="ty,tz,xl[,np[,form]]: this fused tile (form 1: the two-pass step) instead of the "
                         "autotuner's")
    ap.add_argument("--profile-case", default="",
                    help="X,Y,Z: only run --steps steps of a box of this grid with the workload's physics "
                         "(for profilers; no timing)")
    args = ap.parse_args()
    if args.profile_case:
        run_profile_case(args)
        return
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
