"""Benchmark of the XPBD tissue step on GB300.

Workload (default): the kidney-scale block C2 -- 64 x 32(up) x 48 cells, 589,824 Kuhn tets,
105,105 active nodes, per-tet compliance, capsule pressed into the top surface, 20 substeps per
step.  A step is one LCS_Step (one frame: 20 substeps of predict, 6 edge colours, 31 tet colours,
contact, velocity) on one tissue instance.

``value``: steps/s from CUDA events around each frame launch on the library's stream, inputs
resident in HBM, L2 flushed (256 MiB write) before every timed step.  ``e2e``: steps/s of the
public C-ABI call sequence with host buffers (tool command in, node positions out) timed on the
wall clock.  ``--impl reference`` times the reference path's CPU restatement (the reference ships no
CPU solver) on all host cores for the same workload.  ``--gpus N`` runs N independent replicas
(one per rank); a single tissue mesh does not shard.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "XPBD steps/s & constraint proj/s, batched vs plain; adjoint/forward time ratio"
FALLBACK_HBM_GBS = 6800.0


# The CPU baseline: the FP32 restatement of the path in the reference's own operation order (its
# divisions, library power and logarithm, no fused multiply-adds; the oracle's as-written build), on
# the host's cores.  The reference itself has no CPU implementation of the step.
CPU_REFERENCE = ROOT / "oracle" / "_build" / "liboracle_f32w.so"


def measured_peak():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        peaks = json.loads(path.read_text())
        return float(peaks["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic_per_launch(name):
    """Per-launch DRAM bytes of the frame kernel from the committed ncu summary, if one exists."""
    path = ROOT / "profiles" / f"{name}.md"
    if not path.exists():
        return None
    for line in path.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            return float(line.split(":", 1)[1].split()[0])
    return None


def issue_roof(ms_per_launch, name="ncu_batch_frame_c4", schedulers=4):
    """The instruction-issue roof of the batched frame kernel: its warp instructions per launch (from
    the committed ncu summary) issued at one per scheduler per cycle on every SM at the maximum SM
    clock, against the measured launch time."""
    path = ROOT / "profiles" / f"{name}.md"
    instructions = None
    if path.exists():
        for line in path.read_text().splitlines():
            if line.startswith("warp_instructions_per_launch:"):
                instructions = float(line.split(":", 1)[1].split()[0])
    if instructions is None:
        return None
    import torch
    props = torch.cuda.get_device_properties(0)
    sms = props.multi_processor_count
    mhz = 2070.0
    try:
        out = subprocess.run(["nvidia-smi", "--query-gpu=clocks.max.sm", "--format=csv,noheader,nounits", "-i", "0"],
                             capture_output=True, text=True, timeout=20).stdout.split()
        mhz = float(out[0]) if out else mhz
    except (OSError, ValueError, subprocess.TimeoutExpired):
        pass
    limit_ms = instructions / (sms * schedulers * mhz * 1e6) * 1e3
    return {"bound": "issue", "warp_instructions_per_launch": instructions, "issue_limit_ms": limit_ms,
            "ms_per_launch": ms_per_launch, "frac": limit_ms / ms_per_launch, "sms": sms, "sm_max_mhz": mhz}


class ClockSampler:
    """nvidia-smi clock and throttle-reason samples every 50 ms.  The sampler is started, and its
    first sample awaited, before the timed region opens, so nvidia-smi's start-up (which briefly
    holds the driver) falls outside it; the summary keeps the samples taken inside the region (the
    last one before it when the region is shorter than the sampling period)."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.device = device_index
        self.lines, self.proc = [], None
        self.t0 = self.t1 = None
        self.first = threading.Event()

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
            self.first.wait(timeout=10.0)
        except OSError:
            self.proc = None
        self.t0 = time.perf_counter()
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))
            self.first.set()

    def __exit__(self, *exc):
        self.t1 = time.perf_counter()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        inside = [l for t, l in self.lines if self.t0 is not None and self.t0 <= t <= (self.t1 or t)]
        before = [l for t, l in self.lines if self.t0 is not None and t < self.t0]
        use = inside or before[-1:]
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in use:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, flag in zip(names, f[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(inside), "sampled": "inside the timed region" if inside else "just before the timed region"}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def workload_config(args, w, tets, edges, n_active, world):
    """The bench line's `config`: the workload, the same for both arms."""
    return {"workload": w.name, "cells": [64, 32, 48] if args.workload == "c2" else None, "tets": tets,
            "active_nodes": n_active, "lattice_nodes": len(w.grid.positions), "edges": edges,
            "substeps": int(w.params["substeps"]), "parallelism": f"replicas{world}",
            "l2": "flushed before every timed step (256 MiB write)",
            "timing": "CUDA events around each frame launch on the library stream"}


def run_reference_arm(args, world, rank):
    """CPU restatement of the reference path on all host threads, same workload and metric."""
    if rank != 0:
        return
    from genesis_tissue_simulation_gb300 import workloads as W
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    lib = CPU_REFERENCE
    w = W.make(args.workload)
    session = w.open(lib)
    tets, edges = session.tet_count, int(session.functions["LCS_EdgeCount"]())
    try:
        threads = int(session.dll.ORC_Threads())
        for k in range(args.warmup):
            w.command(session, k)
            session.step()
        t0 = time.perf_counter()
        for k in range(args.warmup, args.warmup + args.steps):
            w.command(session, k)
            session.step()
        elapsed = time.perf_counter() - t0
    finally:
        session.close()
    value = args.steps / elapsed
    line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": workload_config(args, w, tets, edges, int((w.grid.active != 0).sum()), world),
            "cpu_baseline": {"value": value, "unit": "steps/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} full steps of {w.name} after {args.warmup} warm-up steps, "
                                       f"CPU restatement in the reference's operation order (FP32, OpenMP within each colour, {threads} threads), "
                                       "wall clock per step (the CPU path has no L2 flush or CUDA events)"},
            "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def call_sequence_wall(name, steps, warmup, lib=None):
    """Wall clock of the plugin call sequence per step (LCS_Step, the rod-phase LCS_DetectCut for the
    blade, LCS_Finalize; both libraries synchronise before LCS_Step returns) on one workload.
    `lib` None: the reference's own CUDA build (oracle/_ref, when it was built on this machine),
    which also reports its own substep timeline (LCS_ProfileRead); the reference ABI has no per-tet
    stiffness, so there the tets take the uniform (E, nu) bake (the arithmetic per step is the
    same).  Otherwise this library, through the workload's own session."""
    reference = lib is None
    import ctypes

    import torch

    from genesis_tissue_simulation_gb300 import workloads as W
    from genesis_tissue_simulation_gb300.native_backend import GraspParams, PlainTissue

    if reference:
        lib = ROOT / "oracle" / "_ref" / "libLiverCudaSim.so"
        if not lib.exists():
            return {"unavailable": "the reference build (oracle/_ref) is not present on this machine"}
    w = W.make(name, steps=warmup + steps + 1)
    p = w.params
    if reference:
        grasp = None
        if p.get("instrument"):
            g = dict(W.DEFAULT_GRASP)
            g["ccd_velocity"] = p["instrument"]["ccd_velocity"]
            grasp = GraspParams(**g)
        m = p["tet_material"]
        s = PlainTissue(w.grid, dt=p["dt"], substeps=p["substeps"], ks=1.0 / p["edge_compliance"], young_pa=m["young_pa"],
                        poisson=m["poisson"], strain_damping_s=p["strain_damping_s"],
                        tear_ratio=(p.get("blade") or {}).get("tear_ratio", 0.0), grasp_params=grasp, dll_path=lib, reference=True)
    else:
        s = w.open(lib)
    try:
        if reference:
            s.set_gravity(*p["gravity"])
            if w.initial_capsule is not None:
                s.set_capsule(w.initial_capsule)
        for k in range(warmup):
            s.step(detect_cut=w.command(s, k))
        torch.cuda.synchronize()
        if reference:
            s.functions["LCS_ProfileEnable"](1)
        t0 = time.perf_counter()
        for k in range(warmup, warmup + steps):
            s.step(detect_cut=w.command(s, k))
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        rc = -1
        if reference:
            substeps = int(p["substeps"])
            ms = np.zeros(3, dtype=np.float32)
            # its timeline is per substep and starts at the first profiled substep of the session
            rc = s.functions["LCS_ProfileRead"](steps * substeps, ms.ctypes.data_as(ctypes.c_void_p))
            s.functions["LCS_ProfileEnable"](0)
    finally:
        s.close()
    out = {"workload": w.name, "wall_steps_per_s": steps / wall, "ms_per_step_wall": 1e3 * wall / steps, "steps": steps}
    if reference:
        out["material"] = "uniform (E, nu) bake (no per-tet stiffness in the reference ABI)"
        if rc == 0:
            out["substep_timeline_ms_per_step"] = float(ms.sum()) / steps
    return out


def workload_measurement(lib, name, steps, warmup, cpu_budget_s=6.0, launch_mode=0):
    """Steps/s of another plain-path workload through the C ABI: device time from the library's
    events around each frame (CUDA events), plus its CPU restatement on all host cores over a
    bounded sample.  C1: 16x8x16 cells, 10 substeps, no tool.  C3: the C2 block with the blade swept
    along its polyline; each step is LCS_Step plus the rod-phase LCS_DetectCut."""
    import ctypes

    import torch

    from genesis_tissue_simulation_gb300 import workloads as W

    w = W.make(name, steps=warmup + steps + 1)
    s = w.open(lib)
    try:
        if launch_mode:   # a fixed launch shape (profiling), else the automatic choice
            assert s.dll.LCS_SetLaunchMode(launch_mode) == 0
        tets, edges = s.tet_count, int(s.functions["LCS_EdgeCount"]())
        for k in range(warmup):
            s.step(detect_cut=w.command(s, k))
        torch.cuda.synchronize()
        s.functions["LCS_ProfileEnable"](1)
        t0 = time.perf_counter()
        for k in range(warmup, warmup + steps):
            s.step(detect_cut=w.command(s, k))
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        ms = np.zeros(3, dtype=np.float32)
        s.check("LCS_ProfileRead", steps, ms.ctypes.data_as(ctypes.c_void_p))
        s.functions["LCS_ProfileEnable"](0)
        revision = s.topology_revision() if w.blade_path else 0
    finally:
        if launch_mode:
            s.dll.LCS_SetLaunchMode(0)
        s.close()
    device_s = float(ms[0]) / 1e3
    substeps = int(w.params["substeps"])
    out = {"workload": w.name, "value": steps / device_s, "unit": "steps/s", "ms_per_step": 1e3 * device_s / steps,
           "wall_steps_per_s": steps / wall, "proj_per_s": steps / device_s * substeps * (edges + tets), "tets": tets,
           "substeps": substeps, "steps": steps, "timing": "CUDA events around each LCS_Step (rod-phase detection timed on the wall clock only)"}
    if w.blade_path:
        out["topology_revision_after"] = int(revision)
    if cpu_budget_s <= 0:
        return out
    # CPU restatement, bounded sample
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    s = w.open(CPU_REFERENCE)
    try:
        threads = int(s.dll.ORC_Threads())
        s.step(detect_cut=w.command(s, 0))
        n, t0 = 0, time.perf_counter()
        while n < steps and time.perf_counter() - t0 < cpu_budget_s:
            s.step(detect_cut=w.command(s, n + 1))
            n += 1
        cpu = n / (time.perf_counter() - t0)
    finally:
        s.close()
    out["cpu_baseline"] = {"value": cpu, "unit": "steps/s", "cores": threads, "kind": "port",
                           "sample": f"steps 2..{n + 1} of {w.name}, CPU restatement FP32 in the reference's operation order, OpenMP {threads} threads"}
    out["gpu_over_cpu"] = out["value"] / cpu
    return out


def cpu_baseline_sample(workload_name, budget_s=15.0, max_steps=40):
    """Time the CPU restatement on a bounded sample of the workload: consecutive steps from the start."""
    from genesis_tissue_simulation_gb300 import workloads as W
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    lib = CPU_REFERENCE
    w = W.make(workload_name)
    session = w.open(lib)
    try:
        threads = int(session.dll.ORC_Threads())
        w.command(session, 0)
        session.step()
        n, t0 = 0, time.perf_counter()
        while n < max_steps and time.perf_counter() - t0 < budget_s:
            w.command(session, n + 1)
            session.step()
            n += 1
        elapsed = time.perf_counter() - t0
    finally:
        session.close()
    return {"value": n / elapsed, "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": f"steps 2..{n + 1} of {w.name} (one warm-up step), CPU restatement FP32 in the reference's operation order, OpenMP {threads} threads, {elapsed:.1f} s"}


def batched_measurement(lib, frames, warmup, plain_sample=16, plain_frames=6, rank=0, world=1):
    """Batched uneven instances: 256 grids with dims U{8..32} x U{4..16}(up) x U{8..32} cells from one
    seed, per-instance log-uniform compliance and capsule path, 10 substeps per frame.

    On N GPUs (torchrun) the instances are split over the ranks by cost (longest processing time,
    no exchange during a frame); each rank times its share, the slowest rank's time counts, and
    the value is all 256 instances' steps over it (strong scaling).  Returns None on ranks > 0.

    Device rate: CUDA events around each graph-replayed frame launch (autotuned launch shape).  The
    packed state (~0.5 GB of node and element tables) exceeds L2, so no flush is added.  End to end:
    the public batch call with the frame's capsule poses from host memory and every instance's node
    positions copied back to host memory.  Plain rate: the single-instance LCS path stepping a
    sample of the same instances, one session each, device time per frame from its own events.
    """
    import ctypes

    import torch

    from genesis_tissue_simulation_gb300 import batch as BT
    from genesis_tissue_simulation_gb300 import workloads as W
    from genesis_tissue_simulation_gb300.native_backend import GraspParams, PlainTissue

    full = BT.make_c4(steps=warmup + 2 * frames + 1)
    shards = BT.shard_instances(BT.instance_costs(full), world)
    w = full.subset(shards[rank]) if world > 1 else full
    grasp = dict(W.DEFAULT_GRASP, ccd_velocity=0.0)
    scale = w.stiffness_scale()
    count = len(full.grids)
    n_active = int(sum(int((g.active != 0).sum()) for g in full.grids))
    with BT.TissueBatch(w.grids, dt=1 / 60, substeps=w.substeps, ks=1e6, strain_damping_s=w.strain_damping_s, stiffness_scale=scale,
                        grasp_params=GraspParams(**grasp), dll_path=lib) as b:
        info = b.info()
        b.set_gravity(0.0, -981.0, 0.0)
        b.set_capsules(w.capsules_at(0))
        tune = b.autotune(trial_steps=2)
        for k in range(warmup):
            b.step_many(w.capsule_array_at(k + 1)[None], use_graph=True)
        torch.cuda.synchronize()
        b.profile(1)
        for k in range(warmup, warmup + frames):
            b.step_many(w.capsule_array_at(k + 1)[None], use_graph=True)
        torch.cuda.synchronize()
        device_s = b.profile_read() / 1e3
        b.profile(0)
        positions = np.empty((b.total_nodes, 3), dtype=np.float32)
        e0 = time.perf_counter()
        for k in range(warmup + frames, warmup + 2 * frames):
            b.step_many(w.capsule_array_at(k + 1)[None], use_graph=True)
            b.positions(out=positions)
        e2e_s = time.perf_counter() - e0
        assert np.isfinite(positions).all(), "non-finite batched state"
        tables = b.element_tables()
        explicit_ms = None
        if tables == "implicit":   # the same frames on the explicit element tables, for comparison
            b.set_element_tables(False)
            b.step_many(w.capsule_array_at(warmup + 2 * frames)[None], use_graph=True)
            torch.cuda.synchronize()
            b.profile(1)
            for k in range(warmup + 2 * frames, warmup + 2 * frames + min(frames, 10)):
                b.step_many(w.capsule_array_at(k + 1)[None], use_graph=True)
            torch.cuda.synchronize()
            explicit_ms = b.profile_read() / min(frames, 10)
            b.profile(0)
            b.set_element_tables(True)
        gathered, gather_s = None, 0.0
        if world > 1:   # the split's only exchange: rank 0 collects every instance's positions
            local = [b.instance_positions(positions, j).copy() for j in range(len(w.grids))]
            g0 = time.perf_counter()
            gathered = BT.gather_instance_positions(shards, local, rank, world)
            gather_s = time.perf_counter() - g0
    counts = torch.tensor([info["nodes"], info["edges"], info["tets"]], dtype=torch.float64, device="cuda")
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([device_s, e2e_s], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(counts)
        device_s, e2e_s = (float(x) for x in t.tolist())
        if rank != 0:
            return None
    info = dict(info, nodes=int(counts[0]), edges=int(counts[1]), tets=int(counts[2]))
    w = full

    # plain path on a size-spread sample of the same instances
    order = np.argsort([g.positions.shape[0] for g in w.grids])
    picks = order[np.linspace(0, count - 1, plain_sample).round().astype(int)]
    plain_ms = []
    for i in picks:
        g = w.grids[i]
        s = PlainTissue(g, dt=1 / 60, substeps=w.substeps, ks=1e6, strain_damping_s=w.strain_damping_s, grasp_params=GraspParams(**grasp), dll_path=lib)
        try:
            mu, kappa = s.tet_stiffness()
            s.set_tet_stiffness(mu * scale[i], kappa * scale[i])
            s.set_gravity(0.0, -981.0, 0.0)
            s.set_capsule(w.capsule_paths[i][0])
            for k in range(4):   # past the automatic launch-shape trials (frames 2-4)
                s.set_capsule(w.capsule_paths[i][k + 1])
                s.step()
            s.functions["LCS_ProfileEnable"](1)
            for k in range(4, 4 + plain_frames):
                s.set_capsule(w.capsule_paths[i][k + 1])
                s.step()
            ms = np.zeros(3, dtype=np.float32)
            s.check("LCS_ProfileRead", plain_frames, ms.ctypes.data_as(ctypes.c_void_p))
            plain_ms.append(float(ms[0]) / plain_frames)
            s.functions["LCS_ProfileEnable"](0)
        finally:
            s.close()
    # the sample is spread evenly over the size order, so its mean stands for the mean instance
    plain_rate = 1e3 / float(np.mean(plain_ms))
    value = count * frames / device_s
    bytes_per_substep = 64 * n_active + 4 * info["tets"]
    achieved = w.substeps * bytes_per_substep / (device_s / frames) / 1e9
    return {
        "workload": "c4: 256 uneven instances, one launch per frame, CUDA graph"
                    + (f", split over {world} GPUs by cost (slowest rank's time)" if world > 1 else ""),
        "value": value, "unit": "instance-steps/s", "ms_per_frame": 1e3 * device_s / frames, "frames": frames,
        "proj_per_s": value * w.substeps * (info["edges"] + info["tets"]) / count,
        "instances": count, "lattice_nodes": info["nodes"], "active_nodes": n_active, "tets": info["tets"],
        "edges": info["edges"], "substeps": w.substeps, "launch": {"mode": tune["mode"], "threads": tune["threads"],
                                                                    "packing": tune["packing"],
                                                                    "autotune_ms_per_frame": tune["ms_per_frame"],
                                                                    "autotune_trials": [[t["mode"], t["threads"], t["packing"], t["element_tables"],
                                                                                         round(t["ms_per_frame"], 3)] for t in tune["trials"]],
                                                                    "element_tables": tables,
                                                                    "explicit_tables_ms_per_frame": explicit_ms},
        "plain_instance_steps_per_s": plain_rate, "plain_sample": f"{len(picks)} instances spread over the size order, "
                                                                  f"{plain_frames} frames each after 4 warm-up frames (past the automatic launch-shape trials)",
        "batched_over_plain": value / plain_rate,
        "e2e": {"value": count * frames / e2e_s, "unit": "instance-steps/s", "h2d_bytes_per_step": 92 * count,
                "d2h_bytes_per_step": 12 * info["nodes"]},
        "l2": "state larger than L2 (no flush)",
        **({"gather": {"instances": len(gathered), "nodes": int(sum(len(p) for p in gathered)), "seconds": gather_s,
                       "how": "torch.distributed.gather_object of each rank's instance positions to rank 0, after the timed frames"}}
           if gathered is not None else {}),
        "roofline": {"bound": "hbm", "achieved": achieved, "unit": "GB/s", "algorithmic_bytes_per_launch": w.substeps * bytes_per_substep,
                     "traffic": ncu_traffic_per_launch("ncu_batch_frame_c4")},
        "issue_roof": issue_roof(1e3 * device_s / frames),
    }


def adjoint_measurement(lib, reps=3):
    """C5 differentiable identification: 32 x 16(up) x 32 cells (98,304 tets), 10 substeps, 50 frames,
    checkpoints every 5 substeps.  Times (wall clock around the synchronous C-ABI calls, after one
    warm-up) the checkpointing forward rollout, the adjoint (recompute + reverse sweep), and the
    plain forward (50 LCS_Step frames) on the same mesh; reports backward / forward."""
    import torch

    from genesis_tissue_simulation_gb300 import diff as D
    from genesis_tissue_simulation_gb300.native_backend import Capsule

    c5 = D.make_c5()
    with c5.open(lib) as t:
        theta = torch.tensor(c5.theta_initial, device="cuda")
        path = torch.tensor(c5.path, device="cuda")
        target = t.forward(torch.tensor(c5.theta_hidden, device="cuda"), path).clone()
        top = torch.tensor(c5.top, device="cuda")
        fwd, bwd = [], []
        for k in range(reps + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            x = t.forward(theta, path)
            t1 = time.perf_counter()
            g = torch.zeros_like(x)
            g[top] = 2.0 * (x[top] - target[top]) / (3 * len(c5.top))
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            grads = t.backward(g)
            t3 = time.perf_counter()
            if k:
                fwd.append(t1 - t0)
                bwd.append(t3 - t2)
        loss = float(((x[top] - target[top]) ** 2).mean())
        info = t.info()
        assert torch.isfinite(grads["theta"]).all() and torch.isfinite(grads["path"]).all()
        # plain forward: the same frames through LCS_Step
        sess = t.session   # its per-tet stiffness is the bake, i.e. the uniform initial estimate's material
        caps = [Capsule(tuple(c5.path[k, :3]), tuple(c5.path[k, 3:]), c5.radius) for k in range(c5.frames + 1)]
        sess.set_capsule(caps[0])
        torch.cuda.synchronize()
        p0 = time.perf_counter()
        for k in range(c5.frames):
            sess.set_capsule(caps[k + 1])
            sess.step()
        torch.cuda.synchronize()
        plain = time.perf_counter() - p0
    f, b = float(np.median(fwd)), float(np.median(bwd))
    frames, substeps = c5.frames, c5.params["substeps"]
    return {"workload": "c5: 32x16x32 cells, 98,304 tets, 10 substeps, 50 frames, checkpoints every 5 substeps",
            "forward_ms": 1e3 * f, "backward_ms": 1e3 * b, "plain_forward_ms": 1e3 * plain, "backward_over_forward": b / f,
            "backward_over_plain_forward": b / plain, "frames_per_s_forward": frames / f, "loss": loss,
            "launch": "grid" if info["grid_launch"] else "one CTA", "ctas": info["ctas"],
            "timing": f"wall clock around each synchronous call, median of {reps} after one warm-up",
            "gradients": "theta [98,304] and capsule path [51, 6]", "substeps": frames * substeps}


def finalize_measurement(lib, calls=50, warmup=3):
    """LCS_Finalize on the C2 lattice after 3 sagging frames: one particle frame pass
    (k_ComputeParticleRot) and one dual-contouring surface rebuild, each its own launch, then a
    stream synchronise; wall clock per call, median.  Device times and DRAM bytes of the two kernels
    come from the committed ncu summaries."""
    from genesis_tissue_simulation_gb300 import workloads as W

    w = W.make("c2", steps=3)
    s = w.open(lib)
    try:
        w.run(s, steps=3)
        times = []
        for k in range(calls + warmup):
            t0 = time.perf_counter()
            s.check("LCS_Finalize")
            if k >= warmup:
                times.append(time.perf_counter() - t0)
        R = s.particle_frames().astype(np.float64)
        surf = s.surface()
    finally:
        s.close()
    gram_err = float(np.abs(np.einsum("nji,njk->nik", R, R) - np.eye(3)).max())
    nodes = len(w.grid.positions)
    ms = 1e3 * float(np.median(times))
    out = {"workload": f"c2 lattice, {nodes:,} nodes ({int((w.grid.active != 0).sum()):,} active), after 3 frames",
           "ms_per_finalize_wall": ms, "frame_nodes": nodes, "surface_triangles": int(len(surf["tri"]) // 3),
           "surface_voxels": int((w.grid.counts > 0).sum()), "surface_edges": int(len(w.grid.surface_edges)),
           "timing": f"wall clock around LCS_Finalize (two launches + stream sync), median of {calls}",
           "max_frame_orthonormality_error": gram_err}
    # the same after 30 frames of the blade workload: cut voxels, walls, internal-face cancellation
    wc = W.make("c3", steps=30)
    s = wc.open(lib)
    try:
        wc.run(s, steps=30)
        times = []
        for k in range(max(calls // 2, 1) + warmup):
            t0 = time.perf_counter()
            s.check("LCS_Finalize")
            if k >= warmup:
                times.append(time.perf_counter() - t0)
        surf = s.surface()
    finally:
        s.close()
    tags = surf["tri"].view(np.uint32)
    out["after_cut"] = {"workload": "c3 blade workload after 30 frames", "ms_per_finalize_wall": 1e3 * float(np.median(times)),
                        "surface_triangles": int(len(tags) // 3), "wall_triangles": int(((tags & 0x40000000) != 0).sum() // 3),
                        "component_vertices": int(((tags & 0x80000000) != 0).sum())}
    for key, name in (("particle_frames", "ncu_particle_frames_c2"), ("surface", "ncu_surface_c2"), ("surface_after_cut", "ncu_surface_c3_cut")):
        path = ROOT / "profiles" / f"{name}.md"
        if not path.exists():
            continue
        entry = {}
        for line in path.read_text().splitlines():
            for field in ("kernel_us_per_launch", "traffic_bytes_per_launch", "algorithmic_bytes_per_launch"):
                if line.startswith(field + ":"):
                    entry[field] = float(line.split(":", 1)[1].split()[0])
        out[key] = entry
    return out


def frames_measurement(lib, calls=50, warmup=3):
    """One particle-frame pass (physics_compute_rotations: k_ComputeParticleRot over every node) on
    the C2 lattice after 3 sagging frames, through GBT_ComputeParticleFrames (launch + stream
    synchronise); wall clock per call, median."""
    from genesis_tissue_simulation_gb300 import workloads as W

    w = W.make("c2", steps=3)
    s = w.open(lib)
    try:
        w.run(s, steps=3)
        fn = s.dll.GBT_ComputeParticleFrames
        times = []
        for k in range(calls + warmup):
            t0 = time.perf_counter()
            assert fn() == 0
            if k >= warmup:
                times.append(time.perf_counter() - t0)
    finally:
        s.close()
    nodes = len(w.grid.positions)
    ms = 1e3 * float(np.median(times))
    return {"workload": f"c2 lattice, {nodes:,} nodes, after 3 frames", "ms_per_pass_wall": ms,
            "nodes_per_s": nodes / (ms / 1e3), "timing": f"wall clock around GBT_ComputeParticleFrames, median of {calls}"}


def cut_topology_measurement(lib, frames=30, warmup=2):
    """The cut topology of the C3 lattice (GBT_CutTopologyBuild: live tets, vertex duplication,
    greedy re-colouring relaxed on the device).  One build before the blade (the session's tables;
    nothing cut), `frames` blade frames, then the first build after them (the relaxation starts from
    the uncut colouring, so every change since the start travels), then `frames` more frames with a
    build after every step (each relaxation starts from the previous step's colouring; a step that
    severed nothing keeps the previous product, and the section counts both kinds of build).  Wall clock
    around the builds and the steps.  Returns the section and the neighbour table of the first build
    after the blade (the CPU baseline leg times the oracle on it)."""
    import ctypes

    from genesis_tissue_simulation_gb300 import workloads as W

    w = W.make("c3", steps=2 * frames + warmup)
    s = w.open(lib)
    counts = np.zeros(4, dtype=np.int32)
    build = lambda: s.check("GBT_CutTopologyBuild", counts.ctypes.data_as(ctypes.c_void_p))
    try:
        build()
        w.run(s, steps=frames)
        t0 = time.perf_counter()
        build()
        first_ms = 1e3 * (time.perf_counter() - t0)
        first = counts.copy()
        nbr = s.neighbors()
        w.run(s, steps=warmup, start=frames)
        build()
        step_ms, build_ms, sweeps = [], [], []
        for k in range(frames + warmup, 2 * frames + warmup):
            t0 = time.perf_counter()
            s.step(detect_cut=w.command(s, k))
            t1 = time.perf_counter()
            build()
            t2 = time.perf_counter()
            step_ms.append(1e3 * (t1 - t0)); build_ms.append(1e3 * (t2 - t1)); sweeps.append(int(counts[3]))
    finally:
        s.close()
    per_step = float(np.mean(step_ms)) + float(np.mean(build_ms))
    rebuilt = [b for b, n in zip(build_ms, sweeps) if n > 0]
    reused = [b for b, n in zip(build_ms, sweeps) if n == 0]
    out = {"workload": f"c3 blade workload, {len(w.grid.positions):,} lattice nodes",
           "first_build_after_frames": frames, "ms_first_build_wall": first_ms, "live_tets": int(first[0]),
           "duplicated_vertices": int(first[1]), "colours": int(first[2]), "relaxation_sweeps": int(first[3]),
           "per_step": {"frames": frames, "ms_build_wall_mean": float(np.mean(build_ms)), "sweeps_mean": float(np.mean(sweeps)),
                        "builds_relaxed": len(rebuilt), "ms_build_wall_mean_relaxed": float(np.mean(rebuilt)) if rebuilt else None,
                        "builds_kept": len(reused), "ms_build_wall_mean_kept": float(np.mean(reused)) if reused else None,
                        "ms_step_wall_mean": float(np.mean(step_ms)), "steps_per_s_with_build": 1e3 / per_step},
           "timing": "wall clock around GBT_CutTopologyBuild (and LCS_Step with the rod-phase detection), host synchronised"}
    return out, nbr


def cut_topology_cpu_sample(nbr, frames=30):
    """CPU baseline of the cut topology: the sequential oracle builds the same product from the same
    neighbour table (one host core)."""
    import ctypes

    from genesis_tissue_simulation_gb300 import workloads as W

    w = W.make("c3", steps=frames)
    o = w.open(str(CPU_REFERENCE))
    try:
        f = o.dll.GBT_SetState
        f.argtypes = (ctypes.c_void_p,) * 8 + (ctypes.c_int, ctypes.c_uint)
        nbr = np.ascontiguousarray(nbr, dtype=np.int32)
        assert f(None, None, nbr.ctypes.data_as(ctypes.c_void_p), None, None, None, None, None, 0, 0) == 0
        counts = np.zeros(4, dtype=np.int32)
        t0 = time.perf_counter()
        o.check("GBT_CutTopologyBuild", counts.ctypes.data_as(ctypes.c_void_p))
        ms = 1e3 * (time.perf_counter() - t0)
    finally:
        o.close()
    return {"value": ms, "unit": "ms per build", "cores": 1, "kind": "port",
            "sample": f"one build of the c3 lattice's cut topology after {frames} blade frames",
            "live_tets": int(counts[0]), "duplicated_vertices": int(counts[1]), "colours": int(counts[2])}


def main():
    parser = argparse.ArgumentParser()
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=30)
    parser.add_argument("--warmup", type=int, default=3)
    parser.add_argument("--impl", default="ours", choices=("ours", "reference"))
    parser.add_argument("--workload", default="c2")
    parser.add_argument("--no-cpu-baseline", action="store_true")
    parser.add_argument("--no-batched", action="store_true")
    parser.add_argument("--no-adjoint", action="store_true")
    parser.add_argument("--no-workloads", action="store_true", help="skip the C1 and C3 lines")
    parser.add_argument("--only", default="all", choices=("all", "batched", "adjoint", "finalize", "frames", "c1", "c3", "cut_topology"),
                        help="run one section alone and print its JSON object (for profiling)")
    parser.add_argument("--batched-frames", type=int, default=20)
    parser.add_argument("--launch-mode", type=int, default=0, choices=(0, 1, 2, 3),
                        help="--only c1/c3: 1 whole GPU, 2 one CTA, 3 one cluster (default: automatic)")
    args = parser.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference_arm(args, world, rank)
        return

    import torch
    import torch.distributed as dist

    from genesis_tissue_simulation_gb300 import build as native_build
    from genesis_tissue_simulation_gb300 import workloads as W

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    if rank == 0 or world == 1:
        native_build.build()
    if world > 1:
        dist.barrier()
    lib = native_build.build()
    if args.only != "all":   # one section alone (profiling runs): its JSON object, no bench line
        section = (batched_measurement(lib, args.batched_frames, max(args.warmup, 3)) if args.only == "batched"
                   else finalize_measurement(lib, calls=max(args.steps, 1), warmup=max(args.warmup, 1)) if args.only == "finalize"
                   else frames_measurement(lib, calls=max(args.steps, 1), warmup=max(args.warmup, 1)) if args.only == "frames"
                   else cut_topology_measurement(lib, warmup=max(args.warmup, 1))[0] if args.only == "cut_topology"
                   else workload_measurement(lib, args.only, max(args.steps, 1), args.warmup, cpu_budget_s=0.0,
                                             launch_mode=args.launch_mode) if args.only in ("c1", "c3")
                   else adjoint_measurement(lib, reps=max(args.steps, 1)))
        print(json.dumps({"only": args.only, **section}), flush=True)
        return

    w = W.make(args.workload, steps=args.warmup + args.steps)
    session = w.open(lib)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    n_active = int((w.grid.active != 0).sum())
    tets = session.tet_count
    edges = int(session.functions["LCS_EdgeCount"]())
    substeps = int(w.params["substeps"])
    try:
        for k in range(args.warmup):
            w.command(session, k)
            session.step()
        torch.cuda.synchronize()
        session.functions["LCS_ProfileEnable"](1)
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        with ClockSampler(torch.cuda.current_device()) as clocks:
            wall0 = time.perf_counter()
            for k in range(args.warmup, args.warmup + args.steps):
                flush.zero_()
                torch.cuda.synchronize()
                w.command(session, k)
                session.check("LCS_Step", session.dt)
            torch.cuda.synchronize()
            wall = time.perf_counter() - wall0
        ms = np.zeros(3, dtype=np.float32)
        session.check("LCS_ProfileRead", args.steps, ms.ctypes.data_as(__import__("ctypes").c_void_p))
        device_s = float(ms[0]) / 1e3
        session.functions["LCS_ProfileEnable"](0)

        # end to end through the public ABI: tool command in from host memory, positions out
        positions = np.empty((len(w.grid.positions), 3), dtype=np.float32)
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        e0 = time.perf_counter()
        for k in range(args.warmup + args.steps, args.warmup + 2 * args.steps):
            w.command(session, min(k, len(w.capsule_path) - 1) if w.capsule_path else k)
            session.check("LCS_Step", session.dt)
            session.check("LCS_Finalize")
            session.check("LCS_GetCornerPos", positions.ctypes.data_as(__import__("ctypes").c_void_p))
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - e0
        assert np.isfinite(positions).all(), "non-finite tissue state"
        # the phase floor: grid barriers per frame launch and one barrier's latency with no work
        barriers = session.frame_barriers()
        barrier_us = session.grid_barrier_floor(20000) if barriers else None
    finally:
        session.close()

    t = torch.tensor([device_s, e2e_s, wall], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    device_s, e2e_s, wall = (float(x) for x in t.tolist())
    batched = None
    if not args.no_batched:   # every rank takes its share of the instances
        batched = batched_measurement(lib, args.batched_frames, max(args.warmup, 3), rank=rank, world=world)
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    value = world * args.steps / device_s
    projections = substeps * (edges + tets)
    bytes_per_substep = 64 * n_active + 4 * tets
    launch_s = device_s / args.steps
    achieved = substeps * bytes_per_substep / launch_s / 1e9
    peak, peak_kind = measured_peak()
    traffic = ncu_traffic_per_launch(f"ncu_frame_kernel_{args.workload}")
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * device_s / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, w, tets, edges, n_active, world),
        "proj_per_s": value * projections, "projections_per_step": projections,
        "wall_steps_per_s": world * args.steps / wall,
        "e2e": {"value": world * args.steps / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": 92 + 4,
                "d2h_bytes_per_step": 12 * len(w.grid.positions) + 12},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind, "algorithmic_bytes_per_launch": substeps * bytes_per_substep},
        "clocks": clocks.summary(),
    }
    if barriers:
        floor_ms = barriers * barrier_us / 1e3
        line["sync_floor"] = {"bound": "grid barrier latency", "barriers_per_launch": barriers, "us_per_barrier": barrier_us,
                              "floor_ms": floor_ms, "ms_per_launch": 1e3 * launch_s, "frac": floor_ms / (1e3 * launch_s),
                              "measured": "GBT_GridBarrierFloor: 20,000 back-to-back barriers on the frame kernel's grid"}
    if not args.no_workloads:
        line["workloads"] = {"c1": workload_measurement(lib, "c1", 100, 5), "c3": workload_measurement(lib, "c3", 30, 3)}
        # the reference's own CUDA build on the same box and plugin call sequence, against ours
        ref = {}
        for key, name, steps in (("c1", "c1", 100), ("c2", args.workload, 30), ("c3", "c3", 30)):
            r = call_sequence_wall(name, steps, 4)   # 4 warm-up frames: past our launch-shape trials
            if "wall_steps_per_s" in r:
                ours = call_sequence_wall(name, steps, 4, lib=lib)
                r["ours_wall_steps_per_s"] = ours["wall_steps_per_s"]
                r["ours_over_reference"] = ours["wall_steps_per_s"] / r["wall_steps_per_s"]
            ref[key] = r
        line["reference_gpu"] = {"timing": "wall clock per step of LCS_Step (+ LCS_DetectCut for the blade) + LCS_Finalize, "
                                           "both libraries on this GPU", **ref}
    if not args.no_adjoint:
        line["adjoint"] = adjoint_measurement(lib)
    if not args.no_workloads:
        line["finalize"] = finalize_measurement(lib)
        line["cut_topology"], cut_nbr = cut_topology_measurement(lib)
    if batched is not None:
        batched["roofline"].update(peak=peak, frac=batched["roofline"]["achieved"] / peak, peak_kind=peak_kind)
        line["batched"] = batched
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample(args.workload)
        if not args.no_workloads:
            line["cpu_baseline"]["cut_topology"] = cut_topology_cpu_sample(cut_nbr)
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
