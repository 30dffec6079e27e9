#!/usr/bin/env python3
"""SSVDAG + CSVDAG build throughput (Mvoxels/s) on one GB300.

Workload: the 2048x2048 fBm heightfield terrain (8 octaves, lacunarity 2,
gain 0.5, heights 0-0.3, skirts + bottom: 8,396,796 float32 triangles) built
at depth 12 (4096^3).  One step = one full build from triangles resident in
HBM: voxelize (GeomOctree::buildSVO) -> SVDAG (toDAG) -> SSVDAG (toSDAG) and
the CSVDAG cross-level merge of the same DAG.  value = voxels per second of
that whole step.  e2e = the same through the C ABI with host buffers:
pinned-host triangles copied in and both result pools copied out every step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU implementation of the same path on the host
cores: the reference's chunked OpenMP build (GeomOctree::buildDAG) followed by
toSDAG and mergeAcrossAllLevels, as restated by the oracle, on a bounded
sample (the first rows of the same terrain) so the run ends in minutes.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "svdag-compression_gb300")
sys.path.insert(0, PKG)

METRIC = "SSVDAG build Mvoxels/s & HBM GB/s, depth 12; lossy nodes saved at <=1% err"
UNIT = "Mvoxels/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--grid", type=int, default=2048)
    ap.add_argument("--levels", type=int, default=12)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-json", default="")
    return ap.parse_args()


def rank_info():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
                except ValueError:
                    continue
        os.unlink(self.f.name)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for _, _, fl in rows for k, v in enumerate(fl) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# algorithmic bytes per kernel family (read + write of the data the algorithm
# must touch once), from the level sizes of the build being timed.
R = 36  # node record: hdr word + 8 child words


def algorithmic_bytes(kernel, info):
    """Bytes one step's launches of `kernel` must move at minimum."""
    lv = info
    if kernel.startswith("k_expand"):
        # per frontier pair: read (tri id, node id) 8 B + triangle 36 B, write hit byte
        return sum(lv["frontier"]) * (8 + 36 + 1)
    if kernel.startswith("k_insert"):
        # read every node key once
        return (sum(lv["svo_inner"]) + sum(lv["dag_inner"])) * R
    if kernel.startswith("k_sdag_candidates"):
        return sum(lv["dag"]) * (R + 8 * 4)
    return None


def run_ours(args, rank, local, world):
    import numpy as np
    import torch

    import svdag_gb300 as sv

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    tris = sv.terrain(args.grid, 8, 0.3, args.seed)
    T = tris.shape[0]
    d_tris = torch.from_numpy(tris).to(dev)
    stream = torch.cuda.Stream(device=dev)
    base = sv.Octree(device=local, stream=stream.cuda_stream)
    base.set_device_triangles(d_tris.data_ptr(), T, keepalive=d_tris)
    have_csv = True

    def step(octree, profile=False):
        nonlocal have_csv
        octree.buildSVO(args.levels)
        octree.toDAG()
        octree.initChildLevels()
        s = octree.clone()
        if profile:
            s.profile(True)
        s.toSDAG()
        c = None
        if have_csv:
            c = octree.clone()
            if profile:
                c.profile(True)
            try:
                c.mergeAcrossAllLevels()
            except sv.SvdagError:
                have_csv = False
                c = None
        return s, c

    for _ in range(max(args.warmup, 0)):
        step(base)
    torch.cuda.synchronize()

    # level structure of this build (for algorithmic bytes)
    st = base.stats()
    voxels = st["n_total_voxels"]

    clocks = ClockSampler(local)
    launches0 = base.stats()["gpu_launches"]
    base.profile(True)
    base.profile_report()
    prof = {}
    extra_launches = 0
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    outs = []
    for _ in range(args.steps):
        s, c = step(base, profile=True)
        for o in (s, c):
            if o is None:
                continue
            for k, (n, ms) in o.profile_report().items():
                a = prof.setdefault(k, [0, 0.0])
                a[0] += n
                a[1] += ms
            extra_launches += o.stats()["gpu_launches"]
        outs.append((s, c))
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms_total = e0.elapsed_time(e1)
    if world > 1:
        t = torch.tensor([ms_total], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_total = float(t.item())
    for k, (n, ms) in base.profile_report().items():
        a = prof.setdefault(k, [0, 0.0])
        a[0] += n
        a[1] += ms
    launches = base.stats()["gpu_launches"] - launches0 + extra_launches
    ms_step = ms_total / args.steps
    value = world * voxels / (ms_step / 1e3) / 1e6

    s_last, c_last = outs[-1]
    sst = s_last.stats()
    cst = c_last.stats() if c_last is not None else None
    # level sizes for the algorithmic-byte model (one extra instrumented build)
    info = level_info(sv, base, s_last, args.levels)

    # --- roofline of the dominant kernel (live CUDA-event durations)
    hbm_peak, peak_src = peaks()
    dom = max(prof.items(), key=lambda kv: kv[1][1]) if prof else None
    roof = None
    if dom:
        name, (n, ms) = dom
        per_launch_ms = ms / n
        launches_per_step = n / args.steps
        ab = algorithmic_bytes(name, info)
        achieved = (ab / launches_per_step) / (per_launch_ms / 1e3) / 1e9 if ab else None
        roof = {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": (achieved / hbm_peak) if achieved else None, "traffic": None,
                "peak_source": peak_src, "avg_launch_ms": per_launch_ms, "share": ms / sum(v[1] for v in prof.values())}

    # --- e2e through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, sv, torch, stream, local, tris, voxels, have_csv)

    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 SAT + u32 keys", "data": "synthetic",
        "config": {"workload": "terrain %dx%d fBm (8 octaves) + skirts, depth %d (%d^3): voxelize -> SVDAG -> "
                               "SSVDAG + CSVDAG" % (args.grid, args.grid, args.levels, 2 ** args.levels),
                   "triangles": int(T), "levels": args.levels, "voxels": int(voxels),
                   "nodes_svo": int(st["n_nodes_svo"]), "nodes_dag": int(st["n_nodes_dag"]),
                   "nodes_sdag": int(sst["n_nodes_sdag"]),
                   "nodes_csvdag": int(cst["n_nodes"]) if cst else None,
                   "csvdag_in_step": bool(have_csv),
                   "frontier_pairs": int(info["frontier"][0]), "sat_fp64_fallbacks": int(info["sat_fallbacks"]),
                   "l2": "inputs larger than L2 (triangles 302 MB, node pools > 129 MB)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "clocks": clk, "gpu_launches": int(launches), "roofline": roof, "e2e": e2e,
        "kernel_ms_per_step": sum(v[1] for v in prof.values()) / args.steps,
        "kernels": {k: {"launches": v[0], "ms_per_step": v[1] / args.steps} for k, v in
                    sorted(prof.items(), key=lambda kv: -kv[1][1])[:12]},
    }
    if args.profile_json:
        with open(args.profile_json, "w") as f:
            json.dump({"prof": prof, "info": info}, f, indent=1)
    return res


def level_info(sv, base, s_last, levels):
    """Frontier and level sizes of one build (for the byte model)."""
    o = base.clone()
    o.buildSVO(levels)
    svo = [o.level_count(l) for l in range(levels)]
    pairs = o.stats()["frontier_pairs"]
    fallbacks = o.stats()["sat_fallbacks"]
    o.toDAG()
    dag = [o.level_count(l) for l in range(levels)]
    o.close()
    return {"svo": svo, "dag": dag, "svo_inner": svo[1:-1], "dag_inner": dag[1:-1], "frontier": [pairs],
            "sdag": [s_last.level_count(l) for l in range(levels)], "sat_fallbacks": fallbacks}


def run_e2e(args, sv, torch, stream, local, tris, voxels, have_csv):
    import numpy as np

    pinned = torch.from_numpy(tris).pin_memory()
    ptr = pinned.data_ptr()
    T = tris.shape[0]
    o = sv.Octree(device=local, stream=stream.cuda_stream)
    lib = sv.load_gpu()
    bb = (ctypes_double6())(*sv.UNIT_BOX)

    def one():
        d2h = 0
        assert lib.svdag_upload_triangles(o._h, ptr, T) == 0
        o.buildSVO(args.levels)
        o.toDAG()
        o.initChildLevels()
        s = o.clone()
        s.toSDAG()
        outs = [s]
        if have_csv:
            c = o.clone()
            c.mergeAcrossAllLevels()
            outs.append(c)
        for x in outs:
            for l in range(args.levels):
                d2h += x.level(l).nbytes
        return d2h

    for _ in range(max(1, args.warmup)):
        one()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(stream)
    d2h = 0
    for _ in range(args.steps):
        d2h = one()
    e1.record(stream)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) * 1e3 / args.steps
    ms = e0.elapsed_time(e1) / args.steps
    del bb
    return {"value": voxels / (ms / 1e3) / 1e6, "unit": UNIT, "ms_per_step": ms, "wall_ms_per_step": wall,
            "h2d_bytes_per_step": int(36 * T), "d2h_bytes_per_step": int(d2h)}


def ctypes_double6():
    import ctypes

    return ctypes.c_double * 6


# ---------------------------------------------------------------------------
def cpu_sample(args, frac_rows):
    import numpy as np

    import svdag_gb300 as sv

    tris = sv.terrain(args.grid, 8, 0.3, args.seed)
    g = args.grid - 1
    rows = max(1, int(g * frac_rows))
    return np.ascontiguousarray(tris[: 2 * g * rows]), rows


def cpu_build(oracle_py, tris, levels, chunked, threads):
    o = oracle_py.OracleOctree()
    t0 = time.perf_counter()
    if chunked:
        o.buildDAG(tris, levels, 2, threads=threads)
    else:
        o.buildSVO(tris, levels)
        o.toDAG()
    o.initChildLevels()
    s = o.clone()
    s.toSDAG()
    c = o.clone()
    c.mergeAcrossAllLevels()
    dt = time.perf_counter() - t0
    return o.stats()["n_total_voxels"], dt


def run_cpu_baseline(args):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py

    frac = 1.0 / 64
    tris, rows = cpu_sample(args, frac)
    vox, dt = cpu_build(oracle_py, tris, args.levels, chunked=False, threads=1)
    return {"value": vox / dt / 1e6, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "first %d of %d terrain rows (%d triangles, %d voxels) at depth %d, full path "
                      "(buildSVO, toDAG, toSDAG, mergeAcrossAllLevels), single thread, %.1f s"
                      % (rows, args.grid - 1, tris.shape[0], vox, args.levels, dt)}


def run_reference(args, rank, world):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py

    if rank != 0:
        return None
    cores = os.cpu_count() or 1
    frac = 1.0 / 64
    tris, rows = cpu_sample(args, frac)
    for _ in range(max(args.warmup, 0)):
        cpu_build(oracle_py, tris, args.levels, chunked=True, threads=cores)
    times = []
    vox = 0
    for _ in range(args.steps):
        vox, dt = cpu_build(oracle_py, tris, args.levels, chunked=True, threads=cores)
        times.append(dt)
    dt = sum(times) / len(times)
    v = vox / dt / 1e6
    sample = ("first %d of %d terrain rows (%d triangles, %d voxels) at depth %d: chunked OpenMP buildDAG "
              "(step level 2) + toSDAG + mergeAcrossAllLevels, restated CPU port" %
              (rows, args.grid - 1, tris.shape[0], vox, args.levels))
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 SAT + u32 keys", "data": "synthetic", "impl": "reference",
            "config": {"workload": "terrain %dx%d fBm (8 octaves) + skirts, depth %d (%d^3): voxelize -> SVDAG -> "
                                   "SSVDAG + CSVDAG" % (args.grid, args.grid, args.levels, 2 ** args.levels),
                       "sample": sample},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    rank, local, world = rank_info()
    if args.impl == "reference":
        res = run_reference(args, rank, world)
        if res is not None:
            print(json.dumps(res))
        return
    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    res = run_ours(args, rank, local, world)
    if rank == 0:
        if not args.no_cpu_baseline:
            res["cpu_baseline"] = run_cpu_baseline(args)
        print(json.dumps(res))
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
