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
import concurrent.futures
import ctypes
import datetime
import hashlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "svdag-compression_gb300")
sys.path.insert(0, PKG)

METRIC = "SSVDAG build Mvoxels/s & HBM GB/s, depth 12; lossy nodes saved at <=1% err"
UNIT = "Mvoxels/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 20; 300 frames for raycast and 25 fills for floodfill, about a "
                         "second of timed work so that the clock sampler sees it)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["terrain", "city", "batch", "lossy", "raycast", "floodfill"],
                    default="terrain",
                    help="terrain: 2048^2 fBm terrain at depth 12 (the headline); city: 4096^2 terrain + 200,000 "
                         "boxes at depth 15, chunked build with step level 1; batch: 256 voxel-brick chunks of "
                         "depths 7-11 (value noise, 5-40%% fill), batched SSVDAG + CSVDAG; lossy: 2048^2 terrain + "
                         "5,000 boxes at depth 11, lossy LSVDAG with exact and learned pair proposals; raycast: "
                         "1920x1080 frames of the depth-12 terrain's encoded SSVDAG, the viewer's DDA traversal; "
                         "floodfill: hidden-geometry flood fill of the depth-12 terrain's SVO")
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--pixel-tolerance", type=float, default=1.0)
    ap.add_argument("--top-k", type=int, default=384)
    ap.add_argument("--train-pairs", type=int, default=2000000)
    ap.add_argument("--epochs", type=int, default=1)
    ap.add_argument("--train-batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--chunks", type=int, default=256)
    ap.add_argument("--max-depth", type=int, default=11)
    ap.add_argument("--grid", type=int, default=None)
    ap.add_argument("--levels", type=int, default=None)
    ap.add_argument("--step-level", type=int, default=None, help="buildDAG step level (0 = buildSVO + toDAG)")
    ap.add_argument("--boxes", type=int, default=200000)
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--reduction-sms", type=int, default=None,
                    help="SMs the SSVDAG and CSVDAG reductions may take while the next step builds (pipelined "
                         "steps; default a quarter of the GPU, all of it for a chunked build; 0 = all)")
    ap.add_argument("--no-pipeline", action="store_true",
                    help="terrain/city: run the timed steps one after another instead of overlapping a step's "
                         "SSVDAG / CSVDAG reductions with the next step's voxelization")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-json", default="")
    a = ap.parse_args()
    if a.steps is None:
        a.steps = {"raycast": 300, "floodfill": 25}.get(a.workload, 20)
    city = a.workload == "city"
    if a.grid is None:
        a.grid = 4096 if city else 2048
    if a.levels is None:
        a.levels = 15 if city else (11 if a.workload == "lossy" else 12)
    if a.step_level is None:
        a.step_level = 1 if city else 0
    if a.seed is None:
        a.seed = 15 if city else 7
    return a


def scene(args, sv):
    if args.workload == "city":
        return sv.city(args.grid, args.boxes, args.levels, args.seed)
    return sv.terrain(args.grid, 8, 0.3, args.seed)


def workload_name(args):
    if args.workload == "city":
        return ("city: %dx%d fBm terrain + %d boxes (footprints 8-256 voxels, log-normal heights, median 64), "
                "depth %d (%d^3), chunked buildDAG step level %d -> SVDAG -> SSVDAG + CSVDAG"
                % (args.grid, args.grid, args.boxes, args.levels, 2 ** args.levels, args.step_level))
    return ("terrain %dx%d fBm (8 octaves) + skirts, depth %d (%d^3): voxelize -> SVDAG -> SSVDAG + CSVDAG"
            % (args.grid, args.grid, args.levels, 2 ** args.levels)
            + (", chunked buildDAG step level %d" % args.step_level if args.step_level else ""))


def rank_info():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def max_over_ranks(value, torch, device, world):
    """The largest of the ranks' values (replicas: the job's time is its
    slowest rank's); the value itself on one rank.  `device` holds the
    reduction tensor: a CUDA device under NCCL, the CPU under gloo."""
    if world <= 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        self.t0 = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def mark(self):
        """Start of the timed region (rows before it are discarded)."""
        self.t0 = datetime.datetime.now()

    def stop(self):
        if self.p is None:
            return None
        t1 = datetime.datetime.now()
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
                if len(parts) < 10:
                    continue
                try:
                    ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f")
                    if self.t0 is not None and not (self.t0 <= ts <= t1):
                        continue
                    rows.append((float(parts[2]), float(parts[3]), parts[6:10]))
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
# Algorithmic bytes (the data each phase must touch once).  R = node record:
# mask/mirror word + 8 child words.  N_l, D_l, S_l, C_l = SVO, DAG, SDAG and
# CSVDAG nodes of level l; T = triangles.
#   B_vox  = 36 T + 36 sum_l N_l
#   B_dag  = sum_{l>=1} (R + 4) N_l + R D_l + 64 N_{l-1}
#   B_sdag = sum_l (R + 8 + 5) D_l + R S_l + 64 D_{l-1}
#   B_csv  = sum_l (R + 16) D_l + R C_l
R = 36

# DRAM bytes (read + write) per launch measured by ncu on the full default
# workload (the 12 k_expand launches of one timed step, averaged; per-launch
# figures in profiles/k_expand_terrain2048_L12_dram.txt).  Valid for the
# default terrain workload only.
KERNEL_DRAM_BYTES_PER_LAUNCH = {"k_expand": 543215189}


def model_bytes(info, T):
    N, D, S, C = info["svo"], info["dag"], info["sdag"], info["csv"]
    L = len(D)
    b_vox = 36 * T + 36 * info["svo_total"]
    b_dag = sum((R + 4) * N[l] + R * D[l] + 64 * N[l - 1] for l in range(1, L)) if N else None
    b_sdag = sum((R + 13) * D[l] + R * S[l] + (64 * D[l - 1] if l else 0) for l in range(L))
    b_csv = sum((R + 16) * D[l] + R * C[l] for l in range(L)) if C else None
    return {"k_expand": b_vox, "vox": b_vox, "dag": b_dag, "sdag": b_sdag, "csv": b_csv}


def pool_digest(pool):
    """SHA-256 over a node pool's levels (u64 node count, then the 48-byte
    records: hdr, children, child levels, invariant) -- the form of the
    digests in tests/golden/golden.json, which the reference's own build
    made on the same seeded scenes."""
    import numpy as np

    h = hashlib.sha256()
    for lev in pool:
        h.update(np.uint64(len(lev)).tobytes())
        h.update(np.ascontiguousarray(lev).tobytes())
    return h.hexdigest()


def golden_case(args):
    """The golden fixture of this workload, if the reference's build was run
    on it (tests/golden/make_golden.py), else None."""
    if args.workload != "terrain" or args.step_level:
        return None
    name = "terrain%d_L%d" % (args.grid, args.levels)
    try:
        with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
            g = json.load(f).get(name)
    except (OSError, ValueError):
        return None
    # the fixture must be of this very scene (seed 7 is the fixture's seed)
    if g is None or args.seed != 7 or g["levels"] != args.levels:
        return None
    return name, g


def parity_check(args, digests, counts):
    """Compares the digests of the last timed step's pools with the golden
    fixture: "golden-match", "golden-mismatch: ..." or None (no fixture)."""
    gc = golden_case(args)
    if gc is None:
        return None, None
    name, g = gc
    bad = [k for k in ("svo", "dag", "sdag", "csv") if k in digests and digests[k] != g[k]["digest"]]
    bad += ["%s counts" % k for k in counts if counts[k] != g[k]["counts"]]
    return ("golden-match" if not bad else "golden-mismatch: " + ", ".join(bad)), name


def run_ours(args, rank, local, world):
    import numpy as np
    import torch

    import svdag_gb300 as sv

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    tris = scene(args, sv)
    T = tris.shape[0]
    d_tris = torch.from_numpy(tris).to(dev)
    stream = torch.cuda.Stream(device=dev)
    red_streams = [torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)]
    red_pool = concurrent.futures.ThreadPoolExecutor(2)
    base = sv.Octree(device=local, stream=stream.cuda_stream)
    base.set_device_triangles(d_tris.data_ptr(), T, keepalive=d_tris)
    have_csv = True

    phase_prof = {}

    def collect(phase, octree):
        for k, (n, ms) in octree.profile_report().items():
            a = phase_prof.setdefault(phase, {}).setdefault(k, [0, 0.0])
            a[0] += n
            a[1] += ms

    def build(octree, profile=False):
        if args.step_level:
            octree.buildDAG(args.levels, args.step_level)
            if profile:
                collect("voxelize", octree)
        else:
            octree.buildSVO(args.levels)
            if profile:
                collect("voxelize", octree)
            octree.toDAG()
        octree.initChildLevels()
        if profile:
            collect("dag", octree)

    def start_reductions(octree, profile=False, cap=0):
        # the SSVDAG and CSVDAG reductions of the same DAG are independent:
        # two clones on their own streams, driven from two host threads (a
        # clone is complete when clone() returns, so the octree may be
        # rebuilt while they run); `cap` SMs each when they share the GPU
        # with the next build
        s = octree.clone(stream=red_streams[0].cuda_stream)
        c = octree.clone(stream=red_streams[1].cuda_stream) if have_csv else None
        for o in (s, c):
            if o is not None:
                o.set_persistent_blocks(cap)
        for o in (s, c):
            if profile and o is not None:
                o.profile(True)

        def merge():
            try:
                c.mergeAcrossAllLevels()
                return True
            except sv.SvdagError:
                return False

        fs = red_pool.submit(s.toSDAG)
        fc = red_pool.submit(merge) if c is not None else None
        return s, c, fs, fc

    def finish(pending, profile=False):
        nonlocal have_csv
        s, c, fs, fc = pending
        fs.result()
        if fc is not None and not fc.result():
            have_csv = False
            c = None
        if profile:
            collect("sdag", s)
            if c is not None:
                collect("csv", c)
        stream.wait_stream(red_streams[0])
        stream.wait_stream(red_streams[1])
        return s, c

    def step(octree, profile=False):
        build(octree, profile)
        return finish(start_reductions(octree, profile), profile)

    for _ in range(max(args.warmup, 0)):
        step(base)
    torch.cuda.synchronize()

    # level structure of this build (for algorithmic bytes)
    st = base.stats()
    voxels = st["n_total_voxels"]

    def timed_region(events, pipelined=False):
        """K steps between two CUDA events on the build stream.  With events,
        every kernel launch is also bracketed by CUDA events on that stream
        (per-kernel durations for the roofline), collected per phase.
        Pipelined: each step's reductions run while the next step voxelizes
        (the last step's reductions end inside the region)."""
        launches0 = base.stats()["gpu_launches"]
        base.profile(events)
        base.profile_report()
        phase_prof.clear()
        extra = 0
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        outs = []
        pending = None
        for _ in range(args.steps):
            if pipelined:
                # step i+1's voxelization overlaps step i's reductions
                build(base)
                if pending is not None:
                    outs.append(finish(pending))
                pending = start_reductions(base, cap=red_sms)
            else:
                outs.append(step(base, profile=events))
        if pending is not None:
            outs.append(finish(pending))
        for s, c in outs:
            for o in (s, c):
                if o is not None:
                    extra += o.stats()["gpu_launches"]
        e1.record(stream)
        torch.cuda.synchronize()
        ms_total = max_over_ranks(e0.elapsed_time(e1), torch, dev, world)
        base.profile(False)
        prof = {}
        for ph in phase_prof.values():
            for k, (n, ms) in ph.items():
                a = prof.setdefault(k, [0, 0.0])
                a[0] += n
                a[1] += ms
        return ms_total, prof, base.stats()["gpu_launches"] - launches0 + extra, outs

    red_sms = reduction_sms(args, torch, dev)

    # timed region: K steps, clocks sampled meanwhile
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.5)  # the sampler is running before the timed region opens
    clocks.mark()
    ms_total, _, launches, outs = timed_region(events=False, pipelined=not args.no_pipeline)
    clk = clocks.stop()
    ms_step = ms_total / args.steps
    value = world * voxels / (ms_step / 1e3) / 1e6
    # one build at a time (no overlap between steps): the latency of a build
    ms_seq = timed_region(events=False, pipelined=False)[0] / args.steps
    # the same K steps again with every launch bracketed by CUDA events on the
    # build stream: per-kernel durations for the roofline (the events add host
    # work per launch, so this region is not the one `value` comes from)
    ms_events, prof, _, _ = timed_region(events=True)

    s_last, c_last = outs[-1]
    sst = s_last.stats()
    cst = c_last.stats() if c_last is not None else None
    # level sizes for the algorithmic-byte model (one extra instrumented build)
    info = level_info(sv, base, s_last, args)

    # --- roofline of the dominant kernel (live CUDA-event durations)
    hbm_peak, peak_src = peaks()
    info["csv"] = [c_last.level_count(l) for l in range(args.levels)] if c_last is not None else None
    B = model_bytes(info, T)
    dom = max(prof.items(), key=lambda kv: kv[1][1]) if prof else None
    roof = None
    if dom:
        name, (n, ms) = dom
        per_launch_ms = ms / n
        launches_per_step = n / args.steps
        ab = B.get(name)  # algorithmic bytes of one step's launches
        achieved = (ab / launches_per_step) / (per_launch_ms / 1e3) / 1e9 if ab else None
        # k_expand is bound by instruction issue (SAT arithmetic), not HBM;
        # its algorithmic bytes over HBM bandwidth are reported all the same
        roof = {"kernel": name, "bound": "issue" if name == "k_expand" else "hbm", "achieved": achieved,
                "peak": hbm_peak, "unit": "GB/s",
                "frac": (achieved / hbm_peak) if achieved else None,
                "traffic": (KERNEL_DRAM_BYTES_PER_LAUNCH.get(name)
                            if args.workload == "terrain" and args.grid == 2048 and args.levels == 12 else None),
                "peak_source": peak_src,
                "avg_launch_ms": per_launch_ms, "share": ms / sum(v[1] for v in prof.values())}
        if name == "k_expand":
            pairs = info["frontier"][0]
            roof["algorithmic_bytes"] = "B_vox = 36 T + 36 sum_l N_l per build, spread over its %d launches" % args.levels
            roof["note"] = ("k_expand is instruction-issue / latency bound (SAT box tests), not HBM bound: ncu on "
                            "its two largest launches of terrain 1024 depth 11 shows issue slots 60-71% busy at 28 "
                            "warps/SM, ALU pipe 51-62%, FMA 16-20%, FP64 <1%, DRAM 3-4% of peak "
                            "(profiles/k_expand_terrain1024_L11.txt)")
            roof["sat"] = {"frontier_pairs_per_s": pairs / (ms / args.steps / 1e3),
                           "child_box_tests_per_s": 8 * pairs / (ms / args.steps / 1e3)}
    # reduction phases (toDAG, toSDAG, cross-level merge): algorithmic bytes
    # over the kernel time of those phases
    red = None
    red_ms = sum(ms for ph in ("dag", "sdag", "csv") for _, ms in phase_prof.get(ph, {}).values()) / args.steps
    if red_ms > 0 and B["dag"] is not None:
        rb = B["dag"] + B["sdag"] + (B["csv"] or 0)
        red = {"bound": "hbm", "achieved": rb / (red_ms / 1e3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
               "frac": rb / (red_ms / 1e3) / 1e9 / hbm_peak, "bytes_per_step": rb, "kernel_ms_per_step": red_ms,
               "phases_ms_per_step": {ph: sum(ms for _, ms in phase_prof.get(ph, {}).values()) / args.steps
                                      for ph in ("voxelize", "dag", "sdag", "csv")}}

    # --- parity of the last timed step's pools with the reference's golden
    # digests (after the timed regions; the SVO comes from level_info's build)
    parity, parity_case = None, None
    if golden_case(args) is not None:
        digests = {"dag": pool_digest(base.pool()), "sdag": pool_digest(s_last.pool())}
        if info.get("svo_digest"):
            digests["svo"] = info["svo_digest"]
        if c_last is not None:
            digests["csv"] = pool_digest(c_last.pool())
        counts = {k: info[k] for k in ("svo", "dag", "sdag", "csv") if info.get(k) is not None}
        parity, parity_case = parity_check(args, digests, counts)

    # --- e2e through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, sv, torch, stream, local, tris, voxels, have_csv)

    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64-exact SAT (certified fp32 filter) + u32 keys", "data": "synthetic",
        "config": {"workload": workload_name(args),
                   "triangles": int(T), "levels": args.levels, "voxels": int(voxels),
                   "nodes_svo": int(st["n_nodes_svo"]), "nodes_dag": int(st["n_nodes_dag"]),
                   "nodes_sdag": int(sst["n_nodes_sdag"]),
                   "nodes_csvdag": int(cst["n_nodes"]) if cst else None,
                   "csvdag_in_step": bool(have_csv),
                   "frontier_pairs": int(info["frontier"][0]), "sat_fp64_fallbacks": int(info["sat_fallbacks"]),
                   "l2": "inputs larger than L2 (triangles %d MB, node pools > 129 MB)" % (36 * T // 10**6),
                   "parity": parity,
                   "parity_detail": ("SHA-256 of the last timed step's SVO, DAG, SSVDAG and CSVDAG pools and their "
                                     "per-level counts against the digests the reference's own build (compiled "
                                     "from its sources) wrote for this scene: tests/golden/golden.json[%s]"
                                     % parity_case) if parity_case else None,
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "clocks": clk, "gpu_launches": int(launches), "roofline": roof, "reduction_roofline": red, "e2e": e2e,
        "pipelined": not args.no_pipeline,
        "reduction_sms": red_sms if not args.no_pipeline else 0,
        "sequential_ms_per_step": ms_seq,
        "kernel_events_region_ms_per_step": ms_events / args.steps,
        "kernel_ms_per_step": sum(v[1] for v in prof.values()) / args.steps,
        "kernels": {k: {"launches": v[0], "ms_per_step": v[1] / args.steps} for k, v in
                    sorted(prof.items(), key=lambda kv: -kv[1][1])[:12]},
    }
    if args.profile_json:
        with open(args.profile_json, "w") as f:
            json.dump({"prof": prof, "info": info}, f, indent=1)
    return res


def level_info(sv, base, s_last, args):
    """Frontier and level sizes of one build (for the byte model).  The
    chunked build exposes only its totals (its SVO never exists whole)."""
    levels = args.levels
    o = base.clone()
    if args.step_level:
        o.buildDAG(levels, args.step_level)
        svo = None
    else:
        o.buildSVO(levels)
        svo = [o.level_count(l) for l in range(levels)]
        svo_digest = pool_digest(o.pool()) if golden_case(args) else None
    st = o.stats()
    if not args.step_level:
        o.toDAG()
    dag = [o.level_count(l) for l in range(levels)]
    o.close()
    return {"svo": svo, "svo_total": st["n_nodes_svo"], "dag": dag, "frontier": [st["frontier_pairs"]],
            "sdag": [s_last.level_count(l) for l in range(levels)], "sat_fallbacks": st["sat_fallbacks"],
            "svo_digest": None if args.step_level else svo_digest}


def reduction_sms(args, torch, dev):
    """SMs each of the SSVDAG and CSVDAG reductions may take while the next
    step builds (their persistent kernels start only when their whole grid
    fits, so a full-GPU grid would wait for, then exclude, the build): a
    quarter of the GPU beside a plain build (buildSVO + one toDAG); all of it
    beside a chunked build (buildDAG), which itself runs a full-GPU toDAG per
    chunk that capped reductions would only hold up (GB300, depth-15 city:
    13,201 Mvoxels/s uncapped, 12,114 with 19 SMs each)."""
    if args.reduction_sms is not None:
        return max(0, args.reduction_sms)
    if args.step_level:
        return 0
    return max(1, torch.cuda.get_device_properties(dev).multi_processor_count // 4)


def run_e2e(args, sv, torch, stream, local, tris, voxels, have_csv):
    """The same step through the C ABI as a host program would call it:
    triangles copied in from pinned host memory (cudaMemcpyAsync into a
    device buffer, then svdag_set_device_triangles), the build, and every
    level of both result pools (headers, children, child levels, invariants)
    copied out into pinned host buffers (svdag_download_level)."""
    import ctypes

    pinned = torch.from_numpy(tris).pin_memory()
    T = tris.shape[0]
    o = sv.Octree(device=local, stream=stream.cuda_stream)
    red_streams = [torch.cuda.Stream(device=local), torch.cuda.Stream(device=local)]
    red_pool = concurrent.futures.ThreadPoolExecutor(2)
    lib = sv.load_gpu()
    # one set of pinned host buffers per result, so that each result is read
    # back by its own host thread as soon as its reduction ends
    caps = [[0], [0]]
    hosts = [{}, {}]

    def buffers(n, k):
        cap, host = caps[k], hosts[k]
        if n > cap[0]:
            cap[0] = max(n, 2 * cap[0])
            host["hdr"] = torch.empty(cap[0], dtype=torch.int32).pin_memory()
            host["ch"] = torch.empty(8 * cap[0], dtype=torch.int32).pin_memory()
            host["cl"] = torch.empty(8 * cap[0], dtype=torch.uint8).pin_memory()
            host["inv"] = torch.empty(cap[0], dtype=torch.uint8).pin_memory()
        return host

    def download(x, sdag):
        nbytes = 0
        n = ctypes.c_uint64()
        for l in range(args.levels):
            assert lib.svdag_level_count(x._h, l, ctypes.byref(n)) == 0
            if n.value == 0:
                continue
            b = buffers(n.value, 0 if sdag else 1)
            leaf = l == args.levels - 1
            ch = None if leaf else b["ch"].data_ptr()
            cl = None if (leaf or sdag) else b["cl"].data_ptr()
            inv = b["inv"].data_ptr() if sdag else None
            assert lib.svdag_download_level(x._h, l, b["hdr"].data_ptr(), ch, cl, inv) == 0
            nbytes += n.value * (4 + (0 if leaf else 32) + (0 if (leaf or sdag) else 8) + (1 if sdag else 0))
        return nbytes

    # the step's triangles copied from pinned host memory into one of two
    # device buffers on a copy stream (cudaMemcpyAsync), then handed to the
    # builder (svdag_set_device_triangles): pipelined, step i+1's copy runs
    # while step i builds; a buffer is refilled only after the build that
    # read it
    dev_tris = [torch.empty_like(pinned, device=torch.device("cuda", local)) for _ in range(2)]
    copy_stream = torch.cuda.Stream(device=local)
    copied = [torch.cuda.Event(), torch.cuda.Event()]
    freed = [torch.cuda.Event(), torch.cuda.Event()]

    def upload(k):
        b = k % 2
        copy_stream.wait_event(freed[b])
        with torch.cuda.stream(copy_stream):
            dev_tris[b].copy_(pinned, non_blocking=True)
            copied[b].record(copy_stream)

    def build_one(k):
        b = k % 2
        stream.wait_event(copied[b])
        assert lib.svdag_set_device_triangles(o._h, dev_tris[b].data_ptr(), T) == 0
        if args.step_level:
            o.buildDAG(args.levels, args.step_level)
        else:
            o.buildSVO(args.levels)
            o.toDAG()
        freed[b].record(stream)
        o.initChildLevels()

    red_sms = 0 if args.no_pipeline else reduction_sms(args, torch, torch.device("cuda", local))

    def start_one():
        s = o.clone(stream=red_streams[0].cuda_stream)
        c = o.clone(stream=red_streams[1].cuda_stream) if have_csv else None
        for x in (s, c):
            if x is not None:
                x.set_persistent_blocks(red_sms)

        def sdag():
            s.toSDAG()
            return download(s, True)

        def csv():
            c.mergeAcrossAllLevels()
            return download(c, False)

        return s, c, red_pool.submit(sdag), (red_pool.submit(csv) if c is not None else None)

    def end_one(p):
        _, _, fs, fc = p
        d2h = fs.result()
        if fc is not None:
            d2h += fc.result()
        stream.wait_stream(red_streams[0])
        stream.wait_stream(red_streams[1])
        return d2h

    for k in range(max(1, args.warmup)):
        upload(k)
        build_one(k)
        end_one(start_one())
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(stream)
    d2h = 0
    pending = None
    upload(0)
    for k in range(args.steps):
        # the next step's upload overlaps this step's build, and this step's
        # build the previous step's reductions and read-back, unless
        # --no-pipeline
        if not args.no_pipeline and k + 1 < args.steps:
            upload(k + 1)
        build_one(k)
        if args.no_pipeline and k + 1 < args.steps:
            upload(k + 1)
        if pending is not None:
            d2h = end_one(pending)
            pending = None
        pending = start_one()
        if args.no_pipeline:
            d2h = end_one(pending)
            pending = None
    if pending is not None:
        d2h = end_one(pending)
    e1.record(stream)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) * 1e3 / args.steps
    ms = e0.elapsed_time(e1) / args.steps
    return {"value": voxels / (ms / 1e3) / 1e6, "unit": UNIT, "ms_per_step": ms, "wall_ms_per_step": wall,
            "h2d_bytes_per_step": int(36 * T), "d2h_bytes_per_step": int(d2h),
            "pipelined": not args.no_pipeline, "reduction_sms": red_sms,
            "path": "C ABI: the step's triangles copied from pinned host memory (cudaMemcpyAsync on a copy stream, "
                    "two device buffers) and handed to svdag_set_device_triangles, build, svdag_download_level "
                    "of every level of the SSVDAG and the CSVDAG into pinned host buffers; step i+1's upload "
                    "overlaps step i's build, which overlaps step i-1's reductions and read-back"}


# ---------------------------------------------------------------------------
def cpu_scene(args, oracle_py, frac_rows=1.0):
    """The workload's scene for the CPU legs, generated by the oracle library
    (same generator source as the GPU arm's; no product library is loaded).
    frac_rows < 1 keeps the first rows of the terrain (warm-up samples)."""
    if args.workload == "city":
        tris = oracle_py.city(args.grid, args.boxes, args.levels, args.seed)
    else:
        tris = oracle_py.terrain(args.grid, 8, 0.3, args.seed)
    if frac_rows >= 1.0:
        return tris, args.grid - 1
    g = args.grid - 1
    rows = max(1, int(g * frac_rows))
    return np.ascontiguousarray(tris[: 2 * g * rows]), rows


def cpu_build(oracle_py, tris, levels, chunked, threads, step_level=2, csv=True):
    """The reference's path on the host: buildDAG (chunked, OpenMP over the
    sub-octrees as geom_octree.cpp:331 does) or buildSVO + toDAG, then
    initChildLevels, and toSDAG and mergeAcrossAllLevels on two copies of
    the DAG -- concurrently in two host threads when threads > 1 (each of
    them is single-threaded in the reference).  Returns (voxels, seconds,
    SVO/DAG/SDAG/CSVDAG node counts)."""
    o = oracle_py.OracleOctree()
    t0 = time.perf_counter()
    if chunked:
        o.buildDAG(tris, levels, step_level, threads=threads)
    else:
        o.buildSVO(tris, levels)
        o.toDAG()
    o.initChildLevels()
    s = o.clone()
    c = o.clone() if csv else None
    if threads > 1 and c is not None:
        with concurrent.futures.ThreadPoolExecutor(2) as ex:
            fs = ex.submit(s.toSDAG)
            fc = ex.submit(c.mergeAcrossAllLevels)
            fs.result()
            fc.result()
    else:
        s.toSDAG()
        if c is not None:
            c.mergeAcrossAllLevels()
    dt = time.perf_counter() - t0
    st = o.stats()
    counts = {"svo": st["n_nodes_svo"], "dag": st["n_nodes_dag"], "sdag": s.stats()["n_nodes_sdag"],
              "csv": c.stats()["n_nodes"] if c is not None else None}
    return st["n_total_voxels"], dt, counts


def run_cpu_baseline(args):
    """One full build of the workload's scene by the oracle port on all host
    cores (chunked OpenMP buildDAG, step level 2, as the reference's
    svbuilder runs it for numBuildSteps = 2)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py

    cores = os.cpu_count() or 1
    step = args.step_level or 2
    if args.workload == "city":
        # the depth-15 city is ~10^4 s of CPU work: a 1/64 slab of its rows
        tris, rows = cpu_scene(args, oracle_py, 1.0 / 64)
        what = "first %d of %d terrain rows of the city scene" % (rows, args.grid - 1)
    else:
        tris, rows = cpu_scene(args, oracle_py)
        what = "the full scene"
    vox, dt, counts = cpu_build(oracle_py, tris, args.levels, chunked=True, threads=cores, step_level=step)
    return {"value": vox / dt / 1e6, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%s (%d triangles, %d voxels) at depth %d, one build: chunked OpenMP buildDAG (step level "
                      "%d) on %d threads, then toSDAG and mergeAcrossAllLevels concurrently on two threads, "
                      "%.1f s" % (what, tris.shape[0], vox, args.levels, step, cores, dt)}


def run_reference(args, rank, world):
    """The reference's CPU path (restated by the oracle: the reference's
    sources are not present where the benchmark runs) on the same workload
    as the GPU arm: every timed step is one full build of the full scene.
    Warm-up steps run the same path on the first 1/16 of the terrain rows
    (thread pool, allocator and caches warm; a full warm-up build would add
    a quarter of a minute each)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py

    if rank != 0:
        return None
    cores = os.cpu_count() or 1
    step = args.step_level or 2
    full = args.workload != "city"
    tris, rows = cpu_scene(args, oracle_py, 1.0 if full else 1.0 / 64)
    warm, _ = cpu_scene(args, oracle_py, 1.0 / 16 if full else 1.0 / 256)
    for _ in range(max(args.warmup, 0)):
        cpu_build(oracle_py, warm, args.levels, chunked=True, threads=cores, step_level=step)
    times = []
    vox = 0
    counts = None
    for _ in range(args.steps):
        vox, dt, counts = cpu_build(oracle_py, tris, args.levels, chunked=True, threads=cores, step_level=step)
        times.append(dt)
    dt = sum(times) / len(times)
    v = vox / dt / 1e6
    sample = ("%s (%d triangles, %d voxels) at depth %d, every step one full build: chunked OpenMP buildDAG (step "
              "level %d, %d threads) + toSDAG and mergeAcrossAllLevels (concurrently, two threads), restated CPU "
              "port of the reference's code; node counts SVO %d, DAG %d, SSVDAG %d, CSVDAG %s"
              % ("the full scene" if full else "first %d of %d terrain rows" % (rows, args.grid - 1),
                 tris.shape[0], vox, args.levels, step, cores, counts["svo"], counts["dag"], counts["sdag"],
                 counts["csv"]))
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 SAT + u32 keys (CPU)", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": workload_name(args), "sample": sample, "same_config": full,
                       "warmup_sample": "first 1/16 of the terrain rows" if full else "first 1/256 of the rows",
                       "step_seconds": times},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_batch(args, rank, local, world):
    """Voxel-brick chunks: the batched build (svdag_batch_*) timed over K
    steps, the plain per-chunk form timed once over the same chunks."""
    import numpy as np
    import torch

    import svdag_gb300 as sv

    torch.cuda.set_device(local)
    rng = np.random.default_rng(args.seed)
    depths = rng.integers(7, args.max_depth + 1, size=args.chunks)
    fills = rng.uniform(0.05, 0.40, size=args.chunks)
    bricks = [sv.noise_bricks(int(d), int(args.seed) * 100003 + i, float(f), local)
              for i, (d, f) in enumerate(zip(depths, fills))]
    in_bytes = sum(b.numel() for b in bricks)
    B = sv.Batch(device=local)
    for d, b in zip(depths, bricks):
        B.add_chunk(int(d), b)
    # settings: autotuned on the batch itself (full builds, untimed; a sample
    # of every 8th chunk picked 2 or 4 reduction streams from run to run)
    B.autotune(max_trials=10)
    tune = B.tuning()
    for _ in range(max(args.warmup, 0)):
        B.build()
    voxels = sum(B.result(i, "dag").stats()["n_total_voxels"] for i in range(args.chunks))
    launches0 = B.stats()["gpu_launches"]
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.5)
    clocks.mark()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    stage = {"dag_ms": 0.0, "reduce_ms": 0.0}
    for _ in range(args.steps):
        # an NVTX range per timed build, so that a profiler can be limited to
        # it (ncu --nvtx --nvtx-include "batch_build/"; ranges are per host
        # thread: the reduction workers' launches fall outside)
        torch.cuda.nvtx.range_push("batch_build")
        B.build()
        torch.cuda.nvtx.range_pop()
        st = B.stats()
        stage["dag_ms"] += st["dag_ms"]
        stage["reduce_ms"] += st["reduce_ms"]
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3 / args.steps
    clk = clocks.stop()
    launches = (B.stats()["gpu_launches"] - launches0) // max(args.steps, 1)
    nodes = [sum(B.result(i, k).stats()["n_nodes"] for i in range(args.chunks)) for k in ("dag", "sdag", "csvdag")]
    B.close()
    # plain per-chunk form over the same chunks, once
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for d, b in zip(depths, bricks):
        o = sv.Octree(device=local)
        o.import_bricks(int(d), b)
        o.toDAG()
        s_ = o.clone()
        s_.toSDAG()
        c_ = o.clone()
        c_.initChildLevels()
        c_.mergeAcrossAllLevels()
        for x in (o, s_, c_):
            x.close()
    torch.cuda.synchronize()
    plain_ms = (time.perf_counter() - t0) * 1e3
    return {
        "metric": METRIC, "value": voxels / (ms / 1e3) / 1e6, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8 bricks + u32 keys", "data": "synthetic",
        "config": {"workload": "batch: %d voxel-brick chunks, depths uniform %d-%d, 3D value noise (period 16 "
                               "voxels) at fills uniform 5-40%%, batched toDAG + per-chunk SSVDAG + CSVDAG"
                               % (args.chunks, 7, args.max_depth),
                   "chunks": args.chunks, "voxels": int(voxels), "input_bytes": int(in_bytes),
                   "nodes_dag": int(nodes[0]), "nodes_sdag": int(nodes[1]), "nodes_csvdag": int(nodes[2]),
                   "chunks_per_s": args.chunks / (ms / 1e3), "plain_chunks_per_s": args.chunks / (plain_ms / 1e3),
                   "speedup_vs_plain": plain_ms / ms, "stage_ms_per_step": {k: v / args.steps for k, v in stage.items()},
                   "tuning": tune, "l2": "inputs larger than L2 (%d MB of bricks)" % (in_bytes // 10**6),
                   "parallelism": "single GPU"},
        "clocks": clk, "gpu_launches": int(launches), "e2e": None,
    }


def run_lossy(args, rank, local, world):
    """Lossy LSVDAG on the DAG of the 2048^2 terrain + 5,000 boxes at depth
    11: the exact proposer and the learned one (training included), each
    timed over K runs on fresh copies of the DAG."""
    import numpy as np
    import torch

    import svdag_gb300 as sv

    torch.cuda.set_device(local)
    L = args.levels
    rng = np.random.default_rng(args.seed)
    res_ = 1 << L
    lo = rng.integers(0, res_ - 64, size=(5000, 3))
    side = rng.integers(1, 65, size=(5000, 3))
    hi = np.minimum(lo + side, res_)
    tris = np.concatenate([sv.terrain(args.grid, 8, 0.3, args.seed), sv.boxes((lo + 0.25) / res_, (hi - 0.25) / res_)])
    base = sv.Octree(device=local)
    base.upload_triangles(tris)
    base.buildSVO(L)
    base.toDAG()
    runs = {}
    clk = None
    for kind in ("exact", "learned"):
        for _ in range(max(args.warmup, 0) if kind == "exact" else 0):
            base.clone().lossy(kind, 3, 5, 0.01)
        if kind == "learned":
            clocks = ClockSampler(local)
            clocks.start()
            time.sleep(0.5)
            clocks.mark()
        times, st = [], None
        for _ in range(args.steps):
            o = base.clone()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            l0 = o.stats()["gpu_launches"]
            st = o.lossy(kind, 3, 5, 0.01, top_k=args.top_k, train_pairs=args.train_pairs, epochs=args.epochs,
                         seed=args.seed, train_batch=args.train_batch, lr=args.lr)
            torch.cuda.synchronize()
            times.append((time.perf_counter() - t0) * 1e3)
            st["gpu_launches"] = o.stats()["gpu_launches"] - l0
            o.close()
        if kind == "learned":
            clk = clocks.stop()
        st["wall_ms"] = sum(times) / len(times)
        st["merges_per_s"] = st["merged"] / (st["wall_ms"] / 1e3)
        st["merges_per_s_without_training"] = st["merged"] / max(1e-9, (st["wall_ms"] - st["train_ms"]) / 1e3)
        st["nodes_saved"] = st["nodes_before"] - st["nodes_after"]
        runs[kind] = st
    ex, le = runs["exact"], runs["learned"]
    voxels = base.stats()["n_total_voxels"]
    return {
        "metric": METRIC, "value": le["merged"] / (le["wall_ms"] / 1e3), "unit": "lossy merges/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": le["wall_ms"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u8 voxels; MLP fp16 tensor-core operands, fp32 accumulation", "clocks": clk,
        "data": "synthetic",
        "config": {"workload": "lossy: %dx%d terrain + 5000 boxes (sides 1-64 voxels), depth %d, candidates 3-5 "
                               "levels above the leaves, merges within 1%% of the subtree cube's voxels" % (
                                   args.grid, args.grid, L),
                   "voxels": int(voxels), "exact": ex, "learned": le,
                   "savings_vs_exact": le["nodes_saved"] / max(1, ex["nodes_saved"]),
                   "throughput_vs_exact": (le["merged"] / le["wall_ms"]) / max(1e-9, ex["merged"] / ex["wall_ms"]),
                   "top_k": args.top_k, "train_pairs": args.train_pairs, "epochs": args.epochs,
                   "train_batch": args.train_batch, "lr": args.lr,
                   "parallelism": "single GPU"},
        "gpu_launches": int(le["gpu_launches"]), "e2e": None,
    }


# the four views of the ray-casting workload (eye, target), unit-cube coordinates
RAY_VIEWS = [((1.1, 0.55, 1.2), (0.5, 0.12, 0.5)), ((-0.5, 0.6, 0.3), (0.6, 0.1, 0.55)),
             ((0.5, 1.6, 0.5001), (0.5, 0.0, 0.5)), ((0.2, 0.32, 0.25), (0.8, 0.12, 0.9))]


def raycast_scene(args, sv, local, path):
    """The depth-12 terrain built on the GPU to an SSVDAG, written as a
    .ssvdag file (host encoder) and read back as arrays."""
    o = sv.Octree(device=local)
    o.upload_triangles(sv.terrain(args.grid, 8, 0.3, args.seed))
    o.buildSVO(args.levels)
    o.toDAG()
    o.initChildLevels()
    o.toSDAG()
    sv.write_encoded(path, "ssvdag", o.pool(), o.stats()["n_nodes"], 3)
    o.close()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py

    return oracle_py.read_ssvdag(path)


def run_raycast(args, rank, local, world):
    """Ray casting of the terrain's encoded SSVDAG: K frames of each of four
    views at 1920x1080 with the viewer's defaults (60-degree field of view,
    300 iterations, pixel tolerance 1), hit records written to HBM."""
    import numpy as np
    import torch

    import svdag_gb300 as sv

    torch.cuda.set_device(local)
    with tempfile.TemporaryDirectory() as td:
        f = raycast_scene(args, sv, local, os.path.join(td, "t.ssvdag"))
    L = args.levels
    W, H = args.width, args.height
    cams = [sv.camera(e, t, W, H, L, pixel_tolerance=args.pixel_tolerance) for e, t in RAY_VIEWS]
    S = sv.Ssvdag(f)
    npix = W * H
    buf = torch.empty(npix * 32, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(max(args.warmup, 0)):
        for c in cams:
            S.raycast_device(c, buf.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.5)
    clocks.mark()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in cams]
    per_view = [0.0] * len(cams)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for i, c in enumerate(cams):
            ev[i][0].record(stream)
            S.raycast_device(c, buf.data_ptr(), stream.cuda_stream)
            ev[i][1].record(stream)
            torch.cuda.synchronize()
            per_view[i] += ev[i][0].elapsed_time(ev[i][1])
    torch.cuda.synchronize()
    wall_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    clk = clocks.stop()
    kernel_ms = sum(per_view) / args.steps  # one step = one frame of each view
    hits = [S.raycast(c) for c in cams]
    stats = [{"hit_frac": float((h["t"] > 0).mean()), "mean_iterations": float(h["iterations"].mean()),
              "device_ms": per_view[i] / args.steps} for i, h in enumerate(hits)]
    # e2e: host hit buffers (device -> host copy of every frame's records)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(max(1, args.steps // 2)):
        for c in cams:
            S.raycast(c)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / max(1, args.steps // 2)
    S.close()
    rays = npix * len(cams)
    iters = sum(float(h["iterations"].sum()) for h in hits)
    # algorithmic bytes per frame: the 32-byte hit records written once; the
    # node reads are cache-resident re-reads of a few MB of encoded nodes
    alg = 32.0 * rays
    peak, src = peaks()
    res = {
        "metric": METRIC, "value": rays / (kernel_ms / 1e3) / 1e6, "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": kernel_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 rays, u16/u8 nodes", "data": "synthetic",
        "config": {"workload": "raycast: %dx%d frames of 4 views of the %dx%d terrain's SSVDAG at depth %d "
                               "(.ssvdag: %d inner words, %d leaf bytes), viewer defaults: 60-degree fov, 300 "
                               "iterations, pixel tolerance %g" % (W, H, args.grid, args.grid, L, f["inner"].size,
                                                                   f["leaves"].size, args.pixel_tolerance),
                   "views": stats, "dda_iterations_per_s": iters / (kernel_ms / 1e3),
                   "l2": "encoded SSVDAG (%d MB) and hit buffer (%d MB) are L2-resident across frames" % (
                       (2 * f["inner"].size + f["leaves"].size) // 10**6, npix * 32 // 10**6),
                   "wall_ms_per_step": wall_ms, "parallelism": "single GPU"},
        "roofline": {"bound": "hbm", "achieved": alg / (kernel_ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": alg / (kernel_ms / 1e3) / 1e9 / peak, "traffic": None,
                     "note": "latency-bound pointer chase (one ray per thread, %.1f DDA iterations per ray); "
                             "peak %s" % (iters / rays, src)},
        "clocks": clk, "gpu_launches": len(cams),
        "e2e": {"value": rays / (e2e_ms / 1e3) / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 32 * rays},
    }
    if not args.no_cpu_baseline:
        res["cpu_baseline"] = raycast_cpu(args, f, cams)
    return res


def raycast_cpu(args, f, cams, frac=4):
    """The oracle's restated traversal on all host cores, each view at 1/frac
    of the resolution per axis with the full-size projection factor (a
    subsample of the same rays' directions)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py

    t = 0.0
    rays = 0
    for c in cams:
        s = dict(c, width=c["width"] // frac, height=c["height"] // frac)
        t0 = time.perf_counter()
        oracle_py.ssvdag_raycast(f, s)
        t += time.perf_counter() - t0
        rays += s["width"] * s["height"]
    return {"value": rays / t / 1e6, "unit": "Mrays/s", "cores": os.cpu_count(), "kind": "port",
            "sample": "the 4 views at %dx%d (1/%d of the rays per view), OpenMP over all cores" % (
                cams[0]["width"] // frac, cams[0]["height"] // frac, frac * frac)}


def run_floodfill(args, rank, local, world):
    """Hidden-geometry flood fill (outside masks) of the depth-12 terrain's
    SVO, K runs on the resident SVO; value = SVO leaf cells (8 per node)
    per second."""
    import torch

    import svdag_gb300 as sv

    torch.cuda.set_device(local)
    o = sv.Octree(device=local)
    o.upload_triangles(sv.terrain(args.grid, 8, 0.3, args.seed))
    o.buildSVO(args.levels)
    lib = o._lib
    e, s_ = ctypes.c_uint64(), ctypes.c_uint64()
    for _ in range(max(args.warmup, 0)):
        assert lib.svdag_flood_fill(o._h, ctypes.byref(e), ctypes.byref(s_)) == 0
    nodes = o.stats()["n_nodes_svo"]
    l0 = o.stats()["gpu_launches"]
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.5)
    clocks.mark()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        assert lib.svdag_flood_fill(o._h, ctypes.byref(e), ctypes.byref(s_)) == 0
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3 / args.steps
    clk = clocks.stop()
    launches = (o.stats()["gpu_launches"] - l0) // max(1, args.steps)
    # e2e: the fill plus every level's masks copied to the host
    t0 = time.perf_counter()
    for _ in range(max(1, args.steps // 2)):
        o.hiddenGeometryFloodfill()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / max(1, args.steps // 2)
    cells = 8 * nodes
    res = {
        "metric": METRIC, "value": cells / (ms / 1e3) / 1e6, "unit": "Mcells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32 links", "data": "synthetic",
        "config": {"workload": "floodfill: outside masks of the %dx%d terrain's SVO at depth %d (%d nodes, %d leaf "
                               "cells)" % (args.grid, args.grid, args.levels, nodes, cells),
                   "outside_empty_cells": e.value, "outside_surface_voxels": s_.value,
                   "l2": "SVO pools and union-find array (%d MB) exceed L2" % ((44 * nodes) // 10**6),
                   "parallelism": "single GPU"},
        "clocks": clk, "gpu_launches": int(launches),
        "e2e": {"value": cells / (e2e_ms / 1e3) / 1e6, "unit": "Mcells/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(nodes)},
    }
    o.close()
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle_py

        g = max(65, args.grid // 4)
        oo = oracle_py.OracleOctree()
        oo.buildSVO(sv.terrain(g, 8, 0.3, args.seed), args.levels - 2)
        n_cpu = oo.stats()["n_nodes_svo"]
        t0 = time.perf_counter()
        oo.hiddenGeometryFloodfill()
        t = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": 8 * n_cpu / t / 1e6, "unit": "Mcells/s", "cores": 1, "kind": "port",
                               "sample": "the %dx%d terrain's SVO at depth %d (%d nodes), the restated reference "
                                         "traversal on one thread" % (g, g, args.levels - 2, n_cpu)}
    return res


def main():
    args = parse()
    rank, local, world = rank_info()
    if args.workload == "floodfill" and args.impl != "reference":
        res = run_floodfill(args, rank, local, world)
        if rank == 0:
            print(json.dumps(res))
        return
    if args.workload == "raycast" and args.impl != "reference":
        res = run_raycast(args, rank, local, world)
        if rank == 0:
            print(json.dumps(res))
        return
    if args.workload in ("batch", "lossy") and args.impl != "reference":
        res = (run_batch if args.workload == "batch" else run_lossy)(args, rank, local, world)
        if rank == 0:
            print(json.dumps(res))
        return
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
