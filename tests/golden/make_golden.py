"""Generates the golden fixtures in this directory by running the REFERENCE
build path (oracle/_ref/ref_dump, compiled from the reference's own sources
by oracle/Makefile) on seeded synthetic scenes.

    python tests/golden/make_golden.py

Each case records the reference's counts and SHA-256 digests of its SVO,
DAG, SDAG and CSVDAG node pools (48-byte records, oracle/ref_dump.cpp) and of
the encoded .svdag/.esvdag/.ussvdag/.ssvdag/.csv.svdag files.  Small cases
also keep their full DAG/SDAG/CSVDAG pools as .npz.
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "svdag-compression_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import svdag_gb300 as sv  # noqa: E402
import oracle_py  # noqa: E402

REF_DUMP = os.path.join(ROOT, "oracle", "_ref", "ref_dump")

# name -> (scene builder, levels, step_levels, keep_full_pools)
CASES = {
    "ico5_L9": (lambda: sv.icosphere(5, 0.4, 0.08, 1234), 9, 0, False),
    "ico5_L7": (lambda: sv.icosphere(5, 0.4, 0.08, 1234), 7, 0, True),
    "ico3_L6": (lambda: sv.icosphere(3, 0.4, 0.08, 99), 6, 0, True),
    "ico4_L8_seed5": (lambda: sv.icosphere(4, 0.35, 0.08, 5), 8, 0, False),
    "terrain65_L8": (lambda: sv.terrain(65, 8, 0.3, 7), 8, 0, True),
    "terrain129_L9": (lambda: sv.terrain(129, 8, 0.3, 11), 9, 0, False),
    "terrain129_L9_step1": (lambda: sv.terrain(129, 8, 0.3, 11), 9, 1, False),
    "terrain257_L10": (lambda: sv.terrain(257, 8, 0.3, 3), 10, 0, False),
    "boxes_L8": (lambda: box_scene(300, 8, 21), 8, 0, False),
    # the benchmark's headline workload: 2048^2 fBm terrain (8,396,796
    # triangles), depth 12, seed 7; the reference's single-threaded build
    # takes minutes here, so it is generated on request (--only)
    "terrain2048_L12": (lambda: sv.terrain(2048, 8, 0.3, 7), 12, 0, False),
}
# cases a plain run skips (regenerate with --only NAME)
ON_REQUEST = {"terrain2048_L12"}


def box_scene(n, levels, seed):
    rng = np.random.default_rng(seed)
    res = 2 ** levels
    lo = rng.integers(0, res - 8, size=(n, 3))
    side = rng.integers(1, 16, size=(n, 3))
    hi = np.minimum(lo + side, res)
    # box faces offset by a quarter voxel so no face lies on a voxel boundary
    return sv.boxes((lo + 0.25) / res, (hi - 0.25) / res)


def sha(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def run_case(name, make, levels, step, keep):
    tris = make()
    with tempfile.TemporaryDirectory() as td:
        obj = os.path.join(td, "scene.obj")
        sv.write_obj(obj, tris, True)
        pre = os.path.join(td, "out")
        r = subprocess.run([REF_DUMP, obj, str(levels), pre] + ([str(step)] if step else []),
                           stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, check=True)
        line = [l for l in r.stdout.splitlines() if l.startswith("REFJSON ")][-1]
        info = json.loads(line[len("REFJSON "):])
        info["missing_correspondence_prints"] = r.stdout.count("Missing correspondence")
        info["step_levels"] = step
        info["n_tris"] = int(tris.shape[0])
        info["tris_sha256"] = hashlib.sha256(np.ascontiguousarray(tris).tobytes()).hexdigest()
        pools = {}
        for kind in ("svo", "dag", "sdag", "csv"):
            p = pre + "." + kind + ".pool"
            if not os.path.exists(p):
                continue
            pool = oracle_py.read_pool(p)
            info[kind] = {"counts": [int(len(l)) for l in pool["pool"]], "digest": oracle_py.pool_digest(pool["pool"]),
                          "nnodes": int(pool["nnodes"]), "nvoxels": int(pool["nvoxels"])}
            pools[kind] = pool["pool"]
        info["files"] = {ext: sha(pre + "." + ext) for ext in ("svdag", "esvdag", "ussvdag", "ssvdag", "csv.svdag")}
        if keep:
            arrs = {}
            for kind in ("dag", "sdag", "csv"):
                for l, lev in enumerate(pools[kind]):
                    arrs["%s_%d" % (kind, l)] = lev
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)
    return info


def main(argv):
    """`make_golden.py` regenerates every default case; `make_golden.py
    --only NAME [NAME ...]` regenerates the named cases and keeps the others
    already in golden.json."""
    path = os.path.join(HERE, "golden.json")
    if argv[:1] == ["--only"]:
        names = argv[1:]
        with open(path) as f:
            out = json.load(f)
    else:
        names = [n for n in CASES if n not in ON_REQUEST]
        out = {}
    for name in names:
        make, levels, step, keep = CASES[name]
        out[name] = run_case(name, make, levels, step, keep)
        print(name, out[name]["dag"]["counts"][-1], out[name].get("nNodesSDAG"), flush=True)
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main(sys.argv[1:])
