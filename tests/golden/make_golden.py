"""Generates the golden fixtures in this directory by running the REFERENCE
build path (oracle/_ref/ref_dump, compiled from the reference's own sources
by oracle/Makefile) on seeded synthetic scenes.

    python tests/golden/make_golden.py

Each case records the reference's counts and SHA-256 digests of its SVO,
DAG, SDAG and CSVDAG node pools (48-byte records, oracle/ref_dump.cpp), of
the pool toSDAG leaves with skipSymmetry (pointer compression only), of the
leavesCenters list buildSVO fills (plain builds), of the pool toSDAG leaves
when run straight on the SVO (plain builds), and of
the encoded .svdag/.esvdag/.ussvdag/.ssvdag/.csv.svdag files; the FLOOD cases
also the outside masks of the reference's hiddenGeometryFloodfill.  Small
cases also keep their full DAG/SDAG/CSVDAG pools as .npz.  `--obj` writes
obj_ingest.json: the triangle soups the reference's Scene::loadObj builds
from seeded OBJ files full of parsing edge cases.
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

sys.path.insert(0, os.path.dirname(HERE))
from _scenes import traverse_points  # noqa: E402

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
    "cavity_L7": (lambda: cavity_scene(), 7, 0, False),
}
# cases whose SVO also goes through the reference's hiddenGeometryFloodfill
# (their start corner cell is empty)
FLOOD = {"ico3_L6", "ico5_L7", "terrain65_L8", "terrain129_L9", "cavity_L7", "ico4_L8_seed5"}
# cases whose .ssvdag encoding goes through the reference's
# EncodedSSVDAG::traverse on traverse_points(levels) (all their child
# pointers are one word, where the reference's decoder reads its own
# encoding; tests/test_traverse.py says what the comparison covers)
TRAVERSE = {"ico3_L6", "ico5_L7"}


# cases whose DAG goes through the reference's toLossyDag up to its MCL
# clustering: name -> (inflation, allowed diff factor, included ref count).
# A stand-in `mcl` records every batch of candidate edges the reference
# writes (edges<lev>.txt, cluster.hpp:145-152) and answers with singleton
# clusters; the edges of the two lowest processed levels (levels - 2, one-bit
# hash probe; levels - 3, hash + diffSubtrees) are kept.
LOSSY = {"terrain65_L8": (2.0, 1.0, 1), "ico5_L7": (2.0, 1.0, 1), "boxes_L8": (2.0, 2.0, 2),
         "terrain129_L9": (2.0, 1.5, 3)}
FAKE_MCL = """#!/bin/sh
# stand-in for the MCL program: keeps the edges file, answers singletons
in="$1"; out=""
while [ $# -gt 0 ]; do if [ "$1" = "-o" ]; then out="$2"; fi; shift; done
cat "$in" >> "$in.all"
awk '{print $1; print $2}' "$in" | sort -n -u > "$out"
"""


def run_lossy(name, obj, levels, params):
    """Runs the reference's toLossyDag on the scene's DAG with the stand-in
    MCL; returns the candidate edges of levels - 2 and levels - 3."""
    with tempfile.TemporaryDirectory() as td:
        home = os.path.join(td, "home")
        os.makedirs(os.path.join(home, "local", "bin"))
        mcl = os.path.join(home, "local", "bin", "mcl")
        with open(mcl, "w") as f:
            f.write(FAKE_MCL)
        os.chmod(mcl, 0o755)
        env = dict(os.environ, HOME=home)
        r = subprocess.run([REF_DUMP, obj, str(levels), os.path.join(td, "out"), "--lossy"] + [str(x) for x in params],
                           cwd=td, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        # the reference's progress logger divides by zero on levels of fewer
        # than 5 nodes (round(size / 10) == 0) and takes the process down
        # there; the levels below it are complete once the next one started
        started = {int(x.split(":")[0]) for x in r.stdout.split("\nLevel ")[1:]}
        out = {}
        for lev in (levels - 2, levels - 3):
            assert r.returncode == 0 or (lev - 1) in started, (name, lev, r.returncode)
            path = os.path.join(td, "edges%d.txt.all" % lev)
            rows = [l.split() for l in open(path)] if os.path.exists(path) else []
            rows.sort(key=lambda t: (int(t[0]), int(t[1])))
            out[lev] = rows
        return out


# seeded OBJ files of tests/_objgen.py (without the face records the
# reference's loader crashes on) run through the reference's Scene::loadObj:
# name -> (seed, lines, final newline)
OBJ_CASES = {"obj_s1": (1, 3000, True), "obj_s2": (2, 60000, True), "obj_s3": (3, 60000, False),
             "obj_s5_short": (5, 20000, True)}
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


def cavity_scene():
    """A closed box shell with a sealed box cavity inside it."""
    outer = sv.boxes(np.array([[0.2, 0.2, 0.2]]), np.array([[0.8, 0.8, 0.8]]))
    inner = sv.boxes(np.array([[0.4, 0.4, 0.4]]), np.array([[0.6, 0.6, 0.6]]))
    return np.concatenate([outer, inner])


def read_levels_u8(path):
    """Per-level byte arrays (u64 count, then count bytes, per level)."""
    raw = open(path, "rb").read()
    out, o = [], 0
    while o < len(raw):
        n = int(np.frombuffer(raw[o:o + 8], np.uint64)[0])
        o += 8
        out.append(np.frombuffer(raw[o:o + n], np.uint8))
        o += n
    return out


def levels_digest(levels):
    h = hashlib.sha256()
    for lev in levels:
        h.update(np.uint64(len(lev)).tobytes())
        h.update(np.ascontiguousarray(lev).tobytes())
    return h.hexdigest()


def sha(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def run_case(name, make, levels, step, keep):
    tris = make()
    with tempfile.TemporaryDirectory() as td:
        obj = os.path.join(td, "scene.obj")
        sv.write_obj(obj, tris, True)
        pre = os.path.join(td, "out")
        extra = ["--sdag-skip", "--leaf-centers", "--sdag-from-svo"] + (["--flood"] if name in FLOOD else [])
        if name in TRAVERSE:
            pts = traverse_points(levels)
            with open(os.path.join(td, "pts.bin"), "wb") as f:
                f.write(np.uint64(pts.shape[0]).tobytes())
                f.write(pts.tobytes())
            extra += ["--traverse", os.path.join(td, "pts.bin")]
        r = subprocess.run([REF_DUMP, obj, str(levels), pre] + ([str(step)] if step else []) + extra,
                           stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, check=True)
        line = [l for l in r.stdout.splitlines() if l.startswith("REFJSON ")][-1]
        info = json.loads(line[len("REFJSON "):])
        info["missing_correspondence_prints"] = r.stdout.count("Missing correspondence")
        skip = [l for l in r.stdout.splitlines() if l.startswith("REFSKIP ")][-1]
        info["nNodesSDAGSkipSymmetry"] = json.loads(skip[len("REFSKIP "):])["nNodesSDAG"]
        info["step_levels"] = step
        info["n_tris"] = int(tris.shape[0])
        info["tris_sha256"] = hashlib.sha256(np.ascontiguousarray(tris).tobytes()).hexdigest()
        pools = {}
        for kind in ("svo", "dag", "sdag", "csv", "sdagskip", "sdagsvo"):
            p = pre + "." + kind + ".pool"
            if not os.path.exists(p):
                continue
            pool = oracle_py.read_pool(p)
            info[kind] = {"counts": [int(len(l)) for l in pool["pool"]], "digest": oracle_py.pool_digest(pool["pool"]),
                          "nnodes": int(pool["nnodes"]), "nvoxels": int(pool["nvoxels"])}
            pools[kind] = pool["pool"]
        info["files"] = {ext: sha(pre + "." + ext) for ext in ("svdag", "esvdag", "ussvdag", "ssvdag", "csv.svdag")}
        if os.path.exists(pre + ".leafctr"):
            raw = open(pre + ".leafctr", "rb").read()
            info["leaf_centers"] = {"count": int(np.frombuffer(raw[:8], np.uint64)[0]),
                                    "sha256": hashlib.sha256(raw[8:]).hexdigest()}
        if name in TRAVERSE:
            res = np.fromfile(pre + ".trav", np.int32)
            np.savez_compressed(os.path.join(HERE, name + "_traverse.npz"), depth=res.astype(np.int8))
            info["traverse"] = {"points": int(res.size), "file": name + "_traverse.npz"}
        if name in LOSSY:
            edges = run_lossy(name, obj, levels, LOSSY[name])
            arrs, info_l = {}, {}
            for lev, rows in edges.items():
                arrs["l%d_src" % lev] = np.array([int(t[0]) for t in rows], np.uint32)
                arrs["l%d_tgt" % lev] = np.array([int(t[1]) for t in rows], np.uint32)
                arrs["l%d_w" % lev] = np.array([t[2] for t in rows], "<U16")
                info_l[str(lev)] = len(rows)
            np.savez_compressed(os.path.join(HERE, name + "_lossy.npz"), **arrs)
            info["lossy"] = {"params": list(LOSSY[name]), "edges": info_l, "file": name + "_lossy.npz"}
        if name in FLOOD:
            masks = read_levels_u8(pre + ".outside")
            info["outside"] = {"counts": [int(len(m)) for m in masks], "digest": levels_digest(masks),
                               "marked": [int(np.count_nonzero(m)) for m in masks]}
        if keep:
            arrs = {}
            for kind in ("dag", "sdag", "csv"):
                for l, lev in enumerate(pools[kind]):
                    arrs["%s_%d" % (kind, l)] = lev
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)
    return info


def run_obj_cases():
    """The reference loader's triangle soup and bounding box for each seeded
    OBJ file (obj_ingest.json): SHA-256 of the float[9] triangles and the
    bbox as float32 bit patterns."""
    sys.path.insert(0, os.path.dirname(HERE))
    from _objgen import make_obj

    out = {}
    for name, (seed, lines, final_nl) in OBJ_CASES.items():
        with tempfile.TemporaryDirectory() as td:
            obj = os.path.join(td, "s.obj")
            with open(obj, "wb") as f:
                f.write(make_obj(seed, lines, final_newline=final_nl, reference_safe=True))
            pre = os.path.join(td, "out")
            subprocess.run([REF_DUMP, obj, "1", pre, "--soup-only"], stdout=subprocess.DEVNULL,
                           stderr=subprocess.DEVNULL, check=True)
            raw = open(pre + ".soup", "rb").read()
            n = int(np.frombuffer(raw[:8], np.uint64)[0])
            bb = np.frombuffer(raw[8:32], np.float32)
            tris = raw[32:]
            assert len(tris) == 36 * n
            out[name] = {"seed": seed, "lines": lines, "final_newline": final_nl, "n_tris": n,
                         "tris_sha256": hashlib.sha256(tris).hexdigest(),
                         "bbox_bits": [int(x) for x in bb.view(np.uint32)]}
        print(name, n, flush=True)
    with open(os.path.join(HERE, "obj_ingest.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


def main(argv):
    """`make_golden.py` regenerates every default case; `make_golden.py
    --only NAME [NAME ...]` regenerates the named cases and keeps the others
    already in golden.json; `make_golden.py --obj` regenerates the OBJ
    loader fixtures."""
    if argv[:1] == ["--obj"]:
        run_obj_cases()
        return
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
