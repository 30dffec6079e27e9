"""Multi-threaded OBJ ingest (Scene::loadObj on host threads): the triangle
soup and bounding box equal a restatement of the reference's parsing rules
(src/symvox/scene.cpp:98-233, buildTriVector :394-416) for every thread
count, on files that put the rules' edge cases on both sides of the pieces'
cut points.  No GPU."""
import hashlib
import json
import os

import numpy as np
import pytest

import svdag_gb300 as sv
from _objgen import make_obj as _make_obj
from _objgen import reference_parse

@pytest.mark.parametrize("seed,n_lines,final_newline", [(1, 3000, True), (2, 60000, True), (3, 60000, False)])
def test_parallel_obj_ingest_matches_the_reference_rules(seed, n_lines, final_newline, tmp_path):
    data = _make_obj(seed, n_lines, final_newline=final_newline)
    p = tmp_path / "s.obj"
    p.write_bytes(data)
    want_t, want_b = reference_parse(data)
    assert want_t.shape[0] > 0
    for threads in (1, 3, 16):
        t, b = sv.load_obj(str(p), threads=threads)
        assert np.array_equal(t.view(np.uint32), want_t.view(np.uint32)), threads
        assert np.array_equal(b.view(np.uint32), want_b.view(np.uint32)), threads


def test_bincache_round_trip(tmp_path):
    data = _make_obj(4, 20000)
    p = tmp_path / "c.obj"
    p.write_bytes(data)
    t0, b0 = sv.load_obj(str(p), threads=8, use_bincache=True, write_bincache=True)
    assert os.path.exists(str(p) + ".bincache")
    t1, b1 = sv.load_obj(str(p), threads=8, use_bincache=True)
    assert np.array_equal(t0.view(np.uint32), t1.view(np.uint32))
    assert np.array_equal(b0.view(np.uint32), b1.view(np.uint32))


def test_synthetic_terrain_obj(tmp_path):
    tris = sv.terrain(129, 8, 0.3, 7)
    p = tmp_path / "t.obj"
    sv.write_obj(str(p), tris)
    t, b = sv.load_obj(str(p), threads=0)
    assert np.array_equal(t.view(np.uint32), tris.reshape(-1, 9).view(np.uint32))
    assert b.tolist() == [0, 0, 0, 1, 1, 1]


with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "obj_ingest.json")) as _f:
    OBJ_GOLDEN = json.load(_f)


@pytest.mark.parametrize("name", sorted(OBJ_GOLDEN))
def test_ingest_matches_the_reference_loader(name, tmp_path):
    """The triangle soup and bounding box equal what the reference's own
    Scene::loadObj (compiled from its sources; tests/golden/make_golden.py
    --obj) built from the same seeded file, for 1, 3 and 16 threads."""
    g = OBJ_GOLDEN[name]
    p = tmp_path / "s.obj"
    p.write_bytes(_make_obj(g["seed"], g["lines"], final_newline=g["final_newline"], reference_safe=True))
    for threads in (1, 3, 16):
        t, b = sv.load_obj(str(p), threads=threads)
        assert t.shape[0] == g["n_tris"], threads
        assert hashlib.sha256(np.ascontiguousarray(t).tobytes()).hexdigest() == g["tris_sha256"], threads
        assert [int(x) for x in b.view(np.uint32)] == g["bbox_bits"], threads
