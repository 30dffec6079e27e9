"""The benchmark's scene at its own size (terrain 2048², depth 12): the files
the GPU encoders write for its DAG, SSVDAG and CSVDAG -- .svdag, .esvdag,
.ussvdag, .ssvdag and the merged .svdag -- have the SHA-256 of the files the
reference itself wrote for the scene (tests/golden/golden.json)."""
import hashlib

import pytest

import svdag_gb300 as sv
from _scenes import SCENES, golden

pytestmark = pytest.mark.gpu
G = golden()


def sha(p):
    with open(p, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def test_headline_files_match_reference(tmp_path):
    name = "terrain2048_L12"
    g = G[name]
    o = sv.Octree()
    o.upload_triangles(SCENES[name]())
    o.buildSVO(g["levels"])
    o.toDAG()
    o.initChildLevels()
    s, c = o.clone(), o.clone()
    s.toSDAG()
    c.mergeAcrossAllLevels()
    out = {}
    for key, x, write in [("svdag", o, lambda x, p: x.save_encoded(p, "svdag")),
                          ("esvdag", o, lambda x, p: x.save_ssvdag(p)),
                          ("ussvdag", s, lambda x, p: x.save_encoded(p, "ussvdag")),
                          ("ssvdag", s, lambda x, p: x.save_ssvdag(p)),
                          ("csv.svdag", c, lambda x, p: x.save_encoded(p, "svdag"))]:
        p = str(tmp_path / ("a." + key))
        write(x, p)
        out[key] = sha(p)
    assert out == g["files"]
