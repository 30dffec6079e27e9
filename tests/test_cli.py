"""The svbuilder CLI on the GPU build path writes the reference's files byte
for byte (golden SHA-256 of the files the reference itself wrote), for the
plain build (numBuildSteps 0) and the chunked one (numBuildSteps 1), with and
without cross-level merging."""
import hashlib
import os
import subprocess

import pytest

import svdag_gb300 as sv
from _scenes import SCENES, golden

pytestmark = pytest.mark.gpu
G = golden()
CLI = os.path.join(os.path.dirname(sv.__file__), "bin", "svbuilder")


def sha(p):
    with open(p, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


@pytest.mark.parametrize("name", ["ico3_L6", "terrain65_L8", "boxes_L8", "terrain129_L9_step1"])
def test_svbuilder_files_match_reference(name, tmp_path):
    g = G[name]
    obj = str(tmp_path / "scene.obj")
    sv.write_obj(obj, SCENES[name](), True)
    L, step = str(g["levels"]), str(g["step_levels"])
    r = subprocess.run([CLI, obj, L, step], cwd=str(tmp_path), stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    base = str(tmp_path / ("scene_" + L))
    got = {ext: sha(base + "." + ext) for ext in ("svdag", "esvdag", "ussvdag", "ssvdag")}
    r = subprocess.run([CLI, obj, L, step, "-c"], cwd=str(tmp_path), stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    got["csv.svdag"] = sha(base + "-multi.svdag")
    assert got == g["files"]
    assert ("Voxels:" in r.stdout) and os.path.exists(str(tmp_path / "stats.txt"))


@pytest.mark.parametrize("name", ["ico3_L6", "ico5_L9", "terrain65_L8", "boxes_L8", "terrain129_L9_step1"])
def test_gpu_encoder_matches_reference_files(name, tmp_path):
    """svdag_encode (the SVDAG / CSVDAG / USSVDAG streams built on the GPU)
    gives the reference's files byte for byte."""
    g = G[name]
    o = sv.Octree()
    o.upload_triangles(SCENES[name]())
    if g["step_levels"]:
        o.buildDAG(g["levels"], g["step_levels"])
    else:
        o.buildSVO(g["levels"])
        o.toDAG()
    o.initChildLevels()
    p = str(tmp_path / "a")
    o.save_encoded(p + ".svdag", "svdag")
    s = o.clone()
    s.toSDAG()
    s.save_encoded(p + ".ussvdag", "ussvdag")
    c = o.clone()
    c.mergeAcrossAllLevels()
    c.save_encoded(p + ".csv.svdag", "svdag")
    got = {ext: sha(p + "." + ext) for ext in ("svdag", "ussvdag", "csv.svdag")}
    assert got == {ext: g["files"][ext] for ext in got}


def test_svbuilder_lossy(tmp_path):
    """svbuilder -l: the DAG's .svdag and .esvdag as the reference writes them
    (its files, byte for byte), then the lossy DAG's files under the
    reference's -l_<infl>_<diff>_<refs> names, equal to the library's lossy
    LSVDAG (exact proposals) encoded by the host writers."""
    name = "terrain129_L9"
    g = G[name]
    obj = str(tmp_path / "scene.obj")
    tris = SCENES[name]()
    sv.write_obj(obj, tris, True)
    L = str(g["levels"])
    r = subprocess.run([CLI, obj, L, "0", "-l", "2", "1", "1"], cwd=str(tmp_path), stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    base = str(tmp_path / ("scene_" + L))
    assert sha(base + ".svdag") == g["files"]["svdag"]
    assert sha(base + ".esvdag") == g["files"]["esvdag"]
    merged = int(r.stdout.split("Lossy LSVDAG       : ")[1].split()[0])
    o = sv.Octree()
    o.upload_triangles(tris)
    o.buildSVO(g["levels"])
    o.toDAG()
    o.initChildLevels()
    st = o.lossy("exact", 3, 5, 0.01)
    assert st["merged"] == merged > 0
    o.initChildLevels()
    want = str(tmp_path / "want.svdag")
    sv.write_encoded(want, "svdag", o.pool(), o.stats()["n_nodes"], 2)
    assert sha(base + "-l_2.0_1.0_1.svdag") == sha(want)
    for ext in ("ussvdag", "ssvdag", "esvdag"):
        assert os.path.getsize(base + "-l_2.0_1.0_1." + ext) > 0
    with open(str(tmp_path / "stats.txt")) as f:
        assert "Lossy stats, 2.00, 1.00, 1" in f.read()
