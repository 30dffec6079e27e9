"""The .svdag / .esvdag / .ussvdag / .ssvdag writers reproduce the reference's
files byte for byte (golden SHA-256 of the files the reference itself wrote),
fed with node pools the oracle pins to the reference."""
import hashlib
import os

import pytest

import oracle_py
import svdag_gb300 as sv
from _scenes import HEAVY, SCENES, golden

G = golden()
CASES = sorted(k for k in G if not G[k]["step_levels"] and k not in HEAVY)


def sha(p):
    with open(p, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


@pytest.mark.parametrize("name", CASES)
def test_files_match_reference(name, tmp_path):
    g = G[name]
    o = oracle_py.OracleOctree()
    o.buildSVO(SCENES[name](), g["levels"])
    o.toDAG()
    o.initChildLevels()
    dag = o.pool()
    nd = o.stats()["n_nodes"]
    s = o.clone()
    s.toSDAG()
    c = o.clone()
    c.mergeAcrossAllLevels()
    out = {}
    p = str(tmp_path / "a.svdag")
    sv.write_encoded(p, "svdag", dag, nd, 2)
    out["svdag"] = sha(p)
    p = str(tmp_path / "a.esvdag")
    sv.write_encoded(p, "ssvdag", dag, nd, 2)
    out["esvdag"] = sha(p)
    p = str(tmp_path / "a.ussvdag")
    sv.write_encoded(p, "ussvdag", s.pool(), s.stats()["n_nodes"], 3)
    out["ussvdag"] = sha(p)
    p = str(tmp_path / "a.ssvdag")
    sv.write_encoded(p, "ssvdag", s.pool(), s.stats()["n_nodes"], 3)
    out["ssvdag"] = sha(p)
    p = str(tmp_path / "a.csv.svdag")
    sv.write_encoded(p, "svdag", c.pool(), c.stats()["n_nodes"], 2)
    out["csv.svdag"] = sha(p)
    assert out == g["files"]


def test_wrong_state_is_refused(tmp_path):
    """The reference's encoders refuse the wrong octree state
    (encoded_svdag.cpp:109-112, encoded_ussvdag.cpp:90-93)."""
    o = oracle_py.OracleOctree()
    o.buildSVO(SCENES["ico3_L6"](), 6)
    o.toDAG()
    with pytest.raises(sv.SvdagError):
        sv.write_encoded(str(tmp_path / "x.ussvdag"), "ussvdag", o.pool(), 1, 2)
    with pytest.raises(sv.SvdagError):
        sv.write_encoded(str(tmp_path / "x.svdag"), "svdag", o.pool(), 1, 3)
