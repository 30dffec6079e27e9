"""The restated EncodedSSVDAG::traverse (oracle) decodes the host encoder's
.ssvdag of an oracle-built SSVDAG back to exactly the voxels that were built
(no GPU).  terrain65_L8 has two-word (32-bit) child pointers, which the
encoder writes high half first; a truncated file reports depth -2 instead of
reading past its arrays."""
import numpy as np
import pytest

import oracle_py
import svdag_gb300 as sv
from _occupancy import occupancy, voxel_centres
from _scenes import SCENES


def _encoded(name, L, tmp_path):
    o = oracle_py.OracleOctree()
    o.buildSVO(SCENES[name](), L)
    grid = occupancy(o.pool())
    o.toDAG()
    o.initChildLevels()
    o.toSDAG()
    p = str(tmp_path / "a.ssvdag")
    sv.write_encoded(p, "ssvdag", o.pool(), o.stats()["n_nodes"], 3)
    return o, grid, oracle_py.read_ssvdag(p)


def _has_two_word_pointers(f):
    inner = f["inner"].astype(np.int64)
    starts = list(f["level_offsets"]) + [inner.size]
    for l in range(len(f["level_offsets"])):
        p = starts[l]
        while p < starts[l + 1]:
            h = int(inner[p])
            codes = [(h >> (2 * c)) & 3 for c in range(8)]
            if any(c >= 2 for c in codes):
                return True
            p += 1 + sum(0 if c == 0 else (1 if c == 1 else 2) for c in codes)
    return False


@pytest.mark.parametrize("name,L", [("ico3_L6", 6), ("terrain65_L8", 8)])
def test_oracle_traverse_decodes_the_built_voxels(name, L, tmp_path):
    o, grid, f = _encoded(name, L, tmp_path)
    if name == "terrain65_L8":
        assert _has_two_word_pointers(f)
    depth = oracle_py.ssvdag_traverse(f, voxel_centres(L))
    assert ((depth == L) == grid.ravel()).all()
    assert int((depth == L).sum()) == o.stats()["n_total_voxels"]


def test_oracle_traverse_truncated_file(tmp_path):
    _, grid, f = _encoded("ico3_L6", 6, tmp_path)
    g = dict(f)
    g["leaves"] = f["leaves"][: f["leaves"].size // 2]
    depth = oracle_py.ssvdag_traverse(g, voxel_centres(6))
    assert (depth == -2).any()
    ok = depth != -2
    assert ((depth[ok] == 6) == grid.ravel()[ok]).all()


@pytest.mark.parametrize("name", ["ico3_L6", "ico5_L7"])
def test_oracle_traverse_matches_the_reference_above_the_bricks(name, tmp_path):
    """The restated traverse equals the reference's own EncodedSSVDAG::traverse
    (compiled from its sources; golden results) on every query whose walk ends
    above the leaf bricks, on the reference's own .ssvdag file; at the bricks
    both walks reach the brick level (the reference reads bricks in another
    order than its encoder writes them)."""
    import hashlib
    import os

    from _scenes import GOLDEN, SCENES, golden, traverse_points

    g = golden()[name]
    L = g["levels"]
    o = oracle_py.OracleOctree()
    o.buildSVO(SCENES[name](), L)
    o.toDAG()
    o.initChildLevels()
    o.toSDAG()
    p = str(tmp_path / "a.ssvdag")
    sv.write_encoded(p, "ssvdag", o.pool(), o.stats()["n_nodes"], 3)
    with open(p, "rb") as fh:
        assert hashlib.sha256(fh.read()).hexdigest() == g["files"]["ssvdag"]
    ref = np.load(os.path.join(GOLDEN, g["traverse"]["file"]))["depth"].astype(np.int32)
    got = oracle_py.ssvdag_traverse(oracle_py.read_ssvdag(p), traverse_points(L))
    above = ref <= L - 3
    assert np.array_equal(got[above], ref[above])
    assert (got[~above] >= L - 2).all()
