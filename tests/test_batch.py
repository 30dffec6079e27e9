"""Voxel-brick chunks against the oracle, chunk by chunk and bit-exact: the
plain per-chunk form (svdag_import_bricks, then the ordinary reductions) and
the batched form (svdag_batch_*: all chunks reduced together, height by
height) both equal the restated reference run on the chunk's node pools
(the NodeData route, then toDAG / toSDAG / initChildLevels +
mergeAcrossAllLevels)."""
import numpy as np
import pytest

import oracle_py
import svdag_gb300 as sv
from test_gpu_parity import first_mismatch

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def oracle_chain(depth, bricks):
    o = oracle_py.OracleOctree()
    o.buildFromBricks(depth, bricks.cpu().numpy())
    o.toDAG()
    dag = o.pool()
    s = o.clone()
    s.toSDAG()
    c = o.clone()
    c.initChildLevels()
    c.mergeAcrossAllLevels()
    return o, dag, s.pool(), c.pool(), o.stats()


def chunks(seed, n, depths=(2, 3, 4, 5, 6, 7)):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        d = int(rng.choice(depths))
        out.append((d, sv.noise_bricks(d, seed * 1000 + i, float(rng.uniform(0.05, 0.40)))))
    return out


@pytest.mark.parametrize("depth,fill", [(3, 0.2), (5, 0.05), (6, 0.4), (7, 0.15)])
def test_import_bricks_matches_oracle(depth, fill):
    b = sv.noise_bricks(depth, 77 + depth, fill)
    ref, dag, sdag, csv, rst = oracle_chain(depth, b)
    o = sv.Octree()
    o.import_bricks(depth, b)
    assert o.stats()["n_total_voxels"] == rst["n_total_voxels"] > 0
    o.toDAG()
    assert first_mismatch(o.pool(), dag) is None
    s = o.clone()
    s.toSDAG()
    assert first_mismatch(s.pool(), sdag) is None
    c = o.clone()
    c.initChildLevels()
    c.mergeAcrossAllLevels()
    assert first_mismatch(c.pool(), csv) is None


def test_batch_matches_oracle_per_chunk():
    cs = chunks(5, 20)
    zero = torch.zeros(8 ** 3, dtype=torch.uint8, device="cuda")
    full = torch.full((8 ** 2,), 255, dtype=torch.uint8, device="cuda")
    cs += [(4, zero), (3, full)]
    B = sv.Batch()
    for d, b in cs:
        B.add_chunk(d, b)
    B.build()
    for i, (d, b) in enumerate(cs):
        _, dag, sdag, csv, rst = oracle_chain(d, b)
        g = B.result(i, "dag")
        assert g.stats()["n_total_voxels"] == rst["n_total_voxels"]
        assert first_mismatch(g.pool(), dag) is None, i
        assert first_mismatch(B.result(i, "sdag").pool(), sdag) is None, i
        assert first_mismatch(B.result(i, "csvdag").pool(), csv) is None, i


def test_batch_settings_and_autotune_keep_results():
    cs = chunks(9, 12, depths=(3, 4, 5, 6))
    B = sv.Batch()
    for d, b in cs:
        B.add_chunk(d, b)
    B.build()
    want = [B.result(i, "sdag").pool() for i in range(len(cs))]
    for tf, th, st in [(1.5, 128, 1), (4.0, 512, 8)]:
        B.set_tuning(tf, th, st)
        B.build()
        for i in range(len(cs)):
            assert first_mismatch(B.result(i, "sdag").pool(), want[i]) is None
    B.autotune(max_trials=6)
    t = B.tuning()
    assert 1.25 <= t["table_factor"] <= 16 and t["streams"] >= 1
    for i in range(len(cs)):
        assert first_mismatch(B.result(i, "sdag").pool(), want[i]) is None
    assert B.stats()["gpu_launches"] > 0


@pytest.mark.parametrize("share", ["1e-9", None])
def test_estimated_tables_keep_results(monkeypatch, share):
    """The per-height hash tables are sized from the distinct-key shares seen
    by earlier builds; a table that proves too small is rebuilt at full size.
    Forced tiny estimates (SVDAG_BATCH_TABLE_SHARE: the smallest table, 2^17
    slots, against the distinct keys of a depth-10 chunk's lowest heights)
    and the learned ones (second build) give the plain form's pools."""
    cs = chunks(13, 6, depths=(4, 5, 6)) + [(10, sv.noise_bricks(10, 4242, 0.3)), (8, sv.noise_bricks(8, 4243, 0.12))]
    want = []
    for d, b in cs:
        o = sv.Octree()
        o.import_bricks(d, b)
        o.toDAG()
        s = o.clone()
        s.toSDAG()
        want.append((o.pool(), s.pool()))
    if share is not None:
        monkeypatch.setenv("SVDAG_BATCH_TABLE_SHARE", share)
    B = sv.Batch()
    for d, b in cs:
        B.add_chunk(d, b)
    for _ in range(2):
        B.build(sdag=True, csvdag=False)
        for i in range(len(cs)):
            assert first_mismatch(B.result(i, "dag").pool(), want[i][0]) is None, i
            assert first_mismatch(B.result(i, "sdag").pool(), want[i][1]) is None, i
    retries = B.stats()["table_retries"]
    if share is not None:
        assert retries > 0
    else:
        assert retries == 0
