"""Lossy LSVDAG on the GPU: the exact-proposer form bit-exact with the
oracle's restatement; the proposer network's forward/backward kernels against
the CPU model; and what training buys over the same network untrained, at
the same proposal budget, against the exact method."""
import numpy as np
import pytest

import mlp_ref
import oracle_py
import svdag_gb300 as sv
from _scenes import box_scene
from test_gpu_parity import first_mismatch

pytestmark = pytest.mark.gpu


def scene(levels, grid, boxes, seed):
    return np.concatenate([sv.terrain(grid, 8, 0.3, seed), box_scene(boxes, levels, seed + 1)])


def gpu_dag(tris, levels):
    o = sv.Octree()
    o.upload_triangles(tris)
    o.buildSVO(levels)
    o.toDAG()
    return o


@pytest.mark.parametrize("levels,grid,boxes", [(9, 129, 200), (10, 257, 400)])
def test_lossy_exact_matches_oracle(levels, grid, boxes):
    tris = scene(levels, grid, boxes, 5)
    ref = oracle_py.OracleOctree()
    ref.buildSVO(tris, levels)
    ref.toDAG()
    merged = ref.lossyExact(3, 5, 0.01)
    o = gpu_dag(tris, levels)
    st = o.lossy("exact", 3, 5, 0.01)
    assert st["merged"] == merged > 0
    assert first_mismatch(o.pool(), ref.pool()) is None
    assert st["nodes_after"] == o.stats()["n_nodes"] < st["nodes_before"]


def test_network_gradients_match_cpu_model():
    m = sv.Mlp(seed=11)
    w = m.params()
    rng = np.random.default_rng(4)
    xa = (rng.random((40, 512)) < 0.3).astype(np.float32)
    xb = (rng.random((40, 512)) < 0.3).astype(np.float32)
    t = rng.random(40).astype(np.float32)
    loss, g = m.loss_grad(xa, xb, t)
    rl, rg = mlp_ref.loss_grad(w, xa, xb, t)
    assert abs(loss - rl) <= 1e-4 * max(1.0, abs(rl))
    assert np.max(np.abs(g - rg)) <= 1e-3 * max(1e-6, np.max(np.abs(rg)))
    e = m.embed(xa)
    assert np.allclose(e, mlp_ref.forward(w, xa.astype(np.float64))[2], rtol=1e-4, atol=1e-4)


def test_training_beats_the_untrained_network():
    levels = 10
    tris = scene(levels, 257, 800, 9)
    base = gpu_dag(tris, levels)
    res = {}
    for kind in ("exact", "learned", "untrained"):
        o = base.clone()
        res[kind] = o.lossy(kind, 3, 5, 0.01, top_k=8, train_pairs=200000, epochs=3, seed=2)
    saved = {k: v["nodes_before"] - v["nodes_after"] for k, v in res.items()}
    assert saved["exact"] > 0
    # the same proposal budget per candidate (top_k): training finds more of
    # the merges, with far fewer exact checks than the exact method
    assert saved["learned"] > saved["untrained"]
    for k in ("learned", "untrained"):
        assert res[k]["pairs_evaluated"] < res["exact"]["pairs_evaluated"]
