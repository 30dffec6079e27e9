"""The restated SSVDAG ray traversal of the viewer's shader (oracle) against
an independent float64 voxel walk over the built voxels (no GPU): at full
resolution every ray finds the same first voxel; with the shader's level of
detail every hit cell holds set voxels; a truncated file is reported."""
import numpy as np
import pytest

import oracle_py
import svdag_gb300 as sv
from _raycheck import camera_rays, coarse, encoded_scene, first_voxel

CASES = [("ico3_L6", 6, (1.6, 1.3, 1.9), (0.5, 0.5, 0.5)),
         ("ico3_L6", 6, (0.45, 0.52, 0.55), (0.9, 0.2, 0.4)),   # camera inside the box
         ("terrain65_L8", 8, (1.3, 0.9, 1.7), (0.5, 0.3, 0.5)),
         ("terrain65_L8", 8, (0.2, 0.6, 0.3), (0.5, 0.3, 0.5))]


@pytest.mark.parametrize("name,L,eye,target", CASES)
def test_full_resolution_hits_match_a_voxel_walk(name, L, eye, target, tmp_path):
    grid, f = encoded_scene(name, L, tmp_path)
    cam = sv.camera(eye, target, 64, 48, L, pixel_tolerance=1e-6)
    hits, rc = oracle_py.ssvdag_raycast(f, cam)
    assert rc == 0
    hit = hits["t"] > 0
    assert hit.any() and (hits["level"][hit] == L - 1).all()
    v = hits["voxel"][hit]
    assert grid[v[:, 0], v[:, 1], v[:, 2]].all()
    agree = 0
    for i, (o, d) in enumerate(camera_rays(cam)):
        got = tuple(int(x) for x in hits["voxel"][i]) if hit[i] else None
        agree += first_voxel(grid, o, d) == got
    assert agree >= 0.995 * hits.size


def test_level_of_detail_hits_are_set_cells(tmp_path):
    L = 8
    grid, f = encoded_scene("terrain65_L8", L, tmp_path)
    for tol, draw in ((1.0, L), (4.0, L), (1e-6, 5)):
        cam = sv.camera((0.2, 0.6, 0.3), (0.5, 0.3, 0.5), 64, 48, L, pixel_tolerance=tol)
        cam["draw_level"] = draw
        hits, rc = oracle_py.ssvdag_raycast(f, cam)
        hit = hits["t"] > 0
        assert rc == 0 and hit.any()
        for lev in np.unique(hits["level"][hit]):
            sel = hit & (hits["level"] == lev)
            v = hits["voxel"][sel]
            g = coarse(grid, (L - 1) - int(lev))
            assert g[v[:, 0], v[:, 1], v[:, 2]].all()
        if draw < L:
            assert (hits["level"][hit] <= draw - 1).all()


def test_truncated_file_is_reported(tmp_path):
    _, f = encoded_scene("ico3_L6", 6, tmp_path)
    g = dict(f)
    g["leaves"] = f["leaves"][: (f["leaves"].size // 16) * 8].copy()
    cam = sv.camera((0.45, 0.52, 0.55), (0.9, 0.2, 0.4), 32, 24, 6, pixel_tolerance=1e-6)
    hits, rc = oracle_py.ssvdag_raycast(g, cam)
    assert rc == -2 and (hits["t"] == -5).any()
