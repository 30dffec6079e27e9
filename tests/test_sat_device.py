"""The voxelizer's certified SAT filter as the GPU runs it (sat.cuh compiled
by nvcc for sm_103a, through svdag_tri_box_children) decides the children of
every case of the stress corpus exactly as the oracle's fp64 restatement of
the reference's testTriBox: random, tangent, on-boundary, one-ulp, dyadic,
degenerate, axis-aligned and non-finite triangles against nodes of levels
0-15 (the same corpus tests/test_sat_filter.py checks with the host build)."""
import os
import subprocess

import numpy as np
import pytest

import svdag_gb300 as sv

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REC = np.dtype([("t", "<f4", (9,)), ("c", "<f8", (3,)), ("k", "<f8"), ("m", "u1")])


def _corpus(tmp_path, n):
    exe = str(tmp_path / "satcheck")
    subprocess.run(["g++", "-O2", "-std=gnu++17", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "svdag-compression_gb300", "csrc"), "-I", os.path.join(ROOT, "oracle"),
                    os.path.join(ROOT, "tests", "sat_filter_check.cpp"),
                    "-L", os.path.join(ROOT, "oracle", "build"), "-loracle",
                    "-Wl,-rpath," + os.path.join(ROOT, "oracle", "build"), "-o", exe], check=True)
    dump = str(tmp_path / "cases.bin")
    r = subprocess.run([exe, str(n), dump], stdout=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stdout  # the host build agrees with the oracle too
    recs = np.fromfile(dump, dtype=REC)
    assert recs.shape[0] == n + 2
    return recs


def test_device_filter_matches_fp64_reference_decisions(tmp_path):
    recs = _corpus(tmp_path, 400000)
    o = sv.Octree()
    masks, fallbacks = o.triBoxChildren(recs["t"], recs["c"], recs["k"])
    bad = np.nonzero(masks != recs["m"])[0]
    assert bad.size == 0, "%d of %d cases differ, first %d: gpu %02x oracle %02x" % (
        bad.size, recs.shape[0], bad[0], masks[bad[0]], recs["m"][bad[0]])
    assert fallbacks > 0  # the corpus does reach the fp64 tier
    # the corpus exercises both outcomes for every child
    for ci in range(8):
        bit = (recs["m"] >> ci) & 1
        assert 0 < bit.sum() < bit.size


def test_device_filter_empty_input():
    o = sv.Octree()
    masks, fb = o.triBoxChildren(np.zeros((0, 9), np.float32), np.zeros((0, 3)), np.zeros(0))
    assert masks.size == 0 and fb == 0
