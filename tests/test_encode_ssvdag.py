"""GPU SSVDAG encoding (svdag_encode_ssvdag): the .ssvdag / .esvdag arrays equal
the host encoder's (byte-exact with the reference's files) for SDAG and DAG
states, including scenes with 32-bit pointers; a cross-level merged octree
is refused; an imported DAG whose child pointers do not match its masks or
the level below is rejected at import."""
import numpy as np
import pytest

import oracle_py
import svdag_gb300 as sv
from _scenes import SCENES, golden

pytestmark = pytest.mark.gpu
G = golden()


@pytest.mark.parametrize("name", ["ico3_L6", "ico5_L7", "terrain65_L8", "terrain129_L9"])
@pytest.mark.parametrize("state", ["dag", "sdag"])
def test_gpu_ssvdag_equals_host_encoder(name, state, tmp_path):
    L = G[name]["levels"] if name in G else 9
    o = sv.Octree()
    o.upload_triangles(SCENES[name]())
    o.buildSVO(L)
    o.toDAG()
    o.initChildLevels()
    if state == "sdag":
        o.toSDAG()
    host = str(tmp_path / "host.ssvdag")
    sv.write_encoded(host, "ssvdag", o.pool(), o.stats()["n_nodes"], 3 if state == "sdag" else 2)
    gpu = str(tmp_path / "gpu.ssvdag")
    o.save_ssvdag(gpu)
    assert open(gpu, "rb").read() == open(host, "rb").read()
    f = oracle_py.read_ssvdag(gpu)
    assert f["level_offsets"].size == L - 2


def test_gpu_ssvdag_refuses_cross_level_merged():
    o = sv.Octree()
    o.upload_triangles(SCENES["ico3_L6"]())
    o.buildSVO(6)
    o.toDAG()
    o.initChildLevels()
    o.mergeAcrossAllLevels()
    with pytest.raises(sv.SvdagError):
        o.encode_ssvdag()


def test_import_rejects_inconsistent_children():
    import ctypes

    lib = sv.load_gpu()
    o = sv.Octree()
    bb = (ctypes.c_float * 6)(0, 0, 0, 1, 1, 1)
    assert lib.svdag_import_begin(o._h, 3, bb, 1.0, 0) == 0
    hdr0 = np.array([0x01], np.uint32)
    ch0 = np.full(8, 0xFFFFFFFE, np.uint32)
    ch0[0] = 5  # level 1 will hold one node
    assert lib.svdag_import_level(o._h, 0, 1, hdr0.ctypes.data, ch0.ctypes.data) == 0
    hdr1 = np.array([0x01], np.uint32)
    ch1 = np.full(8, 0xFFFFFFFE, np.uint32)
    ch1[0] = 0
    assert lib.svdag_import_level(o._h, 1, 1, hdr1.ctypes.data, ch1.ctypes.data) == 1
    # a set bit without a pointer
    assert lib.svdag_import_begin(o._h, 2, bb, 1.0, 0) == 0
    ch0[0] = 0xFFFFFFFE
    assert lib.svdag_import_level(o._h, 1, 1, hdr1.ctypes.data, None) == 0
    assert lib.svdag_import_level(o._h, 0, 1, hdr0.ctypes.data, ch0.ctypes.data) == 1


def test_gpu_ssvdag_large_levels_equal_host_encoder(tmp_path):
    """A 1025^2 terrain at depth 11: levels of 10^5 nodes, so the GPU
    ref-count order runs its parallel partition rounds on real pointer
    counts (mostly 1-2, a long tail) before the bytes are compared."""
    o = sv.Octree()
    o.upload_triangles(sv.terrain(1025, 8, 0.3, 5))
    o.buildSVO(11)
    o.toDAG()
    o.initChildLevels()
    o.toSDAG()
    assert max(o.level_count(l) for l in range(11)) > 100000
    host = str(tmp_path / "host.ssvdag")
    sv.write_encoded(host, "ssvdag", o.pool(), o.stats()["n_nodes"], 3)
    gpu = str(tmp_path / "gpu.ssvdag")
    o.save_ssvdag(gpu)
    assert open(gpu, "rb").read() == open(host, "rb").read()
