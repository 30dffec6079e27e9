"""GPU ray casting of encoded SSVDAGs (svdag_ssvdag_raycast) against the
restated shader traversal (oracle): every field of every pixel's hit record
bit for bit -- distance, level, iteration count, node, cell, normal -- for
cameras outside and inside the box, with the level of detail on and off, a
reduced draw level, an iteration limit and a short t range; the device
buffer path equals the host one; a truncated file is an error."""
import numpy as np
import pytest

import oracle_py
import svdag_gb300 as sv
from _raycheck import encoded_scene

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert np.array_equal(a["t"].view(np.uint32), b["t"].view(np.uint32))
    for k in ("level", "iterations", "node", "voxel", "normal"):
        assert np.array_equal(a[k], b[k]), k


VIEWS = [
    dict(eye=(1.6, 1.3, 1.9), target=(0.5, 0.5, 0.5)),
    dict(eye=(0.45, 0.52, 0.55), target=(0.9, 0.2, 0.4)),
    dict(eye=(0.2, 0.6, 0.3), target=(0.5, 0.3, 0.5), pixel_tolerance=1.0),
    dict(eye=(1.3, 0.9, 1.7), target=(0.5, 0.3, 0.5), pixel_tolerance=4.0),
    dict(eye=(-0.4, 0.5, 0.5), target=(0.5, 0.5, 0.5), up=(0.0, 0.0, 1.0), fovy_deg=90.0),
]


@pytest.mark.parametrize("name,L,builder", [("ico3_L6", 6, "oracle"), ("ico5_L7", 7, "gpu"),
                                             ("terrain65_L8", 8, "gpu")])
def test_raycast_matches_oracle(name, L, builder, tmp_path):
    _, f = encoded_scene(name, L, tmp_path, builder)
    s = sv.Ssvdag(f)
    for v in VIEWS:
        kw = dict(v)
        kw.setdefault("pixel_tolerance", 1e-6)
        cam = sv.camera(kw.pop("eye"), kw.pop("target"), 160, 120, L, **kw)
        got = s.raycast(cam)
        want, rc = oracle_py.ssvdag_raycast(f, cam)
        assert rc == 0
        _same(got, want)
        assert (got["t"] > 0).any()
    cam = sv.camera((0.2, 0.6, 0.3), (0.5, 0.3, 0.5), 96, 64, L, pixel_tolerance=1e-6)
    for change in (dict(draw_level=4), dict(max_iters=20), dict(t_max=0.05)):
        c = dict(cam, **change)
        _same(s.raycast(c), oracle_py.ssvdag_raycast(f, c)[0])
    s.close()


def test_raycast_device_buffer(tmp_path):
    import torch

    _, f = encoded_scene("terrain65_L8", 8, tmp_path, "gpu")
    s = sv.Ssvdag(f)
    cam = sv.camera((1.3, 0.9, 1.7), (0.5, 0.3, 0.5), 200, 150, 8)
    buf = torch.zeros(200 * 150 * 32, dtype=torch.uint8, device="cuda")
    s.raycast_device(cam, buf.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = buf.cpu().numpy().view(sv.HIT)
    _same(got, s.raycast(cam))
    s.close()


def test_raycast_truncated_file_is_an_error(tmp_path):
    _, f = encoded_scene("ico3_L6", 6, tmp_path)
    g = dict(f)
    g["leaves"] = f["leaves"][: (f["leaves"].size // 16) * 8].copy()
    s = sv.Ssvdag(g)
    cam = sv.camera((0.45, 0.52, 0.55), (0.9, 0.2, 0.4), 32, 24, 6, pixel_tolerance=1e-6)
    with pytest.raises(sv.SvdagError):
        s.raycast(cam)
    s.close()
