"""The C-ABI library loads and exports every entry point include/svdag_gpu.h
declares (no compute without a GPU), and the Python mirrors of its structs
have the header's layout."""
import ctypes
import os
import re
import subprocess

import svdag_gb300 as sv

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "svdag_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(svdag_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = header_functions()
    for n in ("svdag_create", "svdag_voxelize", "svdag_reduce_dag", "svdag_reduce_sdag", "svdag_cross_level_merge",
              "svdag_download_level"):
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(sv.gpu_library_path())
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    assert sorted(sv.GPU_SYMBOLS) == header_functions()


def test_status_strings_and_null_handles():
    lib = sv.load_gpu()
    assert lib.svdag_status_string(0) == b"ok"
    assert lib.svdag_status_string(4) == b"out of device memory"
    assert lib.svdag_destroy(None) == 1
    assert lib.svdag_reduce_dag(None) == 1
    assert lib.svdag_reduce_dag_noalloc(None) == 1
    assert lib.svdag_get_stats(None, None) == 1


def test_null_arguments_are_rejected_before_any_device_work():
    lib = sv.load_gpu()
    h = ctypes.c_void_p()
    assert lib.svdag_clone_on(None, None, ctypes.byref(h)) == 1
    assert lib.svdag_flood_fill(None, None, None) == 1
    assert lib.svdag_download_outside_masks(None, 0, None) == 1
    assert lib.svdag_encode(None, 0, None, 0, None) == 1
    assert lib.svdag_ssvdag_free(None) == 1
    assert lib.svdag_ssvdag_raycast(None, None, None, None, 0) == 1
    bb = (ctypes.c_float * 6)(0, 0, 0, 1, 1, 1)
    # arrays missing while their sizes say otherwise
    assert lib.svdag_ssvdag_upload(None, 4, None, 8, None, 1, 5, bb, 1.0, ctypes.byref(h)) == 1
    assert lib.svdag_ssvdag_upload(None, 0, None, 0, None, 0, 5, bb, 1.0, None) == 1
    assert lib.svdag_ssvdag_traverse(None, 0, None, 0, None, 0, 5, bb, 1.0, None, 0, None) == 1
    assert lib.svdag_refcount_order(None, None, 16, None) == 1


def test_create_fails_loudly_without_device():
    import torch

    if torch.cuda.is_available():
        return
    h = ctypes.c_void_p()
    assert sv.load_gpu().svdag_create(ctypes.byref(h), 0, None) == 7  # SVDAG_ERR_NO_DEVICE
    assert not h.value


# (header struct, its Python mirror) -- a mismatch would make the library
# read or write past the Python object
STRUCTS = [("svdag_stats", sv._Stats), ("svdag_lossy_params", sv.LossyParams),
           ("svdag_lossy_stats", sv._LossyStats), ("svdag_batch_tuning", sv.BatchTuning),
           ("svdag_batch_stats", sv._BatchStats), ("svdag_camera", sv._Camera)]


def c_layouts(tmp_path):
    """sizeof and every field's offsetof, as a C compiler lays the header's
    structs out."""
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "svdag_gpu.h"', "int main(void) {"]
    for name, py in STRUCTS:
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (name, name))
        for f, _ in py._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (name, f, name, f))
    lines.append('  printf("svdag_ray_hit size %zu\\n", sizeof(svdag_ray_hit));')
    for f in sv.HIT.names:
        lines.append('  printf("svdag_ray_hit %s %%zu\\n", offsetof(svdag_ray_hit, %s));' % (f, f))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        s, f, v = line.split()
        out[(s, f)] = int(v)
    return out


def test_struct_layouts_match_the_header(tmp_path):
    c = c_layouts(tmp_path)
    for name, py in STRUCTS:
        assert c[(name, "size")] == ctypes.sizeof(py), name
        for f, _ in py._fields_:
            assert c[(name, f)] == getattr(py, f).offset, (name, f)
    assert c[("svdag_ray_hit", "size")] == sv.HIT.itemsize
    for f in sv.HIT.names:
        assert c[("svdag_ray_hit", f)] == sv.HIT.fields[f][1], f
