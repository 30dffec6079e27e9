"""Build recipe for the SVDAG GB300 libraries (in-tree, no cmake).

Products (git-ignored, rebuilt on every machine):
  svdag-compression_gb300/lib/libsvdag_gpu.so   CUDA kernels + C ABI (sm_103a)
  svdag-compression_gb300/lib/libsvdag_host.so  host helpers (scene synthesis, OBJ)
  oracle/build/liboracle.so                     restated CPU oracle (test checker)
  oracle/_ref/{svbuilder,ref_dump}              reference build, only where the
                                                reference sources are present
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB = os.path.join(PKG, "lib")
OBJ = os.path.join(PKG, "_build")
INC = os.path.join(ROOT, "include")
ORACLE = os.path.join(ROOT, "oracle")
# The reference checkout: $SVDAG_REFERENCE, else a "reference" directory
# beside this repository.  Only the checker's build (build_reference) reads it.
REFERENCE = os.environ.get("SVDAG_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))

NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# extra nvcc flags (e.g. tuning macros), whitespace separated
EXTRA_NVCC = os.environ.get("SVDAG_NVCC_FLAGS", "").split()
CU_SOURCES = ["api.cu", "voxelize.cu", "reduce.cu", "csvdag.cu", "chunked.cu", "batch.cu", "lossy.cu", "mlp.cu", "encode.cu", "traverse.cu", "raycast.cu", "floodfill.cu", "noalloc.cu", "refsort.cu", "lossy_ref.cu"]
HOST_SOURCES = ["synth.cpp", "encoders.cpp", "scene.cpp", "geom_octree.cpp"]


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _newer(target, deps):
    """True when `target` exists and is newer than every dependency and than
    this recipe (a change of sources or flags here rebuilds)."""
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in list(deps) + [os.path.abspath(__file__)] if os.path.exists(d))


def _cu_object(src):
    s = os.path.join(PKG, "csrc", src)
    o = os.path.join(OBJ, src.replace(".cu", ".o"))
    deps = [s] + [os.path.join(PKG, "csrc", h) for h in os.listdir(os.path.join(PKG, "csrc")) if h.endswith(".cuh")]
    deps.append(os.path.join(INC, "svdag_gpu.h"))
    if not _newer(o, deps):
        _run([NVCC] + ARCH + EXTRA_NVCC + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INC,
                              "-I", os.path.join(PKG, "csrc"), "-c", s, "-o", o])
    return o


def build_gpu(jobs=8):
    os.makedirs(LIB, exist_ok=True)
    os.makedirs(OBJ, exist_ok=True)
    with ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(_cu_object, CU_SOURCES))
    out = os.path.join(LIB, "libsvdag_gpu.so")
    if not _newer(out, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", out] + objs)
    return out


def build_host():
    os.makedirs(LIB, exist_ok=True)
    srcs = [os.path.join(PKG, "host", s) for s in HOST_SOURCES]
    hdrs = [os.path.join(PKG, "host", h) for h in os.listdir(os.path.join(PKG, "host")) if h.endswith((".h", ".hpp"))]
    out = os.path.join(LIB, "libsvdag_host.so")
    if not _newer(out, srcs + hdrs + [os.path.join(LIB, "libsvdag_gpu.so")]):
        _run([CXX, "-O2", "-std=gnu++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-I", INC,
              "-I", os.path.join(PKG, "host")] + srcs + ["-L", LIB, "-lsvdag_gpu", "-Wl,-rpath,$ORIGIN", "-o", out])
    return out


def build_cli(gpu_lib):
    """svbuilder executable (the reference CLI over the GPU path)."""
    os.makedirs(os.path.join(PKG, "bin"), exist_ok=True)
    srcs = [os.path.join(PKG, "host", s) for s in HOST_SOURCES + ["svbuilder.cpp"]]
    hdrs = [os.path.join(PKG, "host", h) for h in os.listdir(os.path.join(PKG, "host")) if h.endswith((".h", ".hpp"))]
    out = os.path.join(PKG, "bin", "svbuilder")
    if not _newer(out, srcs + hdrs + [gpu_lib]):
        _run([CXX, "-O2", "-std=gnu++17", "-pthread", "-ffp-contract=off", "-I", INC, "-I", os.path.join(PKG, "host")] + srcs +
             ["-L", LIB, "-lsvdag_gpu", "-Wl,-rpath,$ORIGIN/../lib", "-o", out])
    return out


def build_oracle():
    d = os.path.join(ORACLE, "build")
    os.makedirs(d, exist_ok=True)
    # the seeded scene generators are compiled in as well, so that the CPU
    # legs (reference arm, CPU baseline) synthesise their inputs without
    # loading the product's libraries
    srcs = [os.path.join(ORACLE, "svdag_oracle.cpp"), os.path.join(ORACLE, "ssvdag_raycast.cpp"),
            os.path.join(PKG, "host", "synth.cpp")]
    out = os.path.join(d, "liboracle.so")
    if not _newer(out, srcs + [os.path.join(ORACLE, "svdag_oracle.h"), os.path.join(PKG, "host", "svdag_host.h")]):
        _run([CXX, "-O3", "-std=gnu++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
              "-I", os.path.join(PKG, "host")] + srcs + ["-o", out])
    return out


def build_reference():
    """Compiles the reference's own sources against the SpaceLand shim, only
    where the reference tree exists (never on machines without it)."""
    if not os.path.isdir(os.path.join(REFERENCE, "src", "symvox")) or shutil.which("make") is None:
        return None
    _run(["make", "-s", "-C", ORACLE, "REF=" + REFERENCE, "-j8"])
    return os.path.join(ORACLE, "_ref", "ref_dump")


def build_all(with_reference=True):
    with ThreadPoolExecutor(4) as ex:
        fg = ex.submit(build_gpu)
        fg.result()
        fh = ex.submit(build_host)
        fo = ex.submit(build_oracle)
        fr = ex.submit(build_reference) if with_reference else None
        res = {"gpu": fg.result(), "host": fh.result(), "oracle": fo.result()}
        res["cli"] = build_cli(res["gpu"])
        if fr is not None:
            res["reference"] = fr.result()
    return res


if __name__ == "__main__":
    print(build_all())
    sys.exit(0)
