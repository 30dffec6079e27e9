"""The reference-count order restatement (csrc/refsort.cuh) against
libstdc++'s std::sort, as EncodedSSVDAG::encode calls it
(src/symvox/encoded_ssvdag.cpp:266-276), on the CPU: the sequential
introsort, the GPU's round structure with the parallel partition form, and
the heap-sort fallback (also driven by McIlroy's adversary)."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "svdag-compression_gb300", "csrc")


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_refsort_matches_std_sort():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "refsort_harness")
        subprocess.run(["g++", "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "refsort_harness.cpp"), "-o", exe],
                       check=True)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert r.stdout.strip().startswith("ok "), r.stdout
