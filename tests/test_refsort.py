"""GPU reference-count order (svdag_refcount_order) against libstdc++'s
std::sort as EncodedSSVDAG::encode calls it (src/symvox/encoded_ssvdag.cpp:
266-276), through the oracle: seeded count arrays of the shapes real levels
have (mostly 1-2 pointers, a heavy tail), the partition edge sizes, and
McIlroy's adversary, which drives the introsort into its heap-sort
fallback."""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "svdag-compression_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle_py as ora  # noqa: E402
import svdag_gb300 as sv  # noqa: E402

pytestmark = pytest.mark.gpu


def _counts(kind, n, rng):
    if kind == "ones":
        return np.ones(n, np.uint32)
    if kind == "few":
        return rng.integers(1, 4, n).astype(np.uint32)
    if kind == "tail":
        c = np.ones(n, np.uint32)
        m = rng.random(n) < 0.1
        c[m] = rng.integers(2, 50000, int(m.sum()))
        return c
    if kind == "geometric":
        return rng.geometric(0.5, n).astype(np.uint32)
    if kind == "distinct":
        return rng.permutation(n).astype(np.uint32)
    if kind == "ascending":
        return np.arange(n, dtype=np.uint32)
    if kind == "descending":
        return np.arange(n, 0, -1).astype(np.uint32)
    raise ValueError(kind)


@pytest.mark.parametrize("n", [0, 1, 2, 16, 17, 100, 511, 512, 513, 1024, 1025, 1026, 4097, 65536, 100003])
@pytest.mark.parametrize("kind", ["ones", "few", "tail", "geometric", "distinct", "ascending", "descending"])
def test_refcount_order_small(n, kind):
    rng = np.random.default_rng(n * 31 + len(kind))
    c = _counts(kind, n, rng)
    np.testing.assert_array_equal(sv.refcount_order(c), ora.refcount_order(c))


@pytest.mark.parametrize("n,kind", [(1 << 20, "tail"), (3_000_017, "few"), (2_000_003, "geometric"),
                                    (1 << 21, "ones")])
def test_refcount_order_large(n, kind):
    rng = np.random.default_rng(n)
    c = _counts(kind, n, rng)
    np.testing.assert_array_equal(sv.refcount_order(c), ora.refcount_order(c))


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
@pytest.mark.parametrize("n", [600, 5000, 100000])
def test_refcount_order_adversary(n):
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "h")
        subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "svdag-compression_gb300", "csrc"),
                        os.path.join(HERE, "refsort_harness.cpp"), "-o", exe], check=True)
        path = os.path.join(d, "c.bin")
        subprocess.run([exe, "adversary", str(n), path], check=True, timeout=120)
        c = np.fromfile(path, np.uint32)
    assert c.size == n
    np.testing.assert_array_equal(sv.refcount_order(c), ora.refcount_order(c))
