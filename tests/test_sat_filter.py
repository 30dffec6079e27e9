"""The certified fp32 triangle/box filter of the voxelizer (csrc/sat.cuh,
compiled as host code with -ffp-contract=off) makes the same decision as the
oracle's fp64 restatement of the reference test on random, tangent,
on-boundary, one-ulp, dyadic, degenerate and non-finite cases."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_filter_matches_fp64_reference_decisions(tmp_path):
    exe = str(tmp_path / "satcheck")
    subprocess.run(["g++", "-O2", "-std=gnu++17", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "svdag-compression_gb300", "csrc"), "-I", os.path.join(ROOT, "oracle"),
                    os.path.join(ROOT, "tests", "sat_filter_check.cpp"),
                    "-L", os.path.join(ROOT, "oracle", "build"), "-loracle",
                    "-Wl,-rpath," + os.path.join(ROOT, "oracle", "build"), "-o", exe], check=True)
    r = subprocess.run([exe, "400000"], stdout=subprocess.PIPE, text=True)
    line = r.stdout.strip().splitlines()[-1]
    stats = dict(kv.split("=") for kv in line.split())
    assert r.returncode == 0, r.stdout
    assert int(stats["mismatches"]) == 0
    assert int(stats["cases"]) == 8 * 400000 + 16
