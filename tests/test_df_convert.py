"""df_to_double (the integer route from a double-float pair to a correctly rounded
double, used by the mixed-precision kernel matrix) against the FP64 sum on the host."""
import os
import shutil
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CXX = shutil.which("g++") or "g++"


def test_df_to_double_matches_fp64_sum():
    src = os.path.join(ROOT, "tests", "cpp", "test_df_convert.cpp")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "test_df_convert")
        r = subprocess.run([CXX, "-std=c++17", "-O2", "-ffp-contract=off", src, "-o", exe], capture_output=True,
                           text=True)
        assert r.returncode == 0, r.stderr
        r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert " 0 mismatches" in r.stdout
