"""The C++ drop-in (include/sctlgpu.hpp): type-compatible with the reference's
GenericKernel call sites, and the reference's own unit tests pass through it."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "sctl_gb300")
# the installed reference (oracle/install_ref.sh), or SCTL_REF=<checkout>
REF = os.environ.get("SCTL_REF", os.path.join(ROOT, "baseline", "_ref"))
CXX = shutil.which("g++") or "g++"


def build_shim_test(tmp_path):
    exe = os.path.join(str(tmp_path), "test_gpu_shim")
    cmd = [CXX, "-std=c++17", "-O2", "-I", INC, os.path.join(ROOT, "tests", "cpp", "test_gpu_shim.cpp"), "-L", LIBDIR,
           "-lsctlgpu", "-Wl,-rpath," + LIBDIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_compiles_and_links(tmp_path):
    from sctl_gb300 import capi
    capi.load()  # the library must exist for the link
    assert os.path.exists(build_shim_test(tmp_path))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "include", "sctl")), reason="reference headers not present")
def test_shim_types_match_reference_call_sites():
    src = os.path.join(ROOT, "tests", "cpp", "check_reference_types.cpp")
    r = subprocess.run([CXX, "-std=c++17", "-fsyntax-only", "-I", os.path.join(REF, "include"), "-I", INC, src],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_reference_unit_tests_through_shim(cuda, tmp_path):
    exe = build_shim_test(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "PASS (0 check(s) failed)" in r.stdout, r.stdout + r.stderr


def build_dropin_test(tmp_path):
    exe = os.path.join(str(tmp_path), "test_dropin_bio")
    cmd = [CXX, "-std=c++17", "-O2", "-fopenmp", "-I", os.path.join(REF, "include"), "-I", INC,
           os.path.join(ROOT, "tests", "cpp", "test_dropin_bio.cpp"), "-L", LIBDIR, "-lsctlgpu",
           "-Wl,-rpath," + LIBDIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


@pytest.mark.gpu
@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "include", "sctl.hpp")),
                    reason="reference not installed (oracle/install_ref.sh)")
def test_reference_call_sites_run_the_gpu_kernel(cuda, tmp_path):
    """SCTL's own BoundaryIntegralOp::ComputePotential and ParticleFMM::Eval, compiled from the
    installed reference, with sctlgpu::GpuKernel as their kernel type: equal to the same objects
    with SCTL's kernels (FP64 <= 1e-12, mixed <= 1e-10)."""
    exe = build_dropin_test(tmp_path)
    env = dict(os.environ, OMP_NUM_THREADS=os.environ.get("OMP_NUM_THREADS", "8"))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600, env=env)
    print(r.stdout)
    assert r.returncode == 0 and "PASS (0 check(s) failed)" in r.stdout, r.stdout + r.stderr


def build_treecode_test(tmp_path):
    exe = os.path.join(str(tmp_path), "test_treecode_capi")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    cuda_lib = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64")
    cmd = [CXX, "-std=c++17", "-O2", "-I", INC, "-I", cuda_inc, os.path.join(ROOT, "tests", "cpp", "test_treecode_capi.cpp"),
           "-L", LIBDIR, "-lsctlgpu", "-Wl,-rpath," + LIBDIR, "-L", cuda_lib, "-lcudart", "-Wl,-rpath," + cuda_lib,
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


def test_treecode_capi_compiles_and_links(tmp_path):
    from sctl_gb300 import capi
    capi.load()
    assert os.path.exists(build_treecode_test(tmp_path))


@pytest.mark.gpu
def test_treecode_capi_from_cpp(cuda, tmp_path):
    """The treecode bound from C++ as a ParticleFMM integration would: against sctlgpu_eval."""
    exe = build_treecode_test(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "PASS (0 check(s) failed)" in r.stdout, r.stdout + r.stderr
