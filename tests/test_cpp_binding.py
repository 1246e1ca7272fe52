"""The C++ RayTracer subclass (xdg_gb300/cpp/cuda_ray_tracer.*) compiles with
g++ against include/xdgcu.h and links against libxdgcu.so (CPU); the C++
replay of the reference's MeshMock tests passes through it, and its scalar
methods give the batched results when 8 host threads call them at once
(GPU)."""
import os
import subprocess

import pytest

from conftest import ROOT


def compile_cpp_test(out_dir):
    from xdg_gb300 import build
    lib = build.build()
    lib_dir = os.path.dirname(lib)
    exe = os.path.join(out_dir, "test_cuda_ray_tracer")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-ffp-contract=off", "-pthread",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "xdg_gb300", "cpp"),
           os.path.join(ROOT, "tests", "cpp", "test_cuda_ray_tracer.cpp"),
           os.path.join(ROOT, "xdg_gb300", "cpp", "cuda_ray_tracer.cpp"),
           "-L", lib_dir, "-lxdgcu", "-Wl,-rpath," + lib_dir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.fixture(scope="module")
def cpp_exe(tmp_path_factory):
    return compile_cpp_test(str(tmp_path_factory.mktemp("cpp")))


def test_cpp_binding_compiles_and_links(cpp_exe):
    assert os.access(cpp_exe, os.X_OK)


@pytest.mark.gpu
def test_cpp_mock_suite(cuda, cpp_exe):
    r = subprocess.run([cpp_exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 failures" in r.stdout
