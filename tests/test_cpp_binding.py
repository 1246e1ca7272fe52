"""The C++ RayTracer subclass (xdg_gb300/cpp/cuda_ray_tracer.*) compiles with
g++ against include/xdgcu.h and links against libxdgcu.so (CPU); the C++
replay of the reference's MeshMock tests passes through it, and its scalar
methods give the batched results when 8 host threads call them at once
(GPU).

Where the reference source tree is present, the same backend and replay are
also compiled against XDG's own headers (ray_tracing_interface.h,
mesh_manager_interface.h, element_face_accessor.h, with Embree's names
declared by tests/cpp/xdg_shim) and linked with XDG's own
ray_tracing_interface.cpp, mesh_manager_interface.cpp and
element_face_accessor.cpp, the replay running on the reference's MeshMock:
the drop-in builds inside XDG as it is."""
import os
import subprocess

import pytest

from conftest import ROOT

# XDG sources the drop-in links beside it (the RayTracer base class, the
# MeshManager base class, the ElementFaceAccessor factory and what they call)
XDG_SOURCES = ["src/ray_tracing_interface.cpp", "src/mesh_manager_interface.cpp",
               "src/element_face_accessor.cpp", "src/error.cpp", "src/config.cpp",
               "src/geometry/measure.cpp"]


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


def compile_against_xdg(out_dir, ref):
    """The backend, its tool loops and the MeshMock replay against XDG's own
    headers and sources.  RTLibrary gains CUDA when XDG integrates the
    backend (constants.h); until then the replay reports the value CUDA takes
    there, after EMBREE and GPRT."""
    from xdg_gb300 import build
    lib = build.build()
    lib_dir = os.path.dirname(lib)
    exe = os.path.join(out_dir, "test_cuda_ray_tracer_xdg")
    cpp = os.path.join(ROOT, "xdg_gb300", "cpp")
    cmd = (["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-ffp-contract=off", "-pthread",
            "-DXDG_EMBREE3", "-DXDGCU_WITH_XDG_HEADERS",
            "-DXDGCU_RTLIBRARY=static_cast<xdg::RTLibrary>(2)",
            "-I", os.path.join(ROOT, "tests", "cpp", "xdg_shim"),
            "-I", os.path.join(ROOT, "oracle", "ref_shim"),
            "-I", os.path.join(ref, "include"), "-I", os.path.join(ROOT, "include"), "-I", cpp,
            os.path.join(ROOT, "tests", "cpp", "test_cuda_ray_tracer.cpp"),
            os.path.join(cpp, "cuda_ray_tracer.cpp"), os.path.join(cpp, "cuda_tools.cpp")]
           + [os.path.join(ref, s) for s in XDG_SOURCES]
           + ["-L", lib_dir, "-lxdgcu", "-Wl,-rpath," + lib_dir, "-o", exe])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # warnings from the backend's own files, not from XDG's headers
    own = [ln for ln in r.stderr.splitlines() if "warning:" in ln and "/xdg_gb300/" in ln]
    assert not own, "\n".join(own)
    return exe


@pytest.fixture(scope="module")
def xdg_exe(tmp_path_factory, oracle):
    ref = oracle.reference_dir()
    if ref is None:
        pytest.skip("reference source tree not present")
    return compile_against_xdg(str(tmp_path_factory.mktemp("cppxdg")), ref)


def test_cpp_binding_compiles_against_xdg_headers(xdg_exe):
    assert os.access(xdg_exe, os.X_OK)


@pytest.mark.gpu
def test_cpp_mock_suite_on_xdg_meshmock(cuda, xdg_exe):
    r = subprocess.run([xdg_exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 failures" in r.stdout
