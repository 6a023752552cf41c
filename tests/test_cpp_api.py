"""The C++ mirror of mflib's classes (include/mfgpu.hpp) compiles against
the C ABI, links against libmfgpu.so, and on a GPU passes the reference's
known-answer checks (tests/cpp/test_mflib_api.cpp); the ABI's exception
handler maps host exceptions to status codes (tests/cpp/test_abi_exceptions.cpp,
no GPU); the host-side classes pass the reference's C++ tests of them
(tests/cpp/test_host_classes.cpp, no GPU)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_mflib_api.cpp")
LIBDIR = os.path.join(ROOT, "mflib_gb300")
CXX = shutil.which("g++")


def _compile(out, link=True):
    cmd = [CXX, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC]
    if link:
        cmd += ["-o", out, "-L", LIBDIR, "-lmfgpu", "-Wl,-rpath," + LIBDIR]
    else:
        cmd += ["-fsyntax-only"]
    return subprocess.run(cmd, capture_output=True, text=True)


@pytest.mark.skipif(CXX is None, reason="g++ not found")
def test_header_compiles():
    r = _compile(None, link=False)
    assert r.returncode == 0, r.stderr


@pytest.mark.skipif(CXX is None, reason="g++ not found")
def test_links_against_library(tmp_path):
    if not os.path.exists(os.path.join(LIBDIR, "libmfgpu.so")):
        pytest.skip("libmfgpu.so not built")
    r = _compile(str(tmp_path / "t"))
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_cpp_api_on_gpu(tmp_path):
    assert CXX is not None
    exe = str(tmp_path / "test_mflib_api")
    r = _compile(exe)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "ALL PASSED" in run.stdout


@pytest.mark.skipif(CXX is None, reason="g++ not found")
def test_abi_exception_mapping(tmp_path):
    if not os.path.exists(os.path.join(LIBDIR, "libmfgpu.so")):
        pytest.skip("libmfgpu.so not built")
    exe = str(tmp_path / "test_abi_exceptions")
    src = os.path.join(ROOT, "tests", "cpp", "test_abi_exceptions.cpp")
    r = subprocess.run([CXX, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        src, "-o", exe, "-L", LIBDIR, "-lmfgpu", "-Wl,-rpath," + LIBDIR],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "ALL PASSED" in run.stdout


@pytest.mark.skipif(CXX is None, reason="g++ not found")
def test_host_classes(tmp_path):
    """The header's host-side classes against the reference's own C++ tests
    of them (tests/cpp/test_host_classes.cpp); no GPU, no library."""
    exe = str(tmp_path / "test_host_classes")
    r = subprocess.run([CXX, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "test_host_classes.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0 and "ALL PASSED" in run.stdout, run.stdout + run.stderr
