"""Race and memory checks for the threaded host set-up. Its sources are built
into a small driver (tests/setup_sanitizer_driver.cpp) that runs box mesh +
RCM, P1/P2 dofmaps, dof coordinates, exterior and interior facets, sparsity,
colouring, the dual graph and RCM entry points:
- with ThreadSanitizer, on a box large enough for every thread team, at two
  thread counts;
- with AddressSanitizer + UndefinedBehaviorSanitizer and libstdc++'s
  assertions (the reference's Developer/debug checks), on tiny boxes and on
  the large one, serial and threaded.
Any report fails the test."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "dolfinx_gb300", "csrc")

_FLAGS = {
    "thread": ["-fsanitize=thread"],
    "address": ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
                "-D_GLIBCXX_ASSERTIONS"],
}


def _build(tmp_path_factory, kind):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp(kind) / "setup_driver")
    cmd = [cxx, "-std=c++20", "-O1", "-g", *_FLAGS[kind], "-I", os.path.join(ROOT, "include"),
           "-I", CSRC, os.path.join(ROOT, "tests", "setup_sanitizer_driver.cpp"),
           os.path.join(CSRC, "setup.cpp"), os.path.join(CSRC, "timing.cpp"), "-o", exe,
           "-lpthread"]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    if p.returncode != 0:
        pytest.skip(f"{kind} sanitizer build unavailable: " + p.stderr[-300:])
    return exe


@pytest.fixture(scope="module")
def tsan(tmp_path_factory):
    return _build(tmp_path_factory, "thread")


@pytest.fixture(scope="module")
def asan(tmp_path_factory):
    return _build(tmp_path_factory, "address")


def _run(exe, n, threads, env_extra):
    env = dict(os.environ, DFX_NUM_THREADS=str(threads), **env_extra)
    p = subprocess.run([exe, str(n)], capture_output=True, text=True, timeout=600, env=env)
    assert "Sanitizer" not in p.stderr and "runtime error" not in p.stderr, p.stderr[-4000:]
    assert p.returncode == 0, p.stderr[-2000:]
    return p.stdout


@pytest.mark.parametrize("threads", [3, 5])
def test_host_setup_has_no_data_races(tsan, threads):
    out = _run(tsan, 24, threads, {"TSAN_OPTIONS": "halt_on_error=1 exitcode=66"})
    assert out.startswith("nodes 117649 facets 6912 ")


@pytest.mark.parametrize("n,threads", [(1, 5), (2, 5), (24, 1), (24, 5)])
def test_host_setup_is_memory_clean(asan, n, threads):
    out = _run(asan, n, threads, {"ASAN_OPTIONS": "detect_leaks=1:halt_on_error=1"})
    nodes = (2 * n + 1) ** 3
    assert out.startswith(f"nodes {nodes} facets {12 * n * n} ")


@pytest.mark.parametrize("src", ["dolfinx_gb300/csrc/setup.cpp", "dolfinx_gb300/csrc/timing.cpp",
                                 "dolfinx_gb300/csrc/tune.cpp", "oracle/dfx_oracle.cpp"])
def test_host_sources_build_with_developer_flags(src):
    """The reference's Developer build flags (-Wall -Wextra -Werror -pedantic,
    cpp/cmake/modules/DolfinxDeveloperCompilerFlags.cmake) plus libstdc++
    assertions: the host C++ compiles without a warning."""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = subprocess.run([cxx, "-std=c++20", "-O2", "-Wall", "-Wextra", "-Werror", "-pedantic",
                        "-D_GLIBCXX_ASSERTIONS", "-fsyntax-only", "-I",
                        os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"), "-I",
                        CSRC, os.path.join(ROOT, src)], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-3000:]
