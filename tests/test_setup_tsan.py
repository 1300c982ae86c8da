"""Race detection for the threaded host set-up: its sources are built with
ThreadSanitizer into a small driver (tests/setup_tsan_driver.cpp) that runs
the box mesh + RCM, dofmap, dof coordinates, exterior facets and sparsity on
a box large enough for every thread team, at two thread counts. Any race
report fails the test."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "dolfinx_gb300", "csrc")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("tsan") / "setup_tsan")
    cmd = [cxx, "-std=c++20", "-O1", "-g", "-fsanitize=thread", "-I",
           os.path.join(ROOT, "include"), "-I", CSRC,
           os.path.join(ROOT, "tests", "setup_tsan_driver.cpp"),
           os.path.join(CSRC, "setup.cpp"), os.path.join(CSRC, "timing.cpp"),
           "-o", exe, "-lpthread"]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    if p.returncode != 0:
        pytest.skip("ThreadSanitizer build unavailable: " + p.stderr[-300:])
    return exe


@pytest.mark.parametrize("threads", [3, 5])
def test_host_setup_has_no_data_races(driver, threads):
    env = dict(os.environ, DFX_NUM_THREADS=str(threads),
               TSAN_OPTIONS="halt_on_error=1 exitcode=66")
    p = subprocess.run([driver, "24"], capture_output=True, text=True, timeout=600, env=env)
    assert "ThreadSanitizer" not in p.stderr, p.stderr[-4000:]
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.startswith("nodes 117649 facets 6912 ")
