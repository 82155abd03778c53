"""The C ABI from plain C: examples/cube_drop.c (the reference controller's
Cube Drop flow) compiles as C11 against include/pbf_gb300.h and links
against the library without a GPU; on a GPU it runs to completion."""
import os
import subprocess

import pytest

from pbf_gb300 import _lib as L

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "webgpu-fluid-simulation_gb300", "examples", "cube_drop.c")


def _build(tmp_path):
    lib = L.load()
    libdir = os.path.dirname(lib._name)
    exe = str(tmp_path / "cube_drop")
    cmd = ["gcc", "-std=c11", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(REPO, "include"), SRC, "-o",
           exe, "-L", libdir, "-lpbf_gb300", "-Wl,-rpath," + libdir, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_host_compiles_and_links(tmp_path):
    assert os.path.exists(_build(tmp_path))


@pytest.mark.gpu
def test_c_host_runs_cube_drop(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe, "30"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "68921 particles" in r.stdout and "nonfinite 0" in r.stdout
