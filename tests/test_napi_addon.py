"""The Node-API addon (webgpu-fluid-simulation_gb300/napi/pbf_addon.cc) built
against the Node-API declarations of tests/napi_host/node_api.h and loaded by
tests/napi_host/napi_host.cc, a host that stands in for Node (Node is not
installed here).  Without a GPU: registration, TypeErrors for wrong
arguments, library errors as thrown Errors with the pbf_status name.  On a
GPU: the Cube Drop flow, pause, asynchronous reads (the typed array pinned
until synchronize), mesh seeding equal to the C ABI, and the renderer's maps
bit-identical to the C ABI's."""
import os
import subprocess

import pytest

from pbf_gb300 import _lib as L

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADDON = os.path.join(REPO, "webgpu-fluid-simulation_gb300", "napi", "pbf_addon.cc")
HOST_DIR = os.path.join(REPO, "tests", "napi_host")


def _build(tmp_path):
    lib = L.load()
    libdir = os.path.dirname(lib._name)
    so = str(tmp_path / "pbf_gb300.node")
    exe = str(tmp_path / "napi_host")
    common = ["-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", HOST_DIR, "-I", os.path.join(REPO, "include")]
    r = subprocess.run(["g++", *common, "-shared", "-fPIC", "-fvisibility=hidden", "-DNODE_GYP_MODULE_NAME=pbf_gb300",
                        ADDON, "-o", so, "-L", libdir, "-lpbf_gb300", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run(["g++", *common, "-rdynamic", os.path.join(HOST_DIR, "napi_host.cc"), "-o", exe, "-L", libdir,
                        "-lpbf_gb300", "-Wl,-rpath," + libdir, "-ldl"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return so, exe


def test_addon_exports_and_argument_errors(tmp_path):
    so, exe = _build(tmp_path)
    r = subprocess.run([exe, so, "cpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failed checks" in r.stdout


@pytest.mark.gpu
def test_addon_cube_drop_mesh_and_renderer(tmp_path):
    so, exe = _build(tmp_path)
    r = subprocess.run([exe, so, "gpu"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failed checks" in r.stdout
