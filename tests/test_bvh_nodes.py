"""The scene builder's quantised BVH nodes, checked on the host by tests/bvh_nodes_check.cpp (compiled
here against the library's scene builder): the 48-byte nodes decode to the float nodes' children,
every triangle sits in exactly one leaf, and every decoded box contains its float box with the
margin the walk's folded decode needs."""
import os
import shutil
import subprocess

import pytest

from pachydermacoustic_universal_gb300 import build

HERE = os.path.dirname(os.path.abspath(__file__))


def test_quantised_nodes_decode_to_the_float_tree(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    build.build()
    obj = os.path.join(build.OUT_DIR, "scene.cpp.o")
    exe = str(tmp_path / "bvh_nodes_check")
    inc = build._cuda_include(build._nvcc())
    r = subprocess.run([gxx, "-O2", "-std=c++17", "-I" + inc, os.path.join(HERE, "bvh_nodes_check.cpp"), obj, "-o", exe,
                        "-lpthread"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
