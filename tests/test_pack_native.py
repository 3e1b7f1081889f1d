"""Host checks of the device scene packer (no GPU): quantized BVH8 child boxes
are strictly conservative; the BVH8 leaves are the binary tree's leaves, or,
with leaf merging on, each leaf holds one binary subtree's slots and every slot
lies in exactly one leaf; the sphere lights' fp32 CDF copies are the largest
fp32 values not above their fp64 entries."""
import os
import shutil
import subprocess

import pytest

from conftest import PKG_DIR, ROOT


def test_quantized_nodes_conservative(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "pack_check"
    csrc = os.path.join(PKG_DIR, "csrc")
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I" + csrc, "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "native", "pack_check.cpp"), os.path.join(csrc, "pack.cpp"),
           os.path.join(csrc, "host_scene.cpp"), "-pthread", "-o", str(exe)]
    subprocess.run(cmd, check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.count("ok nodes=") == 7
    assert out.stdout.count("ok merged nodes=") == 7
    assert "ok threaded pack" in out.stdout
    assert "ok light cdf" in out.stdout
    assert out.stdout.count("ok overlapping leaves unmerged") == 7
