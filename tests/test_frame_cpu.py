"""The lateral-frame numbering the nest kernels launch over (frame_count /
frame_column in vibe_internal.cuh), compiled for the host and checked
against the direct definition of the frame for every grid up to 40 x 40 and
zone widths up to 22."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_frame_numbering_covers_the_frame_once(tmp_path):
    cuda_inc = "/usr/local/cuda/include"
    if not shutil.which("g++") or not os.path.isdir(cuda_inc):
        pytest.skip("g++ or the CUDA headers absent")
    exe = str(tmp_path / "frame_check")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I" + cuda_inc,
                        "-I" + os.path.join(ROOT, "vibe-model_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "cpp", "frame_check.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == "bad 0", out.stdout
