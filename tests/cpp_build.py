"""Compile tests/cpp/api_example.cpp against include/vibe_gb300.hpp and the
built library (g++, C++17); shared by the CPU and GPU tests."""
import os
import shutil
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "vibe-model_gb300")
SRC = os.path.join(ROOT, "tests", "cpp", "api_example.cpp")


def build(out_dir):
    exe = os.path.join(out_dir, "api_example")
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", PKG, "-lvibe_gb300", "-Wl,-rpath," + PKG]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return exe
