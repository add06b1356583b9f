"""The FP32 step's work planner (host/fp32_host.cpp: tile_pieces, split_ngroup), on the CPU.

Each heat-flux partial row is written by one piece of a tile's velocity chunks and the heat flux
sums the rows, so the pieces must cover every chunk of every tile exactly once.  The check is a
small C++ program linked against the library (tests/tile_pieces_check.cpp)."""
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "meso-lts_gb300"))


def test_tile_pieces_partition_chunks(tmp_path):
    import build
    lib = build.build_library()
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = str(tmp_path / "tile_pieces_check")
    cmd = ["g++", "-O1", "-std=c++17", "-I" + os.path.join(ROOT, "meso-lts_gb300", "csrc"),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(cuda, "include"),
           os.path.join(HERE, "tile_pieces_check.cpp"), "-o", exe, lib,
           "-Wl,-rpath," + os.path.dirname(lib), "-L" + os.path.join(cuda, "lib64"),
           "-Wl,-rpath," + os.path.join(cuda, "lib64"), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail("compile failed:\n" + r.stderr)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
