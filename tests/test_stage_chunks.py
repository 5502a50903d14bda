"""The stage kernel's k-chunks (fw::stage_chunk): the band edges at the bottom PML slab and
at the free surface's band split the planes so that no chunk straddles them.  Host code
only: compiled with nvcc from tests/stage_chunks_check.cu and run on the CPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_chunks_tile_the_planes(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "chunks")
    src = os.path.join(ROOT, "tests", "stage_chunks_check.cu")
    inc = [f"-I{os.path.join(ROOT, 'fwant_gb300', 'csrc')}", f"-I{os.path.join(ROOT, 'include')}"]
    subprocess.run([nvcc, "-std=c++17", *inc, "-o", exe, src], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad 0" in r.stdout
