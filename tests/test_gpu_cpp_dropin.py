"""The reference-style C++ API (include/msvd.hpp) compiles and runs against libofrr_gb300.so."""
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def test_cpp_drop_in(built_lib, tmp_path):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "example_drop_in"
    src = ROOT / "tests" / "cpp" / "example_drop_in.cpp"
    cmd = [nvcc, "-std=c++17", "-O2", "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", str(ROOT / "include"), str(src), "-o", str(exe), "-L", str(built_lib.parent), "-lofrr_gb300",
           f"-Xlinker=-rpath,{built_lib.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), str(tmp_path / "diag")], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0 and "ALL OK" in r.stdout and "MatrixReader ok" in r.stdout, r.stdout + r.stderr
