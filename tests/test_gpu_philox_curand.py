"""The device Philox4x32-10 against cuRAND's Philox4_32_10, run on the
GPU: 2^16 counter blocks over four keys (the engine's walker/step/block
counter layout, the PPR termination block included) must match word for
word (the CPU restatement is pinned to the Random123 known-answer vectors in
test_oracle_golden.py)."""
import os
import shutil
import subprocess

import pytest

from tests.gpu_util import need_gpu

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_device_philox_equals_curand(tmp_path):
    need_gpu()
    from thunderrw_gb300 import build_native as B
    nvcc = B.nvcc()
    if not nvcc or not shutil.which(nvcc):
        pytest.skip("no nvcc")
    exe = str(tmp_path / "philox_curand")
    subprocess.run([nvcc, *B.ARCH, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "thunderrw_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "philox_curand.cu"), "-o", exe], check=True)
    r = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=120)
    assert r.returncode == 0, r.stdout
    assert "0 of 65536 blocks differ" in r.stdout
