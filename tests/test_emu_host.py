"""The integer-pipe binary64 operations of the FP64 kernels
(sphugo_gb300/csrc/fp64emu.cuh: products, sums, quotients by a prepared
divisor, square roots, 1 - x, float-pair splits), compiled for the host by
tests/emu_host_check.cpp with the CUDA intrinsics restated in C++, must return
the host's IEEE round-to-nearest results bit for bit. The device self-check
(sph_selftest_fp64emu, a GPU test) compares the device build with the
hardware instructions."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_integer_pipe_operations_match_host_ieee(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "emu_host_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-w", os.path.join(HERE, "emu_host_check.cpp"),
                    "-o", exe], check=True)
    out = subprocess.run([exe, "3000000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert "differing 0" in out.stdout
