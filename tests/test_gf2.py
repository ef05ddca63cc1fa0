"""The carry-less GF(2) product behind the CRC shifts (csrc/r2p_common.h
clmul32, csrc/k_deflate.cuh gf2_mulmod_t), checked on the host against the
bit-by-bit product."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_table_assisted_product_equals_bitwise(tmp_path):
    exe = tmp_path / "gf2_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "raw2png-conversionthrugpu_gb300", "csrc"),
                    "-o", str(exe), os.path.join(ROOT, "tests", "cpp", "gf2_check.cpp")], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    assert out.strip() == "ok", out
