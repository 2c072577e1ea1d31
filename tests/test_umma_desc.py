"""Encodings of the tcgen05 operands (mesh2hrtf_gb300/csrc/bem_umma.h),
checked field by field on the CPU before any kernel uses them.

Expected values are written out from the PTX ISA tables for tcgen05.mma: the
instruction descriptor of .kind::tf32 / .kind::f16 (D format at bits 4-5,
A / B formats at 7-9 / 10-12, majors at 15 / 16, N >> 3 at 17-22, M >> 4 at
24-28) and the shared-memory matrix descriptor (start >> 4 at 0-13, leading
offset >> 4 at 16-29, stride offset >> 4 at 32-45, version 1 at 46-47,
layout at 61-63 with 2 = 128-byte swizzle), and the 128-byte swizzle of
TMA's CU_TENSOR_MAP_SWIZZLE_128B (16-byte chunk index XOR row mod 8)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "mesh2hrtf_gb300", "csrc")

PROG = r"""
#include <cstdio>
#include "bem_umma.h"
using namespace bem::umma;
int main() {
    std::printf("%u\n", instr_desc(kDF32, kFmtTF32, kFmtTF32, 128, 16));
    std::printf("%u\n", instr_desc(kDF32, kFmtF16, kFmtF16, 64, 256));
    std::printf("%llu\n", (unsigned long long)smem_desc(0x1400, 16, 1024, kLayout128B));
    std::printf("%llu\n", (unsigned long long)smem_desc_advance(smem_desc(0x1400, 16, 1024, kLayout128B), 32));
    for (unsigned r = 0; r < 9; ++r) std::printf("%u %u\n", sw128_offset(r, 0), sw128_offset(r, 5));
    std::printf("%u\n", tmem_addr(0x20, 96, 16));
    return 0;
}
"""


@pytest.fixture(scope="module")
def out(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("umma")
    src = d / "t.cpp"
    src.write_text(PROG)
    exe = d / "t"
    subprocess.run([gxx, "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    return subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")


def test_instruction_descriptor_fields(out):
    v = int(out[0])
    assert (v >> 4) & 3 == 1            # D F32
    assert (v >> 7) & 7 == 2            # A TF32
    assert (v >> 10) & 7 == 2           # B TF32
    assert (v >> 15) & 1 == 0 and (v >> 16) & 1 == 0   # both K-major
    assert (v >> 17) & 63 == 16 >> 3    # N = 16
    assert (v >> 24) & 31 == 128 >> 4   # M = 128
    assert v & 0xF == 0 and (v >> 13) & 3 == 0 and (v >> 29) == 0
    assert v == 0x08040910
    w = int(out[1])
    assert (w >> 7) & 7 == 0 and (w >> 10) & 7 == 0 and (w >> 17) & 63 == 32 and (w >> 24) & 31 == 4


def test_smem_descriptor_fields(out):
    d = int(out[2])
    assert d & 0x3FFF == 0x1400 >> 4
    assert (d >> 16) & 0x3FFF == 1
    assert (d >> 32) & 0x3FFF == 1024 >> 4
    assert (d >> 46) & 3 == 1
    assert (d >> 49) & 7 == 0 and (d >> 52) & 1 == 0
    assert (d >> 61) & 7 == 2
    # a K step of 8 TF32 values (32 bytes) moves only the start address
    assert int(out[3]) - d == 2


def test_swizzle_128b_and_tmem_address(out):
    rows = [tuple(int(t) for t in out[4 + r].split()) for r in range(9)]
    for r, (o0, o5) in enumerate(rows):
        # element 0: chunk 0 lands in chunk r mod 8; element 5 (byte 20): chunk 1 -> 1 ^ (r mod 8)
        assert o0 == r * 128 + ((0 ^ (r % 8)) << 4)
        assert o5 == r * 128 + ((1 ^ (r % 8)) << 4) + 4
    assert int(out[13]) == 0x20 + (96 << 16) + 16
