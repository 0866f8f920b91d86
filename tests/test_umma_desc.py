"""Bit fields of the tcgen05 descriptors (oetqf.jl_gb300/csrc/umma.cuh), decoded on the CPU from a
host-only build of the header: the instruction descriptor of a BF16 x BF16 -> FP32 MMA with K-major
operands, and the shared-memory descriptor of a 128-byte-swizzled K-major tile."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bits(v, lo, n):
    return (v >> lo) & ((1 << n) - 1)


@pytest.fixture(scope="module")
def printed(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("umma") / "umma_desc_print")
    src = os.path.join(ROOT, "tests", "native", "umma_desc_print.cu")
    inc = os.path.join(ROOT, "oetqf.jl_gb300", "csrc")
    subprocess.run([nvcc, "-std=c++17", "-I", inc, "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True,
                   capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    idesc = {(int(a), int(b)): int(v) for k, a, b, v in (l.split() for l in out if l.startswith("idesc"))}
    sdesc = {int(a): int(v) for k, a, v in (l.split() for l in out if l.startswith("sdesc"))}
    return idesc, sdesc


def test_instruction_descriptor_fields(printed):
    idesc, _ = printed
    for (M, N), v in idesc.items():
        assert _bits(v, 0, 4) == 0          # dense, no saturation
        assert _bits(v, 4, 2) == 1          # D in FP32
        assert _bits(v, 6, 1) == 0
        assert _bits(v, 7, 3) == 1          # A in BF16
        assert _bits(v, 10, 3) == 1         # B in BF16
        assert _bits(v, 13, 2) == 0         # no negation
        assert _bits(v, 15, 2) == 0         # A and B K-major
        assert _bits(v, 17, 6) == N >> 3
        assert _bits(v, 23, 1) == 0
        assert _bits(v, 24, 5) == M >> 4
        assert _bits(v, 29, 3) == 0
        assert v < 1 << 32


def test_shared_memory_descriptor_fields(printed):
    _, sdesc = printed
    for addr, v in sdesc.items():
        assert _bits(v, 0, 14) == (addr & 0x3FFFF) >> 4   # start address >> 4
        assert _bits(v, 14, 2) == 0
        assert _bits(v, 16, 14) == 1                     # leading byte offset 16 B (unused by this layout)
        assert _bits(v, 30, 2) == 0
        assert _bits(v, 32, 14) == 1024 >> 4             # 8-row groups of 128-byte rows
        assert _bits(v, 46, 2) == 1                      # descriptor version
        assert _bits(v, 48, 1) == 0
        assert _bits(v, 49, 3) == 0                      # base offset: tiles 1024-byte aligned
        assert _bits(v, 52, 9) == 0
        assert _bits(v, 61, 3) == 2                      # 128-byte swizzle
    # the K-slice advance of the MMA loop (32 bytes = 16 BF16) moves only the start address field
    assert sdesc[0x8000 + 32] - sdesc[0] == (0x8000 + 32) >> 4
