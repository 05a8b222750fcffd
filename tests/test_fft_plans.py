"""FFT plan invariants for every supported length (host code only: nvcc compiles, the CPU runs it)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "pymoresane_gb300", "csrc")

PROGRAM = r'''
#include <cstdio>
#include "fft_plan.cuh"
using namespace msn::fftk;
int main() {
    const int sizes[] = {24, 48, 96, 192, 384, 768, 1536, 3072, 6144, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192};
    for (int m : sizes) {
        const CtPlan p = ct_plan(m);
        long prod = 1;
        int tw = 0;
        bool twbase_ok = true;
        for (int q = 0; q < p.np; ++q) {
            if (p.ns[q] != prod) twbase_ok = false;
            if (q > 0 && p.twbase[q] != tw) twbase_ok = false;
            if (q > 0) tw += p.ns[q] * (p.radix[q] - 1);
            prod *= p.radix[q];
        }
        const bool direct = direct_ok(p, m);   // the predicate the kernels use
        std::printf("%d %d %ld %d %d %d %d %d %d\n", m, p.ok, prod, p.twlen == tw, twbase_ok, p.e, p.fusable, direct,
                    p.w == m / 2 + 1 && p.groups * p.group >= p.w);
    }
    std::printf("%d %d\n", ct_plan(20).ok, ct_plan(12288).ok);
    return 0;
}
'''


def test_plans_for_every_supported_length(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "plans.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "plans"
    subprocess.run([nvcc, "-std=c++20", "--expt-relaxed-constexpr", "-I", CSRC, str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    lines = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    rows = [list(map(int, ln.split())) for ln in lines if ln.strip()]
    for m, ok, prod, twlen_ok, twbase_ok, e, fusable, direct, groups_ok in rows[:-1]:
        assert ok == 1 and prod == m and twlen_ok and twbase_ok and groups_ok, m
        assert e == (24 if m % 3 == 0 else 16)
        # global-fed / global-stored passes for every grid from 256 and 384 up; the PSF product
        # fused between the column passes up to 6144 (8192's fused pass would need 1024 threads,
        # and 192 = 3 * 64 has a first radix-8 stride that is not a multiple of 16): smaller grids
        # and 8192 columns take the staged kernels
        assert direct == (m >= 256 and m != 192), m
        assert fusable == (m >= 256 and m != 192 and m != 8192), m
    assert rows[-1] == [0, 0]   # unsupported lengths are refused
