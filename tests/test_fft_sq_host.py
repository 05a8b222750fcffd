"""Four-step 4096-point transform of the square FFT kernels, run on the CPU.

The 64-point register DFT (both slot orders), the 4096-point twiddles and the
exchange order of pymoresane_gb300/csrc/fft_sq.cuh are host-device code;
nvcc compiles them into a host program here and the transforms are compared
with numpy's FFT (float64) on random data.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "pymoresane_gb300", "csrc")

PROGRAM = r'''
#include <cmath>
#include <cstdio>
#include <vector>
#define MSN_HOST_ONLY
#include "fft_sq.cuh"
using namespace msn::fftk::sq;
struct HostW {
    float2 operator()(int m) const {
        const double a = -2.0 * M_PI * (double)(m & (M - 1)) / M;
        return make_float2((float)std::cos(a), (float)std::sin(a));
    }
};
// thread t holds x[t + 64 j]; returns X[t + 64 k2] (forward or inverse, unnormalised)
template <bool INV, bool TIN_A>
void transform(std::vector<float2> &data) {
    std::vector<float2> buf(SEQ);
    std::vector<std::vector<float2>> regs(R, std::vector<float2>(R));
    for (int t = 0; t < R; ++t) {
        float2 *v = regs[t].data();
        for (int j = 0; j < R; ++j) v[TIN_A ? tslot(j) : j] = data[t + R * j];
        dft64<INV, TIN_A>(v);
        twiddle_t<INV, !TIN_A>(v, t, HostW{});
        for (int k1 = 0; k1 < R; ++k1) buf[k1 * PADR + t] = v[!TIN_A ? tslot(k1) : k1];
    }
    for (int t = 0; t < R; ++t) {
        float2 *v = regs[t].data();
        for (int n1 = 0; n1 < R; ++n1) v[n1] = buf[t * PADR + n1];
        dft64<INV, false>(v);
        for (int k2 = 0; k2 < R; ++k2) data[t + R * k2] = v[tslot(k2)];
    }
}
int main() {
    std::vector<float2> d(M);
    for (int i = 0; i < M; ++i) if (std::scanf("%f %f", &d[i].x, &d[i].y) != 2) return 1;
    std::vector<float2> f = d, g = d, h = d;
    transform<false, false>(f);
    transform<true, false>(g);
    transform<true, true>(h);
    for (int i = 0; i < M; ++i) std::printf("%.9g %.9g %.9g %.9g %.9g %.9g\n", f[i].x, f[i].y, g[i].x, g[i].y, h[i].x, h[i].y);
    return 0;
}
'''


def test_four_step_4096_matches_numpy(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "sq.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "sq"
    subprocess.run([nvcc, "-std=c++20", "--expt-relaxed-constexpr", "-O2", "-I", CSRC, "-I",
                    os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True, capture_output=True)
    rng = np.random.default_rng(3)
    x = (rng.standard_normal(4096) + 1j * rng.standard_normal(4096)).astype(np.complex64)
    inp = "\n".join(f"{v.real:.9g} {v.imag:.9g}" for v in x)
    out = subprocess.run([str(exe)], input=inp, check=True, capture_output=True, text=True).stdout
    a = np.array([list(map(float, ln.split())) for ln in out.strip().split("\n")])
    fwd, inv, inv_t = a[:, 0] + 1j * a[:, 1], a[:, 2] + 1j * a[:, 3], a[:, 4] + 1j * a[:, 5]
    xd = x.astype(np.complex128)
    want_f = np.fft.fft(xd)
    want_i = np.fft.ifft(xd) * 4096
    scale = np.abs(want_f).max()
    assert np.abs(fwd - want_f).max() <= 2e-6 * scale
    assert np.abs(inv - want_i).max() <= 2e-6 * scale
    # transposed pass-A input order (the inverse that follows the PSF product) gives the same transform
    assert np.abs(inv_t - want_i).max() <= 2e-6 * scale
