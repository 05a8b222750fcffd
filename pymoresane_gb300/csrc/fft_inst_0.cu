// Kernel instantiations for FFT lengths: 24 48 96 192 32 64 128 256 (one translation unit per group
// so that the lengths compile in parallel).
#include "fft_kernels.cuh"

namespace msn {
namespace fftk {
MSN_FFT_INSTANTIATE(24)
MSN_FFT_INSTANTIATE(48)
MSN_FFT_INSTANTIATE(96)
MSN_FFT_INSTANTIATE(192)
MSN_FFT_INSTANTIATE(32)
MSN_FFT_INSTANTIATE(64)
MSN_FFT_INSTANTIATE(128)
MSN_FFT_INSTANTIATE(256)
}  // namespace fftk
}  // namespace msn
