// Kernel instantiations for FFT lengths: 6144 8192 (one translation unit per group
// so that the lengths compile in parallel).
#include "fft_kernels.cuh"

namespace msn {
namespace fftk {
MSN_FFT_INSTANTIATE(6144)
MSN_FFT_INSTANTIATE(8192)
}  // namespace fftk
}  // namespace msn
