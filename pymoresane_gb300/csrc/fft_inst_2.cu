// Kernel instantiations for FFT lengths: 1536 2048 (one translation unit per group
// so that the lengths compile in parallel).
#include "fft_kernels.cuh"

namespace msn {
namespace fftk {
MSN_FFT_INSTANTIATE(1536)
MSN_FFT_INSTANTIATE(2048)
}  // namespace fftk
}  // namespace msn
