// Kernel instantiations for FFT lengths: 3072 4096 (one translation unit per group
// so that the lengths compile in parallel).
#include "fft_kernels.cuh"

namespace msn {
namespace fftk {
MSN_FFT_INSTANTIATE(3072)
MSN_FFT_INSTANTIATE(4096)
}  // namespace fftk
}  // namespace msn
