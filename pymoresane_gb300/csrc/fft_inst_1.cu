// Kernel instantiations for FFT lengths: 384 768 512 1024 (one translation unit per group
// so that the lengths compile in parallel).
#include "fft_kernels.cuh"

namespace msn {
namespace fftk {
MSN_FFT_INSTANTIATE(384)
MSN_FFT_INSTANTIATE(768)
MSN_FFT_INSTANTIATE(512)
MSN_FFT_INSTANTIATE(1024)
}  // namespace fftk
}  // namespace msn
