// Four-step FFT convolution kernels for 4096-point grids (see fft_sq.cuh).
#define MSN_SQ_KERNELS
#include "fft_sq.cuh"

#include <cudaTypedefs.h>

namespace msn {
namespace fftk {
namespace sq {

int plane_map(CUtensorMap *map, void *base) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult q;
        void *fn = nullptr;
        MSN_TRY(check_cuda(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q),
                           "cudaGetDriverEntryPointByVersion(cuTensorMapEncodeTiled)"));
        if (q != cudaDriverEntryPointSuccess || !fn)
            return set_error(MSN_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    if ((reinterpret_cast<uintptr_t>(base) & 15u) != 0)
        return set_error(MSN_ERR_INVALID, "FFT workspace plane must be 16-byte aligned");
    const cuuint64_t dims[3] = {4, (cuuint64_t)PAIRS, (cuuint64_t)((W + 1) / 2)};
    const cuuint64_t strides[2] = {16, (cuuint64_t)PAIRS * 16};
    const cuuint32_t box[3] = {4, 1, (cuuint32_t)kBoxG};
    const cuuint32_t estride[3] = {1, 1, 1};
    const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estride,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(MSN_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return MSN_OK;
}

}  // namespace sq
}  // namespace fftk
}  // namespace msn

// Reads and clears the wait-timeout status word of the four-step kernels.
extern "C" int msn_fft_status(unsigned *out) {
    msn::clear_error();
    if (!out) return msn::set_error(MSN_ERR_INVALID, "msn_fft_status: null pointer");
    unsigned v = 0;
    MSN_TRY(msn::check_cuda(cudaMemcpyFromSymbol(&v, msn::fftk::sq::g_sq_status, sizeof(v)), "read status"));
    const unsigned zero = 0;
    MSN_TRY(msn::check_cuda(cudaMemcpyToSymbol(msn::fftk::sq::g_sq_status, &zero, sizeof(zero)), "clear status"));
    *out = v;
    return MSN_OK;
}

extern "C" int msn_fft_sq_grids(int *out) {
    msn::clear_error();
    if (!out) return msn::set_error(MSN_ERR_INVALID, "msn_fft_sq_grids: null pointer");
    msn::fftk::sq::SqLaunch c;
    MSN_TRY(msn::fftk::sq::launch_config(&c));
    out[0] = c.fwd_grid;
    out[1] = c.col_grid;
    out[2] = c.inv_grid;
    return MSN_OK;
}
