// kern_f32.cu -- FP32 instantiation of the spectral-step kernels.
#include "gopf_kernels_impl.cuh"

namespace gopf {
template cudaError_t launch_xpass<float>(const XPassArgs<float> &, int, cudaStream_t);
template cudaError_t launch_cpass<float>(const PassArgs<float> &, int, cudaStream_t);
template cudaError_t launch_spass<float>(const PassArgs<float> &, int, cudaStream_t);
} // namespace gopf
