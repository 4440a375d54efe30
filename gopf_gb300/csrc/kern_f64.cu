// kern_f64.cu -- FP64 instantiation of the spectral-step kernels.
#include "gopf_kernels_impl.cuh"

namespace gopf {
template cudaError_t launch_xpass<double>(const XPassArgs<double> &, int, cudaStream_t);
template cudaError_t launch_cpass<double>(const PassArgs<double> &, int, cudaStream_t);
template cudaError_t launch_spass<double>(const PassArgs<double> &, int, cudaStream_t);
} // namespace gopf
