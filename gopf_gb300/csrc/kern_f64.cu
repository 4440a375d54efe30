// kern_f64.cu -- FP64 instantiation of the spectral-step kernels.
#include "gopf_kernels_impl.cuh"

namespace gopf {
template <> cudaError_t launch_xpass<double>(const XPassArgs<double> &a, int LB, cudaStream_t st)
{
    return launch_xpass_generic<double>(a, LB, st);
}
template <> int xpass_red_blocks<double>(const XPassArgs<double> &a, int LB)
{
    return ((a.g.Y + LB - 1) / LB) * a.g.Z;
}
template <> cudaError_t launch_cpass<double>(const PassArgs<double> &a, int LB, cudaStream_t st)
{
    return launch_cpass_generic<double>(a, LB, st);
}
template <> cudaError_t launch_spass<double>(const PassArgs<double> &a, int LB, cudaStream_t st)
{
    return launch_spass_generic<double>(a, LB, st);
}
} // namespace gopf
