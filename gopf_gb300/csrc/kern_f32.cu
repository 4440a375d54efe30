// kern_f32.cu -- FP32 instantiation of the spectral-step kernels, with the
// register-resident 256-point kernels serving the launches they cover.
#include "fast256.cuh"
#include "gopf_kernels_impl.cuh"

namespace gopf {

static bool fast_x(const XPassArgs<float> &a)
{
    return a.allow_fast && a.g.X == 256 && a.g.Y % f256::XROWS == 0 && a.in_mode == XIN_SPECTRAL &&
           a.program == XP_POLY && !a.rout && !a.red && !a.red2 && a.ngrp_out > 0;
}

static bool fast_y(const PassArgs<float> &a)
{
    if (!a.allow_fast || a.plan.n != 256 || a.g.Y != 256) return false;
    if (a.mode == PM_FWD || a.mode == PM_INV) return true;
    return (a.mode == PM_FUSED || a.mode == PM_INIT) && a.g.Z == 1 && a.nbuf <= 2 && a.upd.rk_stage == 0;
}

static bool fast_z(const PassArgs<float> &a)
{
    return a.allow_fast && a.plan.n == 256 && a.g.Z == 256 && a.g.S % 16 == 0 &&
           (a.mode == PM_FUSED || a.mode == PM_INIT) && a.nbuf <= 2 && a.upd.rk_stage == 0;
}

template <> cudaError_t launch_xpass<float>(const XPassArgs<float> &a, int LB, cudaStream_t st)
{
    if (fast_x(a)) {
        dim3 grid(a.g.Y / f256::XROWS, a.g.Z);
        if (a.ngrp_out == 1) f256::k_x256<1><<<grid, f256::NT, 0, st>>>(a);
        else f256::k_x256<0><<<grid, f256::NT, 0, st>>>(a);
        return cudaGetLastError();
    }
    return launch_xpass_generic<float>(a, LB, st);
}

template <> cudaError_t launch_cpass<float>(const PassArgs<float> &a, int LB, cudaStream_t st)
{
    if (fast_y(a)) {
        const long long nlines = (long long)a.g.Z * a.g.KX;
        const bool fused = (a.mode == PM_FUSED || a.mode == PM_INIT);
        dim3 grid((unsigned)((nlines + 15) / 16), fused ? 1 : a.nbuf);
        if (fused && a.nbuf > 1) f256::k_y256<2><<<grid, f256::NT, 0, st>>>(a);
        else f256::k_y256<1><<<grid, f256::NT, 0, st>>>(a);
        return cudaGetLastError();
    }
    return launch_cpass_generic<float>(a, LB, st);
}

template <> cudaError_t launch_spass<float>(const PassArgs<float> &a, int LB, cudaStream_t st)
{
    if (fast_z(a)) {
        if (a.nbuf > 1) f256::k_z256_fused<2><<<(unsigned)(a.g.S / 16), f256::NT, 0, st>>>(a);
        else f256::k_z256_fused<1><<<(unsigned)(a.g.S / 16), f256::NT, 0, st>>>(a);
        return cudaGetLastError();
    }
    return launch_spass_generic<float>(a, LB, st);
}

} // namespace gopf
