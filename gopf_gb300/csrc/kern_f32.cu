// kern_f32.cu -- FP32 instantiation of the spectral-step kernels, with the
// register-resident 256-point kernels serving the launches they cover.
#include <algorithm>
#include <mutex>
#include <utility>

#include "fast256.cuh"
#include "fastline.cuh"
#include "gopf_kernels_impl.cuh"
#include "elastic256.cuh"
#include "x256_io.cuh"

namespace gopf {

// Launch k with the programmatic-serialization attribute when pdl is set: the kernel may start while
// the stream's previous kernel finishes (it waits for that kernel's data with griddepcontrol.wait).
template <typename... KArgs, typename... Args>
static cudaError_t launch_k(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, bool pdl,
                            Args &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

// [Z][S] view of a z-pass array with lines x 256 boxes
static bool z_map(CUtensorMap *m, const float2 *p, const Geom &g, int lines = 16)
{
    const unsigned long long dims[2] = {(unsigned long long)g.S, (unsigned long long)g.Z};
    const unsigned long long strides[1] = {(unsigned long long)g.S * sizeof(float2)};
    const unsigned box[2] = {(unsigned)lines, (unsigned)f256::N};
    return encode_map_8b(m, p, 2, dims, strides, box);
}

// [Z][KX][Y] view of an x-pass array with {rows, KX, 1} boxes
static bool x_map(CUtensorMap *m, const float2 *p, const Geom &g, int rows = f256::XROWS)
{
    const unsigned long long dims[3] = {(unsigned long long)g.Y, (unsigned long long)g.KX, (unsigned long long)g.Z};
    const unsigned long long strides[2] = {(unsigned long long)g.Y * sizeof(float2),
                                           (unsigned long long)g.S * sizeof(float2)};
    const unsigned box[3] = {(unsigned)rows, (unsigned)g.KX, 1};
    return encode_map_8b(m, p, 3, dims, strides, box);
}

static bool launch_x_tma(const XPassArgs<float> &a, cudaStream_t st, cudaError_t *err)
{
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
        attr_err = cudaFuncSetAttribute(f256::k_x256_tma<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        f256::x256_tma_smem_bytes());
        if (attr_err == cudaSuccess)
            attr_err = cudaFuncSetAttribute(f256::k_x256_tma<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            f256::x256_tma_smem_bytes());
    });
    if (attr_err != cudaSuccess || a.g.KX != 129 || a.ngrp_out > GOPF_MAX_GROUPS) return false;
    CUtensorMap mi, mo[GOPF_MAX_GROUPS];
    const bool one = (a.ngrp_out == 1 && (a.identity || (a.pw.deg[0] >= 0 && a.pw.deg[0] <= 6)));
    if (one && (a.allow_fast & 8) && a.g.Y % f256::XH_ROWS == 0) {
        // one dense polynomial group on half-height tiles: eight blocks per SM
        static std::once_flag once_h;
        static cudaError_t attr_h = cudaSuccess;
        std::call_once(once_h, [] {
            attr_h = cudaFuncSetAttribute(f256::k_x256_th, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          f256::x256_th_smem_bytes());
        });
        if (attr_h != cudaSuccess || !x_map(&mi, a.in, a.g, f256::XH_ROWS)) return false;
        f256::k_x256_th<<<dim3(a.g.Y / f256::XH_ROWS, a.g.Z), f256::XH_NT, f256::x256_th_smem_bytes(), st>>>(a, mi);
        *err = cudaGetLastError();
        return true;
    }
    if (!x_map(&mi, a.in, a.g)) return false;
    if (one) {
        // one dense polynomial group: four blocks per SM, direct stores
        f256::k_x256_tl<<<dim3(a.g.Y / f256::XROWS, a.g.Z), f256::NT, f256::x256_tl_smem_bytes(), st>>>(a, mi);
        *err = cudaGetLastError();
        return true;
    }
    for (int b = 0; b < GOPF_MAX_GROUPS; ++b) {
        if (b < a.ngrp_out) {
            if (!x_map(&mo[b], a.out[b], a.g)) return false;
        } else {
            mo[b] = mo[0];
        }
    }
    dim3 grid(a.g.Y / f256::XROWS, a.g.Z);
    if (a.ngrp_out == 1)
        f256::k_x256_tma<1><<<grid, f256::NT, f256::x256_tma_smem_bytes(), st>>>(a, mi, mo[0], mo[1], mo[2], mo[3]);
    else
        f256::k_x256_tma<0><<<grid, f256::NT, f256::x256_tma_smem_bytes(), st>>>(a, mi, mo[0], mo[1], mo[2], mo[3]);
    *err = cudaGetLastError();
    return true;
}

// Launch the TMA z kernel; false when a tensor map cannot be made (the caller
// then launches the plain-load kernel).
static bool launch_z_tma(const PassArgs<float> &a, cudaStream_t st, cudaError_t *err)
{
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
        const void *k[4] = {(const void *)f256::k_z256_tma<1, false>, (const void *)f256::k_z256_tma<2, false>,
                            (const void *)f256::k_z256_tma<1, true>, (const void *)f256::k_z256_tma<2, true>};
        for (int i = 0; i < 4 && attr_err == cudaSuccess; ++i)
            attr_err = cudaFuncSetAttribute(k[i], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            f256::z256_tma_smem_bytes(1 + (i & 1)));
    });
    if (attr_err != cudaSuccess) return false;
    CUtensorMap mU0, mU1, mS, mT;
    const bool nz = (a.upd.noise.kind != 0 || a.upd.filt != nullptr);
    if (a.nbuf == 1 && (a.allow_fast & 16) && a.g.S % f256::ZH_LINES == 0) {
        // one group on half-width tiles: six blocks per SM
        static std::once_flag once_h;
        static cudaError_t attr_h = cudaSuccess;
        std::call_once(once_h, [] {
            attr_h = cudaFuncSetAttribute(f256::k_z256_th<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          f256::z256_th_smem_bytes());
            if (attr_h == cudaSuccess)
                attr_h = cudaFuncSetAttribute(f256::k_z256_th<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              f256::z256_th_smem_bytes());
        });
        if (attr_h != cudaSuccess || !z_map(&mU0, a.buf[0], a.g, f256::ZH_LINES) ||
            !z_map(&mT, a.tout, a.g, f256::ZH_LINES) || !z_map(&mS, a.state, a.g, f256::ZH_LINES))
            return false;
        const unsigned gh = (unsigned)(a.g.S / f256::ZH_LINES);
        const bool pdl = (a.allow_fast & ALLOW_PDL) != 0;
        *err = launch_k(nz ? f256::k_z256_th<true> : f256::k_z256_th<false>, dim3(gh), dim3(f256::ZH_NT),
                        f256::z256_th_smem_bytes(), st, pdl, a, mU0, mS, mT);
        return true;
    }
    if (!z_map(&mU0, a.buf[0], a.g) || !z_map(&mT, a.tout, a.g) || !z_map(&mS, a.state, a.g)) return false;
    if (a.nbuf > 1) {
        if (!z_map(&mU1, a.buf[1], a.g)) return false;
    } else {
        mU1 = mU0;
    }
    const unsigned grid = (unsigned)(a.g.S / 16);
    const int sm1 = f256::z256_tma_smem_bytes(1), sm2 = f256::z256_tma_smem_bytes(2);
    if (a.nbuf > 1) {
        if (nz) f256::k_z256_tma<2, true><<<grid, f256::NT, sm2, st>>>(a, mU0, mU1, mS, mT);
        else f256::k_z256_tma<2, false><<<grid, f256::NT, sm2, st>>>(a, mU0, mU1, mS, mT);
    } else {
        if (nz) f256::k_z256_tma<1, true><<<grid, f256::NT, sm1, st>>>(a, mU0, mU1, mS, mT);
        else f256::k_z256_tma<1, false><<<grid, f256::NT, sm1, st>>>(a, mU0, mU1, mS, mT);
    }
    *err = cudaGetLastError();
    return true;
}

static bool fast_x(const XPassArgs<float> &a)
{
    return a.allow_fast && a.g.X == 256 && a.g.Y % f256::XROWS == 0 && a.in_mode == XIN_SPECTRAL &&
           a.program == XP_POLY && !a.rout && !a.red && !a.red2 && a.ngrp_out > 0;
}

static bool fast_y(const PassArgs<float> &a)
{
    if (!a.allow_fast || a.plan.n != 256 || a.g.Y != 256) return false;
    if (a.mode == PM_FWD || a.mode == PM_INV) return true;
    return (a.mode == PM_FUSED || a.mode == PM_INIT) && a.g.Z == 1 && a.nbuf <= 2 && a.upd.rk_stage == 0 &&
           a.upd.etd == 0 && a.upd.nxs == 0 && a.upd.nxf == 0 && a.upd.nsrc == 0 && a.upd.nimp <= 4;
}

static bool fast_z(const PassArgs<float> &a)
{
    return a.allow_fast && a.plan.n == 256 && a.g.Z == 256 && a.g.S % 16 == 0 &&
           (a.mode == PM_FUSED || a.mode == PM_INIT) && a.nbuf <= 2 && a.upd.rk_stage == 0 && a.upd.etd == 0 &&
           a.upd.nxs == 0 && a.upd.nxf == 0 && a.upd.nsrc == 0 && a.upd.nimp <= 4;
}

// the elastic term's passes on 256-point axes (elastic256.cuh)
static bool fast_x_elq(const XPassArgs<float> &a)
{
    return a.allow_fast && a.g.X == 256 && a.g.Y % f256::XROWS == 0 && a.in_mode == XIN_SPECTRAL &&
           a.program == XP_ELASTIC_Q && !a.rout && !a.red && !a.red2;
}

static bool fast_z_elk(const PassArgs<float> &a)
{
    return a.allow_fast && a.plan.n == 256 && a.g.Z == 256 && a.g.S % 16 == 0 && a.mode == PM_ELASTIC_K;
}

// 256-column x passes that start or end in real space
static bool fast_x_c2r(const XPassArgs<float> &a)
{
    return (a.allow_fast & 2) && a.g.X == 256 && a.g.KX == 129 && a.g.Y % f256::XROWS == 0 &&
           a.in_mode == XIN_SPECTRAL && a.program == XP_POLY && a.ngrp_out == 0 && (a.rout || a.red) && !a.red2;
}

static bool fast_x_r2c(const XPassArgs<float> &a)
{
    return (a.allow_fast & 2) && a.g.X == 256 && a.g.KX == 129 && a.g.Y % f256::XROWS == 0 && a.in_mode == XIN_REAL &&
           a.program == XP_POLY && !a.rout && !a.red && !a.red2 && a.ngrp_out >= 1 && a.ngrp_out <= GOPF_MAX_GROUPS;
}

static cudaError_t io_attributes()
{
    static std::once_flag once;
    static cudaError_t err = cudaSuccess;
    std::call_once(once, [] {
        const int sm = f256::x256_io_smem_bytes();
        err = cudaFuncSetAttribute(f256::k_x256_c2r, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(f256::k_x256_r2c<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(f256::k_x256_r2c<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    });
    return err;
}

static bool launch_x_io(const XPassArgs<float> &a, cudaStream_t st, cudaError_t *err)
{
    if (io_attributes() != cudaSuccess) return false;
    dim3 grid(a.g.Y / f256::XROWS, a.g.Z);
    const int sm = f256::x256_io_smem_bytes();
    if (fast_x_c2r(a)) {
        CUtensorMap mi;
        if (!x_map(&mi, a.in, a.g)) return false;
        f256::k_x256_c2r<<<grid, f256::NT, sm, st>>>(a, mi);
        *err = cudaGetLastError();
        return true;
    }
    if (fast_x_r2c(a)) {
        CUtensorMap mo[GOPF_MAX_GROUPS];
        for (int b = 0; b < GOPF_MAX_GROUPS; ++b) {
            if (b < a.ngrp_out) {
                if (!x_map(&mo[b], a.out[b], a.g)) return false;
            } else {
                mo[b] = mo[0];
            }
        }
        if (a.ngrp_out == 1) f256::k_x256_r2c<1><<<grid, f256::NT, sm, st>>>(a, mo[0], mo[1], mo[2], mo[3]);
        else f256::k_x256_r2c<0><<<grid, f256::NT, sm, st>>>(a, mo[0], mo[1], mo[2], mo[3]);
        *err = cudaGetLastError();
        return true;
    }
    return false;
}

template <> int xpass_red_blocks<float>(const XPassArgs<float> &a, int LB)
{
    if (fast_x_c2r(a)) return (a.g.Y / f256::XROWS) * a.g.Z;
    return ((a.g.Y + LB - 1) / LB) * a.g.Z;
}

// ---- the register-resident line engine for 2D lines of 384 ... 1024 (fastline.cuh) ----

// NB: threads per block; 0 is the engine's default (256, or 192 for 384 and 768), half of that serves
// grids too small to give every SM two blocks of the default size (twice the blocks per SM, each with
// half the lines, so the launch bounds double the blocks per SM at the same registers per thread)
template <int L, int NG, int NB>
__global__ void __launch_bounds__(fl::Geo<L, NB>::NT, NB ? 6 : 3) k_yline(const PassArgs<float> a)
{
    fl::yline_tile<L, NG, NB>(a, blockIdx.x);
}
template <int L, int NB>
__global__ void __launch_bounds__(fl::Geo<L, NB>::NT, NB ? 6 : 3) k_yline_pass(const PassArgs<float> a)
{
    fl::yline_pass_tile<L, NB>(a, blockIdx.x, blockIdx.y, a.mode == PM_INV);
}
template <int L, int NB> __global__ void __launch_bounds__(fl::Geo<L, NB>::NT, NB ? 6 : 3) k_xline(const XPassArgs<float> a)
{
    fl::xline_tile<L, false, NB>(a, blockIdx.x, blockIdx.y);
}
// one dense polynomial group of degree <= 6: one line in registers, four blocks per SM
template <int L, int NB> __global__ void __launch_bounds__(fl::Geo<L, NB>::NT, NB ? 8 : 4) k_xline1(const XPassArgs<float> a)
{
    fl::xline_tile<L, true, NB>(a, blockIdx.x, blockIdx.y);
}

// the adjoint step's x pass (XP_ADJ): two lines in registers, so half the default blocks per SM
template <int L, int NB>
__global__ void __launch_bounds__(fl::Geo<L, NB>::NT, NB ? 4 : 2) k_xline_adj(const XPassArgs<float> a)
{
    fl::xline_adj_tile<L, NB>(a, blockIdx.x, blockIdx.y);
}

// half of the engine's default block (a multiple of the line's T threads and of a warp)
template <int L> constexpr int half_nb() { return fl::Geo<L>::NT / 2; }

// blocks a grid of `blocks` default-size blocks leaves per SM: fewer than two asks for half-size blocks
static bool small_grid(long long blocks)
{
    static int nsm = 0;
    if (!nsm) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1)
            nsm = 152;
    }
    return blocks < 2LL * nsm;
}

static bool line_len(int n) { return n == 384 || n == 512 || n == 768 || n == 1024; }

static bool fast_x_line(const XPassArgs<float> &a)
{
    return a.allow_fast && line_len(a.g.X) && a.in_mode == XIN_SPECTRAL && a.program == XP_POLY && !a.identity &&
           !a.rout && !a.red && !a.red2 && a.ngrp_out > 0;
}

// the 2D fused Euler update without noise, filters, symbols or field terms
static bool fast_y_line(const PassArgs<float> &a)
{
    const UpdTable &u = a.upd;
    return a.allow_fast && line_len(a.plan.n) && a.g.Y == a.plan.n && a.g.Z == 1 && a.mode == PM_FUSED && a.nbuf <= 2 &&
           u.rk_stage == 0 && u.etd == 0 && u.nxs == 0 && u.nxf == 0 && u.nsrc == 0 && u.nimp <= 4 && !u.noise.kind &&
           !u.filt;
}

template <typename K> static cudaError_t line_smem(K kern, int bytes)
{
    return bytes > 48 * 1024 ? cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)
                             : cudaSuccess;
}

template <int L, int NB> static cudaError_t launch_xline_nb(const XPassArgs<float> &a, cudaStream_t st)
{
    typedef fl::Geo<L, NB> G;
    if (a.g.Y % (2 * G::LPB)) return cudaErrorNotSupported;
    const dim3 grid(a.g.Y / (2 * G::LPB), a.g.Z);
    if (a.ngrp_out == 1 && a.pw.deg[0] >= 0 && a.pw.deg[0] <= 6) {
        static const cudaError_t attr1 = line_smem(k_xline1<L, NB>, fl::xline_smem_bytes<L, NB>());
        if (attr1 != cudaSuccess) return attr1;
        k_xline1<L, NB><<<grid, G::NT, fl::xline_smem_bytes<L, NB>(), st>>>(a);
        return cudaGetLastError();
    }
    static const cudaError_t attr = line_smem(k_xline<L, NB>, fl::xline_smem_bytes<L, NB>());
    if (attr != cudaSuccess) return attr;
    k_xline<L, NB><<<grid, G::NT, fl::xline_smem_bytes<L, NB>(), st>>>(a);
    return cudaGetLastError();
}

template <int L> static cudaError_t launch_xline(const XPassArgs<float> &a, cudaStream_t st)
{
    typedef fl::Geo<L> G;
    if (small_grid((long long)(a.g.Y / (2 * G::LPB)) * a.g.Z)) return launch_xline_nb<L, half_nb<L>()>(a, st);
    return launch_xline_nb<L, 0>(a, st);
}

template <int L, int NB> static cudaError_t launch_xline_adj_nb(const XPassArgs<float> &a, cudaStream_t st)
{
    typedef fl::Geo<L, NB> G;
    if (a.g.Y % (2 * G::LPB)) return cudaErrorNotSupported;
    static const cudaError_t attr = line_smem(k_xline_adj<L, NB>, fl::xline_smem_bytes<L, NB>());
    if (attr != cudaSuccess) return attr;
    k_xline_adj<L, NB><<<dim3(a.g.Y / (2 * G::LPB), a.g.Z), G::NT, fl::xline_smem_bytes<L, NB>(), st>>>(a);
    return cudaGetLastError();
}

template <int L> static cudaError_t launch_xline_adj(const XPassArgs<float> &a, cudaStream_t st)
{
    typedef fl::Geo<L> G;
    if (small_grid((long long)(a.g.Y / (2 * G::LPB)) * a.g.Z)) return launch_xline_adj_nb<L, half_nb<L>()>(a, st);
    return launch_xline_adj_nb<L, 0>(a, st);
}

// the adjoint's x pass on the line engine: spectral inputs, the real rows in and out, one output
static bool fast_x_line_adj(const XPassArgs<float> &a)
{
    return a.allow_fast && line_len(a.g.X) && a.in_mode == XIN_SPECTRAL && a.program == XP_ADJ && a.in && a.in2 &&
           a.rin && a.rout && a.ngrp_out == 1 && !a.red && !a.red2;
}

// plain forward / inverse y transforms of every buffer on the line engine (sides 384 ... 1024)
static bool fast_y_line_pass(const PassArgs<float> &a)
{
    return a.allow_fast && (a.mode == PM_FWD || a.mode == PM_INV) && line_len(a.plan.n) && a.g.Y == a.plan.n &&
           a.nbuf >= 1;
}

template <int L, int NB> static cudaError_t launch_yline_pass_nb(const PassArgs<float> &a, cudaStream_t st)
{
    typedef fl::Geo<L, NB> G;
    static const cudaError_t attr = line_smem(k_yline_pass<L, NB>, fl::yline_smem_bytes<L, NB>());
    if (attr != cudaSuccess) return attr;
    const long long nlines = (long long)a.g.Z * a.g.KX;
    k_yline_pass<L, NB><<<dim3((unsigned)((nlines + G::LPB - 1) / G::LPB), (unsigned)a.nbuf), G::NT,
                          fl::yline_smem_bytes<L, NB>(), st>>>(a);
    return cudaGetLastError();
}

template <int L> static cudaError_t launch_yline_pass(const PassArgs<float> &a, cudaStream_t st)
{
    typedef fl::Geo<L> G;
    const long long blocks = ((long long)a.g.Z * a.g.KX + G::LPB - 1) / G::LPB * a.nbuf;
    if (small_grid(blocks)) return launch_yline_pass_nb<L, half_nb<L>()>(a, st);
    return launch_yline_pass_nb<L, 0>(a, st);
}

template <int L, int NG, int NB> static cudaError_t launch_yline_nb(const PassArgs<float> &a, cudaStream_t st)
{
    typedef fl::Geo<L, NB> G;
    static const cudaError_t attr = line_smem(k_yline<L, NG, NB>, fl::yline_smem_bytes<L, NB>());
    if (attr != cudaSuccess) return attr;
    k_yline<L, NG, NB><<<(unsigned)((a.g.KX + G::LPB - 1) / G::LPB), G::NT, fl::yline_smem_bytes<L, NB>(), st>>>(a);
    return cudaGetLastError();
}

template <int L, int NG> static cudaError_t launch_yline(const PassArgs<float> &a, cudaStream_t st)
{
    typedef fl::Geo<L> G;
    if (small_grid((a.g.KX + G::LPB - 1) / G::LPB)) return launch_yline_nb<L, NG, half_nb<L>()>(a, st);
    return launch_yline_nb<L, NG, 0>(a, st);
}

static bool launch_x_line(const XPassArgs<float> &a, cudaStream_t st, cudaError_t *e)
{
    if (fast_x_line_adj(a)) {
        switch (a.g.X) {
        case 384: *e = launch_xline_adj<384>(a, st); break;
        case 512: *e = launch_xline_adj<512>(a, st); break;
        case 768: *e = launch_xline_adj<768>(a, st); break;
        default: *e = launch_xline_adj<1024>(a, st); break;
        }
        return *e != cudaErrorNotSupported;
    }
    if (!fast_x_line(a)) return false;
    switch (a.g.X) {
    case 384: *e = launch_xline<384>(a, st); break;
    case 512: *e = launch_xline<512>(a, st); break;
    case 768: *e = launch_xline<768>(a, st); break;
    default: *e = launch_xline<1024>(a, st); break;
    }
    return *e != cudaErrorNotSupported;
}

static bool launch_y_line(const PassArgs<float> &a, cudaStream_t st, cudaError_t *e)
{
    if (!fast_y_line(a)) return false;
    const bool two = a.nbuf > 1;
    switch (a.plan.n) {
    case 384: *e = two ? launch_yline<384, 2>(a, st) : launch_yline<384, 1>(a, st); break;
    case 512: *e = two ? launch_yline<512, 2>(a, st) : launch_yline<512, 1>(a, st); break;
    case 768: *e = two ? launch_yline<768, 2>(a, st) : launch_yline<768, 1>(a, st); break;
    default: *e = two ? launch_yline<1024, 2>(a, st) : launch_yline<1024, 1>(a, st); break;
    }
    return true;
}

template <> cudaError_t launch_xpass<float>(const XPassArgs<float> &a, int LB, cudaStream_t st)
{
    {
        cudaError_t e;
        if (launch_x_io(a, st, &e)) return e;
    }
    if (fast_x_elq(a)) {
        static std::once_flag once;
        static cudaError_t attr = cudaSuccess;
        std::call_once(once, [] {
            attr = cudaFuncSetAttribute(f256::k_x256_elq, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        f256::x256_elq_smem_bytes());
        });
        if (attr != cudaSuccess) return attr;
        f256::k_x256_elq<<<dim3(a.g.Y / f256::XROWS, a.g.Z), f256::NT, f256::x256_elq_smem_bytes(), st>>>(a);
        return cudaGetLastError();
    }
    if (fast_x(a)) {
        cudaError_t e;
        if ((a.allow_fast & 2) && launch_x_tma(a, st, &e)) return e;
        dim3 grid(a.g.Y / f256::XROWS, a.g.Z);
        if (a.ngrp_out == 1) f256::k_x256<1><<<grid, f256::NT, 0, st>>>(a);
        else f256::k_x256<0><<<grid, f256::NT, 0, st>>>(a);
        return cudaGetLastError();
    }
    {
        cudaError_t e;
        if (launch_x_line(a, st, &e)) return e;
    }
    return launch_xpass_generic<float>(a, LB, st);
}

template <> cudaError_t launch_cpass<float>(const PassArgs<float> &a, int LB, cudaStream_t st)
{
    if (fast_y(a)) {
        const long long nlines = (long long)a.g.Z * a.g.KX;
        const bool fused = (a.mode == PM_FUSED || a.mode == PM_INIT);
        dim3 grid((unsigned)((nlines + 15) / 16), fused ? 1 : a.nbuf);
        const bool nz = fused && (a.upd.noise.kind != 0 || a.upd.filt != nullptr);
        const bool pdl = (a.allow_fast & ALLOW_PDL) != 0;
        if (fused && a.nbuf > 1)
            return launch_k(nz ? f256::k_y256<2, true> : f256::k_y256<2, false>, grid, dim3(f256::NT), 0, st, pdl, a);
        return launch_k(nz ? f256::k_y256<1, true> : f256::k_y256<1, false>, grid, dim3(f256::NT), 0, st, pdl, a);
    }
    {
        cudaError_t e;
        if (launch_y_line(a, st, &e)) return e;
    }
    if (fast_y_line_pass(a)) {
        switch (a.plan.n) {
        case 384: return launch_yline_pass<384>(a, st);
        case 512: return launch_yline_pass<512>(a, st);
        case 768: return launch_yline_pass<768>(a, st);
        default: return launch_yline_pass<1024>(a, st);
        }
    }
    return launch_cpass_generic<float>(a, LB, st);
}

template <> cudaError_t launch_spass<float>(const PassArgs<float> &a, int LB, cudaStream_t st)
{
    if (fast_z_elk(a)) {
        f256::k_z256_elk<<<(unsigned)(a.g.S / 16), f256::NT, 0, st>>>(a);
        return cudaGetLastError();
    }
    if (fast_z(a)) {
        cudaError_t e;
        if ((a.allow_fast & 2) && launch_z_tma(a, st, &e)) return e;
        const unsigned grid = (unsigned)(a.g.S / 16);
        const bool nz = (a.upd.noise.kind != 0 || a.upd.filt != nullptr);
        if (a.nbuf > 1) {
            if (nz) f256::k_z256_fused<2, true><<<grid, f256::NT, 0, st>>>(a);
            else f256::k_z256_fused<2, false><<<grid, f256::NT, 0, st>>>(a);
        } else {
            if (nz) f256::k_z256_fused<1, true><<<grid, f256::NT, 0, st>>>(a);
            else f256::k_z256_fused<1, false><<<grid, f256::NT, 0, st>>>(a);
        }
        return cudaGetLastError();
    }
    return launch_spass_generic<float>(a, LB, st);
}

} // namespace gopf
