// x256_io.cuh -- 256-column x passes that start or end in real space (FP32).
//
// k_x256_c2r: half spectrum -> real rows (download, the Newton residual, the
//   adjoint's state readout) and/or the FP64 block sums behind gopf_reduce.
// k_x256_r2c: real rows -> r2c of the pointwise groups (upload, the Newton
//   residual's FFT(x) and FFT(g(x))).
// Both use the register-resident 256-point engine of fast256.cuh on 32 rows
// (16 packed row pairs) of one depth plane per block.  Real rows move
// through a [32][257]-float shared tile: the odd pitch makes both the
// row-pair accesses of the transform and the row-contiguous global accesses
// conflict free, and every global access of a warp is 128 contiguous bytes.
#pragma once
#include "fast256.cuh"
#include "gopf_kernels_impl.cuh"

namespace gopf {
namespace f256 {

constexpr int XR_PITCH = N + 1;

__host__ __device__ constexpr int x256_io_smem_bytes()
{
    return 128 + XT_XCH_BYTES + XT_TILE_BYTES + N * 8 + GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1) * 4 + 16;
}

// half spectrum -> real rows (a.rout, optional) and FP64 partial sums (a.red, optional; one
// [RED_SLOTS] row per block, blocks ordered blockIdx.y * gridDim.x + blockIdx.x)
__global__ void __launch_bounds__(NT, 3) k_x256_c2r(const XPassArgs<float> a, const __grid_constant__ CUtensorMap mIn)
{
    extern __shared__ unsigned char c_dsm[];
    unsigned char *base = c_dsm + ((128u - (smem_u32(c_dsm) & 127u)) & 127u);
    float2 *s_x = reinterpret_cast<float2 *>(base);                           // input tile, then exchange slots
    float *s_r = reinterpret_cast<float *>(base + XT_XCH_BYTES);              // real rows [32][257]
    float2 *s_tw = reinterpret_cast<float2 *>(base + XT_XCH_BYTES + XT_TILE_BYTES);
    uint64_t *bar = reinterpret_cast<uint64_t *>(s_tw + N);
    int *s_ok = reinterpret_cast<int *>(bar + 1);

    const Geom &g = a.g;
    const int tid = threadIdx.x;
    const int j = tid & 15, r = tid >> 4;
    const int y0 = blockIdx.x * XROWS;
    const int z = blockIdx.y;
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        mbar_arrive_expect_tx(bar, (uint32_t)XT_TILE_BYTES);
        tma_load_3d(s_x, &mIn, y0, 0, z, bar);
    }
    load_twiddles(s_tw, a.twX);
    if (tid == 0) *s_ok = tma_wait_or_flag(bar, 0, a.status) ? 1 : 0;
    __syncthreads();
    if (!*s_ok) return;

    float2 v[16];
    load_pair_line(s_x, r, j, v);
    __syncthreads();
    auto at = [&](int x, int y) -> float2 & { return s_x[(x * 16 + y) * 16 + j]; };
    fft256<true>(v, r, s_tw, at);
    // v[i] = c(row 2j, col r + 16 i) + i c(row 2j+1, col r + 16 i)

    if (a.red) {
        // Per thread in FP32 with compensation (GB300's FP64 rate is 1/64 of FP32): Kahan sums of the
        // values and of their exact squares (v*v plus its FMA residual); FP64 from the block level on.
        float s = 0.f, sc = 0.f, q = 0.f, qc = 0.f, mn = INFINITY, mx = -INFINITY;
        int nf = 0;
        auto kahan = [](float &acc, float &comp, float x) {
            const float y = x - comp;
            const float t = acc + y;
            comp = (t - acc) - y;
            acc = t;
        };
#pragma unroll
        for (int i = 0; i < 16; ++i) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const float c = h ? v[i].y : v[i].x;
                kahan(s, sc, c);
                const float p = c * c;
                kahan(q, qc, p);
                qc -= fmaf(c, c, -p); // the square's rounding residual
                mn = fminf(mn, c);
                mx = fmaxf(mx, c);
                nf += isfinite(c) ? 0 : 1;
            }
        }
        double vals[RED_SLOTS];
#pragma unroll
        for (int k = 0; k < RED_SLOTS; ++k) vals[k] = 0.0;
        vals[RED_SUM] = (double)s - (double)sc;
        vals[RED_SUMSQ] = (double)q - (double)qc;
        __shared__ double shred[8 * RED_SLOTS];
        block_reduce_store<RED_SUMSQ + 1>(vals, a.red, shred); // the two sums in FP64
        // the extremes in FP32 and the count in integers (exact), converted once per block
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            nf += __shfl_xor_sync(0xffffffffu, nf, o);
        }
        __shared__ float shmm[2][NT / 32];
        __shared__ int shnf[NT / 32];
        if ((tid & 31) == 0) {
            shmm[0][tid >> 5] = mn;
            shmm[1][tid >> 5] = mx;
            shnf[tid >> 5] = nf;
        }
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < NT / 32; ++w) {
                shmm[0][0] = fminf(shmm[0][0], shmm[0][w]);
                shmm[1][0] = fmaxf(shmm[1][0], shmm[1][w]);
                shnf[0] += shnf[w];
            }
            double *row = a.red + (long long)(blockIdx.y * gridDim.x + blockIdx.x) * RED_SLOTS;
            row[RED_MIN] = (double)shmm[0][0];
            row[RED_MAX] = (double)shmm[1][0];
            row[RED_NONFINITE] = (double)shnf[0];
        }
    }
    if (a.rout) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int k = r + 16 * i;
            s_r[(2 * j) * XR_PITCH + k] = v[i].x;
            s_r[(2 * j + 1) * XR_PITCH + k] = v[i].y;
        }
        __syncthreads();
        float *__restrict__ out = a.rout + ((long long)z * g.Y + y0) * N;
#pragma unroll 8
        for (int q = 0; q < XROWS; ++q) out[q * N + tid] = s_r[q * XR_PITCH + tid];
    }
}

// real rows -> r2c of the pointwise groups into a.out[grp] (a.identity: group 0 is the field itself)
template <int NG>
__global__ void __launch_bounds__(NT, 3)
    k_x256_r2c(const XPassArgs<float> a, const __grid_constant__ CUtensorMap mO0, const __grid_constant__ CUtensorMap mO1,
               const __grid_constant__ CUtensorMap mO2, const __grid_constant__ CUtensorMap mO3)
{
    extern __shared__ unsigned char r_dsm[];
    unsigned char *base = r_dsm + ((128u - (smem_u32(r_dsm) & 127u)) & 127u);
    float2 *s_x = reinterpret_cast<float2 *>(base);                        // real rows, then exchange slots
    float2 *s_o = reinterpret_cast<float2 *>(base + XT_XCH_BYTES);         // output tile [129][32]
    float2 *s_tw = reinterpret_cast<float2 *>(base + XT_XCH_BYTES + XT_TILE_BYTES);
    float *s_poly = reinterpret_cast<float *>(s_tw + N);
    float *s_r = reinterpret_cast<float *>(s_x);

    const Geom &g = a.g;
    const int tid = threadIdx.x;
    const int j = tid & 15, r = tid >> 4;
    const int y0 = blockIdx.x * XROWS;
    const int z = blockIdx.y;
    const float *__restrict__ in = a.rin + ((long long)z * g.Y + y0) * N;
#pragma unroll 8
    for (int q = 0; q < XROWS; ++q) s_r[q * XR_PITCH + tid] = in[q * N + tid];
    for (int t = tid; t < GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1); t += NT)
        s_poly[t] = (float)a.pw.dense[t / (GOPF_MAX_DEG + 1)][t % (GOPF_MAX_DEG + 1)];
    load_twiddles(s_tw, a.twX);
    __syncthreads();
    float2 v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int k = r + 16 * i;
        v[i] = make_float2(s_r[(2 * j) * XR_PITCH + k], s_r[(2 * j + 1) * XR_PITCH + k]);
    }
    __syncthreads();
    auto at = [&](int x, int y) -> float2 & { return s_x[(x * 16 + y) * 16 + j]; };

    const int ng = (NG == 1) ? 1 : a.ngrp_out;
    for (int grp = 0; grp < ng; ++grp) {
        float2 w[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) w[i] = v[i];
        if (!(a.identity && grp == 0)) apply_poly(w, a, grp, s_poly + grp * (GOPF_MAX_DEG + 1));
        fft256<false>(w, r, s_tw, at);
#pragma unroll
        for (int i = 0; i < 16; ++i) s_x[(r + 16 * i) * 16 + j] = w[i];
        if (grp > 0 && tid == 0) bulk_wait_read_all(); // the previous group's store has read s_o
        __syncthreads();
        separate_pairs(s_x, s_o, tid);
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            const CUtensorMap *m = (grp == 0) ? &mO0 : (grp == 1) ? &mO1 : (grp == 2) ? &mO2 : &mO3;
            tma_store_3d(m, y0, 0, z, s_o);
            bulk_commit();
        }
    }
    if (tid == 0) bulk_wait_read_all();
}

} // namespace f256
} // namespace gopf
