// elastic256.cuh -- the Khachaturyan term's two passes on 256-point axes (FP32), built from the
// register-resident 256-point engine of fast256.cuh.
//
// The elastic term (pf/homoLinElast.go:47-98) costs, per step, a forward transform of H(c), the
// multiplication by the elastic symbol b(k)/N and an inverse transform (the displacements and
// strains of elasticity/linearElasticity.go:33-83 folded into b(k)), then the pointwise factor
// s H'(c) (w - 2 e0 H(c)) and its forward transform.  On a 256^3 grid:
// - k_z256_elk: the last-axis part of the first chain (forward z, times b(k)/N, inverse z),
//   one read and one write of the array;
// - k_x256_elq: c2r of T (the field) and of w, the pointwise factor, r2c into the output,
//   two reads and one write.
#pragma once

namespace gopf {
namespace f256 {

// PM_ELASTIC_K along z: lines are 16 consecutive inner indices i0 + l of the S = KX*Y plane.
static __global__ void __launch_bounds__(NT, 3) k_z256_elk(const PassArgs<float> a)
{
    __shared__ __align__(16) float2 s_x[N * 16];
    __shared__ float2 s_tw[N];
    const int l = threadIdx.x & 15, r = threadIdx.x >> 4;
    const long long i0 = (long long)blockIdx.x * 16;
    const long long S = a.g.S;
    float2 *__restrict__ buf = a.buf[0];
    const float *__restrict__ bsym = a.bsym;
    float2 v[16];
    float b[16]; // the symbol's values are requested with the line, before the transform
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = buf[i0 + l + (long long)(r + 16 * i) * S];
#pragma unroll
    for (int i = 0; i < 16; ++i) b[i] = __ldg(&bsym[i0 + l + (long long)(r + 16 * i) * S]);
    load_twiddles(s_tw, a.tw);
    __syncthreads();
    auto at = [&](int x, int y) -> float2 & { return s_x[(x * 16 + y) * 16 + l]; };
    fft256<false>(v, r, s_tw, at);
    const float invN = (float)a.upd.invN;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const float bi = b[i] * invN;
        v[i] = make_float2(v[i].x * bi, v[i].y * bi);
    }
    fft256<true>(v, r, s_tw, at);
#pragma unroll
    for (int i = 0; i < 16; ++i) buf[i0 + l + (long long)(r + 16 * i) * S] = v[i];
}

// XP_ELASTIC_Q along x for 32 rows (16 row pairs) of one depth plane: out[0] = r2c(escale H'(c)
// (w - 2 e0 H(c))) with c = c2r(in), w = c2r(in2).  Thread t = r*16 + j (j = row pair).  Both
// [129][32] input tiles are requested at the start with 16-byte asynchronous copies, so the second
// one arrives while the first is transformed.
__host__ __device__ constexpr int x256_elq_smem_bytes() { return (N * 16 + 64 + 129 * XROWS) * 8; }

static __global__ void __launch_bounds__(NT, 2) k_x256_elq(const XPassArgs<float> a)
{
    extern __shared__ __align__(16) unsigned char elq_dsm[];
    float2 *s_x = reinterpret_cast<float2 *>(elq_dsm); // [N * 16 + 64]: tile of in, then the exchange slots
    float2 *s_w = s_x + N * 16 + 64;                    // [129][32]: tile of in2
    __shared__ float2 s_tw[N];
    const Geom &g = a.g;
    const int j = threadIdx.x & 15, r = threadIdx.x >> 4;
    const int y0 = blockIdx.x * XROWS;
    const long long sbase = (long long)blockIdx.y * g.S + y0;
    const int KX = g.KX, Y = g.Y;
    auto request = [&](const float2 *__restrict__ in, float2 *dst) {
        for (int e = threadIdx.x; e < KX * (XROWS / 2); e += NT) {
            const int kx = e >> 4, c = e & 15;
            fl::cp_async16(&dst[kx * XROWS + 2 * c], &in[sbase + (long long)kx * Y + 2 * c]);
        }
        fl::cp_async_commit();
    };
    request(a.in, s_x);
    request(a.in2, s_w);
    load_twiddles(s_tw, a.twX);
    auto at = [&](int x, int y) -> float2 & { return s_x[(x * 16 + y) * 16 + j]; };
    float2 c[16], w[16];
    fl::cp_async_wait<1>();
    __syncthreads();
    load_pair_line(s_x, r, j, c);
    __syncthreads(); // the tile becomes the exchange slots
    fft256<true>(c, r, s_tw, at);
    fl::cp_async_wait<0>();
    __syncthreads(); // s_w has arrived; the exchange slots are free again
    load_pair_line(s_w, r, j, w);
    fft256<true>(w, r, s_tw, at);
    __syncthreads();
    const float e0 = (float)a.e0, es = (float)a.escale;
#pragma unroll
    for (int i = 0; i < 16; ++i)
        c[i] = make_float2(elastic_q<float>(c[i].x, w[i].x, e0, es), elastic_q<float>(c[i].y, w[i].y, e0, es));
    x_fwd_store(c, a.out[0], r, j, s_tw, at, s_x, sbase, KX, Y);
}

} // namespace f256
} // namespace gopf
