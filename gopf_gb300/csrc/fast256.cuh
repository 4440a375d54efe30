// fast256.cuh -- register-resident 256-point passes for FP32 (sm_103a).
//
// Every pass of a 256-long axis uses one engine: n = 16*n1 + n2, k = k1 + 16*k2,
//   X[k1 + 16 k2] = sum_n2 W16^(n2 k2) * [ W256^(n2 k1) * sum_n1 x[16 n1 + n2] W16^(n1 k1) ].
// A thread owns one line's elements r + 16 i (i = 0..15): it transforms them
// with a radix-16 DFT in registers, applies the W256 twiddles, exchanges
// through shared memory once (element (a = r, b = k1) -> (a = n2, b = r)) and
// finishes with a second radix-16 DFT.  The result is again "r + 16 i", so
// the forward transform, the k-space update and the inverse transform chain
// in registers and global memory is touched once per element and direction.
//
// The x axis (real, 256 columns) packs two rows a, b as one complex line
// a + i b: its 256-point inverse transform of the Hermitian-extended half
// spectra gives both rows at once, and the forward transform of
// g(a) + i g(b) is separated with X_a(k) = (Z(k) + conj Z(-k))/2,
// X_b(k) = (Z(k) - conj Z(-k))/(2i).
#pragma once
#include "gopf_kernels.cuh"

namespace gopf {
namespace f256 {

constexpr int N = 256;
constexpr int R = 16;
constexpr int NT = 256; // threads per block: 16 lines x 16 radix positions

// 256-point FFT of the thread's v[i] = x[r + 16 i]; result v[i] = X[r + 16 i].
// at(a, b) is the shared-memory slot of element (a, b) of this thread's line.
template <bool INV, typename AT>
__device__ __forceinline__ void fft256(float2 (&v)[16], int r, const float2 *__restrict__ tw, AT &&at)
{
    dft16<INV>(v);
#pragma unroll
    for (int k1 = 1; k1 < 16; ++k1) {
        const float2 w = tw[k1 * 16 + r]; // W256^(r k1), laid out [k1][r]: conflict free
        v[k1] = INV ? cmulc(v[k1], w) : cmul(v[k1], w);
    }
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) at(r, k1) = v[k1];
    __syncthreads();
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) v[n2] = at(n2, r);
    dft16<INV>(v);
    __syncthreads(); // slots may be reused after return
}

// s_tw[k1*16 + r] = W256^(r*k1)
__device__ __forceinline__ void load_twiddles(float2 *s_tw, const float2 *__restrict__ tw)
{
    for (int t = threadIdx.x; t < N; t += blockDim.x) s_tw[t] = tw[(t & 15) * (t >> 4)];
}

__device__ __forceinline__ float fsqf(int i, int n)
{
    const int j = (2 * i > n) ? (n - i) : i;
    const float f = (float)j / (float)n;
    return f * f;
}

// k-space update of one element (pf/euler.go:32-34 with the term algebra of pf/rhsBuilder.go)
__device__ __forceinline__ float2 euler_update(float2 c0, const float2 *U, int ngrp, const UpdTable &u, float mk,
                                               const float *gsc, float dt, float *Lout)
{
    float2 nhat = make_float2(0.f, 0.f);
    for (int b = 0; b < ngrp; ++b) {
        float f = gsc[b];
        for (int q = 0; q < u.glap[b]; ++q) f *= mk;
        nhat.x += f * U[b].x;
        nhat.y += f * U[b].y;
    }
    float L = 0.f;
    for (int q = u.nimp - 1; q >= 0; --q) L = L * mk + (float)u.imp[q];
    *Lout = L;
    const float rden = 1.f / (1.f - dt * L);
    return make_float2((c0.x + dt * nhat.x) * rden, (c0.y + dt * nhat.y) * rden);
}

// ---------------------------------------------------------------------------
// z axis (strided), fused forward -> update -> inverse.  Lines are 16
// consecutive inner indices i0 + l of the S = KX*Y plane; thread t = r*16 + l.
// ---------------------------------------------------------------------------
template <int NG>
__global__ void __launch_bounds__(NT, 2) k_z256_fused(const PassArgs<float> a)
{
    __shared__ __align__(16) float2 s_x[N * 16];
    __shared__ float2 s_tw[N];
    __shared__ float s_fl[16], s_fz[N];
    const Geom &g = a.g;
    const int l = threadIdx.x & 15, r = threadIdx.x >> 4;
    const long long i0 = (long long)blockIdx.x * 16;
    const long long S = g.S;
    const float2 *__restrict__ U0 = a.buf[0];
    const int ngrp = (NG == 1) ? (a.upd.ngrp > 0 ? 1 : 0) : a.upd.ngrp;
    const bool init = (a.mode == PM_INIT);

    float2 v[16], sv[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = U0[i0 + l + (long long)(r + 16 * i) * S];
    if (!init) { // the state's loads overlap the forward transform
#pragma unroll
        for (int i = 0; i < 16; ++i) sv[i] = a.state[i0 + l + (long long)(r + 16 * i) * S];
    }
    load_twiddles(s_tw, a.tw);
    if (threadIdx.x < 16) {
        const long long q = i0 + threadIdx.x;
        const int kx = (int)(q / g.Y), y = (int)(q - (long long)kx * g.Y);
        const float fx = (float)kx / (float)g.X;
        s_fl[threadIdx.x] = fx * fx + fsqf(y, g.Y);
    }
    s_fz[threadIdx.x] = fsqf(threadIdx.x, g.Z);
    __syncthreads();
    auto at = [&](int x, int y) -> float2 & { return s_x[(x * 16 + y) * 16 + l]; };
    fft256<false>(v, r, s_tw, at);

    float2 w[NG == 1 ? 1 : 16];
    if (NG > 1 && ngrp > 1) {
        const float2 *__restrict__ U1 = a.buf[1];
#pragma unroll
        for (int i = 0; i < 16; ++i) w[i] = U1[i0 + l + (long long)(r + 16 * i) * S];
        fft256<false>(reinterpret_cast<float2(&)[16]>(w), r, s_tw, at);
    }

    const UpdTable &u = a.upd;
    const float dt = (float)u.dt, invN = (float)u.invN;
    float gsc[2];
    gsc[0] = (u.gscale[0]) ? (float)(*u.gscale[0]) : 1.f;
    gsc[1] = (ngrp > 1 && u.gscale[1]) ? (float)(*u.gscale[1]) : 1.f;
    const float fourpi2 = 39.478417604357434f;
    float2 *__restrict__ state = a.state;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int k = r + 16 * i;
        const long long gi = i0 + l + (long long)k * S;
        float2 cn;
        if (init) {
            cn = v[i];
        } else {
            const float mk = -fourpi2 * (s_fl[l] + s_fz[k]);
            float2 U[2] = {v[i], (NG > 1) ? w[NG > 1 ? i : 0] : v[i]};
            float L;
            cn = euler_update(sv[i], U, ngrp, u, mk, gsc, dt, &L);
        }
        state[gi] = cn;
        v[i] = make_float2(cn.x * invN, cn.y * invN);
    }
    fft256<true>(v, r, s_tw, at);
    float2 *__restrict__ T = a.tout;
#pragma unroll
    for (int i = 0; i < 16; ++i) T[i0 + l + (long long)(r + 16 * i) * S] = v[i];
}

// ---------------------------------------------------------------------------
// y axis (contiguous lines of 256), forward or inverse in place, or the 2D
// fused update.  Thread t = l*16 + r: a half-warp reads 128 contiguous bytes.
// Shared slots are swizzled so both exchange directions are conflict free.
// ---------------------------------------------------------------------------
template <int NG>
__global__ void __launch_bounds__(NT, NG == 1 ? 3 : 2) k_y256(const PassArgs<float> a)
{
    __shared__ __align__(16) float2 s_x[N * 16];
    __shared__ float2 s_tw[N];
    __shared__ float s_fl[16], s_fy[N];
    const Geom &g = a.g;
    const int r = threadIdx.x & 15, l = threadIdx.x >> 4;
    const long long nlines = (long long)g.Z * g.KX;
    const long long q = (long long)blockIdx.x * 16 + l;
    const bool valid = q < nlines;
    const bool fused = (a.mode == PM_FUSED || a.mode == PM_INIT);
    float2 *__restrict__ buf = fused ? a.buf[0] : a.buf[blockIdx.y];
    const float2 zero = make_float2(0.f, 0.f);

    float2 v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = valid ? buf[q * N + r + 16 * i] : zero;
    load_twiddles(s_tw, a.tw);
    if (fused) {
        if (threadIdx.x < 16) {
            const long long qq = (long long)blockIdx.x * 16 + threadIdx.x;
            float f2 = 0.f;
            if (qq < nlines) {
                const int zz = (int)(qq / g.KX), kx = (int)(qq - (long long)zz * g.KX);
                const float fx = (float)kx / (float)g.X;
                f2 = fx * fx + fsqf(zz, g.Z);
            }
            s_fl[threadIdx.x] = f2;
        }
        s_fy[threadIdx.x] = fsqf(threadIdx.x, g.Y);
    }
    __syncthreads();
    auto at = [&](int x, int y) -> float2 & { return s_x[l * N + x * 16 + ((x + y) & 15)]; };
    if (!fused) {
        if (a.mode == PM_FWD) fft256<false>(v, r, s_tw, at);
        else fft256<true>(v, r, s_tw, at);
#pragma unroll
        for (int i = 0; i < 16; ++i)
            if (valid) buf[q * N + r + 16 * i] = v[i];
        return;
    }
    fft256<false>(v, r, s_tw, at);
    const int ngrp = (NG == 1) ? (a.upd.ngrp > 0 ? 1 : 0) : a.upd.ngrp;
    float2 w[NG == 1 ? 1 : 16];
    if (NG > 1 && ngrp > 1) {
        const float2 *__restrict__ U1 = a.buf[1];
#pragma unroll
        for (int i = 0; i < 16; ++i) w[i] = valid ? U1[q * N + r + 16 * i] : zero;
        fft256<false>(reinterpret_cast<float2(&)[16]>(w), r, s_tw, at);
    }
    const UpdTable &u = a.upd;
    const float dt = (float)u.dt, invN = (float)u.invN;
    float gsc[2];
    gsc[0] = (u.gscale[0]) ? (float)(*u.gscale[0]) : 1.f;
    gsc[1] = (ngrp > 1 && u.gscale[1]) ? (float)(*u.gscale[1]) : 1.f;
    const float fourpi2 = 39.478417604357434f;
    float2 *__restrict__ state = a.state;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int k = r + 16 * i;
        const long long gi = q * N + k;
        float2 cn = zero;
        if (valid) {
            if (a.mode == PM_INIT) {
                cn = v[i];
            } else {
                const float mk = -fourpi2 * (s_fl[l] + s_fy[k]);
                float2 U[2] = {v[i], (NG > 1) ? w[NG > 1 ? i : 0] : v[i]};
                float L;
                cn = euler_update(state[gi], U, ngrp, u, mk, gsc, dt, &L);
            }
            state[gi] = cn;
        }
        v[i] = make_float2(cn.x * invN, cn.y * invN);
    }
    fft256<true>(v, r, s_tw, at);
    float2 *__restrict__ T = a.tout;
#pragma unroll
    for (int i = 0; i < 16; ++i)
        if (valid) T[q * N + r + 16 * i] = v[i];
}

// ---------------------------------------------------------------------------
// x axis: c2r -> pointwise polynomials -> r2c for 32 rows (16 row pairs) of
// one depth plane.  Thread t = r*16 + j (j = row pair).
// ---------------------------------------------------------------------------
constexpr int XROWS = 32;

template <typename F> __device__ __forceinline__ float polyf(const PwTable &pw, int grp, float c)
{
    const int d = pw.deg[grp];
    if (d >= 0) {
        float acc = (float)pw.dense[grp][d];
        for (int q = d - 1; q >= 0; --q) acc = acc * c + (float)pw.dense[grp][q];
        return acc;
    }
    float acc = 0.f;
    const int nt = pw.nterm[grp];
    for (int t = 0; t < nt; ++t) {
        const int p = pw.pw[grp][t];
        float x = 1.f;
        for (int i = 0; i < p; ++i) x *= c;
        acc += (float)pw.coef[grp][t] * x;
    }
    return acc;
}

// NG == 1: one output group, transformed in place; NG == 0: any number of groups
template <int NG>
__global__ void __launch_bounds__(NT, 2) k_x256(const XPassArgs<float> a)
{
    // spectral tile [129][32] during c2r input, then exchange slots [256][16]
    __shared__ __align__(16) float2 s_x[N * 16 + 64];
    __shared__ float2 s_tw[N];
    const Geom &g = a.g;
    const int j = threadIdx.x & 15, r = threadIdx.x >> 4;
    const int y0 = blockIdx.x * XROWS;
    const int z = blockIdx.y;
    const long long sbase = (long long)z * g.S + y0;
    const int KX = g.KX, Y = g.Y;
    load_twiddles(s_tw, a.twX);
    // stage the half spectrum of the 32 rows (kx = 0..128), 256 contiguous bytes per kx
    const float2 *__restrict__ in = a.in;
    for (int e = threadIdx.x; e < KX * XROWS; e += NT) {
        const int kx = e >> 5, y = e & 31;
        s_x[e] = in[sbase + (long long)kx * Y + y];
    }
    __syncthreads();
    // Hermitian extension, rows (2j, 2j+1) packed as a + i b
    float2 v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int k = r + 16 * i;
        if (k <= 128) {
            const float4 ab = *reinterpret_cast<const float4 *>(&s_x[k * XROWS + 2 * j]);
            v[i] = make_float2(ab.x - ab.w, ab.y + ab.z);
        } else {
            const float4 ab = *reinterpret_cast<const float4 *>(&s_x[(N - k) * XROWS + 2 * j]);
            v[i] = make_float2(ab.x + ab.w, -ab.y + ab.z);
        }
    }
    __syncthreads();
    auto at = [&](int x, int y) -> float2 & { return s_x[(x * 16 + y) * 16 + j]; };
    fft256<true>(v, r, s_tw, at);
    // v[i] = c(row 2j, col r + 16 i) + i c(row 2j+1, col r + 16 i)
    const int ng = (NG == 1) ? 1 : a.ngrp_out;
    for (int grp = 0; grp < ng; ++grp) {
        float2 wbuf[NG == 1 ? 1 : 16];
        float2(&w)[16] = (NG == 1) ? v : reinterpret_cast<float2(&)[16]>(wbuf);
#pragma unroll
        for (int i = 0; i < 16; ++i)
            w[i] = a.identity ? v[i] : make_float2(polyf<float>(a.pw, grp, v[i].x), polyf<float>(a.pw, grp, v[i].y));
        fft256<false>(w, r, s_tw, at);
        // w[i] = G(k = r + 16 i); separate the two rows' half spectra
#pragma unroll
        for (int i = 0; i < 16; ++i) s_x[(r + 16 * i) * 16 + j] = w[i];
        __syncthreads();
        float2 *__restrict__ out = a.out[grp];
        for (int e = threadIdx.x; e < KX * XROWS; e += NT) {
            const int kx = e >> 5, y = e & 31, jj = y >> 1;
            const float2 P = s_x[kx * 16 + jj];
            const float2 Q = s_x[((N - kx) & (N - 1)) * 16 + jj];
            float2 o;
            if ((y & 1) == 0) o = make_float2(0.5f * (P.x + Q.x), 0.5f * (P.y - Q.y));
            else o = make_float2(0.5f * (P.y + Q.y), 0.5f * (Q.x - P.x));
            out[sbase + (long long)kx * Y + y] = o;
        }
        __syncthreads();
    }
}

} // namespace f256
} // namespace gopf
