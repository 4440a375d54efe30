// fft_core.cuh -- shared-memory Stockham FFT engine for sm_103a.
//
// A tile holds LB independent lines of a transform of length n in shared
// memory with layout buf[pos * pitch + line].  Consecutive threads work on
// consecutive lines of the same position, so every shared-memory access of a
// half-warp (FP32) or quarter-warp (FP64) covers 128 contiguous bytes and is
// bank-conflict free, and tiles loaded from a strided axis of global memory
// land in shared memory without any shuffle.
//
// Transform convention (matches pfutil/fftWrap.go:26-39): forward uses
// exp(-2 pi i jk/n), backward exp(+2 pi i jk/n); both unnormalised.
//
// Stages are in-place: every thread first loads and transforms its
// butterflies into registers, the block synchronises, then all threads write.
// The per-thread register budget PERB bounds the butterflies per thread: the
// launch must provide blockDim.x >= LB * n / PERB threads.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "gopf_types.h"

namespace gopf {

template <typename V> struct RealOf;
template <> struct RealOf<float2> { typedef float type; };
template <> struct RealOf<double2> { typedef double type; };

template <typename V> __device__ __forceinline__ V cmk(typename RealOf<V>::type x, typename RealOf<V>::type y)
{
    V r;
    r.x = x;
    r.y = y;
    return r;
}
template <typename V> __device__ __forceinline__ V cadd(V a, V b) { return cmk<V>(a.x + b.x, a.y + b.y); }
template <typename V> __device__ __forceinline__ V csub(V a, V b) { return cmk<V>(a.x - b.x, a.y - b.y); }
template <typename V> __device__ __forceinline__ V cmul(V a, V b)
{
    return cmk<V>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename V> __device__ __forceinline__ V cmulc(V a, V b)
{
    return cmk<V>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename V> __device__ __forceinline__ V cconj(V a) { return cmk<V>(a.x, -a.y); }
template <typename V> __device__ __forceinline__ V cscale(V a, typename RealOf<V>::type s) { return cmk<V>(a.x * s, a.y * s); }
// multiply by -i (forward) or +i (inverse)
template <bool INV, typename V> __device__ __forceinline__ V cmul_mi(V a)
{
    return INV ? cmk<V>(-a.y, a.x) : cmk<V>(a.y, -a.x);
}

// ------------------------------------------------------------------
// Small DFTs in registers
// ------------------------------------------------------------------

template <bool INV, typename V> __device__ __forceinline__ void dft2(V &a, V &b)
{
    V t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <bool INV, typename V> __device__ __forceinline__ void dft4(V &v0, V &v1, V &v2, V &v3)
{
    V a0 = cadd(v0, v2), a1 = csub(v0, v2);
    V a2 = cadd(v1, v3), a3 = cmul_mi<INV>(csub(v1, v3));
    v0 = cadd(a0, a2);
    v2 = csub(a0, a2);
    v1 = cadd(a1, a3);
    v3 = csub(a1, a3);
}

template <bool INV, typename V> __device__ __forceinline__ void dft3(V &v0, V &v1, V &v2)
{
    typedef typename RealOf<V>::type R;
    const R s3 = (R)0.86602540378443864676372317075294;
    V t1 = cadd(v1, v2);
    V t2 = csub(v0, cscale(t1, (R)0.5));
    V d = csub(v1, v2);
    // forward: -i*s3*d ; inverse: +i*s3*d
    V t3 = cscale(cmul_mi<INV>(d), s3);
    v0 = cadd(v0, t1);
    v1 = cadd(t2, t3);
    v2 = csub(t2, t3);
}

// multiply by W_16^m (forward) or its conjugate (inverse)
template <int M, bool INV, typename V> __device__ __forceinline__ V tw16(V a)
{
    typedef typename RealOf<V>::type R;
    const R c1 = (R)0.92387953251128675613, s1 = (R)0.38268343236508977173, h = (R)0.70710678118654752440;
    R c, s; // W = c - i s (forward)
    switch (M & 15) {
    case 0: return a;
    case 1: c = c1; s = s1; break;
    case 2: c = h; s = h; break;
    case 3: c = s1; s = c1; break;
    case 4: return cmul_mi<INV>(a);
    case 6: c = -h; s = h; break;
    case 9: c = -c1; s = -s1; break;
    default: c = 1; s = 0; break;
    }
    if (INV) s = -s;
    return cmk<V>(a.x * c + a.y * s, a.y * c - a.x * s);
}

template <bool INV, typename V> __device__ __forceinline__ void dft8(V *v)
{
    typedef typename RealOf<V>::type R;
    const R h = (R)0.70710678118654752440;
    dft4<INV>(v[0], v[2], v[4], v[6]);
    dft4<INV>(v[1], v[3], v[5], v[7]);
    // O_k * W8^k
    V o1 = v[3], o2 = v[5], o3 = v[7];
    // W8^1 = h(1 - i) forward
    V w1 = INV ? cmk<V>(h * (o1.x - o1.y), h * (o1.y + o1.x)) : cmk<V>(h * (o1.x + o1.y), h * (o1.y - o1.x));
    V w2 = cmul_mi<INV>(o2);
    // W8^3 = h(-1 - i) forward
    V w3 = INV ? cmk<V>(h * (-o3.x - o3.y), h * (-o3.y + o3.x)) : cmk<V>(h * (-o3.x + o3.y), h * (-o3.y - o3.x));
    V e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6], o0 = v[1];
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, w1);
    v[5] = csub(e1, w1);
    v[2] = cadd(e2, w2);
    v[6] = csub(e2, w2);
    v[3] = cadd(e3, w3);
    v[7] = csub(e3, w3);
}

template <bool INV, typename V> __device__ __forceinline__ void dft16(V *v)
{
    // n = 4*n2 + n1 ; k = k1 + 4*k2
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) dft4<INV>(v[n1], v[4 + n1], v[8 + n1], v[12 + n1]);
    // now v[4*k1 + n1] holds A_{n1}[k1]; twiddle by W16^{n1*k1}
    v[5] = tw16<1, INV>(v[5]);
    v[6] = tw16<2, INV>(v[6]);
    v[7] = tw16<3, INV>(v[7]);
    v[9] = tw16<2, INV>(v[9]);
    v[10] = tw16<4, INV>(v[10]);
    v[11] = tw16<6, INV>(v[11]);
    v[13] = tw16<3, INV>(v[13]);
    v[14] = tw16<6, INV>(v[14]);
    v[15] = tw16<9, INV>(v[15]);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) dft4<INV>(v[4 * k1 + 0], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
    // v[4*k1 + k2] holds X[k1 + 4*k2]; transpose 4x4 into natural order
    V t[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) t[k1 + 4 * k2] = v[4 * k1 + k2];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = t[i];
}

// DFT of odd prime length P (5, 7) from its definition, pairing n and P - n:
//   X_0 = x_0 + sum_n t_n,   t_n = x_n + x_{P-n},   u_n = x_n - x_{P-n}   (n = 1 .. (P-1)/2)
//   a_m = x_0 + sum_n cos(2 pi n m / P) t_n,   b_m = sum_n sin(2 pi n m / P) u_n
//   X_m = a_m - i b_m,   X_{P-m} = a_m + i b_m   (forward; the inverse flips the sign of i)
template <int P> struct PrimeTab;
template <> struct PrimeTab<5> {
    // cos, sin of 2 pi q / 5, q = 0 .. 4
    __device__ static constexpr double c(int q)
    {
        return q == 0 ? 1.0 : (q == 1 || q == 4) ? 0.30901699437494742410 : -0.80901699437494742410;
    }
    __device__ static constexpr double s(int q)
    {
        return q == 0 ? 0.0 : q == 1 ? 0.95105651629515357212 : q == 2 ? 0.58778525229247312917
               : q == 3 ? -0.58778525229247312917 : -0.95105651629515357212;
    }
};
template <> struct PrimeTab<7> {
    __device__ static constexpr double c(int q)
    {
        return q == 0 ? 1.0 : (q == 1 || q == 6) ? 0.62348980185873353053
               : (q == 2 || q == 5) ? -0.22252093395631440429 : -0.90096886790241912624;
    }
    __device__ static constexpr double s(int q)
    {
        return q == 0 ? 0.0 : q == 1 ? 0.78183148246802980871 : q == 2 ? 0.97492791218182360702
               : q == 3 ? 0.43388373911755812048 : q == 4 ? -0.43388373911755812048
               : q == 5 ? -0.97492791218182360702 : -0.78183148246802980871;
    }
};

template <int P, bool INV, typename V> __device__ __forceinline__ void dft_prime(V *v)
{
    typedef typename RealOf<V>::type R;
    constexpr int H = (P - 1) / 2;
    V t[H], u[H];
#pragma unroll
    for (int n = 1; n <= H; ++n) {
        t[n - 1] = cadd(v[n], v[P - n]);
        u[n - 1] = csub(v[n], v[P - n]);
    }
    const V x0 = v[0];
    V sum = x0;
#pragma unroll
    for (int n = 0; n < H; ++n) sum = cadd(sum, t[n]);
    v[0] = sum;
#pragma unroll
    for (int m = 1; m <= H; ++m) {
        V a = x0, b = cmk<V>((R)0, (R)0);
#pragma unroll
        for (int n = 1; n <= H; ++n) {
            const R cc = (R)PrimeTab<P>::c((n * m) % P), ss = (R)PrimeTab<P>::s((n * m) % P);
            a = cadd(a, cscale(t[n - 1], cc));
            b = cadd(b, cscale(u[n - 1], ss));
        }
        const V ib = cmul_mi<INV>(b); // -i b forward, +i b inverse
        v[m] = cadd(a, ib);
        v[P - m] = csub(a, ib);
    }
}

template <int R, bool INV, typename V> __device__ __forceinline__ void dft(V *v)
{
    if (R == 2) dft2<INV>(v[0], v[1]);
    else if (R == 3) dft3<INV>(v[0], v[1], v[2]);
    else if (R == 4) dft4<INV>(v[0], v[1], v[2], v[3]);
    else if (R == 5) dft_prime<5, INV>(v);
    else if (R == 7) dft_prime<7, INV>(v);
    else if (R == 8) dft8<INV>(v);
    else if (R == 16) dft16<INV>(v);
}

// ------------------------------------------------------------------
// Plans
// ------------------------------------------------------------------

// ------------------------------------------------------------------
// One in-place Stockham stage over a tile
// ------------------------------------------------------------------

template <int RAD, bool INV, int LB, int PERB, typename V>
__device__ __noinline__ void fft_stage(V *buf, int pitch, int n, int ns, int nsmask, int twmul, const V *__restrict__ tw)
{
    constexpr int MAXPER = (PERB + RAD - 1) / RAD;
    constexpr int LBSH = (LB == 1) ? 0 : (LB == 2) ? 1 : (LB == 4) ? 2 : (LB == 8) ? 3 : (LB == 16) ? 4 : 5;
    const int m = n / RAD; // butterflies per line
    const int total = m * LB;
    const int nt = blockDim.x;
    V v[MAXPER][RAD];
#pragma unroll
    for (int p = 0; p < MAXPER; ++p) {
        const int bf = threadIdx.x + p * nt;
        if (bf < total) {
            const int line = bf & (LB - 1);
            const int j = bf >> LBSH;
#pragma unroll
            for (int r = 0; r < RAD; ++r) v[p][r] = buf[(j + r * m) * pitch + line];
            const int k = (nsmask >= 0) ? (j & nsmask) : (j % ns);
            if (k != 0) {
#pragma unroll
                for (int r = 1; r < RAD; ++r) {
                    V w = __ldg(&tw[r * k * twmul]);
                    v[p][r] = INV ? cmulc(v[p][r], w) : cmul(v[p][r], w);
                }
            }
            dft<RAD, INV>(v[p]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int p = 0; p < MAXPER; ++p) {
        const int bf = threadIdx.x + p * nt;
        if (bf < total) {
            const int line = bf & (LB - 1);
            const int j = bf >> LBSH;
            const int k = (nsmask >= 0) ? (j & nsmask) : (j % ns);
            const int base = (j - k) * RAD + k;
#pragma unroll
            for (int r = 0; r < RAD; ++r) buf[(base + r * ns) * pitch + line] = v[p][r];
        }
    }
    __syncthreads();
}

// Full transform of a tile (caller must __syncthreads() before, and the
// last stage ends with a barrier).
template <bool INV, int LB, int PERB, typename V>
__device__ __forceinline__ void fft_tile(V *buf, int pitch, const LinePlan &pl, const V *__restrict__ tw)
{
    for (int s = 0; s < pl.nst; ++s) {
        const int R = pl.rad[s];
        const int ns = pl.ns[s], msk = pl.nsmask[s], twm = pl.twmul[s];
        if (R == 16) fft_stage<16, INV, LB, PERB>(buf, pitch, pl.n, ns, msk, twm, tw);
        else if (R == 8) fft_stage<8, INV, LB, PERB>(buf, pitch, pl.n, ns, msk, twm, tw);
        else if (R == 4) fft_stage<4, INV, LB, PERB>(buf, pitch, pl.n, ns, msk, twm, tw);
        else if (R == 3) fft_stage<3, INV, LB, PERB>(buf, pitch, pl.n, ns, msk, twm, tw);
        else if (R == 5) fft_stage<5, INV, LB, PERB>(buf, pitch, pl.n, ns, msk, twm, tw);
        else if (R == 7) fft_stage<7, INV, LB, PERB>(buf, pitch, pl.n, ns, msk, twm, tw);
        else fft_stage<2, INV, LB, PERB>(buf, pitch, pl.n, ns, msk, twm, tw);
    }
}

// ------------------------------------------------------------------
// Compile-time plans: the same stages as a runtime LinePlan of length N (radix 3s first, then
// 2^(a mod 4), then 16s; the twiddle stride of a table of N * TWS entries), but with every
// index known to the compiler and each stage inlined.  Results are bitwise those of fft_tile.
// ------------------------------------------------------------------

template <int N> struct CtPlan {
    __host__ __device__ static constexpr int pow2(int n) { return (n % 2 == 0) ? 1 + pow2(n / 2) : 0; }
    __host__ __device__ static constexpr int odd(int n) { return (n % 2 == 0) ? odd(n / 2) : n; }
    __host__ __device__ static constexpr int pow3(int n) { return (n % 3 == 0) ? 1 + pow3(n / 3) : 0; }
    static constexpr int a = pow2(N), b = pow3(odd(N));
    static constexpr int nst = b + ((a % 4) ? 1 : 0) + a / 4;
    __host__ __device__ static constexpr int rad(int s) { return (s < b) ? 3 : ((a % 4) && s == b) ? (1 << (a % 4)) : 16; }
    __host__ __device__ static constexpr int ns(int s) { return (s == 0) ? 1 : ns(s - 1) * rad(s - 1); }
};

template <int RAD, bool INV, int LB, int PERB, int N, int NS, int TWM, typename V>
__device__ __forceinline__ void fft_stage_ct(V *buf, int pitch, const V *__restrict__ tw)
{
    constexpr int MAXPER = (PERB + RAD - 1) / RAD;
    constexpr int LBSH = (LB == 1) ? 0 : (LB == 2) ? 1 : (LB == 4) ? 2 : (LB == 8) ? 3 : (LB == 16) ? 4 : 5;
    constexpr int m = N / RAD;
    constexpr int total = m * LB;
    constexpr bool p2 = (NS & (NS - 1)) == 0;
    const int nt = blockDim.x;
    V v[MAXPER][RAD];
#pragma unroll
    for (int p = 0; p < MAXPER; ++p) {
        const int bf = threadIdx.x + p * nt;
        if (bf < total) {
            const int line = bf & (LB - 1);
            const int j = bf >> LBSH;
#pragma unroll
            for (int r = 0; r < RAD; ++r) v[p][r] = buf[(j + r * m) * pitch + line];
            const int k = p2 ? (j & (NS - 1)) : (j % NS);
            if (k != 0) {
#pragma unroll
                for (int r = 1; r < RAD; ++r) {
                    V w = __ldg(&tw[r * k * TWM]);
                    v[p][r] = INV ? cmulc(v[p][r], w) : cmul(v[p][r], w);
                }
            }
            dft<RAD, INV>(v[p]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int p = 0; p < MAXPER; ++p) {
        const int bf = threadIdx.x + p * nt;
        if (bf < total) {
            const int line = bf & (LB - 1);
            const int j = bf >> LBSH;
            const int k = p2 ? (j & (NS - 1)) : (j % NS);
            const int base = (j - k) * RAD + k;
#pragma unroll
            for (int r = 0; r < RAD; ++r) buf[(base + r * NS) * pitch + line] = v[p][r];
        }
    }
    __syncthreads();
}

template <bool INV, int LB, int PERB, int N, int TWS, int S = 0, typename V>
__device__ __forceinline__ void fft_tile_ct(V *buf, int pitch, const V *__restrict__ tw)
{
    if constexpr (S < CtPlan<N>::nst) {
        constexpr int R = CtPlan<N>::rad(S), NS = CtPlan<N>::ns(S);
        fft_stage_ct<R, INV, LB, PERB, N, NS, N * TWS / (NS * R)>(buf, pitch, tw);
        fft_tile_ct<INV, LB, PERB, N, TWS, S + 1>(buf, pitch, tw);
    }
}

// a tile transform with a compile-time plan when NCT > 0, else the runtime plan
template <bool INV, int LB, int PERB, int NCT, int TWS, typename V>
__device__ __forceinline__ void fft_tile_any(V *buf, int pitch, const LinePlan &pl, const V *__restrict__ tw)
{
    if constexpr (NCT > 0) fft_tile_ct<INV, LB, PERB, NCT, TWS>(buf, pitch, tw);
    else fft_tile<INV, LB, PERB>(buf, pitch, pl, tw);
}

} // namespace gopf
