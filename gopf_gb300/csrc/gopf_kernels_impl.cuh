// gopf_kernels.cu -- spectral semi-implicit step kernels (sm_103a).
//
// Per Euler step of a single-field model (pf/euler.go:16-47) the device runs
//   3D: x-pass (c2r -> pointwise terms -> r2c), y-pass forward,
//       z-pass (forward -> k-space update -> inverse), y-pass inverse;
//   2D: x-pass, y-pass (forward -> update -> inverse).
// The state is kept as c-hat; the real field only exists in shared memory
// inside the x-pass.  The pointwise derived fields of pf/util.go:57-64 and
// the explicit/implicit term algebra of pf/rhsBuilder.go:125-190 are applied
// in registers: explicit terms with the same LAP power are summed in real
// space before their common forward transform, and the implicit symbol
// sum_p a_p (-k^2)^p (pf/model.go:306-314, pf/diffOp.go:25-30) is evaluated
// per frequency in the last-axis pass.
#pragma once
#include "gopf_kernels.cuh"
#include "noise.cuh"
#include <math.h>

namespace gopf {

template <int LB> struct Log2 { static constexpr int v = (LB == 1) ? 0 : 1 + Log2<LB / 2>::v; };
template <> struct Log2<1> { static constexpr int v = 0; };

// Asynchronous global -> shared copy of one element (a 4-byte or 8-byte real, or an 8-byte or
// 16-byte complex value), or zeros when `valid` is false; the copy size is the element's own, so
// both addresses need only the element's alignment.  The copies of a tile are issued back to back
// and completed together by ga_wait() before the barrier that publishes the tile.
template <typename V> __device__ __forceinline__ void ga_copy(V *dst, const V *src, bool valid)
{
    static_assert(sizeof(V) == 4 || sizeof(V) == 8 || sizeof(V) == 16, "cp.async copies 4, 8 or 16 bytes");
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const int n = valid ? (int)sizeof(V) : 0;
    if constexpr (sizeof(V) == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(n) : "memory");
    else if constexpr (sizeof(V) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src), "r"(n) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(n) : "memory");
}
__device__ __forceinline__ void ga_wait()
{
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

template <typename R> __device__ __forceinline__ R poly_eval(const PwTable &pw, int grp, R c)
{
    const int d = pw.deg[grp];
    if (d >= 0) { // Horner; for a monomial c^p this is exactly the repeated product
        R acc = (R)pw.dense[grp][d];
        for (int q = d - 1; q >= 0; --q) acc = acc * c + (R)pw.dense[grp][q];
        return acc;
    }
    R acc = (R)0;
    const int nt = pw.nterm[grp];
    for (int t = 0; t < nt; ++t) {
        const int p = pw.pw[grp][t];
        R x = (R)1;
        for (int i = 0; i < p; ++i) x *= c;
        acc += (R)pw.coef[grp][t] * x;
    }
    return acc;
}

// A thread's share of a real-space block reduction (sum, sum of squares, min, max, non-finite count).
// FP32 values are summed in FP32 with Kahan compensation (the exact square's rounding residual
// included), their extremes and count kept in FP32 and integers, and converted once; FP64 values
// are summed plainly in FP64.  FP64 arithmetic runs at a small fraction of the FP32 rate on this GPU.
template <typename R> struct RedAcc {
    double s = 0.0, q = 0.0, mn = INFINITY, mx = -INFINITY, nf = 0.0;
    __device__ __forceinline__ void add(R v)
    {
        s += v;
        q += v * v;
        mn = fmin(mn, v);
        mx = fmax(mx, v);
        nf += isfinite(v) ? 0.0 : 1.0;
    }
    __device__ __forceinline__ void add_sum(R v) { s += v; }
    __device__ __forceinline__ void store(double *vals) const
    {
        vals[RED_SUM] = s;
        vals[RED_SUMSQ] = q;
        vals[RED_MIN] = mn;
        vals[RED_MAX] = mx;
        vals[RED_NONFINITE] = nf;
    }
};
template <> struct RedAcc<float> {
    float s = 0.f, sc = 0.f, q = 0.f, qc = 0.f, mn = INFINITY, mx = -INFINITY;
    int nf = 0;
    __device__ __forceinline__ static void kahan(float &acc, float &comp, float x)
    {
        const float y = x - comp;
        const float t = acc + y;
        comp = (t - acc) - y;
        acc = t;
    }
    __device__ __forceinline__ void add(float v)
    {
        kahan(s, sc, v);
        const float p = v * v;
        kahan(q, qc, p);
        qc -= fmaf(v, v, -p); // the square's rounding residual
        mn = fminf(mn, v);
        mx = fmaxf(mx, v);
        nf += isfinite(v) ? 0 : 1;
    }
    __device__ __forceinline__ void add_sum(float v) { kahan(s, sc, v); }
    __device__ __forceinline__ void store(double *vals) const
    {
        vals[RED_SUM] = (double)s - (double)sc;
        vals[RED_SUMSQ] = (double)q - (double)qc;
        vals[RED_MIN] = (double)mn;
        vals[RED_MAX] = (double)mx;
        vals[RED_NONFINITE] = (double)nf;
    }
};

// block-wide reduction of the first NS of the RED_SLOTS doubles into red[block] (the others are
// not written: nothing reads them)
template <int NS = RED_NONFINITE + 1>
__device__ __forceinline__ void block_reduce_store(double *vals, double *red, double *sh)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        double v = vals[s];
        for (int o = 16; o > 0; o >>= 1) {
            double w = __shfl_xor_sync(0xffffffffu, v, o);
            if (s == RED_MIN) v = fmin(v, w);
            else if (s == RED_MAX) v = fmax(v, w);
            else v += w;
        }
        if (lane == 0) sh[warp * RED_SLOTS + s] = v;
    }
    __syncthreads();
    if (threadIdx.x < NS) {
        const int s = threadIdx.x;
        double v = sh[s];
        for (int w = 1; w < nw; ++w) {
            double u = sh[w * RED_SLOTS + s];
            if (s == RED_MIN) v = fmin(v, u);
            else if (s == RED_MAX) v = fmax(v, u);
            else v += u;
        }
        red[(long long)(blockIdx.y * gridDim.x + blockIdx.x) * RED_SLOTS + s] = v;
    }
    __syncthreads();
}

// Load the spectral tile (z, all kx, LB rows from y0) of `in`, undo the r2c
// packing and inverse transform along x: on return A[m*LB + l] = (c[2m],
// c[2m+1]) of row y0 + l (times the transform's normalisation).
// Odd column counts X (no Nyquist column, KX = (X + 1)/2): rows 2p and 2p + 1 of the tile form one
// complex line c_2p + i c_2p+1 of length X, transformed by the length-X plan (planH holds it), so
// the tile holds A[x * LB/2 + p] = (c_2p[x], c_2p+1[x]).  The half spectra are Hermitian-extended
// into the line from a staging copy of the tile (stage: KX * LB elements after the block's tiles).
template <typename R, int LB, int PERB>
__device__ __forceinline__ void xload_c2r_odd(typename VecOf<R>::type *A, typename VecOf<R>::type *stage,
                                              const typename VecOf<R>::type *__restrict__ in, long long sbase,
                                              int nl, const Geom &g, const LinePlan &planX,
                                              const typename VecOf<R>::type *__restrict__ twX)
{
    typedef typename VecOf<R>::type V;
    constexpr int LBSH = Log2<LB>::v, P = LB / 2;
    const int X = g.X, KX = g.KX, Y = g.Y;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int e = tid; e < KX * LB; e += nt) {
        const int kx = e >> LBSH, l = e & (LB - 1);
        ga_copy(&stage[e], in + sbase + (long long)kx * Y + (l < nl ? l : 0), l < nl);
    }
    ga_wait();
    __syncthreads();
    for (int e = tid; e < KX * P; e += nt) {
        const int kx = e / P, q = e - kx * P;
        const V a = stage[kx * LB + 2 * q], b = stage[kx * LB + 2 * q + 1];
        A[kx * P + q] = cmk<V>(a.x - b.y, a.y + b.x); // A(k) + i B(k)
        if (kx > 0) A[(X - kx) * P + q] = cmk<V>(a.x + b.y, b.x - a.y); // conj A(k) + i conj B(k) at X - k
    }
    __syncthreads();
    fft_tile<true, P, PERB>(A, P, planX, twX);
}

template <typename R, int LB, int PERB, int NCT = 0>
__device__ __forceinline__ void xload_c2r(typename VecOf<R>::type *A, const typename VecOf<R>::type *__restrict__ in,
                                          long long sbase, int nl, const Geom &g, const LinePlan &planH,
                                          const typename VecOf<R>::type *__restrict__ twX,
                                          typename VecOf<R>::type *stage = nullptr)
{
    typedef typename VecOf<R>::type V;
    if constexpr (NCT == 0) {
        if (g.X & 1) {
            xload_c2r_odd<R, LB, PERB>(A, stage, in, sbase, nl, g, planH, twX);
            return;
        }
    }
    constexpr int LBSH = Log2<LB>::v;
    const int H = NCT ? NCT : g.H, KX = H + 1, Y = g.Y;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int e = tid; e < KX * LB; e += nt) {
        const int kx = e >> LBSH, l = e & (LB - 1);
        ga_copy(&A[e], in + sbase + (long long)kx * Y + (l < nl ? l : 0), l < nl);
    }
    ga_wait();
    __syncthreads();
    const int npair = H / 2 + 1;
    for (int e = tid; e < npair * LB; e += nt) {
        const int k = e >> LBSH, l = e & (LB - 1);
        if (k == 0) {
            const V a0 = A[l], b0 = A[H * LB + l];
            const V s = cadd(a0, cconj(b0)), d = csub(a0, cconj(b0));
            A[l] = cmk<V>(s.x - d.y, s.y + d.x);
        } else {
            const int k2 = H - k;
            const V av = A[k * LB + l], bv = A[k2 * LB + l];
            const V s = cadd(av, cconj(bv)), d = csub(av, cconj(bv));
            const V t = cmulc(d, __ldg(&twX[k]));
            const V zk = cmk<V>(s.x - t.y, s.y + t.x);
            if (k2 != k) {
                const V s2 = cadd(bv, cconj(av)), d2 = csub(bv, cconj(av));
                const V t2 = cmulc(d2, __ldg(&twX[k2]));
                A[k2 * LB + l] = cmk<V>(s2.x - t2.y, s2.y + t2.x);
            }
            A[k * LB + l] = zk;
        }
    }
    __syncthreads();
    fft_tile_any<true, LB, PERB, NCT, 2>(A, LB, planH, twX);
}

// r2c along x of the packed real rows in B (B[m*LB+l] = (g[2m], g[2m+1])) and
// store the half spectrum of the tile into out.
template <typename R, int LB, int PERB, int NCT = 0>
__device__ __forceinline__ void xr2c_store(typename VecOf<R>::type *B, typename VecOf<R>::type *__restrict__ out,
                                           long long sbase, int nl, const Geom &g, const LinePlan &planH,
                                           const typename VecOf<R>::type *__restrict__ twX)
{
    typedef typename VecOf<R>::type V;
    if constexpr (NCT == 0) {
        if (g.X & 1) { // odd X: forward transform of the row pairs, then X_a(k) = (Z(k) + conj Z(-k))/2
                       // (row 2p) and X_b(k) = (Z(k) - conj Z(-k))/(2i) (row 2p + 1)
            constexpr int P = LB / 2;
            const int X = g.X, KX = g.KX, Y = g.Y;
            fft_tile<false, P, PERB>(B, P, planH, twX);
            const R half = (R)0.5;
            for (int e = threadIdx.x; e < KX * LB; e += blockDim.x) {
                const int kx = e / LB, l = e - kx * LB, q = l >> 1;
                const V z = B[kx * P + q], w = B[(kx ? X - kx : 0) * P + q];
                const V o = (l & 1) ? cmk<V>(half * (z.y + w.y), half * (w.x - z.x))
                                    : cmk<V>(half * (z.x + w.x), half * (z.y - w.y));
                if (l < nl) out[sbase + (long long)kx * Y + l] = o;
            }
            __syncthreads();
            return;
        }
    }
    constexpr int LBSH = Log2<LB>::v;
    const int H = NCT ? NCT : g.H, KX = H + 1, Y = g.Y;
    const int tid = threadIdx.x, nt = blockDim.x;
    fft_tile_any<false, LB, PERB, NCT, 2>(B, LB, planH, twX);
    const int npair = H / 2 + 1;
    const R half = (R)0.5;
    for (int e = tid; e < npair * LB; e += nt) {
        const int k = e >> LBSH, l = e & (LB - 1);
        if (k == 0) {
            const V z0 = B[l];
            B[l] = cmk<V>(z0.x + z0.y, (R)0);
            B[H * LB + l] = cmk<V>(z0.x - z0.y, (R)0);
        } else {
            const int k2 = H - k;
            const V av = B[k * LB + l], bv = B[k2 * LB + l];
            const V s = cadd(av, cconj(bv)), d = csub(av, cconj(bv));
            const V t = cmul(__ldg(&twX[k]), d);
            const V xk = cmk<V>(half * (s.x + t.y), half * (s.y - t.x));
            if (k2 != k) {
                const V s2 = cadd(bv, cconj(av)), d2 = csub(bv, cconj(av));
                const V t2 = cmul(__ldg(&twX[k2]), d2);
                B[k2 * LB + l] = cmk<V>(half * (s2.x + t2.y), half * (s2.y - t2.x));
            }
            B[k * LB + l] = xk;
        }
    }
    __syncthreads();
    for (int e = tid; e < KX * LB; e += nt) {
        const int kx = e >> LBSH, l = e & (LB - 1);
        if (l < nl) out[sbase + (long long)kx * Y + l] = B[e];
    }
    __syncthreads();
}

// The Khachaturyan pointwise factor (pf/homoLinElast.go:10-17, 69-97):
// s * H'(c) * (w - 2 e0 H(c)) with H = 3c^2 - 2c^3, H' = 6c - 6c^2.
template <typename R> __device__ __forceinline__ R elastic_q(R c, R w, R e0, R s)
{
    const R Hc = (R)3 * c * c - (R)2 * c * c * c;
    const R dH = (R)6 * c - (R)6 * c * c;
    return s * (dH * (w - (R)2 * e0 * Hc));
}

// ------------------------------------------------------------------
// x-pass: c2r (or real load) -> pointwise -> r2c
// ------------------------------------------------------------------

// One x-pass tile: LB rows starting at row ty*LB of depth plane z.  MULTI: the multi-field
// program only (a separate instantiation, so the single-field kernels do not carry its registers).
// NCT > 0: the x transform has the compile-time length NCT (== g.H).
// Element e of a real-space tile holds two reals.  Even X: A[m*LB + l] = (c[2m], c[2m+1]) of row
// y0 + l; odd X: A[x*LB/2 + p] = (c[x] of row y0 + 2p, c[x] of row y0 + 2p + 1).  tile_rows gives the
// tile-relative rows of the two reals and tile_count the number of elements.
template <int LB> __device__ __forceinline__ void tile_rows(bool odd, int e, int &r0, int &r1)
{
    if (odd) {
        const int p = e & (LB / 2 - 1);
        r0 = 2 * p;
        r1 = 2 * p + 1;
    } else {
        r0 = r1 = e & (LB - 1);
    }
}

// One x-pass tile: LB rows starting at row ty*LB of depth plane z.  MULTI: the multi-field
// program only (a separate instantiation, so the single-field kernels do not carry its registers).
// NCT > 0: the x transform has the compile-time length NCT (== g.H).
template <typename R, int LB, int PERB, bool MULTI = false, int NCT = 0>
__device__ __forceinline__ void xpass_tile(const XPassArgs<R> &a, int ty, int z)
{
    typedef typename VecOf<R>::type V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int LBSH = Log2<LB>::v;
    const Geom &g = a.g;
    const bool odd = (NCT == 0) && (g.X & 1);
    const int H = NCT ? NCT : g.H, KX = H + 1, Y = g.Y;
    const int npos = odd ? g.X * (LB / 2) : H * LB; // tile elements (two reals each)
    V *A = reinterpret_cast<V *>(smem_raw);
    V *B = A + KX * LB;
    const int y0 = ty * LB;
    const int nl = min(LB, Y - y0);
    const long long sbase = (long long)z * g.S + y0;
    const int tid = threadIdx.x, nt = blockDim.x;
    const V zero = cmk<V>((R)0, (R)0);
    const V *__restrict__ twX = a.twX;
    (void)zero;
    (void)LBSH;

    // real rows of field rin into tile T (asynchronous copies; rows past the grid read as zeros)
    auto load_real = [&](V *T, const R *rin) {
        if (odd) {
            const R *base = rin + ((long long)z * Y + y0) * g.X;
            for (int e = tid; e < npos; e += nt) {
                const int x = e / (LB / 2), p = e - x * (LB / 2);
                R *d = reinterpret_cast<R *>(&T[e]);
                ga_copy(d, base + (long long)(2 * p < nl ? 2 * p : 0) * g.X + x, 2 * p < nl);
                ga_copy(d + 1, base + (long long)(2 * p + 1 < nl ? 2 * p + 1 : 0) * g.X + x, 2 * p + 1 < nl);
            }
        } else {
            const V *rin2 = reinterpret_cast<const V *>(rin) + ((long long)z * Y + y0) * H;
            for (int e = tid; e < LB * H; e += nt) {
                const int l = e / H, m = e - l * H;
                ga_copy(&T[m * LB + l], rin2 + (long long)(l < nl ? l : 0) * H + m, l < nl);
            }
        }
    };

    if constexpr (MULTI) {
        // one tile per field, then each group's monomials into the tile after them
        const MonoTable &mt = a.mono;
        const int tsz = KX * LB;
        V *Bm = A + mt.nin * tsz;
        V *stage = A + (mt.nin + 1) * tsz;
        if (a.in_mode == XIN_SPECTRAL) {
            for (int f = 0; f < mt.nin; ++f)
                xload_c2r<R, LB, PERB, NCT>(A + f * tsz, a.inF[f], sbase, nl, g, a.planH, twX, stage);
        } else { // real rows of every field (rinF[f])
            for (int f = 0; f < mt.nin; ++f) load_real(A + f * tsz, a.rinF[f]);
            ga_wait();
            __syncthreads();
        }
        if (a.red) { // FP64 block sum of one field's real-space values (the rows of this tile)
            double vals[RED_SLOTS];
#pragma unroll
            for (int s = 0; s < RED_SLOTS; ++s) vals[s] = 0.0;
            vals[RED_MIN] = INFINITY;
            vals[RED_MAX] = -INFINITY;
            const V *F = A + a.redfield * tsz;
            RedAcc<R> acc;
            for (int e = tid; e < npos; e += nt) {
                int r0, r1;
                tile_rows<LB>(odd, e, r0, r1);
                if (r0 < nl) acc.add_sum(F[e].x);
                if (r1 < nl) acc.add_sum(F[e].y);
            }
            double tmp[RED_SLOTS];
            acc.store(tmp);
            vals[RED_SUM] = tmp[RED_SUM];
            __shared__ double shredm[32 * RED_SLOTS];
            block_reduce_store<1>(vals, a.red, shredm); // the volume integral: the sum only
        }
        for (int grp = 0; grp < mt.ngrp; ++grp) {
            RedAcc<R> gacc;
            for (int e = tid; e < npos; e += nt) {
                R vx = (R)0, vy = (R)0;
                for (int m = 0; m < mt.nmono[grp]; ++m) {
                    R px = (R)mt.coef[grp][m], py = px;
                    for (int f = 0; f < mt.nin; ++f) {
                        const V c = A[f * tsz + e];
                        for (int i = 0; i < mt.pw[grp][m][f]; ++i) {
                            px *= c.x;
                            py *= c.y;
                        }
                    }
                    vx += px;
                    vy += py;
                }
                Bm[e] = cmk<V>(vx, vy);
                if (a.red2 && grp == a.redgrp) {
                    int r0, r1;
                    tile_rows<LB>(odd, e, r0, r1);
                    if (r0 < nl) gacc.add_sum(vx);
                    if (r1 < nl) gacc.add_sum(vy);
                }
            }
            if (a.red2 && grp == a.redgrp) {
                double vals[RED_SLOTS];
                gacc.store(vals);
                __shared__ double shredm2[32 * RED_SLOTS];
                block_reduce_store<1>(vals, a.red2, shredm2); // the indicator integral: the sum only
            }
            __syncthreads();
            xr2c_store<R, LB, PERB, NCT>(Bm, a.out[grp], sbase, nl, g, a.planH, twX);
        }
        return;
    }

    V *stage = A + 2 * KX * LB;
    if (a.in_mode == XIN_SPECTRAL) {
        xload_c2r<R, LB, PERB, NCT>(A, a.in, sbase, nl, g, a.planH, twX, stage);
    } else {
        load_real(A, a.rin);
        ga_wait();
        __syncthreads();
    }

    if (a.rout && a.program != XP_ADJ) {
        if (odd) {
            R *base = a.rout + ((long long)z * Y + y0) * g.X;
            for (int e = tid; e < npos; e += nt) {
                const int x = e / (LB / 2), p = e - x * (LB / 2);
                if (2 * p < nl) base[(long long)(2 * p) * g.X + x] = A[e].x;
                if (2 * p + 1 < nl) base[(long long)(2 * p + 1) * g.X + x] = A[e].y;
            }
        } else {
            V *rout2 = reinterpret_cast<V *>(a.rout) + ((long long)z * Y + y0) * H;
            for (int e = tid; e < LB * H; e += nt) {
                const int l = e / H, m = e - l * H;
                if (l < nl) rout2[(long long)l * H + m] = A[m * LB + l];
            }
        }
    }
    if (a.red) {
        RedAcc<R> acc;
        for (int e = tid; e < npos; e += nt) {
            int r0, r1;
            tile_rows<LB>(odd, e, r0, r1);
            const V c = A[e];
            if (r0 < nl) acc.add(c.x);
            if (r1 < nl) acc.add(c.y);
        }
        double vals[RED_SLOTS];
        acc.store(vals);
        __shared__ double shred[32 * RED_SLOTS];
        block_reduce_store(vals, a.red, shred);
    }

    if (a.program == XP_ADJ) {
        // A = mu (from in, above), B = nu = c2r(in2); c from the real rows of rin; lambda into rout
        // and into B, then r2c(lambda) into out[0]
        xload_c2r<R, LB, PERB, NCT>(B, a.in2, sbase, nl, g, a.planH, twX, stage);
        const R dtM = (R)a.adj_dtM;
        for (int e = tid; e < npos; e += nt) {
            R cx, cy;
            int r0, r1;
            tile_rows<LB>(odd, e, r0, r1);
            if (odd) {
                const int x = e / (LB / 2);
                const R *base = a.rin + ((long long)z * Y + y0) * g.X + x;
                cx = (r0 < nl) ? base[(long long)r0 * g.X] : (R)0;
                cy = (r1 < nl) ? base[(long long)r1 * g.X] : (R)0;
            } else {
                const int m = e >> LBSH;
                const V c2 = (r0 < nl) ? reinterpret_cast<const V *>(a.rin)[((long long)z * Y + y0 + r0) * H + m] : zero;
                cx = c2.x;
                cy = c2.y;
            }
            const V mu = A[e], nu = B[e];
            const V lam = cmk<V>(mu.x - dtM * ((R)3 * cx * cx - (R)1) * nu.x, mu.y - dtM * ((R)3 * cy * cy - (R)1) * nu.y);
            B[e] = lam;
            if (a.rout) {
                if (odd) {
                    const int x = e / (LB / 2);
                    R *base = a.rout + ((long long)z * Y + y0) * g.X + x;
                    if (r0 < nl) base[(long long)r0 * g.X] = lam.x;
                    if (r1 < nl) base[(long long)r1 * g.X] = lam.y;
                } else if (r0 < nl) {
                    reinterpret_cast<V *>(a.rout)[((long long)z * Y + y0 + r0) * H + (e >> LBSH)] = lam;
                }
            }
        }
        __syncthreads();
        xr2c_store<R, LB, PERB, NCT>(B, a.out[0], sbase, nl, g, a.planH, twX);
        return;
    }

    if (a.program == XP_ELASTIC_Q) {
        // w = c2r(in2) into B, then q into B, then r2c into out[0]
        xload_c2r<R, LB, PERB, NCT>(B, a.in2, sbase, nl, g, a.planH, twX, stage);
        const R e0 = (R)a.e0, es = (R)a.escale;
        for (int e = tid; e < npos; e += nt) {
            const V c = A[e], w = B[e];
            B[e] = cmk<V>(elastic_q<R>(c.x, w.x, e0, es), elastic_q<R>(c.y, w.y, e0, es));
        }
        __syncthreads();
        xr2c_store<R, LB, PERB, NCT>(B, a.out[0], sbase, nl, g, a.planH, twX);
        return;
    }

    for (int grp = 0; grp < a.ngrp_out; ++grp) {
        RedAcc<R> gacc;
        for (int e = tid; e < npos; e += nt) {
            const V c = A[e];
            const V r = a.identity ? c : cmk<V>(poly_eval<R>(a.pw, grp, c.x), poly_eval<R>(a.pw, grp, c.y));
            B[e] = r;
            if (a.red2 && grp == a.redgrp) {
                int r0, r1;
                tile_rows<LB>(odd, e, r0, r1);
                if (r0 < nl) gacc.add_sum(r.x);
                if (r1 < nl) gacc.add_sum(r.y);
            }
        }
        if (a.red2 && grp == a.redgrp) {
            double vals[RED_SLOTS];
            gacc.store(vals);
            __shared__ double shred2[32 * RED_SLOTS];
            block_reduce_store<1>(vals, a.red2, shred2); // the indicator integral: the sum only
        }
        __syncthreads();
        xr2c_store<R, LB, PERB, NCT>(B, a.out[grp], sbase, nl, g, a.planH, twX);
    }
}

// ------------------------------------------------------------------
// y (contiguous) and z (strided) passes
// ------------------------------------------------------------------

template <typename R> __device__ __forceinline__ R fsq_index(int i, int n)
{
    const int j = (2 * i > n) ? (n - i) : i;
    const R f = (R)j / (R)n;
    return f * f;
}

// Tile element mapping:
//   CONTIG : tile = LB consecutive lines q0.. of length n; global (q, p) = q*n + p
//            smem pitch LB+1, iteration line-major (a warp reads 32 consecutive p)
//   STRIDED: tile = LB consecutive inner indices i0.. of a pos-stride S array;
//            global (p, i) = p*S + i; smem pitch LB; iteration pos-major (LB
//            consecutive i form one 128-byte segment)
template <int LB, bool CONTIG, typename F> __device__ __forceinline__ void tile_foreach(int n, F &&f)
{
    constexpr int LBSH = Log2<LB>::v;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (CONTIG) {
        if (n >= nt) {
            for (int l = 0; l < LB; ++l)
#pragma unroll 4
                for (int p = tid; p < n; p += nt) f(p, l);
        } else {
            for (int e = tid; e < n * LB; e += nt) {
                const int l = e / n;
                f(e - l * n, l);
            }
        }
    } else {
#pragma unroll 4
        for (int e = tid; e < n * LB; e += nt) f(e >> LBSH, e & (LB - 1));
    }
}

// One tile of a y (CONTIG) or z pass: LB lines starting at line tile*LB;
// bsel selects the buffer in the FWD/INV modes.
// EXTRA = false compiles the plain Euler update only (no noise, modal filter, implicit user
// terms, RK4 stages or ImplicitEuler modes): the batched sweep, which rejects those, uses it.
// NCT > 0: the transform has the compile-time length NCT (== a.plan.n).
template <typename R, int LB, int PERB, bool CONTIG, bool EXTRA = true, int NCT = 0>
__device__ __forceinline__ void pass_tile(const PassArgs<R> &a, long long tix, int bsel)
{
    typedef typename VecOf<R>::type V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int pitch = CONTIG ? LB + 1 : LB;
    const Geom &g = a.g;
    const int n = NCT ? NCT : a.plan.n;
    const int tid = threadIdx.x, nt = blockDim.x;
    const long long nlines = CONTIG ? (long long)g.Z * g.KX : g.S;
    const long long l0 = tix * LB;
    const int nl = (int)min((long long)LB, nlines - l0);
    const long long pstride = CONTIG ? 1 : g.S;
    const long long lstride = CONTIG ? n : 1;
    const long long gbase = l0 * lstride;
    const int tile = n * pitch;
    V *sm = reinterpret_cast<V *>(smem_raw);
    const V zero = cmk<V>((R)0, (R)0);
    auto gidx = [&](int p, int l) -> long long { return gbase + p * pstride + l * lstride; };
    auto load = [&](V *dst, const V *__restrict__ src) { // completed by ga_wait() before the next barrier
        tile_foreach<LB, CONTIG>(n, [&](int p, int l) { ga_copy(&dst[p * pitch + l], src + gidx(p, l < nl ? l : 0), l < nl); });
    };
    auto store = [&](V *__restrict__ dst, const V *s) {
        tile_foreach<LB, CONTIG>(n, [&](int p, int l) {
            if (l < nl) dst[gidx(p, l)] = s[p * pitch + l];
        });
    };

    if (a.mode == PM_FWD || a.mode == PM_INV) {
        V *__restrict__ buf = a.buf[bsel];
        load(sm, buf);
        ga_wait();
        __syncthreads();
        if (a.mode == PM_FWD) fft_tile_any<false, LB, PERB, NCT, 1>(sm, pitch, a.plan, a.tw);
        else fft_tile_any<true, LB, PERB, NCT, 1>(sm, pitch, a.plan, a.tw);
        store(buf, sm);
        return;
    }

    if (a.mode == PM_ELASTIC_K) {
        // w-hat = b(k) * H-hat / N along the last axis, then back (pf/homoLinElast.go:53-75)
        V *__restrict__ buf = a.buf[0];
        load(sm, buf);
        ga_wait();
        __syncthreads();
        fft_tile_any<false, LB, PERB, NCT, 1>(sm, pitch, a.plan, a.tw);
        const R invN = (R)a.upd.invN;
        tile_foreach<LB, CONTIG>(n, [&](int p, int l) {
            if (l >= nl) return;
            const R b = a.bsym[gidx(p, l)] * invN;
            const V v = sm[p * pitch + l];
            sm[p * pitch + l] = cmk<V>(v.x * b, v.y * b);
        });
        __syncthreads();
        fft_tile_any<true, LB, PERB, NCT, 1>(sm, pitch, a.plan, a.tw);
        store(buf, sm);
        return;
    }

    // FUSED / INIT: all groups are loaded and forward transformed
    const int nb = a.nbuf;
    // squared frequencies: per line (the two axes the line does not run along)
    // and per position (the axis it runs along), in cycles/sample
    R *fline = reinterpret_cast<R *>(sm + nb * tile);
    R *fpos = fline + LB;
    for (int b = 0; b < nb; ++b) load(sm + b * tile, a.buf[b]);
    ga_wait();
    for (int l = tid; l < LB; l += nt) {
        const long long q = l0 + l;
        R f2 = (R)0;
        if (q < nlines) {
            if (CONTIG) { // line = (z, kx), position = y
                const int zz = (int)(q / g.KX), kx = (int)(q - (long long)zz * g.KX);
                const R fx = (R)kx / (R)g.X;
                f2 = fx * fx + fsq_index<R>(zz, g.Z);
            } else { // line = (kx, y), position = z
                const int kx = (int)(q / g.Y), y = (int)(q - (long long)kx * g.Y);
                const R fx = (R)kx / (R)g.X;
                f2 = fx * fx + fsq_index<R>(y, g.Y);
            }
        }
        fline[l] = f2;
    }
    for (int p = tid; p < n; p += nt) fpos[p] = CONTIG ? fsq_index<R>(p, g.Y) : fsq_index<R>(p, g.Z);
    __syncthreads();
    for (int b = 0; b < nb; ++b) fft_tile_any<false, LB, PERB, NCT, 1>(sm + b * tile, pitch, a.plan, a.tw);

    const UpdTable &u = a.upd;
    const R dt = (R)u.dt, invN = (R)u.invN;
    R gsc[GOPF_MAX_GROUPS];
#pragma unroll
    for (int b = 0; b < GOPF_MAX_GROUPS; ++b) gsc[b] = (b < u.ngrp && u.gscale[b]) ? (R)(*u.gscale[b]) : (R)1;
    const R fourpi2 = (R)39.478417604357434475337963999504; // 4 pi^2
    V *__restrict__ state = a.state;
    tile_foreach<LB, CONTIG>(n, [&](int p, int l) {
        if (l >= nl) return;
        const long long gi = gidx(p, l);
        V cn;
        if (a.mode == PM_INIT) {
            cn = sm[p * pitch + l];
        } else {
            const R mk = -fourpi2 * (fline[l] + fpos[p]); // -k^2
            V nhat = zero;
            for (int b = 0; b < u.ngrp; ++b) {
                R f = gsc[b];
                for (int q = 0; q < u.glap[b]; ++q) f *= mk;
                const V tv = sm[b * tile + p * pitch + l];
                nhat.x += f * tv.x;
                nhat.y += f * tv.y;
            }
            if (EXTRA && u.nxf) { // explicit terms in another field's c-hat (multi-field Euler)
                for (int q = 0; q < u.nxf; ++q) {
                    R f = (R)u.xf_coef[q];
                    for (int i = 0; i < u.xf_lap[q]; ++i) f *= mk;
                    const V sv = static_cast<const V *>(u.xf_src[q])[gi];
                    nhat.x += f * sv.x;
                    nhat.y += f * sv.y;
                }
            }
            if (EXTRA && u.nsrc) {
                // Source.Eval with the reference's Freq (row, col, depth; +1/2 kept at Nyquist).  The
                // real field carries the Hermitian part of exp(-2 pi i f.pos): on Nyquist components the
                // phase factor exp(-i pi pos_j) of k and -k averages to cos(pi sum pos_j)
                long long kx, yy, zz;
                if (CONTIG) {
                    const long long q = l0 + l;
                    zz = q / g.KX;
                    kx = q - zz * g.KX;
                    yy = p;
                } else {
                    const long long i = l0 + l;
                    kx = i / g.Y;
                    yy = i - kx * g.Y;
                    zz = p;
                }
                const double f[3] = {(double)((2 * yy > g.Y) ? yy - g.Y : yy) / (double)g.Y, (double)kx / (double)g.X,
                                     (double)((2 * zz > g.Z) ? zz - g.Z : zz) / (double)g.Z};
                const int dim = (g.Z > 1) ? 3 : 2;
                const unsigned long long st = *u.src_ctr;
                for (int sidx = 0; sidx < u.nsrc; ++sidx) {
                    const double amp = u.src_amp[(long long)u.src_row[sidx] * u.src_stride + (long long)st];
                    double ph = 0.0, npos = 0.0;
                    bool nyq = false;
                    for (int j = 0; j < dim; ++j) {
                        if (f[j] == 0.5) {
                            nyq = true;
                            npos += u.src_pos[sidx][j];
                        } else {
                            ph += f[j] * u.src_pos[sidx][j];
                        }
                    }
                    double sn, cs;
                    sincospi(2.0 * ph, &sn, &cs);
                    const double fac = nyq ? amp * cospi(npos) : amp;
                    nhat.x += (R)(fac * cs);
                    nhat.y -= (R)(fac * sn);
                }
            }
            if (EXTRA && u.noise.kind) {
                long long kx, yy, zz;
                if (CONTIG) {
                    const long long q = l0 + l;
                    zz = q / g.KX;
                    kx = q - zz * g.KX;
                    yy = p;
                } else {
                    const long long i = l0 + l;
                    kx = i / g.Y;
                    yy = i - kx * g.Y;
                    zz = p;
                }
                double nr, ni;
                noise_term(u.noise, g.X, g.Y, g.Z, kx, yy, zz, (double)mk, nr, ni);
                nhat.x += (R)nr;
                nhat.y += (R)ni;
            }
            // implicit symbol L = sum_p imp[p] (-k^2)^p
            R L = (R)0;
            for (int q = u.nimp - 1; q >= 0; --q) L = L * mk + (R)u.imp[q];
            // With a tensorial Hessian the reference's symbol differs between k and -k on Nyquist
            // lines (Freq keeps +1/2 for both).  Its complex field then carries an anti-Hermitian
            // part; the real field is the Hermitian part of its step, i.e. the update divides by
            // the mean of 1/(1 - a L(k)) and 1/(1 - a L(-k)).  Lm is L(-k); Lm == L elsewhere.
            R Lm = L;
            if (EXTRA && u.nxs) { // implicit user terms with a per-frequency symbol (XSym)
                long long kx, yy, zz;
                if (CONTIG) {
                    const long long q = l0 + l;
                    zz = q / g.KX;
                    kx = q - zz * g.KX;
                    yy = p;
                } else {
                    const long long i = l0 + l;
                    kx = i / g.Y;
                    yy = i - kx * g.Y;
                    zz = p;
                }
                const int dim = (g.Z > 1) ? 3 : 2;
                // the reference's Freq: row, col, depth in cycles per sample, +1/2 kept at Nyquist
                const double f[3] = {(double)((2 * yy > g.Y) ? yy - g.Y : yy) / (double)g.Y, (double)kx / (double)g.X,
                                     (double)((2 * zz > g.Z) ? zz - g.Z : zz) / (double)g.Z};
                double fm[3]; // Freq of the conjugate node
                for (int j = 0; j < 3; ++j) fm[j] = (f[j] == 0.5) ? 0.5 : -f[j];
                const double pi2 = 9.8696044010893586188344909998762; // pi^2
                auto xsym = [&](const XSym &x, const double *ff) -> double {
                    double sym = 0.0;
                    if (x.kind == 1) {
                        for (int j = 0; j < dim; ++j) sym += -4.0 * pi2 * ff[j] * ff[j] * x.K[j * x.dk + j];
                        for (int j = 0; j < dim; ++j)
                            for (int k2 = j + 1; k2 < dim; ++k2) sym += -8.0 * pi2 * ff[j] * ff[k2] * x.K[j * x.dk + k2];
                    } else {
                        double r2 = 0.0;
                        for (int j = 0; j < dim; ++j) r2 += ff[j] * ff[j];
                        const double fr = sqrt(r2), lo = x.threshold / 3.0;
                        double qv;
                        if (fr < lo) qv = 0.0;
                        else if (fr > x.threshold) qv = 1.0;
                        else {
                            const double xx = 1.5 * (fr - lo) / x.threshold;
                            qv = 2.0 * xx * xx - 3.0 * xx * xx * xx;
                        }
                        double pw = 1.0;
                        for (int q = 0; q < x.power; ++q) pw *= fr;
                        sym = -x.eps * qv * pw;
                    }
                    double lapf = 1.0;
                    for (int q = 0; q < x.lap; ++q) lapf *= (double)mk;
                    return x.coef * lapf * sym;
                };
                double addp = 0.0, addm = 0.0;
                for (int xi = 0; xi < u.nxs; ++xi) {
                    addp += xsym(u.xs[xi], f);
                    addm += xsym(u.xs[xi], fm);
                }
                Lm = L + (R)addm;
                L += (R)addp;
            }
            // (c, a) -> c / (1 - a L), or the mean over k and -k where their symbols differ
            auto implicit_div = [&](V c, R a) -> V {
                const R d = (R)1 - a * L;
                if (Lm == L) return cmk<V>(c.x / d, c.y / d);
                const R r = (R)0.5 * ((R)1 / d + (R)1 / ((R)1 - a * Lm));
                return cmk<V>(c.x * r, c.y * r);
            };
            const V c0 = state[gi];
            if (EXTRA && u.etd == 1) { // ImplicitEuler: the explicit RHS at the step's start
                a.rkF[gi] = nhat;
                sm[p * pitch + l] = zero;
                return;
            }
            if (EXTRA && u.etd == 2) {
                // ImplicitEuler residual (pf/implicitEuler.go:68-94): c_n e^(L dt) + integral of the RHS
                // interpolated linearly between N_n and N(x) (nonlinearIntegral, :151-162), in FP64
                const double Ld = (double)L, dtd = u.dt;
                const double f = exp(Ld * dtd);
                const V np = a.rkF[gi];
                double ir, ii;
                if (fabs(Ld) < 1e-5) {
                    ir = 0.5 * dtd * ((double)nhat.x + (double)np.x * f);
                    ii = 0.5 * dtd * ((double)nhat.y + (double)np.y * f);
                } else {
                    const double c1 = (f - 1.0) / Ld, c2 = (f - Ld * dtd - 1.0) / (Ld * Ld);
                    const double br = ((double)nhat.x - (double)np.x) / dtd, bi = ((double)nhat.y - (double)np.y) / dtd;
                    ir = (double)np.x * c1 + br * c2;
                    ii = (double)np.y * c1 + bi * c2;
                }
                const V xh = sm[u.ngrp * tile + p * pitch + l];
                const double rr = (double)xh.x - ((double)c0.x * f + ir);
                const double ri = (double)xh.y - ((double)c0.y * f + ii);
                sm[p * pitch + l] = cmk<V>((R)(rr * u.invN), (R)(ri * u.invN));
                return;
            }
            if (EXTRA && u.rk_stage > 0) {
                const R af = (R)u.rk_afin;
                V F = (u.rk_stage == 1) ? c0 : a.rkF[gi];
                F = cmk<V>(F.x + af * nhat.x, F.y + af * nhat.y);
                if (u.rk_stage < 4) {
                    a.rkF[gi] = F;
                    const R ay = (R)u.rk_ay;
                    const V nx = implicit_div(cmk<V>(c0.x + ay * nhat.x, c0.y + ay * nhat.y), (R)u.rk_fden);
                    sm[p * pitch + l] = cmk<V>(nx.x * invN, nx.y * invN);
                    return; // the state changes only in the last stage
                }
                cn = implicit_div(F, dt);
            } else {
                cn = implicit_div(cmk<V>(c0.x + dt * nhat.x, c0.y + dt * nhat.y), dt);
            }
            if (EXTRA && u.filt) { // ApplyModalFilter (pf/util.go:125-132), Vandeven.Eval (pf/vandeven.go:30-40)
                const R *__restrict__ tab = static_cast<const R *>(u.filt);
                const int nf = u.nfilt;
                const R x = sqrt(fline[l] + fpos[p]) * (R)0.63661977236758134307553505349006;
                const R nn = (R)(nf - 1);
                const int idx = (int)(x * nn);
                R sg;
                if (idx >= nf - 1) {
                    sg = tab[nf - 1];
                } else {
                    const R dx = (R)1 / nn;
                    sg = tab[idx] + (x - (R)idx * dx) * (tab[idx + 1] - tab[idx]) / dx;
                }
                cn = cmk<V>(cn.x * sg, cn.y * sg);
            }
        }
        state[gi] = cn;
        sm[p * pitch + l] = cmk<V>(cn.x * invN, cn.y * invN);
    });
    __syncthreads();
    fft_tile_any<true, LB, PERB, NCT, 1>(sm, pitch, a.plan, a.tw);
    store(a.tout, sm);
}

template <typename R, int LB, int PERB, bool MULTI = false>
__global__ void __launch_bounds__(256, (sizeof(R) == 4 ? 3 : 2)) k_xpass(const XPassArgs<R> a)
{
    xpass_tile<R, LB, PERB, MULTI>(a, blockIdx.x, blockIdx.y);
}

template <typename R, int LB, int PERB, bool CONTIG>
__global__ void __launch_bounds__(256, (sizeof(R) == 4 ? 3 : 2)) k_pass(const PassArgs<R> a)
{
    pass_tile<R, LB, PERB, CONTIG>(a, blockIdx.x, blockIdx.y);
}

// ------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------

template <typename R> constexpr int perb() { return 16; }

// Threads per block: enough for the per-thread register budget of the
// Stockham stages (blockDim >= LB*n/PERB), at most the 256 of __launch_bounds__.
static int pick_threads(long long work_items, int perb_)
{
    long long need = (work_items + perb_ - 1) / perb_;
    int nt = 128;
    while (nt < need && nt < 256) nt *= 2;
    return nt;
}
static bool threads_ok(long long work_items, int perb_) { return (work_items + perb_ - 1) / perb_ <= 256; }

// Raise a kernel's dynamic shared-memory limit only when a launch needs more
// than before, so launches recorded into a CUDA graph set no attributes.
// (Per device; the library drives one device per process in practice.)
template <typename K> static cudaError_t ensure_smem(K kern, int smem, int &have)
{
    if (smem <= have) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) have = smem;
    return e;
}

inline int xpass_smem_bytes(const Geom &g, int LB, int vbytes, int ntiles) { return ntiles * g.KX * LB * vbytes; }
inline int cpass_smem_bytes(const Geom &g, int n, int LB, int nbuf, int vbytes) { return nbuf * n * (LB + 1) * vbytes; }
inline int spass_smem_bytes(const Geom &g, int n, int LB, int nbuf, int vbytes) { return nbuf * n * LB * vbytes; }

template <typename R, int LB> static cudaError_t launch_xpass_lb(const XPassArgs<R> &a, cudaStream_t st)
{
    typedef typename VecOf<R>::type V;
    const bool multi = (a.program == XP_MULTI);
    const bool odd = (a.g.X & 1) != 0; // odd column count: a staging tile and length-X row-pair lines
    const int smem = xpass_smem_bytes(a.g, LB, sizeof(V), (multi ? a.mono.nin + 1 : 2) + (odd ? 1 : 0));
    const long long work = odd ? (long long)(LB / 2) * a.g.X : (long long)LB * a.g.H;
    if (!threads_ok(work, perb<R>())) return cudaErrorInvalidConfiguration;
    const int nt = pick_threads(work, perb<R>());
    dim3 grid((a.g.Y + LB - 1) / LB, a.g.Z);
    cudaError_t e;
    if (multi) {
        auto kern = k_xpass<R, LB, perb<R>(), true>;
        static int have = 48 * 1024; // one per kernel instantiation
        if ((e = ensure_smem(kern, smem, have)) != cudaSuccess) return e;
        kern<<<grid, nt, smem, st>>>(a);
    } else {
        auto kern = k_xpass<R, LB, perb<R>(), false>;
        static int have = 48 * 1024;
        if ((e = ensure_smem(kern, smem, have)) != cudaSuccess) return e;
        kern<<<grid, nt, smem, st>>>(a);
    }
    return cudaGetLastError();
}

template <typename R> static cudaError_t launch_xpass_generic(const XPassArgs<R> &a, int LB, cudaStream_t st)
{
    if constexpr (sizeof(R) == 4) {
        if (LB == 16) return launch_xpass_lb<R, 16>(a, st);
        if (LB == 8) return launch_xpass_lb<R, 8>(a, st);
        if (LB == 4) return launch_xpass_lb<R, 4>(a, st);
    } else {
        if (LB == 8) return launch_xpass_lb<R, 8>(a, st);
        if (LB == 4) return launch_xpass_lb<R, 4>(a, st);
    }
    return cudaErrorInvalidValue;
}

template <typename R, int LB, bool CONTIG> static cudaError_t launch_pass_lb(const PassArgs<R> &a, cudaStream_t st)
{
    typedef typename VecOf<R>::type V;
    const int n = a.plan.n;
    const bool fused = (a.mode == PM_FUSED || a.mode == PM_INIT);
    const int nsm = fused ? a.nbuf : 1;
    int smem = CONTIG ? cpass_smem_bytes(a.g, n, LB, nsm, sizeof(V)) : spass_smem_bytes(a.g, n, LB, nsm, sizeof(V));
    if (fused) smem += (LB + n) * (int)sizeof(R); // frequency tables
    auto kern = k_pass<R, LB, perb<R>(), CONTIG>;
    static int have = 48 * 1024; // one per kernel instantiation
    cudaError_t e = ensure_smem(kern, smem, have);
    if (e != cudaSuccess) return e;
    if (!threads_ok((long long)LB * n, perb<R>())) return cudaErrorInvalidConfiguration;
    const int nt = pick_threads((long long)LB * n, perb<R>());
    const long long nlines = CONTIG ? (long long)a.g.Z * a.g.KX : a.g.S;
    dim3 grid((unsigned)((nlines + LB - 1) / LB), fused ? 1 : a.nbuf);
    kern<<<grid, nt, smem, st>>>(a);
    return cudaGetLastError();
}

template <typename R> static cudaError_t launch_cpass_generic(const PassArgs<R> &a, int LB, cudaStream_t st)
{
    if constexpr (sizeof(R) == 4) {
        if (LB == 16) return launch_pass_lb<R, 16, true>(a, st);
        if (LB == 8) return launch_pass_lb<R, 8, true>(a, st);
        if (LB == 4) return launch_pass_lb<R, 4, true>(a, st);
    } else {
        if (LB == 8) return launch_pass_lb<R, 8, true>(a, st);
        if (LB == 4) return launch_pass_lb<R, 4, true>(a, st);
    }
    return cudaErrorInvalidValue;
}

template <typename R> static cudaError_t launch_spass_generic(const PassArgs<R> &a, int LB, cudaStream_t st)
{
    if constexpr (sizeof(R) == 4) {
        if (LB == 16) return launch_pass_lb<R, 16, false>(a, st);
        if (LB == 8) return launch_pass_lb<R, 8, false>(a, st);
        if (LB == 4) return launch_pass_lb<R, 4, false>(a, st);
    } else {
        if (LB == 8) return launch_pass_lb<R, 8, false>(a, st);
        if (LB == 4) return launch_pass_lb<R, 4, false>(a, st);
    }
    return cudaErrorInvalidValue;
}

} // namespace gopf
