// fastline.cuh -- register-resident FP32 line transforms of length L = 16 T (T = 16, 24, 32, 48,
// 64: L = 256, 384, 512, 768, 1024) for the batched 2D sweep.
//
// A line is held by T threads, 16 values each.  Forward transform (decimation in time):
//   A: thread r holds x[r + T i] (i < 16): radix-16 DFT over i in registers, twiddle W_L^(r k1)
//      -> Y[r][k1]; exchange through shared memory;
//   B: X[k1 + 16 k2] = sum_r W_T^(r k2) Y[r][k1], a DFT of length T = P U per k1.
//      U = 1, 2, 4 (T = 16, 32, 64): r = U s + u, a radix-16 DFT over s in registers, twiddle
//      W_T^(u c), then a radix-U DFT across the U threads of a column by warp shuffles.
//      U = 3 (T = 48, 24): r = s + P t, k2 = 3 c + d; the thread computing output d forms the
//      radix-3 over t while reading its column from the exchange, then twiddles W_T^(s d) and
//      runs a radix-P DFT over s (P = 16, or two radix-8 DFTs for two columns when T = 24).
// The output stays distributed ("B layout": a thread holds X[k] for one column and one d),
// which is where the k-space update happens.  The inverse transform runs the
// same steps in reverse order with conjugate twiddles (decimation in frequency), so it takes the
// B layout and ends in the A layout x[r + T i] that was loaded: the update pass reads and writes
// every line in place, coalesced.  L = 256 (T = 16, U = 1) is the engine of fast256.cuh.
//
// The x pass packs two real rows a, b as one complex line a + i b of L columns (Hermitian
// extension of their half spectra on input, separation of the two spectra on output), so both
// passes of a 2D step use the same engine with L = the side of the instance.
#pragma once
#include "fast256.cuh"

namespace gopf {
namespace fl {

using f256::pdft16;

template <int L, int NB = 0> struct Geo {
    static constexpr int T = L / 16;                 // threads per line
    static constexpr bool P8 = (T == 24);            // second stage: two radix-8 DFTs per thread
    static constexpr int P = P8 ? 8 : 16;            // radix of the in-register second stage
    static constexpr int U = T / P;                  // threads sharing one column DFT (1, 2, 3, 4)
    // threads per block: 256 (192 when U = 3), or NB (a multiple of T) for smaller blocks
    static constexpr int NT = NB ? NB : (U == 3) ? 192 : 256;
    static constexpr int LPB = NT / T;               // lines per block
    static constexpr int PAD = (T == 24) ? 4 : 0;    // slot offset between lines (bank spread)
    static constexpr int LREG = 16 * T + PAD;        // shared slots per line
    // separation pitch: the readers take (line p, column kx) with p fastest over LPB lines, so a
    // pitch of 32 / LPB (mod 16) float2 spreads a warp's 32 reads over all 16 bank pairs
    static constexpr int SEP = L + 32 / LPB;
    // the x pass's input tile is [2 LPB rows][PX] (kx contiguous): with 4 or 8 rows a pitch of
    // 32 / rows (mod 16) float2 spreads the copies of (row, kx), row fastest, over all 16 bank pairs;
    // with 2 rows, or 16 or 32 rows, the odd KX itself does
    static constexpr int KX = L / 2 + 1;
    static constexpr int PXM = (2 * LPB == 4 || 2 * LPB == 8) ? 32 / (2 * LPB) : 0;
    static constexpr int PX = PXM ? KX + ((PXM - KX % 16) + 16) % 16 : KX;
    static_assert(L == 256 || L == 384 || L == 512 || L == 768 || L == 1024, "line length");
    static_assert(NT % T == 0 && NT % 32 == 0 && LPB >= 1, "whole lines and warps per block");
};

// Barrier over the Geo<L, NB>::NT threads of a tile: __syncthreads when the tile takes a whole 256-thread
// block, else named barrier 1 over its NT threads, so that a larger block (the persistent batch
// kernel's) can leave its other threads out of the tile.
template <int L, int NB = 0> __device__ __forceinline__ void lsync()
{
    if constexpr (Geo<L, NB>::NT == 256) __syncthreads();
    else asm volatile("bar.sync 1, %0;" ::"n"(Geo<L, NB>::NT) : "memory");
}

// First-stage twiddles W_L^(r k1) (r < T, k1 < 16) laid out [k1][r]: the T threads of a line read
// consecutive slots (conflict free) instead of the strided W_L table entries r k1.
template <int L, int NB = 0> __device__ __forceinline__ void load_twr(float2 *twr, const float2 *__restrict__ tw, int nt)
{
    constexpr int T = Geo<L, NB>::T;
    for (int t = threadIdx.x; t < L; t += nt) {
        const int k1 = t / T, r = t - k1 * T;
        twr[t] = tw[r * k1];
    }
}

// low 4 bits of a row -> a permutation whose bit 3 is the row's bit 0: rows that differ in bit 0
// land in opposite halves of the 16 banks (conflict-free column reads for U = 2, 4)
__device__ __forceinline__ int hsw(int row) { return ((row & 1) << 3) | ((row >> 1) & 7); }
__device__ __forceinline__ int slot(int row, int col) { return row * 16 + (col ^ hsw(row)); }

// the thread's role in stage B: column k1 (or the pair a, a + 8), its u, and the d it keeps
template <int L> struct Role {
    int k1, u, d;
    __device__ __forceinline__ Role(int r)
    {
        typedef Geo<L> G; // the role depends on T only
        if constexpr (G::U == 1) {
            k1 = r;
            u = 0;
        } else if constexpr (G::U == 2) {
            u = (r >> 3) & 1;
            k1 = (r & 7) | ((r >> 4) << 3);
        } else if constexpr (G::U == 4) {
            u = (r >> 3) & 3;
            k1 = (r & 7) | ((r >> 5) << 3);
        } else if constexpr (G::P8) { // T = 24
            u = r >> 3;
            k1 = r & 7; // and k1 + 8
        } else { // T = 48
            u = r >> 4;
            k1 = r & 15;
        }
        d = (G::U == 4) ? (((u & 1) << 1) | (u >> 1)) : u;
    }
    // index along the line of the thread's value j in the B layout
    __device__ __forceinline__ int elem(int j) const
    {
        typedef Geo<L> G; // the role depends on T only
        if constexpr (G::U == 3) { // k2 = 3 c + d
            if constexpr (G::P8) return k1 + ((j >> 3) << 3) + 48 * (j & 7) + 16 * d;
            else return k1 + 48 * j + 16 * d;
        } else {
            return k1 + 16 * j + 256 * d;
        }
    }
};

__device__ __forceinline__ float2 cm(float2 a, float2 w) { return make_float2(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x); }
__device__ __forceinline__ float2 cmc(float2 a, float2 w) { return make_float2(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 shfl2(float2 v, int m)
{
    return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}
// multiply by -i (forward) or +i (inverse)
template <bool INV> __device__ __forceinline__ float2 mi(float2 a) { return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x); }

// a + s b on both lanes with one packed FFMA2: for s = +1 or -1 it rounds exactly as a + b or a - b
__device__ __forceinline__ float2 addsub(float2 b, float2 s, float2 a) { return __ffma2_rn(b, s, a); }
__device__ __forceinline__ float2 sign2(bool neg) { return neg ? make_float2(-1.f, -1.f) : make_float2(1.f, 1.f); }

// radix-U DFT across the U threads of a column, U = 2 or 4 (forward keeps d, inverse ends in u).  The
// thread holding the difference of a butterfly takes o - v, the other v + o, both as v * s + o.
template <int U, bool INV> __device__ __forceinline__ void xdft_fwd(float2 (&v)[16], int u)
{
    if constexpr (U == 2) {
        const float2 s = sign2(u != 0);
#pragma unroll
        for (int c = 0; c < 16; ++c) v[c] = addsub(v[c], s, shfl2(v[c], 8));
    } else { // U = 4, u = 2 u1 + u0: first across u1 (lane bit 4), then across u0 (lane bit 3)
        const int u0 = u & 1, u1 = u >> 1;
        const float2 s0 = sign2(u0 != 0), s1 = sign2(u1 != 0);
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            float2 e = addsub(v[c], s1, shfl2(v[c], 16)); // E[u0][d0 = u1]
            if (u0 && u1) e = mi<INV>(e);                // W_4^(u0 d0)
            v[c] = addsub(e, s0, shfl2(e, 8));           // X[d0 + 2 d1], d1 = u0
        }
    }
}

template <int U, bool INV> __device__ __forceinline__ void xdft_inv(float2 (&v)[16], int u)
{
    if constexpr (U == 2) {
        const float2 s = sign2(u != 0);
#pragma unroll
        for (int c = 0; c < 16; ++c) v[c] = addsub(v[c], s, shfl2(v[c], 8));
    } else {
        const int u0 = u & 1, u1 = u >> 1;
        const float2 s0 = sign2(u0 != 0), s1 = sign2(u1 != 0);
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            float2 g = addsub(v[c], s0, shfl2(v[c], 8)); // G[d0 = u1][u0]
            if (u0 && u1) g = mi<INV>(g);               // conj(W_4^(u0 d0)) on the inverse
            v[c] = addsub(g, s1, shfl2(g, 16));
        }
    }
}

// one output of a radix-3 DFT: a0 + W3^d a1 + W3^(2d) a2 (W3 = exp(-2 pi i/3), conjugate on the inverse)
template <bool INV> __device__ __forceinline__ float2 dft3_out(float2 a0, float2 a1, float2 a2, int d)
{
    if (d == 0) return add2(a0, add2(a1, a2));
    const float c3 = -0.5f, s3 = INV ? 0.86602540378443864676f : -0.86602540378443864676f;
    const float sd = (d == 1) ? s3 : -s3;
    return add2(a0, add2(cm(a1, make_float2(c3, sd)), cm(a2, make_float2(c3, -sd))));
}

// radix-8 DFT (natural order in and out) on v[o .. o+7]
template <bool INV> __device__ __forceinline__ void dft8at(float2 (&v)[16], int o)
{
    float2 t[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) t[q] = v[o + q];
    dft8<INV>(t);
#pragma unroll
    for (int q = 0; q < 8; ++q) v[o + q] = t[q];
}

// Forward transform of the thread's line: in v[i] = x[r + T i]; out v[j] = X[ro.elem(j)].
// z: the line's slot region; tw: W_L^t (t < L).  Leaves the slots free (ends with a barrier).
// tail = false (U = 1, 2, 4) leaves out that last barrier: allowed when the next access to the slots
// is line_inv's first store, which writes exactly the slots each thread read here last.
template <int L, int NB = 0>
__device__ __forceinline__ void line_fwd(float2 (&v)[16], int r, const Role<L> &ro, float2 *z, const float2 *tw,
                                         const float2 *twr, bool tail = true)
{
    typedef Geo<L, NB> G;
    pdft16<false>(v);
#pragma unroll
    for (int k1 = 1; k1 < 16; ++k1) v[k1] = cm(v[k1], twr[k1 * G::T + r]);
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) z[slot(r, k1)] = v[k1];
    lsync<L, NB>();
    if constexpr (G::U == 3) {
        // T = 3 P: r = s + P t, k2 = 3 c + d.  The thread's output d: radix-3 over t (reading the
        // three rows of each s), twiddle W_T^(s d) = W_L^(16 s d), radix-P over s.
        constexpr int P = G::P;
#pragma unroll
        for (int h = 0; h < 16 / P; ++h)
#pragma unroll
            for (int s = 0; s < P; ++s) {
                const int col = ro.k1 + 8 * h;
                v[P * h + s] = dft3_out<false>(z[slot(s, col)], z[slot(s + P, col)], z[slot(s + 2 * P, col)], ro.d);
            }
        lsync<L, NB>();
        if (ro.d)
#pragma unroll
            for (int j = 0; j < 16; ++j)
                if (j % P) v[j] = cm(v[j], tw[16 * ro.d * (j % P)]);
        if constexpr (G::P8) {
            dft8at<false>(v, 0);
            dft8at<false>(v, 8);
        } else {
            pdft16<false>(v);
        }
    } else {
#pragma unroll
        for (int s = 0; s < 16; ++s) v[s] = z[slot(G::U * s + ro.u, ro.k1)];
        if (tail) lsync<L, NB>();
        pdft16<false>(v);
        if (G::U > 1 && ro.u)
#pragma unroll
            for (int c = 1; c < 16; ++c) v[c] = cm(v[c], tw[16 * ro.u * c]);
        if constexpr (G::U == 2 || G::U == 4) xdft_fwd<G::U, false>(v, ro.u);
    }
}

// Inverse (unnormalised) transform: in v[j] = X[ro.elem(j)]; out v[i] = x[r + T i] * L.
// tail = false leaves out the last barrier (after the final slot reads): allowed when the slots are
// not touched again before a barrier of the caller.
template <int L, int NB = 0>
__device__ __forceinline__ void line_inv(float2 (&v)[16], int r, const Role<L> &ro, float2 *z, const float2 *tw,
                                         const float2 *twr, bool tail = true)
{
    typedef Geo<L, NB> G;
    if constexpr (G::U == 3) {
        // reverse of the forward: radix-P over c, conjugate twiddle, then the radix-3 over d is
        // formed by the reading thread r = s + P t from the three d slots of (s, column)
        constexpr int P = G::P;
        if constexpr (G::P8) {
            dft8at<true>(v, 0);
            dft8at<true>(v, 8);
        } else {
            pdft16<true>(v);
        }
        if (ro.d)
#pragma unroll
            for (int j = 0; j < 16; ++j)
                if (j % P) v[j] = cmc(v[j], tw[16 * ro.d * (j % P)]);
#pragma unroll
        for (int h = 0; h < 16 / P; ++h)
#pragma unroll
            for (int s = 0; s < P; ++s) z[slot(ro.d * P + s, ro.k1 + 8 * h)] = v[P * h + s];
        lsync<L, NB>();
        const int s0 = r % P, t0 = r / P;
#pragma unroll
        for (int k1 = 0; k1 < 16; ++k1)
            v[k1] = dft3_out<true>(z[slot(s0, k1)], z[slot(P + s0, k1)], z[slot(2 * P + s0, k1)], t0);
        if (tail) lsync<L, NB>();
    } else {
        if constexpr (G::U == 2 || G::U == 4) xdft_inv<G::U, true>(v, ro.u);
        if (G::U > 1 && ro.u)
#pragma unroll
            for (int c = 1; c < 16; ++c) v[c] = cmc(v[c], tw[16 * ro.u * c]);
        pdft16<true>(v);
#pragma unroll
        for (int s = 0; s < 16; ++s) z[slot(G::U * s + ro.u, ro.k1)] = v[s];
        lsync<L, NB>();
#pragma unroll
        for (int k1 = 0; k1 < 16; ++k1) v[k1] = z[slot(r, k1)];
        if (tail) lsync<L, NB>();
    }
#pragma unroll
    for (int k1 = 1; k1 < 16; ++k1) v[k1] = cmc(v[k1], twr[k1 * G::T + r]);
    pdft16<true>(v);
}

template <int L, int NB = 0> constexpr int yline_smem_bytes() { return (Geo<L, NB>::LPB * Geo<L, NB>::LREG + L + L + L) * 8; }

// One y tile of the 2D fused Euler update (pf/euler.go:16-47; plain form, no noise or filter):
// LPB lines q0 .. of length L = g.Y, groups a.buf[0 .. ng), c-hat a.state, T <- inverse(c_new/N).
template <int L, int NG, int NB = 0> __device__ __forceinline__ void yline_tile(const PassArgs<float> &a, long long tile)
{
    typedef Geo<L, NB> G;
    extern __shared__ __align__(16) unsigned char fl_dsm[];
    float2 *s_x = reinterpret_cast<float2 *>(fl_dsm);
    float2 *s_tw = s_x + G::LPB * G::LREG;
    float2 *s_twr = s_tw + L;
    float *s_fy = reinterpret_cast<float *>(s_twr + L);
    const Geom &g = a.g;
    const int l = threadIdx.x / G::T, r = threadIdx.x - l * G::T;
    const long long nlines = (long long)g.Z * g.KX;
    const long long q = tile * G::LPB + l;
    const bool valid = q < nlines;
    float2 *z = s_x + l * G::LREG;
    const float2 zero = make_float2(0.f, 0.f);
    for (int t = threadIdx.x; t < L; t += G::NT) {
        s_tw[t] = a.tw[t];
        s_fy[t] = f256::fsqf(t, g.Y);
    }
    load_twr<L, NB>(s_twr, a.tw, G::NT);
    const Role<L> ro(r);
    const float2 *__restrict__ U0 = a.buf[0];
    float2 *__restrict__ state = a.state;
    float2 v[16], cs[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = valid ? U0[q * L + r + G::T * i] : zero;
    // c-hat of the thread's B-layout elements, requested before the transform so that its
    // latency overlaps the forward FFT
#pragma unroll
    for (int j = 0; j < 16; ++j) cs[j] = valid ? state[q * L + ro.elem(j)] : zero;
    lsync<L, NB>();
    const UpdTable &u = a.upd;
    const int ngrp = (NG == 1) ? (u.ngrp > 0 ? 1 : 0) : u.ngrp;
    // the last forward transform before line_inv needs no trailing barrier
    line_fwd<L, NB>(v, r, ro, z, s_tw, s_twr, NG > 1 && ngrp > 1);
    float2 w[NG == 1 ? 1 : 16];
    if (NG > 1 && ngrp > 1) {
        const float2 *__restrict__ U1 = a.buf[1];
#pragma unroll
        for (int i = 0; i < 16; ++i) w[i] = valid ? U1[q * L + r + G::T * i] : zero;
        line_fwd<L, NB>(reinterpret_cast<float2(&)[16]>(w), r, ro, z, s_tw, s_twr, false);
    }
    const f256::UpdRegs R = f256::load_upd(u, ngrp);
    float fl = 0.f;
    if (valid) {
        const int zz = (int)(q / g.KX), kx = (int)(q - (long long)zz * g.KX);
        const float fx = (float)kx / (float)g.X;
        fl = fx * fx + f256::fsqf(zz, g.Z);
    }
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const int k = ro.elem(j);
        float2 cn = zero;
        if (valid) {
            const float mk = -39.478417604357434f * (fl + s_fy[k]);
            cn = f256::euler_update<NG>(R, cs[j], v[j], (NG > 1) ? w[NG > 1 ? j : 0] : v[j], mk);
            state[q * L + k] = cn;
        }
        v[j] = make_float2(cn.x * R.invN, cn.y * R.invN);
    }
    // the tile ends here: the block exits, or its caller passes a barrier before the next tile
    line_inv<L, NB>(v, r, ro, z, s_tw, s_twr, false);
    float2 *__restrict__ T = a.tout;
#pragma unroll
    for (int i = 0; i < 16; ++i)
        if (valid) T[q * L + r + G::T * i] = v[i];
}

// Forward or inverse (unnormalised) transforms of LPB lines of buf, in place, with no update: the
// y passes of PM_FWD and PM_INV (L = g.Y, lines q = z KX + kx).  The forward transform leaves a line in
// the B layout, stored at its natural positions elem(j); the inverse reads those and ends in the A
// layout.  Shared memory as yline_tile (the frequency table unused).
template <int L, int NB = 0> __device__ __forceinline__ void yline_pass_tile(const PassArgs<float> &a, long long tile, int b, bool inv)
{
    typedef Geo<L, NB> G;
    extern __shared__ __align__(16) unsigned char fl_dsm[];
    float2 *s_x = reinterpret_cast<float2 *>(fl_dsm);
    float2 *s_tw = s_x + G::LPB * G::LREG;
    float2 *s_twr = s_tw + L;
    const Geom &g = a.g;
    const int l = threadIdx.x / G::T, r = threadIdx.x - l * G::T;
    const long long nlines = (long long)g.Z * g.KX;
    const long long q = tile * G::LPB + l;
    const bool valid = q < nlines;
    float2 *z = s_x + l * G::LREG;
    const float2 zero = make_float2(0.f, 0.f);
    float2 *__restrict__ buf = a.buf[b];
    const Role<L> ro(r);
    float2 v[16];
    if (!inv) {
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = valid ? buf[q * L + r + G::T * i] : zero;
    } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = valid ? buf[q * L + ro.elem(j)] : zero;
    }
    for (int t = threadIdx.x; t < L; t += G::NT) s_tw[t] = a.tw[t];
    load_twr<L, NB>(s_twr, a.tw, G::NT);
    lsync<L, NB>();
    if (!inv) {
        line_fwd<L, NB>(v, r, ro, z, s_tw, s_twr);
#pragma unroll
        for (int j = 0; j < 16; ++j)
            if (valid) buf[q * L + ro.elem(j)] = v[j];
    } else {
        line_inv<L, NB>(v, r, ro, z, s_tw, s_twr);
#pragma unroll
        for (int i = 0; i < 16; ++i)
            if (valid) buf[q * L + r + G::T * i] = v[i];
    }
}

// one shared array holds, in turn, the spectral tile [2 LPB rows][PX], the exchange slots of the
// LPB lines and the separation slots [LPB][SEP]; then two twiddle tables and the polynomial
// coefficients
template <int L, int NB = 0> __host__ __device__ constexpr int xline_area()
{
    constexpr int a = 2 * Geo<L, NB>::LPB * Geo<L, NB>::PX, b = Geo<L, NB>::LPB * Geo<L, NB>::LREG, c = Geo<L, NB>::LPB * Geo<L, NB>::SEP;
    return (a > b ? (a > c ? a : c) : (b > c ? b : c));
}
template <int L, int NB = 0> constexpr int xline_smem_bytes()
{
    return (xline_area<L, NB>() + 2 * L) * 8 + GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1) * 4;
}

// 16-byte asynchronous global -> shared copy (no register staging), completed by cp_async_wait
__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
// 8-byte asynchronous copy (through L1: the neighbouring rows of the same sector follow at once)
__device__ __forceinline__ void cp_async8(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Request the spectral tile of x tile ty (kx = 0 .. L/2, rows y0 .. y0 + 2 LPB) into area[row][kx]
// (pitch PX) with 8-byte asynchronous copies, row fastest (g.Y must be a multiple of 2 LPB).
template <int L, int NB = 0>
__device__ __forceinline__ void xline_request_from(float2 *area, const float2 *__restrict__ in, const Geom &g, int ty, int zp)
{
    typedef Geo<L, NB> G;
    constexpr int KX = G::KX, RB = 2 * G::LPB;
    const long long sbase = (long long)zp * g.S + (long long)ty * RB;
    for (int e = threadIdx.x; e < KX * RB; e += G::NT) {
        const int kx = e / RB, row = e - kx * RB;
        cp_async8(&area[row * G::PX + kx], &in[sbase + (long long)kx * g.Y + row]);
    }
    cp_async_commit();
}
template <int L, int NB = 0> __device__ __forceinline__ void xline_request(float2 *area, const XPassArgs<float> &a, int ty, int zp)
{
    xline_request_from<L, NB>(area, a.in, a.g, ty, zp);
}

// Rows (2l, 2l + 1) of the tile as one complex line a + i b of L columns, Hermitian-extended, in
// the A layout (v[i] = column r + T i), conjugated: conj(A(k) + i B(k)) for k <= L/2 and
// conj(conj A(L - k) + i conj B(L - k)) above.  Consecutive r read consecutive slots.
template <int L, int NB = 0> __device__ __forceinline__ void xline_gather_conj(const float2 *s_a, int l, int r, float2 (&v)[16])
{
    typedef Geo<L, NB> G;
    constexpr int H = L / 2;
    const float2 *ra = s_a + (2 * l) * G::PX, *rb = ra + G::PX;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int k = r + G::T * i;
        const bool lo = (i < 8) || (i == 8 && r == 0); // k <= H
        const int kk = lo ? k : L - k;
        const float2 A = ra[kk], B = rb[kk];
        // lo: A + i B = (A.x - B.y, A.y + B.x); hi: conj A + i conj B = (A.x + B.y, B.x - A.y)
        v[i] = lo ? make_float2(A.x - B.y, -(A.y + B.x)) : make_float2(A.x + B.y, A.y - B.x);
    }
    (void)H;
}

// The separation slots of the line's forward spectrum Z (A layout, v holding conj Z) and the
// coalesced stores of the two rows' half spectra X_a(k) = (Z(k) + conj Z(-k))/2 (row 2p) and
// X_b(k) = (Z(k) - conj Z(-k))/(2i) (row 2p + 1).
template <int L, int NB = 0>
__device__ __forceinline__ void xline_separate(float2 (&v)[16], float2 *s_sep, int l, int r, float2 *__restrict__ out,
                                               long long sbase, int y0, int Y)
{
    typedef Geo<L, NB> G;
    constexpr int KX = G::KX;
#pragma unroll
    for (int i = 0; i < 16; ++i) s_sep[l * G::SEP + r + G::T * i] = make_float2(v[i].x, -v[i].y);
    lsync<L, NB>();
    for (int e = threadIdx.x; e < KX * G::LPB; e += G::NT) {
        const int kx = e / G::LPB, p = e - kx * G::LPB;
        const float2 P = s_sep[p * G::SEP + kx];
        const float2 Q = s_sep[p * G::SEP + (kx ? L - kx : 0)];
        if (y0 + 2 * p < Y)
            *reinterpret_cast<float4 *>(&out[sbase + (long long)kx * Y + 2 * p]) =
                make_float4(0.5f * (P.x + Q.x), 0.5f * (P.y - Q.y), 0.5f * (P.y + Q.y), 0.5f * (Q.x - P.x));
    }
    lsync<L, NB>();
}

// One x tile from its spectral tile in area (which then serves as exchange and separation
// space): c2r of 2 LPB rows -> polynomial groups -> r2c into a.out[grp] (L = g.X columns).
// The inverse transform is the forward line transform of the conjugate (A layout in, B layout
// out) and the forward transform the inverse line transform of the conjugate (B in, A out), so
// the tile is read and the spectra are separated in the A layout, where a line's threads touch
// consecutive slots.  s_poly: this instance's dense polynomial coefficients.  Ends with a barrier.
// ONE: exactly one output group, a dense polynomial of degree <= 6 (the caller checks), so only one
// line is held in registers and the polynomial is unrolled for its degree
template <int L, bool ONE = false, int NB = 0>
__device__ __forceinline__ void xline_compute(float2 *s_a, const XPassArgs<float> &a, int ty, int zp,
                                              const float2 *s_tw, const float2 *s_twr, const float *s_poly)
{
    typedef Geo<L, NB> G;
    constexpr int RB = 2 * G::LPB;
    float2 *s_sep = s_a; // [LPB][SEP], once the exchange is done
    const Geom &g = a.g;
    const int l = threadIdx.x / G::T, r = threadIdx.x - l * G::T;
    const int y0 = ty * RB;
    const long long sbase = (long long)zp * g.S + y0;
    const int Y = g.Y;
    const Role<L> ro(r);
    float2 v[16];
    xline_gather_conj<L, NB>(s_a, l, r, v);
    lsync<L, NB>(); // the tile becomes the exchange slots
    float2 *z = s_a + l * G::LREG;
    line_fwd<L, NB>(v, r, ro, z, s_tw, s_twr, false); // line_inv comes next
    // conj(v[j]) = c(row 2l, col elem(j)) + i c(row 2l + 1, col elem(j)) (times L)
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j].y = -v[j].y;
    // group grp from w: polynomial, forward transform as conj(inverse(conj w)), separation
    auto emit = [&](float2(&w)[16], int grp) {
        if (!a.identity) f256::apply_poly(w, a, grp, s_poly + grp * (GOPF_MAX_DEG + 1));
#pragma unroll
        for (int j = 0; j < 16; ++j) w[j].y = -w[j].y;
        line_inv<L, NB>(w, r, ro, z, s_tw, s_twr);
        xline_separate<L, NB>(w, s_sep, l, r, a.out[grp], sbase, y0, Y);
    };
    if constexpr (ONE) {
        switch (a.pw.deg[0]) {
        case 0: f256::poly_regs<0>(v, s_poly); break;
        case 1: f256::poly_regs<1>(v, s_poly); break;
        case 2: f256::poly_regs<2>(v, s_poly); break;
        case 3: f256::poly_regs<3>(v, s_poly); break;
        case 4: f256::poly_regs<4>(v, s_poly); break;
        case 5: f256::poly_regs<5>(v, s_poly); break;
        default: f256::poly_regs<6>(v, s_poly); break;
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j].y = -v[j].y;
        line_inv<L, NB>(v, r, ro, z, s_tw, s_twr);
        xline_separate<L, NB>(v, s_sep, l, r, a.out[0], sbase, y0, Y);
        return;
    }
    // every group but the last works on a copy; the last one on v itself, so that a single group
    // (the usual case) does not hold two lines in registers
    const int ng = a.ngrp_out;
    for (int grp = 0; grp + 1 < ng; ++grp) {
        float2 w[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) w[i] = v[i];
        emit(w, grp);
    }
    if (ng > 0) emit(v, ng - 1);
}

template <int L, int NB = 0>
__device__ __forceinline__ void load_xconsts(const XPassArgs<float> &a, float2 *s_tw, float2 *s_twr, float *s_poly)
{
    for (int t = threadIdx.x; t < L; t += Geo<L, NB>::NT) s_tw[t] = a.twX[t];
    load_twr<L, NB>(s_twr, a.twX, Geo<L, NB>::NT);
    for (int t = threadIdx.x; t < GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1); t += Geo<L, NB>::NT)
        s_poly[t] = (float)a.pw.dense[t / (GOPF_MAX_DEG + 1)][t % (GOPF_MAX_DEG + 1)];
}

// One x tile: 2 LPB rows from row ty * 2 LPB of depth plane zp (g.Y a multiple of 2 LPB).
// The adjoint step's x pass (program XP_ADJ) on one x tile: mu = c2r(in) and nu = c2r(in2) along x,
// c from the real rows rin, lambda = mu - dtM (3 c^2 - 1) nu into the real rows rout and, forward
// transformed and separated, into out[0] (in place of in when out[0] == in: the tile is read first).
template <int L, int NB = 0> __device__ __forceinline__ void xline_adj_tile(const XPassArgs<float> &a, int ty, int zp)
{
    typedef Geo<L, NB> G;
    extern __shared__ __align__(16) unsigned char fl_dsm[];
    float2 *s_a = reinterpret_cast<float2 *>(fl_dsm);
    float2 *s_tw = s_a + xline_area<L, NB>();
    float2 *s_twr = s_tw + L;
    float *s_poly = reinterpret_cast<float *>(s_twr + L);
    constexpr int RB = 2 * G::LPB;
    const Geom &g = a.g;
    const int l = threadIdx.x / G::T, r = threadIdx.x - l * G::T;
    const int y0 = ty * RB;
    const Role<L> ro(r);
    float2 *z = s_a + l * G::LREG;
    float2 mu[16], nu[16];
    xline_request_from<L, NB>(s_a, a.in, g, ty, zp);
    load_xconsts<L, NB>(a, s_tw, s_twr, s_poly);
    cp_async_wait<0>();
    lsync<L, NB>();
    xline_gather_conj<L, NB>(s_a, l, r, mu);
    lsync<L, NB>(); // the tile becomes the exchange slots
    line_fwd<L, NB>(mu, r, ro, z, s_tw, s_twr);
    xline_request_from<L, NB>(s_a, a.in2, g, ty, zp);
    cp_async_wait<0>();
    lsync<L, NB>();
    xline_gather_conj<L, NB>(s_a, l, r, nu);
    lsync<L, NB>();
    line_fwd<L, NB>(nu, r, ro, z, s_tw, s_twr);
    // conj(mu[j]) = mu(row 2l, col elem(j)) + i mu(row 2l + 1, col elem(j)); nu likewise
    const float dtM = (float)a.adj_dtM;
    const long long row0 = ((long long)zp * g.Y + y0 + 2 * l) * g.X;
    const float *__restrict__ rin = a.rin + row0;
    float *__restrict__ rout = a.rout + row0;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const int col = ro.elem(j);
        const float cx = rin[col], cy = rin[g.X + col];
        const float lx = mu[j].x - dtM * (3.f * cx * cx - 1.f) * nu[j].x;
        const float ly = -mu[j].y - dtM * (3.f * cy * cy - 1.f) * (-nu[j].y);
        rout[col] = lx;
        rout[g.X + col] = ly;
        mu[j] = make_float2(lx, -ly); // conjugated again for the forward transform
    }
    line_inv<L, NB>(mu, r, ro, z, s_tw, s_twr);
    xline_separate<L, NB>(mu, s_a, l, r, a.out[0], (long long)zp * g.S + y0, y0, g.Y);
}

template <int L, bool ONE = false, int NB = 0> __device__ __forceinline__ void xline_tile(const XPassArgs<float> &a, int ty, int zp)
{
    extern __shared__ __align__(16) unsigned char fl_dsm[];
    float2 *s_a = reinterpret_cast<float2 *>(fl_dsm);
    float2 *s_tw = s_a + xline_area<L, NB>();
    float2 *s_twr = s_tw + L;
    float *s_poly = reinterpret_cast<float *>(s_twr + L);
    xline_request<L, NB>(s_a, a, ty, zp);
    load_xconsts<L, NB>(a, s_tw, s_twr, s_poly);
    cp_async_wait<0>();
    lsync<L, NB>();
    xline_compute<L, ONE, NB>(s_a, a, ty, zp, s_tw, s_twr, s_poly);
}

} // namespace fl
} // namespace gopf
