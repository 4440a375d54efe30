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
#include "noise.cuh"
#include "tma.cuh"

namespace gopf {
namespace f256 {

constexpr int N = 256;
constexpr int R = 16;
constexpr int NT = 256; // threads per block: 16 lines x 16 radix positions

// ---------------------------------------------------------------------------
// Radix-16 on packed FP32x2 (Blackwell's two-lane FADD2/FFMA2): a complex
// add or subtract is one instruction.  Each lane rounds once, exactly as the
// scalar code does, so the results are bitwise those of dft16 in fft_core.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

// a -/+ i d (forward: a - i d = (a.x + d.y, a.y - d.x); inverse: a + i d), with the swapped pair of d
template <bool INV> __device__ __forceinline__ float2 pmi_add(float2 a, float2 d)
{
    const float2 sw = make_float2(d.y, d.x);
    return __ffma2_rn(sw, INV ? make_float2(-1.f, 1.f) : make_float2(1.f, -1.f), a);
}

template <bool INV> __device__ __forceinline__ void pdft4(float2 &v0, float2 &v1, float2 &v2, float2 &v3)
{
    const float2 a0 = padd(v0, v2), a1 = psub(v0, v2);
    const float2 a2 = padd(v1, v3), d = psub(v1, v3);
    v0 = padd(a0, a2);
    v2 = psub(a0, a2);
    v1 = pmi_add<INV>(a1, d);
    v3 = pmi_add<!INV>(a1, d);
}

template <bool INV> __device__ __forceinline__ void pdft16(float2 (&v)[16])
{
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) pdft4<INV>(v[n1], v[4 + n1], v[8 + n1], v[12 + n1]);
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
    for (int k1 = 0; k1 < 4; ++k1) pdft4<INV>(v[4 * k1 + 0], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
    float2 t[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) t[k1 + 4 * k2] = v[4 * k1 + k2];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = t[i];
}

// 256-point FFT of the thread's v[i] = x[r + 16 i]; result v[i] = X[r + 16 i].
// at(a, b) is the shared-memory slot of element (a, b) of this thread's line.
// WARP: the 16 threads of every line are one half-warp and its slots are its
// own, so the exchange only has to be ordered within the warp.
// Programmatic dependent launch.  pdl_trigger lets the next kernel of the stream be scheduled once
// every block of this one has started; pdl_wait (before a thread's first access to data an earlier
// kernel produced or still reads) returns once the previous kernel has completed and its writes are
// visible.  Both do nothing in a kernel that was not launched as a programmatic dependent.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void xsync(bool warp)
{
    if (warp) __syncwarp();
    else __syncthreads();
}

// TR: the exchange stores thread r's values in column r (at(k1, r)) and reads row r, the transpose
// of the default; the arithmetic is the same.  A transform in the transposed form writes exactly the
// slots the same thread read in a default-form transform just before it, so that transform may end
// without its trailing barrier (TAIL = false) when the transposed one follows.
template <bool INV, bool WARP = false, bool TAIL = true, bool TR = false, typename AT>
__device__ __forceinline__ void fft256(float2 (&v)[16], int r, const float2 *__restrict__ tw, AT &&at)
{
    pdft16<INV>(v);
#pragma unroll
    for (int k1 = 1; k1 < 16; ++k1) {
        const float2 w = tw[k1 * 16 + r]; // W256^(r k1), laid out [k1][r]: conflict free
        v[k1] = INV ? cmulc(v[k1], w) : cmul(v[k1], w);
    }
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) {
        if (TR) at(k1, r) = v[k1];
        else at(r, k1) = v[k1];
    }
    xsync(WARP);
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) v[n2] = TR ? at(r, n2) : at(n2, r);
    pdft16<INV>(v);
    if (TAIL) xsync(WARP); // slots may be reused after return
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

// Kernels with the update take NZ: true only for models with a noise term or a
// modal filter, so the Philox/Box-Muller and filter code is not carried by the
// plain instantiations.

// k-space update coefficients staged in registers once per thread
struct UpdRegs {
    float dt, invN;
    int ng;
    float gs[2];
    int gl[2];
    int nimp;
    float imp[4];
};

__device__ __forceinline__ UpdRegs load_upd(const UpdTable &u, int ng)
{
    UpdRegs R;
    R.dt = (float)u.dt;
    R.invN = (float)u.invN;
    R.ng = ng;
#pragma unroll
    for (int b = 0; b < 2; ++b) {
        // a group the model does not have contributes nothing (scale 0)
        R.gs[b] = (b < ng) ? (u.gscale[b] ? (float)(*u.gscale[b]) : 1.f) : 0.f;
        R.gl[b] = (b < ng) ? u.glap[b] : 0;
    }
    R.nimp = u.nimp; // at most 4 on this path (the launchers check)
#pragma unroll
    for (int q = 0; q < 4; ++q) R.imp[q] = (q < u.nimp) ? (float)u.imp[q] : 0.f;
    return R;
}

// m^p for a uniform 0 <= p < 8 without branches in the unrolled update loops
__device__ __forceinline__ float mkpow(float mk, int p)
{
    const float m2 = mk * mk;
    float f = (p & 1) ? mk : 1.f;
    f *= (p & 2) ? m2 : 1.f;
    if (p & 4) f *= m2 * m2;
    return f;
}

// ApplyModalFilter (pf/util.go:125-132) with the Vandeven.Eval interpolation (pf/vandeven.go:30-40):
// c * filter(2|f|/pi), |f|^2 = f2 in cycles per sample
__device__ __forceinline__ float2 modal_filter(const UpdTable &u, float2 c, float f2)
{
    const float *__restrict__ tab = static_cast<const float *>(u.filt);
    const int n = u.nfilt;
    const float x = sqrtf(f2) * 0.636619772367581343f;
    const float nn = (float)(n - 1);
    const int idx = (int)(x * nn);
    float s;
    if (idx >= n - 1) {
        s = tab[n - 1];
    } else {
        const float dx = 1.f / nn;
        s = tab[idx] + (x - (float)idx * dx) * (tab[idx + 1] - tab[idx]) / dx;
    }
    return make_float2(c.x * s, c.y * s);
}

// 1/d from the hardware reciprocal estimate refined by one Newton step (error well below
// an FP32 ulp before the final rounding; d is near 1 here, never denormal)
__device__ __forceinline__ float recip_nr(float d)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d));
    return r * (2.f - d * r);
}

// k-space update of one element (pf/euler.go:32-34 with the term algebra of pf/rhsBuilder.go):
// c <- (c + dt sum_b s_b m^p_b U_b) / (1 - dt L(m)),  m = -k^2
template <int NG>
__device__ __forceinline__ float2 euler_update(const UpdRegs &R, float2 c0, float2 U0, float2 U1, float mk)
{
    const float f0 = R.gs[0] * mkpow(mk, R.gl[0]);
    float2 nh = make_float2(f0 * U0.x, f0 * U0.y);
    if (NG > 1 && R.ng > 1) {
        const float f1 = R.gs[1] * mkpow(mk, R.gl[1]);
        nh.x += f1 * U1.x;
        nh.y += f1 * U1.y;
    }
    const float L = ((R.imp[3] * mk + R.imp[2]) * mk + R.imp[1]) * mk + R.imp[0];
    const float rden = recip_nr(1.f - R.dt * L);
    return make_float2((c0.x + R.dt * nh.x) * rden, (c0.y + R.dt * nh.y) * rden);
}

// ---------------------------------------------------------------------------
// z axis (strided), fused forward -> update -> inverse.  Lines are 16
// consecutive inner indices i0 + l of the S = KX*Y plane; thread t = r*16 + l.
// ---------------------------------------------------------------------------
template <int NG, bool NZ>
__global__ void __launch_bounds__(NT, NG == 1 ? 3 : 2) k_z256_fused(const PassArgs<float> a)
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

    float2 v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = U0[i0 + l + (long long)(r + 16 * i) * S];
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
    const UpdRegs R = load_upd(u, ngrp);
    const float fourpi2 = 39.478417604357434f;
    const float fl = s_fl[l];
    float2 *__restrict__ state = a.state;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int k = r + 16 * i;
        const long long gi = i0 + l + (long long)k * S;
        float2 cn;
        if (init) {
            cn = v[i];
        } else {
            const float mk = -fourpi2 * (fl + s_fz[k]);
            float2 c0 = state[gi];
            if (NZ && u.noise.kind) { // noise enters as dt * N_noise, folded into c0 before the division
                const long long q = i0 + l, kx = q / g.Y, yy = q - kx * g.Y;
                double nr, ni;
                noise_term(u.noise, g.X, g.Y, g.Z, kx, yy, k, (double)mk, nr, ni);
                c0.x += R.dt * (float)nr;
                c0.y += R.dt * (float)ni;
            }
            cn = euler_update<NG>(R, c0, v[i], (NG > 1) ? w[NG > 1 ? i : 0] : v[i], mk);
            if (NZ && u.filt) cn = modal_filter(u, cn, fl + s_fz[k]);
        }
        state[gi] = cn;
        v[i] = make_float2(cn.x * R.invN, cn.y * R.invN);
    }
    fft256<true>(v, r, s_tw, at);
    float2 *__restrict__ T = a.tout;
#pragma unroll
    for (int i = 0; i < 16; ++i) T[i0 + l + (long long)(r + 16 * i) * S] = v[i];
}

// ---------------------------------------------------------------------------
// z axis with TMA tiles.  The same transform and update as k_z256_fused, but
// the block's input tiles (group 0, group 1, c-hat: 16 inner indices x 256 z
// = 32 KB each) arrive in shared memory through one tensor copy apiece, and
// the c-hat and T tiles leave the same way.  The threads never wait on
// individual global loads: three blocks per SM overlap one block's copies
// with the others' transforms.  Tensor maps: [Z][S] of 8-byte elements, box
// {16, 256}.
// ---------------------------------------------------------------------------
constexpr int ZT_TILE_BYTES = 16 * N * 8;

__host__ __device__ constexpr int z256_tma_smem_bytes(int ng)
{
    return 128 /* alignment slack */ + ZT_TILE_BYTES * (ng + 1) + N * 8 /* twiddles */ + N * 4 /* fz */ +
           16 * 4 /* fl */ + 16 /* barrier, flag */;
}

template <int NG, bool NZ>
__global__ void __launch_bounds__(NT, NG == 1 ? 3 : 2)
    k_z256_tma(const PassArgs<float> a, const __grid_constant__ CUtensorMap mU0, const __grid_constant__ CUtensorMap mU1,
               const __grid_constant__ CUtensorMap mS, const __grid_constant__ CUtensorMap mT)
{
    pdl_trigger(); // the inverse y pass may be scheduled as soon as every block runs
    extern __shared__ unsigned char z_dsm[];
    unsigned char *base = z_dsm + ((128u - (smem_u32(z_dsm) & 127u)) & 127u);
    float2 *tU0 = reinterpret_cast<float2 *>(base);
    float2 *tU1 = reinterpret_cast<float2 *>(base + ZT_TILE_BYTES);
    float2 *tS = reinterpret_cast<float2 *>(base + ZT_TILE_BYTES * NG);
    float2 *s_tw = reinterpret_cast<float2 *>(base + ZT_TILE_BYTES * (NG + 1));
    float *s_fz = reinterpret_cast<float *>(s_tw + N);
    float *s_fl = s_fz + N;
    uint64_t *bar = reinterpret_cast<uint64_t *>(s_fl + 16);
    int *s_ok = reinterpret_cast<int *>(bar + 1);

    const Geom &g = a.g;
    const int l = threadIdx.x & 15, r = threadIdx.x >> 4;
    const int i0 = blockIdx.x * 16;
    const bool init = (a.mode == PM_INIT);
    const int ngrp = (NG == 1) ? (a.upd.ngrp > 0 ? 1 : 0) : a.upd.ngrp;
    const bool two = (NG > 1 && ngrp > 1);

    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t bytes = (uint32_t)ZT_TILE_BYTES * (1u + (two ? 1u : 0u) + (init ? 0u : 1u));
        mbar_arrive_expect_tx(bar, bytes);
        tma_load_2d(tU0, &mU0, i0, 0, bar);
        if (two) tma_load_2d(tU1, &mU1, i0, 0, bar);
        if (!init) tma_load_2d(tS, &mS, i0, 0, bar);
    }
    load_twiddles(s_tw, a.tw);
    if (threadIdx.x < 16) {
        const int q = i0 + threadIdx.x;
        const int kx = q / g.Y, y = q - kx * g.Y;
        const float fx = (float)kx / (float)g.X;
        s_fl[threadIdx.x] = fx * fx + fsqf(y, g.Y);
    }
    s_fz[threadIdx.x] = fsqf(threadIdx.x, g.Z);
    if (threadIdx.x == 0) *s_ok = tma_wait_or_flag(bar, 0, a.status) ? 1 : 0;
    __syncthreads();
    if (!*s_ok) return;

    float2 v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = tU0[(r + 16 * i) * 16 + l];
    __syncthreads(); // the group-0 tile becomes the exchange buffer
    auto at = [&](int x, int y) -> float2 & { return tU0[(x * 16 + y) * 16 + l]; };
    fft256<false>(v, r, s_tw, at);

    float2 w[NG == 1 ? 1 : 16];
    if (two) {
#pragma unroll
        for (int i = 0; i < 16; ++i) w[i] = tU1[(r + 16 * i) * 16 + l];
        fft256<false>(reinterpret_cast<float2(&)[16]>(w), r, s_tw, at);
    }

    const UpdTable &u = a.upd;
    const UpdRegs R = load_upd(u, ngrp);
    const float fourpi2 = 39.478417604357434f;
    const float fl = s_fl[l];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int k = r + 16 * i;
        float2 cn;
        if (init) {
            cn = v[i];
        } else {
            const float mk = -fourpi2 * (fl + s_fz[k]);
            float2 c0 = tS[k * 16 + l];
            if (NZ && u.noise.kind) {
                const long long q = i0 + l, kx = q / g.Y, yy = q - kx * g.Y;
                double nr, ni;
                noise_term(u.noise, g.X, g.Y, g.Z, kx, yy, k, (double)mk, nr, ni);
                c0.x += R.dt * (float)nr;
                c0.y += R.dt * (float)ni;
            }
            cn = euler_update<NG>(R, c0, v[i], (NG > 1) ? w[NG > 1 ? i : 0] : v[i], mk);
            if (NZ && u.filt) cn = modal_filter(u, cn, fl + s_fz[k]);
        }
        tS[k * 16 + l] = cn; // each thread rewrites exactly the elements it read
        v[i] = make_float2(cn.x * R.invN, cn.y * R.invN);
    }
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
        tma_store_2d(&mS, i0, 0, tS);
        bulk_commit();
    }
    fft256<true>(v, r, s_tw, at);
#pragma unroll
    for (int i = 0; i < 16; ++i) tU0[(r + 16 * i) * 16 + l] = v[i];
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
        tma_store_2d(&mT, i0, 0, tU0);
        bulk_commit();
        bulk_wait_read_all(); // the tiles stay allocated until both stores have read them
    }
}

// ---------------------------------------------------------------------------
// y axis (contiguous lines of 256), forward or inverse in place, or the 2D
// fused update.  Thread t = l*16 + r: a half-warp reads 128 contiguous bytes.
// Shared slots are swizzled so both exchange directions are conflict free.
// ---------------------------------------------------------------------------
template <int NG, bool NZ>
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
    const bool pdl = (a.allow_fast & ALLOW_PDL) != 0;
    pdl_trigger();

    // a programmatic dependent sets up its tables while the previous kernel finishes, then waits
    // for its data; otherwise the line is requested first, so that its latency hides behind the tables
    float2 v[16];
    if (!pdl)
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
    if (pdl) {
        pdl_wait();
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = valid ? buf[q * N + r + 16 * i] : zero;
    }
    __syncthreads();
    auto at = [&](int x, int y) -> float2 & { return s_x[l * N + x * 16 + ((x + y) & 15)]; };
    if (!fused) {
        if (a.mode == PM_FWD) fft256<false, true>(v, r, s_tw, at);
        else fft256<true, true>(v, r, s_tw, at);
#pragma unroll
        for (int i = 0; i < 16; ++i)
            if (valid) buf[q * N + r + 16 * i] = v[i];
        return;
    }
    fft256<false, true>(v, r, s_tw, at);
    const int ngrp = (NG == 1) ? (a.upd.ngrp > 0 ? 1 : 0) : a.upd.ngrp;
    float2 w[NG == 1 ? 1 : 16];
    if (NG > 1 && ngrp > 1) {
        const float2 *__restrict__ U1 = a.buf[1];
#pragma unroll
        for (int i = 0; i < 16; ++i) w[i] = valid ? U1[q * N + r + 16 * i] : zero;
        fft256<false, true>(reinterpret_cast<float2(&)[16]>(w), r, s_tw, at);
    }
    const UpdTable &u = a.upd;
    const UpdRegs R = load_upd(u, ngrp);
    const float fourpi2 = 39.478417604357434f;
    const float fl = s_fl[l];
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
                const float mk = -fourpi2 * (fl + s_fy[k]);
                float2 c0 = state[gi];
                if (NZ && u.noise.kind) {
                    const long long zz = q / g.KX, kx = q - zz * g.KX;
                    double nr, ni;
                    noise_term(u.noise, g.X, g.Y, g.Z, kx, k, zz, (double)mk, nr, ni);
                    c0.x += R.dt * (float)nr;
                    c0.y += R.dt * (float)ni;
                }
                cn = euler_update<NG>(R, c0, v[i], (NG > 1) ? w[NG > 1 ? i : 0] : v[i], mk);
                if (NZ && u.filt) cn = modal_filter(u, cn, fl + s_fy[k]);
            }
            state[gi] = cn;
        }
        v[i] = make_float2(cn.x * R.invN, cn.y * R.invN);
    }
    fft256<true, true>(v, r, s_tw, at);
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

// Rows 2j and 2j+1 of a [129 kx][32 y] half-spectrum tile as one complex line a + i b of 256
// columns, Hermitian-extended: column k holds A(k) + i B(k) for k <= 128 and
// conj A(256 - k) + i conj B(256 - k) above.  k = r + 16 i is <= 128 exactly when i < 8, or i == 8
// and r == 0, so only i == 8 needs a (uniform-cost) select.
__device__ __forceinline__ void load_pair_line(const float2 *__restrict__ t, int r, int j, float2 (&v)[16])
{
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int k = r + 16 * i;
        if (i < 8) {
            const float4 ab = *reinterpret_cast<const float4 *>(&t[k * XROWS + 2 * j]);
            v[i] = make_float2(ab.x - ab.w, ab.y + ab.z);
        } else if (i > 8) {
            const float4 ab = *reinterpret_cast<const float4 *>(&t[(N - k) * XROWS + 2 * j]);
            v[i] = make_float2(ab.x + ab.w, -ab.y + ab.z);
        } else {
            const bool lo = (r == 0);
            const float4 ab = *reinterpret_cast<const float4 *>(&t[(lo ? 128 : N - k) * XROWS + 2 * j]);
            v[i] = lo ? make_float2(ab.x - ab.w, ab.y + ab.z) : make_float2(ab.x + ab.w, -ab.y + ab.z);
        }
    }
}

// Separation of a transformed row pair Z = FFT(a + i b) into the rows' half spectra,
// X_a(k) = (Z(k) + conj Z(-k))/2 (row 2p) and X_b(k) = (Z(k) - conj Z(-k))/(2i) (row 2p + 1),
// from the exchange slots z[k*16 + p] into the output tile o[kx][32].  A thread takes pair
// p = tid % 16 at kx = tid/16 + 16 q and writes both rows with one 16-byte store; kx = 128 falls
// to the first 16 threads.
__device__ __forceinline__ void separate_pairs(const float2 *__restrict__ z, float2 *__restrict__ o, int tid)
{
    const int p = tid & 15, k0 = tid >> 4;
    auto one = [&](int kx) {
        const float2 P = z[kx * 16 + p];
        const float2 Q = z[((N - kx) & (N - 1)) * 16 + p];
        *reinterpret_cast<float4 *>(&o[kx * XROWS + 2 * p]) =
            make_float4(0.5f * (P.x + Q.x), 0.5f * (P.y - Q.y), 0.5f * (P.y + Q.y), 0.5f * (Q.x - P.x));
    };
#pragma unroll
    for (int q = 0; q < 8; ++q) one(k0 + 16 * q);
    if (k0 == 0) one(128);
}

// Forward transform of the packed row pair and separation of the two rows' half spectra into
// out (v is overwritten).
template <typename AT>
__device__ __forceinline__ void x_fwd_store(float2 (&v)[16], float2 *__restrict__ out, int r, int j,
                                            const float2 *s_tw, AT &&at, float2 *s_x, long long sbase, int KX, int Y)
{
    fft256<false>(v, r, s_tw, at);
#pragma unroll
    for (int i = 0; i < 16; ++i) s_x[(r + 16 * i) * 16 + j] = v[i];
    __syncthreads();
    // a thread takes pair p = tid % 16 at kx = tid / 16 + 16 q and writes both rows (2p, 2p + 1)
    // with one 16-byte store: a half-warp covers the 256 contiguous bytes of one kx row
    const int p = threadIdx.x & 15, k0 = threadIdx.x >> 4;
    float2 *o = out + sbase + (long long)k0 * Y + 2 * p;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int kx = k0 + 16 * q;
        const float2 P = s_x[kx * 16 + p];
        const float2 Q = s_x[((N - kx) & (N - 1)) * 16 + p];
        *reinterpret_cast<float4 *>(o + (long long)(16 * q) * Y) =
            make_float4(0.5f * (P.x + Q.x), 0.5f * (P.y - Q.y), 0.5f * (P.y + Q.y), 0.5f * (Q.x - P.x));
    }
    if (k0 == 0) { // kx = 128
        const float2 P = s_x[128 * 16 + p];
        *reinterpret_cast<float4 *>(out + sbase + 128LL * Y + 2 * p) =
            make_float4(0.5f * (P.x + P.x), 0.5f * (P.y - P.y), 0.5f * (P.y + P.y), 0.5f * (P.x - P.x));
    }
    __syncthreads();
    (void)KX;
}

// Pointwise polynomial of the packed row pair, forward transform and separation
// of the two rows' half spectra into out[grp] (v is overwritten).
template <typename AT>
__device__ __forceinline__ void xpoint_fwd_store(float2 (&v)[16], const XPassArgs<float> &a, int grp,
                                                 const float *s_poly, int r, int j, const float2 *s_tw, AT &&at,
                                                 float2 *s_x, long long sbase, int KX, int Y)
{
    if (!a.identity) {
        const int d = a.pw.deg[grp];
        const float *cf = s_poly + grp * (GOPF_MAX_DEG + 1);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            float px, py;
            if (d >= 0) {
                px = cf[d];
                py = cf[d];
                for (int q = d - 1; q >= 0; --q) {
                    px = px * v[i].x + cf[q];
                    py = py * v[i].y + cf[q];
                }
            } else {
                px = polyf<float>(a.pw, grp, v[i].x);
                py = polyf<float>(a.pw, grp, v[i].y);
            }
            v[i] = make_float2(px, py);
        }
    }
    x_fwd_store(v, a.out[grp], r, j, s_tw, at, s_x, sbase, KX, Y);
}


// NG == 1: one output group, transformed in place; NG == 0: any number of groups
template <int NG>
__global__ void __launch_bounds__(NT, 2) k_x256(const XPassArgs<float> a)
{
    // spectral tile [129][32] during c2r input, then exchange slots [256][16]
    __shared__ __align__(16) float2 s_x[N * 16 + 64];
    __shared__ float2 s_tw[N];
    __shared__ float s_poly[GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1)];
    const Geom &g = a.g;
    const int j = threadIdx.x & 15, r = threadIdx.x >> 4;
    for (int t = threadIdx.x; t < GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1); t += NT)
        s_poly[t] = (float)a.pw.dense[t / (GOPF_MAX_DEG + 1)][t % (GOPF_MAX_DEG + 1)];
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
    load_pair_line(s_x, r, j, v);
    __syncthreads();
    auto at = [&](int x, int y) -> float2 & { return s_x[(x * 16 + y) * 16 + j]; };
    fft256<true>(v, r, s_tw, at);
    // v[i] = c(row 2j, col r + 16 i) + i c(row 2j+1, col r + 16 i)
    if (NG == 1) {
        xpoint_fwd_store(v, a, 0, s_poly, r, j, s_tw, at, s_x, sbase, KX, Y);
    } else {
        for (int grp = 0; grp < a.ngrp_out; ++grp) {
            float2 w[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) w[i] = v[i];
            xpoint_fwd_store(w, a, grp, s_poly, r, j, s_tw, at, s_x, sbase, KX, Y);
        }
    }
}


// ---------------------------------------------------------------------------
// x axis with TMA tiles.  The block's input is the [129 kx][32 y] half
// spectrum of 32 rows of one depth plane (one 3D tensor copy); each output
// group's [129][32] tile is assembled in shared memory by the separation step
// and leaves as one tensor store.  Per thread, the separation works on a fixed
// row y = tid mod 32 and kx = tid/32 + 8 q, so no index arithmetic is 64-bit.
// Tensor map: [Z][KX][Y] of 8-byte elements, box {32, KX, 1}.
// ---------------------------------------------------------------------------
constexpr int XT_TILE_BYTES = 129 * XROWS * 8;          // 33,024
constexpr int XT_XCH_BYTES = (N * 16 + 64) * 8;         // exchange slots [256][16] (+ pad)

__host__ __device__ constexpr int x256_tma_smem_bytes()
{
    return 128 + XT_XCH_BYTES + XT_TILE_BYTES + N * 8 + GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1) * 4 + 16;
}

// g(c) on both packed rows at once: Horner on FP32x2 pairs (one FFMA2 per degree), rounding
// exactly as the scalar Horner of each component
template <int D> __device__ __forceinline__ void poly_regs(float2 (&v)[16], const float *cf)
{
    float2 c[GOPF_MAX_DEG + 1];
#pragma unroll
    for (int q = 0; q <= D; ++q) c[q] = make_float2(cf[q], cf[q]);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        float2 acc = c[D];
#pragma unroll
        for (int q = D - 1; q >= 0; --q) acc = __ffma2_rn(acc, v[i], c[q]);
        v[i] = acc;
    }
}

// g(c) of group grp on both packed rows, with the degree resolved once per block
__device__ __forceinline__ void apply_poly(float2 (&v)[16], const XPassArgs<float> &a, int grp, const float *cf)
{
    switch (a.pw.deg[grp]) {
    case 0: poly_regs<0>(v, cf); return;
    case 1: poly_regs<1>(v, cf); return;
    case 2: poly_regs<2>(v, cf); return;
    case 3: poly_regs<3>(v, cf); return;
    case 4: poly_regs<4>(v, cf); return;
    case 5: poly_regs<5>(v, cf); return;
    case 6: poly_regs<6>(v, cf); return;
    default: break;
    }
    const int d = a.pw.deg[grp];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        float px, py;
        if (d >= 0) {
            px = cf[d];
            py = cf[d];
            for (int q = d - 1; q >= 0; --q) {
                px = px * v[i].x + cf[q];
                py = py * v[i].y + cf[q];
            }
        } else {
            px = polyf<float>(a.pw, grp, v[i].x);
            py = polyf<float>(a.pw, grp, v[i].y);
        }
        v[i] = make_float2(px, py);
    }
}

template <int NG>
__global__ void __launch_bounds__(NT, 3)
    k_x256_tma(const XPassArgs<float> a, const __grid_constant__ CUtensorMap mIn, const __grid_constant__ CUtensorMap mO0,
               const __grid_constant__ CUtensorMap mO1, const __grid_constant__ CUtensorMap mO2,
               const __grid_constant__ CUtensorMap mO3)
{
    pdl_trigger(); // the forward y pass may be scheduled as soon as every block runs
    extern __shared__ unsigned char x_dsm[];
    unsigned char *base = x_dsm + ((128u - (smem_u32(x_dsm) & 127u)) & 127u);
    float2 *s_x = reinterpret_cast<float2 *>(base);                        // input tile, then exchange slots
    float2 *s_o = reinterpret_cast<float2 *>(base + XT_XCH_BYTES);         // output tile [129][32]
    float2 *s_tw = reinterpret_cast<float2 *>(base + XT_XCH_BYTES + XT_TILE_BYTES);
    float *s_poly = reinterpret_cast<float *>(s_tw + N);
    uint64_t *bar = reinterpret_cast<uint64_t *>(s_poly + GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1));
    int *s_ok = reinterpret_cast<int *>(bar + 1);

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
    for (int t = tid; t < GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1); t += NT)
        s_poly[t] = (float)a.pw.dense[t / (GOPF_MAX_DEG + 1)][t % (GOPF_MAX_DEG + 1)];
    load_twiddles(s_tw, a.twX);
    if (tid == 0) *s_ok = tma_wait_or_flag(bar, 0, a.status) ? 1 : 0;
    __syncthreads();
    if (!*s_ok) return;

    // Hermitian extension, rows (2j, 2j+1) packed as a + i b
    float2 v[16];
    load_pair_line(s_x, r, j, v);
    __syncthreads();
    auto at = [&](int x, int y) -> float2 & { return s_x[(x * 16 + y) * 16 + j]; };
    fft256<true>(v, r, s_tw, at);
    // v[i] = c(row 2j, col r + 16 i) + i c(row 2j+1, col r + 16 i)

    const int ng = (NG == 1) ? 1 : a.ngrp_out;
    for (int grp = 0; grp < ng; ++grp) {
        float2 w[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) w[i] = v[i];
        if (!a.identity) apply_poly(w, a, grp, s_poly + grp * (GOPF_MAX_DEG + 1));
        fft256<false>(w, r, s_tw, at);
#pragma unroll
        for (int i = 0; i < 16; ++i) s_x[(r + 16 * i) * 16 + j] = w[i];
        if (grp > 0 && tid == 0) bulk_wait_read_all(); // the previous group's store has read s_o
        __syncthreads();
        // separation: X_a(k) = (Z(k) + conj Z(-k))/2 (even rows), X_b(k) = (Z(k) - conj Z(-k))/(2i) (odd rows)
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

// One output group (the Cahn-Hilliard x pass): the tile arrives by one TMA copy as in k_x256_tma,
// but the separated half spectra leave by coalesced stores (a warp writes 256 contiguous bytes of
// one kx row) instead of through an output tile, so a block needs no second 33 KB of shared
// memory and four blocks fit on an SM.
__host__ __device__ constexpr int x256_tl_smem_bytes()
{
    return 128 + XT_XCH_BYTES + N * 8 + GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1) * 4 + 16;
}

static __global__ void __launch_bounds__(NT, 4) k_x256_tl(const XPassArgs<float> a, const __grid_constant__ CUtensorMap mIn)
{
    extern __shared__ unsigned char xl_dsm[];
    unsigned char *base = xl_dsm + ((128u - (smem_u32(xl_dsm) & 127u)) & 127u);
    float2 *s_x = reinterpret_cast<float2 *>(base); // input tile, then exchange slots
    float2 *s_tw = reinterpret_cast<float2 *>(base + XT_XCH_BYTES);
    float *s_poly = reinterpret_cast<float *>(s_tw + N);
    uint64_t *bar = reinterpret_cast<uint64_t *>(s_poly + GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1));
    int *s_ok = reinterpret_cast<int *>(bar + 1);

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
    for (int t = tid; t < GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1); t += NT)
        s_poly[t] = (float)a.pw.dense[t / (GOPF_MAX_DEG + 1)][t % (GOPF_MAX_DEG + 1)];
    load_twiddles(s_tw, a.twX);
    if (tid == 0) *s_ok = tma_wait_or_flag(bar, 0, a.status) ? 1 : 0;
    __syncthreads();
    if (!*s_ok) return;

    float2 v[16];
    load_pair_line(s_x, r, j, v);
    __syncthreads();
    auto at = [&](int x, int y) -> float2 & { return s_x[(x * 16 + y) * 16 + j]; };
    fft256<true>(v, r, s_tw, at);
    switch (a.identity ? -1 : a.pw.deg[0]) { // the launch guarantees a dense degree <= 6
    case 0: poly_regs<0>(v, s_poly); break;
    case 1: poly_regs<1>(v, s_poly); break;
    case 2: poly_regs<2>(v, s_poly); break;
    case 3: poly_regs<3>(v, s_poly); break;
    case 4: poly_regs<4>(v, s_poly); break;
    case 5: poly_regs<5>(v, s_poly); break;
    case 6: poly_regs<6>(v, s_poly); break;
    default: break;
    }
    x_fwd_store(v, a.out[0], r, j, s_tw, at, s_x, (long long)z * a.g.S + y0, a.g.KX, a.g.Y);
}

// ---------------------------------------------------------------------------
// z axis on half-width tiles: 8 lines per block, 128 threads, the group and c-hat tiles
// 16 KB each, so six blocks share an SM (three with k_z256_tma) and more tile loads overlap
// other blocks' transforms.  One explicit group.  A thread t = 8 r + l owns radix position r of
// line l; the exchange slots of the 8 lines are padded to 132 per radix row (both exchange
// directions conflict free).  TMA boxes {8 lines, 256 z}.
// ---------------------------------------------------------------------------
constexpr int ZH_LINES = 8, ZH_NT = 128, ZH_PITCH = 16 * ZH_LINES + 4;
constexpr int ZH_TILE_BYTES = ZH_LINES * N * 8;         // 16,384
constexpr int ZH_XCH_BYTES = 16 * ZH_PITCH * 8;         // 16,896: the group tile, then the exchange

__host__ __device__ constexpr int z256_th_smem_bytes()
{
    return 128 + ZH_XCH_BYTES + ZH_TILE_BYTES + N * 8 + N * 4 + ZH_LINES * 4 + 16;
}

template <bool NZ>
__global__ void __launch_bounds__(ZH_NT, 6)
    k_z256_th(const PassArgs<float> a, const __grid_constant__ CUtensorMap mU0, const __grid_constant__ CUtensorMap mS,
              const __grid_constant__ CUtensorMap mT)
{
    extern __shared__ unsigned char zh_dsm[];
    unsigned char *base = zh_dsm + ((128u - (smem_u32(zh_dsm) & 127u)) & 127u);
    float2 *tU0 = reinterpret_cast<float2 *>(base);
    float2 *tS = reinterpret_cast<float2 *>(base + ZH_XCH_BYTES);
    float2 *s_tw = reinterpret_cast<float2 *>(base + ZH_XCH_BYTES + ZH_TILE_BYTES);
    float *s_fz = reinterpret_cast<float *>(s_tw + N);
    float *s_fl = s_fz + N;
    uint64_t *bar = reinterpret_cast<uint64_t *>(s_fl + ZH_LINES);
    int *s_ok = reinterpret_cast<int *>(bar + 1);

    const Geom &g = a.g;
    const int tid = threadIdx.x;
    const int l = tid & 7, r = tid >> 3;
    const int i0 = blockIdx.x * ZH_LINES;
    const bool init = (a.mode == PM_INIT);
    const int ngrp = (a.upd.ngrp > 0 ? 1 : 0);
    const bool pdl = (a.allow_fast & ALLOW_PDL) != 0;
    pdl_trigger();

    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    // the tiles are requested first, unless the launch is a programmatic dependent: then the
    // tables are set up while the previous kernel finishes, and the tiles requested after its end
    auto request = [&]() {
        if (tid == 0) {
            const uint32_t bytes = (uint32_t)ZH_TILE_BYTES * (1u + (init ? 0u : 1u));
            mbar_arrive_expect_tx(bar, bytes);
            tma_load_2d(tU0, &mU0, i0, 0, bar);
            if (!init) tma_load_2d(tS, &mS, i0, 0, bar);
        }
    };
    if (!pdl) request();
    for (int t = tid; t < N; t += ZH_NT) {
        s_tw[t] = a.tw[(t & 15) * (t >> 4)];
        s_fz[t] = fsqf(t, g.Z);
    }
    if (tid < ZH_LINES) {
        const int q = i0 + tid;
        const int kx = q / g.Y, y = q - kx * g.Y;
        const float fx = (float)kx / (float)g.X;
        s_fl[tid] = fx * fx + fsqf(y, g.Y);
    }
    if (pdl) {
        pdl_wait(); // every thread: the stores below touch T and c-hat
        request();
    }
    if (tid == 0) *s_ok = tma_wait_or_flag(bar, 0, a.status) ? 1 : 0;
    __syncthreads();
    if (!*s_ok) return;

    float2 v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = tU0[(r + 16 * i) * ZH_LINES + l];
    __syncthreads(); // the group tile becomes the exchange slots
    auto at = [&](int x, int y) -> float2 & { return tU0[x * ZH_PITCH + y * ZH_LINES + l]; };
    // no trailing barrier: the one before the c-hat store orders these reads before the inverse's writes
    fft256<false, false, false>(v, r, s_tw, at);

    const UpdTable &u = a.upd;
    const UpdRegs R = load_upd(u, ngrp);
    const float fourpi2 = 39.478417604357434f;
    const float fl = s_fl[l];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int k = r + 16 * i;
        float2 cn;
        if (init) {
            cn = v[i];
        } else {
            const float mk = -fourpi2 * (fl + s_fz[k]);
            float2 c0 = tS[k * ZH_LINES + l];
            if (NZ && u.noise.kind) {
                const long long q = i0 + l, kx = q / g.Y, yy = q - kx * g.Y;
                double nr, ni;
                noise_term(u.noise, g.X, g.Y, g.Z, kx, yy, k, (double)mk, nr, ni);
                c0.x += R.dt * (float)nr;
                c0.y += R.dt * (float)ni;
            }
            cn = euler_update<1>(R, c0, v[i], v[i], mk);
            if (NZ && u.filt) cn = modal_filter(u, cn, fl + s_fz[k]);
        }
        tS[k * ZH_LINES + l] = cn; // each thread rewrites exactly the elements it read
        v[i] = make_float2(cn.x * R.invN, cn.y * R.invN);
    }
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
        tma_store_2d(&mS, i0, 0, tS);
        bulk_commit();
    }
    fft256<true>(v, r, s_tw, at);
#pragma unroll
    for (int i = 0; i < 16; ++i) tU0[(r + 16 * i) * ZH_LINES + l] = v[i];
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
        tma_store_2d(&mT, i0, 0, tU0);
        bulk_commit();
        bulk_wait_read_all(); // the tiles stay allocated until both stores have read them
    }
}

// ---------------------------------------------------------------------------
// One output group on half-height tiles: 16 rows (8 packed row pairs) per block, 128 threads,
// about 19.5 KB of shared memory, so eight blocks share an SM (four with k_x256_tl) and more tile
// loads overlap other blocks' transforms.  A thread t = 8 r + j owns radix position r of row
// pair j.  The exchange slots of the 8 lines are padded to 132 per radix row so that both
// directions of the exchange are conflict free.  The tile arrives by one 3D TMA copy
// ({16 y, 129 kx, 1 z}); the separated spectra leave as 16-byte stores of a row pair.
// ---------------------------------------------------------------------------
constexpr int XH_ROWS = 16, XH_NT = 128, XH_LINES = 8, XH_PITCH = 16 * XH_LINES + 4;
constexpr int XH_TILE_BYTES = 129 * XH_ROWS * 8;       // 16,512
constexpr int XH_XCH_FLOATS2 = 16 * XH_PITCH;          // 2,112 float2 = 16,896 B >= the tile

__host__ __device__ constexpr int x256_th_smem_bytes()
{
    return 128 + XH_XCH_FLOATS2 * 8 + N * 8 + GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1) * 4 + 16;
}

static __global__ void __launch_bounds__(XH_NT, 8) k_x256_th(const XPassArgs<float> a, const __grid_constant__ CUtensorMap mIn)
{
    extern __shared__ unsigned char xh_dsm[];
    unsigned char *base = xh_dsm + ((128u - (smem_u32(xh_dsm) & 127u)) & 127u);
    float2 *s_x = reinterpret_cast<float2 *>(base); // input tile, then exchange slots
    float2 *s_tw = reinterpret_cast<float2 *>(base + XH_XCH_FLOATS2 * 8);
    float *s_poly = reinterpret_cast<float *>(s_tw + N);
    uint64_t *bar = reinterpret_cast<uint64_t *>(s_poly + GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1));
    int *s_ok = reinterpret_cast<int *>(bar + 1);

    const int tid = threadIdx.x;
    const int j = tid & 7, r = tid >> 3;
    const int y0 = blockIdx.x * XH_ROWS;
    const int z = blockIdx.y;
    pdl_trigger(); // the y pass may be scheduled as soon as every x block runs
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        mbar_arrive_expect_tx(bar, (uint32_t)XH_TILE_BYTES);
        tma_load_3d(s_x, &mIn, y0, 0, z, bar);
    }
    for (int t = tid; t < GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1); t += XH_NT)
        s_poly[t] = (float)a.pw.dense[t / (GOPF_MAX_DEG + 1)][t % (GOPF_MAX_DEG + 1)];
    for (int t = tid; t < N; t += XH_NT) s_tw[t] = a.twX[(t & 15) * (t >> 4)];
    if (tid == 0) *s_ok = tma_wait_or_flag(bar, 0, a.status) ? 1 : 0;
    __syncthreads();
    if (!*s_ok) return;

    // Hermitian extension of rows (2j, 2j+1) packed as a + i b: the tile is [129 kx][16 y]
    float2 v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int k = r + 16 * i;
        if (i < 8) {
            const float4 ab = *reinterpret_cast<const float4 *>(&s_x[k * XH_ROWS + 2 * j]);
            v[i] = make_float2(ab.x - ab.w, ab.y + ab.z);
        } else if (i > 8) {
            const float4 ab = *reinterpret_cast<const float4 *>(&s_x[(N - k) * XH_ROWS + 2 * j]);
            v[i] = make_float2(ab.x + ab.w, -ab.y + ab.z);
        } else {
            const bool lo = (r == 0);
            const float4 ab = *reinterpret_cast<const float4 *>(&s_x[(lo ? 128 : N - k) * XH_ROWS + 2 * j]);
            v[i] = lo ? make_float2(ab.x - ab.w, ab.y + ab.z) : make_float2(ab.x + ab.w, -ab.y + ab.z);
        }
    }
    __syncthreads(); // the tile becomes the exchange slots
    auto at = [&](int x, int y) -> float2 & { return s_x[x * XH_PITCH + y * XH_LINES + j]; };
    // the forward transform stores in the transposed form, into the slots each thread read at the
    // end of the inverse one: no barrier between the two
    fft256<true, false, false>(v, r, s_tw, at);
    switch (a.identity ? -1 : a.pw.deg[0]) { // the launch guarantees a dense degree <= 6
    case 0: poly_regs<0>(v, s_poly); break;
    case 1: poly_regs<1>(v, s_poly); break;
    case 2: poly_regs<2>(v, s_poly); break;
    case 3: poly_regs<3>(v, s_poly); break;
    case 4: poly_regs<4>(v, s_poly); break;
    case 5: poly_regs<5>(v, s_poly); break;
    case 6: poly_regs<6>(v, s_poly); break;
    default: break;
    }
    fft256<false, false, true, true>(v, r, s_tw, at);
    // spectrum Z(k) of line j at slot [k][j] (pitch 8 per k), then the row pairs' half spectra
#pragma unroll
    for (int i = 0; i < 16; ++i) s_x[(r + 16 * i) * XH_LINES + j] = v[i];
    __syncthreads();
    const int p = tid & 7, k0 = tid >> 3; // 16 kx per pass
    float2 *o = a.out[0] + (long long)z * a.g.S + y0 + (long long)k0 * a.g.Y + 2 * p;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int kx = k0 + 16 * q;
        const float2 P = s_x[kx * XH_LINES + p];
        const float2 Q = s_x[((N - kx) & (N - 1)) * XH_LINES + p];
        *reinterpret_cast<float4 *>(o + (long long)(16 * q) * a.g.Y) =
            make_float4(0.5f * (P.x + Q.x), 0.5f * (P.y - Q.y), 0.5f * (P.y + Q.y), 0.5f * (Q.x - P.x));
    }
    if (k0 == 0) { // kx = 128
        const float2 P = s_x[128 * XH_LINES + p];
        *reinterpret_cast<float4 *>(a.out[0] + (long long)z * a.g.S + y0 + 128LL * a.g.Y + 2 * p) =
            make_float4(P.x, 0.f, P.y, 0.f);
    }
}

} // namespace f256
} // namespace gopf
