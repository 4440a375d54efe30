// gopf_energy.cu -- energy monitors of a device-resident field.
//
// gopf's solver runs its monitors once per epoch on host fields
// (pf/solver.go:110-117, the Monitor interface of pf/monitor.go:4-6).  These
// two monitors run on the device instead, on the field where it lives, and
// return a few FP64 numbers:
//
// * gopf_free_energy: F = sum_cells sum_p a_p c^p + (kappa/2) sum_cells |grad c|^2.
//   The gradient part comes from the half spectrum by Parseval,
//   sum_cells |grad c|^2 = (1/N) sum_k |k|^2 |c-hat(k)|^2 with k = 2 pi Freq (the
//   symbol the model's LAP uses, pf/diffOp.go:25-30, Nyquist at +1/2), each
//   stored half-spectrum mode counted twice unless it is its own partner
//   (kx = 0 or kx = X/2).  With a = (0, 0, -1/2, 0, 1/4) and kappa = gamma this
//   is the Cahn-Hilliard free energy whose variational derivative is the
//   chemical potential of examples/cahnHilliard/main.go:33.
//
// * gopf_elastic_energy: elasticity.HomogeneousModulusEnergy
//   (elasticity/linearElasticity.go:101-165) of an indicator x (the field, or
//   3c^2 - 2c^3 of it): the effective force of the misfit stress A = C:eps*
//   (elasticity/effectiveForce.go:26-35), the displacement solve
//   (Displacements, :33-63, no Nyquist zeroing), the six strains (Strain,
//   :67-83, Nyquist components of f zeroed), the misfit subtracted where the
//   indicator exceeds 1/2, the energy density (:86-98) summed and divided by
//   sum x.  Every strain is linear in x-hat: eps-hat_mn(k) = x-hat(k) s_mn(k),
//   s_mn = (f~_n v_m + f~_m v_n)/2, v = Gamma'(f)^-1 A f,
//   Gamma'_mn = sum_jl C_mjnl f_j f_l.  The reference keeps real(IFFT(.)), which
//   for a real x is the inverse transform of the part of x-hat s that is
//   Hermitian, i.e. of x-hat (s(k) + s(-k))/2: the symbol is symmetrised here so
//   the strains can use the real-to-complex passes.
//
// All sums are FP64: each thread adds its cells' terms (FP32 terms 16 at a
// time in FP32 first, CellSum), and the threads' and blocks' partial sums are
// combined with Neumaier compensation.  The fields, transforms and per-cell
// terms are in the context's precision.  Work buffers are allocated on the
// first call and kept with the context.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>

#include "gopf_ctx.h"
#include "gopf_kernels.cuh"

using namespace gopf;

struct gopf_energy_work {
    double *part = nullptr; // block partials [EN_BLOCKS][EN_SLOTS]
    double *out = nullptr;  // finished sums [EN_SLOTS]
    void *xh = nullptr;     // half spectrum of the indicator
    void *bh = nullptr;     // half spectra of the six strain components (6 C)
    void *ind = nullptr;    // real indicator (N)
    void *strain = nullptr; // six real strain fields (6 N)
};

int gopf_field_to_real(gopf_ctx *ctx, int f, void *dst);

namespace {

constexpr int EN_BLOCKS = 152 * 8;
// The summing kernels' grid: one wave of four blocks per SM on 152 SMs (with several loads in
// flight per thread), so that their FP64 block epilogue (block_store) runs as few times as
// possible: FP64 instructions are expensive on this GPU
constexpr int EN_BULK_BLOCKS = 152 * 4;
constexpr int EN_SLOTS = 4;
constexpr int EN_THREADS = 256;
constexpr int EN_MAX_DEG = 12;

__device__ __forceinline__ void nadd(double &s, double &c, double v)
{
    const double t = s + v;
    c += (fabs(s) >= fabs(v)) ? (s - t) + v : (v - t) + s;
    s = t;
}

// A thread's running sum of per-cell terms in FP64.  FP32 terms are added 16 at a time in FP32 and
// each such partial once into the FP64 total (FP64 arithmetic runs at a small fraction of the FP32
// rate on this GPU); FP64 terms go straight into the total.
template <typename T> struct CellSum {
    double s = 0.0;
    __device__ __forceinline__ void add(T v) { s += (double)v; }
    __device__ __forceinline__ double total() const { return s; }
};
template <> struct CellSum<float> {
    double s = 0.0;
    float a = 0.f;
    int n = 0;
    __device__ __forceinline__ void add(float v)
    {
        a += v;
        if (++n == 16) {
            s += (double)a;
            a = 0.f;
            n = 0;
        }
    }
    __device__ __forceinline__ double total() const { return s + (double)a; }
};

// Block-wide compensated sum of (s, c) per slot; thread 0 writes part[blockIdx.x][slot].
template <int NS> __device__ void block_store(double (&s)[NS], double (&c)[NS], double *part)
{
    __shared__ double sh_s[EN_THREADS / 32][NS], sh_c[EN_THREADS / 32][NS];
    for (int k = 0; k < NS; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            const double so = __shfl_xor_sync(0xffffffffu, s[k], o), co = __shfl_xor_sync(0xffffffffu, c[k], o);
            c[k] += co;
            nadd(s[k], c[k], so);
        }
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0)
        for (int k = 0; k < NS; ++k) {
            sh_s[w][k] = s[k];
            sh_c[w][k] = c[k];
        }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < NS; ++k) {
            double ss = 0.0, cc = 0.0;
            for (int q = 0; q < EN_THREADS / 32; ++q) {
                cc += sh_c[q][k];
                nadd(ss, cc, sh_s[q][k]);
            }
            part[(long long)blockIdx.x * EN_SLOTS + k] = ss + cc;
        }
}

struct BulkPoly {
    int deg;
    double a[EN_MAX_DEG + 1];
};

// slot 0: sum of the polynomial, slot 2: non-finite cells (slot 1 unused).  A thread adds its cells'
// values with CellSum (at most ceil(n / (EN_BLOCKS EN_THREADS)) of them, 54 at 256^3); the threads'
// and blocks' partial sums are combined with Neumaier compensation.  An FP32 field's polynomial is
// evaluated in FP32 (the cell value itself is FP32), an FP64 field's in FP64.
template <typename R> __global__ void k_bulk(const R *__restrict__ x, long long n, BulkPoly p, double *__restrict__ part)
{
    __shared__ R s_a[EN_MAX_DEG + 1];
    if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q <= EN_MAX_DEG; ++q) s_a[q] = (R)p.a[q];
    __syncthreads();
    double s[1] = {0.0}, c[1] = {0.0};
    CellSum<R> acc;
    unsigned bad = 0;
    auto cell = [&](R v) {
        R h = s_a[p.deg];
        for (int q = p.deg - 1; q >= 0; --q) h = h * v + s_a[q];
        acc.add(h);
        bad += isfinite(v) ? 0u : 1u;
    };
    // 16-byte loads, four per thread in flight (the field is a cudaMalloc'd array: 16-byte aligned)
    typedef typename std::conditional<sizeof(R) == 4, float4, double2>::type Q;
    constexpr int PER = 16 / (int)sizeof(R), U = 4;
    const Q *xq = reinterpret_cast<const Q *>(x);
    const long long nq = n / PER, stride = (long long)gridDim.x * blockDim.x;
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; i + (U - 1) * stride < nq; i += U * stride) {
        Q w[U];
#pragma unroll
        for (int u = 0; u < U; ++u) w[u] = xq[i + u * stride];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const R *e = reinterpret_cast<const R *>(&w[u]);
#pragma unroll
            for (int k = 0; k < PER; ++k) cell(e[k]);
        }
    }
    for (; i < nq; i += stride) {
        const Q w = xq[i];
        const R *e = reinterpret_cast<const R *>(&w);
#pragma unroll
        for (int k = 0; k < PER; ++k) cell(e[k]);
    }
    for (long long j = nq * PER + blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += stride) cell(x[j]);
    // the non-finite count as an integer, the polynomial sum compensated (slot 0)
    __shared__ unsigned s_bad;
    if (threadIdx.x == 0) s_bad = 0;
    __syncthreads();
    const unsigned wbad = __reduce_add_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0 && wbad) atomicAdd(&s_bad, wbad);
    s[0] = acc.total();
    block_store<1>(s, c, part); // its barrier orders the count above
    if (threadIdx.x == 0) {
        part[(long long)blockIdx.x * EN_SLOTS + 1] = 0.0;
        part[(long long)blockIdx.x * EN_SLOTS + 2] = (double)s_bad;
        part[(long long)blockIdx.x * EN_SLOTS + 3] = 0.0;
    }
}

// fold(i, n)^2, from the reciprocal of n
template <typename T> __device__ __forceinline__ T fold2(int i, int n, T inv_n)
{
    const T f = (T)(2 * i > n ? i - n : i) * inv_n;
    return f * f;
}

// slot 0: sum over the full spectrum of |f|^2 |c-hat|^2 (f in cycles per sample).  A block takes
// whole lines (z, kx) of the half spectrum, its threads the y positions; per-thread partial sums by
// CellSum, combined with Neumaier compensation.  An FP32 spectrum's terms are formed in FP32.
template <typename V> __global__ void k_grad(const V *__restrict__ st, Geom g, double *__restrict__ part)
{
    typedef decltype(V().x) T;
    double s[1] = {0.0}, c[1] = {0.0};
    CellSum<T> acc;
    const T iy = (T)1 / (T)g.Y, ix = (T)1 / (T)g.X, iz = (T)1 / (T)g.Z;
    const long long nlines = (long long)g.Z * g.KX;
    // four lines per round, so that each thread has four loads in flight
    constexpr int U = 4;
    for (long long l0 = blockIdx.x; l0 < nlines; l0 += U * (long long)gridDim.x) {
        T fl[U], wt[U];
#pragma unroll
        for (int u = 0; u < U; ++u) { // a line's x and z frequencies and its Hermitian weight (0: no line)
            const long long line = l0 + u * (long long)gridDim.x;
            const int li = (int)line, z = li / g.KX, kx = li - z * g.KX; // Z KX < 2^31 lines
            fl[u] = fold2<T>(kx, g.X, ix) + fold2<T>(z, g.Z, iz);
            wt[u] = line >= nlines ? (T)0 : (kx == 0 || 2 * kx == g.X) ? (T)1 : (T)2;
        }
        for (int y = threadIdx.x; y < g.Y; y += blockDim.x) {
            V v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const long long line = l0 + u * (long long)gridDim.x;
                v[u] = line < nlines ? st[line * g.Y + y] : V();
            }
            const T fy = fold2<T>(y, g.Y, iy);
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (wt[u] != (T)0) acc.add(wt[u] * (fy + fl[u]) * (v[u].x * v[u].x + v[u].y * v[u].y));
        }
    }
    s[0] = acc.total();
    block_store<1>(s, c, part);
}

// one block per slot (EN_SLOTS blocks, so that the FP64 chains run on separate SMs): compensated
// sum of the block partials of that slot (each thread over its partials, then a shuffle tree and
// the warps' results in order, all with Neumaier compensation)
__global__ void k_finish(const double *__restrict__ part, int nblocks, double *__restrict__ out)
{
    __shared__ double sh_s[32], sh_c[32];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, k = blockIdx.x;
    double s = 0.0, c = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) nadd(s, c, part[(long long)b * EN_SLOTS + k]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double so = __shfl_xor_sync(0xffffffffu, s, o), co = __shfl_xor_sync(0xffffffffu, c, o);
        c += co;
        nadd(s, c, so);
    }
    if (lane == 0) {
        sh_s[wp] = s;
        sh_c[wp] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ss = 0.0, cc = 0.0;
        for (int q = 0; q < (int)blockDim.x / 32; ++q) {
            cc += sh_c[q];
            nadd(ss, cc, sh_s[q]);
        }
        out[k] = ss + cc;
    }
}

template <typename R> __global__ void k_indicator(R *__restrict__ x, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double v = (double)x[i];
        x[i] = (R)(3.0 * v * v - 2.0 * v * v * v); // Indicator, pf/homoLinElast.go:10-12
    }
}

struct StrainParams {
    double C[81];
    double A[9];     // C : misfit
    double mis[9];   // misfit strain
    double scale;    // 1/N
};

// The same constants in the precision the per-cell terms are formed in (the context's)
template <typename T> struct StrainConsts {
    T C[81];
    T A[9];
    T mis[9];
    T scale;
};

template <typename T> StrainConsts<T> consts_of(const StrainParams &p)
{
    StrainConsts<T> q;
    for (int i = 0; i < 81; ++i) q.C[i] = (T)p.C[i];
    for (int i = 0; i < 9; ++i) {
        q.A[i] = (T)p.A[i];
        q.mis[i] = (T)p.mis[i];
    }
    q.scale = (T)p.scale;
    return q;
}

// v = Gamma'(f)^-1 A f (0 at f = 0, as Displacements leaves the zero mode), Gaussian elimination
// with partial pivoting.  zero: f is the zero mode (the reference tests |f_i| < 1e-10; the indices
// decide it here)
template <typename T> __device__ __forceinline__ void disp_dir(const StrainConsts<T> &p, const T f[3], bool zero, T v[3])
{
    v[0] = v[1] = v[2] = (T)0;
    if (zero) return;
    T G[3][3], b[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            T e = (T)0;
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int l = 0; l < 3; ++l) e += p.C[m * 27 + j * 9 + n * 3 + l] * f[j] * f[l];
            G[m][n] = e;
        }
        b[m] = p.A[m * 3 + 0] * f[0] + p.A[m * 3 + 1] * f[1] + p.A[m * 3 + 2] * f[2];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        int best = c;
        T bv = fabs(G[c][c]);
#pragma unroll
        for (int r = c + 1; r < 3; ++r)
            if (fabs(G[r][c]) > bv) {
                bv = fabs(G[r][c]);
                best = r;
            }
        // swap rows c and best (selects keep the arrays in registers)
#pragma unroll
        for (int r = c + 1; r < 3; ++r)
            if (best == r) {
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const T t = G[c][k];
                    G[c][k] = G[r][k];
                    G[r][k] = t;
                }
                const T t = b[c];
                b[c] = b[r];
                b[r] = t;
            }
#pragma unroll
        for (int r = c + 1; r < 3; ++r) {
            const T fct = G[r][c] / G[c][c];
#pragma unroll
            for (int k = c; k < 3; ++k) G[r][k] -= fct * G[c][k];
            b[r] -= fct * b[c];
        }
    }
#pragma unroll
    for (int r = 2; r >= 0; --r) {
        T t = b[r];
#pragma unroll
        for (int q = r + 1; q < 3; ++q) t -= G[r][q] * v[q];
        v[r] = t / G[r][r];
    }
}

// strain symbol s_mn(f) = (f~_n v_m + f~_m v_n)/2, f~ with its Nyquist components zeroed (Strain;
// the reference tests ||f_i| - 1/2| < 1e-10, ny[i] is that test on the index)
template <typename T> __device__ __forceinline__ T strain_symbol(const T f[3], const bool ny[3], const T v[3], int m, int n)
{
    const T fm = ny[m] ? (T)0 : f[m];
    const T fn = ny[n] ? (T)0 : f[n];
    return (T)0.5 * (fn * v[m] + fm * v[n]);
}

// index i on an axis of n points in cycles per sample (Nyquist at +1/2), from the reciprocal of n
template <typename T> __device__ __forceinline__ T fold_t(int i, int n, T inv_n) { return (T)(2 * i > n ? i - n : i) * inv_n; }

// strain component q = 00 01 02 11 12 22 -> (m, n)
__host__ __device__ constexpr int strain_m(int q) { return q < 3 ? 0 : q < 5 ? 1 : 2; }
__host__ __device__ constexpr int strain_n(int q) { return q < 3 ? q : q < 5 ? q - 2 : 2; }

// out[q] = x-hat * (s_mn(k) + s_mn(-k)) / 2 / N for the six components q = 00 01 02 11 12 22 (out[q] at
// out + q C).  v(f) and v(-f) are solved once per mode for all six.  A block takes whole lines (z, kx)
// of the half spectrum, its threads the y positions.
template <typename V> __global__ void k_strain6(const V *__restrict__ xh, Geom g, int ndim, StrainConsts<decltype(V().x)> p,
                                               V *__restrict__ out)
{
    typedef decltype(V().x) T;
    const T iy = (T)1 / (T)g.Y, ix = (T)1 / (T)g.X, iz = (T)1 / (T)g.Z;
    const long long nlines = (long long)g.Z * g.KX;
    for (long long line = blockIdx.x; line < nlines; line += gridDim.x) {
        const int li = (int)line, z = li / g.KX, kx = li - z * g.KX; // Z KX < 2^31 lines
        // the reference's order: f[0] row, f[1] col, f[2] depth (0 in 2D: its 3-vector wrapper)
        const T fx = fold_t<T>(kx, g.X, ix), fxm = fold_t<T>((g.X - kx) % g.X, g.X, ix);
        const T fz = ndim == 3 ? fold_t<T>(z, g.Z, iz) : (T)0, fzm = ndim == 3 ? fold_t<T>((g.Z - z) % g.Z, g.Z, iz) : (T)0;
        const bool nyx = 2 * kx == g.X, nyz = ndim == 3 && 2 * z == g.Z; // a mode and its partner alike
        const bool zxz = kx == 0 && (ndim != 3 || z == 0);
        for (int y = threadIdx.x; y < g.Y; y += blockDim.x) {
            const T f[3] = {fold_t<T>(y, g.Y, iy), fx, fz};
            const T fm[3] = {fold_t<T>((g.Y - y) % g.Y, g.Y, iy), fxm, fzm};
            const bool ny[3] = {2 * y == g.Y, nyx, nyz};
            T v[3], vm[3];
            disp_dir<T>(p, f, zxz && y == 0, v);
            disp_dir<T>(p, fm, zxz && y == 0, vm);
            const long long idx = line * g.Y + y;
            const V xv = xh[idx];
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const T sq = (T)0.5 * (strain_symbol<T>(f, ny, v, strain_m(q), strain_n(q)) +
                                      strain_symbol<T>(fm, ny, vm, strain_m(q), strain_n(q))) * p.scale;
                V o;
                o.x = xv.x * sq;
                o.y = xv.y * sq;
                out[(long long)q * g.C + idx] = o;
            }
        }
    }
}

// slot 0: sum of the energy density, slot 1: sum of x; components in the order 00 01 02 11 12 22.
// The density is formed in the field's precision; per-thread sums by CellSum, combined with
// Neumaier compensation.
template <typename R>
__global__ void k_elastic_density(const R *__restrict__ x, const R *__restrict__ strain, long long n, StrainConsts<R> p,
                                  double *__restrict__ part)
{
    double s[2] = {0.0, 0.0}, c[2] = {0.0, 0.0};
    CellSum<R> ad, ax;
    const int ci[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
#pragma unroll 2 // two cells' seven loads in flight
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const R xv = x[i];
        const bool inside = xv > (R)0.5;
        R e[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) e[q] = strain[q * n + i];
        R E[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) E[a][b] = e[ci[a][b]] - (inside ? p.mis[a * 3 + b] : (R)0);
        R d = (R)0;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                R t = (R)0;
#pragma unroll
                for (int k = 0; k < 3; ++k)
#pragma unroll
                    for (int l = 0; l < 3; ++l) t += p.C[a * 27 + b * 9 + k * 3 + l] * E[k][l];
                d += E[a][b] * t;
            }
        ad.add((R)0.5 * d);
        ax.add(xv);
    }
    s[0] = ad.total();
    s[1] = ax.total();
    block_store<2>(s, c, part);
}

int ck(gopf_ctx *ctx, cudaError_t e, const char *where)
{
    if (e == cudaSuccess) return GOPF_OK;
    return gopf_fail(ctx, e == cudaErrorMemoryAllocation ? GOPF_ERR_OOM : GOPF_ERR_CUDA,
                     std::string(where) + ": " + cudaGetErrorString(e));
}

int prepare(gopf_ctx *ctx, int field)
{
    if (!ctx) return GOPF_ERR_ARG;
    if (ctx->device < 0) return gopf_fail(ctx, GOPF_ERR_STATE, "host-only context (device < 0)");
    if (field < 0 || (ctx->nfields > 0 && field >= ctx->nfields) || (ctx->nfields == 0 && field != 0))
        return gopf_fail(ctx, GOPF_ERR_ARG, "bad field id");
    if (!ctx->state_valid) return gopf_fail(ctx, GOPF_ERR_STATE, "field has not been uploaded");
    int rc;
    if ((rc = ck(ctx, cudaSetDevice(ctx->device), "cudaSetDevice"))) return rc;
    if (!ctx->energy) ctx->energy = new gopf_energy_work();
    gopf_energy_work *w = ctx->energy;
    if (!w->part) {
        if ((rc = ck(ctx, gopf_malloc(&w->part, sizeof(double) * EN_BLOCKS * EN_SLOTS), "gopf_malloc"))) return rc;
        if ((rc = ck(ctx, gopf_malloc(&w->out, sizeof(double) * EN_SLOTS), "gopf_malloc"))) return rc;
        ctx->dev_bytes += sizeof(double) * (EN_BLOCKS + 1) * EN_SLOTS;
    }
    return GOPF_OK;
}

unsigned grid_for(long long n) { return (unsigned)std::min<long long>((n + EN_THREADS - 1) / EN_THREADS, EN_BLOCKS); }

// finish the partials of the last kernel and copy the sums to the host (stream-synchronising)
int finish(gopf_ctx *ctx, double *host, int nblocks = EN_BLOCKS)
{
    gopf_energy_work *w = ctx->energy;
    k_finish<<<EN_SLOTS, 128, 0, ctx->stream>>>(w->part, nblocks, w->out);
    int rc;
    if ((rc = ck(ctx, cudaGetLastError(), "finish"))) return rc;
    if ((rc = ck(ctx, cudaMemcpyAsync(host, w->out, sizeof(double) * EN_SLOTS, cudaMemcpyDeviceToHost, ctx->stream),
                 "D2H")))
        return rc;
    return ck(ctx, cudaStreamSynchronize(ctx->stream), "sync");
}

template <typename R> XPassArgs<R> xbase(gopf_ctx *ctx)
{
    typedef typename VecOf<R>::type V;
    XPassArgs<R> a;
    memset(&a, 0, sizeof(a));
    a.g = ctx->g;
    a.planH = ctx->planH;
    a.twX = (const V *)ctx->d_twX;
    a.allow_fast = ctx->use_fast;
    a.status = ctx->d_status;
    return a;
}

template <typename R> PassArgs<R> pbase(gopf_ctx *ctx, bool zaxis, int mode, void *buf)
{
    typedef typename VecOf<R>::type V;
    PassArgs<R> a;
    memset(&a, 0, sizeof(a));
    a.g = ctx->g;
    a.plan = zaxis ? ctx->planZ : ctx->planY;
    a.tw = (const V *)(zaxis ? ctx->d_twZ : ctx->d_twY);
    a.mode = mode;
    a.buf[0] = (V *)buf;
    a.nbuf = 1;
    a.allow_fast = ctx->use_fast;
    a.status = ctx->d_status;
    return a;
}

template <typename R> int free_energy_impl(gopf_ctx *ctx, int field, const BulkPoly &p, double kappa, double *out3)
{
    typedef typename VecOf<R>::type V;
    const Geom &g = ctx->g;
    gopf_energy_work *w = ctx->energy;
    int rc;
    if ((rc = gopf_field_to_real(ctx, field, ctx->d_real))) return rc;
    k_bulk<R><<<EN_BULK_BLOCKS, EN_THREADS, 0, ctx->stream>>>((const R *)ctx->d_real, g.N, p, w->part);
    if ((rc = ck(ctx, cudaGetLastError(), "bulk sums"))) return rc;
    double bulk[EN_SLOTS];
    if ((rc = finish(ctx, bulk, EN_BULK_BLOCKS))) return rc;
    k_grad<V><<<EN_BULK_BLOCKS, EN_THREADS, 0, ctx->stream>>>((const V *)field_state(ctx, field), g, w->part);
    if ((rc = ck(ctx, cudaGetLastError(), "gradient sums"))) return rc;
    double grad[EN_SLOTS];
    if ((rc = finish(ctx, grad, EN_BULK_BLOCKS))) return rc;
    const double fourpi2 = 39.47841760435743;
    out3[0] = bulk[0];
    out3[1] = 0.5 * kappa * fourpi2 * grad[0] / (double)g.N;
    out3[2] = out3[0] + out3[1];
    if (bulk[2] != 0.0) return gopf_fail(ctx, GOPF_ERR_NAN, "the field holds non-finite values");
    return GOPF_OK;
}

template <typename R> int elastic_energy_impl(gopf_ctx *ctx, int field, int indicator, StrainParams p, double *out)
{
    typedef typename VecOf<R>::type V;
    const Geom &g = ctx->g;
    gopf_energy_work *w = ctx->energy;
    int rc;
    if (!w->xh) {
        if ((rc = ck(ctx, gopf_malloc(&w->xh, sizeof(V) * g.C), "gopf_malloc"))) return rc;
        if ((rc = ck(ctx, gopf_malloc(&w->bh, sizeof(V) * 6 * g.C), "gopf_malloc"))) return rc;
        if ((rc = ck(ctx, gopf_malloc(&w->ind, sizeof(R) * g.N), "gopf_malloc"))) return rc;
        if ((rc = ck(ctx, gopf_malloc(&w->strain, sizeof(R) * 6 * g.N), "gopf_malloc"))) return rc;
        ctx->dev_bytes += 7 * sizeof(V) * g.C + 7 * sizeof(R) * g.N;
    }
    // the indicator x in real space
    if ((rc = gopf_field_to_real(ctx, field, w->ind))) return rc;
    if (indicator) {
        k_indicator<R><<<grid_for(g.N), EN_THREADS, 0, ctx->stream>>>((R *)w->ind, g.N);
        if ((rc = ck(ctx, cudaGetLastError(), "indicator"))) return rc;
    }
    // x-hat
    XPassArgs<R> xa = xbase<R>(ctx);
    xa.in_mode = XIN_REAL;
    xa.rin = (const R *)w->ind;
    xa.out[0] = (V *)w->xh;
    xa.ngrp_out = 1;
    xa.identity = 1;
    if ((rc = ck(ctx, launch_xpass<R>(xa, ctx->LBx, ctx->stream), "x pass"))) return rc;
    if ((rc = ck(ctx, launch_cpass<R>(pbase<R>(ctx, false, PM_FWD, w->xh), ctx->LBy, ctx->stream), "y pass"))) return rc;
    if (g.Z > 1 &&
        (rc = ck(ctx, launch_spass<R>(pbase<R>(ctx, true, PM_FWD, w->xh), ctx->LBz, ctx->stream), "z pass")))
        return rc;
    // the six strains: symbols times x-hat / N (one kernel for all six), then each inverse
    // transformed to real rows
    p.scale = 1.0 / (double)g.N;
    const StrainConsts<R> pc = consts_of<R>(p);
    {
        const long long nl = (long long)g.Z * g.KX;
        const unsigned nb = (unsigned)std::min<long long>(nl, (long long)EN_BLOCKS * 4);
        k_strain6<V><<<nb, EN_THREADS, 0, ctx->stream>>>((const V *)w->xh, g, ctx->ndim, pc, (V *)w->bh);
        if ((rc = ck(ctx, cudaGetLastError(), "strain symbols"))) return rc;
    }
    for (int q = 0; q < 6; ++q) {
        V *bq = (V *)w->bh + (long long)q * g.C;
        if (g.Z > 1 &&
            (rc = ck(ctx, launch_spass<R>(pbase<R>(ctx, true, PM_INV, bq), ctx->LBz, ctx->stream), "z pass")))
            return rc;
        if ((rc = ck(ctx, launch_cpass<R>(pbase<R>(ctx, false, PM_INV, bq), ctx->LBy, ctx->stream), "y pass")))
            return rc;
        XPassArgs<R> xo = xbase<R>(ctx);
        xo.in_mode = XIN_SPECTRAL;
        xo.in = (const V *)bq;
        xo.rout = (R *)w->strain + (long long)q * g.N;
        if ((rc = ck(ctx, launch_xpass<R>(xo, ctx->LBx, ctx->stream), "x pass"))) return rc;
    }
    k_elastic_density<R><<<EN_BULK_BLOCKS, EN_THREADS, 0, ctx->stream>>>((const R *)w->ind, (const R *)w->strain, g.N, pc,
                                                                     w->part);
    if ((rc = ck(ctx, cudaGetLastError(), "energy density"))) return rc;
    double sums[EN_SLOTS];
    if ((rc = finish(ctx, sums, EN_BULK_BLOCKS))) return rc;
    if (!(sums[1] != 0.0)) return gopf_fail(ctx, GOPF_ERR_ARG, "the indicator sums to zero (no volume)");
    *out = sums[0] / sums[1];
    return GOPF_OK;
}

} // namespace

void gopf_energy_free(gopf_ctx *ctx)
{
    gopf_energy_work *w = ctx->energy;
    if (!w) return;
    void *ptrs[] = {w->part, w->out, w->xh, w->bh, w->ind, w->strain};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    delete w;
    ctx->energy = nullptr;
}

extern "C" int gopf_free_energy(gopf_ctx *ctx, int field, const double *coefs, int ncoefs, double kappa, double *out3)
{
    int rc;
    if ((rc = prepare(ctx, field))) return rc;
    if (!out3 || (ncoefs > 0 && !coefs)) return gopf_fail(ctx, GOPF_ERR_ARG, "null argument");
    if (ncoefs < 0 || ncoefs > EN_MAX_DEG + 1)
        return gopf_fail(ctx, GOPF_ERR_ARG, "the bulk polynomial takes 0 to 13 coefficients (degree <= 12)");
    BulkPoly p;
    memset(&p, 0, sizeof(p));
    p.deg = ncoefs > 0 ? ncoefs - 1 : 0;
    for (int q = 0; q < ncoefs; ++q) p.a[q] = coefs[q];
    gopf_nvtx_scope trace("gopf_free_energy");
    return (ctx->prec == GOPF_FP32) ? free_energy_impl<float>(ctx, field, p, kappa, out3)
                                    : free_energy_impl<double>(ctx, field, p, kappa, out3);
}

extern "C" int gopf_elastic_energy(gopf_ctx *ctx, int field, int indicator, const double *C81, const double *misfit9,
                                   double *out)
{
    int rc;
    if ((rc = prepare(ctx, field))) return rc;
    if (!C81 || !misfit9 || !out) return gopf_fail(ctx, GOPF_ERR_ARG, "null argument");
    StrainParams p;
    memset(&p, 0, sizeof(p));
    memcpy(p.C, C81, sizeof(p.C));
    memcpy(p.mis, misfit9, sizeof(p.mis));
    for (int i = 0; i < 3; ++i) // A = C : misfit (Rank4.ContractLast, elasticity/rank4.go:62-75)
        for (int j = 0; j < 3; ++j) {
            double a = 0.0;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) a += C81[i * 27 + j * 9 + k * 3 + l] * misfit9[k * 3 + l];
            p.A[i * 3 + j] = a;
        }
    gopf_nvtx_scope trace("gopf_elastic_energy");
    return (ctx->prec == GOPF_FP32) ? elastic_energy_impl<float>(ctx, field, indicator != 0, p, out)
                                    : elastic_energy_impl<double>(ctx, field, indicator != 0, p, out);
}
