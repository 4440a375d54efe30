// gopf_terms.cu -- device pieces of gopf's user-defined hot terms.
//
// Khachaturyan elasticity (pf/homoLinElast.go:47-99).  The reference
// evaluates, per step, FFT(H), the effective force (elasticity/effectiveForce.go:26-35),
// a 3x3 LU solve per frequency for the displacement
// (elasticity/linearElasticity.go:33-63), the strains (67-83) and one
// inverse + one forward transform per strain component.  All of that is
// linear in H-hat, so it collapses to a scalar symbol
//     b(k) = sum_{i<D} (A f~)_i (Gamma(f)^-1 A f)_i ,
//     Gamma_mn(f) = sum_jl C_mjnl f_j f_l ,   A = C : eps*  (elasticity/rank4.go:62-75),
// where f~ is f with Nyquist components zeroed, as Strain does.  The term is
// then FFT[ H'(c) (IFFT(b H-hat)/N - 2 e0 H(c)) ].  b is tabulated once per
// context in FP64 (this kernel) and stored in the state precision.  Because
// the reference keeps f = +0.5 for both k and -k on Nyquist planes, its b is
// not even there and its term has a small anti-Hermitian part; a real field
// can only carry the Hermitian part, which is b symmetrised over (k, -k).
//
// VolumeConservingLP (pf/volumeConserving.go:31-50): the Lagrange multiplier
// update after every step, done on the device from FP64 block sums of the
// field and of the indicator so that the step stays capturable in a graph.
#include <cmath>

#include "gopf_ctx.h"
#include "gopf_kernels.cuh"

namespace gopf {

struct ElasticParams {
    double C[81];
    double A[9];
    int ndim;
};

__device__ __forceinline__ double fold_freq(long long i, long long n)
{
    double f = (double)i / (double)n;
    return (f > 0.5) ? f - 1.0 : f;
}

__device__ double elastic_b(const ElasticParams &p, const double f[3])
{
    const double tol = 1e-10;
    if (fabs(f[0]) < tol && fabs(f[1]) < tol && fabs(f[2]) < tol) return 0.0;
    double ft[3];
    for (int d = 0; d < 3; ++d) ft[d] = (fabs(fabs(f[d]) - 0.5) < tol) ? 0.0 : f[d];
    double G[3][3], v[3];
    for (int m = 0; m < 3; ++m) {
        for (int n = 0; n < 3; ++n) {
            double e = 0.0;
            for (int j = 0; j < 3; ++j)
                for (int l = 0; l < 3; ++l) e += p.C[m * 27 + j * 9 + n * 3 + l] * f[j] * f[l];
            G[m][n] = e;
        }
        v[m] = p.A[m * 3 + 0] * f[0] + p.A[m * 3 + 1] * f[1] + p.A[m * 3 + 2] * f[2];
    }
    // Gaussian elimination with partial pivoting
    for (int c = 0; c < 3; ++c) {
        int best = c;
        for (int r = c + 1; r < 3; ++r)
            if (fabs(G[r][c]) > fabs(G[best][c])) best = r;
        if (best != c) {
            for (int k = 0; k < 3; ++k) {
                double t = G[c][k];
                G[c][k] = G[best][k];
                G[best][k] = t;
            }
            double t = v[c];
            v[c] = v[best];
            v[best] = t;
        }
        for (int r = c + 1; r < 3; ++r) {
            const double fct = G[r][c] / G[c][c];
            for (int k = c; k < 3; ++k) G[r][k] -= fct * G[c][k];
            v[r] -= fct * v[c];
        }
    }
    double u[3];
    for (int r = 2; r >= 0; --r) {
        double s = v[r];
        for (int q = r + 1; q < 3; ++q) s -= G[r][q] * u[q];
        u[r] = s / G[r][r];
    }
    double b = 0.0;
    for (int i = 0; i < p.ndim; ++i) {
        const double af = p.A[i * 3 + 0] * ft[0] + p.A[i * 3 + 1] * ft[1] + p.A[i * 3 + 2] * ft[2];
        b += af * u[i];
    }
    return b;
}

// out[z][kx][y] = (b(f) + b(f(-k))) / 2
template <typename R> __global__ void k_elastic_symbol(Geom g, ElasticParams p, R *__restrict__ out)
{
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < g.C;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long z = idx / g.S;
        const long long rem = idx - z * g.S;
        const long long kx = rem / g.Y;
        const long long y = rem - kx * g.Y;
        // reference order: f[0] row (y), f[1] col (kx), f[2] depth (z)
        double f[3] = {fold_freq(y, g.Y), fold_freq(kx, g.X), (p.ndim == 3) ? fold_freq(z, g.Z) : 0.0};
        double fm[3] = {fold_freq((g.Y - y) % g.Y, g.Y), fold_freq((g.X - kx) % g.X, g.X),
                        (p.ndim == 3) ? fold_freq((g.Z - z) % g.Z, g.Z) : 0.0};
        out[idx] = (R)(0.5 * (elastic_b(p, f) + elastic_b(p, fm)));
    }
}

__device__ __forceinline__ void vc_nadd(double &s, double &c, double v)
{
    const double t = s + v;
    c += (fabs(s) >= fabs(v)) ? (s - t) + v : (v - t) + s;
    s = t;
}

// vc = [lambda, current_integral, indicator_integral_prev, count, coef*lambda].  One block of
// VC_THREADS threads: each thread folds a strided share of both arrays' RED_SUM partials with
// Neumaier compensation, a fixed-order shuffle tree and the warps' results in order combine them
// (deterministic), and thread 0 updates the multiplier.  The FP64 dependency chain per thread stays
// short however many x-pass blocks there are (FP64 runs at a small fraction of the FP32 rate here).
constexpr int VC_THREADS = 256;
__global__ void __launch_bounds__(VC_THREADS)
    k_volcons_finalize(const double *__restrict__ red_field, const double *__restrict__ red_ind, int nblocks, double dt,
                       double coef, double *__restrict__ vc)
{
    double si = 0.0, ci = 0.0, ss = 0.0, cs = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        vc_nadd(si, ci, red_field[(long long)b * RED_SLOTS + RED_SUM]);
        vc_nadd(ss, cs, red_ind[(long long)b * RED_SLOTS + RED_SUM]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double xi = __shfl_xor_sync(0xffffffffu, si, o), xci = __shfl_xor_sync(0xffffffffu, ci, o);
        const double xs = __shfl_xor_sync(0xffffffffu, ss, o), xcs = __shfl_xor_sync(0xffffffffu, cs, o);
        ci += xci;
        vc_nadd(si, ci, xi);
        cs += xcs;
        vc_nadd(ss, cs, xs);
    }
    __shared__ double sh[4][VC_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        sh[0][w] = si;
        sh[1][w] = ci;
        sh[2][w] = ss;
        sh[3][w] = cs;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    double I = 0.0, Ic = 0.0, S = 0.0, Sc = 0.0;
    for (int q = 0; q < (int)blockDim.x / 32; ++q) {
        Ic += sh[1][q];
        vc_nadd(I, Ic, sh[0][q]);
        Sc += sh[3][q];
        vc_nadd(S, Sc, sh[2][q]);
    }
    I += Ic;
    S += Sc;
    const double count = vc[3];
    if (count == 1.0) {
        vc[1] = I; // IsFirstUpdate: remember the integral, keep the multiplier
    } else if (count >= 2.0) {
        vc[0] = vc[0] - (I - vc[1]) / (dt * vc[2]);
        vc[1] = I;
    }
    vc[2] = S;
    vc[3] = count + 1.0;
    vc[4] = coef * vc[0];
}

// Hermitian projection of the self-conjugate planes kx = 0 and (even X) kx = X/2 of the
// half spectrum: c(k) <- (c(k) + conj c(-k)) / 2 for the pairs (ky, kz) <-> (-ky, -kz).
// A real field cannot feed back into the anti-Hermitian part of these planes,
// so without the projection FFT round-off there grows like 1/(1 - dt L(k)) per
// step in the unstable band of L (the complex-field reference carries that
// part in its imaginary component, where the nonlinearity damps it).
template <typename V> __global__ void k_hermitian_planes(V *__restrict__ c, Geom g, unsigned long long *stepctr)
{
    if (stepctr && blockIdx.x == 0 && threadIdx.x == 0) *stepctr += 1; // after this step's noise draws
    const long long per = (long long)g.Y * g.Z;
    const int nplanes = (g.X & 1) ? 1 : 2; // odd X has no Nyquist plane
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < nplanes * per;
         idx += (long long)gridDim.x * blockDim.x) {
        const int plane = (int)(idx / per);
        const long long r = idx - plane * per;
        const long long z = r / g.Y, y = r - z * g.Y;
        const long long zp = (g.Z - z) % g.Z, yp = (g.Y - y) % g.Y;
        if (z * g.Y + y > zp * g.Y + yp) continue; // the partner's thread does the pair
        const long long kx = plane ? g.H : 0;
        const long long ia = z * g.S + kx * g.Y + y, ib = zp * g.S + kx * g.Y + yp;
        const V a = c[ia], b = c[ib];
        V m;
        m.x = (a.x + b.x) * 0.5f;
        m.y = (a.y - b.y) * 0.5f;
        c[ia] = m;
        m.y = -m.y;
        c[ib] = m;
    }
}

} // namespace gopf

using namespace gopf;

cudaError_t gopf_launch_hermitian_planes(gopf_ctx *ctx, void *state, cudaStream_t st)
{
    const long long n = ((ctx->g.X & 1) ? 1LL : 2LL) * ctx->g.Y * ctx->g.Z;
    const unsigned blocks = (unsigned)std::min<long long>((n + 255) / 256, 152 * 8);
    unsigned long long *ctr = (state == ctx->d_state && ctx->noise.kind) ? ctx->d_stepctr : nullptr;
    if (!st) st = ctx->stream;
    if (ctx->prec == GOPF_FP32) k_hermitian_planes<float2><<<blocks, 256, 0, st>>>((float2 *)state, ctx->g, ctr);
    else k_hermitian_planes<double2><<<blocks, 256, 0, st>>>((double2 *)state, ctx->g, ctr);
    return cudaGetLastError();
}

int gopf_elastic_table(gopf_ctx *ctx)
{
    ElasticParams p;
    memcpy(p.C, ctx->el_C, sizeof(p.C));
    memcpy(p.A, ctx->el_A, sizeof(p.A));
    p.ndim = ctx->ndim;
    const size_t eb = (ctx->prec == GOPF_FP32) ? sizeof(float) : sizeof(double);
    if (!ctx->d_bsym) {
        cudaError_t e = gopf_malloc(&ctx->d_bsym, eb * ctx->g.C);
        if (e != cudaSuccess) return gopf_fail(ctx, GOPF_ERR_OOM, "gopf_malloc(elastic symbol)");
        ctx->dev_bytes += eb * ctx->g.C;
    }
    const unsigned blocks = (unsigned)std::min<long long>((ctx->g.C + 255) / 256, 152 * 32);
    if (ctx->prec == GOPF_FP32) k_elastic_symbol<float><<<blocks, 256, 0, ctx->stream>>>(ctx->g, p, (float *)ctx->d_bsym);
    else k_elastic_symbol<double><<<blocks, 256, 0, ctx->stream>>>(ctx->g, p, (double *)ctx->d_bsym);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return gopf_fail(ctx, GOPF_ERR_CUDA, std::string("elastic symbol: ") + cudaGetErrorString(e));
    return GOPF_OK;
}

cudaError_t gopf_launch_volcons_finalize(gopf_ctx *ctx, const double *red_field, int nblocks)
{
    k_volcons_finalize<<<1, VC_THREADS, 0, ctx->stream>>>(red_field, ctx->d_red2, nblocks, ctx->vc_dt, ctx->vc_coef,
                                                        ctx->d_vc);
    return cudaGetLastError();
}
