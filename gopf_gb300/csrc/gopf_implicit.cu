// gopf_implicit.cu -- ImplicitEuler (pf/implicitEuler.go) on the device.
//
// The reference solves, once per step, the real-space system F(x) = 0 with
//   F(x) = x - IFFT(c_n e^(L dt) + I(L, N(x), N_n)) / N       (updateEquation, :68-94)
// where I integrates the explicit RHS interpolated linearly between N_n (the
// RHS at the step's start) and N(x) (nonlinearIntegral, :151-162).  It starts
// Newton-Krylov from one explicit Euler step (:182-190) and uses the
// DefaultNonLinSolver controls (:221-228): at most 50 Newton iterations, a
// finite-difference Jacobian with step 1e-3 and a 6-point stencil, tolerance
// 1e-7, GMRES for the linear systems.  The solver library is a third-party
// dependency (github.com/davidkleiven/gononlin v0.2.2 with gonum's GMRES); this
// file restates the published method:
//
//   Newton:  x <- x + d,  J(x) d = -F(x),  until max|F(x)| <= tol
//   J v    ~ sum_k w_k F(x + k h' v) / h'   (central differences, 2/4/6/8 points),
//            h' = step * sqrt(n) so that the perturbation's RMS per cell is `step`
//   GMRES  : Arnoldi with classical Gram-Schmidt applied twice, Givens rotations,
//            no restart (at most `restart` Krylov vectors), relative tolerance 1e-8
//
// F, the vector updates and the inner products run on the device; the host
// only holds the small Hessenberg matrix.  Every inner product is an FP64
// accumulation finished in a fixed order, so a solve is reproducible.  In FP32
// mode the tolerance is raised to 32 ulp of max|x| when tol is below that.
#include <cfloat>
#include <cmath>
#include <string>
#include <vector>

#include "gopf_ctx.h"

int gopf_fail(gopf_ctx *ctx, int code, const std::string &msg);
int gopf_ie_rhs(gopf_ctx *ctx, void *nprev, void *tmp0);
int gopf_ie_residual(gopf_ctx *ctx, const void *x, void *F, const void *chat0, const void *nprev, void *tmp0);
int gopf_ie_euler_guess(gopf_ctx *ctx, void *x0);
int gopf_ie_rhs_multi(gopf_ctx *ctx, void *nprev, void *const *grp);
int gopf_ie_residual_multi(gopf_ctx *ctx, const void *x, void *F, const void *chat0, const void *nprev,
                           void *const *grp);
int gopf_real_to_state(gopf_ctx *ctx, const void *src);

namespace {

constexpr int kBlocks = 304; // partial-sum blocks (2 per SM)
constexpr int kThreads = 256;

template <typename R> __global__ void k_axpby(long long n, double a, const R *__restrict__ x, double b,
                                              const R *__restrict__ y, R *__restrict__ out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (R)(a * (double)x[i] + b * (double)y[i]);
}

__device__ __forceinline__ double block_sum(double v, double *sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
    return s;
}

// part[i * gridDim.x + block] = sum over the block's share of w * V_i, i < k
template <typename R>
__global__ void k_dots(long long n, const R *__restrict__ w, R *const *__restrict__ V, int k, double *__restrict__ part)
{
    __shared__ double sh[32];
    for (int i = 0; i < k; ++i) {
        const R *__restrict__ v = V[i];
        double s = 0.0;
        for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x)
            s += (double)w[j] * (double)v[j];
        s = block_sum(s, sh);
        if (threadIdx.x == 0) part[i * gridDim.x + blockIdx.x] = s;
    }
}

// part[block] = sum of squares, part[gridDim.x + block] = max |x|
template <typename R> __global__ void k_norms(long long n, const R *__restrict__ x, double *__restrict__ part)
{
    __shared__ double sh[32];
    double s = 0.0, m = 0.0;
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
        const double v = (double)x[j];
        s += v * v;
        m = fmax(m, fabs(v));
    }
    s = block_sum(s, sh);
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ double shm[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) shm[warp] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, shm[w]);
        part[blockIdx.x] = s;
        part[gridDim.x + blockIdx.x] = fmax(m, shm[0]);
    }
}

// out[i] = sum of the nb partials of row i (rows < k), in block order; row k: max of row k's partials
// when with_max is set.  One thread per row: nb is a few hundred.
__global__ void k_finish_rows(const double *__restrict__ part, int nb, int k, int with_max, double *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < k) {
        double s = 0.0;
        for (int b = 0; b < nb; ++b) s += part[(long long)i * nb + b];
        out[i] = s;
    } else if (with_max && i == k) {
        double m = 0.0;
        for (int b = 0; b < nb; ++b) m = fmax(m, part[(long long)k * nb + b]);
        out[k] = m;
    }
}

// w -= sum_i h[i] V_i
template <typename R>
__global__ void k_sub_combo(long long n, R *__restrict__ w, R *const *__restrict__ V, const double *__restrict__ h, int k)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
        double s = (double)w[j];
        for (int i = 0; i < k; ++i) s -= h[i] * (double)V[i][j];
        w[j] = (R)s;
    }
}

// x += sum_i y[i] V_i
template <typename R>
__global__ void k_add_combo(long long n, R *__restrict__ x, R *const *__restrict__ V, const double *__restrict__ y, int k)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
        double s = (double)x[j];
        for (int i = 0; i < k; ++i) s += y[i] * (double)V[i][j];
        x[j] = (R)s;
    }
}

} // namespace

struct gopf_ie_work {
    int prec = 0;
    long long n = 0;
    int restart = 0;
    size_t rb = 0; // bytes of one real vector
    void *x = nullptr, *F = nullptr, *xp = nullptr, *Fp = nullptr, *w = nullptr;
    std::vector<void *> V;
    void **d_V = nullptr;
    void *chat0 = nullptr, *nprev = nullptr, *tmp0 = nullptr; // chat0, nprev: one spectrum per field
    int nfields = 1;
    std::vector<void *> grp; // several fields: spectral scratch of the x-pass outputs
    double *d_part = nullptr, *d_out = nullptr, *d_coef = nullptr;
    double *h_out = nullptr; // pinned
};

void gopf_ie_free(gopf_ctx *ctx)
{
    gopf_ie_work *ws = ctx->ie;
    if (!ws) return;
    void *ptrs[] = {ws->x, ws->F, ws->xp, ws->Fp, ws->w, ws->d_V, ws->chat0, ws->nprev, ws->tmp0, ws->d_part,
                    ws->d_out, ws->d_coef};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (void *p : ws->V)
        if (p) cudaFree(p);
    for (void *p : ws->grp)
        if (p) cudaFree(p);
    if (ws->h_out) cudaFreeHost(ws->h_out);
    delete ws;
    ctx->ie = nullptr;
}

namespace {

#define IE_CK(call)                                                                                                    \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess)                                                                                         \
            return gopf_fail(ctx, GOPF_ERR_CUDA, std::string("implicit Euler: ") + cudaGetErrorString(e_));          \
    } while (0)

int ie_alloc(gopf_ctx *ctx)
{
    const int restart = ctx->nk_restart;
    const int nf = ctx->multi ? ctx->nfields : 1;
    const int ngrp = ctx->multi ? ctx->mono_rk.ngrp + nf + 1 : 0;
    if (ctx->ie && ctx->ie->restart == restart && ctx->ie->nfields == nf && (int)ctx->ie->grp.size() == ngrp)
        return GOPF_OK;
    gopf_ie_free(ctx);
    gopf_ie_work *ws = new gopf_ie_work();
    ctx->ie = ws;
    ws->prec = ctx->prec;
    ws->nfields = nf;
    ws->n = ctx->g.N * nf; // [field 0 | field 1 | ...] (fields2vec, pf/implicitEuler.go:44-66)
    ws->restart = restart;
    ws->rb = (size_t)ws->n * (ctx->prec == GOPF_FP32 ? sizeof(float) : sizeof(double));
    const size_t cb = (size_t)ctx->g.C * (ctx->prec == GOPF_FP32 ? sizeof(float2) : sizeof(double2));
    void **vecs[] = {&ws->x, &ws->F, &ws->xp, &ws->Fp, &ws->w};
    for (void **p : vecs) IE_CK(gopf_malloc(p, ws->rb));
    ws->V.assign(restart + 1, nullptr);
    for (auto &p : ws->V) IE_CK(gopf_malloc(&p, ws->rb));
    IE_CK(gopf_malloc(&ws->d_V, sizeof(void *) * (restart + 1)));
    IE_CK(cudaMemcpy(ws->d_V, ws->V.data(), sizeof(void *) * (restart + 1), cudaMemcpyHostToDevice));
    IE_CK(gopf_malloc(&ws->chat0, cb * nf));
    IE_CK(gopf_malloc(&ws->nprev, cb * nf));
    IE_CK(gopf_malloc(&ws->tmp0, cb));
    ws->grp.assign(ngrp, nullptr);
    for (auto &p : ws->grp) IE_CK(gopf_malloc(&p, cb));
    ctx->dev_bytes += cb * (2 * (nf - 1) + ngrp);
    IE_CK(gopf_malloc(&ws->d_part, sizeof(double) * kBlocks * (restart + 2)));
    IE_CK(gopf_malloc(&ws->d_out, sizeof(double) * (restart + 2)));
    IE_CK(gopf_malloc(&ws->d_coef, sizeof(double) * (restart + 2)));
    IE_CK(cudaMallocHost(&ws->h_out, sizeof(double) * (restart + 2)));
    ctx->dev_bytes += ws->rb * (5 + restart + 1) + 3 * cb;
    return GOPF_OK;
}

// The solver's vector kernels, typed by the context's precision.
struct Vec {
    gopf_ctx *ctx;
    gopf_ie_work *ws;
    cudaStream_t st;

    int axpby(double a, const void *x, double b, const void *y, void *out)
    {
        if (ws->prec == GOPF_FP32)
            k_axpby<float><<<kBlocks * 2, kThreads, 0, st>>>(ws->n, a, (const float *)x, b, (const float *)y, (float *)out);
        else
            k_axpby<double><<<kBlocks * 2, kThreads, 0, st>>>(ws->n, a, (const double *)x, b, (const double *)y,
                                                              (double *)out);
        IE_CK(cudaGetLastError());
        return GOPF_OK;
    }
    // h_out[i] = <w, V_i>, i < k (synchronising)
    int dots(const void *w, int k)
    {
        if (ws->prec == GOPF_FP32)
            k_dots<float><<<kBlocks, kThreads, 0, st>>>(ws->n, (const float *)w, (float *const *)ws->d_V, k, ws->d_part);
        else
            k_dots<double><<<kBlocks, kThreads, 0, st>>>(ws->n, (const double *)w, (double *const *)ws->d_V, k,
                                                         ws->d_part);
        IE_CK(cudaGetLastError());
        k_finish_rows<<<(k + 64) / 64, 64, 0, st>>>(ws->d_part, kBlocks, k, 0, ws->d_out);
        IE_CK(cudaGetLastError());
        IE_CK(cudaMemcpyAsync(ws->h_out, ws->d_out, sizeof(double) * k, cudaMemcpyDeviceToHost, st));
        IE_CK(cudaStreamSynchronize(st));
        return GOPF_OK;
    }
    // (||x||_2, max|x|) (synchronising)
    int norms(const void *x, double *l2, double *linf)
    {
        if (ws->prec == GOPF_FP32) k_norms<float><<<kBlocks, kThreads, 0, st>>>(ws->n, (const float *)x, ws->d_part);
        else k_norms<double><<<kBlocks, kThreads, 0, st>>>(ws->n, (const double *)x, ws->d_part);
        IE_CK(cudaGetLastError());
        k_finish_rows<<<1, 64, 0, st>>>(ws->d_part, kBlocks, 1, 1, ws->d_out);
        IE_CK(cudaGetLastError());
        IE_CK(cudaMemcpyAsync(ws->h_out, ws->d_out, sizeof(double) * 2, cudaMemcpyDeviceToHost, st));
        IE_CK(cudaStreamSynchronize(st));
        *l2 = std::sqrt(ws->h_out[0]);
        *linf = ws->h_out[1];
        return GOPF_OK;
    }
    int sub_combo(void *w, const double *h, int k)
    {
        IE_CK(cudaMemcpyAsync(ws->d_coef, h, sizeof(double) * k, cudaMemcpyHostToDevice, st));
        if (ws->prec == GOPF_FP32)
            k_sub_combo<float><<<kBlocks * 2, kThreads, 0, st>>>(ws->n, (float *)w, (float *const *)ws->d_V, ws->d_coef, k);
        else
            k_sub_combo<double><<<kBlocks * 2, kThreads, 0, st>>>(ws->n, (double *)w, (double *const *)ws->d_V,
                                                                  ws->d_coef, k);
        IE_CK(cudaGetLastError());
        return GOPF_OK;
    }
    int add_combo(void *x, const double *y, int k)
    {
        IE_CK(cudaMemcpyAsync(ws->d_coef, y, sizeof(double) * k, cudaMemcpyHostToDevice, st));
        if (ws->prec == GOPF_FP32)
            k_add_combo<float><<<kBlocks * 2, kThreads, 0, st>>>(ws->n, (float *)x, (float *const *)ws->d_V, ws->d_coef, k);
        else
            k_add_combo<double><<<kBlocks * 2, kThreads, 0, st>>>(ws->n, (double *)x, (double *const *)ws->d_V,
                                                                  ws->d_coef, k);
        IE_CK(cudaGetLastError());
        // the host coefficients must outlive the asynchronous copy
        IE_CK(cudaStreamSynchronize(st));
        return GOPF_OK;
    }
};

// central-difference weights for f'(0) with 2, 4, 6 or 8 points: d ~ sum_k w_k (f(k h) - f(-k h)) / h
int stencil_weights(int pts, double *w)
{
    switch (pts) {
    case 2: w[0] = 1.0 / 2.0; return 1;
    case 4: w[0] = 8.0 / 12.0; w[1] = -1.0 / 12.0; return 2;
    case 6: w[0] = 45.0 / 60.0; w[1] = -9.0 / 60.0; w[2] = 1.0 / 60.0; return 3;
    case 8: w[0] = 672.0 / 840.0; w[1] = -168.0 / 840.0; w[2] = 32.0 / 840.0; w[3] = -3.0 / 840.0; return 4;
    default: return 0;
    }
}

} // namespace

// One ImplicitEuler step of the context's fields (one Newton-Krylov solve over all of them).
int gopf_ie_step(gopf_ctx *ctx)
{
    gopf_nvtx_scope trace("implicit_euler_step");
    int rc;
    if ((rc = ie_alloc(ctx))) return rc;
    gopf_ie_work *ws = ctx->ie;
    Vec vo{ctx, ws, ctx->stream};
    cudaStream_t st = ctx->stream;
    const long long n = ws->n;
    double wst[4];
    const int nw = stencil_weights(ctx->nk_stencil, wst);
    if (nw == 0) return gopf_fail(ctx, GOPF_ERR_ARG, "finite-difference stencil must have 2, 4, 6 or 8 points");

    // N_n, c_n, and the explicit Euler start
    const bool multi = ctx->multi;
    if ((rc = multi ? gopf_ie_rhs_multi(ctx, ws->nprev, ws->grp.data()) : gopf_ie_rhs(ctx, ws->nprev, ws->tmp0)))
        return rc;
    const size_t cb = (size_t)ctx->g.C * (ctx->prec == GOPF_FP32 ? sizeof(float2) : sizeof(double2));
    for (int f = 0; f < ws->nfields; ++f)
        IE_CK(cudaMemcpyAsync((char *)ws->chat0 + f * cb, field_state(ctx, f), cb, cudaMemcpyDeviceToDevice, st));
    if ((rc = gopf_ie_euler_guess(ctx, ws->x))) return rc;

    auto Feval = [&](const void *x, void *F) {
        return multi ? gopf_ie_residual_multi(ctx, x, F, ws->chat0, ws->nprev, ws->grp.data())
                     : gopf_ie_residual(ctx, x, F, ws->chat0, ws->nprev, ws->tmp0);
    };

    double fl2 = 0.0, finf = 0.0, xl2 = 0.0, xinf = 0.0;
    if ((rc = Feval(ws->x, ws->F))) return rc;
    if ((rc = vo.norms(ws->F, &fl2, &finf))) return rc;
    double tol = ctx->nk_tol;
    if (ctx->prec == GOPF_FP32) {
        if ((rc = vo.norms(ws->x, &xl2, &xinf))) return rc;
        tol = std::max(tol, 32.0 * FLT_EPSILON * std::max(1.0, xinf));
    }
    const int m = ws->restart;
    const double hstep = ctx->nk_step * std::sqrt((double)n);
    std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1), hcol(m + 1), y(m);
    int newton = 0, krylov_total = 0;
    bool converged = finf <= tol;
    while (!converged && newton < ctx->nk_maxiter) {
        // GMRES for J d = -F, d = sum y_i V_i
        const double beta = fl2;
        if (!(beta > 0.0) || !std::isfinite(beta)) break;
        if ((rc = vo.axpby(-1.0 / beta, ws->F, 0.0, ws->F, ws->V[0]))) return rc;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int k = 0;
        for (int j = 0; j < m; ++j) {
            // w = J V_j by central differences
            IE_CK(cudaMemsetAsync(ws->w, 0, ws->rb, st));
            for (int q = 0; q < nw; ++q) {
                const double kh = (double)(q + 1) * hstep;
                for (int sgn = 1; sgn >= -1; sgn -= 2) {
                    if ((rc = vo.axpby(1.0, ws->x, sgn * kh, ws->V[j], ws->xp))) return rc;
                    if ((rc = Feval(ws->xp, ws->Fp))) return rc;
                    if ((rc = vo.axpby(1.0, ws->w, sgn * wst[q] / hstep, ws->Fp, ws->w))) return rc;
                }
            }
            // classical Gram-Schmidt, twice
            std::fill(hcol.begin(), hcol.end(), 0.0);
            for (int pass = 0; pass < 2; ++pass) {
                if ((rc = vo.dots(ws->w, j + 1))) return rc;
                std::vector<double> hh(ws->h_out, ws->h_out + j + 1);
                for (int i = 0; i <= j; ++i) hcol[i] += hh[i];
                if ((rc = vo.sub_combo(ws->w, hh.data(), j + 1))) return rc;
                IE_CK(cudaStreamSynchronize(st)); // hh is a host temporary
            }
            double wl2, winf;
            if ((rc = vo.norms(ws->w, &wl2, &winf))) return rc;
            hcol[j + 1] = wl2;
            // Givens rotations
            for (int i = 0; i < j; ++i) {
                const double a = hcol[i], b = hcol[i + 1];
                hcol[i] = cs[i] * a + sn[i] * b;
                hcol[i + 1] = -sn[i] * a + cs[i] * b;
            }
            const double a = hcol[j], b = hcol[j + 1];
            const double r = std::hypot(a, b);
            cs[j] = (r > 0.0) ? a / r : 1.0;
            sn[j] = (r > 0.0) ? b / r : 0.0;
            hcol[j] = r;
            hcol[j + 1] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = hcol[i];
            k = j + 1;
            ++krylov_total;
            const bool done = std::fabs(g[j + 1]) <= ctx->nk_krylov_rtol * beta || !(wl2 > 1e-300);
            if (done) break;
            if ((rc = vo.axpby(1.0 / wl2, ws->w, 0.0, ws->w, ws->V[j + 1]))) return rc;
        }
        // back substitution
        for (int i = k - 1; i >= 0; --i) {
            double s = g[i];
            for (int c = i + 1; c < k; ++c) s -= H[(size_t)i * m + c] * y[c];
            y[i] = s / H[(size_t)i * m + i];
        }
        if ((rc = vo.add_combo(ws->x, y.data(), k))) return rc;
        ++newton;
        if ((rc = Feval(ws->x, ws->F))) return rc;
        if ((rc = vo.norms(ws->F, &fl2, &finf))) return rc;
        converged = finf <= tol;
    }
    ctx->nk_last_newton = newton;
    ctx->nk_last_krylov = krylov_total;
    ctx->nk_last_residual = finf;
    ctx->nk_last_converged = converged ? 1 : 0;
    // the solution becomes the state (res.X -> vec2fields, :201-205)
    if ((rc = gopf_real_to_state(ctx, ws->x))) return rc;
    return GOPF_OK;
}
