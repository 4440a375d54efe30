// gopf_adjoint.cu -- hand-written adjoint of the semi-implicit Cahn-Hilliard step.
//
// Forward (the reference's Euler step, pf/euler.go:16-47, for the string
// "dconc/dt = M*LAP MU - M*gamma*LAP^2 conc" with MU = conc^3 - conc):
//     c_{n+1} = D (c_n - dt M K f(c_n)),   K = -lap <-> k^2,  D = (1 + dt M gamma K^2)^-1,
//     f(c) = c^3 - c.
// K and D are real, symmetric Fourier multipliers, so the transposed step is
//     lambda_n = (1 - dt M diag f'(c_n) K) D lambda_{n+1},   f'(c) = 3 c^2 - 1,
// and with L = loss(c_T), lambda_T = dL/dc_T:
//     dL/dgamma = -dt M   sum_n <lambda_{n+1}, K^2 D c_{n+1}>
//     dL/dM     = -sum_n [ dt gamma <lambda_{n+1}, K^2 D c_{n+1}> + dt <lambda_{n+1}, D K f(c_n)> ]
//     dL/dc_0   = lambda_0.
// Inner products are taken in k space (Parseval, half spectrum weighted 2
// off the self-conjugate planes).  The forward run keeps the field every
// `every` steps; the backward run recomputes each segment from its
// checkpoint and walks it backwards.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gopf_ctx.h"
#include "gopf_kernels.cuh"

namespace gopf {

template <typename R> __global__ void k_fpoly(const R *__restrict__ c, R *__restrict__ f, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const R x = c[i];
        f[i] = x * x * x - x;
    }
}

// lambda <- mu - dt M (3 c^2 - 1) nu
template <typename R>
__global__ void k_adj_real(const R *__restrict__ mu, const R *__restrict__ nu, const R *__restrict__ c, R *__restrict__ lam,
                           R dtM, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const R x = c[i];
        lam[i] = mu[i] - dtM * ((R)3 * x * x - (R)1) * nu[i];
    }
}

// k space: mu = D lam / N, nu = k^2 D lam / N (in place of lam-hat and f-hat),
// plus the two gradient sums (FP64, atomically accumulated per block).
template <typename R>
__global__ void k_adj_kspace(Geom g, typename VecOf<R>::type *__restrict__ lamh, typename VecOf<R>::type *__restrict__ fh,
                             const typename VecOf<R>::type *__restrict__ ch, double dtMg, double invN, double *__restrict__ sums)
{
    typedef typename VecOf<R>::type V;
    double s1 = 0.0, s2 = 0.0;
    const double fourpi2 = 39.478417604357434475337963999504;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < g.C;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long z = idx / g.S;
        const long long rem = idx - z * g.S;
        const long long kx = rem / g.Y;
        const long long y = rem - kx * g.Y;
        const long long jy = (2 * y > g.Y) ? g.Y - y : y;
        const long long jz = (2 * z > g.Z) ? g.Z - z : z;
        const double fx = (double)kx / g.X, fy = (double)jy / g.Y, fz = (double)jz / g.Z;
        const double k2 = fourpi2 * (fx * fx + fy * fy + fz * fz);
        const double D = 1.0 / (1.0 + dtMg * k2 * k2);
        const double w = (kx == 0 || 2 * kx == g.X) ? 1.0 : 2.0;
        const V l = lamh[idx], c = ch[idx], f = fh[idx];
        // Re(conj(l) * c) and Re(conj(l) * f)
        s1 += w * k2 * k2 * D * ((double)l.x * (double)c.x + (double)l.y * (double)c.y);
        s2 += w * k2 * D * ((double)l.x * (double)f.x + (double)l.y * (double)f.y);
        const R a = (R)(D * invN), b = (R)(D * k2 * invN);
        V mu, nu;
        mu.x = l.x * a;
        mu.y = l.y * a;
        nu.x = l.x * b;
        nu.y = l.y * b;
        lamh[idx] = mu;
        fh[idx] = nu;
    }
    // block reduction
    __shared__ double sh1[32], sh2[32];
    for (int o = 16; o > 0; o >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        sh1[warp] = s1;
        sh2[warp] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) {
            a += sh1[w];
            b += sh2[w];
        }
        atomicAdd(&sums[0], a);
        atomicAdd(&sums[1], b);
    }
}

} // namespace gopf

using namespace gopf;

struct gopf_adjoint_state {
    int nsteps = 0, every = 0;
    double gamma = 0.0, M = 0.0, dt = 0.0;
    void *d_ckpt = nullptr;  // (nsteps/every + 1) real fields
    void *d_seg = nullptr;   // every + 1 real fields
    void *d_r[4] = {nullptr, nullptr, nullptr, nullptr}; // real work: lambda, f, mu, nu
    void *d_s[3] = {nullptr, nullptr, nullptr};           // spectral work
    double *d_sums = nullptr;
    int nckpt = 0;
};

static int afail(gopf_ctx *ctx, cudaError_t e, const char *w)
{
    return gopf_fail(ctx, e == cudaErrorMemoryAllocation ? GOPF_ERR_OOM : GOPF_ERR_CUDA,
                     std::string(w) + ": " + cudaGetErrorString(e));
}

#define ACK(call)                                                                                                      \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess) return afail(ctx, e_, #call);                                                           \
    } while (0)

static unsigned ew(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 152 * 16); }

// real device array -> spectrum (unnormalised forward transform)
template <typename R> static cudaError_t r2c(gopf_ctx *ctx, const R *real, typename VecOf<R>::type *spec)
{
    typedef typename VecOf<R>::type V;
    XPassArgs<R> xa;
    memset(&xa, 0, sizeof(xa));
    xa.g = ctx->g;
    xa.planH = ctx->planH;
    xa.twX = (const V *)ctx->d_twX;
    xa.in_mode = XIN_REAL;
    xa.rin = real;
    xa.out[0] = spec;
    xa.ngrp_out = 1;
    xa.identity = 1;
    xa.allow_fast = ctx->use_fast;
    cudaError_t e = launch_xpass<R>(xa, ctx->LBx, ctx->stream);
    if (e != cudaSuccess) return e;
    PassArgs<R> pa;
    memset(&pa, 0, sizeof(pa));
    pa.g = ctx->g;
    pa.plan = ctx->planY;
    pa.tw = (const V *)ctx->d_twY;
    pa.mode = PM_FWD;
    pa.buf[0] = spec;
    pa.nbuf = 1;
    pa.allow_fast = ctx->use_fast;
    if ((e = launch_cpass<R>(pa, ctx->LBy, ctx->stream)) != cudaSuccess) return e;
    if (ctx->g.Z > 1) {
        pa.plan = ctx->planZ;
        pa.tw = (const V *)ctx->d_twZ;
        if ((e = launch_spass<R>(pa, ctx->LBz, ctx->stream)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// spectrum -> real device array (unnormalised inverse transform; spec is overwritten)
template <typename R> static cudaError_t c2r(gopf_ctx *ctx, typename VecOf<R>::type *spec, R *real)
{
    typedef typename VecOf<R>::type V;
    cudaError_t e;
    PassArgs<R> pa;
    memset(&pa, 0, sizeof(pa));
    pa.g = ctx->g;
    pa.mode = PM_INV;
    pa.buf[0] = spec;
    pa.nbuf = 1;
    pa.allow_fast = ctx->use_fast;
    if (ctx->g.Z > 1) {
        pa.plan = ctx->planZ;
        pa.tw = (const V *)ctx->d_twZ;
        if ((e = launch_spass<R>(pa, ctx->LBz, ctx->stream)) != cudaSuccess) return e;
    }
    pa.plan = ctx->planY;
    pa.tw = (const V *)ctx->d_twY;
    if ((e = launch_cpass<R>(pa, ctx->LBy, ctx->stream)) != cudaSuccess) return e;
    XPassArgs<R> xa;
    memset(&xa, 0, sizeof(xa));
    xa.g = ctx->g;
    xa.planH = ctx->planH;
    xa.twX = (const V *)ctx->d_twX;
    xa.in_mode = XIN_SPECTRAL;
    xa.in = spec;
    xa.rout = real;
    xa.allow_fast = ctx->use_fast;
    return launch_xpass<R>(xa, ctx->LBx, ctx->stream);
}

// real field of the current state (c = c2r of T) into dst
int gopf_state_to_real(gopf_ctx *ctx, void *dst);
int gopf_real_to_state(gopf_ctx *ctx, const void *src);
int gopf_step_device(gopf_ctx *ctx, long long n);

template <typename R> static int adj_backward(gopf_ctx *ctx, gopf_adjoint_state *st, const double *lamT_host,
                                              double *dgamma, double *dM, double *dc0_host)
{
    typedef typename VecOf<R>::type V;
    const long long N = ctx->g.N;
    const size_t rb = sizeof(R) * N;
    R *lam = (R *)st->d_r[0], *f = (R *)st->d_r[1], *mu = (R *)st->d_r[2], *nu = (R *)st->d_r[3];
    V *Sl = (V *)st->d_s[0], *Sf = (V *)st->d_s[1], *Sc = (V *)st->d_s[2];
    // lambda_T (host FP64) -> device R
    std::vector<R> h(N);
    for (long long i = 0; i < N; ++i) h[i] = (R)lamT_host[i];
    ACK(cudaMemcpyAsync(lam, h.data(), rb, cudaMemcpyHostToDevice, ctx->stream));
    ACK(cudaMemsetAsync(st->d_sums, 0, 2 * sizeof(double), ctx->stream));
    const double dtM = st->dt * st->M, dtMg = st->dt * st->M * st->gamma, invN = 1.0 / (double)N;
    const int nseg = (st->nsteps + st->every - 1) / st->every;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int s0 = seg * st->every;
        const int s1 = std::min(st->nsteps, s0 + st->every);
        // recompute c_{s0} .. c_{s1}
        int rc;
        if ((rc = gopf_real_to_state(ctx, (char *)st->d_ckpt + (size_t)seg * rb))) return rc;
        ACK(cudaMemcpyAsync(st->d_seg, (char *)st->d_ckpt + (size_t)seg * rb, rb, cudaMemcpyDeviceToDevice, ctx->stream));
        for (int n = s0; n < s1; ++n) {
            if ((rc = gopf_step_device(ctx, 1))) return rc;
            if ((rc = gopf_state_to_real(ctx, (char *)st->d_seg + (size_t)(n + 1 - s0) * rb))) return rc;
        }
        for (int n = s1 - 1; n >= s0; --n) {
            const R *cn = (const R *)((char *)st->d_seg + (size_t)(n - s0) * rb);
            const R *cn1 = (const R *)((char *)st->d_seg + (size_t)(n + 1 - s0) * rb);
            k_fpoly<R><<<ew(N), 256, 0, ctx->stream>>>(cn, f, N);
            ACK(cudaGetLastError());
            ACK(r2c<R>(ctx, f, Sf));
            ACK(r2c<R>(ctx, cn1, Sc));
            ACK(r2c<R>(ctx, lam, Sl));
            k_adj_kspace<R><<<ew(ctx->g.C), 256, 0, ctx->stream>>>(ctx->g, Sl, Sf, Sc, dtMg, invN, st->d_sums);
            ACK(cudaGetLastError());
            ACK(c2r<R>(ctx, Sl, mu));
            ACK(c2r<R>(ctx, Sf, nu));
            k_adj_real<R><<<ew(N), 256, 0, ctx->stream>>>(mu, nu, cn, lam, (R)dtM, N);
            ACK(cudaGetLastError());
        }
    }
    double sums[2];
    ACK(cudaMemcpyAsync(sums, st->d_sums, sizeof(sums), cudaMemcpyDeviceToHost, ctx->stream));
    ACK(cudaMemcpyAsync(h.data(), lam, rb, cudaMemcpyDeviceToHost, ctx->stream));
    ACK(cudaStreamSynchronize(ctx->stream));
    const double S1 = sums[0] * invN, S2 = sums[1] * invN;
    if (dgamma) *dgamma = -st->dt * st->M * S1;
    if (dM) *dM = -st->dt * st->gamma * S1 - st->dt * S2;
    if (dc0_host)
        for (long long i = 0; i < N; ++i) dc0_host[i] = (double)h[i];
    return GOPF_OK;
}

static gopf_adjoint_state *adj_state(gopf_ctx *ctx);

extern "C" int gopf_adjoint_forward(gopf_ctx *ctx, double gamma, double M, double dt, int nsteps, int every,
                                    const double *c0, double *cT)
{
    if (!ctx || !c0 || nsteps < 1 || every < 1 || !(dt > 0.0)) return gopf_fail(ctx, GOPF_ERR_ARG, "bad argument");
    if (ctx->device < 0) return gopf_fail(ctx, GOPF_ERR_STATE, "host-only context");
    ACK(cudaSetDevice(ctx->device));
    // the model: dconc/dt = M*LAP MU - M*gamma*LAP^2 conc, MU = conc^3 - conc
    gopf_derived mu;
    memset(&mu, 0, sizeof(mu));
    mu.kind = GOPF_DER_POLY;
    mu.nfac = 2;
    mu.field[0] = mu.field[1] = 0;
    mu.power[0] = 3;
    mu.power[1] = 1;
    mu.coef[0] = 1.0;
    mu.coef[1] = -1.0;
    gopf_term t[2];
    memset(t, 0, sizeof(t));
    t[0].coef = M;
    t[0].lap = 1;
    t[0].source = GOPF_SRC_DERIVED;
    t[1].implicit = 1;
    t[1].coef = -M * gamma;
    t[1].lap = 2;
    int rc = gopf_set_terms(ctx, 1, &mu, 1, t, 2);
    if (rc) return rc;
    if ((rc = gopf_set_stepper(ctx, GOPF_STEPPER_EULER, dt))) return rc;
    gopf_adjoint_state *st = adj_state(ctx);
    const long long N = ctx->g.N;
    const size_t rb = (ctx->prec == GOPF_FP32 ? sizeof(float) : sizeof(double)) * N;
    const size_t sb = (ctx->prec == GOPF_FP32 ? sizeof(float2) : sizeof(double2)) * ctx->g.C;
    const int nck = (nsteps + every - 1) / every + 1;
    if (st->nckpt < nck || st->every != every) {
        if (st->d_ckpt) cudaFree(st->d_ckpt);
        if (st->d_seg) cudaFree(st->d_seg);
        ACK(gopf_malloc(&st->d_ckpt, rb * nck));
        ACK(gopf_malloc(&st->d_seg, rb * (every + 1)));
        st->nckpt = nck;
    }
    for (int i = 0; i < 4; ++i)
        if (!st->d_r[i]) ACK(gopf_malloc(&st->d_r[i], rb));
    for (int i = 0; i < 3; ++i)
        if (!st->d_s[i]) ACK(gopf_malloc(&st->d_s[i], sb));
    if (!st->d_sums) ACK(gopf_malloc(&st->d_sums, 2 * sizeof(double)));
    st->nsteps = nsteps;
    st->every = every;
    st->gamma = gamma;
    st->M = M;
    st->dt = dt;
    if ((rc = gopf_field_upload_real(ctx, 0, c0, (size_t)N))) return rc;
    for (int n = 0; n < nsteps; ++n) {
        if (n % every == 0 && (rc = gopf_state_to_real(ctx, (char *)st->d_ckpt + (size_t)(n / every) * rb))) return rc;
        if ((rc = gopf_step_device(ctx, 1))) return rc;
    }
    if (cT) return gopf_field_download_real(ctx, 0, cT, (size_t)N);
    ACK(cudaStreamSynchronize(ctx->stream));
    return GOPF_OK;
}

extern "C" int gopf_adjoint_backward(gopf_ctx *ctx, const double *lamT, double *dgamma, double *dM, double *dc0)
{
    if (!ctx || !lamT) return gopf_fail(ctx, GOPF_ERR_ARG, "bad argument");
    gopf_adjoint_state *st = adj_state(ctx);
    if (st->nsteps < 1) return gopf_fail(ctx, GOPF_ERR_STATE, "run gopf_adjoint_forward first");
    ACK(cudaSetDevice(ctx->device));
    return (ctx->prec == GOPF_FP32) ? adj_backward<float>(ctx, st, lamT, dgamma, dM, dc0)
                                    : adj_backward<double>(ctx, st, lamT, dgamma, dM, dc0);
}

// one adjoint workspace per context, released with gopf_adjoint_release (or at exit)
#include <map>
#include <mutex>
static std::map<gopf_ctx *, gopf_adjoint_state *> g_adj;
static std::mutex g_adj_mu;

static gopf_adjoint_state *adj_state(gopf_ctx *ctx)
{
    std::lock_guard<std::mutex> lk(g_adj_mu);
    auto it = g_adj.find(ctx);
    if (it != g_adj.end()) return it->second;
    gopf_adjoint_state *s = new gopf_adjoint_state();
    g_adj[ctx] = s;
    return s;
}

extern "C" int gopf_adjoint_release(gopf_ctx *ctx)
{
    std::lock_guard<std::mutex> lk(g_adj_mu);
    auto it = g_adj.find(ctx);
    if (it == g_adj.end()) return GOPF_OK;
    gopf_adjoint_state *s = it->second;
    cudaSetDevice(ctx->device);
    void *ptrs[] = {s->d_ckpt, s->d_seg, s->d_r[0], s->d_r[1], s->d_r[2], s->d_r[3], s->d_s[0], s->d_s[1], s->d_s[2],
                    s->d_sums};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete s;
    g_adj.erase(it);
    return GOPF_OK;
}
