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
// checkpoint and walks it backwards.  A segment's recompute and backward
// walk are one captured CUDA graph (replayed for every segment of that
// length); a backward step is five launches in 2D: the x pass forming
// r2c_x(c^3 - c) from the step's x-spectral field, one y pass forward-transforming that and lambda, the k-space
// product and gradient sums, one inverse y pass, and an x pass that forms
// lambda_n = mu - dt M (3c^2 - 1) nu and its r2c_x for the next step (the register line engine's
// passes where they serve the length).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gopf_ctx.h"
#include "gopf_kernels.cuh"

namespace gopf {

// k space: mu = D lam / N, nu = k^2 D lam / N (in place of lam-hat and f-hat),
// plus the two gradient sums (FP64, atomically accumulated per block).  The per-mode
// arithmetic runs in the state's precision (FP64 is a small fraction of the FP32 rate on this
// GPU); only the accumulation is FP64.  Indices are 32-bit (C < 2^31).
template <typename R>
__global__ void k_adj_kspace(Geom g, typename VecOf<R>::type *__restrict__ lamh, typename VecOf<R>::type *__restrict__ fh,
                             const typename VecOf<R>::type *__restrict__ ch, double dtMg, double invN, double *__restrict__ sums)
{
    typedef typename VecOf<R>::type V;
    double s1 = 0.0, s2 = 0.0;
    const R fourpi2 = (R)39.478417604357434475337963999504;
    const R a_dt = (R)dtMg, a_inv = (R)invN;
    const unsigned C = (unsigned)g.C, S = (unsigned)g.S, Y = (unsigned)g.Y;
    const R rX = (R)1 / (R)g.X, rY = (R)1 / (R)g.Y, rZ = (R)1 / (R)g.Z;
    for (unsigned idx = blockIdx.x * blockDim.x + threadIdx.x; idx < C; idx += gridDim.x * blockDim.x) {
        const unsigned z = idx / S;
        const unsigned rem = idx - z * S;
        const unsigned kx = rem / Y;
        const unsigned y = rem - kx * Y;
        const unsigned jy = (2 * y > Y) ? Y - y : y;
        const unsigned jz = (2 * z > (unsigned)g.Z) ? (unsigned)g.Z - z : z;
        const R fx = (R)kx * rX, fy = (R)jy * rY, fz = (R)jz * rZ;
        const R k2 = fourpi2 * (fx * fx + fy * fy + fz * fz);
        const R D = (R)1 / ((R)1 + a_dt * k2 * k2);
        const R w = (kx == 0 || 2 * kx == (unsigned)g.X) ? (R)1 : (R)2;
        const V l = lamh[idx], c = ch[idx], f = fh[idx];
        // Re(conj(l) * c) and Re(conj(l) * f)
        s1 += (double)(w * k2 * k2 * D * (l.x * c.x + l.y * c.y));
        s2 += (double)(w * k2 * D * (l.x * f.x + l.y * f.y));
        const R a = D * a_inv, b = D * k2 * a_inv;
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
    void *d_segs = nullptr;  // every + 1 spectra (c-hat of the recomputed steps)
    void *d_segT = nullptr;  // every + 1 x-spectral fields (T of the recomputed steps)
    void *d_stage = nullptr; // the checkpoint a segment graph starts from
    void *d_r[4] = {nullptr, nullptr, nullptr, nullptr}; // real work: lambda (the others unused)
    void *d_s[3] = {nullptr, nullptr, nullptr};           // spectral work
    double *d_sums = nullptr;
    int nckpt = 0;
    // captured segment sweeps (recompute + backward), full length and the shorter last one
    cudaGraphExec_t g_full = nullptr, g_tail = nullptr;
    int g_full_len = 0, g_tail_len = 0;
    double g_key[3] = {0.0, 0.0, 0.0}; // gamma, M, dt the graphs were captured with
    double model_key[3] = {0.0, 0.0, 0.0}; // gamma, M, dt of the model installed on the context
    bool model_set = false;
};

static void adj_drop_graphs(gopf_adjoint_state *st)
{
    if (st->g_full) cudaGraphExecDestroy(st->g_full);
    if (st->g_tail) cudaGraphExecDestroy(st->g_tail);
    st->g_full = st->g_tail = nullptr;
    st->g_full_len = st->g_tail_len = 0;
}

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

// real field of the current state (c = c2r of T) into dst
int gopf_state_to_real(gopf_ctx *ctx, void *dst);
int gopf_real_to_state(gopf_ctx *ctx, const void *src);
int gopf_step_device(gopf_ctx *ctx, long long n);

// One segment's sweep, stream-ordered (captured into a graph by the caller): recompute c_{s0+1} ..
// c_{s0+len} from the checkpoint in d_stage, keeping each step's real field and c-hat, then walk
// the steps backwards.  Per backward step n, with Lx = the x-transformed lambda_{n+1} in S[0]:
//   x pass   : f(c_n) = c_n^3 - c_n from T_n (c2r, polynomial, r2c along x)  -> S[1]
//   y (z)    : forward of S[1] and S[0] in one launch                        -> F, Lambda
//   k space  : the two gradient sums; mu-hat = D Lambda / N -> S[0], nu-hat = k^2 D Lambda / N -> S[1]
//   (z) y    : inverse of S[0] and S[1] in one launch
//   x pass   : lambda_n = mu - dt M (3 c_n^2 - 1) nu (into the real lambda) and r2c along x -> S[0]
template <typename R> static int adj_segment(gopf_ctx *ctx, gopf_adjoint_state *st, int len)
{
    typedef typename VecOf<R>::type V;
    const Geom &g = ctx->g;
    const size_t rb = sizeof(R) * g.N, sb = sizeof(V) * g.C;
    R *lam = (R *)st->d_r[0];
    V *S0 = (V *)st->d_s[0], *S1 = (V *)st->d_s[1];
    const double dtM = st->dt * st->M, dtMg = st->dt * st->M * st->gamma, invN = 1.0 / (double)g.N;
    // narrow tiles on grids too small to fill the GPU with the context's tile widths (512^2: 32
    // x-pass blocks at 16 rows per tile, 128 at 4)
    const int lbx = ((long long)(g.Y / ctx->LBx) * g.Z < 2 * 152) ? 4 : ctx->LBx;
    const int lby = ((long long)(g.KX / ctx->LBy) * g.Z < 2 * 152) ? 4 : ctx->LBy;
    int rc;
    if ((rc = gopf_real_to_state(ctx, st->d_stage))) return rc;
    ACK(cudaMemcpyAsync(st->d_seg, st->d_stage, rb, cudaMemcpyDeviceToDevice, ctx->stream));
    ACK(cudaMemcpyAsync(st->d_segT, ctx->d_T, sb, cudaMemcpyDeviceToDevice, ctx->stream));
    for (int n = 0; n < len; ++n) {
        if ((rc = gopf_step_device(ctx, 1))) return rc;
        if ((rc = gopf_state_to_real(ctx, (char *)st->d_seg + (size_t)(n + 1) * rb))) return rc;
        ACK(cudaMemcpyAsync((char *)st->d_segs + (size_t)(n + 1) * sb, ctx->d_state, sb, cudaMemcpyDeviceToDevice,
                            ctx->stream));
        ACK(cudaMemcpyAsync((char *)st->d_segT + (size_t)(n + 1) * sb, ctx->d_T, sb, cudaMemcpyDeviceToDevice,
                            ctx->stream));
    }
    for (int n = len - 1; n >= 0; --n) {
        const R *cn = (const R *)((char *)st->d_seg + (size_t)n * rb);
        const V *chat1 = (const V *)((char *)st->d_segs + (size_t)(n + 1) * sb);
        // f(c_n) from the step's own x-spectral field T_n: the c2r, the polynomial and the r2c of
        // one x pass (the register line engine where it serves the length)
        XPassArgs<R> xa;
        memset(&xa, 0, sizeof(xa));
        xa.g = g;
        xa.planH = ctx->planH;
        xa.twX = (const V *)ctx->d_twX;
        xa.allow_fast = ctx->use_fast;
        xa.status = ctx->d_status;
        xa.in_mode = XIN_SPECTRAL;
        xa.in = (const V *)((char *)st->d_segT + (size_t)n * sb);
        xa.out[0] = S1;
        xa.ngrp_out = 1;
        xa.pw.ngrp = 1;
        xa.pw.nterm[0] = 2;
        xa.pw.pw[0][0] = 3;
        xa.pw.coef[0][0] = 1.0;
        xa.pw.pw[0][1] = 1;
        xa.pw.coef[0][1] = -1.0;
        pw_densify(xa.pw);
        ACK(launch_xpass<R>(xa, lbx, ctx->stream));
        PassArgs<R> pa;
        memset(&pa, 0, sizeof(pa));
        pa.g = g;
        pa.plan = ctx->planY;
        pa.tw = (const V *)ctx->d_twY;
        pa.mode = PM_FWD;
        pa.buf[0] = S1;
        pa.buf[1] = S0;
        pa.nbuf = 2;
        pa.allow_fast = ctx->use_fast;
        pa.status = ctx->d_status;
        ACK(launch_cpass<R>(pa, lby, ctx->stream));
        if (g.Z > 1) {
            PassArgs<R> za = pa;
            za.plan = ctx->planZ;
            za.tw = (const V *)ctx->d_twZ;
            ACK(launch_spass<R>(za, ctx->LBz, ctx->stream));
        }
        k_adj_kspace<R><<<ew(g.C), 256, 0, ctx->stream>>>(g, S0, S1, chat1, dtMg, invN, st->d_sums);
        ACK(cudaGetLastError());
        pa.mode = PM_INV;
        pa.buf[0] = S0;
        pa.buf[1] = S1;
        if (g.Z > 1) {
            PassArgs<R> za = pa;
            za.plan = ctx->planZ;
            za.tw = (const V *)ctx->d_twZ;
            ACK(launch_spass<R>(za, ctx->LBz, ctx->stream));
        }
        ACK(launch_cpass<R>(pa, lby, ctx->stream));
        XPassArgs<R> xj;
        memset(&xj, 0, sizeof(xj));
        xj.g = g;
        xj.planH = ctx->planH;
        xj.twX = (const V *)ctx->d_twX;
        xj.allow_fast = ctx->use_fast;
        xj.status = ctx->d_status;
        xj.in_mode = XIN_SPECTRAL;
        xj.program = XP_ADJ;
        xj.in = S0;
        xj.in2 = S1;
        xj.rin = cn;
        xj.rout = lam;
        xj.out[0] = S0;
        xj.ngrp_out = 1;
        xj.adj_dtM = dtM;
        ACK(launch_xpass<R>(xj, lbx, ctx->stream));
    }
    return GOPF_OK;
}

template <typename R> static int adj_capture(gopf_ctx *ctx, gopf_adjoint_state *st, int len, cudaGraphExec_t *exec)
{
    cudaGraph_t graph;
    ACK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const long long step0 = ctx->step;
    int rc = adj_segment<R>(ctx, st, len);
    ctx->step = step0; // capturing runs nothing
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    if (rc) {
        if (e == cudaSuccess) cudaGraphDestroy(graph);
        return rc;
    }
    ACK(e);
    e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    ACK(e);
    return GOPF_OK;
}

template <typename R> static int adj_backward(gopf_ctx *ctx, gopf_adjoint_state *st, const double *lamT_host,
                                              double *dgamma, double *dM, double *dc0_host)
{
    typedef typename VecOf<R>::type V;
    const long long N = ctx->g.N;
    const size_t rb = sizeof(R) * N;
    R *lam = (R *)st->d_r[0];
    V *S0 = (V *)st->d_s[0];
    // lambda_T (host FP64) -> device R, and its r2c along x into S[0]
    std::vector<R> h(N);
    for (long long i = 0; i < N; ++i) h[i] = (R)lamT_host[i];
    ACK(cudaMemcpyAsync(lam, h.data(), rb, cudaMemcpyHostToDevice, ctx->stream));
    ACK(cudaMemsetAsync(st->d_sums, 0, 2 * sizeof(double), ctx->stream));
    {
        XPassArgs<R> xa;
        memset(&xa, 0, sizeof(xa));
        xa.g = ctx->g;
        xa.planH = ctx->planH;
        xa.twX = (const V *)ctx->d_twX;
        xa.allow_fast = ctx->use_fast;
        xa.status = ctx->d_status;
        xa.in_mode = XIN_REAL;
        xa.rin = lam;
        xa.out[0] = S0;
        xa.ngrp_out = 1;
        xa.identity = 1;
        ACK(launch_xpass<R>(xa, ctx->LBx, ctx->stream));
    }
    const double key[3] = {st->gamma, st->M, st->dt};
    if (memcmp(key, st->g_key, sizeof(key)) != 0) { // the graphs bake in gamma, M and dt
        adj_drop_graphs(st);
        memcpy(st->g_key, key, sizeof(key));
    }
    const double invN = 1.0 / (double)N;
    const int nseg = (st->nsteps + st->every - 1) / st->every;
    int rc;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int len = std::min(st->nsteps, (seg + 1) * st->every) - seg * st->every;
        ACK(cudaMemcpyAsync(st->d_stage, (char *)st->d_ckpt + (size_t)seg * rb, rb, cudaMemcpyDeviceToDevice,
                            ctx->stream));
        cudaGraphExec_t *ge = (len == st->every) ? &st->g_full : &st->g_tail;
        int *glen = (len == st->every) ? &st->g_full_len : &st->g_tail_len;
        if (!*ge || *glen != len) {
            if (*ge) cudaGraphExecDestroy(*ge);
            *ge = nullptr;
            if ((rc = adj_capture<R>(ctx, st, len, ge))) return rc;
            *glen = len;
        }
        ACK(cudaGraphLaunch(*ge, ctx->stream));
        ctx->step += len;
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
    if (ctx->d_status) { // a bounded tile wait that ran out inside the sweep
        unsigned stv = 0;
        ACK(cudaMemcpy(&stv, ctx->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost));
        if (stv) {
            ACK(cudaMemset(ctx->d_status, 0, sizeof(unsigned)));
            return gopf_fail(ctx, GOPF_ERR_TIMEOUT, "a device copy did not complete in time");
        }
    }
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
    gopf_adjoint_state *st = adj_state(ctx);
    int rc;
    // the model and stepper are installed again only when gamma, M or dt change: installing them
    // drops the context's captured step graphs, which repeated evaluations (a fit) can reuse
    const double mkey[3] = {gamma, M, dt};
    if (!st->model_set || memcmp(mkey, st->model_key, sizeof(mkey)) != 0 || !ctx->initialised ||
        ctx->stepper != GOPF_STEPPER_EULER || ctx->dt != dt) {
        if ((rc = gopf_set_terms(ctx, 1, &mu, 1, t, 2))) return rc;
        if ((rc = gopf_set_stepper(ctx, GOPF_STEPPER_EULER, dt))) return rc;
        memcpy(st->model_key, mkey, sizeof(mkey));
        st->model_set = true;
    }
    const long long N = ctx->g.N;
    const size_t rb = (ctx->prec == GOPF_FP32 ? sizeof(float) : sizeof(double)) * N;
    const size_t sb = (ctx->prec == GOPF_FP32 ? sizeof(float2) : sizeof(double2)) * ctx->g.C;
    const int nck = (nsteps + every - 1) / every + 1;
    if (st->nckpt < nck || st->every != every) {
        adj_drop_graphs(st); // they point into the buffers replaced here
        if (st->d_ckpt) cudaFree(st->d_ckpt);
        if (st->d_seg) cudaFree(st->d_seg);
        if (st->d_segs) cudaFree(st->d_segs);
        if (st->d_segT) cudaFree(st->d_segT);
        st->d_ckpt = st->d_seg = st->d_segs = st->d_segT = nullptr;
        ACK(gopf_malloc(&st->d_ckpt, rb * nck));
        ACK(gopf_malloc(&st->d_seg, rb * (every + 1)));
        ACK(gopf_malloc(&st->d_segs, sb * (every + 1)));
        ACK(gopf_malloc(&st->d_segT, sb * (every + 1)));
        st->nckpt = nck;
    }
    if (!st->d_stage) ACK(gopf_malloc(&st->d_stage, rb));
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
    // one checkpoint per segment, the segment's steps replayed from the context's step graphs
    for (int s0 = 0; s0 < nsteps; s0 += every) {
        if ((rc = gopf_state_to_real(ctx, (char *)st->d_ckpt + (size_t)(s0 / every) * rb))) return rc;
        if ((rc = gopf_step(ctx, std::min(every, nsteps - s0)))) return rc;
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
    adj_drop_graphs(s);
    void *ptrs[] = {s->d_ckpt, s->d_seg,  s->d_segs, s->d_segT, s->d_stage, s->d_r[0], s->d_r[1],
                    s->d_r[2], s->d_r[3], s->d_s[0], s->d_s[1],  s->d_s[2],  s->d_sums};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete s;
    g_adj.erase(it);
    return GOPF_OK;
}
