// gopf_api.cu -- C ABI of the GB300 spectral stepper: contexts, device
// buffers, plans, the step sequence and its CUDA-graph replay.
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gopf_ctx.h"
#include "gopf_kernels.cuh"

using namespace gopf;

// ------------------------------------------------------------------
// errors
// ------------------------------------------------------------------

int gopf_fail(gopf_ctx *ctx, int code, const std::string &msg)
{
    if (ctx) ctx->err = msg;
    return code;
}

static int cuda_fail(gopf_ctx *ctx, cudaError_t e, const char *where)
{
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    return gopf_fail(ctx, e == cudaErrorMemoryAllocation ? GOPF_ERR_OOM : GOPF_ERR_CUDA, m);
}

#define CK(call)                                                                                                       \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);                                                       \
    } while (0)

extern "C" const char *gopf_status_string(int s)
{
    switch (s) {
    case GOPF_OK: return "ok";
    case GOPF_ERR_ARG: return "bad argument";
    case GOPF_ERR_CUDA: return "CUDA error";
    case GOPF_ERR_OOM: return "out of device memory";
    case GOPF_ERR_NAN: return "non-finite value in field";
    case GOPF_ERR_TIMEOUT: return "device wait timed out";
    case GOPF_ERR_UNSUPPORTED: return "unsupported on the device";
    case GOPF_ERR_STATE: return "call out of order";
    case GOPF_ERR_PARSE: return "equation parse error";
    default: return "unknown status";
    }
}

extern "C" const char *gopf_last_error(const gopf_ctx *ctx)
{
    return ctx ? ctx->err.c_str() : "null context";
}

// ------------------------------------------------------------------
// plans and twiddle tables
// ------------------------------------------------------------------

// Runtime Stockham plan of length n over a twiddle table of n * tws entries.  variant 0: radix 3s,
// 5s, 7s, then 2^(a mod 4), then 16s; variant 1: the power of two in radix-8 stages (a 2 or 4 for
// the remainder); variant 2: in radix-4 stages.  All variants use the same table.
bool gopf_make_plan(int n, int tws, int variant, LinePlan &pl)
{
    memset(&pl, 0, sizeof(pl));
    pl.n = n;
    if (n < 1) return false;
    int m = n, a = 0, b = 0, c5 = 0, c7 = 0;
    while (m % 2 == 0) { m /= 2; ++a; }
    while (m % 3 == 0) { m /= 3; ++b; }
    while (m % 5 == 0) { m /= 5; ++c5; }
    while (m % 7 == 0) { m /= 7; ++c7; }
    if (m != 1) return false;
    // radix 3s, 5s, 7s, then 2^(a mod 4), then 16s (for 2^a 3^b the order of the compile-time plans)
    std::vector<int> rad;
    for (int i = 0; i < b; ++i) rad.push_back(3);
    for (int i = 0; i < c5; ++i) rad.push_back(5);
    for (int i = 0; i < c7; ++i) rad.push_back(7);
    const int q = (variant == 1) ? 3 : (variant == 2) ? 2 : 4; // log2 of the main radix
    if (a % q) rad.push_back(1 << (a % q));
    for (int i = 0; i < a / q; ++i) rad.push_back(1 << q);
    if ((int)rad.size() > GOPF_MAX_STAGES) return false;
    pl.nst = (int)rad.size();
    int ns = 1;
    for (int s = 0; s < pl.nst; ++s) {
        pl.rad[s] = rad[s];
        pl.ns[s] = ns;
        pl.nsmask[s] = ((ns & (ns - 1)) == 0) ? ns - 1 : -1;
        pl.twmul[s] = (int)((long long)n * tws / ((long long)ns * rad[s]));
        ns *= rad[s];
    }
    return true;
}

template <typename R> static int upload_table(gopf_ctx *ctx, int n, void **dptr)
{
    typedef typename VecOf<R>::type V;
    std::vector<V> h(n);
    for (int t = 0; t < n; ++t) {
        long double ang = -2.0L * 3.141592653589793238462643383279502884L * (long double)t / (long double)n;
        h[t].x = (R)cosl(ang);
        h[t].y = (R)sinl(ang);
    }
    CK(gopf_malloc(dptr, sizeof(V) * n));
    ctx->dev_bytes += sizeof(V) * n;
    CK(cudaMemcpy(*dptr, h.data(), sizeof(V) * n, cudaMemcpyHostToDevice));
    return GOPF_OK;
}

// ------------------------------------------------------------------
// small elementwise kernels
// ------------------------------------------------------------------

template <typename R>
__global__ void k_c128_to_real(const double2 *__restrict__ in, R *__restrict__ out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (R)in[i].x;
}

template <typename R>
__global__ void k_real_to_c128(const R *__restrict__ in, double2 *__restrict__ out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = make_double2((double)in[i], 0.0);
}

template <typename R>
__global__ void k_double_to_real(const double *__restrict__ in, R *__restrict__ out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (R)in[i];
}

template <typename R>
__global__ void k_real_to_double(const R *__restrict__ in, double *__restrict__ out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

// Final cross-block reduction: one block per slot (launched with RED_NONFINITE + 1 blocks of a
// multiple of 32 threads).  Each thread folds a strided share of the block partials (the sums with
// Neumaier compensation); a fixed-order shuffle tree and the warps' results in order then combine
// the (sum, error) pairs, adding each combination's rounding error to the error terms.  The result
// is deterministic, and the slots' FP64 dependency chains run on separate SMs (GB300 runs FP64 at a
// small fraction of its FP32 rate).
__global__ void k_finish_reduce(const double *__restrict__ part, int nblocks, double *__restrict__ out)
{
    // one block per slot (RED_SUM, RED_SUMSQ: Neumaier; RED_MIN, RED_MAX; RED_NONFINITE: a count), so
    // that the slots' FP64 chains run on separate SMs
    const int slot = blockIdx.x;
    const bool comp = (slot == RED_SUM || slot == RED_SUMSQ);
    double v = (slot == RED_MIN) ? INFINITY : (slot == RED_MAX) ? -INFINITY : 0.0, c = 0.0;
    auto nsum = [](double &s, double &cc, double x) {
        const double t = s + x;
        cc += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
        s = t;
    };
    auto combine = [&](double x, double xc) {
        if (comp) {
            c += xc;
            nsum(v, c, x);
        } else if (slot == RED_MIN) {
            v = fmin(v, x);
        } else if (slot == RED_MAX) {
            v = fmax(v, x);
        } else {
            v += x;
        }
    };
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) combine(part[(long long)b * RED_SLOTS + slot], 0.0);
    for (int o = 16; o > 0; o >>= 1) {
        const double x = __shfl_xor_sync(0xffffffffu, v, o), xc = __shfl_xor_sync(0xffffffffu, c, o);
        combine(x, xc);
    }
    __shared__ double s_v[32], s_c[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        s_v[w] = v;
        s_c[w] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        v = (slot == RED_MIN) ? INFINITY : (slot == RED_MAX) ? -INFINITY : 0.0;
        c = 0.0;
        for (int q = 0; q < (int)blockDim.x / 32; ++q) combine(s_v[q], s_c[q]);
        out[slot] = comp ? v + c : v;
    }
}

// Number of non-finite values among n reals.  A non-finite cell makes every
// coefficient of the spectrum non-finite and vice versa, so counting over the
// spectral state answers "is the field finite" without a transform.
template <typename R> __global__ void k_count_nonfinite(const R *__restrict__ x, long long n, unsigned *__restrict__ count)
{
    unsigned local = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        local += isfinite(x[i]) ? 0u : 1u;
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, local);
}

cudaError_t gopf_malloc(void **p, size_t bytes)
{
    static std::atomic<long long> countdown{-2}; // -2: not read yet, -1: hook off
    long long c = countdown.load();
    if (c == -2) {
        const char *e = std::getenv("GOPF_TEST_FAIL_ALLOC");
        const long long k = e ? std::atoll(e) : 0;
        long long expect = -2;
        countdown.compare_exchange_strong(expect, k > 0 ? k : -1);
    }
    if (countdown.load() > 0 && countdown.fetch_sub(1) == 1) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}

static unsigned ew_blocks(long long n)
{
    long long b = (n + 255) / 256;
    return (unsigned)std::min<long long>(b, 152 * 16);
}

// ------------------------------------------------------------------
// context
// ------------------------------------------------------------------

static int set_device(gopf_ctx *ctx)
{
    if (ctx->device < 0)
        return gopf_fail(ctx, GOPF_ERR_STATE, "host-only context (device < 0): model definition only");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
    return GOPF_OK;
}

static int check_len(int n, const char *what, gopf_ctx *ctx)
{
    LinePlan p;
    if (!gopf_make_plan(n, 1, 0, p))
        return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED,
                         std::string(what) + " length " + std::to_string(n) + " must be 2^a*3^b*5^c*7^d");
    return GOPF_OK;
}

template <typename R> static int ctx_alloc(gopf_ctx *ctx)
{
    typedef typename VecOf<R>::type V;
    const Geom &g = ctx->g;
    CK(gopf_malloc(&ctx->d_state, sizeof(V) * g.C));
    CK(gopf_malloc(&ctx->d_T, sizeof(V) * g.C));
    CK(gopf_malloc(&ctx->d_real, sizeof(R) * g.N));
    CK(gopf_malloc(&ctx->d_c128, sizeof(double2) * g.N));
    ctx->dev_bytes += 2 * sizeof(V) * g.C + sizeof(R) * g.N + sizeof(double2) * g.N;
    ctx->nred_blocks = ((g.Y + ctx->LBx - 1) / ctx->LBx) * g.Z;
    CK(gopf_malloc(&ctx->d_red, sizeof(double) * RED_SLOTS * ctx->nred_blocks));
    CK(gopf_malloc(&ctx->d_redout, sizeof(double) * RED_SLOTS));
    // [0] status word, [1] non-finite count, [2..3] the first-wait limit of the bounded waits in ns
    // (an unsigned long long; 0 = the built-in 2 s)
    CK(gopf_malloc(&ctx->d_status, 4 * sizeof(unsigned)));
    CK(cudaMemset(ctx->d_status, 0, 4 * sizeof(unsigned)));
    ctx->dev_bytes += sizeof(double) * RED_SLOTS * (ctx->nred_blocks + 1) + sizeof(unsigned);
    CK(cudaMemset(ctx->d_state, 0, sizeof(V) * g.C));
    CK(cudaMemset(ctx->d_T, 0, sizeof(V) * g.C));
    int rc;
    if ((rc = upload_table<R>(ctx, g.X, &ctx->d_twX))) return rc;
    if ((rc = upload_table<R>(ctx, g.Y, &ctx->d_twY))) return rc;
    if (g.Z > 1 && (rc = upload_table<R>(ctx, g.Z, &ctx->d_twZ))) return rc;
    return GOPF_OK;
}

void gopf_ie_free(gopf_ctx *ctx);
int gopf_ie_step(gopf_ctx *ctx);
void gopf_sdd_free(gopf_ctx *ctx);
int gopf_sdd_step(gopf_ctx *ctx, long long nsteps);
void gopf_io_free(gopf_ctx *ctx);
void gopf_energy_free(gopf_ctx *ctx);

static void ctx_free(gopf_ctx *ctx)
{
    gopf_io_free(ctx);
    gopf_energy_free(ctx);
    gopf_ie_free(ctx);
    gopf_sdd_free(ctx);
    if (ctx->gexec1) cudaGraphExecDestroy(ctx->gexec1);
    if (ctx->gexecK) cudaGraphExecDestroy(ctx->gexecK);
    void *ptrs[] = {ctx->d_state, ctx->d_T, ctx->d_real, ctx->d_c128, ctx->d_red, ctx->d_redout,
                    ctx->d_twX,   ctx->d_twY, ctx->d_twZ};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (int i = 1; i < GOPF_MAX_GROUPS; ++i)
        if (ctx->d_U[i]) cudaFree(ctx->d_U[i]);
    for (int f = 1; f < GOPF_MAX_FIELDS; ++f) {
        if (ctx->d_fstate[f]) cudaFree(ctx->d_fstate[f]);
        if (ctx->d_fT[f]) cudaFree(ctx->d_fT[f]);
        if (ctx->d_frkF[f]) cudaFree(ctx->d_frkF[f]);
    }
    for (int i = 0; i < GOPF_MAX_XOUT; ++i)
        if (ctx->d_mU[i]) cudaFree(ctx->d_mU[i]);
    void *more[] = {ctx->d_bsym,    ctx->d_U0,     ctx->d_UH,     ctx->d_vc,     ctx->d_red2,   ctx->d_rkF,
                    ctx->d_stepctr, ctx->d_status, ctx->d_filter, ctx->d_srcamp, ctx->d_srcctr, ctx->d_vcred};
    for (void *p : more)
        if (p) cudaFree(p);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    if (ctx->side_stream) cudaStreamDestroy(ctx->side_stream);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
}

extern "C" int gopf_ctx_create(int ndim, const int *domain_size, int precision, int device, gopf_ctx **out)
{
    if (!out) return GOPF_ERR_ARG;
    *out = nullptr;
    if ((ndim != 2 && ndim != 3) || !domain_size) return GOPF_ERR_ARG;
    if (precision != GOPF_FP32 && precision != GOPF_FP64) return GOPF_ERR_ARG;
    gopf_ctx *ctx = new gopf_ctx();
    ctx->device = device;
    ctx->ndim = ndim;
    ctx->prec = precision;
    for (int d = 0; d < ndim; ++d) {
        if (domain_size[d] < 1) { delete ctx; return GOPF_ERR_ARG; }
        ctx->dims[d] = domain_size[d];
    }
    if (ndim == 3 && !(domain_size[0] == domain_size[1] && domain_size[1] == domain_size[2])) {
        // pfutil/fftWrap.go plans FFTW over [n0][n1][n2] while Freq/Pos use depth-major
        // node order; the two agree only for cubes, so only cubes are accepted in 3D.
        ctx->err = "3D domains must be cubic (the reference's FFT and Freq conventions agree only for cubes)";
        *out = ctx;
        return GOPF_ERR_UNSUPPORTED;
    }
    Geom &g = ctx->g;
    g.X = ctx->dims[1];
    g.Y = ctx->dims[0];
    g.Z = (ndim == 3) ? ctx->dims[2] : 1;
    *out = ctx;
    const bool oddx = (g.X % 2) != 0; // odd column counts: row pairs through length-X transforms
    int rc;
    if ((rc = check_len(oddx ? g.X : g.X / 2, oddx ? "column" : "half column", ctx))) return rc;
    if ((rc = check_len(g.Y, "row", ctx))) return rc;
    if ((rc = check_len(g.Z, "depth", ctx))) return rc;
    g.H = g.X / 2;
    g.KX = g.H + 1;
    g.S = (long long)g.KX * g.Y;
    g.C = g.S * g.Z;
    g.N = (long long)g.X * g.Y * g.Z;
    const int vb = (precision == GOPF_FP32) ? 8 : 16;
    ctx->LBx = lb_for(oddx ? g.KX : g.H, vb);
    ctx->LBy = lb_for(g.Y, vb);
    ctx->LBz = lb_for(g.Z, vb);
    if ((long long)ctx->LBx * g.H > 4096 || (long long)ctx->LBy * g.Y > 4096 || (long long)ctx->LBz * g.Z > 4096)
        return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "axis longer than 1024 (2048 columns) is not supported");
    // Small grids: narrower tiles (down to 4 lines), so that each pass of the generic kernels has
    // about two tiles per SM; a pass of a few tiles otherwise takes as long as one block's
    // transforms (FP64 arithmetic runs at a small fraction of the FP32 rate).  The tile width does
    // not change a line's arithmetic.
    {
        int nsm = 152;
        if (device >= 0) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
        auto narrow = [&](int lb, long long lines) {
            while (lb > 4 && (lines + lb - 1) / lb < 2LL * nsm) lb /= 2;
            return lb;
        };
        ctx->LBx = narrow(ctx->LBx, (long long)g.Y * g.Z);
        ctx->LBy = narrow(ctx->LBy, (long long)g.KX * g.Z);
        if (g.Z > 1) ctx->LBz = narrow(ctx->LBz, g.S);
    }
    if (oddx) gopf_make_plan(g.X, 1, 0, ctx->planH); // the x transform of the row pairs
    else gopf_make_plan(g.H, 2, 0, ctx->planH);
    gopf_make_plan(g.Y, 1, 0, ctx->planY);
    gopf_make_plan(g.Z, 1, 0, ctx->planZ);
    if (device < 0) return GOPF_OK; // host-only: equations can be defined and compiled, nothing runs
    if ((rc = set_device(ctx))) return rc;
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->side_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamCreate");
    ctx->stream = ctx->own_stream;
    rc = (precision == GOPF_FP32) ? ctx_alloc<float>(ctx) : ctx_alloc<double>(ctx);
    return rc;
}

extern "C" int gopf_adjoint_release(gopf_ctx *ctx);

extern "C" int gopf_ctx_destroy(gopf_ctx *ctx)
{
    if (!ctx) return GOPF_ERR_ARG;
    if (ctx->device >= 0) gopf_adjoint_release(ctx);
    if (ctx->device >= 0) {
        cudaSetDevice(ctx->device);
        if (ctx->stream) cudaStreamSynchronize(ctx->stream);
        ctx_free(ctx);
    }
    delete ctx;
    return GOPF_OK;
}

static void invalidate_graphs(gopf_ctx *ctx)
{
    if (ctx->gexec1) cudaGraphExecDestroy(ctx->gexec1);
    if (ctx->gexecK) cudaGraphExecDestroy(ctx->gexecK);
    ctx->gexec1 = ctx->gexecK = nullptr;
    ctx->graphs_dirty = true;
}

extern "C" int gopf_set_stream(gopf_ctx *ctx, void *s)
{
    if (!ctx) return GOPF_ERR_ARG;
    int rc;
    if ((rc = set_device(ctx))) return rc;
    ctx->stream = s ? (cudaStream_t)s : ctx->own_stream;
    return GOPF_OK;
}

extern "C" int gopf_set_option(gopf_ctx *ctx, int opt, long long v)
{
    if (!ctx) return GOPF_ERR_ARG;
    if (opt == GOPF_OPT_CHECK_FINITE) ctx->check_finite = (int)(v != 0);
    else if (opt == GOPF_OPT_USE_GRAPHS) ctx->use_graphs = (int)(v != 0);
    else if (opt == GOPF_OPT_FAST_KERNELS) ctx->use_fast = (int)(v != 0);
    else if (opt == GOPF_OPT_DIRECT_HOST) ctx->use_direct_host = (int)(v != 0);
    else if (opt == GOPF_OPT_TMA) ctx->use_tma = (int)(v != 0);
    else if (opt == GOPF_OPT_Z_LINES) {
        if (v != 8 && v != 16) return gopf_fail(ctx, GOPF_ERR_ARG, "the z tile width is 8 or 16 lines");
        ctx->z_lines = (int)v;
    } else if (opt == GOPF_OPT_PDL) {
        ctx->use_pdl = (int)(v != 0);
    } else if (opt == GOPF_OPT_X_ROWS) {
        if (v != 16 && v != 32) return gopf_fail(ctx, GOPF_ERR_ARG, "the x tile height is 16 or 32 rows");
        ctx->x_rows = (int)v;
    }
    else if (opt == GOPF_OPT_WAIT_LIMIT_NS) {
        if (v < 0) return gopf_fail(ctx, GOPF_ERR_ARG, "negative wait limit");
        if (!ctx->d_status) return gopf_fail(ctx, GOPF_ERR_STATE, "context has no device");
        int rc;
        if ((rc = set_device(ctx))) return rc;
        const unsigned long long lim = (unsigned long long)v;
        CK(cudaMemcpyAsync(ctx->d_status + 2, &lim, sizeof(lim), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        return GOPF_OK; // kernels read the limit at run time: captured graphs stay valid
    } else return gopf_fail(ctx, GOPF_ERR_ARG, "unknown option");
    invalidate_graphs(ctx); // captured launches carry the old choice
    return GOPF_OK;
}

// ------------------------------------------------------------------
// model compilation: term table -> device tables
// ------------------------------------------------------------------

// Expand a derived field of field 0 into polynomial terms (coef, power).
static int derived_poly(gopf_ctx *ctx, const gopf_derived &d, std::vector<std::pair<double, int>> &out)
{
    out.clear();
    switch (d.kind) {
    case GOPF_DER_PRODUCT: {
        int p = 0;
        for (int j = 0; j < d.nfac; ++j) {
            if (d.field[j] != 0)
                return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "derived fields of several fields are not on the device yet");
            if (d.power[j] < 0) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "negative powers are not on the device");
            p += d.power[j];
        }
        out.push_back({1.0, p});
        break;
    }
    case GOPF_DER_POLY:
        for (int j = 0; j < d.nfac; ++j) {
            if (d.field[j] != 0)
                return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "derived fields of several fields are not on the device yet");
            if (d.power[j] < 0) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "negative powers are not on the device");
            out.push_back({d.coef[j], d.power[j]});
        }
        break;
    case GOPF_DER_MPOLY:
        for (int j = 0; j < d.nfac; ++j) {
            const unsigned packed = (unsigned)d.power[j];
            if (packed >> 8)
                return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "derived fields of several fields are not on the device yet");
            out.push_back({d.coef[j], (int)packed});
        }
        break;
    case GOPF_DER_INDICATOR: out = {{3.0, 2}, {-2.0, 3}}; break;
    case GOPF_DER_INDICATOR_D: out = {{6.0, 1}, {-6.0, 2}}; break;
    case GOPF_DER_INDICATOR_HD: out = {{18.0, 3}, {-30.0, 4}, {12.0, 5}}; break;
    case GOPF_DER_WHITE_NOISE:
        return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "white noise enters only as a term of its own");
    default: return gopf_fail(ctx, GOPF_ERR_ARG, "unknown derived-field kind");
    }
    return GOPF_OK;
}

static unsigned long long noise_seed_of(gopf_ctx *ctx, int derived_index)
{
    if (derived_index < (int)ctx->def.derived_names.size()) {
        const std::string &nm = ctx->def.derived_names[derived_index];
        for (auto &nz : ctx->def.noise)
            if (nz.kind == 1 && nz.name == nm) return nz.seed;
    }
    return 0;
}

static int add_poly_to_group(gopf_ctx *ctx, PwTable &pw, int grp, const std::vector<std::pair<double, int>> &poly,
                             double coef)
{
    for (auto &pc : poly) {
        int at = -1; // merge equal powers
        for (int q = 0; q < pw.nterm[grp]; ++q)
            if (pw.pw[grp][q] == pc.second) at = q;
        if (at < 0) {
            if (pw.nterm[grp] >= GOPF_MAX_POLY) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "polynomial too long");
            at = pw.nterm[grp]++;
            pw.pw[grp][at] = pc.second;
            pw.coef[grp][at] = 0.0;
        }
        pw.coef[grp][at] += coef * pc.first;
    }
    return GOPF_OK;
}

static int alloc_spectral(gopf_ctx *ctx, void **p)
{
    if (ctx->device < 0 || *p) return GOPF_OK;
    const size_t vb = (ctx->prec == GOPF_FP32) ? sizeof(float2) : sizeof(double2);
    cudaError_t e = gopf_malloc(p, vb * ctx->g.C);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "gopf_malloc(work buffer)");
    ctx->dev_bytes += vb * ctx->g.C;
    return GOPF_OK;
}

// Block sums of the volume-conserving term: enough slots for any x-pass grid (tile width >= 4).
static long long vc_red_blocks(const gopf_ctx *ctx) { return (long long)((ctx->g.Y + 3) / 4) * ctx->g.Z; }

static int alloc_volcons(gopf_ctx *ctx, bool field_sums)
{
    const size_t bytes = sizeof(double) * RED_SLOTS * (size_t)vc_red_blocks(ctx);
    if (!ctx->d_vc) {
        CK(gopf_malloc(&ctx->d_vc, sizeof(double) * 8));
        CK(gopf_malloc(&ctx->d_red2, bytes));
        ctx->dev_bytes += sizeof(double) * 8 + bytes;
    }
    if (field_sums && !ctx->d_vcred) {
        CK(gopf_malloc(&ctx->d_vcred, bytes));
        ctx->dev_bytes += bytes;
    }
    CK(cudaMemset(ctx->d_vc, 0, sizeof(double) * 8));
    return GOPF_OK;
}

// HomogeneousModulusLinElast's constants (pf/homoLinElast.go:47-99): the stiffness, the effective
// stress A = C : misfit (elasticity/rank4.go:62-75) and the misfit energy density e0
// (elasticity/linearElasticity.go:86-98).
static void set_elastic_params(gopf_ctx *ctx, const gopf_modeldef::Elastic &e, const gopf_special &sp)
{
    memcpy(ctx->el_C, e.C, sizeof(ctx->el_C));
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double a = 0.0;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) a += e.C[i * 27 + j * 9 + k * 3 + l] * e.misfit[k * 3 + l];
            ctx->el_A[i * 3 + j] = a;
        }
    double e0 = 0.0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l)
                    e0 += e.C[i * 27 + j * 9 + k * 3 + l] * e.misfit[i * 3 + j] * e.misfit[k * 3 + l];
    ctx->el_e0 = 0.5 * e0;
    ctx->el_coef = sp.coef;
    ctx->el_lap = sp.lap;
}

static int find_derived(const gopf_ctx *ctx, const std::string &name)
{
    for (size_t i = 0; i < ctx->def.derived_names.size(); ++i)
        if (ctx->def.derived_names[i] == name) return (int)i;
    return -1;
}

// ---- multi-field models ----


struct Mono {
    double coef;
    unsigned char pw[GOPF_MAX_FIELDS];
};

// A derived field as monomials of the model's fields (pf/util.go:38-65: products of
// field powers; RegisterFunction polynomials and the indicator functions of one field).
static int derived_mono(gopf_ctx *ctx, const gopf_derived &d, std::vector<Mono> &out)
{
    out.clear();
    auto field_ok = [&](int f, int p) {
        return f >= 0 && f < ctx->nfields && p >= 0 && p <= 64;
    };
    if (d.kind == GOPF_DER_PRODUCT) {
        Mono m{1.0, {0, 0, 0, 0}};
        for (int j = 0; j < d.nfac; ++j) {
            if (!field_ok(d.field[j], d.power[j]))
                return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "derived field with a negative or too large power");
            m.pw[d.field[j]] = (unsigned char)(m.pw[d.field[j]] + d.power[j]);
        }
        out.push_back(m);
        return GOPF_OK;
    }
    if (d.kind == GOPF_DER_POLY) {
        for (int j = 0; j < d.nfac; ++j) {
            if (!field_ok(d.field[j], d.power[j]))
                return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "polynomial with a negative or too large power");
            Mono m{d.coef[j], {0, 0, 0, 0}};
            m.pw[d.field[j]] = (unsigned char)d.power[j];
            out.push_back(m);
        }
        return GOPF_OK;
    }
    if (d.kind == GOPF_DER_MPOLY) {
        for (int j = 0; j < d.nfac; ++j) {
            Mono m{d.coef[j], {0, 0, 0, 0}};
            const unsigned packed = (unsigned)d.power[j];
            for (int f = 0; f < GOPF_MAX_FIELDS; ++f) {
                const int p = (int)((packed >> (8 * f)) & 0xffu);
                if (p && !field_ok(f, p))
                    return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "polynomial of a field the model does not have");
                m.pw[f] = (unsigned char)p;
            }
            out.push_back(m);
        }
        return GOPF_OK;
    }
    if (d.kind == GOPF_DER_WHITE_NOISE)
        return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "white noise enters only as a term of its own");
    std::vector<std::pair<double, int>> poly;
    gopf_derived d0 = d;
    d0.field[0] = 0; // derived_poly expands the indicator kinds of one field
    int rc = derived_poly(ctx, d0, poly);
    if (rc) return rc;
    if (!field_ok(d.field[0], 0)) return gopf_fail(ctx, GOPF_ERR_ARG, "bad field index");
    for (auto &pc : poly) {
        Mono m{pc.first, {0, 0, 0, 0}};
        m.pw[d.field[0]] = (unsigned char)pc.second;
        out.push_back(m);
    }
    return GOPF_OK;
}

// Term table of a model with several fields -> one monomial table for the shared x-pass and
// one update table per equation (equation e evolves field e, pf/euler.go:33-44).
//
// Euler.Step updates the fields one after the other in place, in k space, before any inverse
// transform (pf/euler.go:31-42): an explicit term that is another field f itself (a Field brick,
// "LAP conc" in the phi equation) reads f's c-hat as it is at that moment, i.e. already updated
// when f < e.  Derived fields were synced at the start of the step.  So with kfield set (the
// Euler plan) such terms stay in k space (UpdTable::xf_*) and read the state arrays, which the
// per-equation updates rewrite in the same order.  RK4 evaluates every right-hand side after all
// fields of a stage are formed (pf/rk4.go:101-127): its plan (kfield false) puts them in the
// x-pass like any product.
static int build_multi_plan(gopf_ctx *ctx, bool kfield, std::vector<gopf_ctx::EqPlan> &eqs, MonoTable &mt,
                            int &nextra)
{
    const int nf = ctx->nfields;
    eqs.assign(nf, gopf_ctx::EqPlan());
    for (auto &ep : eqs) {
        memset(&ep, 0, sizeof(ep));
        for (int b = 0; b < GOPF_MAX_GROUPS; ++b) ep.ubuf[b] = -1;
    }
    // per equation: groups keyed by LAP power, each a list of monomials
    std::vector<std::vector<std::vector<Mono>>> gm(nf);
    std::vector<int> maxp(nf, 0);
    int noise_eq = -1; // the equation with the model's noise term (WhiteNoise / ConservativeNoise)
    double noise_strength = 0.0;
    unsigned long long noise_seed = 0;
    for (const gopf_term &t : ctx->terms) {
        if (t.eq < 0 || t.eq >= nf) return gopf_fail(ctx, GOPF_ERR_ARG, "term refers to an equation that does not exist");
        if (t.lap < 0 || t.lap >= GOPF_MAX_IMP) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "LAP power out of range");
        gopf_ctx::EqPlan &ep = eqs[t.eq];
        UpdTable &u = ep.upd;
        if (t.implicit) {
            u.imp[t.lap] += t.coef;
            maxp[t.eq] = std::max(maxp[t.eq], t.lap + 1);
            continue;
        }
        std::vector<Mono> ms;
        if (t.source == GOPF_SRC_FIELD) {
            if (t.src_index < 0 || t.src_index >= nf) return gopf_fail(ctx, GOPF_ERR_ARG, "bad field index");
            if (kfield) {
                int at = -1;
                for (int q = 0; q < u.nxf; ++q)
                    if (ep.xf_field[q] == t.src_index && u.xf_lap[q] == t.lap) at = q;
                if (at < 0) {
                    if (u.nxf >= GOPF_MAX_FIELDS)
                        return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "too many field terms in one equation");
                    at = u.nxf++;
                    ep.xf_field[at] = t.src_index;
                    u.xf_lap[at] = t.lap;
                    u.xf_coef[at] = 0.0;
                }
                u.xf_coef[at] += t.coef;
                continue;
            }
            Mono m{1.0, {0, 0, 0, 0}};
            m.pw[t.src_index] = 1;
            ms.push_back(m);
        } else if (t.source == GOPF_SRC_DERIVED) {
            if (t.src_index < 0 || t.src_index >= (int)ctx->der.size())
                return gopf_fail(ctx, GOPF_ERR_ARG, "bad derived-field index");
            if (ctx->der[t.src_index].kind == GOPF_DER_WHITE_NOISE) { // drawn in the equation's update
                if (noise_eq >= 0) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "one noise term per model");
                noise_eq = t.eq;
                u.noise.kind = 1;
                u.noise.coef = t.coef;
                u.noise.lap = t.lap;
                noise_strength = ctx->der[t.src_index].coef[0];
                noise_seed = noise_seed_of(ctx, t.src_index);
                continue;
            }
            int rc = derived_mono(ctx, ctx->der[t.src_index], ms);
            if (rc) return rc;
        } else {
            return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED,
                             "a term without a field (constant in k space) has no device implementation");
        }
        int grp = -1;
        for (int b = 0; b < u.ngrp; ++b)
            if (u.glap[b] == t.lap) grp = b;
        if (grp < 0) {
            if (u.ngrp >= GOPF_MAX_GROUPS) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "too many distinct LAP powers");
            grp = u.ngrp++;
            u.glap[grp] = t.lap;
            gm[t.eq].emplace_back();
        }
        for (const Mono &m : ms) { // merge equal power vectors
            bool merged = false;
            for (Mono &q : gm[t.eq][grp])
                if (!memcmp(q.pw, m.pw, sizeof(m.pw))) {
                    q.coef += t.coef * m.coef;
                    merged = true;
                }
            if (!merged) {
                if ((int)gm[t.eq][grp].size() >= GOPF_MAX_MONO)
                    return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "too many distinct products in one term group");
                gm[t.eq][grp].push_back({t.coef * m.coef, {m.pw[0], m.pw[1], m.pw[2], m.pw[3]}});
            }
        }
    }
    // The elastic and volume-conserving terms are stepped with Euler only (gopf_step rejects RK4
    // for them), so only the Euler plan carries them.
    bool have_el = false, have_vc = false;
    for (const gopf_special &sp : ctx->specials) {
        if (sp.eq < 0 || sp.eq >= nf) return gopf_fail(ctx, GOPF_ERR_ARG, "term refers to an equation that does not exist");
        if (sp.kind == 1) {
            if (have_el) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "one elastic term per model");
            have_el = true;
            if (!kfield) continue;
            const gopf_modeldef::Elastic &e = ctx->def.elastic[sp.index];
            if (e.field < 0 || e.field >= nf) return gopf_fail(ctx, GOPF_ERR_ARG, "bad field index");
            if (eqs[sp.eq].upd.ngrp >= GOPF_MAX_GROUPS)
                return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "too many term groups with the elastic term");
            ctx->el_field = e.field;
            ctx->el_eq = sp.eq;
            set_elastic_params(ctx, e, sp);
            continue;
        }
        if (sp.kind == 2) {
            if (have_vc) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "one volume-conserving term per model");
            have_vc = true;
            if (!kfield) continue;
            const gopf_modeldef::Volcons &v = ctx->def.volcons[sp.index];
            if (v.field < 0 || v.field >= nf) return gopf_fail(ctx, GOPF_ERR_ARG, "bad field index");
            const int did = find_derived(ctx, v.indicator);
            if (did < 0) return gopf_fail(ctx, GOPF_ERR_ARG, "VolumeConservingLP: Indicator is not a derived field");
            std::vector<Mono> ms;
            int rc = derived_mono(ctx, ctx->def.derived[did], ms);
            if (rc) return rc;
            if ((int)ms.size() > GOPF_MAX_MONO)
                return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "too many distinct products in one term group");
            // a group of its own: the update scales it by the device multiplier
            UpdTable &u = eqs[sp.eq].upd;
            if (u.ngrp >= GOPF_MAX_GROUPS) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "too many term groups");
            const int grp = u.ngrp++;
            u.glap[grp] = sp.lap;
            gm[sp.eq].emplace_back(ms);
            ctx->vc_field = v.field;
            ctx->vc_eq = sp.eq;
            ctx->vc_local = grp;
            ctx->vc_dt = v.dt;
            ctx->vc_coef = sp.coef;
            continue;
        }
        if (sp.kind == 3) {
            const gopf_modeldef::Noise &nz = ctx->def.noise[sp.index];
            if (noise_eq >= 0) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "one noise term per model");
            noise_eq = sp.eq;
            UpdTable &u = eqs[sp.eq].upd;
            u.noise.kind = 2;
            u.noise.coef = sp.coef;
            u.noise.lap = sp.lap;
            noise_strength = nz.strength;
            noise_seed = nz.seed;
            continue;
        }
        if (sp.kind != 4) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "user-defined term kind has no device implementation");
        const gopf_modeldef::ImplicitSym &is = ctx->def.isym[sp.index];
        UpdTable &u = eqs[sp.eq].upd;
        if (u.nxs >= GOPF_MAX_XSYM) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "too many implicit user terms");
        XSym &x = u.xs[u.nxs++];
        memset(&x, 0, sizeof(x));
        x.kind = is.kind;
        x.coef = sp.coef;
        x.lap = sp.lap;
        memcpy(x.K, is.K, sizeof(x.K));
        x.dk = (is.nk == 9) ? 3 : 2;
        x.eps = is.eps;
        x.threshold = is.threshold;
        x.power = is.power;
    }
    memset(&mt, 0, sizeof(mt));
    mt.nin = nf;
    nextra = 0;
    for (int e = 0; e < nf; ++e) {
        UpdTable &u = eqs[e].upd;
        u.nimp = maxp[e];
        eqs[e].first = mt.ngrp;
        for (int b = 0; b < u.ngrp; ++b) {
            if (mt.ngrp >= GOPF_MAX_XOUT)
                return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "too many term groups over all equations");
            const int j = mt.ngrp++;
            mt.nmono[j] = (int)gm[e][b].size();
            for (int m = 0; m < mt.nmono[j]; ++m) {
                mt.coef[j][m] = gm[e][b][m].coef;
                memcpy(mt.pw[j][m], gm[e][b][m].pw, GOPF_MAX_FIELDS);
            }
            // the first group goes into T of the field, except where the elastic step still
            // reads that T after the x-pass
            eqs[e].ubuf[b] = (b == 0 && !(kfield && have_el && e == ctx->el_field)) ? -1 : nextra++;
        }
    }
    if (noise_eq >= 0) { // the draw's parameters, as in a single-field model; the counter is set at compile
        NoiseParams &nz = eqs[noise_eq].upd.noise;
        nz.ndim = ctx->ndim;
        nz.amp = sqrt((double)ctx->g.N * 2.0 * noise_strength);
        nz.seed_lo = (uint32_t)(noise_seed & 0xffffffffu);
        nz.seed_hi = (uint32_t)(noise_seed >> 32);
    }
    if (kfield) {
        ctx->noise_eq = noise_eq;
        ctx->has_elastic = have_el;
        ctx->has_volcons = have_vc;
        ctx->vc_group = have_vc ? eqs[ctx->vc_eq].first + ctx->vc_local : -1;
        ctx->mono_H = -1;
        if (have_el) { // H(c) = 3c^2 - 2c^3 of the elastic field, an output of its own (pf/homoLinElast.go:10-12)
            if (mt.ngrp >= GOPF_MAX_XOUT)
                return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "too many term groups over all equations");
            const int j = mt.ngrp++;
            mt.nmono[j] = 2;
            mt.coef[j][0] = 3.0;
            mt.pw[j][0][ctx->el_field] = 2;
            mt.coef[j][1] = -2.0;
            mt.pw[j][1][ctx->el_field] = 3;
            ctx->mono_H = j;
        }
    }
    return GOPF_OK;
}

static int compile_multi(gopf_ctx *ctx)
{
    const int nf = ctx->nfields;
    if (nf > GOPF_MAX_FIELDS)
        return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "at most " + std::to_string(GOPF_MAX_FIELDS) + " fields per model");
    std::vector<gopf_ctx::EqPlan> eqs, eqs_rk;
    MonoTable mt, mt_rk;
    int nx = 0, nx_rk = 0, rc;
    if ((rc = build_multi_plan(ctx, true, eqs, mt, nx))) return rc;
    if ((rc = build_multi_plan(ctx, false, eqs_rk, mt_rk, nx_rk))) return rc;
    const int nextra = std::max(nx, nx_rk);
    // x-pass tile width: nf + 1 tiles of KX x LB elements in shared memory
    const int vb = (ctx->prec == GOPF_FP32) ? 8 : 16;
    auto smem_of = [&](int lbx) { return (long long)(nf + 1) * ctx->g.KX * lbx * vb; };
    int lb = ctx->LBx;
    while (lb > 4 && smem_of(lb) > 200 * 1024) lb /= 2;
    if (smem_of(lb) > 200 * 1024)
        return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "too many fields for this column count (shared memory)");
    if (ctx->device >= 0) {
        for (int f = 1; f < nf; ++f) {
            const bool fresh = !ctx->d_fstate[f];
            if ((rc = alloc_spectral(ctx, &ctx->d_fstate[f]))) return rc;
            if ((rc = alloc_spectral(ctx, &ctx->d_fT[f]))) return rc;
            if (fresh) { // fields start at zero, like pf.NewField(name, n, nil)
                const size_t vbytes = (size_t)vb * ctx->g.C;
                CK(cudaMemset(ctx->d_fstate[f], 0, vbytes));
                CK(cudaMemset(ctx->d_fT[f], 0, vbytes));
            }
        }
        for (int i = 0; i < nextra; ++i)
            if ((rc = alloc_spectral(ctx, &ctx->d_mU[i]))) return rc;
    }
    ctx->multi = true;
    ctx->eqs = eqs;
    ctx->mono = mt;
    ctx->eqs_rk = eqs_rk;
    ctx->mono_rk = mt_rk;
    ctx->LBm = lb;
    memset(&ctx->pw, 0, sizeof(ctx->pw));
    // ctx->upd only carries the modal filter (gopf_set_modal_filter); each equation's table is in eqs
    UpdTable u0;
    memset(&u0, 0, sizeof(u0));
    u0.filt = ctx->upd.nfilt ? ctx->d_filter : nullptr;
    u0.nfilt = ctx->upd.nfilt;
    ctx->upd = u0;
    ctx->ngroups = mt.ngrp;
    memset(&ctx->noise, 0, sizeof(ctx->noise));
    if (ctx->noise_eq >= 0) {
        // the step counter keying the draws advances with field 0's Hermitian projection, once per step
        if (ctx->device >= 0) {
            if (!ctx->d_stepctr) {
                CK(gopf_malloc(&ctx->d_stepctr, sizeof(unsigned long long)));
                ctx->dev_bytes += sizeof(unsigned long long);
            }
            CK(cudaMemset(ctx->d_stepctr, 0, sizeof(unsigned long long)));
        }
        for (auto *plan : {&ctx->eqs, &ctx->eqs_rk})
            (*plan)[ctx->noise_eq].upd.noise.step = ctx->d_stepctr;
        ctx->noise = ctx->eqs[ctx->noise_eq].upd.noise;
    }
    if (ctx->device >= 0 && ctx->has_elastic) {
        if ((rc = alloc_spectral(ctx, &ctx->d_UH))) return rc;
        if ((rc = set_device(ctx))) return rc;
        if ((rc = gopf_elastic_table(ctx))) return rc;
    }
    if (ctx->device >= 0 && ctx->has_volcons) {
        if ((rc = alloc_volcons(ctx, true))) return rc;
        ctx->eqs[ctx->vc_eq].upd.gscale[ctx->vc_local] = ctx->d_vc + 4;
    }
    ctx->el_primed = false;
    ctx->initialised = true;
    invalidate_graphs(ctx);
    return GOPF_OK;
}

int gopf_compile_model(gopf_ctx *ctx)
{
    if (ctx->nfields < 1) return gopf_fail(ctx, GOPF_ERR_ARG, "the model has no fields");
    if (ctx->nfields > 1) return compile_multi(ctx);
    ctx->multi = false;
    ctx->noise_eq = -1;
    PwTable pw;
    memset(&pw, 0, sizeof(pw));
    UpdTable u;
    memset(&u, 0, sizeof(u));
    NoiseParams noise;
    memset(&noise, 0, sizeof(noise));
    double noise_strength = 0.0;
    unsigned long long noise_seed = 0;
    int maxp = 0;
    for (const gopf_term &t : ctx->terms) {
        if (t.eq != 0) return gopf_fail(ctx, GOPF_ERR_ARG, "term refers to an equation that does not exist");
        if (t.lap < 0 || t.lap >= GOPF_MAX_IMP) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "LAP power out of range");
        if (t.implicit) {
            u.imp[t.lap] += t.coef;
            maxp = std::max(maxp, t.lap + 1);
            continue;
        }
        std::vector<std::pair<double, int>> poly;
        if (t.source == GOPF_SRC_FIELD) {
            if (t.src_index != 0) return gopf_fail(ctx, GOPF_ERR_ARG, "bad field index");
            poly = {{1.0, 1}};
        } else if (t.source == GOPF_SRC_DERIVED) {
            if (t.src_index < 0 || t.src_index >= (int)ctx->der.size())
                return gopf_fail(ctx, GOPF_ERR_ARG, "bad derived-field index");
            if (ctx->der[t.src_index].kind == GOPF_DER_WHITE_NOISE) {
                if (noise.kind) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "one noise term per model");
                noise.kind = 1;
                noise.coef = t.coef;
                noise.lap = t.lap;
                noise_strength = ctx->der[t.src_index].coef[0];
                noise_seed = noise_seed_of(ctx, t.src_index);
                continue;
            }
            int rc = derived_poly(ctx, ctx->der[t.src_index], poly);
            if (rc) return rc;
        } else {
            return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED,
                             "a term without a field (constant in k space) has no device implementation");
        }
        int grp = -1;
        for (int b = 0; b < u.ngrp; ++b)
            if (u.glap[b] == t.lap) grp = b;
        if (grp < 0) {
            if (u.ngrp >= GOPF_MAX_GROUPS) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "too many distinct LAP powers");
            grp = u.ngrp++;
            u.glap[grp] = t.lap;
        }
        int rc = add_poly_to_group(ctx, pw, grp, poly, t.coef);
        if (rc) return rc;
    }
    // user-defined terms that run on the device
    ctx->has_elastic = false;
    ctx->has_volcons = false;
    ctx->vc_group = -1;
    for (const gopf_special &sp : ctx->specials) {
        if (sp.eq != 0) return gopf_fail(ctx, GOPF_ERR_ARG, "term refers to an equation that does not exist");
        if (sp.kind == 1) {
            if (ctx->has_elastic) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "one elastic term per model");
            const gopf_modeldef::Elastic &e = ctx->def.elastic[sp.index];
            if (e.field != 0) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "elastic term must act on field 0");
            ctx->has_elastic = true;
            ctx->el_field = ctx->el_eq = 0;
            set_elastic_params(ctx, e, sp);
        } else if (sp.kind == 2) {
            if (ctx->has_volcons) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "one volume-conserving term per model");
            const gopf_modeldef::Volcons &v = ctx->def.volcons[sp.index];
            if (v.field != 0) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "volume-conserving term must act on field 0");
            const int did = find_derived(ctx, v.indicator);
            if (did < 0) return gopf_fail(ctx, GOPF_ERR_ARG, "VolumeConservingLP: Indicator is not a derived field");
            std::vector<std::pair<double, int>> poly;
            int rc = derived_poly(ctx, ctx->def.derived[did], poly);
            if (rc) return rc;
            if (u.ngrp >= GOPF_MAX_GROUPS) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "too many term groups");
            const int grp = u.ngrp++;
            u.glap[grp] = sp.lap;
            if ((rc = add_poly_to_group(ctx, pw, grp, poly, 1.0))) return rc;
            ctx->has_volcons = true;
            ctx->vc_group = grp;
            ctx->vc_dt = v.dt;
            ctx->vc_coef = sp.coef;
        } else if (sp.kind == 3) {
            const gopf_modeldef::Noise &nz = ctx->def.noise[sp.index];
            if (noise.kind) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "one noise term per model");
            noise.kind = 2;
            noise.coef = sp.coef;
            noise.lap = sp.lap;
            noise_strength = nz.strength;
            noise_seed = nz.seed;
        } else if (sp.kind == 4) {
            const gopf_modeldef::ImplicitSym &is = ctx->def.isym[sp.index];
            if (u.nxs >= GOPF_MAX_XSYM) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "too many implicit user terms");
            XSym &x = u.xs[u.nxs++];
            memset(&x, 0, sizeof(x));
            x.kind = is.kind;
            x.coef = sp.coef;
            x.lap = sp.lap;
            memcpy(x.K, is.K, sizeof(x.K));
            x.dk = (is.nk == 9) ? 3 : 2;
            x.eps = is.eps;
            x.threshold = is.threshold;
            x.power = is.power;
        } else {
            return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "user-defined term kind has no device implementation");
        }
    }
    if (noise.kind) {
        noise.ndim = ctx->ndim;
        noise.amp = sqrt((double)ctx->g.N * 2.0 * noise_strength);
        noise.seed_lo = (uint32_t)(noise_seed & 0xffffffffu);
        noise.seed_hi = (uint32_t)(noise_seed >> 32);
    }
    if (ctx->has_elastic && u.ngrp + 1 > GOPF_MAX_GROUPS)
        return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "too many term groups with the elastic term");
    pw.ngrp = u.ngrp;
    pw_densify(pw);
    u.nimp = maxp;
    if (noise.kind && ctx->device >= 0) {
        if (!ctx->d_stepctr) {
            CK(gopf_malloc(&ctx->d_stepctr, sizeof(unsigned long long)));
            ctx->dev_bytes += sizeof(unsigned long long);
        }
        CK(cudaMemset(ctx->d_stepctr, 0, sizeof(unsigned long long)));
        noise.step = ctx->d_stepctr;
    }
    u.noise = noise;
    ctx->noise = noise;
    ctx->pw = pw;
    u.filt = ctx->upd.nfilt ? ctx->d_filter : nullptr; // a filter set earlier survives a re-init
    u.nfilt = ctx->upd.nfilt;
    ctx->upd = u;
    ctx->ngroups = u.ngrp;
    // the elastic step's x-pass also emits H(c) = 3c^2 - 2c^3 as an extra group
    ctx->pw_el = pw;
    if (ctx->has_elastic) {
        const int gH = pw.ngrp;
        ctx->pw_el.ngrp = gH + 1;
        ctx->pw_el.nterm[gH] = 2;
        ctx->pw_el.pw[gH][0] = 2;
        ctx->pw_el.coef[gH][0] = 3.0;
        ctx->pw_el.pw[gH][1] = 3;
        ctx->pw_el.coef[gH][1] = -2.0;
        pw_densify(ctx->pw_el);
    }
    if (ctx->device >= 0) {
        int rc;
        for (int b = 1; b < std::max(1, u.ngrp); ++b)
            if ((rc = alloc_spectral(ctx, &ctx->d_U[b]))) return rc;
        if (ctx->has_elastic) {
            if ((rc = alloc_spectral(ctx, &ctx->d_U0))) return rc;
            if ((rc = alloc_spectral(ctx, &ctx->d_UH))) return rc;
            if ((rc = set_device(ctx))) return rc;
            if ((rc = gopf_elastic_table(ctx))) return rc;
        }
        if (ctx->has_volcons) {
            if ((rc = alloc_volcons(ctx, false))) return rc;
            ctx->upd.gscale[ctx->vc_group] = ctx->d_vc + 4;
        }
    }
    ctx->el_primed = false;
    ctx->initialised = true;
    invalidate_graphs(ctx);
    return GOPF_OK;
}

extern "C" int gopf_set_terms(gopf_ctx *ctx, int nfields, const gopf_derived *derived, int nderived,
                              const gopf_term *terms, int nterms)
{
    if (!ctx || nfields < 1 || nderived < 0 || nterms < 0 || (nderived && !derived) || (nterms && !terms))
        return gopf_fail(ctx, GOPF_ERR_ARG, "bad term table");
    int rc;
    if (ctx->device >= 0 && (rc = set_device(ctx))) return rc;
    ctx->nfields = nfields;
    ctx->der.assign(derived, derived + nderived);
    ctx->terms.assign(terms, terms + nterms);
    ctx->specials.clear();
    return gopf_compile_model(ctx);
}

extern "C" int gopf_get_terms(gopf_ctx *ctx, gopf_term *terms, int capacity, int *nterms)
{
    if (!ctx || !nterms) return GOPF_ERR_ARG;
    *nterms = (int)ctx->terms.size();
    for (int i = 0; i < *nterms && i < capacity; ++i) terms[i] = ctx->terms[i];
    return GOPF_OK;
}

extern "C" int gopf_get_derived(gopf_ctx *ctx, gopf_derived *der, int capacity, int *nder)
{
    if (!ctx || !nder) return GOPF_ERR_ARG;
    *nder = (int)ctx->der.size();
    for (int i = 0; i < *nder && i < capacity; ++i) der[i] = ctx->der[i];
    return GOPF_OK;
}

extern "C" int gopf_equation_summary(gopf_ctx *ctx, int eq, int *ne, int *ni)
{
    if (!ctx || !ne || !ni) return GOPF_ERR_ARG;
    *ne = *ni = 0;
    for (const gopf_term &t : ctx->terms)
        if (t.eq == eq) (t.implicit ? *ni : *ne) += 1;
    for (const gopf_special &s : ctx->specials)
        if (s.eq == eq) (s.kind == 4 ? *ni : *ne) += 1; // kind 4: implicit user terms (RHS.Denum)
    return GOPF_OK;
}

extern "C" int gopf_set_stepper(gopf_ctx *ctx, int stepper, double dt)
{
    if (!ctx) return GOPF_ERR_ARG;
    if (stepper != GOPF_STEPPER_EULER && stepper != GOPF_STEPPER_RK4 && stepper != GOPF_STEPPER_IMPLICIT_EULER &&
        stepper != GOPF_STEPPER_SDD)
        return gopf_fail(ctx, GOPF_ERR_ARG, "unknown stepper");
    if (!(dt > 0.0) || !std::isfinite(dt)) return gopf_fail(ctx, GOPF_ERR_ARG, "dt must be positive");
    ctx->stepper = stepper;
    ctx->dt = dt;
    invalidate_graphs(ctx);
    return GOPF_OK;
}

// ------------------------------------------------------------------
// pass helpers
// ------------------------------------------------------------------

template <typename R> static XPassArgs<R> xargs(gopf_ctx *ctx)
{
    typedef typename VecOf<R>::type V;
    XPassArgs<R> a;
    memset(&a, 0, sizeof(a));
    a.g = ctx->g;
    a.planH = ctx->planH;
    a.twX = (const V *)ctx->d_twX;
    a.allow_fast = ctx->use_fast ? ((ctx->use_tma ? 3 : 1) | (ctx->x_rows == 16 ? 8 : 0) | (ctx->z_lines == 8 ? 16 : 0))
                                 : 0;
    a.status = ctx->d_status;
    return a;
}

template <typename R> static PassArgs<R> pargs(gopf_ctx *ctx, bool zaxis)
{
    typedef typename VecOf<R>::type V;
    PassArgs<R> a;
    memset(&a, 0, sizeof(a));
    a.g = ctx->g;
    a.plan = zaxis ? ctx->planZ : ctx->planY;
    a.tw = (const V *)(zaxis ? ctx->d_twZ : ctx->d_twY);
    a.allow_fast = ctx->use_fast ? ((ctx->use_tma ? 3 : 1) | (ctx->x_rows == 16 ? 8 : 0) | (ctx->z_lines == 8 ? 16 : 0))
                                 : 0;
    a.status = ctx->d_status;
    return a;
}

static void prof_mark(gopf_ctx *ctx)
{
    if (ctx->prof_events && ctx->prof_next < ctx->prof_events->size())
        cudaEventRecord((*ctx->prof_events)[ctx->prof_next++], ctx->stream);
}

#define LK(call)                                                                                                       \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess) return e_;                                                                              \
        prof_mark(ctx);                                                                                                \
    } while (0)

// From T (after the inverse y/z passes) produce real rows and/or reductions.
template <typename R> static XPassArgs<R> xargs_out(gopf_ctx *ctx, R *rout, double *red, int f = 0)
{
    XPassArgs<R> xa = xargs<R>(ctx);
    xa.in_mode = XIN_SPECTRAL;
    xa.in = (const typename VecOf<R>::type *)field_T(ctx, f);
    xa.rout = rout;
    xa.red = red;
    xa.ngrp_out = 0;
    return xa;
}

template <typename R> static cudaError_t enqueue_xpass_out(gopf_ctx *ctx, R *rout, double *red, int f = 0)
{
    return launch_xpass<R>(xargs_out<R>(ctx, rout, red, f), ctx->LBx, ctx->stream);
}

// Load real field d_real into the state of field f: c-hat = FFT(c), T = partial inverse of c-hat/N.
template <typename R> static cudaError_t enqueue_load_state(gopf_ctx *ctx, int f = 0)
{
    typedef typename VecOf<R>::type V;
    V *T = (V *)field_T(ctx, f);
    V *state = (V *)field_state(ctx, f);
    XPassArgs<R> xa = xargs<R>(ctx);
    xa.in_mode = XIN_REAL;
    xa.rin = (const R *)ctx->d_real;
    xa.out[0] = T;
    xa.ngrp_out = 1;
    xa.identity = 1;
    LK(launch_xpass<R>(xa, ctx->LBx, ctx->stream));
    UpdTable u;
    memset(&u, 0, sizeof(u));
    u.invN = 1.0 / (double)ctx->g.N;
    if (ctx->g.Z > 1) {
        PassArgs<R> pa = pargs<R>(ctx, false);
        pa.mode = PM_FWD;
        pa.buf[0] = T;
        pa.nbuf = 1;
        LK(launch_cpass<R>(pa, ctx->LBy, ctx->stream));
        PassArgs<R> sa = pargs<R>(ctx, true);
        sa.mode = PM_INIT;
        sa.buf[0] = T;
        sa.nbuf = 1;
        sa.state = state;
        sa.tout = T;
        sa.upd = u;
        LK(launch_spass<R>(sa, ctx->LBz, ctx->stream));
        LK(gopf_launch_hermitian_planes(ctx, state));
        pa.mode = PM_INV;
        LK(launch_cpass<R>(pa, ctx->LBy, ctx->stream));
    } else {
        PassArgs<R> pa = pargs<R>(ctx, false);
        pa.mode = PM_INIT;
        pa.buf[0] = T;
        pa.nbuf = 1;
        pa.state = state;
        pa.tout = T;
        pa.upd = u;
        LK(launch_cpass<R>(pa, ctx->LBy, ctx->stream));
        LK(gopf_launch_hermitian_planes(ctx, state));
    }
    return cudaSuccess;
}

// One Euler step (pf/euler.go:16-47) of a single-field model.
//   x-pass      : c2r(T) -> polynomial groups g_b(c) (+ H(c) for elasticity) -> r2c
//   [volcons]   : Lagrange-multiplier update from the x-pass's FP64 block sums
//   [elastic]   : H-hat -> b(k) H-hat / N -> w(x); x-pass q = s H'(c)(w - 2 e0 H(c)) -> r2c
//   last axis   : forward, c-hat <- (c-hat + dt sum_b m^lap_b U_b)/(1 - dt L(m)), T <- inverse(c-hat/N)
// The elastic part runs from the second step on: the reference's h-field is
// zero until the first OnStepFinished (pf/homoLinElast.go:130-145).
// The point sources of equation eq into its update table (pointers of the current amplitude table).
static void apply_sources(const gopf_ctx *ctx, UpdTable &u, int eq)
{
    u.nsrc = 0;
    for (size_t k = 0; k < ctx->sources.size(); ++k) {
        const gopf_ctx::SourceDef &sd = ctx->sources[k];
        if (sd.eq != eq || u.nsrc >= GOPF_MAX_SRC) continue;
        for (int d = 0; d < 3; ++d) u.src_pos[u.nsrc][d] = sd.pos[d];
        u.src_row[u.nsrc] = (int)k;
        ++u.nsrc;
    }
    u.src_amp = ctx->d_srcamp;
    u.src_stride = (int)ctx->src_len;
    u.src_ctr = ctx->d_srcctr;
}

// the sources' step counter advances once per step (after every launch of the step)
__global__ void k_src_tick(unsigned long long *ctr) { *ctr += 1ull; }

template <typename R> static cudaError_t enqueue_euler(gopf_ctx *ctx)
{
    typedef typename VecOf<R>::type V;
    const bool el = ctx->has_elastic && ctx->el_primed;
    const int G = ctx->ngroups;
    const int GE = G + (el ? 1 : 0); // groups entering the update
    V *T = (V *)ctx->d_T;
    V *UH = (V *)ctx->d_UH;
    V *U[GOPF_MAX_GROUPS];
    U[0] = el ? (V *)ctx->d_U0 : T;
    for (int b = 1; b < GOPF_MAX_GROUPS; ++b) U[b] = (V *)ctx->d_U[b];
    if (el) U[G] = UH;
    UpdTable u = ctx->upd;
    u.dt = ctx->dt;
    u.invN = 1.0 / (double)ctx->g.N;
    apply_sources(ctx, u, 0);
    if (el) {
        u.ngrp = GE;
        u.glap[G] = ctx->el_lap;
        u.gscale[G] = nullptr;
    }
    const bool is3d = ctx->g.Z > 1;
    // the plain step's forward y, fused z and inverse y launches as programmatic dependents of the
    // kernel before them (not under per-kernel profiling, which records events between kernels; the
    // elastic step's chain measured 0.2-1 % slower so and keeps plain stream order)
    const int pdl = (ctx->use_pdl && !ctx->prof_events) ? ALLOW_PDL : 0;
    if (GE > 0) {
        XPassArgs<R> xa = xargs<R>(ctx);
        xa.in_mode = XIN_SPECTRAL;
        xa.in = T;
        for (int b = 0; b < GE; ++b) xa.out[b] = U[b];
        xa.ngrp_out = GE;
        xa.pw = el ? ctx->pw_el : ctx->pw;
        if (ctx->has_volcons) {
            xa.red = ctx->d_red;
            xa.red2 = ctx->d_red2;
            xa.redgrp = ctx->vc_group;
        }
        LK(launch_xpass<R>(xa, ctx->LBx, ctx->stream));
    }
    if (ctx->has_volcons) LK(gopf_launch_volcons_finalize(ctx, ctx->d_red, ctx->nred_blocks));
    if (el) {
        if (is3d) {
            PassArgs<R> pa = pargs<R>(ctx, false);
            pa.mode = PM_FWD;
            for (int b = 0; b < GE; ++b) pa.buf[b] = U[b];
            pa.nbuf = GE;
            LK(launch_cpass<R>(pa, ctx->LBy, ctx->stream));
        }
        PassArgs<R> ka = pargs<R>(ctx, is3d);
        ka.mode = PM_ELASTIC_K;
        ka.buf[0] = UH;
        ka.nbuf = 1;
        ka.upd = u;
        ka.bsym = (const R *)ctx->d_bsym;
        LK(is3d ? launch_spass<R>(ka, ctx->LBz, ctx->stream) : launch_cpass<R>(ka, ctx->LBy, ctx->stream));
        if (is3d) {
            PassArgs<R> ia = pargs<R>(ctx, false);
            ia.mode = PM_INV;
            ia.buf[0] = UH;
            ia.nbuf = 1;
            LK(launch_cpass<R>(ia, ctx->LBy, ctx->stream));
        }
        XPassArgs<R> xc = xargs<R>(ctx);
        xc.in_mode = XIN_SPECTRAL;
        xc.in = T;
        xc.program = XP_ELASTIC_Q;
        xc.in2 = UH;
        xc.out[0] = UH;
        xc.ngrp_out = 1;
        xc.e0 = ctx->el_e0;
        xc.escale = ctx->el_coef;
        LK(launch_xpass<R>(xc, ctx->LBx, ctx->stream));
        if (is3d) {
            PassArgs<R> pa = pargs<R>(ctx, false);
            pa.mode = PM_FWD;
            pa.buf[0] = UH;
            pa.nbuf = 1;
            LK(launch_cpass<R>(pa, ctx->LBy, ctx->stream));
        }
    } else if (is3d && GE > 0) {
        PassArgs<R> pa = pargs<R>(ctx, false);
        pa.mode = PM_FWD;
        for (int b = 0; b < GE; ++b) pa.buf[b] = U[b];
        pa.nbuf = GE;
        pa.allow_fast |= pdl;
        LK(launch_cpass<R>(pa, ctx->LBy, ctx->stream));
    }
    // with no explicit term the last pass reads c-hat only (identity contribution when ngrp == 0)
    const int nb = std::max(GE, 1);
    PassArgs<R> fa = pargs<R>(ctx, is3d);
    if (is3d && !el && GE > 0) fa.allow_fast |= pdl; // after the forward y pass
    fa.mode = PM_FUSED;
    for (int b = 0; b < nb; ++b) fa.buf[b] = U[b];
    fa.nbuf = nb;
    fa.state = (V *)ctx->d_state;
    fa.tout = T;
    fa.upd = u;
    LK(is3d ? launch_spass<R>(fa, ctx->LBz, ctx->stream) : launch_cpass<R>(fa, ctx->LBy, ctx->stream));
    // The projection touches only c-hat, the inverse y pass only T: outside per-kernel profiling
    // they run as two branches (a fork/join that a captured graph keeps).
    const bool fork = is3d && !ctx->prof_events;
    if (fork) {
        LK(cudaEventRecord(ctx->ev_fork, ctx->stream));
        LK(cudaStreamWaitEvent(ctx->side_stream, ctx->ev_fork, 0));
        LK(gopf_launch_hermitian_planes(ctx, ctx->d_state, ctx->side_stream));
        LK(cudaEventRecord(ctx->ev_join, ctx->side_stream));
    } else {
        LK(gopf_launch_hermitian_planes(ctx, ctx->d_state));
    }
    if (is3d) {
        PassArgs<R> ia = pargs<R>(ctx, false);
        ia.mode = PM_INV;
        ia.buf[0] = T;
        ia.nbuf = 1;
        if (!el) ia.allow_fast |= pdl;
        LK(launch_cpass<R>(ia, ctx->LBy, ctx->stream));
    }
    if (fork) LK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
    return cudaSuccess;
}

// One RK4 step (pf/rk4.go:29-127): four explicit-RHS evaluations, each an
// x-pass + forward y + a fused last-axis pass that accumulates
// F = c + dt(k1 + 2k2 + 2k3 + k4)/6 and forms the next stage's input
// (c + a k)/(1 - a L); the last stage sets c = F/(1 - dt L).
template <typename R> static cudaError_t enqueue_rk4(gopf_ctx *ctx)
{
    typedef typename VecOf<R>::type V;
    const int G = ctx->ngroups;
    V *T = (V *)ctx->d_T;
    V *U[GOPF_MAX_GROUPS];
    U[0] = T;
    for (int b = 1; b < GOPF_MAX_GROUPS; ++b) U[b] = (V *)ctx->d_U[b];
    const bool is3d = ctx->g.Z > 1;
    const double dt = ctx->dt;
    const double afin[4] = {dt / 6.0, dt / 3.0, dt / 3.0, dt / 6.0};
    const double ay[3] = {0.5 * dt, 0.5 * dt, dt};
    for (int stage = 1; stage <= 4; ++stage) {
        if (G > 0) {
            XPassArgs<R> xa = xargs<R>(ctx);
            xa.in_mode = XIN_SPECTRAL;
            xa.in = T;
            for (int b = 0; b < G; ++b) xa.out[b] = U[b];
            xa.ngrp_out = G;
            xa.pw = ctx->pw;
            LK(launch_xpass<R>(xa, ctx->LBx, ctx->stream));
            if (is3d) {
                PassArgs<R> pa = pargs<R>(ctx, false);
                pa.mode = PM_FWD;
                for (int b = 0; b < G; ++b) pa.buf[b] = U[b];
                pa.nbuf = G;
                LK(launch_cpass<R>(pa, ctx->LBy, ctx->stream));
            }
        }
        UpdTable u = ctx->upd;
        u.dt = dt;
        u.invN = 1.0 / (double)ctx->g.N;
        apply_sources(ctx, u, 0); // RK4 evaluates every stage at the step's start time (pf/rk4.go:101-127)
        u.rk_stage = stage;
        u.rk_afin = afin[stage - 1];
        u.rk_ay = (stage < 4) ? ay[stage - 1] : 0.0;
        u.rk_fden = (stage < 4) ? ay[stage - 1] : dt;
        const int nb = std::max(G, 1);
        PassArgs<R> fa = pargs<R>(ctx, is3d);
        fa.mode = PM_FUSED;
        for (int b = 0; b < nb; ++b) fa.buf[b] = U[b];
        fa.nbuf = nb;
        fa.state = (V *)ctx->d_state;
        fa.tout = T;
        fa.upd = u;
        fa.rkF = (V *)ctx->d_rkF;
        LK(is3d ? launch_spass<R>(fa, ctx->LBz, ctx->stream) : launch_cpass<R>(fa, ctx->LBy, ctx->stream));
        if (stage == 4) LK(gopf_launch_hermitian_planes(ctx, ctx->d_state));
        if (is3d) {
            PassArgs<R> ia = pargs<R>(ctx, false);
            ia.mode = PM_INV;
            ia.buf[0] = T;
            ia.nbuf = 1;
            LK(launch_cpass<R>(ia, ctx->LBy, ctx->stream));
        }
    }
    return cudaSuccess;
}

// One Euler (rk_stage 0) step or one RK4 stage of a multi-field model (pf/euler.go:16-47 and
// pf/rk4.go:29-127 loop over m.Fields; every field's RHS sees every field at the stage's start):
//   x-pass   : c2r of T of every field -> monomial groups of every equation -> r2c
//   per eq.  : [3D] forward y of its groups; fused last-axis update of its c-hat, T <- inverse
//   per field: Hermitian projection; [3D] inverse y of all T in one launch
template <typename R> static cudaError_t enqueue_multi_stage(gopf_ctx *ctx, int stage)
{
    typedef typename VecOf<R>::type V;
    const int nf = ctx->nfields;
    const bool is3d = ctx->g.Z > 1;
    const double dt = ctx->dt;
    const std::vector<gopf_ctx::EqPlan> &eqs = (stage > 0) ? ctx->eqs_rk : ctx->eqs;
    const MonoTable &mono = (stage > 0) ? ctx->mono_rk : ctx->mono;
    auto gbuf = [&](int e, int b) -> V * {
        const int k = eqs[e].ubuf[b];
        return (V *)(k < 0 ? field_T(ctx, e) : ctx->d_mU[k]);
    };
    // the elastic term (pf/homoLinElast.go:47-98) from the second step on: H(c) of its field is
    // the last x-pass output; before that the term sees the reference's zero field and is left out
    const bool euler = (stage == 0);
    const bool el = euler && ctx->has_elastic && ctx->el_primed;
    const bool vc = euler && ctx->has_volcons;
    V *UH = (V *)ctx->d_UH;
    MonoTable xm = mono;
    if (euler && ctx->has_elastic && !el) xm.ngrp = ctx->mono_H; // H(c) is the last output
    if (xm.ngrp > 0) {
        XPassArgs<R> xa = xargs<R>(ctx);
        xa.in_mode = XIN_SPECTRAL;
        xa.program = XP_MULTI;
        xa.allow_fast = 0;
        for (int f = 0; f < nf; ++f) xa.inF[f] = (const V *)field_T(ctx, f);
        for (int e = 0; e < nf; ++e)
            for (int b = 0; b < eqs[e].upd.ngrp; ++b) xa.out[eqs[e].first + b] = gbuf(e, b);
        if (el) xa.out[ctx->mono_H] = UH;
        xa.ngrp_out = xm.ngrp;
        xa.mono = xm;
        if (vc) { // block sums of the field and of the indicator group (pf/volumeConserving.go:30-50)
            xa.red = ctx->d_vcred;
            xa.redfield = ctx->vc_field;
            xa.red2 = ctx->d_red2;
            xa.redgrp = ctx->vc_group;
        }
        LK(launch_xpass<R>(xa, ctx->LBm, ctx->stream));
    }
    if (vc) LK(gopf_launch_volcons_finalize(ctx, ctx->d_vcred, ((ctx->g.Y + ctx->LBm - 1) / ctx->LBm) * ctx->g.Z));
    if (el) {
        // H-hat -> w = b(k) H-hat / N in real space -> q = s H'(c) (w - 2 e0 H(c)) -> q-hat, as the
        // single-field step does, with c the elastic field's T from before this step's updates
        PassArgs<R> pa = pargs<R>(ctx, false);
        pa.buf[0] = UH;
        pa.nbuf = 1;
        if (is3d) {
            pa.mode = PM_FWD;
            LK(launch_cpass<R>(pa, ctx->LBy, ctx->stream));
        }
        PassArgs<R> ka = pargs<R>(ctx, is3d);
        ka.mode = PM_ELASTIC_K;
        ka.buf[0] = UH;
        ka.nbuf = 1;
        ka.upd.invN = 1.0 / (double)ctx->g.N;
        ka.bsym = (const R *)ctx->d_bsym;
        LK(is3d ? launch_spass<R>(ka, ctx->LBz, ctx->stream) : launch_cpass<R>(ka, ctx->LBy, ctx->stream));
        if (is3d) {
            pa.mode = PM_INV;
            LK(launch_cpass<R>(pa, ctx->LBy, ctx->stream));
        }
        XPassArgs<R> xc = xargs<R>(ctx);
        xc.in_mode = XIN_SPECTRAL;
        xc.in = (const V *)field_T(ctx, ctx->el_field);
        xc.program = XP_ELASTIC_Q;
        xc.in2 = UH;
        xc.out[0] = UH;
        xc.ngrp_out = 1;
        xc.e0 = ctx->el_e0;
        xc.escale = ctx->el_coef;
        LK(launch_xpass<R>(xc, ctx->LBx, ctx->stream));
        if (is3d) {
            pa.mode = PM_FWD;
            LK(launch_cpass<R>(pa, ctx->LBy, ctx->stream));
        }
    }
    for (int e = 0; e < nf; ++e) {
        const gopf_ctx::EqPlan &ep = eqs[e];
        const int G = ep.upd.ngrp;
        if (is3d && G > 0) {
            PassArgs<R> pa = pargs<R>(ctx, false);
            pa.mode = PM_FWD;
            for (int b = 0; b < G; ++b) pa.buf[b] = gbuf(e, b);
            pa.nbuf = G;
            LK(launch_cpass<R>(pa, ctx->LBy, ctx->stream));
        }
        UpdTable u = ep.upd;
        u.dt = dt;
        u.invN = 1.0 / (double)ctx->g.N;
        u.filt = ctx->upd.filt;
        u.nfilt = ctx->upd.nfilt;
        apply_sources(ctx, u, e);
        for (int q = 0; q < u.nxf; ++q) u.xf_src[q] = field_state(ctx, ep.xf_field[q]);
        if (stage > 0) {
            const double afin[4] = {dt / 6.0, dt / 3.0, dt / 3.0, dt / 6.0};
            const double ay[3] = {0.5 * dt, 0.5 * dt, dt};
            u.rk_stage = stage;
            u.rk_afin = afin[stage - 1];
            u.rk_ay = (stage < 4) ? ay[stage - 1] : 0.0;
            u.rk_fden = (stage < 4) ? ay[stage - 1] : dt;
        }
        const bool el_here = el && e == ctx->el_eq;
        if (el_here) { // the elastic term as one more group, already forward transformed
            u.ngrp = G + 1;
            u.glap[G] = ctx->el_lap;
            u.gscale[G] = nullptr;
        }
        const int GE = G + (el_here ? 1 : 0);
        const int nb = std::max(GE, 1);
        PassArgs<R> fa = pargs<R>(ctx, is3d);
        fa.mode = PM_FUSED;
        for (int b = 0; b < G; ++b) fa.buf[b] = gbuf(e, b);
        if (el_here) fa.buf[G] = UH;
        if (GE == 0) fa.buf[0] = gbuf(e, 0);
        fa.nbuf = nb;
        fa.state = (V *)field_state(ctx, e);
        fa.tout = (V *)field_T(ctx, e);
        fa.upd = u;
        fa.rkF = (V *)field_rkF(ctx, e);
        LK(is3d ? launch_spass<R>(fa, ctx->LBz, ctx->stream) : launch_cpass<R>(fa, ctx->LBy, ctx->stream));
    }
    if (stage == 0 || stage == 4)
        for (int f = 0; f < nf; ++f) LK(gopf_launch_hermitian_planes(ctx, field_state(ctx, f)));
    if (is3d) {
        PassArgs<R> ia = pargs<R>(ctx, false);
        ia.mode = PM_INV;
        for (int f = 0; f < nf; ++f) ia.buf[f] = (V *)field_T(ctx, f);
        ia.nbuf = nf;
        LK(launch_cpass<R>(ia, ctx->LBy, ctx->stream));
    }
    return cudaSuccess;
}

template <typename R> static cudaError_t enqueue_steps(gopf_ctx *ctx, int n)
{
    for (int i = 0; i < n; ++i) {
        if (ctx->multi) {
            if (ctx->stepper == GOPF_STEPPER_RK4)
                for (int s = 1; s <= 4; ++s) LK(enqueue_multi_stage<R>(ctx, s));
            else
                LK(enqueue_multi_stage<R>(ctx, 0));
        } else {
            LK(ctx->stepper == GOPF_STEPPER_RK4 ? enqueue_rk4<R>(ctx) : enqueue_euler<R>(ctx));
        }
        if (!ctx->sources.empty()) {
            k_src_tick<<<1, 1, 0, ctx->stream>>>(ctx->d_srcctr);
            LK(cudaGetLastError());
        }
    }
    return cudaSuccess;
}

extern "C" int gopf_add_source(gopf_ctx *ctx, int eq, const double *pos, int npos, int *source_id)
{
    if (!ctx || !pos || npos != ctx->ndim) return gopf_fail(ctx, GOPF_ERR_ARG, "a source needs one coordinate per dimension");
    const int neq = std::max(ctx->nfields, (int)ctx->def.equations.size());
    if (eq < 0 || (neq > 0 && eq >= neq)) return gopf_fail(ctx, GOPF_ERR_ARG, "bad equation index");
    int per_eq = 0;
    for (const gopf_ctx::SourceDef &sd : ctx->sources) per_eq += (sd.eq == eq);
    if (per_eq >= GOPF_MAX_SRC)
        return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "at most " + std::to_string(GOPF_MAX_SRC) + " sources per equation");
    gopf_ctx::SourceDef sd;
    sd.eq = eq;
    for (int d = 0; d < 3; ++d) sd.pos[d] = (d < npos) ? pos[d] : 0.0;
    ctx->sources.push_back(sd);
    if (source_id) *source_id = (int)ctx->sources.size() - 1;
    ctx->src_len = 0; // amplitudes must be given again for every source
    invalidate_graphs(ctx);
    return GOPF_OK;
}

extern "C" int gopf_set_source_amplitudes(gopf_ctx *ctx, const double *amps, int nsources, int nsteps)
{
    if (!ctx || !amps || nsteps < 1) return gopf_fail(ctx, GOPF_ERR_ARG, "null table or no steps");
    if (nsources != (int)ctx->sources.size())
        return gopf_fail(ctx, GOPF_ERR_ARG, "one row of amplitudes per source, in gopf_add_source order");
    int rc;
    if ((rc = set_device(ctx))) return rc;
    const size_t need = (size_t)nsources * (size_t)nsteps;
    if (need > ctx->srcamp_cap || !ctx->d_srcctr) {
        if (ctx->d_srcamp) cudaFree(ctx->d_srcamp);
        ctx->d_srcamp = nullptr;
        CK(gopf_malloc(&ctx->d_srcamp, sizeof(double) * need));
        ctx->srcamp_cap = need;
        if (!ctx->d_srcctr) CK(gopf_malloc(&ctx->d_srcctr, sizeof(unsigned long long)));
    }
    CK(cudaStreamSynchronize(ctx->stream)); // steps in flight may still read the old table
    CK(cudaMemcpy(ctx->d_srcamp, amps, sizeof(double) * need, cudaMemcpyHostToDevice));
    CK(cudaMemset(ctx->d_srcctr, 0, sizeof(unsigned long long)));
    ctx->src_base = ctx->step;
    ctx->src_len = nsteps;
    invalidate_graphs(ctx); // the table's stride is part of the captured launches
    return GOPF_OK;
}

static cudaError_t enqueue_steps_any(gopf_ctx *ctx, int n)
{
    return (ctx->prec == GOPF_FP32) ? enqueue_steps<float>(ctx, n) : enqueue_steps<double>(ctx, n);
}

static int capture_graph(gopf_ctx *ctx, int nsteps, cudaGraphExec_t *exec)
{
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue_steps_any(ctx, nsteps);
    cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &graph);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "capture");
    if (e2 != cudaSuccess) return cuda_fail(ctx, e2, "cudaStreamEndCapture");
    // count the kernel nodes: the number of launches one replay makes
    size_t nn = 0, nk = 0;
    if (cudaGraphGetNodes(graph, nullptr, &nn) == cudaSuccess && nn > 0) {
        std::vector<cudaGraphNode_t> nodes(nn);
        if (cudaGraphGetNodes(graph, nodes.data(), &nn) == cudaSuccess)
            for (size_t i = 0; i < nn; ++i) {
                cudaGraphNodeType t;
                if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++nk;
            }
    }
    (nsteps == 1 ? ctx->graph_kernels1 : ctx->graph_kernelsK) = (long long)nk;
    e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGraphInstantiate");
    return GOPF_OK;
}

// ------------------------------------------------------------------
// field transfer
// ------------------------------------------------------------------

static int require_ready(gopf_ctx *ctx, int field)
{
    if (field < 0 || (ctx->nfields > 0 && field >= ctx->nfields) || (ctx->nfields == 0 && field != 0))
        return gopf_fail(ctx, GOPF_ERR_ARG, "bad field id");
    return GOPF_OK;
}

// Device address of a host buffer the GPU may read and write directly (pinned or registered
// host memory under unified addressing), or nullptr for pageable memory, which goes through a
// staging copy.  On Grace-Blackwell the direct path streams over NVLink-C2C from every SM
// instead of through one copy engine.
static void *direct_host_ptr(gopf_ctx *ctx, const void *p)
{
    if (!ctx->use_direct_host) return nullptr;
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (pa.type == cudaMemoryTypeHost && pa.devicePointer) ? pa.devicePointer : nullptr;
}

template <typename R> static int upload_impl(gopf_ctx *ctx, const double *data, bool complex_in, int f)
{
    const long long N = ctx->g.N;
    if (void *dp = direct_host_ptr(ctx, data)) {
        if (complex_in)
            k_c128_to_real<R><<<ew_blocks(N), 256, 0, ctx->stream>>>((const double2 *)dp, (R *)ctx->d_real, N);
        else
            k_double_to_real<R><<<ew_blocks(N), 256, 0, ctx->stream>>>((const double *)dp, (R *)ctx->d_real, N);
        CK(cudaGetLastError());
        CK(enqueue_load_state<R>(ctx, f));
        CK(cudaStreamSynchronize(ctx->stream));
        return GOPF_OK;
    }
    if (complex_in) {
        CK(cudaMemcpyAsync(ctx->d_c128, data, sizeof(double2) * N, cudaMemcpyHostToDevice, ctx->stream));
        k_c128_to_real<R><<<ew_blocks(N), 256, 0, ctx->stream>>>(ctx->d_c128, (R *)ctx->d_real, N);
    } else {
        CK(cudaMemcpyAsync(ctx->d_c128, data, sizeof(double) * N, cudaMemcpyHostToDevice, ctx->stream));
        k_double_to_real<R><<<ew_blocks(N), 256, 0, ctx->stream>>>((const double *)ctx->d_c128, (R *)ctx->d_real, N);
    }
    CK(cudaGetLastError());
    CK(enqueue_load_state<R>(ctx, f));
    CK(cudaStreamSynchronize(ctx->stream));
    return GOPF_OK;
}

template <typename R> static int download_impl(gopf_ctx *ctx, double *data, bool complex_out, int f)
{
    const long long N = ctx->g.N;
    CK(enqueue_xpass_out<R>(ctx, (R *)ctx->d_real, nullptr, f));
    if (void *dp = direct_host_ptr(ctx, data)) {
        if (complex_out)
            k_real_to_c128<R><<<ew_blocks(N), 256, 0, ctx->stream>>>((const R *)ctx->d_real, (double2 *)dp, N);
        else
            k_real_to_double<R><<<ew_blocks(N), 256, 0, ctx->stream>>>((const R *)ctx->d_real, (double *)dp, N);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(ctx->stream));
        return GOPF_OK;
    }
    if (complex_out) {
        k_real_to_c128<R><<<ew_blocks(N), 256, 0, ctx->stream>>>((const R *)ctx->d_real, ctx->d_c128, N);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(data, ctx->d_c128, sizeof(double2) * N, cudaMemcpyDeviceToHost, ctx->stream));
    } else {
        k_real_to_double<R><<<ew_blocks(N), 256, 0, ctx->stream>>>((const R *)ctx->d_real, (double *)ctx->d_c128, N);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(data, ctx->d_c128, sizeof(double) * N, cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return GOPF_OK;
}

static int transfer(gopf_ctx *ctx, int field, double *data, size_t n, bool up, bool cplx)
{
    if (!ctx || !data) return gopf_fail(ctx, GOPF_ERR_ARG, "null argument");
    gopf_nvtx_scope trace(up ? "gopf_field_upload" : "gopf_field_download");
    int rc;
    if ((rc = require_ready(ctx, field))) return rc;
    if ((long long)n != ctx->g.N)
        return gopf_fail(ctx, GOPF_ERR_ARG, "Inconsistent domain size and number of grid points");
    if ((rc = set_device(ctx))) return rc;
    if (up) {
        rc = (ctx->prec == GOPF_FP32) ? upload_impl<float>(ctx, data, cplx, field)
                                      : upload_impl<double>(ctx, data, cplx, field);
        if (!rc) ctx->state_valid = true;
        return rc;
    }
    if (!ctx->state_valid) return gopf_fail(ctx, GOPF_ERR_STATE, "field has not been uploaded");
    return (ctx->prec == GOPF_FP32) ? download_impl<float>(ctx, data, cplx, field)
                                    : download_impl<double>(ctx, data, cplx, field);
}

extern "C" int gopf_field_upload(gopf_ctx *ctx, int f, const double *d, size_t n)
{
    return transfer(ctx, f, const_cast<double *>(d), n, true, true);
}
extern "C" int gopf_field_download(gopf_ctx *ctx, int f, double *d, size_t n) { return transfer(ctx, f, d, n, false, true); }
extern "C" int gopf_field_upload_real(gopf_ctx *ctx, int f, const double *d, size_t n)
{
    return transfer(ctx, f, const_cast<double *>(d), n, true, false);
}
extern "C" int gopf_field_download_real(gopf_ctx *ctx, int f, double *d, size_t n)
{
    return transfer(ctx, f, d, n, false, false);
}

// ------------------------------------------------------------------
// reductions
// ------------------------------------------------------------------

// Read and clear the device status word (stream-synchronising).  A set bit
// means a bounded device wait ran out: the step's results are not valid.
static int check_device_status(gopf_ctx *ctx)
{
    unsigned st = 0;
    CK(cudaMemcpyAsync(&st, ctx->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (st) {
        CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(unsigned), ctx->stream));
        return gopf_fail(ctx, GOPF_ERR_TIMEOUT, "a device copy did not complete in time (status " + std::to_string(st) + ")");
    }
    return GOPF_OK;
}

static int reduce_all(gopf_ctx *ctx, double *host5, int f = 0)
{
    cudaError_t e = (ctx->prec == GOPF_FP32) ? enqueue_xpass_out<float>(ctx, nullptr, ctx->d_red, f)
                                             : enqueue_xpass_out<double>(ctx, nullptr, ctx->d_red, f);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "reduction pass");
    const int nb = (ctx->prec == GOPF_FP32)
                       ? xpass_red_blocks<float>(xargs_out<float>(ctx, nullptr, ctx->d_red, f), ctx->LBx)
                       : xpass_red_blocks<double>(xargs_out<double>(ctx, nullptr, ctx->d_red, f), ctx->LBx);
    if (nb > ctx->nred_blocks) return gopf_fail(ctx, GOPF_ERR_STATE, "reduction partials exceed their buffer");
    k_finish_reduce<<<RED_NONFINITE + 1, 128, 0, ctx->stream>>>(ctx->d_red, nb, ctx->d_redout);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(host5, ctx->d_redout, sizeof(double) * 5, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return GOPF_OK;
}

// Non-finite values in the state (stream-synchronising); GOPF_ERR_NAN when there are any.
static int check_finite_state(gopf_ctx *ctx)
{
    unsigned *cnt = ctx->d_status + 1;
    CK(cudaMemsetAsync(cnt, 0, sizeof(unsigned), ctx->stream));
    const long long nr = 2 * ctx->g.C;
    const unsigned blocks = (unsigned)std::min<long long>((nr + 255) / 256, 152 * 8);
    for (int f = 0; f < std::max(ctx->nfields, 1); ++f) {
        const void *st = field_state(ctx, f);
        if (ctx->prec == GOPF_FP32) k_count_nonfinite<float><<<blocks, 256, 0, ctx->stream>>>((const float *)st, nr, cnt);
        else k_count_nonfinite<double><<<blocks, 256, 0, ctx->stream>>>((const double *)st, nr, cnt);
        CK(cudaGetLastError());
    }
    unsigned h = 0;
    CK(cudaMemcpyAsync(&h, cnt, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (h)
        return gopf_fail(ctx, GOPF_ERR_NAN, "field contains non-finite values after step " + std::to_string(ctx->step) +
                                                " (" + std::to_string(h) + " non-finite spectral components)");
    return GOPF_OK;
}

extern "C" int gopf_reduce(gopf_ctx *ctx, int field, int what, double *out)
{
    if (!ctx || !out) return gopf_fail(ctx, GOPF_ERR_ARG, "null argument");
    gopf_nvtx_scope trace("gopf_reduce");
    int rc;
    if ((rc = require_ready(ctx, field))) return rc;
    if (what < 0 || what > GOPF_RED_NONFINITE) return gopf_fail(ctx, GOPF_ERR_ARG, "unknown reduction");
    if (!ctx->state_valid) return gopf_fail(ctx, GOPF_ERR_STATE, "field has not been uploaded");
    if ((rc = set_device(ctx))) return rc;
    double r[5];
    if ((rc = reduce_all(ctx, r, field))) return rc;
    *out = r[what];
    return GOPF_OK;
}

// PointMonitor.Add (pf/monitor.go:27-30) for n sites: the real field at node i is the inverse x
// transform of T's row (z, y) at column x, c = Re T(0) + (-1)^x Re T(X/2) + 2 sum_{0<kx<X/2} Re(T(kx)
// e^{2 pi i kx x / X}) (T is c-hat/N already inverse-transformed along z and y; no Nyquist term for
// odd X).  One warp per
// site, FP64 sums.
template <typename R>
__global__ void k_point_values(const typename VecOf<R>::type *__restrict__ T, Geom g, const long long *__restrict__ sites,
                               int n, double *__restrict__ out)
{
    const int w = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (w >= n) return;
    const long long i = sites[w];
    const long long x = i % g.X, y = (i / g.X) % g.Y, z = i / ((long long)g.X * g.Y);
    double acc = 0.0;
    for (int kx = lane; kx < g.KX; kx += 32) {
        const typename VecOf<R>::type t = T[z * g.S + (long long)kx * g.Y + y];
        if (kx == 0 || 2 * kx == g.X) { // self-conjugate columns (the Nyquist one only for even X)
            acc += ((kx == 0 || (x & 1) == 0) ? 1.0 : -1.0) * (double)t.x;
        } else {
            double sn, cs;
            sincospi(2.0 * (double)(((long long)kx * x) % g.X) / (double)g.X, &sn, &cs);
            acc += 2.0 * ((double)t.x * cs - (double)t.y * sn);
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) out[w] = acc;
}

extern "C" int gopf_volcons_multiplier(gopf_ctx *ctx, double *out)
{
    if (!ctx || !out) return gopf_fail(ctx, GOPF_ERR_ARG, "null argument");
    if (!ctx->initialised || !ctx->has_volcons || !ctx->d_vc)
        return gopf_fail(ctx, GOPF_ERR_STATE, "the model has no volume-conserving term");
    int rc;
    if ((rc = set_device(ctx))) return rc;
    double vc[4];
    CK(cudaMemcpyAsync(vc, ctx->d_vc, sizeof(vc), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    // The device applies OnStepFinished's update (pf/volumeConserving.go:30-50) at the start of
    // the next step, where it is first needed; after n >= 2 steps the update of step n is still
    // pending: lambda - (I_n - I_{n-1}) / (dt * indicator integral of step n).
    *out = vc[0];
    if (vc[3] >= 2.0) {
        double r[5];
        const int f = ctx->multi ? ctx->vc_field : 0;
        if ((rc = reduce_all(ctx, r, f))) return rc;
        *out = vc[0] - (r[GOPF_RED_SUM] - vc[1]) / (ctx->vc_dt * vc[2]);
    }
    return GOPF_OK;
}

extern "C" int gopf_point_values(gopf_ctx *ctx, int field, const long long *sites, int n, double *out)
{
    if (!ctx || !sites || !out || n < 1) return gopf_fail(ctx, GOPF_ERR_ARG, "null argument or no sites");
    gopf_nvtx_scope trace("gopf_point_values");
    int rc;
    if ((rc = require_ready(ctx, field))) return rc;
    if (!ctx->state_valid) return gopf_fail(ctx, GOPF_ERR_STATE, "field has not been uploaded");
    if ((long long)n > ctx->g.N) return gopf_fail(ctx, GOPF_ERR_ARG, "more sites than nodes");
    for (int k = 0; k < n; ++k)
        if (sites[k] < 0 || sites[k] >= ctx->g.N) return gopf_fail(ctx, GOPF_ERR_ARG, "site outside the domain");
    if ((rc = set_device(ctx))) return rc;
    // scratch: the sites and the values share the transfer buffer (16 N bytes)
    long long *d_sites = reinterpret_cast<long long *>(ctx->d_c128);
    double *d_out = reinterpret_cast<double *>(d_sites + n);
    CK(cudaMemcpyAsync(d_sites, sites, sizeof(long long) * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
    const unsigned blocks = (unsigned)(((long long)n * 32 + 255) / 256);
    if (ctx->prec == GOPF_FP32)
        k_point_values<float><<<blocks, 256, 0, ctx->stream>>>((const float2 *)field_T(ctx, field), ctx->g, d_sites, n, d_out);
    else
        k_point_values<double><<<blocks, 256, 0, ctx->stream>>>((const double2 *)field_T(ctx, field), ctx->g, d_sites, n,
                                                                d_out);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, d_out, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return GOPF_OK;
}

// ------------------------------------------------------------------
// stepping
// ------------------------------------------------------------------

// Work buffers of the stepper beyond the context's own (RK4's accumulator), allocated on first use.
static int stepper_buffers(gopf_ctx *ctx)
{
    int rc;
    if (ctx->stepper == GOPF_STEPPER_RK4) {
        if (ctx->has_elastic || ctx->has_volcons || ctx->noise.kind)
            return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "user-defined and noise terms are stepped with Euler only");
        if ((rc = alloc_spectral(ctx, &ctx->d_rkF))) return rc;
        if (ctx->multi)
            for (int f = 1; f < ctx->nfields; ++f)
                if ((rc = alloc_spectral(ctx, &ctx->d_frkF[f]))) return rc;
    }
    return GOPF_OK;
}

// The graphs a run of `left` graph-stepped steps replays: one step, and graphK steps when the run is
// that long.  Capturing records the launches without running them.
static int ensure_graphs(gopf_ctx *ctx, long long left)
{
    int rc;
    if (!ctx->gexec1 && (rc = capture_graph(ctx, 1, &ctx->gexec1))) return rc;
    if (left >= ctx->graphK && !ctx->gexecK && (rc = capture_graph(ctx, ctx->graphK, &ctx->gexecK))) return rc;
    return GOPF_OK;
}

extern "C" int gopf_prepare_graphs(gopf_ctx *ctx, long long nsteps)
{
    if (!ctx) return GOPF_ERR_ARG;
    if (nsteps < 0) return gopf_fail(ctx, GOPF_ERR_ARG, "negative step count");
    if (!ctx->initialised) return gopf_fail(ctx, GOPF_ERR_STATE, "model not initialised (gopf_init/gopf_set_terms)");
    if (!(ctx->dt > 0.0)) return gopf_fail(ctx, GOPF_ERR_STATE, "no stepper set (gopf_set_stepper)");
    if (!ctx->state_valid) return gopf_fail(ctx, GOPF_ERR_STATE, "field has not been uploaded");
    int rc;
    if ((rc = set_device(ctx))) return rc;
    if (!ctx->use_graphs || ctx->stepper == GOPF_STEPPER_SDD || ctx->stepper == GOPF_STEPPER_IMPLICIT_EULER)
        return GOPF_OK; // host-driven steppers replay no graphs
    if ((rc = stepper_buffers(ctx))) return rc;
    if (ctx->has_elastic && !ctx->el_primed) return GOPF_OK; // the first elastic step is not replayed
    return ensure_graphs(ctx, nsteps);
}

extern "C" int gopf_step(gopf_ctx *ctx, long long nsteps)
{
    if (!ctx) return GOPF_ERR_ARG;
    gopf_nvtx_scope trace("gopf_step");
    if (nsteps < 0) return gopf_fail(ctx, GOPF_ERR_ARG, "negative step count");
    if (!ctx->initialised) return gopf_fail(ctx, GOPF_ERR_STATE, "model not initialised (gopf_init/gopf_set_terms)");
    if (!(ctx->dt > 0.0)) return gopf_fail(ctx, GOPF_ERR_STATE, "no stepper set (gopf_set_stepper)");
    if (!ctx->state_valid) return gopf_fail(ctx, GOPF_ERR_STATE, "field has not been uploaded");
    int rc;
    if ((rc = set_device(ctx))) return rc;
    if ((rc = stepper_buffers(ctx))) return rc;
    if (!ctx->sources.empty()) {
        if (ctx->stepper == GOPF_STEPPER_SDD || ctx->stepper == GOPF_STEPPER_IMPLICIT_EULER)
            return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "sources are stepped with Euler and RK4");
        if (ctx->step < ctx->src_base || ctx->step + nsteps > ctx->src_base + ctx->src_len)
            return gopf_fail(ctx, GOPF_ERR_STATE,
                             "source amplitudes do not cover these steps (gopf_set_source_amplitudes)");
    }
    if (ctx->stepper == GOPF_STEPPER_SDD) {
        // a host-driven saddle search (pf/sdd.go): no graphs
        if ((rc = gopf_sdd_step(ctx, nsteps))) return rc;
        ctx->step += nsteps;
        if (ctx->check_finite) {
            if ((rc = check_device_status(ctx))) return rc;
            if ((rc = check_finite_state(ctx))) return rc;
        }
        return GOPF_OK;
    }
    if (ctx->stepper == GOPF_STEPPER_IMPLICIT_EULER) {
        if (ctx->has_elastic || ctx->has_volcons || ctx->noise.kind)
            return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "user-defined and noise terms are stepped with Euler only");
        if (!ctx->multi && ctx->ngroups + 1 > GOPF_MAX_GROUPS)
            return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "implicit Euler supports at most 3 explicit groups");
        if (ctx->multi) { // the residual adds FFT(x_f) to each equation's groups and to the x-pass outputs
            if (ctx->mono_rk.ngrp + ctx->nfields > GOPF_MAX_XOUT)
                return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "implicit Euler: too many term groups over all equations");
            for (const auto &ep : ctx->eqs_rk)
                if (ep.upd.ngrp + 1 > GOPF_MAX_GROUPS)
                    return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "implicit Euler supports at most 3 explicit groups");
        }
        // a host-driven Newton-Krylov solve per step: no graphs
        for (long long s = 0; s < nsteps; ++s) {
            if ((rc = gopf_ie_step(ctx))) return rc;
            ++ctx->step;
        }
        if (ctx->check_finite) {
            if ((rc = check_device_status(ctx))) return rc;
            if ((rc = check_finite_state(ctx))) return rc;
        }
        return GOPF_OK;
    }
    long long left = nsteps;
    if (ctx->has_elastic && !ctx->el_primed && left > 0) {
        // first step ever: the elastic term sees the reference's zero h-field
        cudaError_t e = enqueue_steps_any(ctx, 1);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "step");
        ctx->el_primed = true;
        invalidate_graphs(ctx);
        --left;
    }
    if (ctx->use_graphs) {
        if ((rc = ensure_graphs(ctx, left))) return rc;
        while (left >= ctx->graphK) {
            CK(cudaGraphLaunch(ctx->gexecK, ctx->stream));
            left -= ctx->graphK;
        }
        while (left > 0) {
            CK(cudaGraphLaunch(ctx->gexec1, ctx->stream));
            --left;
        }
    } else {
        cudaError_t e = enqueue_steps_any(ctx, (int)std::min<long long>(left, 1 << 30));
        if (e != cudaSuccess) return cuda_fail(ctx, e, "step");
    }
    ctx->step += nsteps;
    if (ctx->check_finite) {
        if ((rc = check_device_status(ctx))) return rc;
        if ((rc = check_finite_state(ctx))) return rc;
    }
    return GOPF_OK;
}

// ---- device-side helpers for the adjoint (stream-ordered, no synchronisation) ----

int gopf_field_to_real(gopf_ctx *ctx, int f, void *dst)
{
    cudaError_t e = (ctx->prec == GOPF_FP32) ? enqueue_xpass_out<float>(ctx, (float *)dst, nullptr, f)
                                             : enqueue_xpass_out<double>(ctx, (double *)dst, nullptr, f);
    return (e == cudaSuccess) ? GOPF_OK : cuda_fail(ctx, e, "state to real");
}

int gopf_state_to_real(gopf_ctx *ctx, void *dst) { return gopf_field_to_real(ctx, 0, dst); }

// src = [field 0 | field 1 | ...] (one field for single-field models)
int gopf_real_to_state(gopf_ctx *ctx, const void *src)
{
    const size_t rb = (ctx->prec == GOPF_FP32 ? sizeof(float) : sizeof(double)) * ctx->g.N;
    const int nf = ctx->multi ? ctx->nfields : 1;
    for (int f = 0; f < nf; ++f) {
        CK(cudaMemcpyAsync(ctx->d_real, (const char *)src + f * rb, rb, cudaMemcpyDeviceToDevice, ctx->stream));
        cudaError_t e = (ctx->prec == GOPF_FP32) ? enqueue_load_state<float>(ctx, f) : enqueue_load_state<double>(ctx, f);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "real to state");
    }
    ctx->state_valid = true;
    return GOPF_OK;
}

int gopf_step_device(gopf_ctx *ctx, long long n)
{
    cudaError_t e = enqueue_steps_any(ctx, (int)n);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "step");
    ctx->step += n;
    return GOPF_OK;
}

// ---- device pieces of ImplicitEuler (pf/implicitEuler.go), stream-ordered ----

// N_n = the explicit RHS of the current state (read from T) in k space, into nprev.
// tmp0 is a spectral scratch buffer; T and the state are left unchanged.
template <typename R> static cudaError_t enqueue_ie_rhs(gopf_ctx *ctx, void *nprev, void *tmp0)
{
    typedef typename VecOf<R>::type V;
    const int G = ctx->ngroups;
    const bool is3d = ctx->g.Z > 1;
    if (G == 0) return cudaMemsetAsync(nprev, 0, sizeof(V) * ctx->g.C, ctx->stream);
    V *U[GOPF_MAX_GROUPS];
    U[0] = (V *)tmp0;
    for (int b = 1; b < GOPF_MAX_GROUPS; ++b) U[b] = (V *)ctx->d_U[b];
    XPassArgs<R> xa = xargs<R>(ctx);
    xa.in_mode = XIN_SPECTRAL;
    xa.in = (const V *)ctx->d_T;
    for (int b = 0; b < G; ++b) xa.out[b] = U[b];
    xa.ngrp_out = G;
    xa.pw = ctx->pw;
    LK(launch_xpass<R>(xa, ctx->LBx, ctx->stream));
    if (is3d) {
        PassArgs<R> pa = pargs<R>(ctx, false);
        pa.mode = PM_FWD;
        for (int b = 0; b < G; ++b) pa.buf[b] = U[b];
        pa.nbuf = G;
        LK(launch_cpass<R>(pa, ctx->LBy, ctx->stream));
    }
    PassArgs<R> fa = pargs<R>(ctx, is3d);
    fa.mode = PM_FUSED;
    for (int b = 0; b < G; ++b) fa.buf[b] = U[b];
    fa.nbuf = G;
    fa.state = (V *)ctx->d_state;
    fa.tout = U[0];
    fa.upd = ctx->upd;
    fa.upd.dt = ctx->dt;
    fa.upd.invN = 1.0 / (double)ctx->g.N;
    fa.upd.etd = 1;
    fa.upd.filt = nullptr; // ImplicitEuler ignores filters (pf/implicitEuler.go:209-213)
    fa.rkF = (V *)nprev;
    LK(is3d ? launch_spass<R>(fa, ctx->LBz, ctx->stream) : launch_cpass<R>(fa, ctx->LBy, ctx->stream));
    return cudaSuccess;
}

// F(x) = x - IFFT(c_n e^(L dt) + I(L, N(x), N_n)) / N for a real field x (updateEquation,
// pf/implicitEuler.go:68-94).  Uses T, the group buffers and tmp0 as work space.
template <typename R>
static cudaError_t enqueue_ie_residual(gopf_ctx *ctx, const R *x, R *F, const void *chat0, const void *nprev,
                                       void *tmp0)
{
    typedef typename VecOf<R>::type V;
    const int G = ctx->ngroups;
    const bool is3d = ctx->g.Z > 1;
    V *U[GOPF_MAX_GROUPS];
    U[0] = (V *)ctx->d_T;
    for (int b = 1; b < GOPF_MAX_GROUPS; ++b) U[b] = (V *)ctx->d_U[b];
    U[G] = (V *)tmp0; // FFT(x)
    PwTable pw = ctx->pw;
    pw.ngrp = G + 1;
    pw.nterm[G] = 1;
    pw.pw[G][0] = 1;
    pw.coef[G][0] = 1.0;
    pw_densify(pw);
    XPassArgs<R> xa = xargs<R>(ctx);
    xa.in_mode = XIN_REAL;
    xa.rin = x;
    for (int b = 0; b <= G; ++b) xa.out[b] = U[b];
    xa.ngrp_out = G + 1;
    xa.pw = pw;
    LK(launch_xpass<R>(xa, ctx->LBx, ctx->stream));
    if (is3d) {
        PassArgs<R> pa = pargs<R>(ctx, false);
        pa.mode = PM_FWD;
        for (int b = 0; b <= G; ++b) pa.buf[b] = U[b];
        pa.nbuf = G + 1;
        LK(launch_cpass<R>(pa, ctx->LBy, ctx->stream));
    }
    PassArgs<R> fa = pargs<R>(ctx, is3d);
    fa.mode = PM_FUSED;
    for (int b = 0; b <= G; ++b) fa.buf[b] = U[b];
    fa.nbuf = G + 1;
    fa.state = (V *)const_cast<void *>(chat0);
    fa.tout = (V *)ctx->d_T;
    fa.upd = ctx->upd;
    fa.upd.dt = ctx->dt;
    fa.upd.invN = 1.0 / (double)ctx->g.N;
    fa.upd.etd = 2;
    fa.upd.filt = nullptr;
    fa.rkF = (V *)const_cast<void *>(nprev);
    LK(is3d ? launch_spass<R>(fa, ctx->LBz, ctx->stream) : launch_cpass<R>(fa, ctx->LBy, ctx->stream));
    if (is3d) {
        PassArgs<R> ia = pargs<R>(ctx, false);
        ia.mode = PM_INV;
        ia.buf[0] = (V *)ctx->d_T;
        ia.nbuf = 1;
        LK(launch_cpass<R>(ia, ctx->LBy, ctx->stream));
    }
    return enqueue_xpass_out<R>(ctx, F, nullptr);
}

// Models of several fields (ImplicitEuler.Step over m.Fields, pf/implicitEuler.go:68-94, 165-207):
// the unknown is [field 0 | field 1 | ...] in real space, every right-hand side is evaluated from
// all fields at once (the RK4 plan: field terms are x-pass products), and grp[j] are spectral
// scratch buffers, j < (monomial groups) + (fields).  The RHS pass leaves T and the state alone.
template <typename R> static cudaError_t enqueue_ie_rhs_multi(gopf_ctx *ctx, void *nprev, void *const *grp)
{
    typedef typename VecOf<R>::type V;
    const int nf = ctx->nfields;
    const bool is3d = ctx->g.Z > 1;
    const std::vector<gopf_ctx::EqPlan> &eqs = ctx->eqs_rk;
    const MonoTable &mono = ctx->mono_rk;
    const long long C = ctx->g.C;
    if (mono.ngrp > 0) {
        XPassArgs<R> xa = xargs<R>(ctx);
        xa.in_mode = XIN_SPECTRAL;
        xa.program = XP_MULTI;
        xa.allow_fast = 0;
        for (int f = 0; f < nf; ++f) xa.inF[f] = (const V *)field_T(ctx, f);
        for (int j = 0; j < mono.ngrp; ++j) xa.out[j] = (V *)grp[j];
        xa.ngrp_out = mono.ngrp;
        xa.mono = mono;
        LK(launch_xpass<R>(xa, ctx->LBm, ctx->stream));
    }
    for (int e = 0; e < nf; ++e) {
        const int G = eqs[e].upd.ngrp, first = eqs[e].first;
        if (is3d && G > 0) {
            PassArgs<R> pa = pargs<R>(ctx, false);
            pa.mode = PM_FWD;
            for (int b = 0; b < G; ++b) pa.buf[b] = (V *)grp[first + b];
            pa.nbuf = G;
            LK(launch_cpass<R>(pa, ctx->LBy, ctx->stream));
        }
        PassArgs<R> fa = pargs<R>(ctx, is3d);
        fa.mode = PM_FUSED;
        const int nb = std::max(G, 1);
        for (int b = 0; b < nb; ++b) fa.buf[b] = (V *)grp[G > 0 ? first + b : mono.ngrp];
        fa.nbuf = nb;
        fa.state = (V *)field_state(ctx, e);
        fa.tout = (V *)grp[mono.ngrp + nf]; // written as zeros
        fa.upd = eqs[e].upd;
        fa.upd.dt = ctx->dt;
        fa.upd.invN = 1.0 / (double)ctx->g.N;
        fa.upd.etd = 1;
        fa.upd.filt = nullptr;
        fa.rkF = (V *)nprev + e * C;
        LK(is3d ? launch_spass<R>(fa, ctx->LBz, ctx->stream) : launch_cpass<R>(fa, ctx->LBy, ctx->stream));
    }
    return cudaSuccess;
}

// F_f(x) = x_f - IFFT(c_f e^(L dt) + I(L, N_f(x), N_f,n)) / N for every field f; T is work space.
template <typename R>
static cudaError_t enqueue_ie_residual_multi(gopf_ctx *ctx, const R *x, R *F, const void *chat0, const void *nprev,
                                             void *const *grp)
{
    typedef typename VecOf<R>::type V;
    const int nf = ctx->nfields;
    const bool is3d = ctx->g.Z > 1;
    const std::vector<gopf_ctx::EqPlan> &eqs = ctx->eqs_rk;
    const long long C = ctx->g.C, N = ctx->g.N;
    // the equations' groups, then FFT_x(x_f) of every field (one monomial x_f each)
    MonoTable mono = ctx->mono_rk;
    const int G0 = mono.ngrp;
    for (int f = 0; f < nf; ++f) {
        const int j = mono.ngrp++;
        mono.nmono[j] = 1;
        mono.coef[j][0] = 1.0;
        memset(mono.pw[j][0], 0, GOPF_MAX_FIELDS);
        mono.pw[j][0][f] = 1;
    }
    XPassArgs<R> xa = xargs<R>(ctx);
    xa.in_mode = XIN_REAL;
    xa.program = XP_MULTI;
    xa.allow_fast = 0;
    for (int f = 0; f < nf; ++f) xa.rinF[f] = x + f * N;
    for (int j = 0; j < mono.ngrp; ++j) xa.out[j] = (V *)grp[j];
    xa.ngrp_out = mono.ngrp;
    xa.mono = mono;
    LK(launch_xpass<R>(xa, ctx->LBm, ctx->stream));
    for (int e = 0; e < nf; ++e) {
        const int G = eqs[e].upd.ngrp, first = eqs[e].first;
        V *buf[GOPF_MAX_GROUPS];
        for (int b = 0; b < G; ++b) buf[b] = (V *)grp[first + b];
        buf[G] = (V *)grp[G0 + e]; // FFT(x_e)
        if (is3d) {
            PassArgs<R> pa = pargs<R>(ctx, false);
            pa.mode = PM_FWD;
            for (int b = 0; b <= G; ++b) pa.buf[b] = buf[b];
            pa.nbuf = G + 1;
            LK(launch_cpass<R>(pa, ctx->LBy, ctx->stream));
        }
        PassArgs<R> fa = pargs<R>(ctx, is3d);
        fa.mode = PM_FUSED;
        for (int b = 0; b <= G; ++b) fa.buf[b] = buf[b];
        fa.nbuf = G + 1;
        fa.state = (V *)const_cast<void *>(chat0) + e * C;
        fa.tout = (V *)field_T(ctx, e);
        fa.upd = eqs[e].upd;
        fa.upd.dt = ctx->dt;
        fa.upd.invN = 1.0 / (double)N;
        fa.upd.etd = 2;
        fa.upd.filt = nullptr;
        fa.rkF = (V *)const_cast<void *>(nprev) + e * C;
        LK(is3d ? launch_spass<R>(fa, ctx->LBz, ctx->stream) : launch_cpass<R>(fa, ctx->LBy, ctx->stream));
    }
    if (is3d) {
        PassArgs<R> ia = pargs<R>(ctx, false);
        ia.mode = PM_INV;
        for (int f = 0; f < nf; ++f) ia.buf[f] = (V *)field_T(ctx, f);
        ia.nbuf = nf;
        LK(launch_cpass<R>(ia, ctx->LBy, ctx->stream));
    }
    for (int f = 0; f < nf; ++f) LK(enqueue_xpass_out<R>(ctx, F + f * N, nullptr, f));
    return cudaSuccess;
}

int gopf_ie_rhs_multi(gopf_ctx *ctx, void *nprev, void *const *grp)
{
    cudaError_t e = (ctx->prec == GOPF_FP32) ? enqueue_ie_rhs_multi<float>(ctx, nprev, grp)
                                             : enqueue_ie_rhs_multi<double>(ctx, nprev, grp);
    return (e == cudaSuccess) ? GOPF_OK : cuda_fail(ctx, e, "implicit Euler: RHS");
}

int gopf_ie_residual_multi(gopf_ctx *ctx, const void *x, void *F, const void *chat0, const void *nprev,
                           void *const *grp)
{
    cudaError_t e = (ctx->prec == GOPF_FP32)
                        ? enqueue_ie_residual_multi<float>(ctx, (const float *)x, (float *)F, chat0, nprev, grp)
                        : enqueue_ie_residual_multi<double>(ctx, (const double *)x, (double *)F, chat0, nprev, grp);
    return (e == cudaSuccess) ? GOPF_OK : cuda_fail(ctx, e, "implicit Euler: residual");
}

int gopf_ie_rhs(gopf_ctx *ctx, void *nprev, void *tmp0)
{
    cudaError_t e = (ctx->prec == GOPF_FP32) ? enqueue_ie_rhs<float>(ctx, nprev, tmp0)
                                             : enqueue_ie_rhs<double>(ctx, nprev, tmp0);
    return (e == cudaSuccess) ? GOPF_OK : cuda_fail(ctx, e, "implicit Euler: RHS");
}

int gopf_ie_residual(gopf_ctx *ctx, const void *x, void *F, const void *chat0, const void *nprev, void *tmp0)
{
    cudaError_t e = (ctx->prec == GOPF_FP32)
                        ? enqueue_ie_residual<float>(ctx, (const float *)x, (float *)F, chat0, nprev, tmp0)
                        : enqueue_ie_residual<double>(ctx, (const double *)x, (double *)F, chat0, nprev, tmp0);
    return (e == cudaSuccess) ? GOPF_OK : cuda_fail(ctx, e, "implicit Euler: residual");
}

// One explicit Euler step of the state (the Newton start, pf/implicitEuler.go:182-190); x0 <- real field.
// (several fields: Euler.Step's in-place sweep over the fields, then x0 = [field 0 | field 1 | ...])
int gopf_ie_euler_guess(gopf_ctx *ctx, void *x0)
{
    const bool f32 = (ctx->prec == GOPF_FP32);
    cudaError_t e;
    if (ctx->multi) e = f32 ? enqueue_multi_stage<float>(ctx, 0) : enqueue_multi_stage<double>(ctx, 0);
    else e = f32 ? enqueue_euler<float>(ctx) : enqueue_euler<double>(ctx);
    const int nf = ctx->multi ? ctx->nfields : 1;
    for (int f = 0; f < nf && e == cudaSuccess; ++f)
        e = f32 ? enqueue_xpass_out<float>(ctx, (float *)x0 + f * ctx->g.N, nullptr, f)
                : enqueue_xpass_out<double>(ctx, (double *)x0 + f * ctx->g.N, nullptr, f);
    return (e == cudaSuccess) ? GOPF_OK : cuda_fail(ctx, e, "implicit Euler: explicit guess");
}

// NewVandeven (pf/vandeven.go:13-27): the 1000-point table
// 1 - Gamma(2p)/Gamma(p)^2 * integral_0^x (t(1-t))^(p-1) dt by the trapezoid rule.
extern "C" int gopf_vandeven_table(int order, double *out, int n)
{
    if (order < 1 || !out || n != 1000) return GOPF_ERR_ARG;
    const double pref = std::tgamma((double)(2 * order)) / (std::tgamma((double)order) * std::tgamma((double)order));
    const double dx = 1.0 / 999.0;
    out[0] = 1.0;
    for (int i = 1; i < 1000; ++i) {
        const double x = (double)i * dx, x1 = x - dx;
        const double i2 = std::pow(x * (1.0 - x), (double)(order - 1));
        const double i1 = std::pow(x1 * (1.0 - x1), (double)(order - 1));
        out[i] = out[i - 1] - pref * 0.5 * (i1 + i2) * dx;
    }
    return GOPF_OK;
}

extern "C" int gopf_set_modal_filter(gopf_ctx *ctx, const double *table, int n)
{
    if (!ctx) return GOPF_ERR_ARG;
    if (n == 0 || !table) {
        ctx->upd.filt = nullptr;
        ctx->upd.nfilt = 0;
        invalidate_graphs(ctx);
        return GOPF_OK;
    }
    if (n < 2 || n > 65536) return gopf_fail(ctx, GOPF_ERR_ARG, "a filter table needs 2 to 65536 samples");
    if (!ctx->initialised) return gopf_fail(ctx, GOPF_ERR_STATE, "set the filter after gopf_init");
    int rc;
    if ((rc = set_device(ctx))) return rc;
    if (ctx->d_filter) {
        cudaFree(ctx->d_filter);
        ctx->d_filter = nullptr;
    }
    const size_t eb = (ctx->prec == GOPF_FP32) ? sizeof(float) : sizeof(double);
    CK(gopf_malloc(&ctx->d_filter, eb * (size_t)n));
    if (ctx->prec == GOPF_FP32) {
        std::vector<float> t(table, table + n);
        CK(cudaMemcpy(ctx->d_filter, t.data(), eb * (size_t)n, cudaMemcpyHostToDevice));
    } else {
        CK(cudaMemcpy(ctx->d_filter, table, eb * (size_t)n, cudaMemcpyHostToDevice));
    }
    ctx->upd.filt = ctx->d_filter;
    ctx->upd.nfilt = n;
    invalidate_graphs(ctx);
    return GOPF_OK;
}

extern "C" int gopf_set_newton_krylov(gopf_ctx *ctx, int maxiter, double step_size, double tol, int stencil,
                                      int restart)
{
    if (!ctx) return GOPF_ERR_ARG;
    if (maxiter < 0 || !(step_size > 0.0) || !(tol > 0.0) || restart < 1 || restart > 1000)
        return gopf_fail(ctx, GOPF_ERR_ARG, "bad Newton-Krylov controls");
    if (stencil != 2 && stencil != 4 && stencil != 6 && stencil != 8)
        return gopf_fail(ctx, GOPF_ERR_ARG, "finite-difference stencil must have 2, 4, 6 or 8 points");
    ctx->nk_maxiter = maxiter;
    ctx->nk_step = step_size;
    ctx->nk_tol = tol;
    ctx->nk_stencil = stencil;
    ctx->nk_restart = restart;
    return GOPF_OK;
}

extern "C" int gopf_newton_stats(gopf_ctx *ctx, int *newton_iters, int *krylov_iters, double *residual, int *converged)
{
    if (!ctx) return GOPF_ERR_ARG;
    if (newton_iters) *newton_iters = ctx->nk_last_newton;
    if (krylov_iters) *krylov_iters = ctx->nk_last_krylov;
    if (residual) *residual = ctx->nk_last_residual;
    if (converged) *converged = ctx->nk_last_converged;
    return GOPF_OK;
}

extern "C" int gopf_synchronize(gopf_ctx *ctx)
{
    if (!ctx) return GOPF_ERR_ARG;
    int rc;
    if ((rc = set_device(ctx))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return check_device_status(ctx);
}

extern "C" int gopf_get_time(gopf_ctx *ctx, double *t)
{
    if (!ctx || !t) return GOPF_ERR_ARG;
    *t = (double)ctx->step * ctx->dt; // Euler.GetTime (pf/euler.go:50-52)
    return GOPF_OK;
}

extern "C" int gopf_get_step(gopf_ctx *ctx, long long *s)
{
    if (!ctx || !s) return GOPF_ERR_ARG;
    *s = ctx->step;
    return GOPF_OK;
}

// ------------------------------------------------------------------
// Freq / ConjugateNode (pfutil/fftWrap.go:41-95)
// ------------------------------------------------------------------

extern "C" int gopf_freq(gopf_ctx *ctx, long long i, double *out)
{
    if (!ctx || !out) return GOPF_ERR_ARG;
    const long long n0 = ctx->dims[0], n1 = ctx->dims[1];
    if (i < 0 || i >= ctx->g.N) return gopf_fail(ctx, GOPF_ERR_ARG, "node index out of range");
    const long long col = i % n1, row = (i / n1) % n0;
    out[0] = (double)row / (double)n0;
    out[1] = (double)col / (double)n1;
    if (ctx->ndim == 3) out[2] = (double)(i / (n0 * n1)) / (double)ctx->dims[2];
    for (int d = 0; d < ctx->ndim; ++d)
        if (out[d] > 0.5) out[d] -= 1.0;
    return GOPF_OK;
}

extern "C" long long gopf_conjugate_node(gopf_ctx *ctx, long long i)
{
    if (!ctx || i < 0 || i >= ctx->g.N) return -1;
    const long long n0 = ctx->dims[0], n1 = ctx->dims[1];
    const long long c = i % n1, r = (i / n1) % n0;
    long long cd = 0;
    if (ctx->ndim == 3) {
        const long long d = i / (n0 * n1);
        cd = (ctx->dims[2] - d) % ctx->dims[2];
    }
    return cd * n0 * n1 + ((n0 - r) % n0) * n1 + (n1 - c) % n1;
}

extern "C" int gopf_device_bytes(gopf_ctx *ctx, size_t *bytes)
{
    if (!ctx || !bytes) return GOPF_ERR_ARG;
    *bytes = ctx->dev_bytes;
    return GOPF_OK;
}

static void step_slots(gopf_ctx *ctx, std::vector<std::string> &names, std::vector<double> &bytes);

extern "C" int gopf_kernel_launches(gopf_ctx *ctx, long long nsteps, long long *count)
{
    if (!ctx || !count || nsteps < 0) return GOPF_ERR_ARG;
    if (ctx->use_graphs && ctx->stepper != GOPF_STEPPER_IMPLICIT_EULER && ctx->graph_kernels1 > 0 &&
        (nsteps < ctx->graphK || ctx->graph_kernelsK > 0)) {
        *count = (nsteps / ctx->graphK) * ctx->graph_kernelsK + (nsteps % ctx->graphK) * ctx->graph_kernels1;
        return GOPF_OK;
    }
    return gopf_fail(ctx, GOPF_ERR_STATE, "launch counts are known for graph-replayed steps after the graphs exist");
}

extern "C" int gopf_kernels_per_step(gopf_ctx *ctx, int *n)
{
    if (!ctx || !n) return GOPF_ERR_ARG;
    std::vector<std::string> names;
    std::vector<double> bytes;
    step_slots(ctx, names, bytes);
    *n = (int)names.size();
    return GOPF_OK;
}

// ------------------------------------------------------------------
// per-kernel profiling of one step
// ------------------------------------------------------------------

// Kernel slots of one step with their algorithmic HBM bytes (each pass reads
// and writes its arrays once).
static void step_slots(gopf_ctx *ctx, std::vector<std::string> &names, std::vector<double> &bytes)
{
    const double vb = (ctx->prec == GOPF_FP32) ? 8.0 : 16.0;
    const double C = (double)ctx->g.C * vb;
    const bool el = ctx->has_elastic && ctx->el_primed;
    const int G = ctx->ngroups;
    const int GE = G + (el ? 1 : 0);
    const int nb = std::max(GE, 1);
    const bool is3d = ctx->g.Z > 1;
    names.clear();
    bytes.clear();
    auto add = [&](const char *n, double b) {
        names.push_back(n);
        bytes.push_back(b);
    };
    if (GE > 0) add("xpass_pointwise", (1.0 + GE) * C);
    if (ctx->has_volcons) add("volcons_multiplier", 0.0);
    if (el) {
        if (is3d) add("ypass_forward", 2.0 * GE * C);
        add(is3d ? "zpass_elastic_symbol" : "ypass_elastic_symbol", 2.0 * C + C / 2.0);
        if (is3d) add("ypass_inverse", 2.0 * C);
        add("xpass_elastic", 3.0 * C);
        if (is3d) add("ypass_forward", 2.0 * C);
    } else if (is3d && GE > 0) {
        add("ypass_forward", 2.0 * GE * C);
    }
    add(is3d ? "zpass_update" : "ypass_update", (nb + 3.0) * C);
    add("hermitian_planes", 4.0 * C / ctx->g.KX);
    if (is3d) add("ypass_inverse", 2.0 * C);
}

extern "C" int gopf_profile_step(gopf_ctx *ctx, int nsteps, double *avg_ms, double *alg_bytes, int capacity, int *nslots)
{
    if (!ctx || !nslots || nsteps < 1) return gopf_fail(ctx, GOPF_ERR_ARG, "bad argument");
    if (!ctx->initialised || !ctx->state_valid || !(ctx->dt > 0.0))
        return gopf_fail(ctx, GOPF_ERR_STATE, "model, stepper and field must be set before profiling");
    if (ctx->stepper != GOPF_STEPPER_EULER || ctx->multi)
        return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "profiling covers the Euler step of single-field models");
    if (ctx->has_elastic && !ctx->el_primed) return gopf_fail(ctx, GOPF_ERR_STATE, "take one step before profiling");
    int rc;
    if ((rc = set_device(ctx))) return rc;
    std::vector<std::string> names;
    std::vector<double> bytes;
    step_slots(ctx, names, bytes);
    const size_t ns = names.size();
    *nslots = (int)ns;
    // The step's launches with a CUDA event between consecutive kernels, nsteps times.
    std::vector<cudaEvent_t> ev(1 + ns * nsteps);
    for (auto &e : ev) CK(cudaEventCreate(&e));
    std::vector<double> acc(ns, 0.0);
    cudaError_t e = cudaSuccess;
    CK(cudaEventRecord(ev[0], ctx->stream));
    ctx->prof_events = &ev;
    ctx->prof_next = 1;
    for (int s = 0; s < nsteps && e == cudaSuccess; ++s)
        e = (ctx->prec == GOPF_FP32) ? enqueue_euler<float>(ctx) : enqueue_euler<double>(ctx);
    ctx->prof_events = nullptr;
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess && ctx->prof_next != ev.size()) e = cudaErrorInvalidValue;
    if (e == cudaSuccess) {
        for (int s = 0; s < nsteps; ++s)
            for (size_t k = 0; k < ns; ++k) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, ev[s * ns + k], ev[s * ns + k + 1]);
                acc[k] += ms;
            }
        ctx->step += nsteps;
    }
    for (auto &x : ev) cudaEventDestroy(x);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "profile");
    for (size_t k = 0; k < ns && (int)k < capacity; ++k) {
        if (avg_ms) avg_ms[k] = acc[k] / nsteps;
        if (alg_bytes) alg_bytes[k] = bytes[k];
    }
    return GOPF_OK;
}

extern "C" int gopf_profile_slot_name(gopf_ctx *ctx, int slot, char *buf, int buflen)
{
    if (!ctx || !buf || buflen < 1) return GOPF_ERR_ARG;
    std::vector<std::string> names;
    std::vector<double> bytes;
    step_slots(ctx, names, bytes);
    if (slot < 0 || slot >= (int)names.size()) return gopf_fail(ctx, GOPF_ERR_ARG, "bad slot");
    snprintf(buf, buflen, "%s", names[slot].c_str());
    return GOPF_OK;
}

// FourierTransform.FFT/IFFT on host []complex128 is provided by gopf_fft.cu.
