// gopf_fft.cu -- pfutil.FourierTransform on host []complex128 data.
//
// FFTWWrapper.FFT/IFFT (pfutil/fftWrap.go:26-39) transform a complex field in
// place, unnormalised.  This entry point serves callers that use the
// FourierTransform interface directly (tests, one-off transforms); it is not
// on the stepping path.  A complex field a + i b is transformed as two real
// fields through the device r2c/c2r passes and recombined on the host:
//   forward : F(a + i b) = F(a) + i F(b), each expanded from its half spectrum
//   backward: X = A + i B with A, B Hermitian, A(k) = (X(k) + conj X(-k))/2,
//             B(k) = (X(k) - conj X(-k))/(2i); result = c2r(A) + i c2r(B).
#include <complex>
#include <cstring>
#include <vector>

#include "gopf_ctx.h"
#include "gopf_kernels.cuh"

using namespace gopf;

namespace {

struct FftScratch {
    void *buf = nullptr;
};

int ck(gopf_ctx *ctx, cudaError_t e, const char *where)
{
    if (e == cudaSuccess) return GOPF_OK;
    return gopf_fail(ctx, e == cudaErrorMemoryAllocation ? GOPF_ERR_OOM : GOPF_ERR_CUDA,
                     std::string(where) + ": " + cudaGetErrorString(e));
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
    return a;
}

// real host field -> half spectrum (host, layout [Z][KX][Y])
template <typename R>
int forward_real(gopf_ctx *ctx, void *dbuf, const std::vector<double> &in, std::vector<std::complex<double>> &half)
{
    typedef typename VecOf<R>::type V;
    const Geom &g = ctx->g;
    std::vector<R> hr(g.N);
    for (long long i = 0; i < g.N; ++i) hr[i] = (R)in[i];
    int rc;
    if ((rc = ck(ctx, cudaMemcpyAsync(ctx->d_real, hr.data(), sizeof(R) * g.N, cudaMemcpyHostToDevice, ctx->stream),
                 "H2D")))
        return rc;
    XPassArgs<R> xa = xbase<R>(ctx);
    xa.in_mode = XIN_REAL;
    xa.rin = (const R *)ctx->d_real;
    xa.out[0] = (V *)dbuf;
    xa.ngrp_out = 1;
    xa.identity = 1;
    if ((rc = ck(ctx, launch_xpass<R>(xa, ctx->LBx, ctx->stream), "x pass"))) return rc;
    if ((rc = ck(ctx, launch_cpass<R>(pbase<R>(ctx, false, PM_FWD, dbuf), ctx->LBy, ctx->stream), "y pass"))) return rc;
    if (g.Z > 1 && (rc = ck(ctx, launch_spass<R>(pbase<R>(ctx, true, PM_FWD, dbuf), ctx->LBz, ctx->stream), "z pass")))
        return rc;
    std::vector<V> hv(g.C);
    if ((rc = ck(ctx, cudaMemcpyAsync(hv.data(), dbuf, sizeof(V) * g.C, cudaMemcpyDeviceToHost, ctx->stream), "D2H")))
        return rc;
    if ((rc = ck(ctx, cudaStreamSynchronize(ctx->stream), "sync"))) return rc;
    half.resize(g.C);
    for (long long i = 0; i < g.C; ++i) half[i] = std::complex<double>((double)hv[i].x, (double)hv[i].y);
    return GOPF_OK;
}

// half spectrum (host) -> real host field (unnormalised inverse)
template <typename R>
int backward_real(gopf_ctx *ctx, void *dbuf, const std::vector<std::complex<double>> &half, std::vector<double> &out)
{
    typedef typename VecOf<R>::type V;
    const Geom &g = ctx->g;
    std::vector<V> hv(g.C);
    for (long long i = 0; i < g.C; ++i) {
        hv[i].x = (R)half[i].real();
        hv[i].y = (R)half[i].imag();
    }
    int rc;
    if ((rc = ck(ctx, cudaMemcpyAsync(dbuf, hv.data(), sizeof(V) * g.C, cudaMemcpyHostToDevice, ctx->stream), "H2D")))
        return rc;
    if (g.Z > 1 && (rc = ck(ctx, launch_spass<R>(pbase<R>(ctx, true, PM_INV, dbuf), ctx->LBz, ctx->stream), "z pass")))
        return rc;
    if ((rc = ck(ctx, launch_cpass<R>(pbase<R>(ctx, false, PM_INV, dbuf), ctx->LBy, ctx->stream), "y pass"))) return rc;
    XPassArgs<R> xa = xbase<R>(ctx);
    xa.in_mode = XIN_SPECTRAL;
    xa.in = (const V *)dbuf;
    xa.rout = (R *)ctx->d_real;
    if ((rc = ck(ctx, launch_xpass<R>(xa, ctx->LBx, ctx->stream), "x pass"))) return rc;
    std::vector<R> hr(g.N);
    if ((rc = ck(ctx, cudaMemcpyAsync(hr.data(), ctx->d_real, sizeof(R) * g.N, cudaMemcpyDeviceToHost, ctx->stream),
                 "D2H")))
        return rc;
    if ((rc = ck(ctx, cudaStreamSynchronize(ctx->stream), "sync"))) return rc;
    out.resize(g.N);
    for (long long i = 0; i < g.N; ++i) out[i] = (double)hr[i];
    return GOPF_OK;
}

// spectral index of (z, y, x) for x <= H
inline long long sidx(const Geom &g, long long z, long long y, long long x) { return z * g.S + x * g.Y + y; }

template <typename R> int fft_impl(gopf_ctx *ctx, int sign, double *data)
{
    const Geom &g = ctx->g;
    void *dbuf = nullptr;
    int rc = ck(ctx, gopf_malloc(&dbuf, sizeof(typename VecOf<R>::type) * g.C), "cudaMalloc");
    if (rc) return rc;
    std::complex<double> *x = reinterpret_cast<std::complex<double> *>(data);
    std::vector<double> a(g.N), b(g.N);
    if (sign < 0) {
        for (long long i = 0; i < g.N; ++i) { a[i] = x[i].real(); b[i] = x[i].imag(); }
        std::vector<std::complex<double>> ha, hb;
        if (!(rc = forward_real<R>(ctx, dbuf, a, ha)) && !(rc = forward_real<R>(ctx, dbuf, b, hb))) {
            const std::complex<double> I(0.0, 1.0);
            for (long long z = 0; z < g.Z; ++z)
                for (long long y = 0; y < g.Y; ++y)
                    for (long long c = 0; c < g.X; ++c) {
                        std::complex<double> A, B;
                        if (c <= g.H) {
                            A = ha[sidx(g, z, y, c)];
                            B = hb[sidx(g, z, y, c)];
                        } else {
                            const long long s = sidx(g, (g.Z - z) % g.Z, (g.Y - y) % g.Y, g.X - c);
                            A = std::conj(ha[s]);
                            B = std::conj(hb[s]);
                        }
                        x[(z * g.Y + y) * g.X + c] = A + I * B;
                    }
        }
    } else {
        std::vector<std::complex<double>> ha(g.C), hb(g.C);
        const std::complex<double> I(0.0, 1.0);
        for (long long z = 0; z < g.Z; ++z)
            for (long long y = 0; y < g.Y; ++y)
                for (long long c = 0; c <= g.H; ++c) {
                    const std::complex<double> X = x[(z * g.Y + y) * g.X + c];
                    const long long cz = (g.Z - z) % g.Z, cy = (g.Y - y) % g.Y, cc = (g.X - c) % g.X;
                    const std::complex<double> Xm = std::conj(x[(cz * g.Y + cy) * g.X + cc]);
                    ha[sidx(g, z, y, c)] = 0.5 * (X + Xm);
                    hb[sidx(g, z, y, c)] = (X - Xm) / (2.0 * I);
                }
        if (!(rc = backward_real<R>(ctx, dbuf, ha, a)) && !(rc = backward_real<R>(ctx, dbuf, hb, b))) {
            for (long long i = 0; i < g.N; ++i) x[i] = std::complex<double>(a[i], b[i]);
        }
    }
    cudaFree(dbuf);
    return rc;
}

} // namespace

extern "C" int gopf_fft(gopf_ctx *ctx, int sign, double *data, size_t n)
{
    if (!ctx || !data) return gopf_fail(ctx, GOPF_ERR_ARG, "null argument");
    if (sign != -1 && sign != 1) return gopf_fail(ctx, GOPF_ERR_ARG, "sign must be -1 or +1");
    if ((long long)n != ctx->g.N) return gopf_fail(ctx, GOPF_ERR_ARG, "Inconsistent domain size and number of grid points");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return gopf_fail(ctx, GOPF_ERR_CUDA, cudaGetErrorString(e));
    return (ctx->prec == GOPF_FP32) ? fft_impl<float>(ctx, sign, data) : fft_impl<double>(ctx, sign, data);
}
