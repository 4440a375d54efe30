// gopf_noalloc.cu -- a field reduction that allocates no memory.
//
// gopf_reduce works through a context, whose constructor allocates device
// buffers (among them the block partial sums of the reduction).  Some callers
// cannot allocate device memory at the point where they want a reduction: a
// host integration that hands the library memory it manages itself, code
// running under a memory budget enforced outside the CUDA allocator, or a
// process whose allocator must not be touched between a pool's set-up and its
// tear-down.  gopf_reduce_noalloc serves them: it reduces a real FP64 field the
// caller already holds in device memory, and its only scratch is the
// file-scope device array below.
//
// The scratch is g_noalloc_scratch: (GOPF_NOALLOC_MAX_BLOCKS + 1) rows of 8
// doubles, about 1 MiB.  Every GPU that loads the library holds it until the
// process exits.  One row holds the partial sums of each block of 4096
// elements; the last row holds the final result.  So a call accepts at most
// GOPF_NOALLOC_MAX_BLOCKS * 4096 = 67,108,864 elements.
//
// Every call shares the array.  Each block overwrites its whole row and the
// final row is written in full, so nothing has to start at zero.  Calls that
// overlap on the GPU (different streams, or different host threads without
// ordering) race on the array and must be serialised by the caller.
//
// Host code cannot use the array's name as a device address.  Every call looks
// the address up with cudaGetSymbolAddress while the caller's device (and
// context) is current, so a device reset or another context made current on
// the device never leaves a stale address behind.  The first call on a device
// also loads the library's device code there; make that first call before any
// stream capture.  The call is synchronous: it waits on its stream until the
// result is on the host.
#include <cmath>
#include <string>

#include <cuda_runtime.h>

#include "../../include/gopf_gpu.h"

#define GOPF_NOALLOC_ELEMS_PER_BLOCK 4096
#define GOPF_NOALLOC_SLOTS 8

static __device__ __align__(256) double g_noalloc_scratch[(GOPF_NOALLOC_MAX_BLOCKS + 1) * GOPF_NOALLOC_SLOTS];

namespace {

__device__ __forceinline__ void neumaier_add(double &sum, double &err, double v)
{
    const double t = sum + v;
    err += (fabs(sum) >= fabs(v)) ? (sum - t) + v : (v - t) + sum;
    sum = t;
}

// slots: 0 sum, 1 sum of squares, 2 min, 3 max, 4 non-finite count (as gopf_reduce)
__global__ void k_noalloc_partials(const double *__restrict__ x, long long n, double *__restrict__ rows)
{
    const long long b0 = (long long)blockIdx.x * GOPF_NOALLOC_ELEMS_PER_BLOCK;
    const long long b1 = (b0 + GOPF_NOALLOC_ELEMS_PER_BLOCK < n) ? b0 + GOPF_NOALLOC_ELEMS_PER_BLOCK : n;
    // Neumaier-compensated sums per thread, folded with their error terms at each combination
    double s = 0.0, sc = 0.0, q = 0.0, qc = 0.0, mn = INFINITY, mx = -INFINITY, nf = 0.0;
    for (long long i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
        const double v = x[i];
        neumaier_add(s, sc, v);
        neumaier_add(q, qc, v * v);
        mn = fmin(mn, v);
        mx = fmax(mx, v);
        nf += isfinite(v) ? 0.0 : 1.0;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double so = __shfl_xor_sync(0xffffffffu, s, o), sco = __shfl_xor_sync(0xffffffffu, sc, o);
        const double qo = __shfl_xor_sync(0xffffffffu, q, o), qco = __shfl_xor_sync(0xffffffffu, qc, o);
        sc += sco;
        neumaier_add(s, sc, so);
        qc += qco;
        neumaier_add(q, qc, qo);
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        nf += __shfl_xor_sync(0xffffffffu, nf, o);
    }
    __shared__ double sh[32][5];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        sh[warp][0] = s + sc;
        sh[warp][1] = q + qc;
        sh[warp][2] = mn;
        sh[warp][3] = mx;
        sh[warp][4] = nf;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) / 32;
        double bs = sh[0][0], bsc = 0.0, bq = sh[0][1], bqc = 0.0;
        for (int w = 1; w < nw; ++w) {
            neumaier_add(bs, bsc, sh[w][0]);
            neumaier_add(bq, bqc, sh[w][1]);
            sh[0][2] = fmin(sh[0][2], sh[w][2]);
            sh[0][3] = fmax(sh[0][3], sh[w][3]);
            sh[0][4] += sh[w][4];
        }
        double *row = rows + (long long)blockIdx.x * GOPF_NOALLOC_SLOTS;
        row[0] = bs + bsc;
        row[1] = bq + bqc;
        for (int k = 2; k < 5; ++k) row[k] = sh[0][k];
        for (int k = 5; k < GOPF_NOALLOC_SLOTS; ++k) row[k] = 0.0;
    }
}

// Neumaier sums of the block rows into the result row (one thread)
__global__ void k_noalloc_finish(const double *__restrict__ rows, int nblocks, double *__restrict__ res)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0, sc = 0.0, q = 0.0, qc = 0.0, mn = INFINITY, mx = -INFINITY, nf = 0.0;
    for (int b = 0; b < nblocks; ++b) {
        const double *row = rows + (long long)b * GOPF_NOALLOC_SLOTS;
        double v = row[0], t = s + v;
        sc += (fabs(s) >= fabs(v)) ? (s - t) + v : (v - t) + s;
        s = t;
        v = row[1];
        t = q + v;
        qc += (fabs(q) >= fabs(v)) ? (q - t) + v : (v - t) + q;
        q = t;
        mn = fmin(mn, row[2]);
        mx = fmax(mx, row[3]);
        nf += row[4];
    }
    res[0] = s + sc;
    res[1] = q + qc;
    res[2] = mn;
    res[3] = mx;
    res[4] = nf;
    for (int k = 5; k < GOPF_NOALLOC_SLOTS; ++k) res[k] = 0.0;
}

thread_local std::string g_err;

int fail(int code, const std::string &m)
{
    g_err = m;
    return code;
}

// Device address of the scratch array in the current device's current context.  Looked up on
// every call: the lookup allocates nothing, and an address cached across a device reset or a
// change of context would point at memory that no longer holds the array.
int scratch_address(double **out)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
        return fail(GOPF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    *out = (double *)p;
    return GOPF_OK;
}

} // namespace

extern "C" int gopf_reduce_noalloc(const double *field, size_t n, double *out, void *stream)
{
    if (!field || !out) return fail(GOPF_ERR_ARG, "null argument");
    if (n == 0) return fail(GOPF_ERR_ARG, "empty field");
    const unsigned long long maxn = (unsigned long long)GOPF_NOALLOC_MAX_BLOCKS * GOPF_NOALLOC_ELEMS_PER_BLOCK;
    if ((unsigned long long)n > maxn)
        return fail(GOPF_ERR_ARG, "field of " + std::to_string((unsigned long long)n) +
                                      " elements exceeds the no-allocation limit of " + std::to_string(maxn));
    double *scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const int nblocks = (int)((n + GOPF_NOALLOC_ELEMS_PER_BLOCK - 1) / GOPF_NOALLOC_ELEMS_PER_BLOCK);
    double *result = scratch + (long long)GOPF_NOALLOC_MAX_BLOCKS * GOPF_NOALLOC_SLOTS;
    k_noalloc_partials<<<nblocks, 256, 0, s>>>(field, (long long)n, scratch);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        k_noalloc_finish<<<1, 32, 0, s>>>(scratch, nblocks, result);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, result, 5 * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(GOPF_ERR_CUDA, std::string("reduce: ") + cudaGetErrorString(e));
    return GOPF_OK;
}

extern "C" const char *gopf_noalloc_last_error(void) { return g_err.c_str(); }
