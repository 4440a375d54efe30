// gopf_batch.cu -- many independent instances stepped by shared launches.
//
// The parameter-sweep workflow of gopf (one FieldDB per swept run, README.md:21-33)
// steps every instance separately.  A batch takes N contexts of arbitrary
// (2D) sizes, each with its own equation, coefficients and dt, and steps them
// together: one persistent x-pass launch and one persistent fused y-pass
// launch per step walk a work list of (instance, tile) items ordered largest
// first, so small instances no longer leave the GPU idle and the launch
// overhead is paid once per pass instead of once per instance.  The step
// (three launches) is captured in a CUDA graph and replayed.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "gopf_ctx.h"
#include "gopf_kernels_impl.cuh"

namespace gopf {

template <typename R> struct BatchInst {
    XPassArgs<R> xa;
    PassArgs<R> pa;
    int lbx, lby;
    long long herm_off; // first element of this instance in the projection index space
};

template <typename R, int LB> __device__ __forceinline__ void batch_x_item(const XPassArgs<R> &a, int ty)
{
    xpass_tile<R, LB, 16>(a, ty, 0);
}

template <typename R>
__global__ void __launch_bounds__(256, (sizeof(R) == 4 ? 3 : 2))
    k_batch_xpass(const BatchInst<R> *__restrict__ inst, const int2 *__restrict__ items, int nitems)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        __syncthreads(); // shared memory of the previous item is free
        const int2 it = items[w];
        const BatchInst<R> &b = inst[it.x];
        if (b.xa.ngrp_out == 0) continue;
        if (b.lbx == 16) batch_x_item<R, 16>(b.xa, it.y);
        else if (b.lbx == 8) batch_x_item<R, 8>(b.xa, it.y);
        else batch_x_item<R, 4>(b.xa, it.y);
    }
}

template <typename R>
__global__ void __launch_bounds__(256, (sizeof(R) == 4 ? 3 : 2))
    k_batch_ypass(const BatchInst<R> *__restrict__ inst, const int2 *__restrict__ items, int nitems)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        __syncthreads();
        const int2 it = items[w];
        const BatchInst<R> &b = inst[it.x];
        if (b.lby == 16) pass_tile<R, 16, 16, true, false>(b.pa, it.y, 0);
        else if (b.lby == 8) pass_tile<R, 8, 16, true, false>(b.pa, it.y, 0);
        else pass_tile<R, 4, 16, true, false>(b.pa, it.y, 0);
    }
}

// Hermitian projection of the kx = 0 and kx = X/2 lines of every instance (2D)
template <typename R>
__global__ void k_batch_herm(const BatchInst<R> *__restrict__ inst, int ninst, long long total)
{
    typedef typename VecOf<R>::type V;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = ninst - 1;
        while (lo < hi) { // last instance with herm_off <= idx
            const int mid = (lo + hi + 1) >> 1;
            if (inst[mid].herm_off <= idx) lo = mid;
            else hi = mid - 1;
        }
        const BatchInst<R> &b = inst[lo];
        const Geom &g = b.pa.g;
        const long long r = idx - b.herm_off;
        const int plane = (int)(r / g.Y);
        const long long y = r - (long long)plane * g.Y;
        const long long yp = (g.Y - y) % g.Y;
        if (y > yp) continue;
        const long long kx = plane ? g.H : 0;
        V *c = b.pa.state;
        const long long ia = kx * g.Y + y, ib = kx * g.Y + yp;
        const V a = c[ia], bb = c[ib];
        V m;
        m.x = (a.x + bb.x) * (R)0.5;
        m.y = (a.y - bb.y) * (R)0.5;
        c[ia] = m;
        m.y = -m.y;
        c[ib] = m;
    }
}

} // namespace gopf

using namespace gopf;

struct gopf_batch {
    std::vector<gopf_ctx *> ctx;
    int device = 0;
    int prec = GOPF_FP32;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    void *d_inst = nullptr;
    int2 *d_xitems = nullptr, *d_yitems = nullptr;
    int nx = 0, ny = 0;
    long long herm_total = 0;
    int smem_x = 0, smem_y = 0;
    int grid_x = 0, grid_y = 0;
    cudaGraphExec_t g1 = nullptr, gK = nullptr;
    int K = 16;
    std::string err;
};

static int bfail(gopf_batch *b, int code, const std::string &m)
{
    if (b) b->err = m;
    return code;
}

#define BCK(call)                                                                                                      \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess) return bfail(b, GOPF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));    \
    } while (0)

template <typename R> static int batch_build(gopf_batch *b)
{
    typedef typename VecOf<R>::type V;
    std::vector<BatchInst<R>> inst(b->ctx.size());
    std::vector<int2> xi, yi;
    std::vector<std::pair<int, int2>> xs, ys; // (cost, item)
    long long hoff = 0;
    const int vb = sizeof(V);
    for (size_t i = 0; i < b->ctx.size(); ++i) {
        gopf_ctx *c = b->ctx[i];
        BatchInst<R> &bi = inst[i];
        memset(&bi, 0, sizeof(bi));
        const Geom &g = c->g;
        const int G = c->ngroups;
        XPassArgs<R> &xa = bi.xa;
        xa.g = g;
        xa.planH = c->planH;
        xa.twX = (const V *)c->d_twX;
        xa.in_mode = XIN_SPECTRAL;
        xa.in = (const V *)c->d_T;
        xa.out[0] = (V *)c->d_T;
        for (int q = 1; q < GOPF_MAX_GROUPS; ++q) xa.out[q] = (V *)c->d_U[q];
        xa.ngrp_out = G;
        xa.pw = c->pw;
        PassArgs<R> &pa = bi.pa;
        pa.g = g;
        pa.plan = c->planY;
        pa.tw = (const V *)c->d_twY;
        pa.mode = PM_FUSED;
        const int nb = std::max(G, 1);
        for (int q = 0; q < nb; ++q) pa.buf[q] = q == 0 ? (V *)c->d_T : (V *)c->d_U[q];
        pa.nbuf = nb;
        pa.state = (V *)c->d_state;
        pa.tout = (V *)c->d_T;
        pa.upd = c->upd;
        pa.upd.dt = c->dt;
        pa.upd.invN = 1.0 / (double)g.N;
        bi.lbx = c->LBx;
        bi.lby = c->LBy;
        bi.herm_off = hoff;
        hoff += 2LL * g.Y;
        const int ntx = (g.Y + c->LBx - 1) / c->LBx;
        for (int t = 0; t < ntx; ++t) xs.push_back({g.H * c->LBx, make_int2((int)i, t)});
        const int nty = (int)((g.KX + c->LBy - 1) / c->LBy);
        for (int t = 0; t < nty; ++t) ys.push_back({g.Y * c->LBy, make_int2((int)i, t)});
        b->smem_x = std::max(b->smem_x, xpass_smem_bytes(g, c->LBx, vb));
        b->smem_y = std::max(b->smem_y, cpass_smem_bytes(g, g.Y, c->LBy, nb, vb) + (c->LBy + g.Y) * (int)sizeof(R));
    }
    auto bycost = [](const std::pair<int, int2> &a, const std::pair<int, int2> &c) { return a.first > c.first; };
    std::stable_sort(xs.begin(), xs.end(), bycost);
    std::stable_sort(ys.begin(), ys.end(), bycost);
    for (auto &p : xs) xi.push_back(p.second);
    for (auto &p : ys) yi.push_back(p.second);
    b->nx = (int)xi.size();
    b->ny = (int)yi.size();
    b->herm_total = hoff;
    BCK(gopf_malloc(&b->d_inst, sizeof(BatchInst<R>) * inst.size()));
    BCK(cudaMemcpy(b->d_inst, inst.data(), sizeof(BatchInst<R>) * inst.size(), cudaMemcpyHostToDevice));
    BCK(gopf_malloc(&b->d_xitems, sizeof(int2) * std::max(1, b->nx)));
    BCK(gopf_malloc(&b->d_yitems, sizeof(int2) * std::max(1, b->ny)));
    BCK(cudaMemcpy(b->d_xitems, xi.data(), sizeof(int2) * b->nx, cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->d_yitems, yi.data(), sizeof(int2) * b->ny, cudaMemcpyHostToDevice));
    BCK(cudaFuncSetAttribute(k_batch_xpass<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, b->smem_x));
    BCK(cudaFuncSetAttribute(k_batch_ypass<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, b->smem_y));
    int nsm = 0, bx = 0, by = 0;
    BCK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, b->device));
    BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bx, k_batch_xpass<R>, 256, b->smem_x));
    BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&by, k_batch_ypass<R>, 256, b->smem_y));
    b->grid_x = std::max(1, std::min(b->nx, nsm * std::max(bx, 1)));
    b->grid_y = std::max(1, std::min(b->ny, nsm * std::max(by, 1)));
    return GOPF_OK;
}

template <typename R> static cudaError_t batch_enqueue(gopf_batch *b)
{
    const BatchInst<R> *inst = (const BatchInst<R> *)b->d_inst;
    k_batch_xpass<R><<<b->grid_x, 256, b->smem_x, b->stream>>>(inst, b->d_xitems, b->nx);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_batch_ypass<R><<<b->grid_y, 256, b->smem_y, b->stream>>>(inst, b->d_yitems, b->ny);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const unsigned hb = (unsigned)std::min<long long>((b->herm_total + 255) / 256, 152 * 4);
    k_batch_herm<R><<<hb, 256, 0, b->stream>>>(inst, (int)b->ctx.size(), b->herm_total);
    return cudaGetLastError();
}

static cudaError_t batch_enqueue_any(gopf_batch *b, int n)
{
    for (int i = 0; i < n; ++i) {
        cudaError_t e = (b->prec == GOPF_FP32) ? batch_enqueue<float>(b) : batch_enqueue<double>(b);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

static int batch_capture(gopf_batch *b, int n, cudaGraphExec_t *exec)
{
    cudaGraph_t graph;
    BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = batch_enqueue_any(b, n);
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &graph);
    if (e != cudaSuccess) return bfail(b, GOPF_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
    if (e2 != cudaSuccess) return bfail(b, GOPF_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e2));
    e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return bfail(b, GOPF_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
    return GOPF_OK;
}

extern "C" int gopf_batch_create(gopf_ctx *const *ctxs, int n, gopf_batch **out)
{
    if (!out || !ctxs || n < 1) return GOPF_ERR_ARG;
    *out = nullptr;
    gopf_batch *b = new gopf_batch();
    *out = b;
    for (int i = 0; i < n; ++i) {
        gopf_ctx *c = ctxs[i];
        if (!c) return bfail(b, GOPF_ERR_ARG, "null context");
        if (i == 0) {
            b->device = c->device;
            b->prec = c->prec;
        }
        if (c->device != b->device || c->prec != b->prec)
            return bfail(b, GOPF_ERR_ARG, "all contexts of a batch share one device and precision");
        if (c->device < 0) return bfail(b, GOPF_ERR_STATE, "host-only context");
        if (c->ndim != 2) return bfail(b, GOPF_ERR_UNSUPPORTED, "batches step 2D contexts");
        if (!c->initialised || !(c->dt > 0.0) || !c->state_valid)
            return bfail(b, GOPF_ERR_STATE, "every context needs its model, stepper and field set");
        if (c->stepper != GOPF_STEPPER_EULER || c->has_elastic || c->has_volcons || c->noise.kind || c->upd.filt || c->upd.nxs)
            return bfail(b, GOPF_ERR_UNSUPPORTED, "batches step Euler models without user-defined terms, noise or filters");
        if (c->multi) return bfail(b, GOPF_ERR_UNSUPPORTED, "batches step single-field models");
        b->ctx.push_back(c);
    }
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return bfail(b, GOPF_ERR_CUDA, cudaGetErrorString(e));
    e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bfail(b, GOPF_ERR_CUDA, cudaGetErrorString(e));
    b->stream = b->own_stream;
    // the contexts' own streams may still hold work
    for (gopf_ctx *c : b->ctx) cudaStreamSynchronize(c->stream);
    return (b->prec == GOPF_FP32) ? batch_build<float>(b) : batch_build<double>(b);
}

extern "C" int gopf_batch_destroy(gopf_batch *b)
{
    if (!b) return GOPF_ERR_ARG;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->g1) cudaGraphExecDestroy(b->g1);
    if (b->gK) cudaGraphExecDestroy(b->gK);
    void *ptrs[] = {b->d_inst, b->d_xitems, b->d_yitems};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    delete b;
    return GOPF_OK;
}

extern "C" const char *gopf_batch_last_error(const gopf_batch *b) { return b ? b->err.c_str() : "null batch"; }

extern "C" int gopf_batch_set_stream(gopf_batch *b, void *s)
{
    if (!b) return GOPF_ERR_ARG;
    if (b->g1) cudaGraphExecDestroy(b->g1);
    if (b->gK) cudaGraphExecDestroy(b->gK);
    b->g1 = b->gK = nullptr;
    b->stream = s ? (cudaStream_t)s : b->own_stream;
    return GOPF_OK;
}

extern "C" int gopf_batch_step(gopf_batch *b, long long nsteps)
{
    if (!b || nsteps < 0) return GOPF_ERR_ARG;
    BCK(cudaSetDevice(b->device));
    int rc;
    if (!b->g1 && (rc = batch_capture(b, 1, &b->g1))) return rc;
    if (nsteps >= b->K && !b->gK && (rc = batch_capture(b, b->K, &b->gK))) return rc;
    long long left = nsteps;
    while (left >= b->K) {
        BCK(cudaGraphLaunch(b->gK, b->stream));
        left -= b->K;
    }
    while (left-- > 0) BCK(cudaGraphLaunch(b->g1, b->stream));
    for (gopf_ctx *c : b->ctx) c->step += nsteps;
    // later calls on the contexts' own streams must see the batch's work
    BCK(cudaStreamSynchronize(b->stream));
    return GOPF_OK;
}

extern "C" int gopf_batch_kernels_per_step(gopf_batch *b, int *n)
{
    if (!b || !n) return GOPF_ERR_ARG;
    *n = 3;
    return GOPF_OK;
}
