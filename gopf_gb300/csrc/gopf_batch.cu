// gopf_batch.cu -- many independent instances stepped by shared launches.
//
// The parameter-sweep workflow of gopf (one FieldDB per swept run, README.md:21-33)
// steps every instance separately.  A batch takes N contexts of arbitrary
// (2D) sizes, each with its own equation, coefficients and dt, and steps them
// together.  Instances are grouped into size classes; per step each class
// present gets one x-pass launch and one fused y-pass launch over its
// (instance, tile) items, ordered largest first, so small instances no longer
// leave the GPU idle and the launch overhead is paid once per class instead of
// once per instance.  When the classes of both passes cover the same instances,
// each class is a chain on its own branch of the captured graph: x pass, y pass
// and the Hermitian projection of its own instances, for every step of the
// graph, with one fork and one join per graph (3 launches per class and step),
// so a class never waits for another between steps.  Otherwise the classes of
// a pass run as parallel branches and one projection of every instance ends
// each step (2 x classes + 1 launches).
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "fastline.cuh"
#include "gopf_ctx.h"
#include "gopf_kernels_impl.cuh"

namespace gopf {

template <typename R> struct BatchInst {
    XPassArgs<R> xa;
    PassArgs<R> pa;
    int lbx, lby;
};

template <typename R, int LB> __device__ __forceinline__ void batch_x_item(const XPassArgs<R> &a, int ty)
{
    xpass_tile<R, LB, 16>(a, ty, 0);
}

// Copy an instance's pass arguments into shared memory (as 8-byte words) for the item: the tile
// code then reads them there instead of the compiler staging the whole struct in local memory.
template <typename T> __device__ __forceinline__ void stage_args(T *dst, const T *src)
{
    static_assert(sizeof(T) % 8 == 0, "pass arguments are 8-byte aligned");
    const unsigned long long *s = reinterpret_cast<const unsigned long long *>(src);
    unsigned long long *d = reinterpret_cast<unsigned long long *>(dst);
    for (int k = threadIdx.x; k < (int)(sizeof(T) / 8); k += blockDim.x) d[k] = s[k];
}

template <typename R>
__global__ void __launch_bounds__(256, (sizeof(R) == 4 ? 3 : 2))
    k_batch_xpass(const BatchInst<R> *__restrict__ inst, const int2 *__restrict__ items, int nitems)
{
    __shared__ __align__(16) XPassArgs<R> s_a;
    __shared__ int s_lb;
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        __syncthreads(); // shared memory of the previous item is free
        const int2 it = items[w];
        stage_args(&s_a, &inst[it.x].xa);
        if (threadIdx.x == 0) s_lb = inst[it.x].lbx;
        __syncthreads();
        if (s_a.ngrp_out == 0) continue;
        if (s_lb == 16) batch_x_item<R, 16>(s_a, it.y);
        else if (s_lb == 8) batch_x_item<R, 8>(s_a, it.y);
        else batch_x_item<R, 4>(s_a, it.y);
    }
}

template <typename R>
__global__ void __launch_bounds__(256, (sizeof(R) == 4 ? 3 : 2))
    k_batch_ypass(const BatchInst<R> *__restrict__ inst, const int2 *__restrict__ items, int nitems)
{
    __shared__ __align__(16) PassArgs<R> s_a;
    __shared__ int s_lb;
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        __syncthreads();
        const int2 it = items[w];
        stage_args(&s_a, &inst[it.x].pa);
        if (threadIdx.x == 0) s_lb = inst[it.x].lby;
        __syncthreads();
        if (s_lb == 16) pass_tile<R, 16, 16, true, false>(s_a, it.y, 0);
        else if (s_lb == 8) pass_tile<R, 8, 16, true, false>(s_a, it.y, 0);
        else pass_tile<R, 4, 16, true, false>(s_a, it.y, 0);
    }
}

// Size classes of the sweep's sides (128 ... 1024) in FP32: one kernel per (length, tile width)
// with a compile-time plan, every stage inlined with its radix, stride and twiddle step known.
// One block per item (a persistent loop around the inlined stages makes the compiler spill
// kilobytes per thread); each class is its own launch with its own register allocation, and the
// classes of a pass run as parallel branches of the step's graph.  The (length, tile width)
// pairs are those lb_for gives the contexts; any other instance goes through k_batch_xpass /
// k_batch_ypass.
template <int LB, int H>
__global__ void __launch_bounds__(256, 3) k_batch_x_ct(const BatchInst<float> *__restrict__ inst,
                                                      const int2 *__restrict__ items, int nitems)
{
    const int2 it = items[blockIdx.x];
    const XPassArgs<float> &a = inst[it.x].xa;
    if (a.ngrp_out == 0) return;
    xpass_tile<float, LB, 16, false, H>(a, it.y, 0);
}

template <int LB, int N>
__global__ void __launch_bounds__(256, 3) k_batch_y_ct(const BatchInst<float> *__restrict__ inst,
                                                      const int2 *__restrict__ items, int nitems)
{
    const int2 it = items[blockIdx.x];
    pass_tile<float, LB, 16, true, false, N>(inst[it.x].pa, it.y, 0);
}

// Sides 256 ... 1024 in FP32 go further, to the register-resident line engine (fastline.cuh):
// one block per tile of rows (x) or lines (y).
template <int L>
__global__ void __launch_bounds__(fl::Geo<L>::NT, 3) k_batch_xl(const BatchInst<float> *__restrict__ inst,
                                                               const int2 *__restrict__ items, int nitems)
{
    // the instance's arguments in shared memory: read from global memory, the fields the tile
    // code needs would be held in registers for its whole length (and spill)
    __shared__ __align__(16) XPassArgs<float> s_a;
    const int2 it = items[blockIdx.x];
    stage_args(&s_a, &inst[it.x].xa);
    __syncthreads();
    if (s_a.ngrp_out == 0) return;
    fl::xline_tile<L>(s_a, it.y, 0);
}

// Instances with one dense polynomial group (Cahn-Hilliard): one line in registers, four blocks per SM.
template <int L>
__global__ void __launch_bounds__(fl::Geo<L>::NT, 4) k_batch_xl1(const BatchInst<float> *__restrict__ inst,
                                                                const int2 *__restrict__ items, int nitems)
{
    __shared__ __align__(16) XPassArgs<float> s_a;
    const int2 it = items[blockIdx.x];
    stage_args(&s_a, &inst[it.x].xa);
    __syncthreads();
    fl::xline_tile<L, true>(s_a, it.y, 0);
}

template <int L, int NG>
__global__ void __launch_bounds__(fl::Geo<L>::NT, 3) k_batch_yl(const BatchInst<float> *__restrict__ inst,
                                                               const int2 *__restrict__ items, int nitems)
{
    const int2 it = items[blockIdx.x];
    fl::yline_tile<L, NG>(inst[it.x].pa, it.y);
}

// Classes: 0 any size (runtime plan); 1 .. 6 compile-time plans (x by H, y by the line length);
// 11 .. 15 the line engine for sides FL_L (y: 11 .. 15 one group, 21 .. 25 two groups; x: 31 .. 35
// for instances with one dense polynomial group).
constexpr int NCLASS = 36;
constexpr int XCLS_H[7] = {0, 64, 128, 192, 256, 384, 512}, XCLS_LB[7] = {0, 16, 16, 16, 16, 8, 8};
constexpr int YCLS_N[7] = {0, 128, 256, 384, 512, 768, 1024}, YCLS_LB[7] = {0, 16, 16, 8, 8, 4, 4};
constexpr int FL_L[5] = {256, 384, 512, 768, 1024};
constexpr int FL_LPB[5] = {fl::Geo<256>::LPB, fl::Geo<384>::LPB, fl::Geo<512>::LPB, fl::Geo<768>::LPB,
                           fl::Geo<1024>::LPB};
constexpr int FL_NT[5] = {fl::Geo<256>::NT, fl::Geo<384>::NT, fl::Geo<512>::NT, fl::Geo<768>::NT, fl::Geo<1024>::NT};
constexpr int FL_XSMEM[5] = {fl::xline_smem_bytes<256>(), fl::xline_smem_bytes<384>(), fl::xline_smem_bytes<512>(),
                             fl::xline_smem_bytes<768>(), fl::xline_smem_bytes<1024>()};
constexpr int FL_YSMEM[5] = {fl::yline_smem_bytes<256>(), fl::yline_smem_bytes<384>(), fl::yline_smem_bytes<512>(),
                             fl::yline_smem_bytes<768>(), fl::yline_smem_bytes<1024>()};

template <typename R> static const void *x_kernel(int cls)
{
    if constexpr (sizeof(R) == 4) {
        switch (cls) {
        case 1: return (const void *)k_batch_x_ct<16, 64>;
        case 2: return (const void *)k_batch_x_ct<16, 128>;
        case 3: return (const void *)k_batch_x_ct<16, 192>;
        case 4: return (const void *)k_batch_x_ct<16, 256>;
        case 5: return (const void *)k_batch_x_ct<8, 384>;
        case 6: return (const void *)k_batch_x_ct<8, 512>;
        case 11: return (const void *)k_batch_xl<256>;
        case 12: return (const void *)k_batch_xl<384>;
        case 13: return (const void *)k_batch_xl<512>;
        case 14: return (const void *)k_batch_xl<768>;
        case 15: return (const void *)k_batch_xl<1024>;
        case 31: return (const void *)k_batch_xl1<256>;
        case 32: return (const void *)k_batch_xl1<384>;
        case 33: return (const void *)k_batch_xl1<512>;
        case 34: return (const void *)k_batch_xl1<768>;
        case 35: return (const void *)k_batch_xl1<1024>;
        default: break;
        }
    }
    return (const void *)k_batch_xpass<R>;
}

template <typename R> static const void *y_kernel(int cls)
{
    if constexpr (sizeof(R) == 4) {
        switch (cls) {
        case 1: return (const void *)k_batch_y_ct<16, 128>;
        case 2: return (const void *)k_batch_y_ct<16, 256>;
        case 3: return (const void *)k_batch_y_ct<8, 384>;
        case 4: return (const void *)k_batch_y_ct<8, 512>;
        case 5: return (const void *)k_batch_y_ct<4, 768>;
        case 6: return (const void *)k_batch_y_ct<4, 1024>;
        case 11: return (const void *)k_batch_yl<256, 1>;
        case 12: return (const void *)k_batch_yl<384, 1>;
        case 13: return (const void *)k_batch_yl<512, 1>;
        case 14: return (const void *)k_batch_yl<768, 1>;
        case 15: return (const void *)k_batch_yl<1024, 1>;
        case 21: return (const void *)k_batch_yl<256, 2>;
        case 22: return (const void *)k_batch_yl<384, 2>;
        case 23: return (const void *)k_batch_yl<512, 2>;
        case 24: return (const void *)k_batch_yl<768, 2>;
        case 25: return (const void *)k_batch_yl<1024, 2>;
        default: break;
        }
    }
    return (const void *)k_batch_ypass<R>;
}

// Hermitian projection of the kx = 0 and kx = X/2 lines of the instances hinst[0 .. n): element
// idx < total of the projection index space belongs to listed instance j, the last with
// hoff[j] <= idx (hoff: prefix sums of the instances' line lengths, 1 or 2 lines of Y each)
template <typename R>
__global__ void k_batch_herm(const BatchInst<R> *__restrict__ inst, const int *__restrict__ hinst,
                             const long long *__restrict__ hoff, int n, long long total)
{
    typedef typename VecOf<R>::type V;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (hoff[mid] <= idx) lo = mid;
            else hi = mid - 1;
        }
        const BatchInst<R> &b = inst[hinst[lo]];
        const Geom &g = b.pa.g;
        const long long r = idx - hoff[lo];
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

// one projection launch: the instances it covers and their offsets in its index space
struct BatchHerm {
    int *d_inst = nullptr;
    long long *d_off = nullptr;
    int n = 0;
    long long total = 0;
};

// one launch of a pass: the items of one size class
struct BatchLaunch {
    const void *fn = nullptr;
    int2 *d_items = nullptr;
    int nitems = 0;
    int grid = 0, smem = 0, threads = 256;
    std::vector<int> inst; // the instances it covers (sorted)
};

// How one instance's passes run: the kernel family of each pass (GOPF_BATCH_LINE: the register line
// engine, GOPF_BATCH_STOCKHAM_CT: compile-time Stockham plans, GOPF_BATCH_STOCKHAM: runtime plans,
// GOPF_BATCH_AUTO: the built-in preference in that order), and for the runtime plans the tile
// width (0: the context's) and the plan variant (gopf_make_plan).
struct BatchChoice {
    int xfam = GOPF_BATCH_AUTO, yfam = GOPF_BATCH_AUTO;
    int lbx = 0, lby = 0;
    int xplan = 0, yplan = 0;
};

struct gopf_batch {
    std::vector<gopf_ctx *> ctx;
    std::vector<BatchChoice> choice; // requested, per instance
    std::vector<BatchChoice> eff;    // in effect after the last build, per instance
    int device = 0;
    int prec = GOPF_FP32;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    void *d_inst = nullptr;
    std::vector<BatchLaunch> xl, yl; // the x and y passes, one launch per size class present
    // When the x and y classes cover the same instance sets (square instances), class i's y pass
    // depends only on class i's x pass: each class runs x then y on its own branch (chain[i] =
    // indices into xl, yl), with no pass-wide join.  Empty: two pass-wide phases.
    // Every step of a chain ends with the projection of its own instances (hchain[i]), so the
    // chains need no join between steps: a captured graph of n steps forks once, runs each chain's
    // n steps on its branch and joins once.  Without chains every step ends with hall.
    std::vector<std::pair<int, int>> chain;
    std::vector<BatchHerm> hchain;
    BatchHerm hall;
    std::vector<cudaStream_t> side;  // branch streams of a pass's launches
    std::vector<cudaEvent_t> ev;     // [0] fork, [1 ..] joins
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

// a runtime-plan tile width the generic batch kernels take for a transform of length n
// (256 threads hold lb * n / 16 butterfly inputs)
static bool batch_lb_ok(int lb, int n) { return (lb == 4 || lb == 8 || lb == 16) && lb * n <= 4096; }

template <typename R> static int batch_build(gopf_batch *b)
{
    typedef typename VecOf<R>::type V;
    std::vector<BatchInst<R>> inst(b->ctx.size());
    std::vector<std::pair<int, int2>> xs[NCLASS], ys[NCLASS]; // (cost, item) per size class
    int smem_x[NCLASS] = {0}, smem_y[NCLASS] = {0}, thr_x[NCLASS], thr_y[NCLASS];
    for (int k = 0; k < NCLASS; ++k) thr_x[k] = thr_y[k] = 256;
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
        int xc = 0, yc = 0, fx = -1, fy = -1;
        if (sizeof(R) == 4) {
            for (int k = 1; k < 7; ++k) {
                if (g.H == XCLS_H[k] && c->LBx == XCLS_LB[k] && !(g.X & 1)) xc = k;
                if (g.Y == YCLS_N[k] && c->LBy == YCLS_LB[k]) yc = k;
            }
            for (int k = 0; k < 5; ++k) {
                if (g.X == FL_L[k] && g.Y % (2 * FL_LPB[k]) == 0) fx = k;
                if (g.Y == FL_L[k] && nb <= 2 && c->upd.nimp <= 4) fy = k;
            }
        }
        // the requested families where they serve this instance, else the built-in preference
        const BatchChoice &ch = b->choice[i];
        BatchChoice &ef = b->eff[i];
        ef = BatchChoice();
        int xf = ch.xfam, yf = ch.yfam;
        if ((xf == GOPF_BATCH_LINE && fx < 0) || (xf == GOPF_BATCH_STOCKHAM_CT && xc == 0)) xf = GOPF_BATCH_AUTO;
        if ((yf == GOPF_BATCH_LINE && fy < 0) || (yf == GOPF_BATCH_STOCKHAM_CT && yc == 0)) yf = GOPF_BATCH_AUTO;
        if (xf == GOPF_BATCH_AUTO) xf = fx >= 0 ? GOPF_BATCH_LINE : xc > 0 ? GOPF_BATCH_STOCKHAM_CT : GOPF_BATCH_STOCKHAM;
        if (yf == GOPF_BATCH_AUTO) yf = fy >= 0 ? GOPF_BATCH_LINE : yc > 0 ? GOPF_BATCH_STOCKHAM_CT : GOPF_BATCH_STOCKHAM;
        if (xf != GOPF_BATCH_LINE) fx = -1;
        if (yf != GOPF_BATCH_LINE) fy = -1;
        if (xf == GOPF_BATCH_STOCKHAM) {
            xc = 0;
            const bool odd = (g.X & 1) != 0; // odd X: row pairs through length-X transforms
            if (batch_lb_ok(ch.lbx, odd ? g.KX : g.H)) bi.lbx = ch.lbx;
            if (ch.xplan && gopf_make_plan(odd ? g.X : g.H, odd ? 1 : 2, ch.xplan, xa.planH)) ef.xplan = ch.xplan;
            else xa.planH = c->planH;
        }
        if (yf == GOPF_BATCH_STOCKHAM) {
            yc = 0;
            if (batch_lb_ok(ch.lby, g.Y)) bi.lby = ch.lby;
            if (ch.yplan && gopf_make_plan(g.Y, 1, ch.yplan, pa.plan)) ef.yplan = ch.yplan;
            else pa.plan = c->planY;
        }
        ef.xfam = xf;
        ef.yfam = yf;
        ef.lbx = (xf == GOPF_BATCH_STOCKHAM) ? bi.lbx : 0;
        ef.lby = (yf == GOPF_BATCH_STOCKHAM) ? bi.lby : 0;
        if (fx >= 0) { // line engine: tiles of 2 LPB rows (31 ..: one dense polynomial group)
            const bool one = (G == 1 && c->pw.deg[0] >= 0 && c->pw.deg[0] <= 6);
            xc = (one ? 31 : 11) + fx;
            const int ntx = g.Y / (2 * FL_LPB[fx]);
            for (int t = 0; t < ntx; ++t) xs[xc].push_back({g.X * 2 * FL_LPB[fx], make_int2((int)i, t)});
            smem_x[xc] = FL_XSMEM[fx];
            thr_x[xc] = FL_NT[fx];
        } else {
            const int lb = bi.lbx;
            const int ntx = (g.Y + lb - 1) / lb;
            for (int t = 0; t < ntx; ++t) xs[xc].push_back({g.H * lb, make_int2((int)i, t)});
            smem_x[xc] = std::max(smem_x[xc], xpass_smem_bytes(g, lb, vb, (g.X & 1) ? 3 : 2));
        }
        if (fy >= 0) { // line engine: tiles of LPB lines
            yc = (nb > 1 ? 21 : 11) + fy;
            const int nty = (int)((g.KX + FL_LPB[fy] - 1) / FL_LPB[fy]);
            for (int t = 0; t < nty; ++t) ys[yc].push_back({g.Y * FL_LPB[fy], make_int2((int)i, t)});
            smem_y[yc] = FL_YSMEM[fy];
            thr_y[yc] = FL_NT[fy];
        } else {
            const int lb = bi.lby;
            const int nty = (int)((g.KX + lb - 1) / lb);
            for (int t = 0; t < nty; ++t) ys[yc].push_back({g.Y * lb, make_int2((int)i, t)});
            smem_y[yc] = std::max(smem_y[yc], cpass_smem_bytes(g, g.Y, lb, nb, vb) + (lb + g.Y) * (int)sizeof(R));
        }
    }
    BCK(gopf_malloc(&b->d_inst, sizeof(BatchInst<R>) * inst.size()));
    BCK(cudaMemcpy(b->d_inst, inst.data(), sizeof(BatchInst<R>) * inst.size(), cudaMemcpyHostToDevice));
    int nsm = 0;
    BCK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, b->device));
    auto bycost = [](const std::pair<int, int2> &a, const std::pair<int, int2> &c) { return a.first > c.first; };
    // one launch per class present, largest classes first (they start first in the graph)
    auto make = [&](std::vector<std::pair<int, int2>> *lists, const int *smem, const int *thr, bool xpass,
                    std::vector<BatchLaunch> &out) -> int {
        std::vector<std::pair<long long, int>> order;
        for (int k = 0; k < NCLASS; ++k)
            if (!lists[k].empty()) {
                long long cost = 0;
                for (auto &p : lists[k]) cost += p.first;
                order.push_back({cost, k});
            }
        std::sort(order.begin(), order.end(), [](auto &a, auto &c) { return a.first > c.first; });
        for (auto &o : order) {
            const int k = o.second;
            std::stable_sort(lists[k].begin(), lists[k].end(), bycost);
            std::vector<int2> items;
            for (auto &p : lists[k]) items.push_back(p.second);
            BatchLaunch L;
            for (auto &it : items) L.inst.push_back(it.x);
            std::sort(L.inst.begin(), L.inst.end());
            L.inst.erase(std::unique(L.inst.begin(), L.inst.end()), L.inst.end());
            L.fn = xpass ? x_kernel<R>(k) : y_kernel<R>(k);
            L.nitems = (int)items.size();
            L.smem = smem[k];
            L.threads = thr[k];
            BCK(gopf_malloc(&L.d_items, sizeof(int2) * items.size()));
            out.push_back(L); // owned by the batch from here on (freed with it)
            BCK(cudaMemcpy(L.d_items, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice));
            BCK(cudaFuncSetAttribute(L.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, L.smem));
            int occ = 0;
            BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, L.fn, L.threads, L.smem));
            // the compile-time classes take one block per item; the generic kernels loop
            out.back().grid = (k > 0) ? L.nitems : std::max(1, std::min(L.nitems, nsm * std::max(occ, 1)));
        }
        return GOPF_OK;
    };
    int rc;
    if ((rc = make(xs, smem_x, thr_x, true, b->xl))) return rc;
    if ((rc = make(ys, smem_y, thr_y, false, b->yl))) return rc;
    b->chain.clear();
    if (b->xl.size() == b->yl.size()) {
        for (size_t i = 0; i < b->xl.size(); ++i)
            for (size_t j = 0; j < b->yl.size(); ++j)
                if (b->xl[i].inst == b->yl[j].inst) b->chain.push_back({(int)i, (int)j});
        if (b->chain.size() != b->xl.size()) b->chain.clear();
    }
    // projection launches: all instances, and each chain's own
    auto make_herm = [&](const std::vector<int> &ids, BatchHerm &h) -> int {
        std::vector<long long> off;
        long long t = 0;
        for (int i : ids) {
            off.push_back(t);
            const Geom &g = b->ctx[i]->g;
            t += ((g.X & 1) ? 1LL : 2LL) * g.Y;
        }
        h.n = (int)ids.size();
        h.total = t;
        BCK(gopf_malloc(&h.d_inst, sizeof(int) * ids.size()));
        BCK(gopf_malloc(&h.d_off, sizeof(long long) * off.size()));
        BCK(cudaMemcpy(h.d_inst, ids.data(), sizeof(int) * ids.size(), cudaMemcpyHostToDevice));
        BCK(cudaMemcpy(h.d_off, off.data(), sizeof(long long) * off.size(), cudaMemcpyHostToDevice));
        return GOPF_OK;
    };
    {
        std::vector<int> all(b->ctx.size());
        for (size_t i = 0; i < all.size(); ++i) all[i] = (int)i;
        if ((rc = make_herm(all, b->hall))) return rc;
        b->hchain.assign(b->chain.size(), BatchHerm());
        for (size_t i = 0; i < b->chain.size(); ++i)
            if ((rc = make_herm(b->xl[b->chain[i].first].inst, b->hchain[i]))) return rc;
    }
    const size_t nbranch = std::max(b->xl.size(), b->yl.size());
    while (b->side.size() + 1 < nbranch) {
        cudaStream_t st;
        BCK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        b->side.push_back(st);
    }
    while (b->ev.size() < nbranch + 1) {
        cudaEvent_t e;
        BCK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        b->ev.push_back(e);
    }
    return GOPF_OK;
}

// The launches of one pass as parallel branches: the first on the batch's stream, the others on
// side streams forked from it and joined back.
template <typename R> static cudaError_t batch_pass(gopf_batch *b, const std::vector<BatchLaunch> &ls)
{
    const BatchInst<R> *inst = (const BatchInst<R> *)b->d_inst;
    cudaError_t e;
    if (ls.size() > 1) {
        if ((e = cudaEventRecord(b->ev[0], b->stream)) != cudaSuccess) return e;
        for (size_t i = 1; i < ls.size(); ++i)
            if ((e = cudaStreamWaitEvent(b->side[i - 1], b->ev[0], 0)) != cudaSuccess) return e;
    }
    for (size_t i = 0; i < ls.size(); ++i) {
        const BatchLaunch &L = ls[i];
        cudaStream_t st = (i == 0) ? b->stream : b->side[i - 1];
        const int2 *items = L.d_items;
        int n = L.nitems;
        void *args[] = {(void *)&inst, (void *)&items, (void *)&n};
        if ((e = cudaLaunchKernel(L.fn, dim3(L.grid), dim3(L.threads), args, (size_t)L.smem, st)) != cudaSuccess)
            return e;
        if (i > 0 && (e = cudaEventRecord(b->ev[i], st)) != cudaSuccess) return e;
    }
    for (size_t i = 1; i < ls.size(); ++i)
        if ((e = cudaStreamWaitEvent(b->stream, b->ev[i], 0)) != cudaSuccess) return e;
    return cudaSuccess;
}

template <typename R> static cudaError_t launch_one(gopf_batch *b, const BatchLaunch &L, cudaStream_t st)
{
    const BatchInst<R> *inst = (const BatchInst<R> *)b->d_inst;
    const int2 *items = L.d_items;
    int n = L.nitems;
    void *args[] = {(void *)&inst, (void *)&items, (void *)&n};
    return cudaLaunchKernel(L.fn, dim3(L.grid), dim3(L.threads), args, (size_t)L.smem, st);
}

template <typename R> static cudaError_t launch_herm(gopf_batch *b, const BatchHerm &h, cudaStream_t st)
{
    const unsigned hb = (unsigned)std::max<long long>(1, std::min<long long>((h.total + 255) / 256, 152 * 4));
    k_batch_herm<R><<<hb, 256, 0, st>>>((const BatchInst<R> *)b->d_inst, h.d_inst, h.d_off, h.n, h.total);
    return cudaGetLastError();
}

// n steps of the class chains: each class runs x, y and its projection n times on its own branch
template <typename R> static cudaError_t batch_chains(gopf_batch *b, int nsteps)
{
    cudaError_t e;
    const size_t n = b->chain.size();
    if (n > 1) {
        if ((e = cudaEventRecord(b->ev[0], b->stream)) != cudaSuccess) return e;
        for (size_t i = 1; i < n; ++i)
            if ((e = cudaStreamWaitEvent(b->side[i - 1], b->ev[0], 0)) != cudaSuccess) return e;
    }
    for (size_t i = 0; i < n; ++i) {
        cudaStream_t st = (i == 0) ? b->stream : b->side[i - 1];
        for (int s = 0; s < nsteps; ++s) {
            if ((e = launch_one<R>(b, b->xl[b->chain[i].first], st)) != cudaSuccess) return e;
            if ((e = launch_one<R>(b, b->yl[b->chain[i].second], st)) != cudaSuccess) return e;
            if ((e = launch_herm<R>(b, b->hchain[i], st)) != cudaSuccess) return e;
        }
        if (i > 0 && (e = cudaEventRecord(b->ev[i], st)) != cudaSuccess) return e;
    }
    for (size_t i = 1; i < n; ++i)
        if ((e = cudaStreamWaitEvent(b->stream, b->ev[i], 0)) != cudaSuccess) return e;
    return cudaSuccess;
}

template <typename R> static cudaError_t batch_enqueue(gopf_batch *b, int nsteps)
{
    if (!b->chain.empty()) return batch_chains<R>(b, nsteps);
    cudaError_t e;
    for (int s = 0; s < nsteps; ++s) {
        if ((e = batch_pass<R>(b, b->xl)) != cudaSuccess) return e;
        if ((e = batch_pass<R>(b, b->yl)) != cudaSuccess) return e;
        if ((e = launch_herm<R>(b, b->hall, b->stream)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

static cudaError_t batch_enqueue_any(gopf_batch *b, int n)
{
    return (b->prec == GOPF_FP32) ? batch_enqueue<float>(b, n) : batch_enqueue<double>(b, n);
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

// Check the contexts and set up the batch's streams; no launches yet.
static int batch_init(gopf_batch *b, gopf_ctx *const *ctxs, int n)
{
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
        if (!c->sources.empty()) return bfail(b, GOPF_ERR_UNSUPPORTED, "batches step models without sources");
        b->ctx.push_back(c);
    }
    b->choice.assign(b->ctx.size(), BatchChoice());
    b->eff.assign(b->ctx.size(), BatchChoice());
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return bfail(b, GOPF_ERR_CUDA, cudaGetErrorString(e));
    e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bfail(b, GOPF_ERR_CUDA, cudaGetErrorString(e));
    b->stream = b->own_stream;
    // the contexts' own streams may still hold work
    for (gopf_ctx *c : b->ctx) cudaStreamSynchronize(c->stream);
    return GOPF_OK;
}

// Free the launches, item lists and graphs of the last build (the streams and events stay).
static void batch_release(gopf_batch *b)
{
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->g1) cudaGraphExecDestroy(b->g1);
    if (b->gK) cudaGraphExecDestroy(b->gK);
    b->g1 = b->gK = nullptr;
    if (b->d_inst) cudaFree(b->d_inst);
    b->d_inst = nullptr;
    for (auto *ls : {&b->xl, &b->yl}) {
        for (BatchLaunch &L : *ls)
            if (L.d_items) cudaFree(L.d_items);
        ls->clear();
    }
    b->chain.clear();
    for (BatchHerm *h : {&b->hall}) {
        if (h->d_inst) cudaFree(h->d_inst);
        if (h->d_off) cudaFree(h->d_off);
        *h = BatchHerm();
    }
    for (BatchHerm &h : b->hchain) {
        if (h.d_inst) cudaFree(h.d_inst);
        if (h.d_off) cudaFree(h.d_off);
    }
    b->hchain.clear();
}

static int batch_rebuild(gopf_batch *b)
{
    batch_release(b);
    return (b->prec == GOPF_FP32) ? batch_build<float>(b) : batch_build<double>(b);
}

extern "C" int gopf_batch_create(gopf_ctx *const *ctxs, int n, gopf_batch **out)
{
    if (!out || !ctxs || n < 1) return GOPF_ERR_ARG;
    *out = nullptr;
    gopf_batch *b = new gopf_batch();
    *out = b;
    int rc = batch_init(b, ctxs, n);
    if (rc) return rc;
    return (b->prec == GOPF_FP32) ? batch_build<float>(b) : batch_build<double>(b);
}

extern "C" int gopf_batch_destroy(gopf_batch *b)
{
    if (!b) return GOPF_ERR_ARG;
    cudaSetDevice(b->device);
    batch_release(b);
    for (cudaStream_t st : b->side) cudaStreamDestroy(st);
    for (cudaEvent_t e : b->ev) cudaEventDestroy(e);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    delete b;
    return GOPF_OK;
}

// ---- the autotuner ----

namespace {

// Instances that tune alike: same sides, precision, group count, one dense polynomial group or not,
// and whether the line engine's y pass can take the update.
typedef std::tuple<int, int, int, int, int, int> TuneKey;
std::mutex g_tune_mu;
std::map<TuneKey, BatchChoice> g_tune_cache;

TuneKey tune_key(const gopf_ctx *c)
{
    const int G = c->ngroups;
    const int one = (G == 1 && c->pw.deg[0] >= 0 && c->pw.deg[0] <= 6) ? 1 : 0;
    const int yl = (std::max(G, 1) <= 2 && c->upd.nimp <= 4) ? 1 : 0;
    return TuneKey(c->g.X, c->g.Y, c->prec, G, one, yl);
}

// Device time (ms) per step of a batch of these contexts with one choice for all of them: the
// 1-step graph is captured, run twice, then timed over `reps` replays with events on the batch's
// stream.  The contexts' fields are advanced (the caller restores them).
int time_choice(gopf_batch *parent, const std::vector<gopf_ctx *> &cs, const BatchChoice &ch, int reps, float *ms)
{
    gopf_batch t;
    int rc = batch_init(&t, cs.data(), (int)cs.size());
    if (!rc) {
        t.choice.assign(cs.size(), ch);
        rc = (t.prec == GOPF_FP32) ? batch_build<float>(&t) : batch_build<double>(&t);
    }
    if (!rc) rc = batch_capture(&t, 1, &t.g1);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (!rc) {
        cudaError_t e = cudaEventCreate(&e0);
        if (e == cudaSuccess) e = cudaEventCreate(&e1);
        for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaGraphLaunch(t.g1, t.stream);
        if (e == cudaSuccess) e = cudaEventRecord(e0, t.stream);
        for (int i = 0; i < reps && e == cudaSuccess; ++i) e = cudaGraphLaunch(t.g1, t.stream);
        if (e == cudaSuccess) e = cudaEventRecord(e1, t.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(t.stream);
        if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
        if (e != cudaSuccess) rc = bfail(parent, GOPF_ERR_CUDA, std::string("tuning: ") + cudaGetErrorString(e));
        else *ms /= (float)reps;
    } else if (rc) {
        parent->err = "tuning: " + t.err;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    batch_release(&t);
    for (cudaStream_t st : t.side) cudaStreamDestroy(st);
    for (cudaEvent_t e : t.ev) cudaEventDestroy(e);
    if (t.own_stream) cudaStreamDestroy(t.own_stream);
    return rc;
}

// candidate choices of one pass for a context (family, tile width, plan variant)
std::vector<BatchChoice> pass_candidates(const gopf_ctx *c, bool xpass, const BatchChoice &base)
{
    std::vector<BatchChoice> out;
    auto add = [&](int fam, int lb, int plan) {
        BatchChoice ch = base;
        if (xpass) {
            ch.xfam = fam;
            ch.lbx = lb;
            ch.xplan = plan;
        } else {
            ch.yfam = fam;
            ch.lby = lb;
            ch.yplan = plan;
        }
        out.push_back(ch);
    };
    if (c->prec == GOPF_FP32) {
        add(GOPF_BATCH_LINE, 0, 0);
        add(GOPF_BATCH_STOCKHAM_CT, 0, 0);
    }
    const bool odd = xpass && (c->g.X & 1);
    const int n = xpass ? (odd ? c->g.KX : c->g.H) : c->g.Y;             // tile-width bound
    const int pn = xpass ? (odd ? c->g.X : c->g.H) : c->g.Y;             // transform length
    for (int lb : {4, 8, 16})
        if (batch_lb_ok(lb, n))
            for (int plan = 0; plan < 3; ++plan) {
                gopf::LinePlan pl;
                if (gopf_make_plan(pn, (xpass && !odd) ? 2 : 1, plan, pl)) add(GOPF_BATCH_STOCKHAM, lb, plan);
            }
    return out;
}

} // namespace

extern "C" int gopf_batch_tune(gopf_batch *b, int reps)
{
    if (!b) return GOPF_ERR_ARG;
    if (reps < 1) reps = 5;
    BCK(cudaSetDevice(b->device));
    BCK(cudaStreamSynchronize(b->stream));
    std::map<TuneKey, std::vector<int>> groups;
    for (size_t i = 0; i < b->ctx.size(); ++i) groups[tune_key(b->ctx[i])].push_back((int)i);
    for (auto &kv : groups) {
        BatchChoice best;
        bool cached = false;
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            auto it = g_tune_cache.find(kv.first);
            if (it != g_tune_cache.end()) {
                best = it->second;
                cached = true;
            }
        }
        if (!cached) {
            std::vector<gopf_ctx *> cs;
            for (int i : kv.second) cs.push_back(b->ctx[i]);
            // keep the fields: back up c-hat and T of every instance of the group
            const size_t vb = (b->prec == GOPF_FP32) ? 8 : 16;
            std::vector<void *> bk;
            std::vector<long long> steps;
            int rc = GOPF_OK;
            for (gopf_ctx *c : cs) {
                void *p = nullptr;
                cudaError_t e = gopf_malloc(&p, 2 * vb * c->g.C);
                if (e != cudaSuccess) { rc = bfail(b, GOPF_ERR_OOM, "tuning: no room for the field backup"); break; }
                bk.push_back(p);
                steps.push_back(c->step);
                e = cudaMemcpy(p, c->d_state, vb * c->g.C, cudaMemcpyDeviceToDevice);
                if (e == cudaSuccess) e = cudaMemcpy((char *)p + vb * c->g.C, c->d_T, vb * c->g.C, cudaMemcpyDeviceToDevice);
                if (e != cudaSuccess) { rc = bfail(b, GOPF_ERR_CUDA, cudaGetErrorString(e)); break; }
            }
            // x pass first (y by the built-in preference), then the y pass with the best x
            for (int pass = 0; pass < 2 && !rc; ++pass) {
                float best_ms = 1e30f;
                BatchChoice winner = best;
                for (const BatchChoice &cand : pass_candidates(cs[0], pass == 0, best)) {
                    float ms = 0.f;
                    if ((rc = time_choice(b, cs, cand, reps, &ms))) break;
                    if (ms < best_ms) {
                        best_ms = ms;
                        winner = cand;
                    }
                }
                best = winner;
            }
            for (size_t k = 0; k < cs.size() && k < bk.size(); ++k) {
                gopf_ctx *c = cs[k];
                cudaMemcpy(c->d_state, bk[k], vb * c->g.C, cudaMemcpyDeviceToDevice);
                cudaMemcpy(c->d_T, (char *)bk[k] + vb * c->g.C, vb * c->g.C, cudaMemcpyDeviceToDevice);
                c->step = steps[k];
                cudaFree(bk[k]);
            }
            if (rc) return rc;
            BCK(cudaDeviceSynchronize());
            std::lock_guard<std::mutex> lk(g_tune_mu);
            g_tune_cache[kv.first] = best;
        }
        for (int i : kv.second) b->choice[i] = best;
    }
    return batch_rebuild(b);
}

extern "C" int gopf_batch_tune_reset(void)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache.clear();
    return GOPF_OK;
}

extern "C" int gopf_batch_force(gopf_batch *b, int xfam, int yfam, int lbx, int lby, int xplan, int yplan)
{
    if (!b) return GOPF_ERR_ARG;
    if (xfam < GOPF_BATCH_AUTO || xfam > GOPF_BATCH_STOCKHAM || yfam < GOPF_BATCH_AUTO || yfam > GOPF_BATCH_STOCKHAM ||
        xplan < 0 || xplan > 2 || yplan < 0 || yplan > 2)
        return bfail(b, GOPF_ERR_ARG, "unknown kernel family or plan variant");
    BCK(cudaSetDevice(b->device));
    BatchChoice ch;
    ch.xfam = xfam;
    ch.yfam = yfam;
    ch.lbx = lbx;
    ch.lby = lby;
    ch.xplan = xplan;
    ch.yplan = yplan;
    for (auto &c : b->choice) c = ch;
    return batch_rebuild(b);
}

extern "C" int gopf_batch_choice(gopf_batch *b, int inst, int *out6)
{
    if (!b || !out6 || inst < 0 || inst >= (int)b->eff.size()) return GOPF_ERR_ARG;
    const BatchChoice &e = b->eff[inst];
    const int v[6] = {e.xfam, e.yfam, e.lbx, e.lby, e.xplan, e.yplan};
    for (int k = 0; k < 6; ++k) out6[k] = v[k];
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
    *n = b->chain.empty() ? (int)(b->xl.size() + b->yl.size()) + 1 : 3 * (int)b->chain.size();
    return GOPF_OK;
}
