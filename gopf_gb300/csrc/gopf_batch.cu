// gopf_batch.cu -- many independent instances stepped by shared launches.
//
// The parameter-sweep workflow of gopf (one FieldDB per swept run, README.md:21-33)
// steps every instance separately.  A batch takes N contexts of arbitrary
// (2D) sizes, each with its own equation, coefficients and dt, and steps them
// together.  Instances are grouped into size classes; per step each class
// present gets one x-pass launch and one fused y-pass launch over its
// (instance, tile) items, ordered largest first, so small instances no longer
// leave the GPU idle.  Two ways to step them, both captured in CUDA graphs of 1
// and 16 steps:
// - persistent (the default where every instance allows it): one kernel launch
//   per graph.  Its blocks take the x and y tiles of every instance and step
//   from one queue; per-instance counters order each instance's tiles
//   (k_batch_persist);
// - chains: when the classes of both passes cover the same instances, each
//   class is a chain on its own branch of the graph: x pass, y pass and the
//   Hermitian projection of its own instances, for every step of the graph,
//   with one fork and one join per graph (3 launches per class and step).
//   Otherwise the classes of a pass run as parallel branches and one projection
//   of every instance ends each step (2 x classes + 1 launches).
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

// ---- the persistent sweep kernel ----
// One launch steps every instance nsteps times.  The items of one step (x tiles, then y tiles, each
// class largest first) are handed out in order from a queue counter; item g of the launch is item
// g % nper of step g / nper.  An x item of step s needs every y item of its instance's step s - 1
// done (it overwrites the rows of T they wrote), a y item every x item of its instance's step s (it
// reads the lines they wrote): per-instance completion counters, incremented after an item's last
// write, carry that.  An item's dependencies always come earlier in the queue, so they were taken by
// running blocks and complete: no wait can deadlock, and every wait is bounded all the same.
// An item {instance, first tile, kind, tiles} covers `tiles` consecutive tiles of one instance and pass;
// the counters count tiles.
// Item kinds: PK_X + c (x pass) and PK_Y + c (y pass) of size class c: 0 .. 4 the line engine's sides
// 256, 384, 512, 768, 1024 (x: one dense polynomial group, y: one group), PK_CT the side 128 on
// compile-time Stockham tiles (x: 16-row tiles of the 64-point half transform, y: 16-line tiles).  A y
// item also projects the self-conjugate lines it owns (kx = 0 and X/2), as k_batch_herm does after a
// pass.  The 192-thread tiles (384, 768) run on the block's first 192 threads under a named barrier.
constexpr int PK_X = 0, PK_Y = 8, PK_CT = 5, PK_TILES = 2;
// lines per y tile of class c
__host__ __device__ constexpr int pk_lpb(int c)
{
    return c == 0 ? fl::Geo<256>::LPB : c == 1 ? fl::Geo<384>::LPB : c == 2 ? fl::Geo<512>::LPB
         : c == 3 ? fl::Geo<768>::LPB : c == 4 ? fl::Geo<1024>::LPB : 16;
}

// The counters' ordering: a block's writes, a barrier, then a release add by one of its threads; the
// waiting block's thread sees the count with an acquire load, then a barrier, then the block reads.
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_release_add(unsigned *p, unsigned v)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Wait until *c >= need, for at most the limit at status + 2 (u64 ns; 0: 2 s).  On timeout flag
// DS_DEP_TIMEOUT in status[0] and return false.
__device__ __noinline__ bool pk_wait(const unsigned *c, unsigned need, unsigned *status)
{
    if (ld_acquire_u32(c) >= need) return true;
    unsigned long long lim = *reinterpret_cast<const volatile unsigned long long *>(status + 2);
    if (!lim) lim = 2000000000ull;
    const unsigned long long t0 = global_ns();
    while (true) {
        __nanosleep(128);
        if (ld_acquire_u32(c) >= need) return true;
        if (global_ns() - t0 > lim) {
            atomicOr(status, (unsigned)DS_DEP_TIMEOUT);
            return false;
        }
    }
}

// The tile kinds are separate (not inlined) functions, so that each gets its own register
// allocation instead of the kernel holding the union of all of them.
template <int L> __device__ __noinline__ void pk_x(const BatchInst<float> *bi, int tile, XPassArgs<float> *s_a)
{
    stage_args(s_a, &bi->xa);
    __syncthreads();
    if (threadIdx.x < fl::Geo<L>::NT) fl::xline_tile<L, true>(*s_a, tile, 0);
}

template <int L> __device__ __noinline__ void pk_y(const BatchInst<float> *bi, int tile)
{
    if (threadIdx.x < fl::Geo<L>::NT) fl::yline_tile<L, 1>(bi->pa, tile);
}

__device__ __noinline__ void pk_x_ct(const BatchInst<float> *bi, int tile, XPassArgs<float> *s_a)
{
    stage_args(s_a, &bi->xa);
    __syncthreads();
    if (s_a->ngrp_out) xpass_tile<float, 16, 16, false, 64>(*s_a, tile, 0);
}

__device__ __noinline__ void pk_y_ct(const BatchInst<float> *bi, int tile, PassArgs<float> *s_a)
{
    stage_args(s_a, &bi->pa);
    __syncthreads();
    pass_tile<float, 16, 16, true, false, 128>(*s_a, tile, 0);
}

// the projection of line kx of a 2D instance's c-hat (the formula of k_batch_herm)
__device__ __forceinline__ void pk_herm_line(float2 *__restrict__ c, long long base, int Y)
{
    for (int y = threadIdx.x; y < Y; y += blockDim.x) {
        const int yp = (Y - y) % Y;
        if (y > yp) continue;
        const float2 a = c[base + y], b = c[base + yp];
        float2 m;
        m.x = (a.x + b.x) * 0.5f;
        m.y = (a.y - b.y) * 0.5f;
        c[base + y] = m;
        m.y = -m.y;
        c[base + yp] = m;
    }
}

__global__ void __launch_bounds__(256, 3)
    k_batch_persist(const BatchInst<float> *__restrict__ inst, const int4 *__restrict__ items, int nper, int nsteps,
                    const int2 *__restrict__ nxy, unsigned *__restrict__ ctr, unsigned *status)
{
    // an item's pass arguments, staged in shared memory (x: XPassArgs, y on Stockham tiles: PassArgs)
    __shared__ __align__(16) unsigned char s_args[sizeof(XPassArgs<float>) > sizeof(PassArgs<float>)
                                                      ? sizeof(XPassArgs<float>)
                                                      : sizeof(PassArgs<float>)];
    XPassArgs<float> *s_xa = reinterpret_cast<XPassArgs<float> *>(s_args);
    __shared__ int s_g;
    __shared__ int4 s_it;
    const int total = nper * nsteps;
    // Thread 0 takes the tickets and waits for the dependencies; the next ticket is taken while the
    // current item runs (its latency hides there).  A block holding a ticket it has not started
    // cannot deadlock the queue: it took that ticket after the one it is running, and every item's
    // dependencies have smaller tickets.
    auto prepare = [&](int g) {
        int4 it = make_int4(0, 0, -1, 0);
        if (g < total) {
            const int s = g / nper;
            it = items[g - s * nper];
            const bool yp = it.z >= PK_Y;
            const unsigned need = yp ? (unsigned)((s + 1) * nxy[it.x].x) : (unsigned)(s * nxy[it.x].y);
            // a wait that ran out skips the item (the step is flagged) but still counts it done
            if (!pk_wait(&ctr[1 + 2 * it.x + (yp ? 0 : 1)], need, status)) g = -1 - g;
        } else {
            g = total;
        }
        s_g = g;
        s_it = it;
    };
    if (threadIdx.x == 0) prepare((int)atomicAdd(ctr, 1u));
    __syncthreads();
    for (;;) {
        const int g = s_g;
        if (g >= total) return;
        const int4 it = s_it;
        int gnext = total;
        if (threadIdx.x == 0) gnext = (int)atomicAdd(ctr, 1u);
        const BatchInst<float> *bi = inst + it.x;
        for (int k = 0; g >= 0 && k < it.w; ++k) {
            const int tile = it.y + k;
            if (k) __syncthreads(); // the previous tile is done with the shared memory
            switch (it.z) {
            case PK_X + 0: pk_x<256>(bi, tile, s_xa); break;
            case PK_X + 1: pk_x<384>(bi, tile, s_xa); break;
            case PK_X + 2: pk_x<512>(bi, tile, s_xa); break;
            case PK_X + 3: pk_x<768>(bi, tile, s_xa); break;
            case PK_X + 4: pk_x<1024>(bi, tile, s_xa); break;
            case PK_X + PK_CT: pk_x_ct(bi, tile, s_xa); break;
            case PK_Y + 0: pk_y<256>(bi, tile); break;
            case PK_Y + 1: pk_y<384>(bi, tile); break;
            case PK_Y + 2: pk_y<512>(bi, tile); break;
            case PK_Y + 3: pk_y<768>(bi, tile); break;
            case PK_Y + 4: pk_y<1024>(bi, tile); break;
            case PK_Y + PK_CT: pk_y_ct(bi, tile, reinterpret_cast<PassArgs<float> *>(s_args)); break;
            default: break;
            }
            if (it.z >= PK_Y) {
                __syncthreads(); // the tile's c-hat writes are done
                const int Y = bi->pa.g.Y, H = bi->pa.g.H;
                const long long q0 = (long long)tile * pk_lpb(it.z - PK_Y);
                const long long q1 = q0 + pk_lpb(it.z - PK_Y);
                if (q0 == 0) pk_herm_line(bi->pa.state, 0, Y);
                if (H >= q0 && H < q1) pk_herm_line(bi->pa.state, (long long)H * Y, Y);
            }
        }
        __syncthreads(); // every write of the item is done, and s_g, s_it are free again
        if (threadIdx.x == 32) // the completion, while thread 0 prepares the next item
            red_release_add(&ctr[1 + 2 * it.x + (it.z >= PK_Y ? 1 : 0)], (unsigned)it.w);
        if (threadIdx.x == 0) prepare(gnext);
        __syncthreads();
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
    // the persistent mode (k_batch_persist): requested mode, mode in effect (1: persistent), the items
    // of one step, per-instance item counts, the queue and completion counters, the launch shape
    int mode = GOPF_BATCH_MODE_AUTO, pmode = 0;
    int4 *d_pitems = nullptr;
    int2 *d_pnxy = nullptr;
    unsigned *d_pctr = nullptr;
    int pnper = 0, pgrid = 0, psmem = 0;
    size_t pctr_bytes = 0;
    unsigned *d_pstatus = nullptr; // [0] flags, [2..3] wait limit (u64 ns, 0: 2 s)
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
        // the batch's own default tile widths (a context narrows its tiles for its own small passes,
        // a batch's passes are wide)
        const bool oddx = (g.X & 1) != 0;
        bi.lbx = lb_for(oddx ? g.KX : g.H, vb);
        bi.lby = lb_for(g.Y, vb);
        int xc = 0, yc = 0, fx = -1, fy = -1;
        if (sizeof(R) == 4) {
            for (int k = 1; k < 7; ++k) {
                if (g.H == XCLS_H[k] && bi.lbx == XCLS_LB[k] && !(g.X & 1)) xc = k;
                if (g.Y == YCLS_N[k] && bi.lby == YCLS_LB[k]) yc = k;
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
    // the persistent mode: every instance on a kind k_batch_persist runs (FP32)
    b->pmode = 0;
    if (b->mode != GOPF_BATCH_MODE_CHAINS) {
        bool ok = (sizeof(R) == 4);
        std::vector<int> xkind(b->ctx.size(), -1), ykind(b->ctx.size(), -1);
        for (int k = 0; k < NCLASS && ok; ++k) {
            int xk = -1, yk = -1;
            if (k >= 31 && k <= 35) xk = PK_X + (k - 31);
            if (k == 1) xk = PK_X + PK_CT;
            if (k >= 11 && k <= 15) yk = PK_Y + (k - 11);
            if (k == 1) yk = PK_Y + PK_CT;
            for (auto &p : xs[k]) {
                if (xk < 0) ok = false;
                xkind[p.second.x] = xk;
            }
            for (auto &p : ys[k]) {
                if (yk < 0) ok = false;
                ykind[p.second.x] = yk;
            }
        }
        for (size_t i = 0; i < b->ctx.size() && ok; ++i)
            if (xkind[i] < 0 || ykind[i] < 0 || (b->ctx[i]->g.X & 1)) ok = false;
        if (!ok && b->mode == GOPF_BATCH_MODE_PERSISTENT)
            return bfail(b, GOPF_ERR_UNSUPPORTED,
                         "the persistent mode takes FP32 instances of sides 128 ... 1024 on the line engine "
                         "(256 ... 1024, one dense polynomial group) or compile-time Stockham tiles (128)");
        if (ok) {
            // one step's items: the x tiles of every class, largest class first, then the y tiles
            std::vector<int4> items;
            std::vector<int2> nxy(b->ctx.size(), make_int2(0, 0));
            int smem = 0;
            for (int pass = 0; pass < 2; ++pass) {
                std::vector<std::pair<long long, int>> order;
                for (int k = 0; k < NCLASS; ++k) {
                    auto &lst = pass ? ys[k] : xs[k];
                    if (lst.empty()) continue;
                    long long cost = 0;
                    for (auto &p : lst) cost += p.first;
                    order.push_back({cost, k});
                    smem = std::max(smem, pass ? smem_y[k] : smem_x[k]);
                }
                std::sort(order.begin(), order.end(), [](auto &a, auto &c) { return a.first > c.first; });
                for (auto &o : order) {
                    // consecutive tiles of an instance, PK_TILES to an item (the class's list holds
                    // each instance's tiles in order, instances largest first)
                    const auto &lst = pass ? ys[o.second] : xs[o.second];
                    for (size_t a = 0; a < lst.size();) {
                        const int i = lst[a].second.x, t0 = lst[a].second.y;
                        int w = 1;
                        while (w < PK_TILES && a + w < lst.size() && lst[a + w].second.x == i &&
                               lst[a + w].second.y == t0 + w)
                            ++w;
                        items.push_back(make_int4(i, t0, pass ? ykind[i] : xkind[i], w));
                        if (pass) nxy[i].y += w;
                        else nxy[i].x += w;
                        a += w;
                    }
                }
            }
            b->pnper = (int)items.size();
            b->psmem = smem;
            b->pctr_bytes = sizeof(unsigned) * (1 + 2 * b->ctx.size());
            int occ = 0;
            cudaError_t fe = cudaFuncSetAttribute(k_batch_persist, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (fe == cudaSuccess) fe = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch_persist, 256, smem);
            if (fe != cudaSuccess || occ < 1) {
                // the kernel does not fit: AUTO steps by the chains, PERSISTENT is refused
                cudaGetLastError();
                if (b->mode == GOPF_BATCH_MODE_PERSISTENT)
                    return bfail(b, GOPF_ERR_UNSUPPORTED, "the persistent batch kernel does not fit an SM");
            } else {
                BCK(gopf_malloc(&b->d_pitems, sizeof(int4) * items.size()));
                BCK(gopf_malloc(&b->d_pnxy, sizeof(int2) * nxy.size()));
                BCK(gopf_malloc(&b->d_pctr, b->pctr_bytes));
                BCK(cudaMemcpy(b->d_pitems, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice));
                BCK(cudaMemcpy(b->d_pnxy, nxy.data(), sizeof(int2) * nxy.size(), cudaMemcpyHostToDevice));
                b->pgrid = nsm * occ;
                b->pmode = 1;
            }
        }
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
    if (b->pmode) {
        if constexpr (sizeof(R) == 4) {
            cudaError_t e = cudaMemsetAsync(b->d_pctr, 0, b->pctr_bytes, b->stream);
            if (e != cudaSuccess) return e;
            k_batch_persist<<<b->pgrid, 256, b->psmem, b->stream>>>((const BatchInst<float> *)b->d_inst, b->d_pitems,
                                                                   b->pnper, nsteps, b->d_pnxy, b->d_pctr,
                                                                   b->d_pstatus);
            return cudaGetLastError();
        }
        return cudaErrorNotSupported;
    }
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
    e = cudaMalloc(&b->d_pstatus, 4 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(b->d_pstatus, 0, 4 * sizeof(unsigned));
    if (e != cudaSuccess) return bfail(b, GOPF_ERR_CUDA, cudaGetErrorString(e));
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
    if (b->d_pitems) cudaFree(b->d_pitems);
    if (b->d_pnxy) cudaFree(b->d_pnxy);
    if (b->d_pctr) cudaFree(b->d_pctr);
    b->d_pitems = nullptr;
    b->d_pnxy = nullptr;
    b->d_pctr = nullptr;
    b->pmode = 0;
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
    if (b->d_pstatus) cudaFree(b->d_pstatus);
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
    if (t.d_pstatus) cudaFree(t.d_pstatus);
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
    // the persistent kernel's kinds are fixed (line engine 256 ... 1024, compile-time Stockham 128)
    if (b->pmode) return GOPF_OK;
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
    if (b->pmode) {
        unsigned flags = 0;
        BCK(cudaMemcpy(&flags, b->d_pstatus, sizeof(unsigned), cudaMemcpyDeviceToHost));
        if (flags) {
            BCK(cudaMemset(b->d_pstatus, 0, sizeof(unsigned)));
            return bfail(b, GOPF_ERR_TIMEOUT, "a persistent batch item's wait for the items it depends on ran out; "
                                              "the fields are not valid (upload them again)");
        }
    }
    return GOPF_OK;
}

extern "C" int gopf_batch_kernels_per_step(gopf_batch *b, int *n)
{
    if (!b || !n) return GOPF_ERR_ARG;
    *n = b->pmode ? 1 : b->chain.empty() ? (int)(b->xl.size() + b->yl.size()) + 1 : 3 * (int)b->chain.size();
    return GOPF_OK;
}

extern "C" int gopf_batch_set_mode(gopf_batch *b, int mode)
{
    if (!b) return GOPF_ERR_ARG;
    if (mode < GOPF_BATCH_MODE_AUTO || mode > GOPF_BATCH_MODE_PERSISTENT)
        return bfail(b, GOPF_ERR_ARG, "unknown batch mode");
    BCK(cudaSetDevice(b->device));
    const int old = b->mode;
    b->mode = mode;
    const int rc = batch_rebuild(b);
    if (rc && mode == GOPF_BATCH_MODE_PERSISTENT) {
        // keep the batch usable in the mode it had
        const std::string msg = b->err;
        b->mode = old;
        if (batch_rebuild(b) == GOPF_OK) b->err = msg;
    }
    return rc;
}

extern "C" int gopf_batch_mode(gopf_batch *b, int *mode)
{
    if (!b || !mode) return GOPF_ERR_ARG;
    *mode = b->pmode ? GOPF_BATCH_MODE_PERSISTENT : GOPF_BATCH_MODE_CHAINS;
    return GOPF_OK;
}

extern "C" int gopf_batch_set_wait_limit(gopf_batch *b, long long ns)
{
    if (!b || ns < 0) return GOPF_ERR_ARG;
    BCK(cudaSetDevice(b->device));
    BCK(cudaStreamSynchronize(b->stream));
    const unsigned long long v = (unsigned long long)ns;
    BCK(cudaMemcpy(b->d_pstatus + 2, &v, sizeof(v), cudaMemcpyHostToDevice));
    return GOPF_OK;
}
