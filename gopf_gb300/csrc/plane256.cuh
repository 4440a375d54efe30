// plane256.cuh -- one depth plane per cluster: inverse y, x pass, forward y (FP32, 256 x 256 planes).
//
// Between two z passes the step needs, for every depth plane, the inverse
// transform along y (rows of the half spectrum), the x pass (c2r, pointwise
// polynomial, r2c) and the forward transform along y.  Done as three
// kernels, each reads and writes the whole spectral array (6C of HBM
// traffic).  Here a cluster of 8 blocks holds one plane (129 x 256 complex,
// 264 KB) in its distributed shared memory and does all three, so the plane
// crosses HBM once in each direction (2C):
//
//   load     block c loads rows kx = 16c .. 16c+15 (block 0 also row 128), one bulk copy each
//   y inv    16 lines per block; line 0 of block 0 packs the real-on-return rows kx = 0 and
//            kx = 128 as A + iB
//   scatter  each value goes to the block that owns its y (rows 32d .. 32d+31) -> [129][32] tile
//   x pass   16 row pairs per block, exactly as the x-pass kernel (c2r, polynomial, r2c)
//   scatter  each spectral value goes to the block that owns its kx -> [16][256] lines
//   y fwd    16 lines per block; line 0 of block 0 is split back into rows 0 and 128
//   store    one bulk copy per block (block 0 also row 128)
//
// Remote writes use st.shared::cluster; cluster barriers separate the
// phases.  The input and output may be the same array: every block has read
// its rows before the first cluster barrier and writes only after the last.
#pragma once
#include "fast256.cuh"

namespace gopf {
namespace f256 {

__device__ __forceinline__ uint32_t cluster_rank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_arrive_relaxed() { asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }
__device__ __forceinline__ uint32_t map_rank(uint32_t laddr, uint32_t rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(laddr), "r"(rank));
    return r;
}
__device__ __forceinline__ void st_cluster(uint32_t addr, float2 v)
{
    asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(v.x), "f"(v.y) : "memory");
}
__device__ __forceinline__ void st_cluster4(uint32_t addr, float4 v)
{
    asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void bulk_store(void *dst, const void *src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)), "r"(bytes)
                 : "memory");
}

constexpr int PL_CLUSTER = 8;
constexpr int PL_LINES = 16;                    // y lines (kx rows) per block
constexpr int PL_TILE = PL_LINES * N * 8;       // 32 KB
constexpr int PL_A = PL_TILE + N * 8 + 256;     // line tile + row 128, reused as the x exchange [256][16] + pad
constexpr int PL_RX = 129 * XROWS * 8;          // [129 kx][32 y] x-pass input

__host__ __device__ constexpr int plane256_smem_bytes()
{
    return 128 + PL_A + PL_RX + N * 8 + GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1) * 4 + 16;
}

// Three blocks per SM: the lines of the forward y pass (Ry) reuse the line
// tile, so the x pass keeps its separated outputs in registers until every
// block of the cluster is done with its tile (one extra cluster barrier).
__global__ void __cluster_dims__(PL_CLUSTER, 1, 1) __launch_bounds__(NT, 3) k_plane256(const XPassArgs<float> a)
{
    extern __shared__ unsigned char pl_dsm[];
    unsigned char *base = pl_dsm + ((128u - (smem_u32(pl_dsm) & 127u)) & 127u);
    float2 *tA = reinterpret_cast<float2 *>(base);
    float2 *rowX = tA + PL_LINES * N; // row kx = 128 (block 0)
    float2 *Rx = reinterpret_cast<float2 *>(base + PL_A);
    float2 *Ry = tA;                  // [16 lines][256 ky], after the x pass
    float2 *s_tw = reinterpret_cast<float2 *>(base + PL_A + PL_RX);
    float *s_poly = reinterpret_cast<float *>(s_tw + N);
    uint64_t *bar = reinterpret_cast<uint64_t *>(s_poly + GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1));
    int *s_ok = reinterpret_cast<int *>(bar + 1);

    const int tid = threadIdx.x;
    const uint32_t c = cluster_rank();
    const long long pbase = (long long)(blockIdx.x / PL_CLUSTER) * a.g.S; // first element of the plane
    cluster_arrive_relaxed(); // matched by the wait before the first remote write

    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
        mbar_arrive_expect_tx(bar, (uint32_t)(PL_TILE + (c == 0 ? N * 8 : 0)));
        bulk_load(tA, a.in + pbase + (long long)PL_LINES * c * N, (uint32_t)PL_TILE, bar);
        if (c == 0) bulk_load(rowX, a.in + pbase + 128LL * N, (uint32_t)(N * 8), bar);
    }
    for (int t = tid; t < GOPF_MAX_GROUPS * (GOPF_MAX_DEG + 1); t += NT)
        s_poly[t] = (float)a.pw.dense[t / (GOPF_MAX_DEG + 1)][t % (GOPF_MAX_DEG + 1)];
    load_twiddles(s_tw, a.twX);
    if (tid == 0) *s_ok = tma_wait_or_flag(bar, 0, a.status) ? 1 : 0;
    __syncthreads();
    const bool ok = *s_ok != 0; // on a timeout the block still takes part in every cluster barrier

    // ---- inverse y: thread t = l*16 + r owns line l's elements r + 16 i
    {
        const int l = tid >> 4, r = tid & 15;
        float2 v[16];
        if (c == 0 && l == 0) {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const float2 A = tA[r + 16 * i], B = rowX[r + 16 * i];
                v[i] = make_float2(A.x - B.y, A.y + B.x);
            }
        } else {
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] = tA[l * N + r + 16 * i];
        }
        __syncthreads();
        auto at = [&](int x, int y) -> float2 & { return tA[l * N + x * 16 + ((x + y) & 15)]; };
        fft256<true, true>(v, r, s_tw, at);

        // scatter to the owners of the rows: y = r + 16 i lives in block i/2 at column r + 16 (i & 1)
        cluster_wait(); // every block of the cluster has started
        const int kx = PL_LINES * (int)c + l;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const uint32_t d = (uint32_t)(i >> 1);
            const int yl = r + 16 * (i & 1);
            if (c == 0 && l == 0) {
                st_cluster(map_rank(smem_u32(&Rx[yl]), d), make_float2(v[i].x, 0.f));
                st_cluster(map_rank(smem_u32(&Rx[128 * XROWS + yl]), d), make_float2(v[i].y, 0.f));
            } else {
                st_cluster(map_rank(smem_u32(&Rx[kx * XROWS + yl]), d), v[i]);
            }
        }
    }
    cluster_arrive();
    cluster_wait();

    // ---- x pass on rows 32c .. 32c+31: thread t = r*16 + j owns row pair j's columns r + 16 i
    {
        const int j = tid & 15, r = tid >> 4;
        float2 v[16];
        load_pair_line(Rx, r, j, v);
        auto at = [&](int x, int y) -> float2 & { return tA[(x * 16 + y) * 16 + j]; };
        fft256<true>(v, r, s_tw, at);
        if (!a.identity) apply_poly(v, a, 0, s_poly);
        fft256<false>(v, r, s_tw, at);
#pragma unroll
        for (int i = 0; i < 16; ++i) tA[(r + 16 * i) * 16 + j] = v[i];
        __syncthreads();
        // separation X_a(k) = (Z(k) + conj Z(-k))/2, X_b(k) = (Z(k) - conj Z(-k))/(2i) into registers,
        // both rows of pair p at once: kx = k0 + 16 q (q = 0..7) goes to block q, line k0, as one
        // 16-byte store; kx = 0 and 128 (both real) go to block 0 line 0 as A + iB
        const int p = tid & 15, k0 = tid >> 4;
        float4 o[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int kx = k0 + 16 * q;
            const float2 P = tA[kx * 16 + p];
            if (kx == 0) {
                const float2 P2 = tA[128 * 16 + p];
                o[q] = make_float4(P.x, P2.x, P.y, P2.y);
            } else {
                const float2 Q = tA[(N - kx) * 16 + p];
                o[q] = make_float4(0.5f * (P.x + Q.x), 0.5f * (P.y - Q.y), 0.5f * (P.y + Q.y), 0.5f * (Q.x - P.x));
            }
        }
        cluster_arrive();
        cluster_wait(); // every block has read its tile: the line buffers may be overwritten
        const uint32_t ry = smem_u32(Ry) + (uint32_t)((k0 * N + XROWS * (int)c + 2 * p) * 8);
#pragma unroll
        for (int q = 0; q < 8; ++q) st_cluster4(map_rank(ry, (uint32_t)q), o[q]);
    }
    cluster_arrive();
    cluster_wait(); // no remote writes after this point

    // ---- forward y on this block's lines
    {
        const int l = tid >> 4, r = tid & 15;
        float2 v[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = Ry[l * N + r + 16 * i];
        __syncthreads();
        auto at = [&](int x, int y) -> float2 & { return Ry[l * N + x * 16 + ((x + y) & 15)]; };
        fft256<false, true>(v, r, s_tw, at);
#pragma unroll
        for (int i = 0; i < 16; ++i) Ry[l * N + r + 16 * i] = v[i];
        __syncthreads();
    }
    float2 *rowB = Rx + N; // block 0: row kx = 128 of the result
    if (c == 0) {
        // line 0 carried A + iB for the real rows kx = 0 (A) and kx = 128 (B)
        float2 *rowA = Rx;
        for (int k = tid; k < N; k += NT) {
            const float2 Z = Ry[k], Zm = Ry[(N - k) & (N - 1)];
            rowA[k] = make_float2(0.5f * (Z.x + Zm.x), 0.5f * (Z.y - Zm.y));
            rowB[k] = make_float2(0.5f * (Z.y + Zm.y), 0.5f * (Zm.x - Z.x));
        }
        __syncthreads();
        for (int k = tid; k < N; k += NT) Ry[k] = rowA[k];
    }
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
        if (ok) {
            float2 *out = a.out[0];
            bulk_store(out + pbase + (long long)PL_LINES * c * N, Ry, (uint32_t)PL_TILE);
            if (c == 0) bulk_store(out + pbase + 128LL * N, rowB, (uint32_t)(N * 8));
            bulk_commit();
        }
        bulk_wait_read_all();
    }
}

} // namespace f256
} // namespace gopf
