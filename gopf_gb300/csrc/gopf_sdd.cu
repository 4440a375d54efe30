// gopf_sdd.cu -- shrinking-dimer dynamics (SDD, pf/sdd.go:86-470) on the device.
//
// SDD walks a dimer of length l(t) = l0 exp(-t/tau_l) (floored at MinDimerLength) with unit
// orientation v towards a saddle point.  Per step (SDD.Step, pf/sdd.go:159-285):
//   rhsStart, rhsEnd = the explicit right-hand sides at c - l v/2 and c + l v/2;
//   per field: work = alpha rhsStart + (1 - alpha) rhsEnd, reflected by the Householder
//   operator I - 2 v v^T, explicit step, then the implicit part through a Sherman-Morrison
//   solve of (I - dt (L - 2 L v v^T)) (householderDenum, :320-339);
//   torque = rhsStart - rhsEnd - l L v, projected orthogonal to v, rotates v; v is renormalised.
// The reference's loop over fields weighs the *first* field's rhsStart/rhsEnd for every field
// (rhsStart[j], j < NumNodes); this implementation does the same.
//
// Device form.  All vectors stay as half spectra in the context's layout S[z][kx][y]:
//   - the shifted fields are T +- (l/2X) FFT_x(v), since T = FFT_x(c)/X (the partial inverse of
//     c-hat/N), so the shift costs one complex axpy instead of a round trip to real space;
//   - every inner product of the reference, sum over all N modes of a(k) conj(b(k)) / N, is a
//     product of two Hermitian spectra: sum over the half spectrum with weight 2 for
//     0 < kx < X/2 and 1 on the kx = 0 and kx = X/2 planes (which hold both k and -k) of
//     Re(a conj b).  One reduction pass gathers every sum a step needs, in FP64;
//   - the update and the torque are elementwise; the torque goes to real space through the
//     usual inverse passes.
// The sequence is host-driven (about 25 launches per step, no graph): SDD is a saddle search,
// not the time-stepping hot loop.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gopf_ctx.h"
#include "gopf_kernels.cuh"

using namespace gopf;

namespace {

constexpr int SDD_NB = 152 * 2;  // reduction blocks per field
constexpr int SDD_NQ = 8;        // partial-sum slots per block and field
enum { Q_A = 0, Q_B, Q_C, Q_D, Q_E, Q_P, Q_DIFF2, Q_DMAX };
enum { G_ETOT = 0, G_VN2 = 1, G_SLOTS = 4 };
enum { M_MAXFORCE = 0, M_FPS = 1, M_MAXTORQUE = 2, M_FNORM = 3, M_FNORMCHG = 4 };

struct Sym { // GetDenum of one equation: L(m) = sum_p imp[p] m^p, m = -k^2
    int nimp;
    double imp[GOPF_MAX_IMP];
};
struct SymSet {
    Sym s[GOPF_MAX_FIELDS];
};
template <typename V> struct Ptrs {
    V *p[GOPF_MAX_FIELDS];
};

// m = -(2 pi |f|)^2 and the Hermitian weight of half-spectrum element i
__device__ __forceinline__ void mode_of(long long i, const Geom &g, double &m, double &w)
{
    const long long z = i / g.S, rem = i - z * g.S;
    const int kx = (int)(rem / g.Y), y = (int)(rem - (long long)kx * g.Y);
    const int yy = (2 * y > g.Y) ? g.Y - y : y;
    const int zz = (2 * z > g.Z) ? g.Z - (int)z : (int)z;
    const double fx = (double)kx / (double)g.X, fy = (double)yy / (double)g.Y, fz = (double)zz / (double)g.Z;
    m = -39.478417604357434475337963999504 * (fx * fx + fy * fy + fz * fz);
    w = (kx == 0 || 2 * kx == g.X) ? 1.0 : 2.0;
}

__device__ __forceinline__ double sym_eval(const Sym &s, double m)
{
    double L = 0.0;
    for (int q = s.nimp - 1; q >= 0; --q) L = L * m + s.imp[q];
    return L;
}

// block sum (slots < nsum) and max (slot nsum, if any) of SDD_NQ doubles into out[0..]
__device__ void block_reduce(double (&v)[SDD_NQ], int nsum, bool with_max, double *out)
{
    __shared__ double sh[32][SDD_NQ];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int q = 0; q < SDD_NQ; ++q) {
        double x = v[q];
        for (int o = 16; o > 0; o >>= 1) {
            const double y = __shfl_xor_sync(0xffffffffu, x, o);
            x = (with_max && q == nsum) ? fmax(x, y) : x + y;
        }
        if (lane == 0) sh[warp][q] = x;
    }
    __syncthreads();
    if (threadIdx.x < SDD_NQ) {
        const int q = threadIdx.x;
        double x = sh[0][q];
        for (int k = 1; k < nw; ++k) x = (with_max && q == nsum) ? fmax(x, sh[k][q]) : x + sh[k][q];
        out[q] = x;
    }
    __syncthreads();
}

// Ts_f = T_f + a Xv_f
template <typename V>
__global__ void k_sdd_shift(Ptrs<V> Ts, Ptrs<const V> T, Ptrs<const V> Xv, double a, long long C)
{
    const int f = blockIdx.y;
    V *__restrict__ o = Ts.p[f];
    const V *__restrict__ t = T.p[f];
    const V *__restrict__ x = Xv.p[f];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < C; i += (long long)gridDim.x * blockDim.x) {
        const V u = t[i], w = x[i];
        o[i].x = u.x + a * w.x;
        o[i].y = u.y + a * w.y;
    }
}

// rhs = sum_b m^glap[b] U_b (GetRHS of one equation from its forward-transformed groups)
template <typename V>
__global__ void k_sdd_combine(V *__restrict__ rhs, Ptrs<const V> U, int ngrp, int4 glap, Geom g)
{
    const int lp[4] = {glap.x, glap.y, glap.z, glap.w};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < g.C; i += (long long)gridDim.x * blockDim.x) {
        double m, w;
        mode_of(i, g, m, w);
        double rx = 0.0, ry = 0.0;
        for (int b = 0; b < ngrp; ++b) {
            double s = 1.0;
            for (int q = 0; q < lp[b]; ++q) s *= m;
            const V u = U.p[b][i];
            rx += s * (double)u.x;
            ry += s * (double)u.y;
        }
        rhs[i].x = rx;
        rhs[i].y = ry;
    }
}

// Every inner product of one step, per field f = blockIdx.y (weights of the half spectrum):
//   A = <work, v>, B = <v, L invD v>, C = <v, L invD c>, D = <v, L invD work>,
//   E = <rs_f - re_f - l L v, v>, P = <c, c>;   work = alpha rs_0 + (1 - alpha) re_0
template <typename V>
__global__ void k_sdd_reduce(Ptrs<const V> rs, Ptrs<const V> re, Ptrs<const V> vh, Ptrs<const V> st, SymSet K,
                             double alpha, double dt, double l, Geom g, double *__restrict__ part)
{
    const int f = blockIdx.y;
    const V *__restrict__ rs0 = rs.p[0], *__restrict__ re0 = re.p[0];
    const V *__restrict__ rsf = rs.p[f], *__restrict__ ref = re.p[f];
    const V *__restrict__ v = vh.p[f], *__restrict__ c = st.p[f];
    double acc[SDD_NQ] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < g.C; i += (long long)gridDim.x * blockDim.x) {
        double m, w;
        mode_of(i, g, m, w);
        const double L = sym_eval(K.s[f], m), Li = L / (1.0 - dt * L);
        const double wx = alpha * (double)rs0[i].x + (1.0 - alpha) * (double)re0[i].x;
        const double wy = alpha * (double)rs0[i].y + (1.0 - alpha) * (double)re0[i].y;
        const double vx = v[i].x, vy = v[i].y, cx = c[i].x, cy = c[i].y;
        const double tx = (double)rsf[i].x - (double)ref[i].x - l * L * vx;
        const double ty = (double)rsf[i].y - (double)ref[i].y - l * L * vy;
        acc[Q_A] += w * (wx * vx + wy * vy);
        acc[Q_B] += w * Li * (vx * vx + vy * vy);
        acc[Q_C] += w * Li * (vx * cx + vy * cy);
        acc[Q_D] += w * Li * (vx * wx + vy * wy);
        acc[Q_E] += w * (tx * vx + ty * vy);
        acc[Q_P] += w * (cx * cx + cy * cy);
    }
    double out[SDD_NQ];
    block_reduce(acc, SDD_NQ, false, out);
    if (threadIdx.x < SDD_NQ) part[((long long)f * gridDim.x + blockIdx.x) * SDD_NQ + threadIdx.x] = out[threadIdx.x];
}

// Sums of the per-block partials: scal[f*8 + q] for the slots [q0, q1); slot qmax (>= 0) is a
// maximum.  Then the step's globals: mode 0 -> E total and the field norm monitors,
// mode 1 -> the force monitors.
__global__ void k_sdd_finish(const double *__restrict__ part, int nf, int nb, int q0, int q1, int qmax,
                             double *__restrict__ scal, double *__restrict__ mon, long long N, int mode)
{
    __shared__ double sh[256];
    for (int f = 0; f < nf; ++f)
        for (int q = q0; q < q1; ++q) {
            double x = 0.0; // sums, or maxima of non-negative values
            for (int b = threadIdx.x; b < nb; b += blockDim.x) {
                const double y = part[((long long)f * nb + b) * SDD_NQ + q];
                x = (q == qmax) ? fmax(x, y) : x + y;
            }
            sh[threadIdx.x] = x;
            __syncthreads();
            for (int s = blockDim.x / 2; s > 0; s >>= 1) {
                if (threadIdx.x < s)
                    sh[threadIdx.x] = (q == qmax) ? fmax(sh[threadIdx.x], sh[threadIdx.x + s]) : sh[threadIdx.x] + sh[threadIdx.x + s];
                __syncthreads();
            }
            if (threadIdx.x == 0) scal[f * SDD_NQ + q] = sh[0];
            __syncthreads();
        }
    if (threadIdx.x != 0) return;
    double *glob = scal + nf * SDD_NQ;
    if (mode == 0) {
        double E = 0.0, P = 0.0;
        for (int f = 0; f < nf; ++f) {
            E += scal[f * SDD_NQ + Q_E];
            P += scal[f * SDD_NQ + Q_P];
        }
        glob[G_ETOT] = E;
        const double fnorm = P / (double)N; // Parseval: sum_x c^2 = sum_k |c-hat|^2 / N
        mon[M_FNORMCHG] = mon[M_FNORM] - fnorm;
        mon[M_FNORM] = fnorm;
    } else {
        double S = 0.0, mx = 0.0;
        for (int f = 0; f < nf; ++f) {
            S += scal[f * SDD_NQ + Q_DIFF2];
            mx = fmax(mx, scal[f * SDD_NQ + Q_DMAX]);
        }
        mon[M_MAXFORCE] = mx;
        mon[M_FPS] = sqrt(S / (double)N / (double)(nf * N));
    }
}

// The centre's update and the torque, per field f = blockIdx.y:
//   d = c + dt (work - 2 <work,v>/N v);  c <- invD (d - v num/den),
//   den = 1 + 2 dt B/N,  num = 2 dt/N (C + dt D - 2 dt (A/N) B)     (Sherman-Morrison)
//   tq = (rs_f - re_f - l L v - v E/N) / N  (into Tq, ready for the inverse passes)
// plus the force monitors |c_new - c|/dt.  T receives c_new/N for the inverse passes.
template <typename V>
__global__ void k_sdd_update(Ptrs<const V> rs, Ptrs<const V> re, Ptrs<const V> vh, Ptrs<V> st, Ptrs<V> T, Ptrs<V> Tq,
                             SymSet K, double alpha, double dt, double l, Geom g, const double *__restrict__ scal,
                             int nf, double *__restrict__ part)
{
    const int f = blockIdx.y;
    const double invN = 1.0 / (double)g.N;
    const double *sf = scal + f * SDD_NQ;
    const double Etot = scal[nf * SDD_NQ + G_ETOT];
    const double dot = sf[Q_A] * invN;
    const double den = 1.0 + 2.0 * dt * sf[Q_B] * invN;
    const double num = 2.0 * dt * invN * (sf[Q_C] + dt * sf[Q_D] - 2.0 * dt * dot * sf[Q_B]);
    const double qv = num / den;
    const V *__restrict__ rs0 = rs.p[0], *__restrict__ re0 = re.p[0];
    const V *__restrict__ rsf = rs.p[f], *__restrict__ ref = re.p[f];
    const V *__restrict__ v = vh.p[f];
    V *__restrict__ c = st.p[f];
    V *__restrict__ t = T.p[f];
    V *__restrict__ tq = Tq.p[f];
    double acc[SDD_NQ] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < g.C; i += (long long)gridDim.x * blockDim.x) {
        double m, w;
        mode_of(i, g, m, w);
        const double L = sym_eval(K.s[f], m), invD = 1.0 / (1.0 - dt * L);
        const double wx = alpha * (double)rs0[i].x + (1.0 - alpha) * (double)re0[i].x;
        const double wy = alpha * (double)rs0[i].y + (1.0 - alpha) * (double)re0[i].y;
        const double vx = v[i].x, vy = v[i].y, cx = c[i].x, cy = c[i].y;
        const double dx = cx + dt * (wx - 2.0 * dot * vx), dy = cy + dt * (wy - 2.0 * dot * vy);
        const double nx = invD * (dx - qv * vx), ny = invD * (dy - qv * vy);
        const double fx = (nx - cx) / dt, fy = (ny - cy) / dt;
        const double d2 = fx * fx + fy * fy;
        acc[0] += w * d2;
        acc[1] = fmax(acc[1], sqrt(d2));
        c[i].x = nx;
        c[i].y = ny;
        t[i].x = nx * invN;
        t[i].y = ny * invN;
        const double tx = (double)rsf[i].x - (double)ref[i].x - l * L * vx - vx * Etot * invN;
        const double ty = (double)rsf[i].y - (double)ref[i].y - l * L * vy - vy * Etot * invN;
        tq[i].x = tx * invN;
        tq[i].y = ty * invN;
    }
    double out[SDD_NQ];
    block_reduce(acc, 1, true, out);
    if (threadIdx.x < 2) part[((long long)f * gridDim.x + blockIdx.x) * SDD_NQ + Q_DIFF2 + threadIdx.x] = out[threadIdx.x];
}

// v -= dt tq / (l tau); partial sums of |v|^2 and max |tq| (all fields in one vector)
template <typename R>
__global__ void k_sdd_orient(R *__restrict__ v, const R *__restrict__ tq, long long n, double s, double *__restrict__ part)
{
    double acc[SDD_NQ] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double t = (double)tq[i];
        const R nv = (R)((double)v[i] - s * t);
        v[i] = nv;
        acc[0] += (double)nv * (double)nv;
        acc[1] = fmax(acc[1], fabs(t));
    }
    double out[SDD_NQ];
    block_reduce(acc, 1, true, out);
    if (threadIdx.x < 2) part[(long long)blockIdx.x * SDD_NQ + threadIdx.x] = out[threadIdx.x];
}

// total |v|^2 and max |tq| of k_sdd_orient's partials
__global__ void k_sdd_finish_orient(const double *__restrict__ part, int nb, double *__restrict__ glob,
                                    double *__restrict__ mon)
{
    __shared__ double s0[256], s1[256];
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) {
        a += part[(long long)k * SDD_NQ];
        b = fmax(b, part[(long long)k * SDD_NQ + 1]);
    }
    s0[threadIdx.x] = a;
    s1[threadIdx.x] = b;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            s0[threadIdx.x] += s0[threadIdx.x + s];
            s1[threadIdx.x] = fmax(s1[threadIdx.x], s1[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        glob[G_VN2] = s0[0];
        mon[M_MAXTORQUE] = s1[0];
    }
}

template <typename R> __global__ void k_sdd_normalise(R *__restrict__ v, long long n, const double *__restrict__ glob)
{
    const double inv = 1.0 / sqrt(glob[G_VN2]);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        v[i] = (R)((double)v[i] * inv);
}

unsigned ew_grid(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 152 * 8); }

} // namespace

struct gopf_sdd_work {
    int nf = 0;
    int prec = 0;
    long long N = 0, C = 0;
    void *d_v = nullptr;  // orientation, nf * N reals (node order, field after field)
    void *d_tq = nullptr; // torque in real space, nf * N
    void *d_Xv[GOPF_MAX_FIELDS] = {}, *d_Vh[GOPF_MAX_FIELDS] = {}, *d_rs[GOPF_MAX_FIELDS] = {},
         *d_re[GOPF_MAX_FIELDS] = {}, *d_Ts[GOPF_MAX_FIELDS] = {};
    double *d_part = nullptr; // nf * SDD_NB * SDD_NQ
    double *d_scal = nullptr; // nf * SDD_NQ + G_SLOTS
    double *d_mon = nullptr;  // SDDMonitor
    bool oriented = false;
};

static void sdd_free(gopf_sdd_work *w)
{
    if (!w) return;
    void *ptrs[] = {w->d_v, w->d_tq, w->d_part, w->d_scal, w->d_mon};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (int f = 0; f < GOPF_MAX_FIELDS; ++f) {
        void *q[] = {w->d_Xv[f], w->d_Vh[f], w->d_rs[f], w->d_re[f], w->d_Ts[f]};
        for (void *p : q)
            if (p) cudaFree(p);
    }
    delete w;
}

void gopf_sdd_free(gopf_ctx *ctx)
{
    sdd_free(ctx->sdd);
    ctx->sdd = nullptr;
}

// workspace for the context's current model (re-made when the field count or precision changed)
static int sdd_work(gopf_ctx *ctx, gopf_sdd_work **out)
{
    if (ctx->device < 0) return gopf_fail(ctx, GOPF_ERR_STATE, "host-only context");
    if (!ctx->initialised) return gopf_fail(ctx, GOPF_ERR_STATE, "model not initialised (gopf_init/gopf_set_terms)");
    const int nf = std::max(ctx->nfields, 1);
    gopf_sdd_work *w = ctx->sdd;
    if (w && w->nf == nf && w->prec == ctx->prec) {
        *out = w;
        return GOPF_OK;
    }
    gopf_sdd_free(ctx);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return gopf_fail(ctx, GOPF_ERR_CUDA, "cudaSetDevice");
    w = new gopf_sdd_work();
    ctx->sdd = w;
    w->nf = nf;
    w->prec = ctx->prec;
    w->N = ctx->g.N;
    w->C = ctx->g.C;
    const size_t rb = (ctx->prec == GOPF_FP32) ? 4 : 8, vb = 2 * rb;
    auto al = [&](void **p, size_t bytes) -> int {
        cudaError_t e = gopf_malloc(p, bytes);
        if (e != cudaSuccess) return gopf_fail(ctx, GOPF_ERR_OOM, "gopf_malloc(SDD workspace)");
        ctx->dev_bytes += bytes;
        return GOPF_OK;
    };
    int rc;
    if ((rc = al(&w->d_v, rb * (size_t)(nf * w->N)))) return rc;
    if ((rc = al(&w->d_tq, rb * (size_t)(nf * w->N)))) return rc;
    for (int f = 0; f < nf; ++f) {
        void **arrs[] = {&w->d_Xv[f], &w->d_Vh[f], &w->d_rs[f], &w->d_re[f], &w->d_Ts[f]};
        for (void **p : arrs)
            if ((rc = al(p, vb * (size_t)w->C))) return rc;
    }
    if ((rc = al(reinterpret_cast<void **>(&w->d_part), sizeof(double) * (size_t)nf * SDD_NB * SDD_NQ))) return rc;
    if ((rc = al(reinterpret_cast<void **>(&w->d_scal), sizeof(double) * (size_t)(nf * SDD_NQ + G_SLOTS)))) return rc;
    if ((rc = al(reinterpret_cast<void **>(&w->d_mon), sizeof(double) * 5))) return rc;
    if (cudaMemset(w->d_mon, 0, sizeof(double) * 5) != cudaSuccess) return gopf_fail(ctx, GOPF_ERR_CUDA, "memset");
    *out = w;
    return GOPF_OK;
}

// A unit orientation from host values (field after field); returns its length.
static int sdd_set_orientation(gopf_ctx *ctx, const std::vector<double> &v)
{
    gopf_sdd_work *w = nullptr;
    int rc;
    if ((rc = sdd_work(ctx, &w))) return rc;
    if ((long long)v.size() != w->nf * w->N)
        return gopf_fail(ctx, GOPF_ERR_ARG, "orientation length must be nfields * number of nodes");
    double len = 0.0;
    for (double x : v) len += x * x;
    len = std::sqrt(len);
    if (!(len > 0.0) || !std::isfinite(len)) return gopf_fail(ctx, GOPF_ERR_ARG, "orientation has zero or non-finite length");
    ctx->sdd_init_len = len;
    cudaError_t e;
    if (ctx->prec == GOPF_FP32) {
        std::vector<float> h(v.size());
        for (size_t i = 0; i < v.size(); ++i) h[i] = (float)(v[i] / len);
        e = cudaMemcpy(w->d_v, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice);
    } else {
        std::vector<double> h(v.size());
        for (size_t i = 0; i < v.size(); ++i) h[i] = v[i] / len;
        e = cudaMemcpy(w->d_v, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) return gopf_fail(ctx, GOPF_ERR_CUDA, cudaGetErrorString(e));
    if (cudaMemset(w->d_mon, 0, sizeof(double) * 5) != cudaSuccess) return gopf_fail(ctx, GOPF_ERR_CUDA, "memset");
    w->oriented = true;
    ctx->sdd_step = 0; // a new dimer starts at time 0 (NewSDD)
    return GOPF_OK;
}

extern "C" int gopf_sdd_init(gopf_ctx *ctx, const double *init, const double *final, size_t n)
{
    if (!ctx || !init || !final) return gopf_fail(ctx, GOPF_ERR_ARG, "null argument");
    std::vector<double> v(n);
    for (size_t i = 0; i < n; ++i) v[i] = final[i] - init[i];
    return sdd_set_orientation(ctx, v);
}

extern "C" int gopf_sdd_set_orientation(gopf_ctx *ctx, const double *orient, size_t n)
{
    if (!ctx || !orient) return gopf_fail(ctx, GOPF_ERR_ARG, "null argument");
    return sdd_set_orientation(ctx, std::vector<double>(orient, orient + n));
}

extern "C" int gopf_sdd_set_params(gopf_ctx *ctx, double alpha, double tau_orientation, double tau_length,
                                   double init_length, double min_length)
{
    if (!ctx) return GOPF_ERR_ARG;
    if (!(tau_orientation > 0.0) || !(tau_length > 0.0) || !(min_length >= 0.0) || !std::isfinite(alpha))
        return gopf_fail(ctx, GOPF_ERR_ARG, "SDD time constants must be positive and the minimum length >= 0");
    ctx->sdd_alpha = alpha;
    ctx->sdd_tau_orient = tau_orientation;
    ctx->sdd_tau_len = tau_length;
    if (init_length > 0.0) ctx->sdd_init_len = init_length;
    ctx->sdd_min_len = min_length;
    return GOPF_OK;
}

static double dimer_length(const gopf_ctx *ctx, double t)
{
    const double l = ctx->sdd_init_len * std::exp(-t / ctx->sdd_tau_len);
    return (l < ctx->sdd_min_len) ? ctx->sdd_min_len : l;
}

extern "C" int gopf_sdd_dimer_length(gopf_ctx *ctx, double t, double *l)
{
    if (!ctx || !l) return GOPF_ERR_ARG;
    *l = dimer_length(ctx, t);
    return GOPF_OK;
}

extern "C" int gopf_sdd_get_orientation(gopf_ctx *ctx, double *out, size_t n)
{
    if (!ctx || !out) return gopf_fail(ctx, GOPF_ERR_ARG, "null argument");
    gopf_sdd_work *w = ctx->sdd;
    if (!w || !w->oriented) return gopf_fail(ctx, GOPF_ERR_STATE, "no orientation set (gopf_sdd_init)");
    if ((long long)n != w->nf * w->N) return gopf_fail(ctx, GOPF_ERR_ARG, "orientation length mismatch");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return gopf_fail(ctx, GOPF_ERR_CUDA, "cudaSetDevice");
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return gopf_fail(ctx, GOPF_ERR_CUDA, "synchronize");
    cudaError_t e;
    if (ctx->prec == GOPF_FP32) {
        std::vector<float> h(n);
        e = cudaMemcpy(h.data(), w->d_v, sizeof(float) * n, cudaMemcpyDeviceToHost);
        for (size_t i = 0; i < n; ++i) out[i] = h[i];
    } else {
        e = cudaMemcpy(out, w->d_v, sizeof(double) * n, cudaMemcpyDeviceToHost);
    }
    return (e == cudaSuccess) ? GOPF_OK : gopf_fail(ctx, GOPF_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" int gopf_sdd_monitor(gopf_ctx *ctx, double *out5)
{
    if (!ctx || !out5) return gopf_fail(ctx, GOPF_ERR_ARG, "null argument");
    gopf_sdd_work *w = ctx->sdd;
    if (!w) return gopf_fail(ctx, GOPF_ERR_STATE, "no SDD run on this context");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return gopf_fail(ctx, GOPF_ERR_CUDA, "cudaSetDevice");
    cudaError_t e = cudaMemcpyAsync(out5, w->d_mon, sizeof(double) * 5, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return (e == cudaSuccess) ? GOPF_OK : gopf_fail(ctx, GOPF_ERR_CUDA, cudaGetErrorString(e));
}

// ---- one step ----

template <typename R> static XPassArgs<R> sdd_xargs(gopf_ctx *ctx)
{
    XPassArgs<R> a;
    memset(&a, 0, sizeof(a));
    a.g = ctx->g;
    a.planH = ctx->planH;
    a.twX = (const typename VecOf<R>::type *)ctx->d_twX;
    a.allow_fast = ctx->use_fast ? (ctx->use_tma ? 3 : 1) : 0;
    a.status = ctx->d_status;
    return a;
}

template <typename R> static PassArgs<R> sdd_pargs(gopf_ctx *ctx, bool zaxis, int mode)
{
    PassArgs<R> a;
    memset(&a, 0, sizeof(a));
    a.g = ctx->g;
    a.plan = zaxis ? ctx->planZ : ctx->planY;
    a.tw = (const typename VecOf<R>::type *)(zaxis ? ctx->d_twZ : ctx->d_twY);
    a.mode = mode;
    a.allow_fast = ctx->use_fast ? (ctx->use_tma ? 3 : 1) : 0;
    a.status = ctx->d_status;
    return a;
}

#define SK(call)                                                                                                       \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess) return e_;                                                                              \
    } while (0)

// forward (FWD) or inverse (INV) transform of nb spectral arrays along y and, in 3D, z
template <typename R> static cudaError_t yz_pass(gopf_ctx *ctx, int mode, typename VecOf<R>::type *const *bufs, int nb)
{
    const bool is3d = ctx->g.Z > 1;
    for (int b0 = 0; b0 < nb; b0 += GOPF_MAX_GROUPS) {
        const int k = std::min(GOPF_MAX_GROUPS, nb - b0);
        PassArgs<R> ya = sdd_pargs<R>(ctx, false, mode), za = sdd_pargs<R>(ctx, true, mode);
        for (int b = 0; b < k; ++b) ya.buf[b] = za.buf[b] = bufs[b0 + b];
        ya.nbuf = za.nbuf = k;
        if (mode == PM_FWD) {
            SK(launch_cpass<R>(ya, ctx->LBy, ctx->stream));
            if (is3d) SK(launch_spass<R>(za, ctx->LBz, ctx->stream));
        } else {
            if (is3d) SK(launch_spass<R>(za, ctx->LBz, ctx->stream));
            SK(launch_cpass<R>(ya, ctx->LBy, ctx->stream));
        }
    }
    return cudaSuccess;
}

// GetRHS of every equation at the shifted fields Ts (overwritten) into out[f]
template <typename R> static cudaError_t sdd_rhs(gopf_ctx *ctx, gopf_sdd_work *w, void *const *out)
{
    typedef typename VecOf<R>::type V;
    const int nf = w->nf;
    const Geom &g = ctx->g;
    const unsigned grid = ew_grid(g.C);
    if (!ctx->multi) {
        const int G = ctx->ngroups;
        V *U[GOPF_MAX_GROUPS];
        U[0] = (V *)w->d_Ts[0];
        for (int b = 1; b < GOPF_MAX_GROUPS; ++b) U[b] = (V *)ctx->d_U[b];
        if (G > 0) {
            XPassArgs<R> xa = sdd_xargs<R>(ctx);
            xa.in_mode = XIN_SPECTRAL;
            xa.in = U[0];
            for (int b = 0; b < G; ++b) xa.out[b] = U[b];
            xa.ngrp_out = G;
            xa.pw = ctx->pw;
            SK(launch_xpass<R>(xa, ctx->LBx, ctx->stream));
            SK(yz_pass<R>(ctx, PM_FWD, U, G));
        }
        Ptrs<const V> up;
        for (int b = 0; b < GOPF_MAX_FIELDS; ++b) up.p[b] = (b < G) ? U[b] : nullptr;
        const int4 gl = make_int4(ctx->upd.glap[0], ctx->upd.glap[1], ctx->upd.glap[2], ctx->upd.glap[3]);
        k_sdd_combine<V><<<grid, 256, 0, ctx->stream>>>((V *)out[0], up, G, gl, g);
        return cudaGetLastError();
    }
    // several fields: the RK4 plan (every field term from the shifted fields themselves)
    const std::vector<gopf_ctx::EqPlan> &eqs = ctx->eqs_rk;
    auto gbuf = [&](int e, int b) -> V * {
        const int k = eqs[e].ubuf[b];
        return (V *)(k < 0 ? w->d_Ts[e] : ctx->d_mU[k]);
    };
    if (ctx->mono_rk.ngrp > 0) {
        XPassArgs<R> xa = sdd_xargs<R>(ctx);
        xa.in_mode = XIN_SPECTRAL;
        xa.program = XP_MULTI;
        xa.allow_fast = 0;
        for (int f = 0; f < nf; ++f) xa.inF[f] = (const V *)w->d_Ts[f];
        for (int e = 0; e < nf; ++e)
            for (int b = 0; b < eqs[e].upd.ngrp; ++b) xa.out[eqs[e].first + b] = gbuf(e, b);
        xa.ngrp_out = ctx->mono_rk.ngrp;
        xa.mono = ctx->mono_rk;
        SK(launch_xpass<R>(xa, ctx->LBm, ctx->stream));
    }
    for (int e = 0; e < nf; ++e) {
        const int G = eqs[e].upd.ngrp;
        V *U[GOPF_MAX_GROUPS];
        for (int b = 0; b < G; ++b) U[b] = gbuf(e, b);
        if (G > 0) SK(yz_pass<R>(ctx, PM_FWD, U, G));
        Ptrs<const V> up;
        for (int b = 0; b < GOPF_MAX_FIELDS; ++b) up.p[b] = (b < G) ? U[b] : nullptr;
        const int *gl0 = eqs[e].upd.glap;
        k_sdd_combine<V><<<grid, 256, 0, ctx->stream>>>((V *)out[e], up, G, make_int4(gl0[0], gl0[1], gl0[2], gl0[3]), g);
        SK(cudaGetLastError());
    }
    return cudaSuccess;
}

template <typename R> static cudaError_t sdd_step_once(gopf_ctx *ctx, gopf_sdd_work *w)
{
    typedef typename VecOf<R>::type V;
    const int nf = w->nf;
    const Geom &g = ctx->g;
    const long long N = g.N;
    const double dt = ctx->dt;
    const double t = (double)ctx->sdd_step * dt;
    const double l = dimer_length(ctx, t);
    const unsigned grid = ew_grid(g.C);
    cudaStream_t st = ctx->stream;

    // FFT of the orientation: Xv = FFT_x(v) and v-hat
    for (int f = 0; f < nf; ++f) {
        XPassArgs<R> xa = sdd_xargs<R>(ctx);
        xa.in_mode = XIN_REAL;
        xa.rin = (const R *)w->d_v + (long long)f * N;
        xa.out[0] = (V *)w->d_Xv[f];
        xa.ngrp_out = 1;
        xa.identity = 1;
        SK(launch_xpass<R>(xa, ctx->LBx, st));
        SK(cudaMemcpyAsync(w->d_Vh[f], w->d_Xv[f], sizeof(V) * (size_t)g.C, cudaMemcpyDeviceToDevice, st));
    }
    {
        V *vh[GOPF_MAX_FIELDS];
        for (int f = 0; f < nf; ++f) vh[f] = (V *)w->d_Vh[f];
        SK(yz_pass<R>(ctx, PM_FWD, vh, nf));
    }
    Ptrs<V> Ts, Tf, Sf;
    Ptrs<const V> Tc, Xc, RS, RE, VH, SC;
    for (int f = 0; f < GOPF_MAX_FIELDS; ++f) {
        const bool in = f < nf;
        Ts.p[f] = in ? (V *)w->d_Ts[f] : nullptr;
        Tf.p[f] = in ? (V *)field_T(ctx, f) : nullptr;
        Sf.p[f] = in ? (V *)field_state(ctx, f) : nullptr;
        Tc.p[f] = Tf.p[f];
        Xc.p[f] = in ? (const V *)w->d_Xv[f] : nullptr;
        RS.p[f] = in ? (const V *)w->d_rs[f] : nullptr;
        RE.p[f] = in ? (const V *)w->d_re[f] : nullptr;
        VH.p[f] = in ? (const V *)w->d_Vh[f] : nullptr;
        SC.p[f] = Sf.p[f];
    }
    // right-hand sides at the dimer's ends: T -/+ (l/2) T_v, T_v = FFT_x(v) / X
    const dim3 eg(grid, nf);
    k_sdd_shift<V><<<eg, 256, 0, st>>>(Ts, Tc, Xc, -0.5 * l / (double)g.X, g.C);
    SK(cudaGetLastError());
    SK(sdd_rhs<R>(ctx, w, w->d_rs));
    k_sdd_shift<V><<<eg, 256, 0, st>>>(Ts, Tc, Xc, 0.5 * l / (double)g.X, g.C);
    SK(cudaGetLastError());
    SK(sdd_rhs<R>(ctx, w, w->d_re));

    SymSet K;
    memset(&K, 0, sizeof(K));
    for (int f = 0; f < nf; ++f) {
        const UpdTable &u = ctx->multi ? ctx->eqs_rk[f].upd : ctx->upd;
        K.s[f].nimp = u.nimp;
        for (int p = 0; p < u.nimp; ++p) K.s[f].imp[p] = u.imp[p];
    }
    const double alpha = ctx->sdd_alpha;
    k_sdd_reduce<V><<<dim3(SDD_NB, nf), 256, 0, st>>>(RS, RE, VH, SC, K, alpha, dt, l, g, w->d_part);
    SK(cudaGetLastError());
    k_sdd_finish<<<1, 256, 0, st>>>(w->d_part, nf, SDD_NB, Q_A, Q_P + 1, -1, w->d_scal, w->d_mon, N, 0);
    SK(cudaGetLastError());
    k_sdd_update<V><<<dim3(SDD_NB, nf), 256, 0, st>>>(RS, RE, VH, Sf, Tf, Ts, K, alpha, dt, l, g, w->d_scal, nf,
                                                      w->d_part);
    SK(cudaGetLastError());
    k_sdd_finish<<<1, 256, 0, st>>>(w->d_part, nf, SDD_NB, Q_DIFF2, Q_DMAX + 1, Q_DMAX, w->d_scal, w->d_mon, N, 1);
    SK(cudaGetLastError());

    // the new centre: projection of each c-hat, then T = partial inverse of c-hat/N
    for (int f = 0; f < nf; ++f) SK(gopf_launch_hermitian_planes(ctx, field_state(ctx, f), st));
    {
        V *bufs[GOPF_MAX_FIELDS * 2];
        for (int f = 0; f < nf; ++f) {
            bufs[f] = (V *)field_T(ctx, f);
            bufs[nf + f] = (V *)w->d_Ts[f]; // the torque / N
        }
        SK(yz_pass<R>(ctx, PM_INV, bufs, 2 * nf));
    }
    // torque to real space, then the orientation update and renormalisation
    for (int f = 0; f < nf; ++f) {
        XPassArgs<R> xa = sdd_xargs<R>(ctx);
        xa.in_mode = XIN_SPECTRAL;
        xa.in = (const V *)w->d_Ts[f];
        xa.rout = (R *)w->d_tq + (long long)f * N;
        xa.ngrp_out = 0;
        SK(launch_xpass<R>(xa, ctx->LBx, st));
    }
    const long long nv = (long long)nf * N;
    const unsigned og = std::min<unsigned>(ew_grid(nv), SDD_NB);
    const double s = dt / (dimer_length(ctx, t) * ctx->sdd_tau_orient);
    k_sdd_orient<R><<<og, 256, 0, st>>>((R *)w->d_v, (const R *)w->d_tq, nv, s, w->d_part);
    SK(cudaGetLastError());
    k_sdd_finish_orient<<<1, 256, 0, st>>>(w->d_part, (int)og, w->d_scal + nf * SDD_NQ, w->d_mon);
    SK(cudaGetLastError());
    k_sdd_normalise<R><<<ew_grid(nv), 256, 0, st>>>((R *)w->d_v, nv, w->d_scal + nf * SDD_NQ);
    return cudaGetLastError();
}

int gopf_sdd_step(gopf_ctx *ctx, long long nsteps)
{
    gopf_sdd_work *w = ctx->sdd;
    if (!w || !w->oriented || w->nf != std::max(ctx->nfields, 1) || w->prec != ctx->prec)
        return gopf_fail(ctx, GOPF_ERR_STATE, "SDD: set the orientation first (gopf_sdd_init / gopf_sdd_set_orientation)");
    if (!(ctx->dt >= 1e-16)) return gopf_fail(ctx, GOPF_ERR_ARG, "SDD: time step not set");
    if (ctx->upd.nfilt) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "SDD: does not support modal filters");
    if (ctx->has_elastic || ctx->has_volcons || ctx->noise.kind)
        return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "SDD steps polynomial terms (no elastic, volume-conserving or noise term)");
    const int nf = w->nf;
    for (int f = 0; f < nf; ++f) {
        const UpdTable &u = ctx->multi ? ctx->eqs_rk[f].upd : ctx->upd;
        if (u.nxs) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "SDD: implicit user terms with a symbol are not supported");
    }
    if (ctx->g.N * (long long)nf > (1LL << 40)) return gopf_fail(ctx, GOPF_ERR_UNSUPPORTED, "SDD: domain too large");
    for (long long s = 0; s < nsteps; ++s) {
        cudaError_t e = (ctx->prec == GOPF_FP32) ? sdd_step_once<float>(ctx, w) : sdd_step_once<double>(ctx, w);
        if (e != cudaSuccess) return gopf_fail(ctx, GOPF_ERR_CUDA, std::string("SDD step: ") + cudaGetErrorString(e));
        ++ctx->sdd_step;
    }
    return GOPF_OK;
}
