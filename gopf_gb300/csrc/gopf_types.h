// gopf_types.h -- plain data structures shared by host code and kernels.
//
// Spectral layout in HBM (ours, not the reference's): a real field of the
// reference's domainSize [n0 rows, n1 cols, n2 depth] (node index
// depth*n0*n1 + row*n1 + col, pfutil/indexPositionConversion.go:23-34) is kept
// as its half spectrum S[z][kx][y] with kx in [0, n1/2] slowest inside a
// depth plane and the row frequency y fastest.  Every pass then reads either
// whole contiguous lines (the y axis) or 128-byte segments of LB consecutive
// y values (the kx and z axes).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gopf {

#define GOPF_MAX_STAGES 12

struct LinePlan {
    int n;       // complex line length
    int nst;     // number of stages
    int rad[GOPF_MAX_STAGES];
    int ns[GOPF_MAX_STAGES];     // product of the radices of earlier stages
    int nsmask[GOPF_MAX_STAGES]; // ns-1 when ns is a power of two, else -1
    int twmul[GOPF_MAX_STAGES];  // table index multiplier: W_{ns*R}^{q} = tw[q * twmul]
};


#define GOPF_MAX_GROUPS 4
#define GOPF_MAX_POLY 8
#define GOPF_MAX_IMP 9
// multi-field models: fields per model, spectral outputs of one x-pass, monomials per group
#define GOPF_MAX_FIELDS 4
#define GOPF_MAX_SRC 4
#define GOPF_MAX_XOUT 8
#define GOPF_MAX_MONO 8

struct Geom {
    int X, Y, Z; // cols (fastest real axis), rows, depth (1 in 2D)
    int H;       // X/2
    int KX;      // X/2 + 1
    long long S; // KX * Y
    long long C; // S * Z spectral elements
    long long N; // X * Y * Z cells
};

// Real-space pointwise polynomials g_g(c) = sum_t coef[g][t] * c^pw[g][t]
#define GOPF_MAX_DEG 12
struct PwTable {
    int ngrp;
    int nterm[GOPF_MAX_GROUPS];
    int pw[GOPF_MAX_GROUPS][GOPF_MAX_POLY];
    double coef[GOPF_MAX_GROUPS][GOPF_MAX_POLY];
    // the same polynomials in dense form for Horner evaluation (deg < 0: not representable)
    int deg[GOPF_MAX_GROUPS];
    double dense[GOPF_MAX_GROUPS][GOPF_MAX_DEG + 1];
};

// Fill deg/dense from the sparse terms.
inline void pw_densify(PwTable &pw)
{
    for (int g = 0; g < GOPF_MAX_GROUPS; ++g) {
        for (int q = 0; q <= GOPF_MAX_DEG; ++q) pw.dense[g][q] = 0.0;
        int d = 0;
        bool ok = true;
        for (int t = 0; t < pw.nterm[g]; ++t) {
            if (pw.pw[g][t] < 0 || pw.pw[g][t] > GOPF_MAX_DEG) ok = false;
            else {
                pw.dense[g][pw.pw[g][t]] += pw.coef[g][t];
                if (pw.pw[g][t] > d) d = pw.pw[g][t];
            }
        }
        pw.deg[g] = ok ? d : -1;
    }
}

// Real-space pointwise polynomials of several fields (multi-field models):
//   g_j(c_0, .., c_{nin-1}) = sum_m coef[j][m] * prod_f c_f^pw[j][m][f]
// One output group j per (equation, LAP power); the products are the derived fields of
// pf/util.go:38-65 with factors from different fields.
struct MonoTable {
    int nin;  // fields read
    int ngrp; // output groups
    int nmono[GOPF_MAX_XOUT];
    double coef[GOPF_MAX_XOUT][GOPF_MAX_MONO];
    unsigned char pw[GOPF_MAX_XOUT][GOPF_MAX_MONO][GOPF_MAX_FIELDS];
};

// k-space Gaussian noise term (white or conservative), drawn per mode and step
struct NoiseParams {
    int kind;            // 0 none, 1 white (derived field), 2 conservative (D current components)
    int ndim;
    double coef;         // sign * scalars of the term
    int lap;             // LAP power of the term
    double amp;          // sqrt(N * 2S): standard deviation of |x(k)| of a complex mode
    uint32_t seed_lo, seed_hi;
    const unsigned long long *step; // device step counter
};

// Implicit user terms with a per-frequency symbol (added to the denominator sum L):
//   kind 1: TensorialHessian (pf/tensorialHessian.go:38-70): sum_j -4 pi^2 f_j^2 K_jj + sum_{j<k} -8 pi^2 f_j f_k K_jk
//   kind 2: SpectralViscosity (pf/spectralViscosity.go:22-58): -eps * Q(|f|; threshold) * |f|^power
// f in cycles per sample in the reference's order (row, col, depth); the term's sign and LAP
// prefixes give coef * m^lap.
#define GOPF_MAX_XSYM 4
struct XSym {
    int kind;
    double coef;
    int lap;
    double K[9];
    int dk; // 2 or 3: the tensor's dimension
    double eps, threshold;
    int power;
};

// k-space update: c_new = (c + dt * sum_g m^glap[g] U_g) / (1 - dt * sum_p imp[p] m^p),  m = -k^2
struct UpdTable {
    double dt;
    double invN;
    int nimp;                    // number of coefficients in imp (degree + 1)
    double imp[GOPF_MAX_IMP];
    int ngrp;
    int glap[GOPF_MAX_GROUPS];
    // optional device-resident scale of a group (the volume-conserving Lagrange
    // multiplier, updated on the device every step); nullptr = 1
    const double *gscale[GOPF_MAX_GROUPS];
    // RK4 stage (pf/rk4.go:29-127); 0 = Euler.  With k the explicit RHS of this stage:
    //   stage 1: F = c + afin k          else F += afin k
    //   stage < 4: next = (c + ay k) / (1 - fden L)      stage 4: c = F / (1 - dt L)
    int rk_stage;
    double rk_afin, rk_ay, rk_fden;
    NoiseParams noise;
    // ImplicitEuler (pf/implicitEuler.go:68-162); 0 = off.  With N the explicit RHS of the groups:
    //   etd == 1: rkF <- N (the RHS at the step's start), the state is not changed
    //   etd == 2: buf[ngrp] holds FFT(x); tile <- (FFT(x) - c e^(L dt) - I(L, N, rkF)) / N for the
    //             inverse pass (the Newton residual); the state is not changed
    int etd;
    // optional modal filter (pf/util.go:125-132): the updated c-hat is multiplied by
    // filter(2|f|/pi), a table of nfilt samples on [0, 1] (R elements, device memory)
    const void *filt;
    int nfilt;
    // implicit user terms beyond the polynomial (generic kernels only)
    int nxs;
    XSym xs[GOPF_MAX_XSYM];
    // explicit terms of another field of a multi-field Euler step, added in k space:
    // N += xf_coef[q] m^xf_lap[q] xf_src[q](k) (that field's c-hat as it is when this
    // equation's update runs; generic kernels only)
    int nxf;
    double xf_coef[GOPF_MAX_FIELDS];
    int xf_lap[GOPF_MAX_FIELDS];
    const void *xf_src[GOPF_MAX_FIELDS];
    // point sources of this equation (pf/sourceTerm.go:25-30): N += f_s(t) exp(-2 pi i Freq . pos_s),
    // f_s(t) = src_amp[src_row[s] * src_stride + *src_ctr] (the step's entry of a host-supplied
    // table); generic kernels only
    int nsrc;
    int src_row[GOPF_MAX_SRC];
    double src_pos[GOPF_MAX_SRC][3];
    const double *src_amp;
    int src_stride;
    const unsigned long long *src_ctr;
};

// Reduction slots written by the x-pass (FP64, compensated per block)
enum { RED_SUM = 0, RED_SUMSQ = 1, RED_MIN = 2, RED_MAX = 3, RED_NONFINITE = 4, RED_SLOTS = 8 };

enum XInMode { XIN_SPECTRAL = 0, XIN_REAL = 1 };

template <typename R> struct VecOf;
template <> struct VecOf<float> { typedef float2 type; };
template <> struct VecOf<double> { typedef double2 type; };

template <typename R> struct XPassArgs {
    typedef typename VecOf<R>::type V;
    Geom g;
    LinePlan planH;       // complex FFT of length X/2 (table twX, stride 2)
    const V *twX;         // W_X^t, t < X
    int in_mode;          // XIN_SPECTRAL: read spectral tile from in; XIN_REAL: read real rows from rin
    const V *in;
    const R *rin;
    R *rout;              // optional: write real rows of c
    V *out[GOPF_MAX_XOUT];
    int ngrp_out;         // number of spectral outputs (0 = none)
    int identity;         // 1: output group 0 is r2c(c) itself
    PwTable pw;
    double *red;          // optional: per-block partial sums [gridDim.x*gridDim.y][RED_SLOTS]
    // program XP_ELASTIC_Q: out[0] = r2c(escale * H'(c) * (w - 2 e0 H(c))), c = c2r(in), w = c2r(in2)
    int program;
    const V *in2;
    double e0;
    double escale;
    // optional: per-block FP64 sums of group `redgrp`'s real-space values into red2[block]
    int redgrp;
    double *red2;
    int allow_fast; // 1: a specialised kernel may serve this launch
    unsigned *status; // device status word (bounded waits that ran out set bits)
    // program XP_MULTI: inF[f] = T of field f; out[j] = r2c(mono group j)
    const V *inF[GOPF_MAX_FIELDS];
    MonoTable mono;
    int redfield; // XP_MULTI with red: the field whose real-space values are summed into red
    const R *rinF[GOPF_MAX_FIELDS]; // XP_MULTI with XIN_REAL: the real rows of field f
    double adj_dtM; // XP_ADJ: dt M
};

// XP_ADJ (the adjoint step): mu = c2r(in), nu = c2r(in2), c = rin; lambda = mu - adj_dtM (3c^2 - 1) nu
// into rout and r2c(lambda) into out[0]
enum XProgram { XP_POLY = 0, XP_ELASTIC_Q = 1, XP_MULTI = 2, XP_ADJ = 3 };

// PM_ELASTIC_K: forward transform buf[0], multiply by bsym(k)/N, inverse transform in place
enum PassMode { PM_FWD = 0, PM_INV = 1, PM_FUSED = 2, PM_INIT = 3, PM_ELASTIC_K = 4 };

// bit of PassArgs::allow_fast: the launch is a programmatic dependent of the stream's previous
// kernel (the 256-point y and z kernels then set up their tables before waiting for its data)
constexpr int ALLOW_PDL = 64;

template <typename R> struct PassArgs {
    typedef typename VecOf<R>::type V;
    Geom g;
    LinePlan plan;        // transform along this pass's axis
    const V *tw;          // table for plan
    int mode;
    V *buf[GOPF_MAX_GROUPS]; // input groups (transformed in place for FWD/INV)
    int nbuf;
    V *state;             // c-hat (FUSED reads+writes, INIT writes)
    V *tout;              // FUSED/INIT: inverse-transformed c_new/N goes here
    UpdTable upd;
    const R *bsym;        // PM_ELASTIC_K: elastic symbol in the spectral layout
    V *rkF;               // RK4 accumulator (FUSED with upd.rk_stage > 0)
    int allow_fast;       // 1: a specialised kernel may serve this launch
    unsigned *status;     // device status word (bounded waits that ran out set bits)
};

} // namespace gopf
