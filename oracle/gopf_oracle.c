/*
 * gopf_oracle.c -- CPU FP64 restatement of gopf's spectral time-stepping path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the reference computation the GPU
 * library is tested against:
 * only the test-suite, the smoke check and the CPU-baseline leg of the
 * benchmark load it.  Nothing in the product path links or calls it.
 *
 * What it restates (reference = github.com/davidkleiven/gopf):
 *   - fields are complex128 arrays of length N = prod(domainSize), exactly as
 *     pf.Field (pf/model.go:17-20); node order col fastest, then row, then
 *     depth (pfutil/indexPositionConversion.go:23-34);
 *   - the FFT is an unnormalised complex-to-complex transform, forward sign -1,
 *     backward +1, with the 1/N applied by the stepper (pfutil/fftWrap.go:26-39,
 *     pf/euler.go:42-45).  The reference calls FFTW (third party, un-vendored:
 *     github.com/barnex/fftw v0.0.0-20181125072904-b800f77a10de); this file
 *     uses its own mixed-radix Stockham FFT, checked against numpy/pocketfft;
 *   - Freq(i) (pfutil/fftWrap.go:57-74): f in (-0.5, 0.5], +0.5 kept;
 *   - Euler.Step (pf/euler.go:16-47), RK4.Step (pf/rk4.go:29-127),
 *     GetRHS/GetDenum (pf/model.go:283-314), LaplacianN (pf/diffOp.go:25-30),
 *     the Khachaturyan term (pf/homoLinElast.go:47-134 with
 *     elasticity/linearElasticity.go:16-98 and elasticity/effectiveForce.go:26-35),
 *     VolumeConservingLP (pf/volumeConserving.go:19-50),
 *     HomogeneousModulusEnergy (elasticity/linearElasticity.go:101-165).
 *
 * Known deliberate deviations (ulp level): powers of fields use repeated
 * complex multiplication instead of Go's cmplx.Pow, and the 3x3 solve uses
 * Gaussian elimination with partial pivoting instead of gonum's LU.
 *
 * Parity pins: the known-answer tests of the reference (pf/euler_test.go,
 * pf/rk4_test.go, pf/solver_test.go, pf/diffOp_test.go, pf/model_test.go,
 * pf/homoLinElast_test.go, pf/volumeConserving_test.go,
 * elasticity/linearElasticity_test.go) are re-run against this file by
 * tests/test_oracle.py.  Long Cahn-Hilliard trajectories are not pinned by
 * any reference test.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cpx;

#define OR_PI 3.14159265358979323846264338327950288

/* ------------------------------------------------------------------ */
/* 1-D mixed-radix Stockham FFT                                        */
/* ------------------------------------------------------------------ */

#define OR_MAXFAC 40
#define OR_MAXRADIX 64

typedef struct {
    int n;
    int nf;
    int fac[OR_MAXFAC];
    cpx *tw; /* tw[k] = exp(-2 pi i k / n) */
} or_plan1;

static int or_factorize(int n, int *fac)
{
    int nf = 0;
    while (n % 4 == 0) { fac[nf++] = 4; n /= 4; }
    while (n % 2 == 0) { fac[nf++] = 2; n /= 2; }
    for (int p = 3; n > 1; p += 2) {
        while (n % p == 0) {
            if (p > OR_MAXRADIX || nf >= OR_MAXFAC) return -1;
            fac[nf++] = p;
            n /= p;
        }
    }
    return nf;
}

static or_plan1 *or_plan1_create(int n)
{
    or_plan1 *p = (or_plan1 *)calloc(1, sizeof(or_plan1));
    p->n = n;
    p->nf = or_factorize(n, p->fac);
    if (p->nf < 0) { free(p); return NULL; }
    p->tw = (cpx *)malloc(sizeof(cpx) * (size_t)n);
    for (int k = 0; k < n; ++k) {
        double a = -2.0 * OR_PI * (double)k / (double)n;
        p->tw[k] = cos(a) + I * sin(a);
    }
    return p;
}

static void or_plan1_destroy(or_plan1 *p)
{
    if (!p) return;
    free(p->tw);
    free(p);
}

/* In-register DFT of length R with sign (-1 forward, +1 backward). */
static void or_dft(cpx *v, int R, int sign, const or_plan1 *p)
{
    if (R == 2) {
        cpx a = v[0], b = v[1];
        v[0] = a + b;
        v[1] = a - b;
        return;
    }
    if (R == 4) {
        cpx a0 = v[0] + v[2], a1 = v[0] - v[2];
        cpx a2 = v[1] + v[3], a3 = v[1] - v[3];
        /* multiply a3 by (sign * i) */
        cpx a3r = (sign < 0) ? (cimag(a3) - I * creal(a3)) : (-cimag(a3) + I * creal(a3));
        v[0] = a0 + a2;
        v[2] = a0 - a2;
        v[1] = a1 + a3r;
        v[3] = a1 - a3r;
        return;
    }
    if (R == 3) {
        const double s3 = 0.86602540378443864676372317075294;
        cpx t1 = v[1] + v[2];
        cpx t2 = v[0] - 0.5 * t1;
        cpx d = v[1] - v[2];
        /* t3 = sign * i * (sqrt(3)/2) * d */
        cpx t3 = (double)sign * s3 * (-cimag(d) + I * creal(d));
        v[0] = v[0] + t1;
        v[1] = t2 + t3;
        v[2] = t2 - t3;
        return;
    }
    /* generic O(R^2) DFT with roots taken from the plan's table */
    cpx out[OR_MAXRADIX];
    int n = p->n, step = n / R;
    for (int q = 0; q < R; ++q) {
        cpx s = 0;
        for (int r = 0; r < R; ++r) {
            cpx w = p->tw[(size_t)((long)q * r % R) * step];
            if (sign > 0) w = conj(w);
            s += v[r] * w;
        }
        out[q] = s;
    }
    for (int q = 0; q < R; ++q) v[q] = out[q];
}

/* x: length n input/output; w: length n work. */
static void or_fft1(const or_plan1 *p, cpx *x, cpx *w, int sign)
{
    int n = p->n;
    cpx *a = x, *b = w;
    int ns = 1;
    for (int f = 0; f < p->nf; ++f) {
        int R = p->fac[f];
        int m = n / R;
        int twstep = n / (ns * R);
        for (int j = 0; j < m; ++j) {
            cpx v[OR_MAXRADIX];
            int k = j % ns;
            for (int r = 0; r < R; ++r) v[r] = a[j + r * m];
            for (int r = 1; r < R; ++r) {
                cpx t = p->tw[(size_t)r * k * twstep];
                if (sign > 0) t = conj(t);
                v[r] *= t;
            }
            or_dft(v, R, sign, p);
            int base = (j / ns) * ns * R + k;
            for (int r = 0; r < R; ++r) b[base + r * ns] = v[r];
        }
        cpx *t = a; a = b; b = t;
        ns *= R;
    }
    if (a != x) memcpy(x, a, sizeof(cpx) * (size_t)n);
}

/*
 * N-d unnormalised transform of interleaved complex data laid out with
 * shape[0] slowest and shape[ndim-1] fastest.  sign = -1 forward, +1 backward.
 * Returns 0 on success, -1 on unsupported length.
 */
int or_fftn(int ndim, const int *shape, double *data, int sign)
{
    cpx *x = (cpx *)data;
    long total = 1;
    for (int a = 0; a < ndim; ++a) total *= shape[a];
    for (int a = 0; a < ndim; ++a) {
        int L = shape[a];
        if (L == 1) continue;
        long s = 1, outer = 1;
        for (int b = a + 1; b < ndim; ++b) s *= shape[b];
        for (int b = 0; b < a; ++b) outer *= shape[b];
        or_plan1 *p = or_plan1_create(L);
        if (!p) return -1;
        const int B = 8;
        long nblk = (s + B - 1) / B;
        long ntask = outer * nblk;
#pragma omp parallel
        {
            cpx *line = (cpx *)malloc(sizeof(cpx) * (size_t)L * B);
            cpx *work = (cpx *)malloc(sizeof(cpx) * (size_t)L);
#pragma omp for schedule(static)
            for (long t = 0; t < ntask; ++t) {
                long o = t / nblk;
                long ib = (t % nblk) * B;
                int nb = (int)((s - ib) < B ? (s - ib) : B);
                cpx *base = x + o * (long)L * s + ib;
                for (int q = 0; q < nb; ++q)
                    for (int pidx = 0; pidx < L; ++pidx) line[(long)q * L + pidx] = base[(long)pidx * s + q];
                for (int q = 0; q < nb; ++q) or_fft1(p, line + (long)q * L, work, sign);
                for (int q = 0; q < nb; ++q)
                    for (int pidx = 0; pidx < L; ++pidx) base[(long)pidx * s + q] = line[(long)q * L + pidx];
            }
            free(line);
            free(work);
        }
        or_plan1_destroy(p);
    }
    (void)total;
    return 0;
}

int or_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void or_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------ */
/* Freq convention (pfutil/fftWrap.go:41-74)                           */
/* ------------------------------------------------------------------ */

/* dims in the reference's domainSize order: [n0 (rows), n1 (cols), n2 (depth)] */
void or_freq(int ndim, const int *dims, long i, double *res)
{
    long n0 = dims[0], n1 = dims[1];
    long col = i % n1;
    long row = (i / n1) % n0;
    res[0] = (double)row / (double)n0;
    res[1] = (double)col / (double)n1;
    res[2] = 0.0;
    if (ndim > 2) {
        long depth = i / (n0 * n1);
        res[2] = (double)depth / (double)dims[2];
    }
    for (int d = 0; d < ndim; ++d)
        if (res[d] > 0.5) res[d] -= 1.0;
}

long or_conjugate_node(int ndim, const int *dims, long i)
{
    long n0 = dims[0], n1 = dims[1];
    long c = i % n1, r = (i / n1) % n0;
    long cc = (n1 - c) % n1, cr = (n0 - r) % n0, cd = 0;
    if (ndim == 3) {
        long d = i / (n0 * n1);
        cd = (dims[2] - d) % dims[2];
    }
    return cd * n0 * n1 + cr * n1 + cc;
}

/* memory shape (slowest first) for the reference's domainSize */
static void or_mem_shape(int ndim, const int *dims, int *shape)
{
    if (ndim == 2) { shape[0] = dims[0]; shape[1] = dims[1]; }
    else { shape[0] = dims[2]; shape[1] = dims[0]; shape[2] = dims[1]; }
}

/* (-(2 pi |f|)^2)^power  (pf/diffOp.go:25-30) */
static double or_lap_symbol(const double *f, int power)
{
    double nrm = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    double v = -pow(2.0 * OR_PI * nrm, 2.0);
    return pow(v, (double)power);
}

/* ------------------------------------------------------------------ */
/* Model                                                               */
/* ------------------------------------------------------------------ */

enum {
    OR_DER_PRODUCT = 0,     /* prod_j field_j^p_j (pf/util.go:38-65)            */
    OR_DER_POLY = 1,        /* sum_t coef_t * field^p_t (user pointwise function) */
    OR_DER_INDICATOR = 2,   /* 3x^2 - 2x^3            (pf/homoLinElast.go:10-12) */
    OR_DER_INDICATOR_D = 3, /* 6x - 6x^2              (pf/homoLinElast.go:15-17) */
    OR_DER_INDICATOR_HD = 4, /* Indicator(x)*IndicatorDeriv(x)                   */
    OR_DER_MPOLY = 6         /* sum_t coef_t * prod_f field_f^p_tf, a user pointwise function of
                                several fields (examples/strain_single_precipitate/main.go:36-55);
                                power[t] packs p_tf in bits 8f..8f+7                         */
};

enum { OR_SRC_NONE = 0, OR_SRC_FIELD = 1, OR_SRC_DERIVED = 2 };
enum { OR_SPECIAL_NONE = 0, OR_SPECIAL_ELASTIC = 1, OR_SPECIAL_VOLCONS = 2, OR_SPECIAL_HESSIAN = 3, OR_SPECIAL_VISCOSITY = 4 };

#define OR_MAXFAC_D 8
#define OR_MAXTERMS 64
#define OR_MAXDER 16
#define OR_MAXSPECIAL 4

typedef struct {
    int kind;
    int nfac;
    int field[OR_MAXFAC_D];
    int power[OR_MAXFAC_D];
    double coef[OR_MAXFAC_D];
    cpx *data;
} or_derived;

typedef struct {
    int eq;
    int implicit;
    int src_kind, src;
    int special, special_idx;
    cpx coef;
    int lap;   /* LAP power applied to the term (pf/rhsBuilder.go:153-173) */
    int sign_flips; /* prefixes '-' applied after (constructFunc) folded into coef */
} or_term;

/* implicit user terms: TensorialHessian (pf/tensorialHessian.go:38-70), SpectralViscosity
 * (pf/spectralViscosity.go:22-58) */
typedef struct {
    int kind;
    double K[9];
    int nk;
    double eps, threshold;
    int power;
} or_isym;

typedef struct {
    int field;
    double C[81];
    double misfit[9];
    double A[9]; /* C:misfit, the effective stress (elasticity/rank4.go:62-75) */
    double e0;   /* energy density of the misfit (elasticity/linearElasticity.go:86-98) */
    double *h;   /* real-space copy refreshed in OnStepFinished */
    cpx *disp_override; /* optional N x 3 displacement (test hook, pf/homoLinElast_test.go:45-52) */
} or_elastic;

typedef struct {
    int field;
    int indicator; /* derived index */
    double dt;
    double multiplier;
    double current_integral;
    int first;
} or_volcons;

typedef struct {
    int ndim;
    int dims[3];
    int shape[3];
    long N;
    int nfields;
    cpx *fields[8];
    int nder;
    or_derived der[OR_MAXDER];
    int nterms;
    or_term terms[OR_MAXTERMS];
    int nel;
    or_elastic el[OR_MAXSPECIAL];
    int nvc;
    or_volcons vc[OR_MAXSPECIAL];
    int nis;
    or_isym is[OR_MAXSPECIAL];
    long current_step;
    /* point sources (pf/sourceTerm.go): equation, position (row, col, depth), amplitude table
     * amp[step - amp_base] standing for the Go closure f(t) at t = step dt */
    int nsrc;
    int src_eq[OR_MAXSPECIAL];
    double src_pos[OR_MAXSPECIAL][3];
    double *src_amp[OR_MAXSPECIAL];
    long src_len[OR_MAXSPECIAL];
    double *freq; /* 3 * N cached frequencies */
    double *filter; /* modal filter table (ModalFilter.Eval of a Vandeven-style table), NULL = none */
    int nfilter;
} or_model;

or_model *or_model_create(int ndim, const int *dims, int nfields)
{
    if ((ndim != 2 && ndim != 3) || nfields < 1 || nfields > 8) return NULL;
    or_model *m = (or_model *)calloc(1, sizeof(or_model));
    m->ndim = ndim;
    m->N = 1;
    for (int d = 0; d < ndim; ++d) { m->dims[d] = dims[d]; m->N *= dims[d]; }
    or_mem_shape(ndim, dims, m->shape);
    m->nfields = nfields;
    for (int f = 0; f < nfields; ++f) m->fields[f] = (cpx *)calloc((size_t)m->N, sizeof(cpx));
    m->freq = (double *)malloc(sizeof(double) * 3 * (size_t)m->N);
    for (long i = 0; i < m->N; ++i) or_freq(ndim, dims, i, m->freq + 3 * i);
    return m;
}

void or_model_destroy(or_model *m)
{
    if (!m) return;
    for (int k = 0; k < m->nsrc; ++k) free(m->src_amp[k]);
    for (int f = 0; f < m->nfields; ++f) free(m->fields[f]);
    for (int d = 0; d < m->nder; ++d) free(m->der[d].data);
    for (int e = 0; e < m->nel; ++e) { free(m->el[e].h); free(m->el[e].disp_override); }
    free(m->freq);
    free(m->filter);
    free(m);
}

/* NewVandeven (pf/vandeven.go:13-27): 1000-point table of
 * 1 - C(2p) / C(p)^2 * integral_0^x (t(1-t))^(p-1) dt, trapezoid rule, C = Gamma. */
int or_vandeven_table(int order, double *out, int n)
{
    if (order < 1 || n != 1000) return 1;
    const double pref = tgamma((double)(2 * order)) / (tgamma((double)order) * tgamma((double)order));
    const double dx = 1.0 / 999.0;
    out[0] = 1.0;
    for (int i = 1; i < 1000; ++i) {
        const double x = (double)i * dx;
        const double i2 = pow(x * (1.0 - x), (double)(order - 1));
        const double x1 = x - dx;
        const double i1 = pow(x1 * (1.0 - x1), (double)(order - 1));
        out[i] = out[i - 1] - pref * 0.5 * (i1 + i2) * dx;
    }
    return 0;
}

/* Vandeven.Eval (pf/vandeven.go:30-40): linear interpolation in the table, the last entry beyond it */
double or_filter_eval(const double *tab, int n, double x)
{
    const double Nn = (double)(n - 1);
    const int idx = (int)(x * Nn);
    if (idx >= n - 1) return tab[n - 1];
    const double dx = 1.0 / Nn;
    const double dy = tab[idx + 1] - tab[idx];
    const double x0 = (double)idx * dx;
    return tab[idx] + (x - x0) * dy / dx;
}

/* Euler.SetFilter / RK4.SetFilter with a tabulated filter; n = 0 removes it */
int or_set_filter(or_model *m, const double *tab, int n)
{
    free(m->filter);
    m->filter = NULL;
    m->nfilter = 0;
    if (n <= 0) return 0;
    if (n < 2) return 1;
    m->filter = (double *)malloc(sizeof(double) * (size_t)n);
    memcpy(m->filter, tab, sizeof(double) * (size_t)n);
    m->nfilter = n;
    return 0;
}

/* ApplyModalFilter (pf/util.go:125-132): d(k) *= Eval(2 |f| / pi) */
static void or_apply_filter(or_model *m, cpx *d)
{
    if (!m->filter) return;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < m->N; ++i) {
        const double *f = m->freq + 3 * i;
        double r2 = 0.0;
        for (int k = 0; k < m->ndim; ++k) r2 += f[k] * f[k];
        d[i] *= or_filter_eval(m->filter, m->nfilter, sqrt(r2) * 2.0 / 3.14159265358979323846);
    }
}

double *or_field(or_model *m, int f) { return (double *)m->fields[f]; }
double *or_derived_data(or_model *m, int d) { return (double *)m->der[d].data; }
long or_current_step(or_model *m) { return m->current_step; }
void or_set_current_step(or_model *m, long s) { m->current_step = s; }

int or_add_derived(or_model *m, int kind, int nfac, const int *field, const int *power, const double *coef)
{
    if (m->nder >= OR_MAXDER || nfac > OR_MAXFAC_D) return -1;
    or_derived *d = &m->der[m->nder];
    d->kind = kind;
    d->nfac = nfac;
    for (int j = 0; j < nfac; ++j) {
        d->field[j] = field[j];
        d->power[j] = power ? power[j] : 1;
        d->coef[j] = coef ? coef[j] : 1.0;
    }
    d->data = (cpx *)calloc((size_t)m->N, sizeof(cpx));
    return m->nder++;
}

/* coef is the product sign * prod(scalar^power) of pf.ConcreteTerm, lap its LAP power */
int or_add_term(or_model *m, int eq, int implicit, double coef_re, double coef_im, int lap, int src_kind, int src)
{
    if (m->nterms >= OR_MAXTERMS) return -1;
    or_term *t = &m->terms[m->nterms];
    memset(t, 0, sizeof(*t));
    t->eq = eq;
    t->implicit = implicit;
    t->coef = coef_re + I * coef_im;
    t->lap = lap;
    t->src_kind = src_kind;
    t->src = src;
    return m->nterms++;
}

static void or_contract_last(const double *C, const double *eps, double *out)
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) s += C[i * 27 + j * 9 + k * 3 + l] * eps[k * 3 + l];
            out[i * 3 + j] = s;
        }
}

double or_energy_density(const double *C, const double *eps)
{
    double res = 0.0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l)
                    res += C[i * 27 + j * 9 + k * 3 + l] * eps[i * 3 + j] * eps[k * 3 + l];
    return 0.5 * res;
}

/* Explicit term LIN_ELAST on field `field`, scaled by coef * (-k^2)^lap. */
int or_add_elastic(or_model *m, int eq, int field, const double *C, const double *misfit, double coef_re, int lap)
{
    if (m->nel >= OR_MAXSPECIAL || m->nterms >= OR_MAXTERMS) return -1;
    or_elastic *e = &m->el[m->nel];
    memset(e, 0, sizeof(*e));
    e->field = field;
    memcpy(e->C, C, sizeof(double) * 81);
    memcpy(e->misfit, misfit, sizeof(double) * 9);
    or_contract_last(C, misfit, e->A);
    e->e0 = or_energy_density(C, misfit);
    e->h = (double *)calloc((size_t)m->N, sizeof(double));
    or_term *t = &m->terms[m->nterms];
    memset(t, 0, sizeof(*t));
    t->eq = eq;
    t->implicit = 0;
    t->special = OR_SPECIAL_ELASTIC;
    t->special_idx = m->nel;
    t->coef = coef_re;
    t->lap = lap;
    m->nterms++;
    return m->nel++;
}

int or_elastic_set_disp_override(or_model *m, int e, const double *disp /* N x 3 interleaved complex */)
{
    if (e < 0 || e >= m->nel) return -1;
    free(m->el[e].disp_override);
    m->el[e].disp_override = NULL;
    if (disp) {
        m->el[e].disp_override = (cpx *)malloc(sizeof(cpx) * 3 * (size_t)m->N);
        memcpy(m->el[e].disp_override, disp, sizeof(cpx) * 3 * (size_t)m->N);
    }
    return 0;
}

double *or_elastic_hfield(or_model *m, int e) { return m->el[e].h; }

int or_add_volcons(or_model *m, int eq, int field, int indicator, double dt, double coef_re, int lap)
{
    if (m->nvc >= OR_MAXSPECIAL || m->nterms >= OR_MAXTERMS) return -1;
    or_volcons *v = &m->vc[m->nvc];
    memset(v, 0, sizeof(*v));
    v->field = field;
    v->indicator = indicator;
    v->dt = dt;
    v->first = 1;
    or_term *t = &m->terms[m->nterms];
    memset(t, 0, sizeof(*t));
    t->eq = eq;
    t->special = OR_SPECIAL_VOLCONS;
    t->special_idx = m->nvc;
    t->coef = coef_re;
    t->lap = lap;
    m->nterms++;
    return m->nvc++;
}

double or_volcons_multiplier(or_model *m, int v) { return m->vc[v].multiplier; }

/* ---------------- pointwise pieces ---------------- */

static double or_indicator(double x) { return 3.0 * x * x - 2.0 * x * x * x; }
static double or_indicator_deriv(double x) { return 6.0 * x - 6.0 * x * x; }

static cpx or_ipow(cpx x, int p)
{
    cpx r = 1.0;
    if (p < 0) { x = 1.0 / x; p = -p; }
    for (int k = 0; k < p; ++k) r *= x;
    return r;
}

static void or_sync_derived(or_model *m)
{
    for (int d = 0; d < m->nder; ++d) {
        or_derived *D = &m->der[d];
        cpx *out = D->data;
        long N = m->N;
#pragma omp parallel for schedule(static)
        for (long i = 0; i < N; ++i) {
            cpx v;
            switch (D->kind) {
            case OR_DER_PRODUCT:
                v = 1.0;
                for (int j = 0; j < D->nfac; ++j) v *= or_ipow(m->fields[D->field[j]][i], D->power[j]);
                break;
            case OR_DER_POLY: {
                cpx x = m->fields[D->field[0]][i];
                v = 0.0;
                for (int j = 0; j < D->nfac; ++j) v += D->coef[j] * or_ipow(x, D->power[j]);
                break;
            }
            case OR_DER_MPOLY:
                v = 0.0;
                for (int j = 0; j < D->nfac; ++j) {
                    cpx t = D->coef[j];
                    for (int f = 0; f < m->nfields && f < 4; ++f)
                        t *= or_ipow(m->fields[f][i], (D->power[j] >> (8 * f)) & 0xff);
                    v += t;
                }
                break;
            case OR_DER_INDICATOR:
                v = or_indicator(creal(m->fields[D->field[0]][i]));
                break;
            case OR_DER_INDICATOR_D:
                v = or_indicator_deriv(creal(m->fields[D->field[0]][i]));
                break;
            default: {
                double x = creal(m->fields[D->field[0]][i]);
                v = or_indicator(x) * or_indicator_deriv(x);
                break;
            }
            }
            out[i] = v;
        }
    }
}

static void or_fft(or_model *m, cpx *x, int sign) { or_fftn(m->ndim, m->shape, (double *)x, sign); }

static void or_div_n(or_model *m, cpx *x)
{
    double n = (double)m->N;
    long N = m->N;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < N; ++i) x[i] /= n;
}

/* 3x3 real solve with 2 right-hand sides, partial pivoting. */
static void or_solve3(double A[3][3], double B[3][2], double X[3][2])
{
    int piv[3] = {0, 1, 2};
    double M[3][3];
    double R[3][2];
    memcpy(M, A, sizeof(M));
    memcpy(R, B, sizeof(R));
    for (int c = 0; c < 3; ++c) {
        int best = c;
        for (int r = c + 1; r < 3; ++r)
            if (fabs(M[r][c]) > fabs(M[best][c])) best = r;
        if (best != c) {
            for (int k = 0; k < 3; ++k) { double t = M[c][k]; M[c][k] = M[best][k]; M[best][k] = t; }
            for (int k = 0; k < 2; ++k) { double t = R[c][k]; R[c][k] = R[best][k]; R[best][k] = t; }
            int t = piv[c]; piv[c] = piv[best]; piv[best] = t;
        }
        for (int r = c + 1; r < 3; ++r) {
            double f = M[r][c] / M[c][c];
            for (int k = c; k < 3; ++k) M[r][k] -= f * M[c][k];
            for (int k = 0; k < 2; ++k) R[r][k] -= f * R[c][k];
        }
    }
    for (int k = 0; k < 2; ++k)
        for (int r = 2; r >= 0; --r) {
            double s = R[r][k];
            for (int q = r + 1; q < 3; ++q) s -= M[r][q] * X[q][k];
            X[r][k] = s / M[r][r];
        }
}

/* elasticity.Displacements (elasticity/linearElasticity.go:33-63) */
static void or_displacements(or_model *m, const double *C, const cpx *force /* N x 3 */, cpx *disp /* N x 3 */)
{
    long N = m->N;
    const double tol = 1e-10;
    const double fp2 = pow(2.0 * OR_PI, 2);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < N; ++i) {
        const double *f = m->freq + 3 * i;
        if (fabs(f[0]) < tol && fabs(f[1]) < tol && fabs(f[2]) < tol) {
            disp[3 * i] = disp[3 * i + 1] = disp[3 * i + 2] = 0.0;
            continue;
        }
        double G[3][3], B[3][2], X[3][2];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                double e = 0.0;
                for (int j = 0; j < 3; ++j)
                    for (int l = 0; l < 3; ++l) e += C[a * 27 + j * 9 + b * 3 + l] * f[j] * f[l];
                G[a][b] = e * fp2;
            }
        for (int a = 0; a < 3; ++a) { B[a][0] = creal(force[3 * i + a]); B[a][1] = cimag(force[3 * i + a]); }
        or_solve3(G, B, X);
        for (int a = 0; a < 3; ++a) disp[3 * i + a] = X[a][0] + I * X[a][1];
    }
}

/* HomogeneousModulusLinElast.Construct evaluated at the current h-field (pf/homoLinElast.go:47-99). */
static void or_elastic_eval(or_model *m, or_elastic *e, cpx *out)
{
    long N = m->N;
    cpx *work = (cpx *)malloc(sizeof(cpx) * (size_t)N);
    cpx *force = (cpx *)malloc(sizeof(cpx) * 3 * (size_t)N);
    cpx *disp = (cpx *)malloc(sizeof(cpx) * 3 * (size_t)N);
    cpx *strain = (cpx *)malloc(sizeof(cpx) * (size_t)N);
    for (long i = 0; i < N; ++i) out[i] = 0.0;
    for (long i = 0; i < N; ++i) work[i] = or_indicator(e->h[i]);
    or_fft(m, work, -1);
    /* EffectiveForce.Get (elasticity/effectiveForce.go:26-35) for each component */
    for (long i = 0; i < N; ++i) {
        const double *f = m->freq + 3 * i;
        for (int c = 0; c < 3; ++c) {
            cpx s = 0.0;
            for (int j = 0; j < 3; ++j) s += (0.0 - I * (e->A[c * 3 + j] * 2.0 * OR_PI * f[j])) * work[i];
            force[3 * i + c] = s;
        }
    }
    if (e->disp_override)
        memcpy(disp, e->disp_override, sizeof(cpx) * 3 * (size_t)N);
    else
        or_displacements(m, e->C, force, disp);
    for (long i = 0; i < N; ++i) work[i] = or_indicator_deriv(e->h[i]);
    const double tol = 1e-10;
    for (int a = 0; a < m->ndim; ++a)
        for (int b = a; b < m->ndim; ++b) {
            /* elasticity.Strain (elasticity/linearElasticity.go:67-83) */
            for (long i = 0; i < N; ++i) {
                const double *f = m->freq + 3 * i;
                double fm = f[a], fn = f[b];
                if (fabs(fabs(fm) - 0.5) < tol) fm = 0.0;
                if (fabs(fabs(fn) - 0.5) < tol) fn = 0.0;
                strain[i] = (I * OR_PI * fn) * disp[3 * i + a] + (I * OR_PI * fm) * disp[3 * i + b];
            }
            or_fft(m, strain, +1);
            or_div_n(m, strain);
            for (long i = 0; i < N; ++i) strain[i] *= work[i];
            or_fft(m, strain, -1);
            double factor = (a != b) ? 2.0 : 1.0;
            for (long i = 0; i < N; ++i) out[i] += (factor * e->A[a * 3 + b]) * strain[i];
        }
    for (long i = 0; i < N; ++i) work[i] = or_indicator(e->h[i]) * or_indicator_deriv(e->h[i]);
    or_fft(m, work, -1);
    for (long i = 0; i < N; ++i) out[i] -= (2.0 * e->e0) * work[i];
    free(work);
    free(force);
    free(disp);
    free(strain);
}

/* Evaluate one term into out (k space).  Implements ConcreteTerm + constructFunc. */
/* interpolant (pf/spectralViscosity.go:28-38) */
double or_sv_interpolant(double f, double peak)
{
    const double frac = 1.0 / 3.0;
    if (f < frac * peak) return 0.0;
    if (f > peak) return 1.0;
    const double x = 1.5 * (f - frac * peak) / peak;
    return 2.0 * x * x - 3.0 * x * x * x;
}

/* TensorialHessian.GetCoeff (pf/tensorialHessian.go:73-80) */
static double or_hess_coeff(const or_isym *h, int i, int j)
{
    const int d = (h->nk == 9) ? 3 : 2;
    return h->K[i * d + j];
}

/* the symbol of an implicit user term at frequency f (reference order: row, col, depth) */
static double or_isym_eval(const or_model *m, const or_isym *s, const double *f)
{
    if (s->kind == OR_SPECIAL_HESSIAN) {
        double v = 0.0;
        const int dim = m->ndim;
        for (int j = 0; j < dim; ++j) v += -4.0 * OR_PI * OR_PI * f[j] * f[j] * or_hess_coeff(s, j, j);
        for (int j = 0; j < dim; ++j)
            for (int k = j + 1; k < dim; ++k) v += -8.0 * OR_PI * OR_PI * f[j] * f[k] * or_hess_coeff(s, j, k);
        return v;
    }
    double r2 = 0.0;
    for (int j = 0; j < m->ndim; ++j) r2 += f[j] * f[j];
    const double fr = sqrt(r2);
    return -s->eps * or_sv_interpolant(fr, s->threshold) * pow(fr, (double)s->power);
}

int or_add_hessian(or_model *m, int eq, const double *K, int nk, double coef_re, int lap)
{
    if (m->nis >= OR_MAXSPECIAL || m->nterms >= OR_MAXTERMS || (nk != 4 && nk != 9)) return -1;
    or_isym *h = &m->is[m->nis];
    memset(h, 0, sizeof(*h));
    h->kind = OR_SPECIAL_HESSIAN;
    h->nk = nk;
    memcpy(h->K, K, sizeof(double) * (size_t)nk);
    or_term *t = &m->terms[m->nterms++];
    memset(t, 0, sizeof(*t));
    t->eq = eq;
    t->implicit = 1;
    t->special = OR_SPECIAL_HESSIAN;
    t->special_idx = m->nis++;
    t->coef = coef_re;
    t->lap = lap;
    return 0;
}

int or_add_viscosity(or_model *m, int eq, double eps, double threshold, int power, double coef_re, int lap)
{
    if (m->nis >= OR_MAXSPECIAL || m->nterms >= OR_MAXTERMS) return -1;
    or_isym *v = &m->is[m->nis];
    memset(v, 0, sizeof(*v));
    v->kind = OR_SPECIAL_VISCOSITY;
    v->eps = eps;
    v->threshold = threshold;
    v->power = power;
    or_term *t = &m->terms[m->nterms++];
    memset(t, 0, sizeof(*t));
    t->eq = eq;
    t->implicit = 1;
    t->special = OR_SPECIAL_VISCOSITY;
    t->special_idx = m->nis++;
    t->coef = coef_re;
    t->lap = lap;
    return 0;
}

static void or_term_eval(or_model *m, const or_term *t, cpx *out)
{
    long N = m->N;
    if (t->special == OR_SPECIAL_HESSIAN || t->special == OR_SPECIAL_VISCOSITY) {
        const or_isym *s = &m->is[t->special_idx];
        for (long i = 0; i < N; ++i)
            out[i] = t->coef * or_isym_eval(m, s, m->freq + 3 * i) * or_lap_symbol(m->freq + 3 * i, t->lap);
        return;
    }
    if (t->special == OR_SPECIAL_ELASTIC) {
        or_elastic_eval(m, &m->el[t->special_idx], out);
        for (long i = 0; i < N; ++i) out[i] *= t->coef * or_lap_symbol(m->freq + 3 * i, t->lap);
        return;
    }
    if (t->special == OR_SPECIAL_VOLCONS) {
        or_volcons *v = &m->vc[t->special_idx];
        const cpx *ind = m->der[v->indicator].data;
        for (long i = 0; i < N; ++i) out[i] = ind[i] * v->multiplier;
        for (long i = 0; i < N; ++i) out[i] *= t->coef * or_lap_symbol(m->freq + 3 * i, t->lap);
        return;
    }
    const cpx *src = NULL;
    if (t->src_kind == OR_SRC_FIELD) src = m->fields[t->src];
    else if (t->src_kind == OR_SRC_DERIVED) src = m->der[t->src].data;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < N; ++i) {
        cpx v = t->coef;
        if (src) v *= src[i];
        if (t->lap != 0) v *= or_lap_symbol(m->freq + 3 * i, t->lap);
        out[i] = v;
    }
}

static void or_get_rhs(or_model *m, int eq, cpx *rhs, cpx *tmp)
{
    long N = m->N;
    for (long i = 0; i < N; ++i) rhs[i] = 0.0;
    for (int k = 0; k < m->nterms; ++k) {
        const or_term *t = &m->terms[k];
        if (t->eq != eq || t->implicit) continue;
        or_term_eval(m, t, tmp);
        for (long i = 0; i < N; ++i) rhs[i] += tmp[i];
    }
    /* Source.Eval (pf/sourceTerm.go:25-30): f(t) exp(-2 pi i Freq(i) . pos), t = CurrentStep dt */
    for (int k = 0; k < m->nsrc; ++k) {
        if (m->src_eq[k] != eq) continue;
        const long s = m->current_step;
        const double amp = (s >= 0 && s < m->src_len[k]) ? m->src_amp[k][s] : 0.0;
        for (long i = 0; i < N; ++i) {
            const double *f = m->freq + 3 * i;
            double dot = 0.0;
            for (int d = 0; d < m->ndim; ++d) dot += f[d] * m->src_pos[k][d];
            rhs[i] += amp * cexp(-I * 6.283185307179586476925286766559 * dot);
        }
    }
}

/* Model.AddSource(eq, NewSource(pos, f)) with f given as its values at steps 0 .. n - 1 */
int or_add_source(or_model *m, int eq, const double *pos, const double *amps, long n)
{
    if (m->nsrc >= OR_MAXSPECIAL || eq < 0 || eq >= m->nfields || n < 1) return -1;
    const int k = m->nsrc++;
    m->src_eq[k] = eq;
    for (int d = 0; d < 3; ++d) m->src_pos[k][d] = (d < m->ndim) ? pos[d] : 0.0;
    m->src_amp[k] = (double *)malloc(sizeof(double) * (size_t)n);
    memcpy(m->src_amp[k], amps, sizeof(double) * (size_t)n);
    m->src_len[k] = n;
    return k;
}

static void or_get_denum(or_model *m, int eq, cpx *den, cpx *tmp)
{
    long N = m->N;
    for (long i = 0; i < N; ++i) den[i] = 0.0;
    for (int k = 0; k < m->nterms; ++k) {
        const or_term *t = &m->terms[k];
        if (t->eq != eq || !t->implicit) continue;
        or_term_eval(m, t, tmp);
        for (long i = 0; i < N; ++i) den[i] += tmp[i];
    }
}

/* Solver.Propagate's per-step hooks (pf/solver.go:74-82) */
static void or_on_step_finished(or_model *m)
{
    long N = m->N;
    for (int e = 0; e < m->nel; ++e) {
        or_elastic *E = &m->el[e];
        for (long i = 0; i < N; ++i) E->h[i] = creal(m->fields[E->field][i]);
    }
    for (int k = 0; k < m->nvc; ++k) {
        or_volcons *v = &m->vc[k];
        double integ = 0.0;
        for (long i = 0; i < N; ++i) integ += creal(m->fields[v->field][i]);
        double ind = creal(m->der[v->indicator].data[0]);
        if (v->first) {
            v->current_integral = integ;
            v->first = 0;
        } else {
            double dI = integ - v->current_integral;
            v->current_integral = integ;
            v->multiplier = v->multiplier - dI / (v->dt * ind);
        }
    }
}

static void or_fft_fields(or_model *m, int sign)
{
    for (int f = 0; f < m->nfields; ++f) or_fft(m, m->fields[f], sign);
}

static void or_fft_derived(or_model *m)
{
    for (int d = 0; d < m->nder; ++d) or_fft(m, m->der[d].data, -1);
}

static void or_ifft_fields(or_model *m)
{
    for (int f = 0; f < m->nfields; ++f) {
        or_fft(m, m->fields[f], +1);
        or_div_n(m, m->fields[f]);
    }
}

/* Euler.Step (pf/euler.go:16-47); hooks = 1 mirrors Solver.Propagate */
int or_step_euler(or_model *m, double dt, long nsteps, int hooks)
{
    long N = m->N;
    cpx *rhs = (cpx *)malloc(sizeof(cpx) * (size_t)N);
    cpx *den = (cpx *)malloc(sizeof(cpx) * (size_t)N);
    cpx *tmp = (cpx *)malloc(sizeof(cpx) * (size_t)N);
    for (long s = 0; s < nsteps; ++s) {
        or_sync_derived(m);
        or_fft_fields(m, -1);
        or_fft_derived(m);
        for (int f = 0; f < m->nfields; ++f) {
            or_get_rhs(m, f, rhs, tmp);
            or_get_denum(m, f, den, tmp);
            cpx *d = m->fields[f];
#pragma omp parallel for schedule(static)
            for (long j = 0; j < N; ++j) d[j] = (d[j] + dt * rhs[j]) / (1.0 - dt * den[j]);
            or_apply_filter(m, d);
        }
        or_ifft_fields(m);
        m->current_step++;
        if (hooks) or_on_step_finished(m);
    }
    free(rhs);
    free(den);
    free(tmp);
    return 0;
}

/* RK4.Step (pf/rk4.go:29-127).  The reference's Step does not advance
 * CurrentStep (only RK4.Propagate does); `advance` selects that behaviour. */
int or_step_rk4(or_model *m, double dt, long nsteps, int hooks, int advance)
{
    long N = m->N;
    int nf = m->nfields;
    cpx *tmp = (cpx *)malloc(sizeof(cpx) * (size_t)N);
    cpx *den = (cpx *)malloc(sizeof(cpx) * (size_t)N);
    cpx *init[8], *fin[8], *kf[8];
    for (int f = 0; f < nf; ++f) {
        init[f] = (cpx *)malloc(sizeof(cpx) * (size_t)N);
        fin[f] = (cpx *)malloc(sizeof(cpx) * (size_t)N);
        kf[f] = (cpx *)malloc(sizeof(cpx) * (size_t)N);
    }
    const double factors[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
    const double corr[3] = {0.5, 0.5, 1.0};
    for (long s = 0; s < nsteps; ++s) {
        or_sync_derived(m);
        or_fft_fields(m, -1);
        for (int f = 0; f < nf; ++f) {
            memcpy(init[f], m->fields[f], sizeof(cpx) * (size_t)N);
            memcpy(fin[f], m->fields[f], sizeof(cpx) * (size_t)N);
        }
        /* firstCorrection */
        or_fft_derived(m);
        for (int f = 0; f < nf; ++f) or_get_rhs(m, f, kf[f], tmp);
        for (int stage = 0; stage < 4; ++stage) {
            /* PrepareNextCorrection */
            for (int f = 0; f < nf; ++f) {
                for (long j = 0; j < N; ++j) fin[f][j] += (factors[stage] * dt) * kf[f][j];
                memcpy(m->fields[f], init[f], sizeof(cpx) * (size_t)N);
            }
            if (stage == 3) break;
            /* correction */
            double fac = corr[stage];
            for (int f = 0; f < nf; ++f) {
                or_get_denum(m, f, den, tmp);
                cpx *d = m->fields[f];
                for (long j = 0; j < N; ++j) {
                    d[j] += (fac * dt) * kf[f][j];
                    d[j] /= (1.0 - (fac * dt) * den[j]);
                }
                or_fft(m, d, +1);
                or_div_n(m, d);
            }
            or_sync_derived(m);
            or_fft_fields(m, -1);
            or_fft_derived(m);
            for (int f = 0; f < nf; ++f) or_get_rhs(m, f, kf[f], tmp);
        }
        for (int f = 0; f < nf; ++f) {
            or_get_denum(m, f, den, tmp);
            for (long j = 0; j < N; ++j) fin[f][j] /= (1.0 - dt * den[j]);
            memcpy(m->fields[f], fin[f], sizeof(cpx) * (size_t)N);
            or_apply_filter(m, m->fields[f]);
        }
        or_ifft_fields(m);
        if (advance) m->current_step++;
        if (hooks) or_on_step_finished(m);
    }
    for (int f = 0; f < nf; ++f) { free(init[f]); free(fin[f]); free(kf[f]); }
    free(tmp);
    free(den);
    return 0;
}

/* Evaluate the explicit RHS of equation eq on the current (real-space) fields,
 * the way Euler.Step sees it, and return it in k space.  Fields are left
 * unchanged.  Used to check single terms against the reference's unit tests. */
int or_eval_rhs(or_model *m, int eq, double *out)
{
    long N = m->N;
    cpx *tmp = (cpx *)malloc(sizeof(cpx) * (size_t)N);
    cpx *save[8];
    for (int f = 0; f < m->nfields; ++f) {
        save[f] = (cpx *)malloc(sizeof(cpx) * (size_t)N);
        memcpy(save[f], m->fields[f], sizeof(cpx) * (size_t)N);
    }
    or_sync_derived(m);
    or_fft_fields(m, -1);
    or_fft_derived(m);
    or_get_rhs(m, eq, (cpx *)out, tmp);
    for (int f = 0; f < m->nfields; ++f) {
        memcpy(m->fields[f], save[f], sizeof(cpx) * (size_t)N);
        free(save[f]);
    }
    free(tmp);
    return 0;
}

int or_eval_denum(or_model *m, int eq, double *out)
{
    long N = m->N;
    cpx *tmp = (cpx *)malloc(sizeof(cpx) * (size_t)N);
    or_get_denum(m, eq, (cpx *)out, tmp);
    free(tmp);
    return 0;
}

/* elasticity.HomogeneousModulusEnergy (elasticity/linearElasticity.go:101-165) */
double or_homogeneous_modulus_energy(int ndim, const int *dims, double *indicator /* interleaved complex, modified */,
                                     const double *misfit, const double *C)
{
    or_model *m = or_model_create(ndim, dims, 1);
    long N = m->N;
    cpx *ind = (cpx *)indicator;
    double volume = 0.0;
    for (long i = 0; i < N; ++i) volume += creal(ind[i]);
    double A[9];
    or_contract_last(C, misfit, A);
    or_fft(m, ind, -1);
    cpx *force = (cpx *)malloc(sizeof(cpx) * 3 * (size_t)N);
    cpx *disp = (cpx *)malloc(sizeof(cpx) * 3 * (size_t)N);
    cpx *strain = (cpx *)malloc(sizeof(cpx) * (size_t)N);
    double *eps = (double *)calloc(9 * (size_t)N, sizeof(double));
    for (long i = 0; i < N; ++i) {
        const double *f = m->freq + 3 * i;
        for (int c = 0; c < 3; ++c) {
            cpx s = 0.0;
            for (int j = 0; j < 3; ++j) s += (0.0 - I * (A[c * 3 + j] * 2.0 * OR_PI * f[j])) * ind[i];
            force[3 * i + c] = s;
        }
    }
    or_displacements(m, C, force, disp);
    or_fft(m, ind, +1);
    for (long i = 0; i < N; ++i) ind[i] /= (double)N;
    const double tol = 1e-10;
    for (int a = 0; a < 3; ++a)
        for (int b = a; b < 3; ++b) {
            for (long i = 0; i < N; ++i) {
                const double *f = m->freq + 3 * i;
                double fm = f[a], fn = f[b];
                if (fabs(fabs(fm) - 0.5) < tol) fm = 0.0;
                if (fabs(fabs(fn) - 0.5) < tol) fn = 0.0;
                strain[i] = (I * OR_PI * fn) * disp[3 * i + a] + (I * OR_PI * fm) * disp[3 * i + b];
            }
            or_fft(m, strain, +1);
            for (long i = 0; i < N; ++i) {
                double re = creal(strain[i]) / (double)N;
                if (creal(ind[i]) > 0.5) re -= misfit[a * 3 + b];
                eps[9 * i + a * 3 + b] = re;
                eps[9 * i + b * 3 + a] = re;
            }
        }
    double energy = 0.0;
    for (long i = 0; i < N; ++i) energy += or_energy_density(C, eps + 9 * i);
    free(force);
    free(disp);
    free(strain);
    free(eps);
    or_model_destroy(m);
    return energy / volume;
}

/* ------------------------------------------------------------------ */
/* Seeded synthetic input generator (SplitMix64 -> U[0,1))             */
/* ------------------------------------------------------------------ */

static uint64_t or_splitmix64(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

/* out[i] = center + half_width * (2 u_i - 1), u_i = splitmix64(seed)_i >> 11 * 2^-53 */
void or_uniform_field(uint64_t seed, long n, double center, double half_width, double *out)
{
    uint64_t s = seed;
    for (long i = 0; i < n; ++i) {
        double u = (double)(or_splitmix64(&s) >> 11) * (1.0 / 9007199254740992.0);
        out[i] = center + half_width * (2.0 * u - 1.0);
    }
}

/* ------------------------------------------------------------------ */
/* Shrinking-dimer dynamics, SDD (pf/sdd.go:86-470)                    */
/* ------------------------------------------------------------------ */

typedef struct {
    or_model *m;
    double *orient; /* nfields * N, unit length */
    double alpha, dt, tau_orient, tau_len, init_len, min_len;
    long step;
    /* SDDMonitor (pf/sdd.go:27-52): MaxForce, ForcePowerSpectrum, MaxTorque, FieldNorm, FieldNormChange */
    double mon[5];
} or_sdd;

/* NewSDD (pf/sdd.go:118-127): alpha 0.5, both time constants 1 */
or_sdd *or_sdd_create(or_model *m)
{
    or_sdd *s = (or_sdd *)calloc(1, sizeof(or_sdd));
    s->m = m;
    s->orient = (double *)calloc((size_t)m->N * (size_t)m->nfields, sizeof(double));
    s->alpha = 0.5;
    s->tau_orient = 1.0;
    s->tau_len = 1.0;
    return s;
}

void or_sdd_destroy(or_sdd *s)
{
    if (!s) return;
    free(s->orient);
    free(s);
}

void or_sdd_set_params(or_sdd *s, double alpha, double dt, double tau_orient, double tau_len, double init_len,
                       double min_len)
{
    s->alpha = alpha;
    s->dt = dt;
    s->tau_orient = tau_orient;
    s->tau_len = tau_len;
    if (init_len > 0.0) s->init_len = init_len;
    s->min_len = min_len;
}

double *or_sdd_orientation(or_sdd *s) { return s->orient; }
double *or_sdd_monitor(or_sdd *s) { return s->mon; }
double or_sdd_init_length(or_sdd *s) { return s->init_len; }

static void or_sdd_normalise(or_sdd *s, long n)
{
    double len = 0.0;
    for (long i = 0; i < n; ++i) len += s->orient[i] * s->orient[i];
    len = sqrt(len);
    for (long i = 0; i < n; ++i) s->orient[i] /= len;
}

/* Init (pf/sdd.go:386-404): orientation = final - init (real parts, all fields), its length is
 * the initial dimer length. */
void or_sdd_init(or_sdd *s, const double *init, const double *final)
{
    const long n = s->m->N * s->m->nfields;
    double len = 0.0;
    for (long i = 0; i < n; ++i) {
        s->orient[i] = final[i] - init[i];
        len += s->orient[i] * s->orient[i];
    }
    s->init_len = sqrt(len);
    for (long i = 0; i < n; ++i) s->orient[i] /= s->init_len;
}

/* SetInitialOrientation (pf/sdd.go:409-424) */
void or_sdd_set_orientation(or_sdd *s, const double *v)
{
    const long n = s->m->N * s->m->nfields;
    double len = 0.0;
    for (long i = 0; i < n; ++i) len += v[i] * v[i];
    s->init_len = sqrt(len);
    for (long i = 0; i < n; ++i) s->orient[i] = v[i] / s->init_len;
}

/* DimerLength (pf/sdd.go:355-362) */
double or_sdd_dimer_length(const or_sdd *s, double t)
{
    const double l = s->init_len * exp(-t / s->tau_len);
    return (l < s->min_len) ? s->min_len : l;
}

/* householder (pf/sdd.go:303-318): data -= sigma * o * (sum data conj(o)) / num_nodes */
void or_householder(double *data_, const double *orient_, double sigma, long n, long num_nodes)
{
    cpx *data = (cpx *)data_;
    const cpx *o = (const cpx *)orient_;
    cpx dot = 0.0;
    for (long i = 0; i < n; ++i) dot += data[i] * conj(o[i]);
    dot /= (double)num_nodes;
    for (long i = 0; i < n; ++i) data[i] = data[i] - sigma * o[i] * dot;
}

/* diagonalShermannMorrison.dot (pf/sdd.go:456-470): vec <- (D + u v^T)^-1 vec with D^-1 = inv_diag */
void or_dsm_dot(const double *inv_diag_, const double *u_, const double *v_, long n, double *vec_)
{
    const cpx *d = (const cpx *)inv_diag_, *u = (const cpx *)u_, *v = (const cpx *)v_;
    cpx *x = (cpx *)vec_;
    cpx den = 1.0, vdx = 0.0;
    for (long i = 0; i < n; ++i) {
        den += u[i] * d[i] * v[i];
        vdx += v[i] * d[i] * x[i];
    }
    for (long i = 0; i < n; ++i) x[i] = d[i] * x[i] - d[i] * u[i] * vdx / den;
}

/* householderDenum (pf/sdd.go:320-339) followed by its dot: vec <- (I - dt (denum - sigma denum o o^H / n))^-1 vec */
static void or_sdd_denum_solve(const cpx *denum, const cpx *o, double sigma, double dt, long n, cpx *vec, cpx *w3)
{
    cpx *inv = w3, *v = w3 + n;
    for (long i = 0; i < n; ++i) {
        inv[i] = 1.0 / (1.0 - dt * denum[i]);
        v[i] = sigma * denum[i] * dt * conj(o[i]) / (double)n;
    }
    or_dsm_dot((const double *)inv, (const double *)o, (const double *)v, n, (double *)vec);
}

void or_sdd_denum_dot(const double *denum, const double *orient, double sigma, double dt, long n, double *vec)
{
    cpx *w = (cpx *)malloc(sizeof(cpx) * 2 * (size_t)n);
    or_sdd_denum_solve((const cpx *)denum, (const cpx *)orient, sigma, dt, n, (cpx *)vec, w);
    free(w);
}

static void or_sdd_shift(or_sdd *s, double scale)
{
    or_model *m = s->m;
    long k = 0;
    for (int f = 0; f < m->nfields; ++f)
        for (long j = 0; j < m->N; ++j, ++k) m->fields[f][j] += scale * s->orient[k];
}

/* the model's fields (synced derived fields first) to k space, and back */
static void or_sdd_fft(or_model *m)
{
    or_sync_derived(m);
    or_fft_fields(m, -1);
    or_fft_derived(m);
}

/* SDD.Step (pf/sdd.go:159-285) */
int or_sdd_step(or_sdd *s, long nsteps)
{
    or_model *m = s->m;
    const long N = m->N;
    const int nf = m->nfields;
    if (s->dt < 1e-16) return 1; /* checkTimeStep panics */
    cpx *ftO = (cpx *)malloc(sizeof(cpx) * (size_t)N * nf);
    cpx *rs = (cpx *)malloc(sizeof(cpx) * (size_t)N * nf);
    cpx *re = (cpx *)malloc(sizeof(cpx) * (size_t)N * nf);
    cpx *work = (cpx *)malloc(sizeof(cpx) * (size_t)N);
    cpx *orig = (cpx *)malloc(sizeof(cpx) * (size_t)N);
    cpx *tmp = (cpx *)malloc(sizeof(cpx) * (size_t)N);
    cpx *den = (cpx *)malloc(sizeof(cpx) * (size_t)N);
    cpx *w3 = (cpx *)malloc(sizeof(cpx) * 2 * (size_t)N);
    for (long st = 0; st < nsteps; ++st) {
        double fnorm = 0.0;
        for (int f = 0; f < nf; ++f)
            for (long j = 0; j < N; ++j) {
                const double a = cabs(m->fields[f][j]);
                fnorm += a * a;
            }
        s->mon[4] = s->mon[3] - fnorm;
        s->mon[3] = fnorm;
        for (long i = 0; i < N * nf; ++i) ftO[i] = s->orient[i];
        for (int f = 0; f < nf; ++f) or_fft(m, ftO + (long)f * N, -1);
        const double t = (double)s->step * s->dt;
        const double l = or_sdd_dimer_length(s, t);

        or_sdd_shift(s, -0.5 * l); /* start image */
        or_sdd_fft(m);
        for (int f = 0; f < nf; ++f) or_get_rhs(m, f, rs + (long)f * N, tmp);
        or_ifft_fields(m);
        or_sdd_shift(s, l); /* end image */
        or_sdd_fft(m);
        for (int f = 0; f < nf; ++f) or_get_rhs(m, f, re + (long)f * N, tmp);
        or_ifft_fields(m);
        or_sdd_shift(s, -0.5 * l); /* back to the centre */
        or_sdd_fft(m);

        double maxf = 0.0, fps = 0.0;
        for (int f = 0; f < nf; ++f) {
            cpx *d = m->fields[f];
            memcpy(orig, d, sizeof(cpx) * (size_t)N);
            /* the force at the centre: the reference weighs the first field's start and end
             * right-hand sides for every field (rhsStart[j], rhsEnd[j] with j < NumNodes) */
            for (long j = 0; j < N; ++j) work[j] = s->alpha * rs[j] + (1.0 - s->alpha) * re[j];
            or_householder((double *)work, (const double *)(ftO + (long)f * N), 2.0, N, N);
            for (long j = 0; j < N; ++j) d[j] = d[j] + s->dt * work[j];
            or_get_denum(m, f, den, tmp);
            or_sdd_denum_solve(den, ftO + (long)f * N, 2.0, s->dt, N, d, w3);
            for (long j = 0; j < N; ++j) {
                const double diff = cabs((d[j] - orig[j]) / s->dt);
                fps += diff * diff / (double)N;
                if (diff > maxf) maxf = diff;
            }
        }
        s->mon[0] = maxf;
        s->mon[1] = sqrt(fps / (double)(nf * N));

        /* torque: F(start) - F(end) plus the linear part -L v l */
        for (long i = 0; i < N * nf; ++i) rs[i] = rs[i] - re[i];
        for (int f = 0; f < nf; ++f) {
            or_get_denum(m, f, den, tmp);
            for (long j = 0; j < N; ++j) rs[(long)f * N + j] -= den[j] * ftO[(long)f * N + j] * l;
        }
        or_householder((double *)rs, (const double *)ftO, 1.0, N * nf, N);
        for (int f = 0; f < nf; ++f) or_fft(m, rs + (long)f * N, +1);
        for (long i = 0; i < N * nf; ++i) rs[i] /= (double)N;
        double maxt = 0.0;
        const double lt = or_sdd_dimer_length(s, t);
        for (long i = 0; i < N * nf; ++i) {
            s->orient[i] -= s->dt * creal(rs[i]) / (lt * s->tau_orient);
            if (fabs(creal(rs[i])) > maxt) maxt = fabs(creal(rs[i]));
        }
        s->mon[2] = maxt;
        or_sdd_normalise(s, N * nf);
        or_ifft_fields(m);
        s->step++;
    }
    free(ftO);
    free(rs);
    free(re);
    free(work);
    free(orig);
    free(tmp);
    free(den);
    free(w3);
    return 0;
}
