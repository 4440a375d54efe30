/*
 * gopf_gpu.h -- C ABI of the GB300 spectral time stepper.
 *
 * This is the drop-in boundary for gopf's hot path.  A Go program binds it
 * with cgo and gets a pf.TimeStepper whose fields stay resident in device
 * memory between steps.  Every entry point returns an
 * int status (GOPF_OK == 0); nothing throws or aborts across the ABI.  Host
 * pointers are borrowed for the duration of the call only.  A context is not
 * thread-safe: calls on one context must be serialised by the caller.  Each
 * call makes the context's device current, so calls may come from any OS
 * thread.
 *
 * Reference interfaces replaced (github.com/davidkleiven/gopf):
 *   pf.TimeStepper   pf/solver.go:15-19   -> gopf_set_stepper / gopf_step / gopf_get_time
 *   pf.Euler.Step    pf/euler.go:16-47    -> gopf_step (GOPF_STEPPER_EULER)
 *   pf.RK4.Step      pf/rk4.go:29-74      -> gopf_step (GOPF_STEPPER_RK4)
 *   pf.ImplicitEuler.Step pf/implicitEuler.go:165-207 -> gopf_step (GOPF_STEPPER_IMPLICIT_EULER)
 *   pf.SDD (shrinking-dimer dynamics) pf/sdd.go:86-470 -> gopf_step (GOPF_STEPPER_SDD), gopf_sdd_*
 *   pf.FourierTransform pf/solver.go:22-26, pfutil/fftWrap.go:26-95
 *                                         -> gopf_fft / gopf_freq / gopf_conjugate_node
 *   pf.Model.AddField/AddScalar/AddEquation/RegisterFunction/Init
 *                    pf/model.go:133-162,244-260,400-412 -> gopf_add_field ... gopf_init
 *   pf.Build / ConcreteTerm  pf/rhsBuilder.go:26-190 -> gopf_init (equation strings) or
 *                                                      gopf_set_terms (pre-compiled table)
 *   pf.HomogeneousModulusLinElast pf/homoLinElast.go:33-150 -> gopf_register_elastic
 *   pf.VolumeConservingLP pf/volumeConserving.go:8-61 -> gopf_register_volcons
 *   Field.Data access (host <-> device)   -> gopf_field_upload / gopf_field_download
 *   mass check pf/solver_test.go:20-27 -> gopf_reduce
 *   PointMonitor pf/monitor.go:8-30       -> gopf_point_values
 *   Monitor pf/monitor.go:4-6, HomogeneousModulusEnergy elasticity/linearElasticity.go:101-165
 *                                         -> gopf_free_energy / gopf_elastic_energy
 *   Model.AddSource / Source pf/model.go:152-154, pf/sourceTerm.go:14-30 -> gopf_add_source
 */
#ifndef GOPF_GPU_H
#define GOPF_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gopf_ctx gopf_ctx;

/* status codes */
enum {
    GOPF_OK = 0,
    GOPF_ERR_ARG = 1,         /* bad argument (size mismatch: the reference panics, pf/solver.go:55-60) */
    GOPF_ERR_CUDA = 2,        /* CUDA runtime error */
    GOPF_ERR_OOM = 3,         /* device allocation failed */
    GOPF_ERR_NAN = 4,         /* non-finite value detected in a field after stepping */
    GOPF_ERR_TIMEOUT = 5,     /* a bounded device wait gave up */
    GOPF_ERR_UNSUPPORTED = 6, /* model feature with no device implementation (no CPU fallback) */
    GOPF_ERR_STATE = 7,       /* call out of order (e.g. step before init) */
    GOPF_ERR_PARSE = 8        /* equation string could not be parsed (pf/rhsBuilder.go panics) */
};

/* precision of the device state */
enum { GOPF_FP32 = 0, GOPF_FP64 = 1 };

/* time steppers */
enum { GOPF_STEPPER_EULER = 0, GOPF_STEPPER_RK4 = 1, GOPF_STEPPER_IMPLICIT_EULER = 2, GOPF_STEPPER_SDD = 3 };

/* derived-field kinds (real-space pointwise functions of one field) */
enum {
    GOPF_DER_PRODUCT = 0,     /* prod_j field_j^power_j; names like "conc^3" (pf/util.go:38-65) */
    GOPF_DER_POLY = 1,        /* sum_t coef_t * field^power_t (a RegisterFunction polynomial) */
    GOPF_DER_INDICATOR = 2,   /* 3x^2 - 2x^3 (pf/homoLinElast.go:10-12) */
    GOPF_DER_INDICATOR_D = 3, /* 6x - 6x^2 (pf/homoLinElast.go:15-17) */
    GOPF_DER_INDICATOR_HD = 4, /* Indicator(x) * IndicatorDeriv(x) */
    GOPF_DER_WHITE_NOISE = 5,  /* N(0, 2S) per cell and step (WhiteNoise.Generate, pf/noise.go:20-23) */
    GOPF_DER_MPOLY = 6         /* sum_t coef_t * prod_f field_f^p_tf, a polynomial of several fields:
                                  power[t] packs p_tf in bits 8f..8f+7 (fields 0..3), field[] unused */
};

/* noise kinds for gopf_register_noise */
enum {
    GOPF_NOISE_WHITE = 1,       /* a function (derived field) name, as RegisterFunction(name, WhiteNoise.Generate) */
    GOPF_NOISE_CONSERVATIVE = 2 /* a user term name, as RegisterExplicitTerm(name, &ConservativeNoise, ...) */
};

/* term sources */
enum { GOPF_SRC_NONE = 0, GOPF_SRC_FIELD = 1, GOPF_SRC_DERIVED = 2 };

/* reductions over the real field (FP64) */
enum {
    GOPF_RED_SUM = 0,   /* sum of c over cells (total mass) */
    GOPF_RED_SUMSQ = 1, /* sum of c^2 */
    GOPF_RED_MIN = 2,
    GOPF_RED_MAX = 3,
    GOPF_RED_NONFINITE = 4 /* number of NaN/Inf cells */
};

/* options for gopf_set_option */
enum {
    GOPF_OPT_CHECK_FINITE = 0, /* 1 (default): gopf_step synchronises and checks the field for NaN/Inf */
    GOPF_OPT_USE_GRAPHS = 1,   /* 1 (default): steps are replayed from captured CUDA graphs */
    GOPF_OPT_FAST_KERNELS = 2, /* 1 (default): register-resident kernels serve the lengths they cover */
    GOPF_OPT_TMA = 3,          /* 1 (default): those kernels move their tiles with TMA tensor copies;
                                  0: plain loads (value 4 is unused) */
    GOPF_OPT_DIRECT_HOST = 5,  /* 1 (default): pinned host buffers given to upload/download are read and
                                  written by kernels in place; pageable buffers are staged */
    GOPF_OPT_WAIT_LIMIT_NS = 6, /* limit (ns) of a kernel's first wait for a tile copy; 0 (default) = 2 s.
                                  A wait that runs out flags the step (GOPF_ERR_TIMEOUT from gopf_step or
                                  gopf_synchronize), waits up to 2 s more for the copy still in flight and
                                  leaves the tile alone, so the field must be uploaded again.  Meant for
                                  testing that error path; the reference has no counterpart. */
    GOPF_OPT_X_ROWS = 7,        /* rows per tile of the 256-column x pass with one dense polynomial group:
                                  16 (default: 128 threads, eight blocks per SM) or 32 (256 threads,
                                  four blocks per SM); both compute the same values */
    GOPF_OPT_Z_LINES = 8,       /* lines per tile of the 256-point z pass with one explicit group: 8
                                  (default: 128 threads, six blocks per SM) or 16 (256 threads, three
                                  blocks per SM); both compute the same values */
    GOPF_OPT_PDL = 9            /* 1 (default): in the 3D Euler step the forward y, fused z and inverse y
                                  256-point kernels launch as programmatic dependents of the kernel
                                  before them, setting up their tables while it finishes; 0: plain
                                  stream order.  The same values either way */
};

#define GOPF_MAX_FACTORS 8

/* A real-space derived field (what pf.Model.UpdateDerivedFields / RegisterFunction register). */
typedef struct {
    int kind;                      /* GOPF_DER_* */
    int nfac;                      /* number of factors / polynomial terms */
    int field[GOPF_MAX_FACTORS];   /* field ids */
    int power[GOPF_MAX_FACTORS];   /* integer powers */
    double coef[GOPF_MAX_FACTORS]; /* polynomial coefficients (GOPF_DER_POLY) */
} gopf_derived;

/* One term of an equation, as pf.Build produces it (pf/rhsBuilder.go:125-242):
 * value(k) = coef * (-(2 pi |f|)^2)^lap * source(k). */
typedef struct {
    int eq;        /* equation index == index of the field it evolves */
    int implicit;  /* 1: bilinear in the field -> enters the denominator (Denum) */
    double coef;   /* sign * prod(scalar^power) */
    int lap;       /* power of the Laplacian symbol */
    int source;    /* GOPF_SRC_* (ignored for implicit terms) */
    int src_index; /* field id or derived id */
} gopf_term;

/* ---- context ---- */
int gopf_ctx_create(int ndim, const int *domain_size, int precision, int device, gopf_ctx **out);
int gopf_ctx_destroy(gopf_ctx *ctx);
const char *gopf_last_error(const gopf_ctx *ctx);
const char *gopf_status_string(int status);
/* Enqueue all work on this CUDA stream (a cudaStream_t); NULL restores the context's own stream. */
int gopf_set_stream(gopf_ctx *ctx, void *cuda_stream);
int gopf_set_option(gopf_ctx *ctx, int option, long long value);

/* ---- model definition, pf.Model mirror (pf/model.go) ---- */
int gopf_add_field(gopf_ctx *ctx, const char *name, int *field_id);               /* Model.AddField */
int gopf_add_scalar(gopf_ctx *ctx, const char *name, double re, double im);       /* Model.AddScalar */
/* Model.RegisterFunction restricted to device pointwise kinds (GOPF_DER_*). */
int gopf_register_function(gopf_ctx *ctx, const char *name, int kind, const char *field,
                           const double *coefs, const int *powers, int nterms);
/* NewHomogeneousModolus + RegisterExplicitTerm(term_name, ...): C is the 3x3x3x3 stiffness
 * (index i*27+j*9+k*3+l, elasticity/rank4.go:19-21), misfit the 3x3 misfit strain. */
int gopf_register_elastic(gopf_ctx *ctx, const char *term_name, const char *field, const double *C81,
                          const double *misfit9);
/* NewVolumeConservingLP + RegisterExplicitTerm(term_name, ...) */
/* Model.RegisterImplicitTerm with a TensorialHessian (pf/tensorialHessian.go:38-80): K has 4 (2D) or
 * 9 (3D) entries, row-major over the reference's axis order (row, col, depth). */
int gopf_register_hessian(gopf_ctx *ctx, const char *term_name, const double *K, int nk);
/* Model.RegisterImplicitTerm with a SpectralViscosity (pf/spectralViscosity.go:22-58). */
int gopf_register_spectral_viscosity(gopf_ctx *ctx, const char *term_name, double eps, double threshold, int power);
int gopf_register_volcons(gopf_ctx *ctx, const char *term_name, const char *field, const char *indicator,
                          double dt);
/* VolumeConservingLP.Multiplier (pf/volumeConserving.go:9) as the device holds it after the steps
 * taken so far (GOPF_ERR_STATE when the model has no such term). */
int gopf_volcons_multiplier(gopf_ctx *ctx, double *out);
/* Model.RegisterFunction for a closure that is a polynomial of several fields (the chemical
 * potentials of examples/strain_single_precipitate/main.go:36-55, for instance):
 * value = sum_t coefs[t] * prod_f field_f^powers[t * nfields + f], where field f is the f-th
 * field added (AddField order), nfields <= the fields added so far (at most 4), 1 <= nterms <= 8
 * and 0 <= powers <= 64.  Registered as a derived field of kind GOPF_DER_MPOLY. */
int gopf_register_polynomial(gopf_ctx *ctx, const char *name, const double *coefs, const int *powers, int nterms,
                             int nfields);
/* WhiteNoise (pf/noise.go:11-23) registered as a function, or ConservativeNoise
 * (pf/noise.go:25-99) registered as an explicit term, with strength S and a seed for
 * the device's counter-based generator.  The noise is drawn per mode in k space with
 * the statistics of the FFT of real white noise N(0, 2S); it matches the reference
 * statistically, not sample for sample (the reference uses Go's global math/rand). */
int gopf_register_noise(gopf_ctx *ctx, const char *name, int kind, const char *field, double strength,
                        unsigned long long seed);
int gopf_add_equation(gopf_ctx *ctx, const char *equation);                       /* Model.AddEquation */
/* Model.Init + pf.Build: compile every equation into the device term table. */
int gopf_init(gopf_ctx *ctx);
/* Number of explicit/implicit terms of equation eq after gopf_init (Model.Summarize's NE/NI). */
int gopf_equation_summary(gopf_ctx *ctx, int eq, int *n_explicit, int *n_implicit);
/* Copy out the compiled term table (for inspection and tests). */
int gopf_get_terms(gopf_ctx *ctx, gopf_term *terms, int capacity, int *nterms);
int gopf_get_derived(gopf_ctx *ctx, gopf_derived *der, int capacity, int *nder);

/* ---- model definition, pre-compiled (what a Go shim builds from pf.Model.RHS) ---- */
int gopf_set_terms(gopf_ctx *ctx, int nfields, const gopf_derived *derived, int nderived, const gopf_term *terms,
                   int nterms);

/* ---- stepping (pf.TimeStepper) ---- */
int gopf_set_stepper(gopf_ctx *ctx, int stepper, double dt);
/* Euler.SetFilter / RK4.SetFilter (pf/euler.go:61-64, pf/rk4.go:137-140) for a tabulated
 * ModalFilter: after every update c-hat(k) is multiplied by filter(2|f|/pi) (ApplyModalFilter,
 * pf/util.go:125-132), interpolated in the n samples of [0, 1] as Vandeven.Eval does
 * (pf/vandeven.go:30-40).  n = 0 (or table = NULL) removes the filter.  Call after gopf_init.
 * ImplicitEuler ignores filters, as the reference's does. */
int gopf_set_modal_filter(gopf_ctx *ctx, const double *table, int n);
/* NewVandeven(order).Data (pf/vandeven.go:13-27) into out[1000]. */
int gopf_vandeven_table(int order, double *out, int n);
/* ImplicitEuler's Newton-Krylov controls: the fields of nonlin.NewtonKrylov that DefaultNonLinSolver
 * sets (pf/implicitEuler.go:221-228; defaults maxiter 50, step 1e-3, tol 1e-7, stencil 6) plus the
 * GMRES basis size (default 50; each vector is one real field on the device).  tol bounds
 * max|F(x)| of the real-space residual of updateEquation (pf/implicitEuler.go:68-94). */
int gopf_set_newton_krylov(gopf_ctx *ctx, int maxiter, double step_size, double tol, int stencil, int restart);
/* Outcome of the last ImplicitEuler step: Newton iterations, GMRES iterations in total, max|F|,
 * and whether tol was met (the reference logs a warning and keeps the iterate when it is not,
 * pf/implicitEuler.go:199-201; so does gopf_step). */
int gopf_newton_stats(gopf_ctx *ctx, int *newton_iters, int *krylov_iters, double *residual, int *converged);
/* Field.Data <-> device. data is a []complex128 (interleaved re, im; n complex values).
 * Upload takes the real part; the stepped fields are real.  field_id is the field's
 * Model.AddField position: a model may hold up to 4 fields, equation i evolving field i
 * (pf/euler.go:26-47, pf/rk4.go:29-74 loop over m.Fields with m.RHS[i]).  Fields never
 * uploaded start at zero, like pf.NewField(name, n, nil).  Multi-field models step with
 * Euler, RK4 or ImplicitEuler; their explicit terms are products of powers of any fields
 * (gopf_register_polynomial for sums of them) and their implicit terms polynomials in the
 * Laplacian or TensorialHessian / SpectralViscosity symbols.  The elastic, volume-conserving
 * and noise terms (one of each per model, on any field and in any equation) step with Euler. */
int gopf_field_upload(gopf_ctx *ctx, int field_id, const double *data, size_t n);
int gopf_field_download(gopf_ctx *ctx, int field_id, double *data, size_t n);
/* Real-valued variants (n doubles) */
int gopf_field_upload_real(gopf_ctx *ctx, int field_id, const double *data, size_t n);
int gopf_field_download_real(gopf_ctx *ctx, int field_id, double *data, size_t n);
/* Solver.Propagate(nsteps): nsteps steps plus the per-step OnStepFinished hooks of device terms. */
int gopf_step(gopf_ctx *ctx, long long nsteps);
/* Capture the CUDA graphs that gopf_step(ctx, nsteps) replays without running any step, so that a
 * later timed or latency-critical gopf_step pays no capture.  Host-driven steppers (ImplicitEuler,
 * SDD) and contexts with graphs switched off have nothing to prepare; an elastic model prepares
 * after its first step (that step sees the reference's zero h-field and is not replayed).  No
 * counterpart in the reference (pf.Solver has no set-up phase). */
int gopf_prepare_graphs(gopf_ctx *ctx, long long nsteps);
int gopf_get_time(gopf_ctx *ctx, double *t);
int gopf_get_step(gopf_ctx *ctx, long long *step);
int gopf_synchronize(gopf_ctx *ctx);

/* ---- field files (pf/fileIO.go) ----
 * Float64IO.SaveFields / SaveFloat64 (pf/fileIO.go:45-97): the real field as raw big-endian
 * float64 in node order, readable by LoadFloat64 and by the XDMF files of pf.WriteXDMF.  The byte
 * swap runs on the GPU; with async != 0 the call returns once the copy is queued and a host thread
 * writes the file while the device keeps stepping (the next save or gopf_io_wait collects it). */
int gopf_save_float64(gopf_ctx *ctx, int field_id, const char *path, int async);
int gopf_io_wait(gopf_ctx *ctx);
/* LoadFloat64 (pf/fileIO.go:64-83) followed by gopf_field_upload_real: restart from a saved field. */
int gopf_load_float64(gopf_ctx *ctx, int field_id, const char *path);

/* ---- point sources (Model.AddSource, pf/model.go:152-154; Source, pf/sourceTerm.go:14-30) ----
 * A source adds f(t) exp(-2 pi i Freq(k) . pos) to the right-hand side of equation eq (pos: one
 * coordinate per dimension, in the reference's (row, col, depth) order).  f is a Go closure, so
 * its values come from the caller: gopf_set_source_amplitudes takes amps[s * nsteps + i] =
 * f_s(t) for the steps starting at the current one (t = step dt at the start of each step, the
 * time Euler and RK4 pass to GetRHS), for every source in gopf_add_source order; gopf_step
 * fails with GOPF_ERR_STATE for steps the table does not cover.  Euler and RK4 (one or several
 * fields); at most 4 sources per equation.  A real field carries the Hermitian part of the
 * source: for positions off the grid the Nyquist components contribute cos(pi pos) (the
 * reference's complex field also carries an imaginary part there). */
int gopf_add_source(gopf_ctx *ctx, int eq, const double *pos, int npos, int *source_id);
int gopf_set_source_amplitudes(gopf_ctx *ctx, const double *amps, int nsources, int nsteps);

/* ---- shrinking-dimer dynamics (pf/sdd.go), stepped by gopf_step with GOPF_STEPPER_SDD ----
 * The orientation is nfields * N reals, field after field in node order.  gopf_sdd_init is
 * SDD.Init (pf/sdd.go:386-404: final - init, its length the initial dimer length) and
 * gopf_sdd_set_orientation SDD.SetInitialOrientation (:409-424); either starts a new dimer at
 * time 0, as NewSDD does.  gopf_sdd_set_params sets Alpha, TimeConstants.Orientation,
 * TimeConstants.DimerLength, InitDimerLength (when > 0) and MinDimerLength (defaults 0.5, 1, 1,
 * -, 0, pf/sdd.go:118-127).  gopf_sdd_monitor gives the SDDMonitor fields (:27-52): MaxForce,
 * ForcePowerSpectrum, MaxTorque, FieldNorm, FieldNormChange.  SDD steps models with polynomial
 * explicit terms and Laplacian-polynomial implicit terms; it rejects modal filters, as the
 * reference's SetFilter panics (:426-430). */
int gopf_sdd_init(gopf_ctx *ctx, const double *init, const double *final, size_t n);
int gopf_sdd_set_orientation(gopf_ctx *ctx, const double *orientation, size_t n);
int gopf_sdd_set_params(gopf_ctx *ctx, double alpha, double tau_orientation, double tau_length, double init_length,
                        double min_length);
int gopf_sdd_get_orientation(gopf_ctx *ctx, double *orientation, size_t n);
int gopf_sdd_monitor(gopf_ctx *ctx, double *out5);
/* DimerLength(t) (pf/sdd.go:355-362) */
int gopf_sdd_dimer_length(gopf_ctx *ctx, double t, double *length);

/* ---- monitors ---- */
int gopf_reduce(gopf_ctx *ctx, int field_id, int what, double *out);
/* PointMonitor.Add (pf/monitor.go:27-30) for n sites at once: out[k] = real(field[sites[k]]), sites
 * being node indices (pfutil/indexPositionConversion.go:23-34).  Only the n values cross the bus. */
int gopf_point_values(gopf_ctx *ctx, int field_id, const long long *sites, int n, double *out);

/* ---- energy monitors (the Monitor hook of pf/monitor.go:4-6, run per epoch by Solver.Solve,
 * pf/solver.go:110-117), evaluated on the device-resident field ----
 * gopf_free_energy: out3 = {bulk, gradient, total} of
 *   F = sum_cells sum_p coefs[p] c^p + (kappa/2) sum_cells |grad c|^2
 * (0 <= ncoefs <= 13), the gradient part from the spectrum with |k|^2 = 4 pi^2 |Freq|^2, the symbol
 * the model's LAP uses.  coefs = {0, 0, -1/2, 0, 1/4} and kappa = gamma give the free energy of the
 * Cahn-Hilliard string of examples/cahnHilliard/main.go:33.  Per-cell terms in the context's
 * precision (an FP32 context adds them 16 at a time in FP32), FP64 sums with Neumaier compensation
 * of the thread and block partials; GOPF_ERR_NAN when the field holds non-finite values.  No
 * counterpart in the reference (its monitors are user code). */
int gopf_free_energy(gopf_ctx *ctx, int field, const double *coefs, int ncoefs, double kappa, double *out3);
/* elasticity.HomogeneousModulusEnergy (elasticity/linearElasticity.go:101-165) of the indicator x =
 * the field (indicator == 0) or its Indicator 3c^2 - 2c^3 (indicator != 0, pf/homoLinElast.go:10-12):
 * elastic energy over sum x, the misfit subtracted where x > 1/2.  C81 and misfit9 as in
 * gopf_register_elastic.  The transforms and per-cell terms run in the context's precision, the
 * sums in FP64 as for gopf_free_energy. */
int gopf_elastic_energy(gopf_ctx *ctx, int field, int indicator, const double *C81, const double *misfit9,
                        double *out);

/* ---- FourierTransform (pfutil/fftWrap.go) on host data, not a hot path ---- */
/* sign -1: forward FFT, +1: unnormalised backward, of a []complex128 of length N. */
int gopf_fft(gopf_ctx *ctx, int sign, double *data, size_t n);
/* Freq(i): writes ndim frequencies (cycles/sample, (-0.5, 0.5]) */
int gopf_freq(gopf_ctx *ctx, long long i, double *out);
long long gopf_conjugate_node(gopf_ctx *ctx, long long i);

/* ---- adjoint of the semi-implicit Cahn-Hilliard step (no counterpart in the reference) ----
 * Model: dconc/dt = M*LAP MU - M*gamma*LAP^2 conc with MU = conc^3 - conc, Euler
 * (pf/euler.go:16-47).  gopf_adjoint_forward installs that model on the context,
 * runs nsteps steps from the real field c0 (N doubles), keeps the field every
 * `every` steps on the device and writes c_T (N doubles, may be NULL).
 * gopf_adjoint_backward takes lambda_T = dL/dc_T (N doubles) and returns dL/dgamma,
 * dL/dM and dL/dc0 (N doubles, may be NULL), recomputing each checkpoint segment. */
int gopf_adjoint_forward(gopf_ctx *ctx, double gamma, double M, double dt, int nsteps, int every, const double *c0,
                         double *cT);
int gopf_adjoint_backward(gopf_ctx *ctx, const double *lambda_T, double *dgamma, double *dM, double *dc0);
int gopf_adjoint_release(gopf_ctx *ctx);

/* ---- batches: many independent 2D instances stepped by shared launches ----
 * Replaces running one pf.Solver per swept parameter set (the workflow the
 * sweep database serves, README.md:21-33, pf/database.go:67-80); it has no
 * single counterpart in the reference.  Every context keeps its own model,
 * dt and device state; gopf_batch_step(nsteps) advances all of them by
 * nsteps Euler steps, captured in CUDA graphs of 1 and 16 steps.  By default
 * one persistent kernel per graph steps every instance (gopf_batch_set_mode
 * below).  Otherwise each size class gets an x-pass and a y-pass launch per
 * step, plus the projection of the self-conjugate lines.  When the x and y
 * classes cover the same instances each class runs its x, y and projection
 * launches on its own branch for all steps of a graph (3 launches per class
 * and step).  Otherwise the classes of a pass run side by side and one
 * projection of every instance ends each step (2 x classes + 1).
 * gopf_batch_kernels_per_step reports the launches per step (1 when
 * persistent).
 * Contexts must be 2D, single-field, Euler, without user-defined terms, on one
 * device and precision, and stay alive while the batch exists. */
typedef struct gopf_batch gopf_batch;
int gopf_batch_create(gopf_ctx *const *ctxs, int n, gopf_batch **out);
int gopf_batch_destroy(gopf_batch *batch);
const char *gopf_batch_last_error(const gopf_batch *batch);
int gopf_batch_set_stream(gopf_batch *batch, void *cuda_stream);
int gopf_batch_step(gopf_batch *batch, long long nsteps);
int gopf_batch_kernels_per_step(gopf_batch *batch, int *n);
/* Kernel families of a batch pass (no counterpart in the reference; FFTW's measured planning,
 * pfutil/fftWrap.go:19-20 with fftw.MEASURE, plays the same role for its CPU transforms). */
enum {
    GOPF_BATCH_AUTO = -1,        /* the built-in preference: LINE, else STOCKHAM_CT, else STOCKHAM */
    GOPF_BATCH_LINE = 0,         /* register-resident line engine (FP32, sides 256, 384, 512, 768, 1024) */
    GOPF_BATCH_STOCKHAM_CT = 1,  /* Stockham tiles with compile-time plans (FP32, sides 128 ... 1024) */
    GOPF_BATCH_STOCKHAM = 2      /* Stockham tiles with runtime plans (any supported length, FP32 and FP64) */
};
/* Autotuner: for each kind of instance in the batch (sides, precision, term groups) time every
 * candidate of the x pass (family; for runtime plans the tile width 4, 8, 16 and plan variant 0, 1,
 * 2: radix 16, 8 or 4 stages) and then of the y pass on the batch's own instances (reps timed
 * steps each, CUDA events; the fields are restored afterwards), keep the fastest and rebuild the
 * batch.  Choices are cached per process and kind, so later batches of the same kinds tune without
 * timing.  gopf_batch_tune_reset empties the cache. */
int gopf_batch_tune(gopf_batch *batch, int reps);
int gopf_batch_tune_reset(void);
/* Force one choice on every instance (a family that cannot serve an instance falls back to the
 * built-in preference for it; lb 0 keeps the context's tile width) and rebuild the batch. */
int gopf_batch_force(gopf_batch *batch, int xfam, int yfam, int lbx, int lby, int xplan, int yplan);
/* The choice in effect for instance inst: {xfam, yfam, lbx, lby, xplan, yplan}. */
int gopf_batch_choice(gopf_batch *batch, int inst, int *out6);
/* How a batch steps (no counterpart in the reference).
 * GOPF_BATCH_MODE_PERSISTENT: one persistent kernel steps every instance for all the steps of a
 * captured graph (1 or 16 steps per launch). Its blocks take x and y tiles of all instances from
 * one queue; per-instance completion counters order an instance's y tiles after its x tiles and its
 * next x tiles after its y tiles. Each wait is bounded, and one that runs out makes
 * gopf_batch_step return GOPF_ERR_TIMEOUT. It takes FP32 instances of sides 256 ... 1024 with one
 * dense polynomial group (line engine) and of side 128 (compile-time Stockham tiles). The kernel
 * families are then fixed, so gopf_batch_tune keeps them.
 * GOPF_BATCH_MODE_CHAINS: a launch per class and pass, with the classes as graph branches.
 * GOPF_BATCH_MODE_AUTO (default): persistent when every instance allows it, else chains. */
enum { GOPF_BATCH_MODE_AUTO = -1, GOPF_BATCH_MODE_CHAINS = 0, GOPF_BATCH_MODE_PERSISTENT = 1 };
int gopf_batch_set_mode(gopf_batch *batch, int mode);
/* The mode in effect: GOPF_BATCH_MODE_CHAINS or GOPF_BATCH_MODE_PERSISTENT. */
int gopf_batch_mode(gopf_batch *batch, int *mode);
/* Limit (ns) of the persistent kernel's waits for an item's dependencies; 0 (default) = 2 s. Meant for
 * testing the timeout path. */
int gopf_batch_set_wait_limit(gopf_batch *batch, long long ns);

/* ---- sweeps over several GPUs, one process each ----
 * The sweep workflow (README.md:21-33) runs one pf.Solver per parameter set; its instances are
 * independent, so processes split them with no exchange.  gopf_sweep_partition assigns instance i
 * (cells[i] grid cells) to owner[i] in [0, world): greedy bin packing on cells, instances in
 * decreasing size (ties: lower index) to the least-loaded rank (ties: lower rank).  Deterministic,
 * so every process computes the same partition alone; rank_cells (world entries, may be NULL)
 * receives each rank's total.  Host-only: needs no device. */
int gopf_sweep_partition(const long long *cells, int n, int world, int *owner, long long *rank_cells);

/* ---- reduction without device allocation (no counterpart in the reference) ----
 * For callers that cannot allocate device memory at the point of the call (a host
 * that manages all device memory itself, an allocator budget enforced outside CUDA,
 * a pool that must not be touched).  Reduces a real FP64 field the caller holds in
 * device memory; out receives, on the host, {sum, sum of squares, min, max,
 * non-finite count}.  Sums are compensated (Neumaier) as in gopf_reduce, so for a
 * finite field the values agree with gopf_reduce's within rounding.  Non-finite
 * cells: the count is exact, min and max skip NaN (IEEE fmin/fmax) but see +-Inf, and
 * the sums follow IEEE arithmetic (a context cannot hold a single non-finite cell:
 * its spectral state turns every cell non-finite, so gopf_reduce counts them all).
 * Its only scratch is a static device array of GOPF_NOALLOC_MAX_BLOCKS + 1 rows of
 * 8 doubles (about 1 MiB per GPU that loads the library, held until exit), so n is
 * limited to GOPF_NOALLOC_MAX_BLOCKS * 4096 elements; larger n returns GOPF_ERR_ARG.
 * Each call looks the scratch address up with the caller's device current; the first
 * call on a device also loads the device code and should come before any stream
 * capture.  The call is synchronous: it returns once the result is on the host.
 * Calls share the scratch: calls that overlap on the GPU race and must be serialised
 * by the caller.  stream may be NULL (the default stream). */
#define GOPF_NOALLOC_MAX_BLOCKS 16384
int gopf_reduce_noalloc(const double *field, size_t n, double *out, void *cuda_stream);
const char *gopf_noalloc_last_error(void);

/* ---- introspection ---- */
/* Bytes of device memory held by the context. */
int gopf_device_bytes(gopf_ctx *ctx, size_t *bytes);
/* Number of kernel launches enqueued by one step of the current stepper. */
/* Kernel launches that gopf_step(ctx, nsteps) makes through its captured graphs (known once both
 * graphs exist, i.e. after a gopf_step of at least 16 steps).  No counterpart in the reference. */
int gopf_kernel_launches(gopf_ctx *ctx, long long nsteps, long long *count);
int gopf_kernels_per_step(gopf_ctx *ctx, int *n);
/* Run nsteps Euler steps launch by launch with CUDA events between kernels on the
 * context's stream; per kernel slot of one step write the average device time (ms)
 * and the algorithmic HBM bytes (each array read and written once).  Advances the state.
 * (Timing the same step captured as a graph with event nodes gave slightly longer times: the
 * event nodes themselves separate the kernels.)  No counterpart in the reference. */
int gopf_profile_step(gopf_ctx *ctx, int nsteps, double *avg_ms, double *alg_bytes, int capacity, int *nslots);
int gopf_profile_slot_name(gopf_ctx *ctx, int slot, char *buf, int buflen);

#ifdef __cplusplus
}
#endif
#endif /* GOPF_GPU_H */
