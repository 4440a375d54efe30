// gopf_ctx.h -- internal definition of gopf_ctx shared by the C-ABI translation units.
#pragma once
#include <complex>
#include <map>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "../../include/gopf_gpu.h"
#include "gopf_types.h"

// Host-side mirror of the parts of pf.Model that the equation strings refer to.
struct gopf_modeldef {
    std::vector<std::string> fields;                             // Model.Fields names, in AddField order
    std::map<std::string, std::complex<double>> scalars;         // Scalar bricks
    struct Func {
        std::string name;
        int kind;
        int field;
        std::vector<double> coefs;
        std::vector<int> powers;
    };
    std::vector<Func> funcs;                                     // RegisterFunction (device kinds only)
    struct Elastic {
        std::string name;
        int field;
        double C[81];
        double misfit[9];
    };
    std::vector<Elastic> elastic;                                // HomogeneousModulusLinElast terms
    struct Volcons {
        std::string name;
        int field;
        std::string indicator;
        double dt;
    };
    std::vector<Volcons> volcons;                                // VolumeConservingLP terms
    struct Noise {
        std::string name;
        int kind; // 1 white (a derived field), 2 conservative (a user term)
        int field;
        double strength;
        unsigned long long seed;
    };
    std::vector<Noise> noise;                                    // WhiteNoise / ConservativeNoise
    struct ImplicitSym {
        std::string name;
        int kind; // 1 TensorialHessian, 2 SpectralViscosity
        double K[9];
        int nk;
        double eps, threshold;
        int power;
    };
    std::vector<ImplicitSym> isym;                               // RegisterImplicitTerm with a symbol
    std::vector<std::string> equations;                          // AddEquation (spaces removed)
    std::vector<std::string> derived_names;                      // derived fields, in registration order
    std::vector<gopf_derived> derived;
};

// A special (non-polynomial) explicit term attached to an equation.
struct gopf_special {
    int kind; // 1 elastic, 2 volcons
    int index;
    int eq;
    double coef;
    int lap;
};

struct gopf_ie_work;
struct gopf_sdd_work;
struct gopf_io_state;
struct gopf_energy_work;

struct gopf_ctx {
    int device = 0;
    int ndim = 0;
    int dims[3] = {1, 1, 1};
    int prec = GOPF_FP32;
    gopf::Geom g{};
    int LBx = 16, LBy = 16, LBz = 16; // tile widths of the x, y and z passes
    cudaStream_t own_stream = nullptr;
    cudaStream_t side_stream = nullptr;        // second branch of a step (Hermitian projection)
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaStream_t stream = nullptr;

    // device buffers (element type float2/double2 for spectral, float/double for real)
    void *d_state = nullptr;
    void *d_T = nullptr;
    void *d_U[GOPF_MAX_GROUPS] = {nullptr, nullptr, nullptr, nullptr};
    void *d_real = nullptr;
    double2 *d_c128 = nullptr;
    double *d_red = nullptr;
    double *d_redout = nullptr;
    int nred_blocks = 0;
    void *d_twX = nullptr, *d_twY = nullptr, *d_twZ = nullptr;
    gopf::LinePlan planH{}, planY{}, planZ{};
    size_t dev_bytes = 0;

    // model
    gopf_modeldef def;
    bool initialised = false;  // gopf_init / gopf_set_terms done
    int nfields = 0;
    std::vector<gopf_derived> der;
    std::vector<gopf_term> terms;
    std::vector<gopf_special> specials;
    gopf::PwTable pw{};
    gopf::UpdTable upd{};
    int ngroups = 0;

    // stepping
    int stepper = GOPF_STEPPER_EULER;
    double dt = 0.0;
    long long step = 0;
    bool state_valid = false;

    // graphs
    cudaGraphExec_t gexec1 = nullptr;
    cudaGraphExec_t gexecK = nullptr;
    int graphK = 16;
    long long graph_kernels1 = 0, graph_kernelsK = 0; // kernel nodes of the two graphs
    bool graphs_dirty = true;

    // Khachaturyan term (at most one per context)
    bool has_elastic = false;
    double el_C[81] = {0};
    double el_A[9] = {0};
    double el_e0 = 0.0, el_coef = 1.0;
    int el_lap = 0;
    int el_field = 0, el_eq = 0; // multi-field models: the field of H(c) and the equation of the term
    int mono_H = -1;             // multi-field models: index of H(c) in the Euler plan's monomial table
    bool el_primed = false; // false until the first step: the reference's h-field starts at zero
    void *d_bsym = nullptr;
    void *d_U0 = nullptr; // group-0 buffer separate from T (T must survive the elastic step)
    void *d_UH = nullptr; // H-hat, then the elastic term
    gopf::PwTable pw_el{}; // polynomial groups + the indicator H(c)

    // VolumeConservingLP (at most one per context)
    bool has_volcons = false;
    int vc_group = -1;
    double vc_dt = 0.0, vc_coef = 1.0;
    double *d_vc = nullptr;   // [lambda, current integral, previous indicator integral, count, coef*lambda]
    double *d_red2 = nullptr; // block sums of the indicator
    // multi-field models: the term's field and equation, the indicator's index in the monomial
    // table (vc_group), and block sums of the field over the multi-field x-pass grid
    int vc_field = 0, vc_eq = 0, vc_local = -1;
    double *d_vcred = nullptr;

    void *d_rkF = nullptr; // RK4 accumulator

    // Multi-field models (pf.Model with several fields, pf/euler.go:26-40 loops over them).
    // Field 0 keeps d_state / d_T / d_rkF; fields 1.. have their own arrays.  One x-pass reads
    // every field and writes the explicit groups of every equation (mono); each equation then
    // gets its own forward pass and fused update with its own UpdTable.  Equation e's first
    // group lands in T of field e, its further groups in d_mU.
    bool multi = false;
    void *d_fstate[GOPF_MAX_FIELDS] = {nullptr, nullptr, nullptr, nullptr};
    void *d_fT[GOPF_MAX_FIELDS] = {nullptr, nullptr, nullptr, nullptr};
    void *d_frkF[GOPF_MAX_FIELDS] = {nullptr, nullptr, nullptr, nullptr};
    void *d_mU[GOPF_MAX_XOUT] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    struct EqPlan {
        gopf::UpdTable upd; // ngrp, glap, imp, implicit user terms, k-space field terms
        int first;          // index of its first group in mono
        int ubuf[GOPF_MAX_GROUPS]; // -1: T of the field; else an index into d_mU
        int xf_field[GOPF_MAX_FIELDS]; // field of each k-space field term (upd.xf_*)
    };
    std::vector<EqPlan> eqs, eqs_rk; // Euler plan (field terms in k space), RK4 plan
    gopf::MonoTable mono{}, mono_rk{};
    int LBm = 4; // x-pass tile width of the multi-field x-pass (nfields + 1 tiles in shared memory)

    // point sources (Model.AddSource, pf/sourceTerm.go): equation and position; the amplitudes
    // f_s(t) of the steps [src_base, src_base + src_len) in d_srcamp[s * src_len + i], and the
    // device count of steps taken since src_base (the graphs read it)
    struct SourceDef {
        int eq;
        double pos[3];
    };
    std::vector<SourceDef> sources;
    double *d_srcamp = nullptr;
    size_t srcamp_cap = 0;
    unsigned long long *d_srcctr = nullptr;
    long long src_base = 0, src_len = 0;

    // Gaussian noise term (at most one per context) and the device step counter keying it
    gopf::NoiseParams noise{};
    int noise_eq = -1; // multi-field models: the equation drawing the noise (-1: none)
    unsigned long long *d_stepctr = nullptr;
    void *d_filter = nullptr; // modal filter table (precision of the context)
    unsigned *d_status = nullptr; // device status word of the bounded waits (0 = clean)

    // per-kernel profiling (gopf_profile_step): events recorded after each launch
    std::vector<cudaEvent_t> *prof_events = nullptr;
    size_t prof_next = 0;

    int check_finite = 1;
    int use_graphs = 1;
    int use_fast = 1;
    int use_tma = 1;
    int x_rows = 16; // tile height of the one-group 256-point x pass (GOPF_OPT_X_ROWS)
    int z_lines = 8;  // tile width of the one-group 256-point z pass (GOPF_OPT_Z_LINES)
    int use_pdl = 1;  // the step's y, z and y passes as programmatic dependents (GOPF_OPT_PDL)
    int use_direct_host = 1;

    // ImplicitEuler's Newton-Krylov controls (DefaultNonLinSolver, pf/implicitEuler.go:221-228) and
    // the outcome of the last step
    int nk_maxiter = 50;
    double nk_step = 1e-3;
    double nk_tol = 1e-7;
    int nk_stencil = 6;
    int nk_restart = 50;
    double nk_krylov_rtol = 1e-8;
    int nk_last_newton = 0, nk_last_krylov = 0, nk_last_converged = 0;
    double nk_last_residual = 0.0;
    gopf_ie_work *ie = nullptr;
    // shrinking-dimer dynamics (pf/sdd.go): parameters of SDD and its device workspace
    double sdd_alpha = 0.5, sdd_tau_orient = 1.0, sdd_tau_len = 1.0, sdd_init_len = 0.0, sdd_min_len = 0.0;
    long long sdd_step = 0; // SDD.CurrentStep
    gopf_sdd_work *sdd = nullptr;
    gopf_io_state *io = nullptr; // field files: pinned staging buffer and writer thread
    gopf_energy_work *energy = nullptr; // energy monitors (gopf_energy.cu): work buffers
    std::string err;
};

// per-field device arrays: field 0 uses the context's own, fields 1.. the multi-field set
inline void *field_state(gopf_ctx *ctx, int f) { return f == 0 ? ctx->d_state : ctx->d_fstate[f]; }
inline void *field_T(gopf_ctx *ctx, int f) { return f == 0 ? ctx->d_T : ctx->d_fT[f]; }
inline void *field_rkF(gopf_ctx *ctx, int f) { return f == 0 ? ctx->d_rkF : ctx->d_frkF[f]; }

int gopf_fail(gopf_ctx *ctx, int code, const std::string &msg);
bool gopf_make_plan(int n, int tws, int variant, gopf::LinePlan &pl);
int gopf_compile_model(gopf_ctx *ctx);
int gopf_elastic_table(gopf_ctx *ctx);
// the multiplier update of VolumeConservingLP from the block sums of the field (red_field) and of
// the indicator (d_red2) over an x-pass grid of nblocks blocks
cudaError_t gopf_launch_volcons_finalize(gopf_ctx *ctx, const double *red_field, int nblocks);
cudaError_t gopf_launch_hermitian_planes(gopf_ctx *ctx, void *state, cudaStream_t st = nullptr);

// NVTX range for the lifetime of a scope (a host-side trace marker; a no-op unless a profiler
// or tracer is attached)
struct gopf_nvtx_scope {
    explicit gopf_nvtx_scope(const char *name) { nvtxRangePushA(name); }
    ~gopf_nvtx_scope() { nvtxRangePop(); }
};

// cudaMalloc for the library's device buffers.  Test hook: when the environment variable
// GOPF_TEST_FAIL_ALLOC=k is set, the k-th allocation of the process fails with
// cudaErrorMemoryAllocation (host-side fault injection; the GPU is never touched).
cudaError_t gopf_malloc(void **p, size_t bytes);
template <typename T> inline cudaError_t gopf_malloc(T **p, size_t bytes)
{
    return gopf_malloc(reinterpret_cast<void **>(p), bytes);
}
