"""ctypes front end of the CPU FP64 oracle (oracle/gopf_oracle.c).

Test infrastructure only: the test-suite, the smoke check and the CPU-baseline
leg of bench.py use this module as the reference computation.  The product
path never imports it.

The model object mirrors how gopf's pf.Model is driven by pf.Solver:
fields are complex128 arrays in the reference's node order
(pfutil/indexPositionConversion.go:23-34), terms are what pf.Build produces
(pf/rhsBuilder.go:26-54) written out explicitly, and `step_euler(hooks=True)`
is Solver.Propagate (pf/solver.go:70-84) over Euler.Step (pf/euler.go:16-47).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libgopf_oracle.so")
_lib = None

DER_PRODUCT, DER_POLY, DER_INDICATOR, DER_INDICATOR_D, DER_INDICATOR_HD = range(5)
DER_MPOLY = 6
SRC_NONE, SRC_FIELD, SRC_DERIVED = range(3)


def build(force: bool = False) -> str:
    """Compile the oracle with the Makefile beside this file."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "gopf_oracle.c"))
    ):
        r = subprocess.run(["make", "-C", _HERE, "-B" if force else "all"], capture_output=True, text=True)
        if r.returncode != 0:
            # retry without OpenMP (a toolchain without libgomp)
            r = subprocess.run(["make", "-C", _HERE, "-B", "OMPFLAGS="], capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        vp = ctypes.c_void_p
        L.or_fftn.argtypes = [ctypes.c_int, ip, dp, ctypes.c_int]
        L.or_fftn.restype = ctypes.c_int
        L.or_freq.argtypes = [ctypes.c_int, ip, ctypes.c_long, dp]
        L.or_conjugate_node.argtypes = [ctypes.c_int, ip, ctypes.c_long]
        L.or_conjugate_node.restype = ctypes.c_long
        L.or_model_create.argtypes = [ctypes.c_int, ip, ctypes.c_int]
        L.or_model_create.restype = vp
        L.or_model_destroy.argtypes = [vp]
        L.or_field.argtypes = [vp, ctypes.c_int]
        L.or_field.restype = dp
        L.or_derived_data.argtypes = [vp, ctypes.c_int]
        L.or_derived_data.restype = dp
        L.or_add_derived.argtypes = [vp, ctypes.c_int, ctypes.c_int, ip, ip, dp]
        L.or_add_derived.restype = ctypes.c_int
        L.or_add_term.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.or_add_term.restype = ctypes.c_int
        L.or_add_elastic.argtypes = [vp, ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_double, ctypes.c_int]
        L.or_add_elastic.restype = ctypes.c_int
        L.or_elastic_set_disp_override.argtypes = [vp, ctypes.c_int, dp]
        L.or_elastic_hfield.argtypes = [vp, ctypes.c_int]
        L.or_elastic_hfield.restype = dp
        L.or_add_volcons.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_int]
        L.or_add_volcons.restype = ctypes.c_int
        L.or_volcons_multiplier.argtypes = [vp, ctypes.c_int]
        L.or_volcons_multiplier.restype = ctypes.c_double
        L.or_step_euler.argtypes = [vp, ctypes.c_double, ctypes.c_long, ctypes.c_int]
        L.or_step_rk4.argtypes = [vp, ctypes.c_double, ctypes.c_long, ctypes.c_int, ctypes.c_int]
        L.or_eval_rhs.argtypes = [vp, ctypes.c_int, dp]
        L.or_eval_denum.argtypes = [vp, ctypes.c_int, dp]
        L.or_current_step.argtypes = [vp]
        L.or_current_step.restype = ctypes.c_long
        L.or_homogeneous_modulus_energy.argtypes = [ctypes.c_int, ip, dp, dp, dp]
        L.or_homogeneous_modulus_energy.restype = ctypes.c_double
        L.or_uniform_field.argtypes = [ctypes.c_uint64, ctypes.c_long, ctypes.c_double, ctypes.c_double, dp]
        L.or_num_threads.restype = ctypes.c_int
        L.or_set_num_threads.argtypes = [ctypes.c_int]
        L.or_add_hessian.argtypes = [vp, ctypes.c_int, dp, ctypes.c_int, ctypes.c_double, ctypes.c_int]
        L.or_add_hessian.restype = ctypes.c_int
        L.or_add_viscosity.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                       ctypes.c_double, ctypes.c_int]
        L.or_add_viscosity.restype = ctypes.c_int
        L.or_sv_interpolant.argtypes = [ctypes.c_double, ctypes.c_double]
        L.or_sv_interpolant.restype = ctypes.c_double
        L.or_vandeven_table.argtypes = [ctypes.c_int, dp, ctypes.c_int]
        L.or_vandeven_table.restype = ctypes.c_int
        L.or_filter_eval.argtypes = [dp, ctypes.c_int, ctypes.c_double]
        L.or_filter_eval.restype = ctypes.c_double
        L.or_set_filter.argtypes = [vp, dp, ctypes.c_int]
        L.or_set_filter.restype = ctypes.c_int
        L.or_add_source.argtypes = [vp, ctypes.c_int, dp, dp, ctypes.c_long]
        L.or_add_source.restype = ctypes.c_int
        L.or_sdd_create.argtypes = [vp]
        L.or_sdd_create.restype = vp
        L.or_sdd_destroy.argtypes = [vp]
        L.or_sdd_set_params.argtypes = [vp] + [ctypes.c_double] * 6
        L.or_sdd_orientation.argtypes = [vp]
        L.or_sdd_orientation.restype = dp
        L.or_sdd_monitor.argtypes = [vp]
        L.or_sdd_monitor.restype = dp
        L.or_sdd_init_length.argtypes = [vp]
        L.or_sdd_init_length.restype = ctypes.c_double
        L.or_sdd_init.argtypes = [vp, dp, dp]
        L.or_sdd_set_orientation.argtypes = [vp, dp]
        L.or_sdd_dimer_length.argtypes = [vp, ctypes.c_double]
        L.or_sdd_dimer_length.restype = ctypes.c_double
        L.or_sdd_step.argtypes = [vp, ctypes.c_long]
        L.or_sdd_step.restype = ctypes.c_int
        L.or_householder.argtypes = [dp, dp, ctypes.c_double, ctypes.c_long, ctypes.c_long]
        L.or_dsm_dot.argtypes = [dp, dp, dp, ctypes.c_long, dp]
        L.or_sdd_denum_dot.argtypes = [dp, dp, ctypes.c_double, ctypes.c_double, ctypes.c_long, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(seq):
    arr = (ctypes.c_int * len(seq))(*seq)
    return arr


def mem_shape(dims):
    """Memory shape (slowest first) of a field of the reference's domainSize."""
    dims = list(dims)
    return tuple(dims) if len(dims) == 2 else (dims[2], dims[0], dims[1])


def fftn(data: np.ndarray, dims, sign: int = -1) -> np.ndarray:
    """Unnormalised Z2Z transform of a complex field in the reference's node order."""
    x = np.ascontiguousarray(data, dtype=np.complex128).copy()
    shape = mem_shape(dims)
    rc = lib().or_fftn(len(shape), _ip(shape), _dp(x.view(np.float64)), sign)
    if rc != 0:
        raise ValueError("unsupported FFT length")
    return x


def freq(dims, i: int) -> np.ndarray:
    out = np.zeros(3)
    lib().or_freq(len(dims), _ip(list(dims)), i, _dp(out))
    return out[: len(dims)]


def conjugate_node(dims, i: int) -> int:
    return int(lib().or_conjugate_node(len(dims), _ip(list(dims)), i))


def uniform_field(seed: int, n: int, center: float, half_width: float) -> np.ndarray:
    out = np.empty(n, dtype=np.float64)
    lib().or_uniform_field(seed, n, center, half_width, _dp(out))
    return out


def vandeven(order: int) -> np.ndarray:
    """NewVandeven(order).Data (pf/vandeven.go:13-27): the 1000-point filter table."""
    out = np.empty(1000)
    if lib().or_vandeven_table(int(order), _dp(out), 1000) != 0:
        raise ValueError("bad order")
    return out


def sv_interpolant(f: float, peak: float) -> float:
    """interpolant (pf/spectralViscosity.go:28-38)."""
    return float(lib().or_sv_interpolant(float(f), float(peak)))


def filter_eval(table: np.ndarray, x: float) -> float:
    """Vandeven.Eval (pf/vandeven.go:30-40)."""
    t = np.ascontiguousarray(table, dtype=np.float64)
    return float(lib().or_filter_eval(_dp(t), t.size, float(x)))


def set_num_threads(n: int) -> None:
    lib().or_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().or_num_threads())


def free_energy(field: np.ndarray, dims, coefs, kappa: float):
    """(bulk, gradient) parts of F = sum_cells sum_p coefs[p] c^p + (kappa/2) sum_cells |grad c|^2 of a
    real field in node order, the gradient through the spectrum with k = 2 pi Freq: the symbol of
    LaplacianN (pf/diffOp.go:25-30) and the frequencies of pfutil/fftWrap.go:57-74 (Nyquist +1/2,
    the same |k| either sign).  numpy, FP64; test infrastructure only."""
    c = np.asarray(field, dtype=np.float64).reshape(-1)
    bulk = float(np.polynomial.polynomial.polyval(c, np.asarray(coefs, dtype=np.float64)).sum())
    shape = mem_shape(dims)
    ch = np.fft.fftn(c.reshape(shape))
    k2 = np.zeros(shape)
    for ax, n in enumerate(shape):
        f = np.fft.fftfreq(n)
        f[np.isclose(f, -0.5)] = 0.5
        sh = [1] * len(shape)
        sh[ax] = n
        k2 = k2 + (f.reshape(sh)) ** 2
    grad = float(4.0 * np.pi ** 2 * (k2 * np.abs(ch) ** 2).sum() / c.size)
    return bulk, 0.5 * kappa * grad


def homogeneous_modulus_energy(indicator: np.ndarray, dims, misfit, C) -> float:
    ind = np.ascontiguousarray(indicator, dtype=np.complex128).copy()
    mis = np.ascontiguousarray(misfit, dtype=np.float64).reshape(9)
    c = np.ascontiguousarray(C, dtype=np.float64).reshape(81)
    return float(lib().or_homogeneous_modulus_energy(len(dims), _ip(list(dims)), _dp(ind.view(np.float64)),
                                                     _dp(mis), _dp(c)))


class Model:
    """A pf.Model whose RHS is given as the term list pf.Build would produce."""

    def __init__(self, dims, nfields: int = 1):
        self.dims = list(dims)
        self.N = int(np.prod(self.dims))
        self._L = lib()
        self._h = self._L.or_model_create(len(self.dims), _ip(self.dims), nfields)
        if not self._h:
            raise ValueError("bad model shape")
        self.nfields = nfields

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.or_model_destroy(h)
            self._h = None

    # --- data ---
    def field(self, f: int = 0) -> np.ndarray:
        """Live view of field f (complex128, length N)."""
        p = self._L.or_field(self._h, f)
        arr = np.ctypeslib.as_array(p, shape=(2 * self.N,))
        return arr.view(np.complex128)

    def set_field(self, f: int, values) -> None:
        self.field(f)[:] = np.asarray(values, dtype=np.complex128).reshape(-1)

    def derived(self, d: int) -> np.ndarray:
        p = self._L.or_derived_data(self._h, d)
        return np.ctypeslib.as_array(p, shape=(2 * self.N,)).view(np.complex128)

    # --- model construction ---
    def add_product(self, fields, powers) -> int:
        """Derived field prod_j field_j^p_j (pf/util.go:38-65)."""
        d = self._L.or_add_derived(self._h, DER_PRODUCT, len(fields), _ip(fields), _ip(powers), None)
        if d < 0:
            raise RuntimeError("too many derived fields")
        return d

    def add_poly(self, field: int, coefs, powers) -> int:
        """Derived field sum_t coef_t field^p_t (a pointwise user function)."""
        c = np.asarray(coefs, dtype=np.float64)
        d = self._L.or_add_derived(self._h, DER_POLY, len(powers), _ip([field] * len(powers)), _ip(powers), _dp(c))
        if d < 0:
            raise RuntimeError("too many derived fields")
        return d

    def add_mpoly(self, coefs, powers) -> int:
        """Derived field sum_t coef_t prod_f field_f^powers[t][f] (a pointwise user function of
        several fields, e.g. the closures of examples/strain_single_precipitate/main.go:36-55)."""
        p = np.asarray(powers, dtype=np.int64)
        packed = [int(sum(int(p[t, f]) << (8 * f) for f in range(p.shape[1]))) for t in range(p.shape[0])]
        c = np.asarray(coefs, dtype=np.float64)
        d = self._L.or_add_derived(self._h, DER_MPOLY, len(packed), _ip([0] * len(packed)), _ip(packed), _dp(c))
        if d < 0:
            raise RuntimeError("too many derived fields")
        return d

    def add_indicator(self, field: int, kind: int) -> int:
        d = self._L.or_add_derived(self._h, kind, 1, _ip([field]), None, None)
        if d < 0:
            raise RuntimeError("too many derived fields")
        return d

    def add_term(self, eq: int, coef, lap: int = 0, implicit: bool = False, src_kind: int = SRC_NONE, src: int = 0):
        coef = complex(coef)
        return self._L.or_add_term(self._h, eq, int(implicit), coef.real, coef.imag, lap, src_kind, src)

    def add_elastic(self, eq: int, field: int, C, misfit, coef: float = 1.0, lap: int = 0) -> int:
        c = np.ascontiguousarray(C, dtype=np.float64).reshape(81)
        m = np.ascontiguousarray(misfit, dtype=np.float64).reshape(9)
        return self._L.or_add_elastic(self._h, eq, field, _dp(c), _dp(m), float(coef), lap)

    def elastic_disp_override(self, e: int, disp) -> None:
        d = np.ascontiguousarray(disp, dtype=np.complex128).reshape(self.N, 3)
        self._L.or_elastic_set_disp_override(self._h, e, _dp(d.view(np.float64)))

    def elastic_hfield(self, e: int) -> np.ndarray:
        p = self._L.or_elastic_hfield(self._h, e)
        return np.ctypeslib.as_array(p, shape=(self.N,))

    def add_volcons(self, eq: int, field: int, indicator: int, dt: float, coef: float = 1.0, lap: int = 0) -> int:
        return self._L.or_add_volcons(self._h, eq, field, indicator, dt, float(coef), lap)

    def volcons_multiplier(self, v: int) -> float:
        return float(self._L.or_volcons_multiplier(self._h, v))

    def add_hessian(self, eq: int, K, coef: float = 1.0, lap: int = 0) -> None:
        """RegisterImplicitTerm with a TensorialHessian (pf/tensorialHessian.go)."""
        k = np.ascontiguousarray(K, dtype=np.float64).reshape(-1)
        if self._L.or_add_hessian(self._h, eq, _dp(k), k.size, coef, lap) != 0:
            raise ValueError("bad hessian")

    def add_viscosity(self, eq: int, eps: float, threshold: float, power: int, coef: float = 1.0,
                      lap: int = 0) -> None:
        """RegisterImplicitTerm with a SpectralViscosity (pf/spectralViscosity.go)."""
        if self._L.or_add_viscosity(self._h, eq, eps, threshold, power, coef, lap) != 0:
            raise ValueError("bad viscosity term")

    def add_source(self, eq: int, pos, amps) -> int:
        """Model.AddSource(eq, NewSource(pos, f)) (pf/model.go:152-154, pf/sourceTerm.go) with
        f(step dt) = amps[step]."""
        p = np.zeros(3)
        p[: len(pos)] = pos
        a = np.ascontiguousarray(amps, dtype=np.float64)
        k = self._L.or_add_source(self._h, eq, _dp(p), _dp(a), a.size)
        if k < 0:
            raise ValueError("bad source")
        return k

    def set_filter(self, table) -> None:
        """Euler.SetFilter / RK4.SetFilter with a tabulated filter (None removes it)."""
        if table is None:
            self._L.or_set_filter(self._h, None, 0)
            return
        t = np.ascontiguousarray(table, dtype=np.float64)
        self._keep_filter = t
        if self._L.or_set_filter(self._h, _dp(t), t.size) != 0:
            raise ValueError("bad filter table")

    # --- stepping ---
    def step_euler(self, dt: float, nsteps: int, hooks: bool = True) -> None:
        self._L.or_step_euler(self._h, dt, nsteps, int(hooks))

    def step_rk4(self, dt: float, nsteps: int, hooks: bool = True, advance: bool = True) -> None:
        self._L.or_step_rk4(self._h, dt, nsteps, int(hooks), int(advance))

    def eval_rhs(self, eq: int = 0) -> np.ndarray:
        out = np.zeros(self.N, dtype=np.complex128)
        self._L.or_eval_rhs(self._h, eq, _dp(out.view(np.float64)))
        return out

    def eval_denum(self, eq: int = 0) -> np.ndarray:
        out = np.zeros(self.N, dtype=np.complex128)
        self._L.or_eval_denum(self._h, eq, _dp(out.view(np.float64)))
        return out

    @property
    def current_step(self) -> int:
        return int(self._L.or_current_step(self._h))


def cahn_hilliard(dims, gamma: float, M: float = 1.0, splitting: str = "plain") -> Model:
    """Single-field Cahn-Hilliard dc/dt = M lap(c^3 - c - gamma lap c).

    splitting="plain" is the term list pf.Build makes from the string of
    examples/cahnHilliard/main.go:33 with M folded in,
        "dconc/dt = M*LAP conc^3 + mM*LAP conc + mM*gamma*LAP^2 conc"  (mM = -M):
      explicit:  M * (-k^2) * FFT(c^3)
      implicit:  -M * (-k^2) + (-M*gamma) * (-k^2)^2
    splitting="explicit_linear" treats -c explicitly,
        "dconc/dt = M*LAP MU + mM*gamma*LAP^2 conc"  with MU = c^3 - c.
    """
    m = Model(dims, 1)
    if splitting == "plain":
        d = m.add_product([0], [3])
        m.add_term(0, M, lap=1, src_kind=SRC_DERIVED, src=d)
        m.add_term(0, -M, lap=1, implicit=True)
        m.add_term(0, -M * gamma, lap=2, implicit=True)
    elif splitting == "explicit_linear":
        d = m.add_poly(0, [1.0, -1.0], [3, 1])
        m.add_term(0, M, lap=1, src_kind=SRC_DERIVED, src=d)
        m.add_term(0, -M * gamma, lap=2, implicit=True)
    else:
        raise ValueError(splitting)
    return m


def _cdp(a):
    return a.view(np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def householder(data, orient, sigma: float, num_nodes: int) -> np.ndarray:
    """SDD.householder (pf/sdd.go:303-318) on copies of two complex vectors."""
    d = np.array(data, dtype=np.complex128)
    o = np.ascontiguousarray(orient, dtype=np.complex128)
    lib().or_householder(_cdp(d), _cdp(o), float(sigma), d.size, int(num_nodes))
    return d


def dsm_dot(inv_diag, u, v, vec) -> np.ndarray:
    """diagonalShermannMorrison.dot (pf/sdd.go:456-470)."""
    arrs = [np.ascontiguousarray(a, dtype=np.complex128) for a in (inv_diag, u, v)]
    x = np.array(vec, dtype=np.complex128)
    lib().or_dsm_dot(_cdp(arrs[0]), _cdp(arrs[1]), _cdp(arrs[2]), x.size, _cdp(x))
    return x


def sdd_denum_dot(denum, orient, sigma: float, dt: float, vec) -> np.ndarray:
    """SDD.householderDenum(denum, orient, sigma).dot(vec) (pf/sdd.go:320-339)."""
    d = np.ascontiguousarray(denum, dtype=np.complex128)
    o = np.ascontiguousarray(orient, dtype=np.complex128)
    x = np.array(vec, dtype=np.complex128)
    lib().or_sdd_denum_dot(_cdp(d), _cdp(o), float(sigma), float(dt), x.size, _cdp(x))
    return x


class SDD:
    """Shrinking-dimer dynamics stepper (pf/sdd.go) over an oracle Model."""

    def __init__(self, model: Model):
        self.model = model
        self._L = lib()
        self._h = self._L.or_sdd_create(model._h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.or_sdd_destroy(h)
            self._h = None

    def set_params(self, dt: float, alpha: float = 0.5, tau_orient: float = 1.0, tau_len: float = 1.0,
                   init_len: float = 0.0, min_len: float = 0.0) -> None:
        self._L.or_sdd_set_params(self._h, alpha, dt, tau_orient, tau_len, init_len, min_len)

    def init(self, init_fields, final_fields) -> None:
        a = np.ascontiguousarray(np.real(init_fields), dtype=np.float64).reshape(-1)
        b = np.ascontiguousarray(np.real(final_fields), dtype=np.float64).reshape(-1)
        self._L.or_sdd_init(self._h, _dp(a), _dp(b))

    def set_orientation(self, v) -> None:
        a = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
        self._L.or_sdd_set_orientation(self._h, _dp(a))

    def dimer_length(self, t: float) -> float:
        return float(self._L.or_sdd_dimer_length(self._h, t))

    @property
    def init_length(self) -> float:
        return float(self._L.or_sdd_init_length(self._h))

    def step(self, nsteps: int) -> None:
        if self._L.or_sdd_step(self._h, nsteps) != 0:
            raise ValueError("SDD: time step not set")

    def orientation(self) -> np.ndarray:
        p = self._L.or_sdd_orientation(self._h)
        return np.ctypeslib.as_array(p, shape=(self.model.N * self.model.nfields,)).copy()

    def monitor(self) -> dict:
        p = self._L.or_sdd_monitor(self._h)
        v = np.ctypeslib.as_array(p, shape=(5,)).copy()
        return dict(zip(("max_force", "force_power_spectrum", "max_torque", "field_norm", "field_norm_change"), v))
