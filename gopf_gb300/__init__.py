"""gopf_gb300 -- GB300-native spectral time stepping for gopf models.

The product is libgopf_gpu.so (CUDA kernels for sm_103a behind the C ABI of
include/gopf_gpu.h).  This package is the Python front end used by the tests,
the benchmark and the adjoint harness: `Model` mirrors how a Go program
drives pf.Model + pf.Solver (pf/model.go, pf/solver.go), one call per C-ABI
entry point.  There is no CPU fallback: every compute call goes to the
device library and raises GopfError when it fails.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import (  # noqa: F401
    DER_INDICATOR,
    DER_MPOLY,
    DER_INDICATOR_D,
    DER_INDICATOR_HD,
    DER_POLY,
    DER_PRODUCT,
    GOPF_FP32,
    GOPF_FP64,
    RED_MAX,
    RED_MIN,
    RED_NONFINITE,
    RED_SUM,
    RED_SUMSQ,
    SRC_DERIVED,
    SRC_FIELD,
    SRC_NONE,
    GopfDerived,
    GopfTerm,
)

__all__ = ["Model", "Batch", "GopfError", "load", "build"]

_STEPPERS = {"euler": _lib.GOPF_STEPPER_EULER, "rk4": _lib.GOPF_STEPPER_RK4,
             "implicit_euler": _lib.GOPF_STEPPER_IMPLICIT_EULER, "sdd": _lib.GOPF_STEPPER_SDD}


class GopfError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_lib.STATUS.get(status, status)}: {message}")
        self.status = status
        self.message = message


def vandeven(order: int) -> np.ndarray:
    """NewVandeven(order).Data (pf/vandeven.go:13-27), computed by the library."""
    out = np.empty(1000)
    rc = load().gopf_vandeven_table(int(order), _dptr(out), 1000)
    if rc != 0:
        raise GopfError(rc, "bad Vandeven order")
    return out


def load():
    return _lib.load()


def build(force: bool = False) -> str:
    import importlib

    return importlib.import_module(__name__ + ".build").build(force=force)


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Model:
    """A device-resident gopf model: fields, equations, stepper.

    Mirrors pf.NewModel / AddField / AddScalar / RegisterFunction /
    AddEquation / NewSolver / Solve on top of the C ABI.
    """

    def __init__(self, domain_size, precision: str = "fp32", device: int = 0):
        self._L = _lib.load()
        self.domain_size = [int(d) for d in domain_size]
        self.N = int(np.prod(self.domain_size))
        prec = {"fp32": _lib.GOPF_FP32, "fp64": _lib.GOPF_FP64}[precision]
        self.precision = precision
        h = ctypes.c_void_p()
        dims = (ctypes.c_int * len(self.domain_size))(*self.domain_size)
        rc = self._L.gopf_ctx_create(len(self.domain_size), dims, prec, device, ctypes.byref(h))
        self._h = h
        if rc != 0:
            msg = self._L.gopf_last_error(h).decode() if h.value else _lib.STATUS.get(rc, "")
            self.close()
            raise GopfError(rc, msg)
        self.field_names: list[str] = []

    # ---- plumbing ----
    def _ck(self, rc: int) -> None:
        if rc != 0:
            raise GopfError(rc, self._L.gopf_last_error(self._h).decode())

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.gopf_ctx_destroy(h)
        self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_handle: int | None) -> None:
        self._ck(self._L.gopf_set_stream(self._h, ctypes.c_void_p(stream_handle or 0)))

    def set_option(self, option: int, value: int) -> None:
        self._ck(self._L.gopf_set_option(self._h, option, value))

    # ---- pf.Model mirror ----
    def add_field(self, name: str) -> int:
        fid = ctypes.c_int()
        self._ck(self._L.gopf_add_field(self._h, name.encode(), ctypes.byref(fid)))
        self.field_names.append(name)
        return fid.value

    def add_scalar(self, name: str, value) -> None:
        v = complex(value)
        self._ck(self._L.gopf_add_scalar(self._h, name.encode(), v.real, v.imag))

    def register_function(self, name: str, kind: int, field: str, coefs=None, powers=None) -> None:
        n = 0 if coefs is None else len(coefs)
        c = (ctypes.c_double * max(n, 1))(*(coefs or [0.0]))
        p = (ctypes.c_int * max(n, 1))(*(powers or [0]))
        self._ck(self._L.gopf_register_function(self._h, name.encode(), kind, field.encode(), c, p, n))

    def register_polynomial(self, name: str, coefs, powers) -> None:
        """RegisterFunction for a polynomial of several fields: sum_t coefs[t] * prod_f field_f^powers[t][f]
        (f in AddField order; powers has one row per term and one column per field it covers)."""
        p = np.ascontiguousarray(powers, dtype=np.int32)
        if p.ndim != 2 or p.shape[0] != len(coefs):
            raise ValueError("powers needs one row per coefficient")
        c = np.ascontiguousarray(coefs, dtype=np.float64)
        self._ck(self._L.gopf_register_polynomial(self._h, name.encode(), _dptr(c),
                                                  p.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), p.shape[0],
                                                  p.shape[1]))

    def register_elastic(self, name: str, field: str, C, misfit) -> None:
        c = np.ascontiguousarray(C, dtype=np.float64).reshape(81)
        m = np.ascontiguousarray(misfit, dtype=np.float64).reshape(9)
        self._ck(self._L.gopf_register_elastic(self._h, name.encode(), field.encode(), _dptr(c), _dptr(m)))

    def register_hessian(self, name: str, K) -> None:
        """RegisterImplicitTerm(name, &TensorialHessian{K: K}, nil)."""
        k = np.ascontiguousarray(K, dtype=np.float64).reshape(-1)
        self._ck(self._L.gopf_register_hessian(self._h, name.encode(), _dptr(k), k.size))

    def register_spectral_viscosity(self, name: str, eps: float, threshold: float, power: int) -> None:
        """RegisterImplicitTerm(name, &SpectralViscosity{eps, threshold, power}, nil)."""
        self._ck(self._L.gopf_register_spectral_viscosity(self._h, name.encode(), eps, threshold, int(power)))

    def register_volcons(self, name: str, field: str, indicator: str, dt: float) -> None:
        self._ck(self._L.gopf_register_volcons(self._h, name.encode(), field.encode(), indicator.encode(), dt))

    def register_noise(self, name: str, kind: str, field: str, strength: float, seed: int = 0) -> None:
        """WhiteNoise as a function ("white") or ConservativeNoise as a term ("conservative")."""
        k = {"white": _lib.NOISE_WHITE, "conservative": _lib.NOISE_CONSERVATIVE}[kind]
        self._ck(self._L.gopf_register_noise(self._h, name.encode(), k, field.encode(), float(strength), int(seed)))

    def add_equation(self, eq: str) -> None:
        self._ck(self._L.gopf_add_equation(self._h, eq.encode()))

    def init(self) -> None:
        self._ck(self._L.gopf_init(self._h))

    def summary(self, eq: int = 0):
        ne, ni = ctypes.c_int(), ctypes.c_int()
        self._ck(self._L.gopf_equation_summary(self._h, eq, ctypes.byref(ne), ctypes.byref(ni)))
        return ne.value, ni.value

    def terms(self):
        n = ctypes.c_int()
        self._ck(self._L.gopf_get_terms(self._h, None, 0, ctypes.byref(n)))
        arr = (GopfTerm * max(n.value, 1))()
        self._ck(self._L.gopf_get_terms(self._h, arr, n.value, ctypes.byref(n)))
        return [dict(eq=t.eq, implicit=t.implicit, coef=t.coef, lap=t.lap, source=t.source, src_index=t.src_index)
                for t in arr[: n.value]]

    def derived(self):
        n = ctypes.c_int()
        self._ck(self._L.gopf_get_derived(self._h, None, 0, ctypes.byref(n)))
        arr = (GopfDerived * max(n.value, 1))()
        self._ck(self._L.gopf_get_derived(self._h, arr, n.value, ctypes.byref(n)))
        return [dict(kind=d.kind, field=list(d.field[: d.nfac]), power=list(d.power[: d.nfac]),
                     coef=list(d.coef[: d.nfac])) for d in arr[: n.value]]

    def set_terms(self, nfields: int, derived, terms) -> None:
        """Install a pre-compiled term table (dicts with the GopfDerived/GopfTerm fields)."""
        D = (GopfDerived * max(len(derived), 1))()
        for i, d in enumerate(derived):
            D[i].kind = d["kind"]
            D[i].nfac = len(d["field"])
            for j, f in enumerate(d["field"]):
                D[i].field[j] = f
                D[i].power[j] = d.get("power", [1] * len(d["field"]))[j]
                D[i].coef[j] = d.get("coef", [1.0] * len(d["field"]))[j]
        T = (GopfTerm * max(len(terms), 1))()
        for i, t in enumerate(terms):
            T[i].eq = t.get("eq", 0)
            T[i].implicit = int(t.get("implicit", 0))
            T[i].coef = t["coef"]
            T[i].lap = t.get("lap", 0)
            T[i].source = t.get("source", SRC_NONE)
            T[i].src_index = t.get("src_index", 0)
        self._ck(self._L.gopf_set_terms(self._h, nfields, D, len(derived), T, len(terms)))

    # ---- pf.TimeStepper mirror ----
    def set_stepper(self, name: str, dt: float) -> None:
        self._ck(self._L.gopf_set_stepper(self._h, _STEPPERS[name], dt))

    def save_float64(self, path: str, field: int = 0, asynchronous: bool = False) -> None:
        """Float64IO/SaveFloat64: raw big-endian float64 file of the real field (pf/fileIO.go)."""
        self._ck(self._L.gopf_save_float64(self._h, field, path.encode(), int(asynchronous)))

    def io_wait(self) -> None:
        self._ck(self._L.gopf_io_wait(self._h))

    def load_float64(self, path: str, field: int = 0) -> None:
        """LoadFloat64 + upload (restart from a saved field)."""
        self._ck(self._L.gopf_load_float64(self._h, field, path.encode()))

    def set_modal_filter(self, table) -> None:
        """Euler/RK4 SetFilter with a tabulated filter on [0, 1] (None removes it)."""
        if table is None:
            self._ck(self._L.gopf_set_modal_filter(self._h, None, 0))
            return
        t = np.ascontiguousarray(table, dtype=np.float64)
        self._ck(self._L.gopf_set_modal_filter(self._h, _dptr(t), t.size))

    def set_newton_krylov(self, maxiter: int = 50, step_size: float = 1e-3, tol: float = 1e-7, stencil: int = 6,
                          restart: int = 50) -> None:
        """ImplicitEuler's solver controls (pf/implicitEuler.go:221-228 defaults)."""
        self._ck(self._L.gopf_set_newton_krylov(self._h, maxiter, step_size, tol, stencil, restart))

    def kernel_launches(self, nsteps: int) -> int:
        """Kernel launches gopf_step(nsteps) makes through the captured graphs."""
        c = ctypes.c_longlong()
        self._ck(self._L.gopf_kernel_launches(self._h, int(nsteps), ctypes.byref(c)))
        return int(c.value)

    def newton_stats(self):
        """(Newton iterations, GMRES iterations, max|F|, converged) of the last ImplicitEuler step."""
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        r = ctypes.c_double()
        self._ck(self._L.gopf_newton_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(r), ctypes.byref(c)))
        return a.value, b.value, r.value, bool(c.value)

    def upload(self, field: int, data) -> None:
        a = np.ascontiguousarray(np.asarray(data).reshape(-1).astype(np.complex128))
        self._ck(self._L.gopf_field_upload(self._h, field, _dptr(a.view(np.float64)), a.size))

    def upload_real(self, field: int, data) -> None:
        a = np.ascontiguousarray(np.asarray(data, dtype=np.float64).reshape(-1))
        self._ck(self._L.gopf_field_upload_real(self._h, field, _dptr(a), a.size))

    def download(self, field: int = 0) -> np.ndarray:
        out = np.empty(self.N, dtype=np.complex128)
        self._ck(self._L.gopf_field_download(self._h, field, _dptr(out.view(np.float64)), self.N))
        return out

    def download_real(self, field: int = 0) -> np.ndarray:
        out = np.empty(self.N, dtype=np.float64)
        self._ck(self._L.gopf_field_download_real(self._h, field, _dptr(out), self.N))
        return out

    def step(self, nsteps: int) -> None:
        self._ck(self._L.gopf_step(self._h, int(nsteps)))

    def prepare_graphs(self, nsteps: int) -> None:
        """Capture the graphs that step(nsteps) replays, without stepping."""
        self._ck(self._L.gopf_prepare_graphs(self._h, int(nsteps)))

    def synchronize(self) -> None:
        self._ck(self._L.gopf_synchronize(self._h))

    @property
    def time(self) -> float:
        t = ctypes.c_double()
        self._ck(self._L.gopf_get_time(self._h, ctypes.byref(t)))
        return t.value

    @property
    def current_step(self) -> int:
        s = ctypes.c_longlong()
        self._ck(self._L.gopf_get_step(self._h, ctypes.byref(s)))
        return s.value

    # --- point sources (Model.AddSource, pf/sourceTerm.go) ---
    def add_source(self, eq: int, pos) -> int:
        p = np.ascontiguousarray(pos, dtype=np.float64)
        sid = ctypes.c_int()
        self._ck(self._L.gopf_add_source(self._h, eq, _dptr(p), int(p.size), ctypes.byref(sid)))
        return sid.value

    def set_source_amplitudes(self, amps) -> None:
        """amps[s, i] = f_s(t) at the i-th step from the current one, one row per source."""
        a = np.ascontiguousarray(np.atleast_2d(amps), dtype=np.float64)
        self._ck(self._L.gopf_set_source_amplitudes(self._h, _dptr(a), a.shape[0], a.shape[1]))

    # --- shrinking-dimer dynamics (pf/sdd.go); step with set_stepper("sdd", dt) ---
    def sdd_init(self, init, final) -> None:
        """SDD.Init: the orientation is final - init (all fields, field after field)."""
        a = np.ascontiguousarray(np.real(init), dtype=np.float64).reshape(-1)
        b = np.ascontiguousarray(np.real(final), dtype=np.float64).reshape(-1)
        if a.size != b.size:
            raise ValueError("init and final differ in size")
        self._ck(self._L.gopf_sdd_init(self._h, _dptr(a), _dptr(b), a.size))

    def sdd_set_orientation(self, v) -> None:
        """SDD.SetInitialOrientation."""
        a = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
        self._ck(self._L.gopf_sdd_set_orientation(self._h, _dptr(a), a.size))

    def sdd_set_params(self, alpha: float = 0.5, tau_orientation: float = 1.0, tau_length: float = 1.0,
                       init_length: float = 0.0, min_length: float = 0.0) -> None:
        self._ck(self._L.gopf_sdd_set_params(self._h, alpha, tau_orientation, tau_length, init_length, min_length))

    def sdd_orientation(self) -> np.ndarray:
        out = np.empty(self.N * max(1, len(self.field_names)))
        self._ck(self._L.gopf_sdd_get_orientation(self._h, _dptr(out), out.size))
        return out

    def sdd_monitor(self) -> dict:
        out = np.empty(5)
        self._ck(self._L.gopf_sdd_monitor(self._h, _dptr(out)))
        return dict(zip(("max_force", "force_power_spectrum", "max_torque", "field_norm", "field_norm_change"), out))

    def sdd_dimer_length(self, t: float) -> float:
        out = ctypes.c_double()
        self._ck(self._L.gopf_sdd_dimer_length(self._h, t, ctypes.byref(out)))
        return out.value

    def point_values(self, field: int, sites) -> np.ndarray:
        """PointMonitor.Add (pf/monitor.go:27-30) for several sites: the real field there."""
        idx = np.ascontiguousarray(sites, dtype=np.int64)
        out = np.empty(idx.size)
        self._ck(self._L.gopf_point_values(self._h, field, idx.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                                           int(idx.size), _dptr(out)))
        return out

    def reduce(self, field: int, what: int) -> float:
        out = ctypes.c_double()
        self._ck(self._L.gopf_reduce(self._h, field, what, ctypes.byref(out)))
        return out.value

    def free_energy(self, field: int = 0, coefs=(0.0, 0.0, -0.5, 0.0, 0.25), kappa: float = 1.0):
        """(bulk, gradient, total) of sum_cells sum_p coefs[p] c^p + (kappa/2) sum_cells |grad c|^2 on the
        device; the defaults with kappa = gamma are the Cahn-Hilliard free energy."""
        c = np.ascontiguousarray(coefs, dtype=np.float64)
        out = np.empty(3)
        self._ck(self._L.gopf_free_energy(self._h, field, _dptr(c), int(c.size), float(kappa), _dptr(out)))
        return float(out[0]), float(out[1]), float(out[2])

    def elastic_energy(self, C, misfit, field: int = 0, indicator: bool = False) -> float:
        """HomogeneousModulusEnergy (elasticity/linearElasticity.go:101-165) of the field, or of its
        Indicator 3c^2 - 2c^3, on the device."""
        c = np.ascontiguousarray(C, dtype=np.float64).reshape(81)
        m = np.ascontiguousarray(misfit, dtype=np.float64).reshape(9)
        out = ctypes.c_double()
        self._ck(self._L.gopf_elastic_energy(self._h, field, int(indicator), _dptr(c), _dptr(m), ctypes.byref(out)))
        return out.value

    def volcons_multiplier(self) -> float:
        """VolumeConservingLP.Multiplier after the steps taken so far."""
        out = ctypes.c_double()
        self._ck(self._L.gopf_volcons_multiplier(self._h, ctypes.byref(out)))
        return out.value

    def mass(self, field: int = 0) -> float:
        return self.reduce(field, RED_SUM)

    # ---- pfutil.FourierTransform mirror ----
    def fft(self, data, sign: int = -1) -> np.ndarray:
        a = np.ascontiguousarray(np.asarray(data, dtype=np.complex128).reshape(-1)).copy()
        self._ck(self._L.gopf_fft(self._h, sign, _dptr(a.view(np.float64)), a.size))
        return a

    def freq(self, i: int) -> np.ndarray:
        out = (ctypes.c_double * 3)()
        self._ck(self._L.gopf_freq(self._h, i, out))
        return np.array(out[: len(self.domain_size)])

    def conjugate_node(self, i: int) -> int:
        return int(self._L.gopf_conjugate_node(self._h, i))

    @property
    def device_bytes(self) -> int:
        b = ctypes.c_size_t()
        self._ck(self._L.gopf_device_bytes(self._h, ctypes.byref(b)))
        return b.value

    def profile_step(self, nsteps: int):
        """Per-kernel average device time (ms) and algorithmic bytes of one Euler step."""
        ms = (ctypes.c_double * 16)()
        by = (ctypes.c_double * 16)()
        n = ctypes.c_int()
        self._ck(self._L.gopf_profile_step(self._h, int(nsteps), ms, by, 16, ctypes.byref(n)))
        out = []
        buf = ctypes.create_string_buffer(64)
        for k in range(n.value):
            self._ck(self._L.gopf_profile_slot_name(self._h, k, buf, 64))
            out.append(dict(name=buf.value.decode(), ms=ms[k], bytes=by[k]))
        return out

    @property
    def kernels_per_step(self) -> int:
        n = ctypes.c_int()
        self._ck(self._L.gopf_kernels_per_step(self._h, ctypes.byref(n)))
        return n.value


class Batch:
    """Several 2D Models stepped together by shared launches (gopf_batch_*)."""

    def __init__(self, models):
        self._L = _lib.load()
        self.models = list(models)
        arr = (ctypes.c_void_p * len(self.models))(*[m.handle.value for m in self.models])
        h = ctypes.c_void_p()
        rc = self._L.gopf_batch_create(arr, len(self.models), ctypes.byref(h))
        self._h = h
        if rc != 0:
            msg = self._L.gopf_batch_last_error(h).decode() if h.value else ""
            self.close()
            raise GopfError(rc, msg)

    def _ck(self, rc: int) -> None:
        if rc != 0:
            raise GopfError(rc, self._L.gopf_batch_last_error(self._h).decode())

    def step(self, nsteps: int) -> None:
        self._ck(self._L.gopf_batch_step(self._h, int(nsteps)))

    def kernels_per_step(self) -> int:
        n = ctypes.c_int()
        self._ck(self._L.gopf_batch_kernels_per_step(self._h, ctypes.byref(n)))
        return n.value

    def set_stream(self, stream_handle: int | None) -> None:
        self._ck(self._L.gopf_batch_set_stream(self._h, ctypes.c_void_p(stream_handle or 0)))

    def tune(self, reps: int = 5) -> None:
        """Time the candidate kernels of every kind of instance and keep the fastest (cached)."""
        self._ck(self._L.gopf_batch_tune(self._h, int(reps)))

    def force(self, xfam: int = -1, yfam: int = -1, lbx: int = 0, lby: int = 0, xplan: int = 0,
              yplan: int = 0) -> None:
        """One kernel choice for every instance (families BATCH_LINE, BATCH_STOCKHAM_CT, BATCH_STOCKHAM)."""
        self._ck(self._L.gopf_batch_force(self._h, xfam, yfam, lbx, lby, xplan, yplan))

    def choice(self, inst: int) -> dict:
        out = (ctypes.c_int * 6)()
        self._ck(self._L.gopf_batch_choice(self._h, int(inst), out))
        return dict(zip(("xfam", "yfam", "lbx", "lby", "xplan", "yplan"), list(out)))

    def set_mode(self, mode: int) -> None:
        """BATCH_MODE_PERSISTENT (one persistent kernel per captured graph), BATCH_MODE_CHAINS (a launch
        per class and pass) or BATCH_MODE_AUTO (persistent when every instance allows it)."""
        self._ck(self._L.gopf_batch_set_mode(self._h, int(mode)))

    def mode(self) -> int:
        """The mode in effect: BATCH_MODE_PERSISTENT or BATCH_MODE_CHAINS."""
        m = ctypes.c_int()
        self._ck(self._L.gopf_batch_mode(self._h, ctypes.byref(m)))
        return m.value

    def set_wait_limit_ns(self, ns: int) -> None:
        """Limit of the persistent kernel's dependency waits (0: the built-in 2 s)."""
        self._ck(self._L.gopf_batch_set_wait_limit(self._h, int(ns)))

    def launches(self, nsteps: int) -> int:
        """Kernel launches gopf_batch_step(nsteps) makes: one per captured graph replay (16-step
        graphs, then 1-step graphs) in the persistent mode, kernels_per_step() per step otherwise."""
        if self.mode() == _lib.BATCH_MODE_PERSISTENT:
            return nsteps // 16 + nsteps % 16
        return self.kernels_per_step() * nsteps

    @staticmethod
    def tune_reset() -> None:
        _lib.load().gopf_batch_tune_reset()

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.gopf_batch_destroy(h)
        self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
