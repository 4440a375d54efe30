"""gopf_reduce_noalloc: the field reduction for callers that cannot allocate device memory.

Such callers (a host that manages all device memory itself, an allocator
budget enforced outside CUDA) pass a field they already hold on the device;
the entry point's only scratch is a static device array.  Its results must
equal those of gopf_reduce, the context-based reduction, on the same field,
on two calls in a row (the scratch keeps the previous call's contents).
This file is collected last so that a failure here stops a -x run after
every other test has run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_reduce_matches_context_reduce():
    import torch

    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    dims = [64, 64, 64]
    n = 64 ** 3
    c = uniform_field(12, n, 0.25, 0.5)
    m = G.Model(dims, "fp64", device=0)
    m.add_field("c")
    m.upload_real(0, c)
    expect = [m.reduce(0, w) for w in (G.RED_SUM, G.RED_SUMSQ, G.RED_MIN, G.RED_MAX, G.RED_NONFINITE)]
    d = torch.from_numpy(c).to("cuda")
    torch.cuda.synchronize()
    L = G.load()
    for call in range(2):
        out = (ctypes.c_double * 5)()
        rc = L.gopf_reduce_noalloc(ctypes.c_void_p(d.data_ptr()), n, out, None)
        assert rc == 0, L.gopf_noalloc_last_error().decode()
        got = list(out)
        assert abs(got[0] - expect[0]) <= 1e-12 * abs(expect[0])
        assert abs(got[1] - expect[1]) <= 1e-12 * abs(expect[1])
        assert abs(got[2] - expect[2]) <= 1e-12 and abs(got[3] - expect[3]) <= 1e-12
        assert got[4] == expect[4] == 0.0
    # a different, smaller field on the same scratch
    c2 = c[: n // 3] * -2.0
    d2 = torch.from_numpy(c2).to("cuda")
    out = (ctypes.c_double * 5)()
    assert L.gopf_reduce_noalloc(ctypes.c_void_p(d2.data_ptr()), c2.size, out, None) == 0
    assert abs(out[0] - c2.sum()) <= 1e-10 * abs(c2.sum())
    assert out[2] == c2.min() and out[3] == c2.max()


def test_noalloc_non_finite_cells():
    """A field with a NaN and a +Inf: the count is exact (2), min and max skip the NaN but see the
    Inf (IEEE fmin/fmax), and the sums are non-finite.  gopf_reduce of a context cannot be the
    yardstick here: a context holds the spectrum, where one non-finite cell spreads to every cell,
    so its count is the whole field.  The finite cells alone are then checked against gopf_reduce
    of the same field with the two cells replaced by zeros, on two calls in a row."""
    import torch

    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    n = 32 ** 3
    c = uniform_field(13, n, -0.1, 0.4)
    bad = c.copy()
    bad[5] = np.nan
    bad[n - 7] = np.inf
    L = G.load()
    d = torch.from_numpy(bad).to("cuda")
    torch.cuda.synchronize()
    for call in range(2):
        out = (ctypes.c_double * 5)()
        assert L.gopf_reduce_noalloc(ctypes.c_void_p(d.data_ptr()), n, out, None) == 0
        assert out[4] == 2.0
        assert np.isnan(out[0]) and np.isnan(out[1])  # NaN + Inf = NaN
        assert out[3] == np.inf
        assert out[2] == np.nanmin(bad)
    # the finite cells against the context reduction
    fin = bad.copy()
    fin[~np.isfinite(fin)] = 0.0
    m = G.Model([32, 32, 32], "fp64", device=0)
    m.add_field("c")
    m.upload_real(0, fin)
    expect = [m.reduce(0, w) for w in (G.RED_SUM, G.RED_SUMSQ, G.RED_MIN, G.RED_MAX, G.RED_NONFINITE)]
    df = torch.from_numpy(fin).to("cuda")
    torch.cuda.synchronize()
    for call in range(2):
        out = (ctypes.c_double * 5)()
        assert L.gopf_reduce_noalloc(ctypes.c_void_p(df.data_ptr()), n, out, None) == 0
        assert abs(out[0] - expect[0]) <= 1e-12 * max(1.0, abs(expect[0]))
        assert abs(out[1] - expect[1]) <= 1e-12 * abs(expect[1])
        assert abs(out[2] - expect[2]) <= 1e-12 and abs(out[3] - expect[3]) <= 1e-12
        assert out[4] == expect[4] == 0.0
    m.close()


def test_noalloc_rejects_oversized_field():
    import gopf_gb300 as G

    L = G.load()
    out = (ctypes.c_double * 5)()
    too_many = 16384 * 4096 + 1
    rc = L.gopf_reduce_noalloc(ctypes.c_void_p(1), too_many, out, None)
    assert rc == 1
    assert b"exceeds" in L.gopf_noalloc_last_error()
