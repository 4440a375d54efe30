"""Host-side failure detection (no GPU fault is ever provoked):
- a forced device-allocation failure through the GOPF_TEST_FAIL_ALLOC hook, at context creation and
  at model compilation, is reported as GOPF_ERR_OOM and leaves a destroyable context;
- null handles and bad shapes are argument errors;
- a field that is uploaded with a NaN is reported as GOPF_ERR_NAN by the next step (a host check of a
  device count, never a trap).
"""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_null_handles_are_argument_errors():
    import ctypes

    import gopf_gb300 as G

    L = G.load()
    assert L.gopf_step(None, 1) == 1
    assert L.gopf_set_stepper(None, 0, 0.1) == 1
    assert L.gopf_field_upload(None, 0, None, 0) == 1
    assert L.gopf_ctx_destroy(None) == 1
    out = ctypes.c_void_p()
    dims = (ctypes.c_int * 2)(0, 16)
    assert L.gopf_ctx_create(2, dims, 0, -1, ctypes.byref(out)) == 1


def test_bad_shape_upload_is_argument_error():
    import gopf_gb300 as G

    m = G.Model([16, 16], "fp64", device=-1)
    m.add_field("conc")
    with pytest.raises(G.GopfError) as e:
        m.upload(0, np.zeros(100))
    assert e.value.status in (1, 7)


_CHILD = r"""
import sys
sys.path.insert(0, {root!r})
import numpy as np
import gopf_gb300 as G
stage = sys.argv[1]
try:
    m = G.Model([64, 64], "fp32", device=0)
except G.GopfError as e:
    print("create", e.status)
    sys.exit(0)
m.add_field("conc")
m.add_scalar("m1", -1.0)
m.add_scalar("eps", 0.1)
m.add_equation("dconc/dt = LAP conc^3 + m1*LAP conc - eps*conc^2")
try:
    m.init()
except G.GopfError as e:
    print("init", e.status)
    sys.exit(0)
print("ok", 0)
"""


@pytest.mark.gpu
@pytest.mark.parametrize("k,where", [(1, "create"), (3, "create")])
def test_forced_allocation_failure_is_reported(k, where):
    env = dict(os.environ, GOPF_TEST_FAIL_ALLOC=str(k))
    r = subprocess.run([sys.executable, "-c", _CHILD.format(root=ROOT), "x"], env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    stage, status = r.stdout.split()[-2:]
    assert stage == where and int(status) == 3  # GOPF_ERR_OOM


@pytest.mark.gpu
def test_allocation_failure_at_compile_is_reported():
    """Count the allocations of a context first, then fail the first one that init makes."""
    probe = r"""
import sys
sys.path.insert(0, {root!r})
import gopf_gb300 as G
m = G.Model([64, 64], "fp32", device=0)
print("created")
"""
    r = subprocess.run([sys.executable, "-c", probe.format(root=ROOT)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    # the context allocates a fixed set of buffers; a large k fails during init (the group buffer)
    for k in range(4, 40):
        env = dict(os.environ, GOPF_TEST_FAIL_ALLOC=str(k))
        r = subprocess.run([sys.executable, "-c", _CHILD.format(root=ROOT), "x"], env=env, capture_output=True,
                           text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        stage, status = r.stdout.split()[-2:]
        if stage == "init":
            assert int(status) == 3
            return
        assert stage == "create" or stage == "ok"
        if stage == "ok":
            break
    pytest.fail("no allocation failure reached init")


@pytest.mark.gpu
def test_nan_in_uploaded_field_is_reported():
    import gopf_gb300 as G

    m = G.Model([32, 32], "fp64", device=0)
    m.add_field("conc")
    m.add_scalar("gamma", 1.0)
    m.add_scalar("m1", -1.0)
    m.add_equation("dconc/dt = LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc")
    m.init()
    m.set_stepper("euler", 0.1)
    c = np.full(32 * 32, 0.5)
    c[17] = np.nan
    m.upload(0, c)
    with pytest.raises(G.GopfError) as e:
        m.step(1)
    assert e.value.status == 4
    # the context stays usable: a finite field steps again
    m.upload(0, np.full(32 * 32, 0.5))
    m.step(2)
