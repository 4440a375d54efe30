"""Field files in the reference's Float64IO format (pf/fileIO.go:45-97): raw big-endian float64."""
import numpy as np
import pytest


def test_load_rejects_wrong_size(tmp_path):
    import gopf_gb300 as G

    m = G.Model([16, 16], "fp64", device=-1)  # host-only context: the size check runs before any upload
    m.add_field("conc")
    p = tmp_path / "short.bin"
    np.arange(100, dtype=">f8").tofile(p)
    with pytest.raises(G.GopfError) as e:
        m.load_float64(str(p))
    assert e.value.status == 1


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("asynchronous", [False, True])
def test_save_and_load_float64(tmp_path, prec, asynchronous):
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    dims = [32, 32, 32]
    n = 32 ** 3
    m = G.Model(dims, prec, device=0)
    m.add_field("conc")
    m.add_scalar("gamma", 0.5)
    m.add_scalar("m1", -1.0)
    m.add_equation("dconc/dt = LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc")
    m.init()
    m.set_stepper("euler", 0.05)
    m.upload(0, uniform_field(2, n, 0.0, 0.1))
    m.step(10)
    p1 = tmp_path / "f_conc_1.bin"
    m.save_float64(str(p1), asynchronous=asynchronous)
    m.step(5)  # keeps stepping while the file is written
    p2 = tmp_path / "f_conc_2.bin"
    ref2 = m.download_real(0)
    m.save_float64(str(p2), asynchronous=asynchronous)
    m.io_wait()
    a = np.fromfile(p2, dtype=">f8")
    assert a.size == n and np.array_equal(a, ref2)
    assert np.fromfile(p1, dtype=">f8").size == n
    # restart from the file
    m2 = G.Model(dims, prec, device=0)
    m2.add_field("conc")
    m2.add_scalar("gamma", 0.5)
    m2.add_scalar("m1", -1.0)
    m2.add_equation("dconc/dt = LAP conc^3 + m1*LAP conc + m1*gamma*LAP^2 conc")
    m2.init()
    m2.set_stepper("euler", 0.05)
    m2.load_float64(str(p2))
    tol = 1e-6 if prec == "fp32" else 1e-13
    assert np.max(np.abs(m2.download_real(0) - ref2)) < tol
