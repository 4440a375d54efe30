"""GPU parity of the device FFT passes (pfutil.FourierTransform semantics) through the C ABI."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _model(dims, prec):
    import gopf_gb300 as G

    return G.Model(dims, prec, device=0)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 2e-6)])
@pytest.mark.parametrize("dims", [[8, 8], [8, 16], [12, 6], [128, 128], [96, 384], [384, 384], [1024, 1024],
                                  [8, 8, 8], [12, 12, 12], [32, 32, 32], [64, 64, 64]])
def test_fft_forward_backward_matches_numpy(dims, prec, tol):
    rng = np.random.default_rng(3)
    n = int(np.prod(dims))
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    m = _model(dims, prec)
    shape = tuple(dims) if len(dims) == 2 else (dims[2], dims[0], dims[1])
    ref = np.fft.fftn(x.reshape(shape)).ravel()
    y = m.fft(x, -1)
    assert np.abs(y - ref).max() <= tol * np.abs(ref).max()
    back = m.fft(y, +1) / n
    assert np.abs(back - x).max() <= tol * 10 * np.abs(x).max()


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-14), ("fp32", 1e-6)])
@pytest.mark.parametrize("dims", [[8, 8], [128, 128], [256, 256], [768, 768], [16, 16, 16], [256, 256, 256]])
def test_upload_download_round_trip(dims, prec, tol):
    """Upload c, keep c-hat resident, download c = IFFT(FFT(c))/N (pf/euler.go:42-45 normalisation)."""
    from gopf_gb300.synthetic import uniform_field

    n = int(np.prod(dims))
    c = uniform_field(11, n, 0.0, 1.0)
    m = _model(dims, prec)
    m.add_field("c")
    m.upload(0, c)
    d = m.download(0)
    assert np.abs(d.real - c).max() <= tol * 4
    assert np.all(d.imag == 0.0)
    assert abs(m.mass(0) - c.sum()) <= 1e-6 * n * (1 if prec == "fp32" else 1e-6)


def test_freq_matches_oracle(oracle):
    m = _model([8, 8, 8], "fp32")
    for i in range(512):
        assert np.allclose(m.freq(i), oracle.freq([8, 8, 8], i))
        assert m.conjugate_node(i) == oracle.conjugate_node([8, 8, 8], i)
