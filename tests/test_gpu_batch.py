"""Batched stepping of independent, unevenly sized 2D instances (gopf_batch_*).

A batch replaces running one pf.Solver per swept parameter set.  Each
instance keeps its own equation coefficients and dt; the batch must give the
same fields as stepping every context on its own (bitwise, same tile code),
and each instance must match the FP64 oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def ch_ctx(side, prec, gamma, M, dt, c0, fast=True):
    import gopf_gb300 as G

    m = G.Model([side, side], prec, device=0)
    m.set_option(G._lib.OPT_FAST_KERNELS, int(fast))
    m.add_field("conc")
    m.add_scalar("gamma", gamma)
    m.add_scalar("M", M)
    m.add_scalar("mM", -M)
    m.add_equation("dconc/dt = M*LAP conc^3 + mM*LAP conc + mM*gamma*LAP^2 conc")
    m.init()
    m.set_stepper("euler", dt)
    m.upload(0, c0)
    return m


def _params(n):
    from gopf_gb300.synthetic import splitmix64_uniform

    u = splitmix64_uniform(2, 3 * n)
    sides = [16, 32, 48, 64, 96, 128, 24, 72]
    return [(sides[int(u[3 * i] * len(sides))], 0.2 + 1.8 * u[3 * i + 1], 0.5 + 1.5 * u[3 * i + 2]) for i in range(n)]


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_batch_equals_individual_steps(prec):
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    params = _params(12)
    a_models, b_models = [], []
    for i, (side, gamma, M) in enumerate(params):
        c0 = uniform_field(1000 + i, side * side, 0.5, 0.05)
        dt = 0.05 if i % 2 else 0.02
        a_models.append(ch_ctx(side, prec, gamma, M, dt, c0, fast=False))
        b_models.append(ch_ctx(side, prec, gamma, M, dt, c0, fast=False))
    batch = G.Batch(a_models)
    batch.step(37)
    for m in b_models:
        m.step(37)
    for a, b in zip(a_models, b_models):
        assert np.array_equal(a.download(0), b.download(0))
        assert a.current_step == 37


def test_batch_fp64_matches_oracle(oracle):
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    params = _params(6)
    models, refs = [], []
    for i, (side, gamma, M) in enumerate(params):
        c0 = uniform_field(1000 + i, side * side, 0.5, 0.05)
        models.append(ch_ctx(side, "fp64", gamma, M, 0.05, c0))
        o = oracle.cahn_hilliard([side, side], gamma=gamma, M=M)
        o.set_field(0, c0)
        refs.append(o)
    G.Batch(models).step(60)
    for m, o in zip(models, refs):
        o.step_euler(0.05, 60)
        ref = o.field(0).real
        assert np.linalg.norm(m.download(0).real - ref) / np.linalg.norm(ref) <= 1e-11


def test_batch_rejects_mixed_precision():
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    a = ch_ctx(16, "fp32", 1.0, 1.0, 0.05, uniform_field(1, 256, 0.5, 0.05))
    b = ch_ctx(16, "fp64", 1.0, 1.0, 0.05, uniform_field(1, 256, 0.5, 0.05))
    with pytest.raises(G.GopfError):
        G.Batch([a, b])


def test_batch_with_large_instances_runs_and_stays_finite():
    """Sides 256..1024 (the sweep sizes) in one batch, FP32; fields stay finite and mass is conserved."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    models, mass0 = [], []
    for i, side in enumerate([1024, 768, 512, 384, 256, 128]):
        c0 = uniform_field(2000 + i, side * side, 0.5, 0.05)
        m = ch_ctx(side, "fp32", 0.5 + 0.2 * i, 1.0, 0.05, c0)
        models.append(m)
        mass0.append(c0.sum())
    G.Batch(models).step(50)
    for m, m0 in zip(models, mass0):
        d = m.download(0).real
        assert np.all(np.isfinite(d))
        assert abs(d.sum() - m0) / d.size <= 1e-5


def test_batch_size_classes_equal_generic_contexts():
    """The sweep's sides go through one kernel per size class (the register line engine for FP32 sides
    256 ... 1024, compile-time Stockham plans for 128), run as parallel graph branches; they compute
    what the runtime-plan kernels of single contexts compute, to FP32 rounding."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    sides = [1024, 768, 512, 384, 256, 128, 128, 512]
    a_models, b_models = [], []
    for i, side in enumerate(sides):
        c0 = uniform_field(3000 + i, side * side, 0.5, 0.05)
        a_models.append(ch_ctx(side, "fp32", 0.4 + 0.1 * i, 1.0, 0.05, c0, fast=False))
        b_models.append(ch_ctx(side, "fp32", 0.4 + 0.1 * i, 1.0, 0.05, c0, fast=False))
    batch = G.Batch(a_models)
    assert batch.kernels_per_step() == 6 + 6 + 1
    batch.step(12)
    for m in b_models:
        m.step(12)
    for a, b in zip(a_models, b_models):
        x, y = a.download_real(0), b.download_real(0)
        assert np.max(np.abs(x - y)) <= 1e-6 * np.max(np.abs(y))


def test_sweep_draw_fp32_batch_matches_fp64_per_instance():
    """The sweep configuration's own draw (64 instances, sides from {128 ... 1024} by seed 2, gamma ~
    U(0.2, 2), M ~ U(0.5, 2), c0 = 0.5 + U(-0.05, 0.05) with seed 1000 + i, dt 0.05): the first
    instance of every side class, batched in FP32 (line engine for 256 ... 1024), against each
    instance stepped alone in FP64, 200 steps: per-instance rel-L2 <= 1e-4."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import splitmix64_uniform, uniform_field

    sides = [128, 256, 384, 512, 768, 1024]
    u = splitmix64_uniform(2, 3 * 64)
    draw = [(sides[min(int(u[3 * i] * 6), 5)], 0.2 + 1.8 * u[3 * i + 1], 0.5 + 1.5 * u[3 * i + 2]) for i in range(64)]
    first = {}
    for i, p in enumerate(draw):
        first.setdefault(p[0], i)
    assert sorted(first) == sides  # the draw holds every class
    pick = [first[s] for s in sides]
    a, b = [], []
    for i in pick:
        side, gamma, M = draw[i]
        c0 = uniform_field(1000 + i, side * side, 0.5, 0.05)
        a.append(ch_ctx(side, "fp32", gamma, M, 0.05, c0))
        b.append(ch_ctx(side, "fp64", gamma, M, 0.05, c0))
    G.Batch(a).step(200)
    for m in b:
        m.step(200)
    for i, x, y in zip(pick, a, b):
        ref = y.download_real(0)
        err = np.linalg.norm(x.download_real(0) - ref) / np.linalg.norm(ref)
        assert err <= 1e-4, (i, draw[i], err)
