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
    256 ... 1024, compile-time Stockham plans for 128).  Each class is a chain of x pass, y pass and
    the projection of its own instances on its own graph branch (3 launches per class and step,
    no join between steps).  They compute what the runtime-plan kernels of single contexts compute,
    to FP32 rounding, after 12 steps (a 1-step graph and a 16-step graph replay both appear when
    stepping 12 then 20)."""
    import gopf_gb300 as G
    from gopf_gb300.synthetic import uniform_field

    sides = [1024, 768, 512, 384, 256, 128, 128, 512]
    a_models, b_models = [], []
    for i, side in enumerate(sides):
        c0 = uniform_field(3000 + i, side * side, 0.5, 0.05)
        a_models.append(ch_ctx(side, "fp32", 0.4 + 0.1 * i, 1.0, 0.05, c0, fast=False))
        b_models.append(ch_ctx(side, "fp32", 0.4 + 0.1 * i, 1.0, 0.05, c0, fast=False))
    batch = G.Batch(a_models)
    batch.set_mode(G._lib.BATCH_MODE_CHAINS)
    assert batch.kernels_per_step() == 3 * 6
    for n in (12, 20):
        batch.step(n)
        for m in b_models:
            m.step(n)
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


# ---------------------------------------------------------------- kernel choices and the autotuner

def _tune_models(prec, sides, seed0=4000):
    from gopf_gb300.synthetic import uniform_field

    return [ch_ctx(s, prec, 0.4 + 0.1 * i, 1.0 + 0.05 * i, 0.05, uniform_field(seed0 + i, s * s, 0.5, 0.05))
            for i, s in enumerate(sides)]


def test_every_kernel_choice_computes_the_same_fields():
    """Every candidate the autotuner may pick (line engine, compile-time Stockham, runtime Stockham
    with each tile width and plan variant) steps the same FP32 fields to rounding (rel <= 2e-6
    after 12 steps); in FP64 the tile widths agree bitwise and the plan variants to 1e-13."""
    import gopf_gb300 as G
    from gopf_gb300 import _lib as L

    sides = [1024, 768, 512, 384, 256, 128]
    ref = None
    cands = [(L.BATCH_LINE, L.BATCH_LINE, 0, 0, 0, 0), (L.BATCH_STOCKHAM_CT, L.BATCH_STOCKHAM_CT, 0, 0, 0, 0)]
    cands += [(L.BATCH_STOCKHAM, L.BATCH_STOCKHAM, lb, lb, p, p) for lb in (4, 8) for p in (0, 1, 2)]
    for cand in cands:
        ms = _tune_models("fp32", sides)
        b = G.Batch(ms)
        b.force(*cand)
        b.step(12)
        got = [m.download_real(0) for m in ms]
        if ref is None:
            ref = got
        else:
            for x, y in zip(got, ref):
                assert np.linalg.norm(x - y) <= 2e-6 * np.linalg.norm(y), cand
    sides64 = [256, 96, 100]
    base = None
    for lb in (4, 8, 16):
        for p in (0, 1, 2):
            ms = _tune_models("fp64", sides64)
            b = G.Batch(ms)
            b.force(L.BATCH_STOCKHAM, L.BATCH_STOCKHAM, lb, lb, p, p)
            b.step(12)
            got = [m.download_real(0) for m in ms]
            if base is None:
                base = {0: got}
            if p not in base:
                base[p] = got
            for x, y in zip(got, base[p]):  # same plan: the tile width changes nothing
                assert np.array_equal(x, y)
            for x, y in zip(got, base[0]):
                assert np.linalg.norm(x - y) <= 1e-13 * np.linalg.norm(y)


def test_autotuner_picks_valid_choices_and_keeps_fields():
    """gopf_batch_tune times the candidates on the batch's own instances and restores their fields;
    the tuned batch steps exactly like a batch forced to the same choices; a second batch of the same
    kinds takes the cached choices."""
    import gopf_gb300 as G
    from gopf_gb300 import _lib as L

    G.Batch.tune_reset()
    sides = [1024, 512, 384, 256, 128, 128]
    ms = _tune_models("fp32", sides)
    before = [m.download_real(0) for m in ms]
    b = G.Batch(ms)
    b.set_mode(L.BATCH_MODE_CHAINS)  # the persistent kernel's families are fixed
    b.tune(3)
    for m, x in zip(ms, before):
        assert np.array_equal(m.download_real(0), x)  # tuning left the fields alone
        assert m.current_step == 0
    choices = [b.choice(i) for i in range(len(sides))]
    for s, c in zip(sides, choices):
        assert c["xfam"] in (L.BATCH_LINE, L.BATCH_STOCKHAM_CT, L.BATCH_STOCKHAM)
        if s == 128:
            assert c["xfam"] != L.BATCH_LINE and c["yfam"] != L.BATCH_LINE  # no 128-point line engine
        if c["xfam"] == L.BATCH_STOCKHAM:
            assert c["lbx"] in (4, 8, 16) and c["lbx"] * s // 2 <= 4096
    b.step(10)
    tuned = [m.download_real(0) for m in ms]
    # the same choices forced instance by instance (one batch per kind) step identically
    from gopf_gb300.synthetic import uniform_field

    for i, s in enumerate(sides):
        m2 = ch_ctx(s, "fp32", 0.4 + 0.1 * i, 1.0 + 0.05 * i, 0.05, uniform_field(4000 + i, s * s, 0.5, 0.05))
        b2 = G.Batch([m2])
        b2.set_mode(L.BATCH_MODE_CHAINS)
        c = choices[i]
        b2.force(c["xfam"], c["yfam"], c["lbx"], c["lby"], c["xplan"], c["yplan"])
        b2.step(10)
        assert np.array_equal(m2.download_real(0), tuned[i])
    # cached: a new batch of the same kinds gets the same choices
    ms3 = _tune_models("fp32", sides)
    b3 = G.Batch(ms3)
    b3.set_mode(L.BATCH_MODE_CHAINS)
    b3.tune(3)
    assert [b3.choice(i) for i in range(len(sides))] == choices
    # the persistent mode keeps its fixed families: line engine for 256 ... 1024, compile-time
    # Stockham for 128
    ms4 = _tune_models("fp32", sides)
    b4 = G.Batch(ms4)
    assert b4.mode() == L.BATCH_MODE_PERSISTENT
    b4.tune(3)
    for s, i in zip(sides, range(len(sides))):
        fam = L.BATCH_STOCKHAM_CT if s == 128 else L.BATCH_LINE
        assert b4.choice(i)["xfam"] == fam and b4.choice(i)["yfam"] == fam


# ---------------------------------------------------------------- the persistent mode

def test_persistent_mode_equals_chains():
    """The persistent kernel (one launch per captured graph; x and y tiles of every instance from one
    queue; per-instance completion counters; the projection of the self-conjugate lines inside the y
    tiles) steps exactly what the per-class chains step: bitwise after 1, 17 and 38 steps (1-step and
    16-step graphs), sides 128 ... 1024 (256-thread tiles and the 192-thread tiles of 384 and 768)."""
    import gopf_gb300 as G
    from gopf_gb300 import _lib as L

    sides = [1024, 768, 512, 384, 256, 128, 256, 768]
    a = _tune_models("fp32", sides, seed0=5000)
    b = _tune_models("fp32", sides, seed0=5000)
    ba, bb = G.Batch(a), G.Batch(b)
    bb.set_mode(L.BATCH_MODE_CHAINS)
    assert ba.mode() == L.BATCH_MODE_PERSISTENT and bb.mode() == L.BATCH_MODE_CHAINS
    assert ba.kernels_per_step() == 1 and ba.launches(38) == 2 + 6
    for n in (1, 16, 21):
        ba.step(n)
        bb.step(n)
        for x, y in zip(a, b):
            assert np.array_equal(x.download(0), y.download(0))


def test_persistent_mode_rejects_what_it_cannot_step():
    """FP64 instances and sides outside 128 ... 1024 stay on the chains: AUTO falls back, PERSISTENT
    is refused with GOPF_ERR_UNSUPPORTED and leaves the batch stepping in its previous mode."""
    import gopf_gb300 as G
    from gopf_gb300 import _lib as L

    for prec, sides in (("fp64", [256]), ("fp32", [256, 96])):
        ms = _tune_models(prec, sides)
        b = G.Batch(ms)
        assert b.mode() == L.BATCH_MODE_CHAINS
        with pytest.raises(G.GopfError) as e:
            b.set_mode(L.BATCH_MODE_PERSISTENT)
        assert e.value.status == 6
        assert b.mode() == L.BATCH_MODE_CHAINS
        b.step(2)
        ref = _tune_models(prec, sides)
        G.Batch(ref).step(2)
        for x, y in zip(ms, ref):
            assert np.array_equal(x.download(0), y.download(0))


def test_persistent_wait_timeout_is_reported():
    """A dependency-wait limit of 1 ns makes the y tiles of a lone 256^2 instance give up waiting for
    its x tiles: gopf_batch_step reports GOPF_ERR_TIMEOUT.  With the limit restored and the field
    uploaded again the batch steps like a fresh one."""
    import gopf_gb300 as G
    from gopf_gb300 import _lib as L
    from gopf_gb300.synthetic import uniform_field

    c0 = uniform_field(77, 256 * 256, 0.5, 0.05)
    m = ch_ctx(256, "fp32", 0.5, 1.0, 0.05, c0)
    b = G.Batch([m])
    assert b.mode() == L.BATCH_MODE_PERSISTENT
    b.set_wait_limit_ns(1)
    with pytest.raises(G.GopfError) as e:
        b.step(1)
    assert e.value.status == 5
    b.set_wait_limit_ns(0)
    m.upload(0, c0)
    b.step(3)
    f = ch_ctx(256, "fp32", 0.5, 1.0, 0.05, c0)
    fb = G.Batch([f])
    fb.step(3)
    assert np.array_equal(m.download(0), f.download(0))


@pytest.mark.parametrize("side", [384, 512, 768, 1024])
def test_line_engine_block_sizes_match(side):
    """A single 2D context on the line engine takes half-size blocks where the default ones would
    leave SMs without two blocks (every side here); a one-instance batch in the chains mode takes the
    default blocks.  The per-line arithmetic is the same, so both step the same field bitwise (FP32,
    25 steps)."""
    import gopf_gb300 as G
    from gopf_gb300 import _lib as L
    from gopf_gb300.synthetic import uniform_field

    c0 = uniform_field(6000 + side, side * side, 0.5, 0.05)
    a = ch_ctx(side, "fp32", 0.6, 1.2, 0.05, c0)
    b = ch_ctx(side, "fp32", 0.6, 1.2, 0.05, c0)
    a.step(25)
    bb = G.Batch([b])
    bb.set_mode(L.BATCH_MODE_CHAINS)
    bb.step(25)
    assert np.array_equal(a.download(0), b.download(0))


def test_persistent_mode_small_instances_equal_chains():
    """Only small instances (four 128² on the compile-time Stockham tiles, two 256²): few tiles per
    instance, so the persistent kernel's y tiles often wait for their x tiles.  Bitwise equal to the
    chains after 1, 16 and 23 steps."""
    import gopf_gb300 as G
    from gopf_gb300 import _lib as L

    sides = [128, 256, 128, 128, 256, 128]
    a = _tune_models("fp32", sides, seed0=7000)
    b = _tune_models("fp32", sides, seed0=7000)
    ba, bb = G.Batch(a), G.Batch(b)
    bb.set_mode(L.BATCH_MODE_CHAINS)
    assert ba.mode() == L.BATCH_MODE_PERSISTENT
    for n in (1, 15, 7):
        ba.step(n)
        bb.step(n)
    for x, y in zip(a, b):
        assert np.array_equal(x.download(0), y.download(0))
