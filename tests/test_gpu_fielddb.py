"""FieldDB fed from device-resident fields.

- TestLoadFields (pf/database_test.go:364-420) on the device: two fields driven by constant rates
  (0.1 and -0.1, RegisterFunction constants), Euler dt 1, ten epochs of one step with SaveFields
  after each; Load(simID, step) gives 0.1 (step + 1) and -0.1 (step + 1), fields sorted by name,
  and LoadLast the last epoch.
- A batched sweep written with save_sweep: one database per domain size, one simID per instance
  with its parameters as attributes, and every instance's field in its database equal to what the
  device holds.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_reference_load_fields_on_the_device(tmp_path):
    import gopf_gb300 as G
    from gopf_gb300.fielddb import FieldDB

    m = G.Model([4, 4], "fp64", device=0)
    m.add_field("temperature")
    m.add_field("conc")
    m.register_function("RATE_TEMP", G.DER_POLY, "temperature", [0.1], [0])
    m.register_function("RATE_CONC", G.DER_POLY, "conc", [-0.1], [0])
    m.add_equation("dtemperature/dt = RATE_TEMP")
    m.add_equation("dconc/dt = RATE_CONC")
    m.init()
    m.set_stepper("euler", 1.0)
    m.upload(0, np.zeros(16))
    m.upload(1, np.zeros(16))
    db = FieldDB(str(tmp_path / "load.db"), [4, 4])
    for epoch in range(10):  # Solver.Solve(10, 1) with SaveFields as its callback
        m.step(1)
        db.save_model(m, epoch)
    for step in range(10):
        fields = db.load(db.sim_id, step)
        assert [n for n, _ in fields] == ["conc", "temperature"]
        assert np.allclose(fields[0][1], -0.1 * (step + 1), atol=1e-10)
        assert np.allclose(fields[1][1], 0.1 * (step + 1), atol=1e-10)
    last = db.load_last(db.sim_id)
    assert np.allclose(last[1][1], 1.0, atol=1e-10)
    m.close()


def test_sweep_results_go_to_one_database_per_size(tmp_path):
    import sqlite3

    import gopf_gb300 as G
    from gopf_gb300.fielddb import save_sweep
    from gopf_gb300.synthetic import uniform_field

    sides = [256, 128, 256, 384]
    models, params = [], []
    for i, s in enumerate(sides):
        m = G.Model([s, s], "fp32", device=0)
        m.add_field("conc")
        m.add_scalar("gamma", 0.5 + 0.1 * i)
        m.add_scalar("M", 1.0)
        m.add_scalar("mM", -1.0)
        m.add_equation("dconc/dt = M*LAP conc^3 + mM*LAP conc + mM*gamma*LAP^2 conc")
        m.init()
        m.set_stepper("euler", 0.05)
        m.upload(0, uniform_field(500 + i, s * s, 0.5, 0.05))
        models.append(m)
        params.append({"gamma": 0.5 + 0.1 * i, "M": 1.0})
    G.Batch(models).step(20)
    where = save_sweep(models, params, str(tmp_path), epoch=20)
    assert len({p for p, _ in where.values()}) == 3  # 128, 256, 384
    for i, (path, sim) in where.items():
        conn = sqlite3.connect(path)
        vals = conn.execute("SELECT value FROM fields WHERE simID=? AND timestep=20 ORDER BY positionId",
                            (sim,)).fetchall()
        assert np.array_equal(np.array([v[0] for v in vals]), models[i].download_real(0))
        attrs = dict(conn.execute("SELECT key, value FROM simAttributes WHERE simID=?", (sim,)).fetchall())
        assert attrs == params[i]
        conn.close()
