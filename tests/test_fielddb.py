"""FieldDB (pf/database.go) on the host: the file format and the operations, with the reference's
own tests (pf/database_test.go) restated, without a GPU."""
import sqlite3

import numpy as np
import pytest

from gopf_gb300.fielddb import FieldDB, positions


def test_positions_follow_pfutil_pos():
    """pfutil.Pos (pfutil/indexPositionConversion.go:23-44): 2D (row, col, 0); 3D (row, col, depth)."""
    p2 = positions([3, 4])
    assert p2.shape == (12, 3)
    assert p2[5].tolist() == [1, 1, 0] and p2[11].tolist() == [2, 3, 0]
    p3 = positions([2, 3, 4])
    i = 1 * 2 * 3 + 1 * 3 + 2  # depth 1, row 1, col 2
    assert p3[i].tolist() == [1, 2, 1]


def test_tables_and_round_trip(tmp_path):
    db = FieldDB(str(tmp_path / "a.db"), [4, 4], sim_id=17)
    a = np.arange(16, dtype=float)
    b = -np.arange(16, dtype=float) + 0.5j
    db.save_fields([("conc", a), ("eta", b)], 3)
    db.save_fields([("conc", a * 2), ("eta", b)], 5)
    tables = {r[0] for r in db.conn.execute("SELECT name FROM sqlite_master WHERE type='table'")}
    assert tables == {"simIDs", "positions", "fields", "simAttributes", "comments", "simTextAttributes",
                      "timeseries"}
    # positions: automatic ids from 1, fields.positionId is the 0-based node
    assert db.conn.execute("SELECT COUNT(*) FROM positions").fetchone()[0] == 16
    assert db.conn.execute("SELECT MIN(id) FROM positions").fetchone()[0] == 1
    assert db.conn.execute("SELECT MIN(positionId), MAX(positionId) FROM fields").fetchone() == (0, 15)
    got = db.load(17, 3)
    assert [n for n, _ in got] == ["conc", "eta"]
    assert np.array_equal(got[0][1].real, a) and np.array_equal(got[1][1].real, b.real)
    assert np.all(got[1][1].imag == 0.0)  # the real part is stored
    last = db.load_last(17)
    assert np.array_equal(last[0][1].real, a * 2)
    assert db.conn.execute("SELECT simID FROM simIDs").fetchall() == [(17,)]


def test_attributes_comments_timeseries(tmp_path):
    db = FieldDB(str(tmp_path / "b.db"), [2, 2], sim_id=5)
    db.set_attr({"gamma": 1.3, "M": 0.8})
    db.set_text_attr({"model": "cahn-hilliard"})
    db.comment("first line\nsecond line")
    db.time_series({"mass": 1.0, "energy": -2.0}, 10)
    assert dict(db.conn.execute("SELECT key, value FROM simAttributes WHERE simID=5").fetchall()) == \
        {"gamma": 1.3, "M": 0.8}
    assert db.conn.execute("SELECT value FROM comments").fetchone()[0] == "first line second line"
    assert db.conn.execute("SELECT value FROM simTextAttributes").fetchone()[0] == "cahn-hilliard"
    assert sorted(db.conn.execute("SELECT key, value, timestep FROM timeseries").fetchall()) == \
        [("energy", -2.0, 10), ("mass", 1.0, 10)]


def test_domain_size_mismatch_is_refused(tmp_path):
    """insertRealPart panics when the positions table belongs to another domain size."""
    path = str(tmp_path / "c.db")
    FieldDB(path, [4, 4], sim_id=1).save_fields([("c", np.zeros(16))], 0)
    other = FieldDB(path, [8, 2], sim_id=2)
    with pytest.raises(ValueError):
        other.save_fields([("c", np.zeros(16))], 0)
    with pytest.raises(ValueError):
        FieldDB(path, [4, 4], sim_id=3).save_fields([("c", np.zeros(15))], 0)


def test_two_runs_share_a_database(tmp_path):
    """Two simIDs in one file (a sweep of one domain size): each loads its own fields."""
    path = str(tmp_path / "d.db")
    conn = sqlite3.connect(path)
    x, y = FieldDB(conn, [3, 3], sim_id=11), FieldDB(conn, [3, 3], sim_id=12)
    x.save_fields([("c", np.full(9, 1.0))], 0)
    y.save_fields([("c", np.full(9, 2.0))], 0)
    assert conn.execute("SELECT COUNT(*) FROM positions").fetchone()[0] == 9  # populated once
    assert np.all(x.load(11, 0)[0][1].real == 1.0) and np.all(y.load(12, 0)[0][1].real == 2.0)


def test_reference_initialize_populate_insert_and_save(tmp_path):
    """TestInitialize, TestPopulatePositionTable, TestInsertRealPart and TestSaveFields
    (pf/database_test.go:14-174): the seven tables, a non-zero simID, positions in the reference's
    order for 3x3, nine values of one field at timestep 2, and 9 positions plus 18 field rows after
    saving two fields."""
    db = FieldDB(str(tmp_path / "ref.db"), [3, 3])
    db.initialize()
    assert db.initialized and db.sim_id != 0
    names = [r[0] for r in db.conn.execute("SELECT name FROM sqlite_master WHERE type='table' ORDER BY name")]
    assert names == ["comments", "fields", "positions", "simAttributes", "simIDs", "simTextAttributes", "timeseries"]
    assert not db.positions_populated()
    db.populate_positions()
    expect = [[0, 0, 0], [0, 1, 0], [0, 2, 0], [1, 0, 0], [1, 1, 0], [1, 2, 0], [2, 0, 0], [2, 1, 0], [2, 2, 0]]
    assert [list(r) for r in db.conn.execute("SELECT X, Y, Z FROM positions ORDER BY id")] == expect
    db.insert_real_part("myfield", 2, np.arange(9) + 0j)
    rows = db.conn.execute("SELECT name, timestep, value, simID FROM fields ORDER BY id").fetchall()
    assert rows == [("myfield", 2, float(i), db.sim_id) for i in range(9)]
    db2 = FieldDB(str(tmp_path / "save.db"), [3, 3])
    db2.save_fields([("field1", np.zeros(9)), ("field2", np.zeros(9))], 1)
    assert db2.conn.execute("SELECT COUNT(*) FROM positions").fetchone()[0] == 9
    assert db2.conn.execute("SELECT COUNT(*) FROM fields").fetchone()[0] == 18
