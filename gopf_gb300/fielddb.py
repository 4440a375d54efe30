"""FieldDB: gopf's SQLite field database, fed from device-resident fields.

pf.FieldDB (pf/database.go:67-430) stores a run's fields, attributes, comments
and time series in seven tables.  This module keeps the same file format
(the same tables, columns and conventions, so `gopf db ...` and pf.FieldDB.Load
read what it writes) and the same operations:

    SaveFields (database.go:231-243)   -> save_fields / save_model
    Comment (:246-257)                 -> comment
    SetAttr / SetTextAttr (:260-317)   -> set_attr / set_text_attr
    TimeSeries (:318-343)              -> time_series
    Load / LoadLast (:376-430)         -> load / load_last

Differences in how, not what:
- rows go in with one prepared statement per table and one transaction per call
  (executemany over numpy columns) instead of a statement prepared per row;
- save_model downloads the real fields from the device (the library's c2r pass)
  once per epoch, and save_sweep writes a whole batched sweep: one database per
  domain size (a FieldDB holds one size, database.go:347-371), one simID per
  instance with its parameters as attributes.

Reference conventions kept on purpose: positions get automatic ids 1, 2, ...
while fields.positionId is the 0-based node index (database.go:174-199 and
:202-228), the X, Y, Z columns hold pfutil.Pos's (row, col, depth)
(pfutil/indexPositionConversion.go:23-44), the positions table counts as
populated when it holds more than one row, and comments have newlines replaced
by spaces.  It runs on the host and needs Python's sqlite3.
"""
from __future__ import annotations

import os
import random
import sqlite3
from typing import Iterable, Sequence

import numpy as np

_SCHEMA = (
    "CREATE TABLE IF NOT EXISTS simIDs (simID INTEGER UNIQUE, creationTime TEXT)",
    "CREATE TABLE IF NOT EXISTS positions (id INTEGER PRIMARY KEY, X INTEGER, Y INTEGER, Z INTEGER)",
    "CREATE TABLE IF NOT EXISTS fields (id INTEGER PRIMARY KEY, name TEXT, value REAL, positionId INTEGER, "
    "timestep INTEGER, simID INTEGER, FOREIGN KEY(positionId) REFERENCES positions(id), "
    "FOREIGN KEY(simID) REFERENCES simIDs(simID))",
    "CREATE TABLE IF NOT EXISTS simAttributes (key TEXT, value REAL, simID INTEGER, "
    "FOREIGN KEY(simID) REFERENCES fields(simID))",
    "CREATE TABLE IF NOT EXISTS comments (simID INTEGER, value TEXT, FOREIGN KEY(simID) REFERENCES simIds(simID))",
    "CREATE TABLE IF NOT EXISTS simTextAttributes (key TEXT, value TEXT, simID INTEGER, "
    "FOREIGN KEY(simID) REFERENCES simIds(simID))",
    "CREATE TABLE IF NOT EXISTS timeseries (key TEXT, value REAL, timestep INTEGER, simID INTEGER, "
    "FOREIGN KEY(simID) REFERENCES simIds(simID))",
)


def positions(domain_size: Sequence[int]) -> np.ndarray:
    """pfutil.Pos for every node, as rows (X, Y, Z) = (row, col, depth); Z = 0 in 2D."""
    d = [int(x) for x in domain_size]
    n = int(np.prod(d))
    i = np.arange(n, dtype=np.int64)
    col = i % d[1]
    if len(d) == 2:
        return np.stack([i // d[1], col, np.zeros_like(i)], axis=1)
    return np.stack([(i // d[1]) % d[0], col, i // (d[0] * d[1])], axis=1)


class FieldDB:
    """A field database on one SQLite file (or connection) for one domain size."""

    def __init__(self, db, domain_size: Sequence[int] | None = None, sim_id: int | None = None):
        self.conn = db if isinstance(db, sqlite3.Connection) else sqlite3.connect(db)
        self.domain_size = None if domain_size is None else [int(x) for x in domain_size]
        self.sim_id = int(sim_id) if sim_id else 0
        self.initialized = False

    def close(self) -> None:
        self.conn.close()

    # ---- database.go:81-156 ----
    def initialize(self) -> None:
        cur = self.conn.cursor()
        for stmt in _SCHEMA:
            cur.execute(stmt)
        if self.sim_id == 0:
            self.sim_id = random.SystemRandom().randrange(1, 2 ** 31)
        cur.execute("INSERT INTO simIDs (simID, creationTime) VALUES (?, datetime('now', 'localtime'))",
                    (self.sim_id,))
        self.conn.commit()
        self.initialized = True

    def _ensure(self) -> None:
        if not self.initialized:
            self.initialize()

    def positions_populated(self) -> bool:
        return self.conn.execute("SELECT COUNT(*) FROM positions").fetchone()[0] > 1

    def populate_positions(self) -> None:
        pos = positions(self.domain_size)
        with self.conn:
            self.conn.executemany("INSERT INTO positions (X, Y, Z) VALUES (?, ?, ?)", map(tuple, pos.tolist()))

    def domain_size_ok(self) -> bool:
        """database.go:347-371: the largest X, Y (and Z) of the positions table match the domain."""
        if self.domain_size is None:
            return True
        for col, n in zip(("X", "Y", "Z"), self.domain_size):
            mx = self.conn.execute(f"SELECT MAX({col}) FROM positions").fetchone()[0]
            if mx != n - 1:
                return False
        return True

    # ---- database.go:202-243 ----
    def insert_real_part(self, name: str, timestep: int, values: np.ndarray) -> None:
        if not self.domain_size_ok():
            raise ValueError("FieldDB: Domain size does not match the positions table in the database")
        v = np.asarray(values)
        if v.size != int(np.prod(self.domain_size)):
            raise ValueError("FieldDB: The passed array does not match the specified domain size")
        re = np.real(v).astype(np.float64).reshape(-1)
        rows = zip([name] * re.size, re.tolist(), range(re.size), [int(timestep)] * re.size,
                   [self.sim_id] * re.size)
        with self.conn:
            self.conn.executemany(
                "INSERT INTO fields (name, value, positionId, timestep, simID) VALUES (?, ?, ?, ?, ?)", rows)

    def save_fields(self, fields: Iterable[tuple[str, np.ndarray]], epoch: int) -> None:
        """SaveFields for (name, data) pairs, data in node order."""
        self._ensure()
        if not self.positions_populated():
            self.populate_positions()
        for name, data in fields:
            self.insert_real_part(name, epoch, data)

    def save_model(self, model, epoch: int) -> None:
        """SaveFields of a device-resident gopf_gb300.Model: each field's real part comes from the
        device's c2r pass (gopf_field_download_real)."""
        names = model.field_names or ["field"]
        self.save_fields(((nm, model.download_real(f)) for f, nm in enumerate(names)), epoch)

    # ---- database.go:246-343 ----
    def comment(self, text: str) -> None:
        self._ensure()
        with self.conn:
            self.conn.execute("INSERT INTO comments (simID, value) VALUES (?, ?)",
                              (self.sim_id, text.replace("\n", " ")))

    def set_attr(self, attr: dict) -> None:
        self._ensure()
        with self.conn:
            self.conn.executemany("INSERT INTO simAttributes (key, value, simID) VALUES (?, ?, ?)",
                                  [(k, float(v), self.sim_id) for k, v in attr.items()])

    def set_text_attr(self, attr: dict) -> None:
        self._ensure()
        with self.conn:
            self.conn.executemany("INSERT INTO simTextAttributes (key, value, simID) VALUES (?, ?, ?)",
                                  [(k, str(v), self.sim_id) for k, v in attr.items()])

    def time_series(self, data: dict, timestep: int) -> None:
        self._ensure()
        with self.conn:
            self.conn.executemany("INSERT INTO timeseries (key, value, timestep, simID) VALUES (?, ?, ?, ?)",
                                  [(k, float(v), int(timestep), self.sim_id) for k, v in data.items()])

    # ---- database.go:376-430 ----
    def load(self, sim_id: int, timestep: int) -> list[tuple[str, np.ndarray]]:
        """The fields of a run at a timestep, sorted by name, as complex arrays (real part stored)."""
        names = [r[0] for r in self.conn.execute(
            "SELECT DISTINCT name FROM fields WHERE simID=? AND timestep=? ORDER BY name", (sim_id, timestep))]
        n = self.conn.execute("SELECT COUNT(*) FROM positions").fetchone()[0]
        out = {nm: np.zeros(n, dtype=np.complex128) for nm in names}
        for nm, val, pid in self.conn.execute(
                "SELECT name, value, positionId FROM fields WHERE simID=? AND timestep=?", (sim_id, timestep)):
            out[nm][pid] = val
        return [(nm, out[nm]) for nm in names]

    def load_last(self, sim_id: int) -> list[tuple[str, np.ndarray]]:
        ts = self.conn.execute("SELECT MAX(timestep) FROM fields WHERE simID=?", (sim_id,)).fetchone()[0]
        return self.load(sim_id, ts)


def save_sweep(models, params: Sequence[dict], directory: str, epoch: int, prefix: str = "sweep") -> dict:
    """Write every instance of a batched sweep: one database file per domain size
    (<directory>/<prefix>_<rows>x<cols>.db), one simID per instance, the instance's parameters as
    simAttributes and its fields at `epoch`.  Returns {instance index: (path, simID)}."""
    os.makedirs(directory, exist_ok=True)
    conns: dict[tuple, sqlite3.Connection] = {}
    out = {}
    try:
        for i, (m, p) in enumerate(zip(models, params)):
            key = tuple(m.domain_size)
            path = os.path.join(directory, f"{prefix}_{'x'.join(str(d) for d in key)}.db")
            if key not in conns:
                conns[key] = sqlite3.connect(path)
            db = FieldDB(conns[key], m.domain_size)
            db.set_attr(p)
            db.save_model(m, epoch)
            out[i] = (path, db.sim_id)
    finally:
        for c in conns.values():
            c.close()
    return out
