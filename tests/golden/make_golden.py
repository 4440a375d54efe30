"""Generate the golden fixtures in this folder from the FP64 oracle.

    python tests/golden/make_golden.py

Each fixture is a small .npz holding the case parameters, a checksum of the
initial field (so a change of the synthetic generator is caught) and the
oracle's FP64 field after the stated number of steps.  The oracle itself is
pinned by the reference's known-answer tests (tests/test_oracle.py); the
fixtures carry those pinned results to machines where the oracle is not
built, and let the device be checked against fixed numbers rather than a
recomputation.

Cases (all FP64 oracle, the reference's Euler unless stated):
  ch2d_128     Cahn-Hilliard 128^2, gamma=1, M=1, dt=0.1, c0 = 0.5 + U(-0.05, 0.05) seed 0, 1000 steps
  ch3d_32      Cahn-Hilliard 32^3, gamma=0.5, M=1, dt=0.05, c0 = U(-0.1, 0.1) seed 1, 100 steps
  rk4_ch2d_64  Cahn-Hilliard 64^2 with RK4, gamma=1, dt=0.1, c0 = 0.5 + U(-0.05, 0.05) seed 0, 100 steps
  elastic3d_16 CH + Khachaturyan term 16^3 (cubic C11=1, C12=0.6, C44=0.5, misfit 0.01 I), gamma=1,
               dt=0.02, c0 = 0.3 + U(-0.02, 0.02) seed 3, 20 steps
  volcons2d_32 dphi/dt = -phi + phi^2 + volume-conserving multiplier (indicator derivative), dt=0.01,
               c0 = 0.5 + U(-0.3, 0.3) seed 7, 40 steps
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def cubic(c11, c12, c44):
    C = np.zeros((3, 3, 3, 3))
    for i in range(3):
        C[i, i, i, i] = c11
    for i in range(3):
        for j in range(i + 1, 3):
            C[i, i, j, j] = c12
            C[j, j, i, i] = c12
            C[i, j, i, j] = c44
            C[j, i, j, i] = c44
    return C


CASES = {
    "ch2d_128": dict(kind="ch", dims=[128, 128], gamma=1.0, M=1.0, dt=0.1, seed=0, center=0.5, hw=0.05,
                     steps=1000, stepper="euler"),
    "ch3d_32": dict(kind="ch", dims=[32, 32, 32], gamma=0.5, M=1.0, dt=0.05, seed=1, center=0.0, hw=0.1,
                    steps=100, stepper="euler"),
    "rk4_ch2d_64": dict(kind="ch", dims=[64, 64], gamma=1.0, M=1.0, dt=0.1, seed=0, center=0.5, hw=0.05,
                        steps=100, stepper="rk4"),
    "elastic3d_16": dict(kind="elastic", dims=[16, 16, 16], gamma=1.0, M=1.0, dt=0.02, seed=3, center=0.3,
                         hw=0.02, steps=20, stepper="euler"),
    "volcons2d_32": dict(kind="volcons", dims=[32, 32], dt=0.01, seed=7, center=0.5, hw=0.3, steps=40,
                         stepper="euler"),
}


def initial_field(case) -> np.ndarray:
    from gopf_gb300.synthetic import uniform_field

    return uniform_field(case["seed"], int(np.prod(case["dims"])), case["center"], case["hw"])


def checksum(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def oracle_model(O, case, c0):
    dims = case["dims"]
    if case["kind"] == "ch":
        m = O.cahn_hilliard(dims, gamma=case["gamma"], M=case["M"])
    elif case["kind"] == "elastic":
        m = O.cahn_hilliard(dims, gamma=case["gamma"])
        m.add_elastic(0, 0, cubic(1.0, 0.6, 0.5), np.eye(3) * 0.01, coef=-1.0, lap=1)
    elif case["kind"] == "volcons":
        m = O.Model(dims, 1)
        m.set_field(0, c0)
        ind = m.add_indicator(0, O.DER_INDICATOR_D)
        sq = m.add_product([0], [2])
        m.add_term(0, -1.0, implicit=True)
        m.add_volcons(0, 0, ind, case["dt"])
        m.add_term(0, 1.0, src_kind=O.SRC_DERIVED, src=sq)
    else:
        raise ValueError(case["kind"])
    m.set_field(0, c0)
    return m


def run_oracle(O, case) -> np.ndarray:
    c0 = initial_field(case)
    m = oracle_model(O, case, c0)
    if case["stepper"] == "rk4":
        m.step_rk4(case["dt"], case["steps"])
    else:
        m.step_euler(case["dt"], case["steps"])
    return m.field(0).real.copy()


def path(name: str) -> str:
    return os.path.join(HERE, name + ".npz")


def load(name: str):
    z = np.load(path(name), allow_pickle=False)
    return z["field"], str(z["c0_sha256"])


def main():
    from oracle import oracle as O

    O.build()
    for name, case in CASES.items():
        c0 = initial_field(case)
        field = run_oracle(O, case)
        np.savez_compressed(path(name), field=field, c0_sha256=np.array(checksum(c0)))
        print(f"{name}: {field.size} values, |field| = {np.linalg.norm(field):.6e}")


if __name__ == "__main__":
    main()
