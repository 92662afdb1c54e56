"""Residual-terminated velocity iterations in the oracle (no GPU): the stopping rule's contract."""
import numpy as np

from conftest import golden_resolved, load_golden, oracle_blob
from tests.golden.gen_golden import fixture_scenes


def _world(oracle_lib, name="pile200"):
    sc = fixture_scenes()[name][0]
    g = load_golden(name)
    res = golden_resolved(sc, g)
    return sc, oracle_lib.OracleWorld(sc.to_bytes(), oracle_blob(sc, res), oracle_lib.PAIRS_CANONICAL)


def test_fixed_count_is_the_default(oracle_lib):
    sc, w = _world(oracle_lib)
    for _ in range(30):
        w.step(np.float32(sc.dt))
    st = w.stats()
    assert st["max_velocity_iterations"] == sc.velocity_iterations


def test_stops_at_tolerance_or_cap(oracle_lib):
    sc, w = _world(oracle_lib)
    w.set_residual(1e-4, 64)
    for _ in range(60):
        w.step(np.float32(sc.dt))
        st = w.stats()
        assert 1 <= st["max_velocity_iterations"] <= 64
        if st["max_velocity_iterations"] < 64:
            assert st["final_residual"] <= 1e-4


def test_tighter_tolerance_needs_more_iterations(oracle_lib):
    totals = []
    for tol in (1e-2, 1e-4):
        sc, w = _world(oracle_lib)
        w.set_residual(tol, 64)
        total = 0
        for _ in range(40):
            w.step(np.float32(sc.dt))
            total += w.stats()["point_velocity_iterations"]
        totals.append(total)
    assert totals[1] > totals[0]
