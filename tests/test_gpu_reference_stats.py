"""The production path (kzg_step: the GPU broad phase, every overlapping pair once in MakePairKey
order) pinned to the reference itself by the quantities a user sees.

Mode B keeps pairs the reference's QueryPairs drops (include/Kizuri/BroadPhase/BroadPhase.h:90-92)
and orders pairs, constraints and batches differently, so its float bits leave the reference's in
the first steps.  These tests run it for the full length of the reference-traced fixtures and
compare with the reference: its checkpoint states (tests/golden/*.npz, written by the reference
engine) and, for the per-step contact statistics, the oracle in the reference's tree pair order,
which tests/test_oracle_golden.py holds bit-identical to the reference at every step.

Tolerances, fixed before the first measurement:
  * deepest penetration over steps 60..end (max of -separation over all contact points):
    |gpu - reference| <= 0.01 m
  * mean penetration over the same window (all contact points with separation < 0):
    |gpu - reference| <= 0.002 m
  * kinetic energy per unit mass, mean over dynamic bodies of 0.5 |v|^2, averaged over the last
    60 steps: |gpu - reference| <= 0.01 J/kg
  * resting structures (pyramid20, stacks2x2x20): at the last checkpoint every dynamic body within
    0.05 m of its reference position, and each stack's top box height within 0.02 m
  * the convex pile (pile200, a chaotic drop): at the last checkpoint the mean body height within
    0.05 m of the reference's, the sorted height profiles within 0.25 m of each other everywhere,
    and the centre of mass within 0.1 m horizontally
"""
import numpy as np
import pytest

from conftest import golden_resolved, load_golden, oracle_blob
from tests.golden.gen_golden import fixture_scenes

pytestmark = pytest.mark.gpu

FIXTURES = fixture_scenes()


def _contact_stats(hdr, pts):
    if hdr.shape[0] == 0:
        return 0.0, []
    npt = hdr[:, 2].astype(np.int64)
    mask = np.arange(pts.shape[1])[None, :] < npt[:, None]
    sep = pts[:, :, 9][mask]
    pen = -sep[sep < 0.0]
    return (float(pen.max()) if pen.size else 0.0), pen.tolist()


def _run(name):
    from kizuriphysics3d_gb300 import World
    from oracle import pykzo
    sc, steps, _, ckpt = FIXTURES[name]
    g = load_golden(name)
    res = golden_resolved(sc, g)
    dyn = np.array([b.motion == 2 for b in sc.bodies])
    ref = pykzo.OracleWorld(sc.to_bytes(), oracle_blob(sc, res), pykzo.PAIRS_TREE)
    out = {"gpu": {"max": [], "pen": [], "ke": []}, "ref": {"max": [], "pen": [], "ke": []}}
    gpu_ckpt = {}
    with World(sc, resolved=res) as gw:
        for s in range(steps):
            ref.step(np.float32(sc.dt))
            gw.step_fixed()
            for side, (hdr, pts, st) in (("gpu", gw.contact_constraints()[:2] + (gw.state(),)),
                                         ("ref", ref.constraints()[:2] + (ref.state(),))):
                if s >= 60:
                    m, pen = _contact_stats(hdr, pts)
                    out[side]["max"].append(m)
                    out[side]["pen"].extend(pen)
                v = st[dyn, 7:10].astype(np.float64)
                out[side]["ke"].append(float(np.mean(0.5 * np.sum(v * v, axis=1))))
            if s in ckpt:
                gpu_ckpt[s] = gw.state()
        assert gw.get_stats()["device_error"] == 0
        # the oracle's tree-order run is the reference's: same hash at every checkpoint
        assert ref.hash() == int(g["hashes"][steps - 1])
    last = ckpt[-1]
    return sc, g, dyn, out, gpu_ckpt[last], g["ckpt_states"][len(ckpt) - 1]


def _common_checks(out):
    dmax = abs(max(out["gpu"]["max"]) - max(out["ref"]["max"]))
    mg = float(np.mean(out["gpu"]["pen"])) if out["gpu"]["pen"] else 0.0
    mr = float(np.mean(out["ref"]["pen"])) if out["ref"]["pen"] else 0.0
    kg, kr = float(np.mean(out["gpu"]["ke"][-60:])), float(np.mean(out["ref"]["ke"][-60:]))
    print(f"deepest {max(out['gpu']['max']):.4f} vs {max(out['ref']['max']):.4f} m, mean {mg:.5f} vs {mr:.5f} m, "
          f"KE {kg:.5f} vs {kr:.5f} J/kg")
    assert dmax <= 0.01
    assert abs(mg - mr) <= 0.002
    assert abs(kg - kr) <= 0.01


@pytest.mark.parametrize("name", ["pyramid20", "stacks2x2x20"])
def test_resting_structures_match_reference(name, kzg_lib):
    sc, g, dyn, out, gpu_last, ref_last = _run(name)
    _common_checks(out)
    d = np.linalg.norm(gpu_last[dyn, 0:3] - ref_last[dyn, 0:3], axis=1)
    print(f"{name}: {int((d <= 0.05).sum())} of {int(dyn.sum())} bodies within 0.05 m, max {d.max():.4f} m")
    assert (d <= 0.05).all()
    # top box of each stack / of the pyramid: the highest dynamic body per x-z column
    cols = {}
    for i in np.nonzero(dyn)[0]:
        key = (round(float(ref_last[i, 0]) / 1.5), round(float(ref_last[i, 2]) / 1.5))
        if key not in cols or ref_last[i, 1] > ref_last[cols[key], 1]:
            cols[key] = i
    for i in cols.values():
        assert abs(float(gpu_last[i, 1]) - float(ref_last[i, 1])) <= 0.02


def test_convex_pile_matches_reference_statistically(kzg_lib):
    sc, g, dyn, out, gpu_last, ref_last = _run("pile200")
    _common_checks(out)
    yg, yr = gpu_last[dyn, 1], ref_last[dyn, 1]
    d = np.linalg.norm(gpu_last[dyn, 0:3] - ref_last[dyn, 0:3], axis=1)
    print(f"pile200: mean height {yg.mean():.4f} vs {yr.mean():.4f} m; {int((d <= 0.1).sum())} of {int(dyn.sum())} "
          f"bodies within 0.1 m of the reference's pose")
    assert abs(float(yg.mean() - yr.mean())) <= 0.05
    assert float(np.max(np.abs(np.sort(yg) - np.sort(yr)))) <= 0.25
    cg, cr = gpu_last[dyn][:, [0, 2]].mean(axis=0), ref_last[dyn][:, [0, 2]].mean(axis=0)
    assert float(np.linalg.norm(cg - cr)) <= 0.1
