import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C-ABI of libkzg.so")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import pykzo
    pykzo.build()
    return pykzo


@pytest.fixture(scope="session")
def kzg_lib():
    from kizuriphysics3d_gb300 import build, capi
    build.build()
    return capi.load()


def load_golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def golden_resolved(scene, g: dict):
    """Resolved setup (hulls + mass) exactly as the reference computed it."""
    from kizuriphysics3d_gb300.world import HullData, Resolved
    hulls = {}
    for si, s in enumerate(scene.shapes):
        if s.type == 4:
            hulls[si] = HullData(g[f"hull{si}_verts"], g[f"hull{si}_sizes"], g[f"hull{si}_idx"])
    return Resolved(hulls, g["inv_mass"], g["inv_inertia_local"])


def oracle_blob(scene, resolved) -> bytes:
    from oracle import trace as T
    hulls = {i: T.Hull(h.verts, h.sizes, h.idx, 0.0) for i, h in resolved.hulls.items()}
    return T.resolved_blob(scene, hulls, resolved.inv_mass, resolved.inv_inertia_local)


def bits(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


# kzg_body_edit / kzo_body_edit records: op, packed BodyID, wake, reserved, 8 operands
BODY_EDIT_DTYPE = np.dtype([("op", "<u4"), ("body", "<u4"), ("wake", "<u4"), ("reserved", "<u4"),
                            ("v", "<f4", (8,))])


def golden_edits(g: dict, step: int) -> np.ndarray:
    """The body operations a golden fixture's reference run applied before `step`, as edit records
    with packed ids (a stale id is the slot's id with another sequence number)."""
    e = g.get("edits")
    if e is None:
        return np.zeros(0, BODY_EDIT_DTYPE)
    e = e[e["step"] == step]
    out = np.zeros(len(e), BODY_EDIT_DTYPE)
    slot = e["slot"] & 0x7FFFFFFF
    out["body"] = g["packed"][slot] ^ np.where(e["slot"] & 0x80000000, np.uint32(1 << 24), np.uint32(0))
    out["op"], out["wake"], out["v"] = e["op"], e["wake"], e["v"]
    return out


def apply_golden_edits(world, g: dict, step: int) -> None:
    """Apply golden_edits(g, step) to an oracle or GPU world (both take the same records)."""
    e = golden_edits(g, step)
    if len(e):
        world.edit_bodies(e)
