"""Shared comparison helpers of the parity tests (GPU path vs CPU oracle)."""
from __future__ import annotations

import numpy as np


def keyed_contacts(system, base_wall_id: int):
    """{(listing id, partner id or wall id): (tx, ty, tz, velrel)} of the live
    contact list.  A local pair appears under both ids, a pair with a periodic
    image under its local sphere only, so the keys tell the two apart."""
    ids = system.state().id
    o, q, t, v = system.contacts()
    out = {}
    for k in range(len(o)):
        key = (int(ids[o[k]]), int(q[k]))
        if key in out:
            raise AssertionError(f"contact {key} listed twice")
        out[key] = (t[k, 0], t[k, 1], t[k, 2], v[k])
    return out


def by_id(ids, arr):
    order = np.argsort(ids)
    return arr[order]


def assert_same_contact_sets(a: dict, b: dict, what: str = ""):
    ka, kb = set(a), set(b)
    if ka != kb:
        only_a = sorted(ka - kb)[:10]
        only_b = sorted(kb - ka)[:10]
        raise AssertionError(f"{what}: contact sets differ: {len(ka)} vs {len(kb)}; only first {only_a}, "
                             f"only second {only_b}")


def max_rel(a: np.ndarray, b: np.ndarray, scale: np.ndarray) -> float:
    """max |a-b| / scale over rows (scale per row, >0)."""
    d = np.abs(a - b).max(axis=-1) if a.ndim > 1 else np.abs(a - b)
    return float((d / scale).max()) if len(d) else 0.0


def compare_history(a: dict, b: dict, rtol: float, atol_tan: float = 1e-25):
    worst = 0.0
    for k, va in a.items():
        vb = b[k]
        ta, tb = np.array(va[:3]), np.array(vb[:3])
        sc = max(np.abs(ta).max(), np.abs(tb).max(), atol_tan)
        worst = max(worst, float(np.abs(ta - tb).max() / sc))
        sv = max(abs(va[3]), abs(vb[3]), 1e-300)
        worst = max(worst, abs(va[3] - vb[3]) / sv)
    assert worst <= rtol, f"history mismatch: max relative {worst:.3e} > {rtol:.1e}"
    return worst


def force_scale(F: np.ndarray, floor: float) -> np.ndarray:
    return np.maximum(np.abs(F).max(axis=1), floor)
