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


def sorted_contacts(system):
    """(keys, history) of the live contact list, keys = (listing id, partner
    or wall id) packed in 64 bits, sorted; vectorised for millions of records."""
    ids = system.state().id.astype(np.int64)
    o, q, t, v = system.contacts()
    key = (ids[o] << 32) | (np.asarray(q, np.int64) & 0xFFFFFFFF)
    order = np.argsort(key, kind="stable")
    hist = np.concatenate([np.asarray(t, float), np.asarray(v, float)[:, None]], axis=1)
    return key[order], hist[order]


def assert_step_matches(g, o, rtol: float = 1e-12, what: str = ""):
    """After one step of a GPU system g and an oracle system o from identical
    inputs: counters equal, contact sets equal, history, forces and torques
    within rtol relative, ids equal, positions within 1e-13 relative."""
    cg, co = g.counters(), o.counters()
    for k in ("pp", "pw", "cnsv", "nlocal"):
        assert cg[k] == co[k], f"{what}: counter {k}: gpu {cg[k]} oracle {co[k]}"
    kg, hg = sorted_contacts(g)
    ko, ho = sorted_contacts(o)
    assert len(np.unique(kg)) == len(kg), f"{what}: a contact is listed twice"
    np.testing.assert_array_equal(kg, ko, err_msg=f"{what}: contact sets")
    sc = np.maximum(np.maximum(np.abs(hg[:, :3]).max(axis=1), np.abs(ho[:, :3]).max(axis=1)), 1e-25)
    bad = np.nonzero(np.abs(hg[:, :3] - ho[:, :3]).max(axis=1) > rtol * sc)[0]
    assert len(bad) == 0, (f"{what}: tangential history of {len(bad)} contacts; first "
                           + "; ".join(f"key ({kg[b] >> 32}, {kg[b] & 0xFFFFFFFF}) gpu {hg[b].tolist()} "
                                       f"oracle {ho[b].tolist()}" for b in bad[:3]))
    sv = np.maximum(np.maximum(np.abs(hg[:, 3]), np.abs(ho[:, 3])), 1e-300)
    bad = np.nonzero(np.abs(hg[:, 3] - ho[:, 3]) > rtol * sv)[0]
    assert len(bad) == 0, (f"{what}: VelRel_Init of {len(bad)} contacts; first "
                           + "; ".join(f"key ({kg[b] >> 32}, {kg[b] & 0xFFFFFFFF}) gpu {hg[b].tolist()} "
                                       f"oracle {ho[b].tolist()}" for b in bad[:3]))
    Fg, Tg = g.forces()
    Fo, To = o.forces()
    fs = force_scale(Fo, 1e-6 * max(np.abs(Fo).max(), 1e-30))
    ts = force_scale(To, 1e-6 * max(np.abs(To).max(), 1e-30))
    assert np.all(np.abs(Fg - Fo).max(axis=1) <= rtol * fs), f"{what}: force mismatch"
    assert np.all(np.abs(Tg - To).max(axis=1) <= rtol * ts), f"{what}: torque mismatch"
    sg, so = g.state(), o.state()
    np.testing.assert_array_equal(sg.id, so.id)
    np.testing.assert_allclose(sg.posR, so.posR, rtol=1e-13, atol=1e-18)
    return {"pp": cg["pp"], "pw": cg["pw"], "contacts": len(kg)}
