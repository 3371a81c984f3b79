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


def _hertz_terms(pre, case, keys):
    """(ok mask, record, delta, |v_rn|) of the particle-particle keys."""
    nT = case.tables.n_types
    rec = case.tables.bpp.reshape(nT, nT, 11)
    ids = pre.id.astype(np.int64)
    order = np.argsort(ids)
    sid = ids[order]
    a, b = keys >> 32, keys & 0xFFFFFFFF
    ia = np.searchsorted(sid, a)
    ib = np.searchsorted(sid, b)
    ok = (b <= case.opts.base_wall_id) & (ia < len(sid)) & (ib < len(sid))
    ok &= (sid[np.minimum(ia, len(sid) - 1)] == a) & (sid[np.minimum(ib, len(sid) - 1)] == b)
    ia, ib = order[ia[ok]], order[ib[ok]]
    lo = np.where(a[ok] < b[ok], ia, ib)
    hi = np.where(a[ok] < b[ok], ib, ia)
    r = rec[pre.ptype[hi] - 1, pre.ptype[lo] - 1]   # Prtcl_BnryProp(pType(lo), pType(hi))
    x, rad = pre.posR[:, :3], pre.posR[:, 3]
    dvec = x[hi] - x[lo]
    dist = np.linalg.norm(dvec, axis=1)
    nvec = dvec / dist[:, None]
    delta = np.maximum(rad[lo] + rad[hi] - dist, 1e-9 * np.minimum(rad[lo], rad[hi]))
    v, w = pre.linVel[:, 0, :], pre.rotVel[:, 0, :]
    vr = v[lo] - v[hi] + np.cross(rad[lo, None] * w[lo] + rad[hi, None] * w[hi], nvec)
    vrn = np.abs((vr * nvec).sum(axis=1))
    return ok, r, delta, vrn


def hertz_force_scale(pre, case, keys, n):
    """Per particle of the step's input state (index order of `pre`, n
    rows): the sum over its particle-particle Hertz contacts (keys listed
    under both particles) of the magnitudes of the terms its force adds,
    (1 + mu_s) (K d^1.5 + |C_n| d^0.25 |v_rn|) -- the bound of the force's
    rounding when the terms cancel (sums that differ at ~1 ulp per term)."""
    ok, r, delta, vrn = _hertz_terms(pre, case, keys)
    mag = (1.0 + r[:, 8]) * (r[:, 2] * delta ** 1.5 + np.abs(r[:, 4]) * delta ** 0.25 * vrn)
    ids = pre.id.astype(np.int64)
    order = np.argsort(ids)
    owner = order[np.searchsorted(ids[order], (keys >> 32)[ok])]
    out = np.zeros(n)
    np.add.at(out, owner, mag)
    return out


def hertz_spring_scale(pre, case, keys):
    """Rounding scale of the tangential spring of particle-particle Hertz
    contacts (keys: listing id << 32 | partner id), from the state `pre` the
    step started from.  A sliding contact's spring is mu_s |f_n| / k_t with
    f_n = -K d^1.5 - C_n d^0.25 v_rn (Prtcl_ContactForce_inc.f90:32-60): when
    the elastic and damping terms nearly cancel, f_n's rounding is bounded
    relative to the sum of their magnitudes, not to their difference, so the
    scale is mu_s (K d^1.5 + |C_n| d^0.25 |v_rn|) / (K_t d^0.5).  Keys of wall
    contacts get 0 (their bar stays relative to the spring)."""
    out = np.zeros(len(keys))
    ok, r, delta, vrn = _hertz_terms(pre, case, keys)
    out[ok] = r[:, 8] * (r[:, 2] * delta ** 1.5 + np.abs(r[:, 4]) * delta ** 0.25 * vrn) / (r[:, 3] * np.sqrt(delta))
    return out


def assert_step_matches(g, o, rtol: float = 1e-12, what: str = "", pre=None, case=None):
    """After one step of a GPU system g and an oracle system o from identical
    inputs: counters equal, contact sets equal, history, forces and torques
    within rtol relative, ids equal, positions within 1e-13 relative.  With
    the step's input state `pre` and a Hertz `case`, a spring is relative to
    hertz_spring_scale where that exceeds the spring (cancellation in f_n)."""
    cg, co = g.counters(), o.counters()
    for k in ("pp", "pw", "cnsv", "nlocal"):
        assert cg[k] == co[k], f"{what}: counter {k}: gpu {cg[k]} oracle {co[k]}"
    kg, hg = sorted_contacts(g)
    ko, ho = sorted_contacts(o)
    assert len(np.unique(kg)) == len(kg), f"{what}: a contact is listed twice"
    np.testing.assert_array_equal(kg, ko, err_msg=f"{what}: contact sets")
    sc = np.maximum(np.maximum(np.abs(hg[:, :3]).max(axis=1), np.abs(ho[:, :3]).max(axis=1)), 1e-25)
    bad = np.nonzero(np.abs(hg[:, :3] - ho[:, :3]).max(axis=1) > rtol * sc)[0]
    if len(bad) and pre is not None and case is not None and case.opts.cf_type == 2:
        sc2 = np.maximum(sc[bad], hertz_spring_scale(pre, case, kg[bad]))
        bad = bad[np.abs(hg[bad, :3] - ho[bad, :3]).max(axis=1) > rtol * sc2]
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
    if pre is not None and case is not None and case.opts.cf_type == 2 and len(pre.id) == len(Fo):
        # forces in the step's input index order (no delete during the step)
        cs = hertz_force_scale(pre, case, kg, len(Fo))
        fs = np.maximum(fs, cs)
        ts = np.maximum(ts, cs * pre.posR[:, 3])
    badF = np.nonzero(np.abs(Fg - Fo).max(axis=1) > rtol * fs)[0]
    assert len(badF) == 0, (f"{what}: force mismatch on {len(badF)} particles; first "
                            + "; ".join(f"{i}: gpu {Fg[i].tolist()} oracle {Fo[i].tolist()} scale {fs[i]:.3e}"
                                        for i in badF[:3]))
    badT = np.nonzero(np.abs(Tg - To).max(axis=1) > rtol * ts)[0]
    assert len(badT) == 0, (f"{what}: torque mismatch on {len(badT)} particles; first "
                            + "; ".join(f"{i}: gpu {Tg[i].tolist()} oracle {To[i].tolist()} scale {ts[i]:.3e}"
                                        for i in badT[:3]))
    sg, so = g.state(), o.state()
    np.testing.assert_array_equal(sg.id, so.id)
    np.testing.assert_allclose(sg.posR, so.posR, rtol=1e-13, atol=1e-18)
    return {"pp": cg["pp"], "pw": cg["pw"], "contacts": len(kg)}
