"""The search decides most candidate pairs in single precision: coordinates
relative to their cell corner, rejected when d^2 > (ri+rj+M)^2, accepted when
d^2 < (ri+rj-M)^2, and only the band between goes to the reference's FP64
test.  This checks, with float32 arithmetic in the kernel's order, that the
single-precision decisions never contradict the FP64 test, on pairs placed
within a few margins of touching across all 14 cell offsets."""
import numpy as np

f32 = np.float32


def fp64_contact(P, Q):
    dr = P[3] + Q[3]
    dr2 = dr * dr
    dx = P[0] - Q[0]
    d2 = dx * dx
    if d2 > dr2:
        return False
    dy = P[1] - Q[1]
    d2 = dy * dy + d2
    if d2 > dr2:
        return False
    dz = P[2] - Q[2]
    d2 = dz * dz + d2
    return not (d2 > dr2)


def test_single_precision_decisions_agree_with_fp64():
    rng = np.random.default_rng(7)
    cell = 1.2e-3
    x0 = np.array([-1.26e-3, -1.26e-3, -1.26e-3])
    M = f32(32.0 * cell * 2.0 ** -23)
    cellf = f32(cell)
    offsets = [(0, 0, 0), (0, 0, -1), (-1, 0, -1), (-1, 0, 0), (-1, 0, 1)] + \
              [(lx, -1, i) for lx in (-1, 0, 1) for i in (-1, 0, 1)]
    checked = decided = 0
    for trial in range(60000):
        c = rng.integers(1, 480, size=3)
        rel = rng.uniform(0, cell, size=3)
        P = np.empty(4)
        P[:3] = x0 + c * cell + rel
        P[3] = rng.uniform(0.4e-3, 0.6e-3)
        off = np.array(offsets[trial % len(offsets)])
        rq = rng.uniform(0.4e-3, 0.6e-3)
        # a point of the neighbour cell near the sphere of radius P.r + rq
        for _ in range(20):
            u = rng.normal(size=3)
            u /= np.linalg.norm(u)
            dist = (P[3] + rq) * (1.0 + rng.uniform(-6.0, 6.0) * float(M) / (P[3] + rq))
            Qc = P[:3] + u * dist
            cq = np.floor((Qc - x0) / cell).astype(np.int64)
            if np.all(cq == c + off):
                break
        else:
            continue
        Q = np.array([*Qc, rq])
        cp = np.floor((P[:3] - x0) / cell).astype(np.int64)
        Pf = [f32(P[k] - (x0[k] + cp[k] * cell)) for k in range(3)] + [f32(P[3])]
        Qf = [f32(Q[k] - (x0[k] + cq[k] * cell)) for k in range(3)] + [f32(Q[3])]
        o = [f32(cp[k] - cq[k]) * cellf for k in range(3)]
        fx, fy, fz = [(Pf[k] - Qf[k]) + o[k] for k in range(3)]
        d2f = fx * fx + fy * fy + fz * fz
        rs = Pf[3] + Qf[3]
        exact = fp64_contact(P, Q)
        checked += 1
        bhi = rs + M
        if d2f > bhi * bhi:
            assert not exact, (P, Q)
            decided += 1
            continue
        blo = rs - M
        if d2f < blo * blo:
            assert exact, (P, Q)
            decided += 1
    assert checked > 15000 and decided > checked // 2
