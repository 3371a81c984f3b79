"""Loading of the golden fixtures (tests/golden/) for the CPU and GPU tests."""
from __future__ import annotations

import os

import numpy as np

from sdem_gb300 import beds, restart
from tests.golden.cases import CHAIN, GOLDEN, file_name, forces_name

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name: str, itime: int, case):
    """(particles, contacts) of the fixture file of `name` at `itime`."""
    return restart.read_restart(os.path.join(GOLDEN_DIR, file_name(name, itime)), case.opts.tsize,
                                case.opts.rsize, case.tables.radius)


def start(name: str):
    """(case rebuilt from its maker with the input file's particles and
    contacts, steps before the input file)."""
    maker, pre = GOLDEN[name]
    base = maker()
    p, c = load(name, pre, base)
    return beds.Case(base.name, base.opts, base.tables, base.walls, p, contacts=c, fixed=base.fixed), pre


def forces(name: str, itime: int):
    a = np.load(os.path.join(GOLDEN_DIR, forces_name(name, itime)))
    return a[:, :3], a[:, 3:]


def keyed(parts, contacts) -> dict:
    """{(listing id, partner id or wall id): (tx, ty, tz, velrel)} of a contact list."""
    o, q, t, v = contacts
    out = {}
    for k in range(len(o)):
        key = (int(parts.id[o[k]]), int(q[k]))
        if key in out:
            raise AssertionError(f"contact {key} listed twice")
        out[key] = (t[k, 0], t[k, 1], t[k, 2], v[k])
    return out


__all__ = ["CHAIN", "GOLDEN", "GOLDEN_DIR", "load", "start", "forces", "keyed"]
