"""Writes the golden fixtures of this folder (run from the repository root:
python -m tests.golden.make_golden).

The reference ships no golden vectors and cannot be compiled here (no Fortran
compiler), so the outputs come from the CPU oracle (oracle/sdem_oracle.c, the
reference's algorithm restated).  With a Fortran build of the reference, the
same files are made by running it from each input file for 1 and 10 steps
(RestartFlag = T, ifirstDEM = itime + 1, ilastDEM = itime + 1 or + 10) and
gzip-compressing the restart files it writes; the tests then pin both the
oracle and the GPU path to the reference itself.
"""
import gzip
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.oracle import OracleSystem                      # noqa: E402
from sdem_gb300 import beds, restart                         # noqa: E402
from tests.golden.cases import CHAIN, GOLDEN, file_name, forces_name   # noqa: E402


def write_gz(path: str, case, system) -> None:
    with tempfile.TemporaryDirectory() as tmp:
        raw = os.path.join(tmp, "r")
        restart.write_restart(raw, system.state(), system.contacts(), case.opts.tsize, case.opts.rsize,
                              case.opts.base_wall_id)
        with open(raw, "rb") as f, gzip.GzipFile(path, "wb", mtime=0) as g:
            shutil.copyfileobj(f, g)


def main() -> None:
    for name, (maker, pre) in GOLDEN.items():
        case = maker()
        o = OracleSystem(case)
        o.step(pre)
        write_gz(os.path.join(HERE, file_name(name, pre)), case, o)
        # the chain starts from the file, as a restarted run does
        p, c = restart.read_restart(os.path.join(HERE, file_name(name, pre)), case.opts.tsize, case.opts.rsize,
                                    case.tables.radius)
        o2 = OracleSystem(beds.Case(case.name, case.opts, case.tables, case.walls, p, contacts=c, fixed=case.fixed))
        done = 0
        for k in CHAIN:
            o2.step(k - done)
            done = k
            write_gz(os.path.join(HERE, file_name(name, pre + k)), case, o2)
            if k == 1:
                F, T = o2.forces()
                np.save(os.path.join(HERE, forces_name(name, pre + 1)), np.concatenate([F, T], axis=1))
        print(name, case.particles.n, "particles,", o2.counters())


if __name__ == "__main__":
    main()
