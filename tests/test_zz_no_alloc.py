"""The allocation-free entry point sdem_count_contacts_noalloc, for callers
that cannot allocate device memory (a host inside another framework's memory
pool, or code between a pool reset and its next allocation): it counts the
contacts of particles already on the device using a fixed scratch array inside
the library.  Its counts must equal the ones the handle-based path reports
(sdem_step + sdem_counters) for the same positions, on two calls in a row (the
shared scratch keeps the previous call's contents).  Collected last on purpose:
a failure here leaves the rest of the suite already run."""
import ctypes

import numpy as np
import pytest

from sdem_gb300 import beds
from sdem_gb300.capi import (NOALLOC_MAX_PARTICLES, DEMSystem, SdemError, cfg_from_case, count_contacts_noalloc,
                             load)

torch = pytest.importorskip("torch")


def cases():
    return [beds.lattice_cloud_case(800, seed=61),
            beds.lattice_cloud_case(3000, seed=62, ntypes=1, nn=0.995e-3),
            beds.lsd_mono_case(20000)]


@pytest.mark.gpu
@pytest.mark.parametrize("k", [0, 1, 2])
def test_noalloc_counts_match_handle(gpu_lib, k):
    case = cases()[k]
    with DEMSystem(case) as h:
        h.step(1)   # counters of a step describe the positions it started from
        want = h.counters()
    cfg = cfg_from_case(case)
    posR = torch.from_numpy(np.ascontiguousarray(case.particles.posR)).cuda()
    out = torch.zeros(2, dtype=torch.int64, device="cuda")
    for _ in range(2):
        out.fill_(-1)
        count_contacts_noalloc(cfg, float(case.tables.radius.max()), case.particles.n, posR.data_ptr(),
                               out.data_ptr(), torch.cuda.current_stream().cuda_stream)
        got = out.cpu().tolist()
        assert got == [want["pp"], want["cnsv"]], (got, want)


@pytest.mark.gpu
def test_noalloc_refuses_oversize(gpu_lib):
    case = beds.lattice_cloud_case(100, seed=63)
    cfg = cfg_from_case(case)
    with pytest.raises(SdemError) as e:
        count_contacts_noalloc(cfg, float(case.tables.radius.max()), NOALLOC_MAX_PARTICLES + 1, 256, 256)
    assert e.value.code == 8 and "SDEM_NOALLOC_MAX_PARTICLES" in str(e.value)
    big = beds.scaled(case, maxpoint=(1.0, 1.0, 1.0))
    with pytest.raises(SdemError) as e:
        count_contacts_noalloc(cfg_from_case(big), float(case.tables.radius.max()), 10, 256, 256)
    assert e.value.code == 8 and "SDEM_NOALLOC_MAX_CELLS" in str(e.value)
