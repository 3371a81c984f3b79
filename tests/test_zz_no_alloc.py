"""The allocation-free entry point sdem_count_contacts_noalloc, for callers
that cannot allocate device memory (a host inside another framework's memory
pool, or code between a pool reset and its next allocation): it counts the
contacts of particles already on the device using a fixed scratch array inside
the library.  Its counts must equal the ones the handle-based path reports
(sdem_step + sdem_counters) and the oracle's for the same positions, on two
calls in a row (the shared scratch keeps the previous call's contents).
Configurations it does not restate are refused, not miscounted.  Collected
last on purpose: a failure here leaves the rest of the suite already run."""
from dataclasses import replace

import numpy as np
import pytest

from oracle.oracle import OracleSystem
from sdem_gb300 import beds
from sdem_gb300.capi import NOALLOC_MAX_PARTICLES, DEMSystem, SdemError, cfg_from_case, count_contacts_noalloc

torch = pytest.importorskip("torch")

E_ARG, E_GRID, E_CAPACITY, E_UNSUPPORTED = 1, 6, 8, 10


def cases():
    return [beds.lattice_cloud_case(800, seed=61),
            beds.lattice_cloud_case(3000, seed=62, ntypes=1, nn=0.995e-3),
            beds.lsd_mono_case(20000)]


def _count(case, posR_dev, out):
    out.fill_(-1)
    count_contacts_noalloc(cfg_from_case(case), float(case.tables.radius.max()), case.particles.n,
                           posR_dev.data_ptr(), out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    return out.cpu().tolist()


@pytest.mark.gpu
@pytest.mark.parametrize("k", [0, 1, 2])
def test_noalloc_counts_match_handle_and_oracle(gpu_lib, oracle_lib, k):
    case = cases()[k]
    with DEMSystem(case) as h:
        h.step(1)   # counters of a step describe the positions it started from
        want = h.counters()
    orc = OracleSystem(case)
    orc.step(1)
    ref = orc.counters()
    orc.close()
    assert [want["pp"], want["cnsv"]] == [ref["pp"], ref["cnsv"]], (want, ref)
    posR = torch.from_numpy(np.ascontiguousarray(case.particles.posR)).cuda()
    out = torch.zeros(2, dtype=torch.int64, device="cuda")
    for _ in range(2):
        got = _count(case, posR, out)
        assert got == [ref["pp"], ref["cnsv"]], (got, ref)


@pytest.mark.gpu
def test_noalloc_out_of_grid_after_a_larger_call(gpu_lib, oracle_lib):
    """A particle outside the grid is not placed by the binning, so the sort
    positions past the placed ones still hold the previous (larger) call's
    indices; the call must report SDEM_E_GRID without reading them, and the
    next valid call must count correctly."""
    big = beds.lattice_cloud_case(800, seed=64)
    small = beds.lattice_cloud_case(100, seed=65)
    out = torch.zeros(2, dtype=torch.int64, device="cuda")
    _count(big, torch.from_numpy(np.ascontiguousarray(big.particles.posR)).cuda(), out)
    bad = small.particles.posR.copy()
    bad[37, 0] = small.opts.maxpoint[0] + 50.0 * 2.0 * float(small.tables.radius.max())
    with pytest.raises(SdemError) as e:
        _count(small, torch.from_numpy(bad).cuda(), out)
    assert e.value.code == E_GRID and "outside the padded search grid" in str(e.value)
    orc = OracleSystem(small)
    orc.step(1)
    ref = orc.counters()
    orc.close()
    got = _count(small, torch.from_numpy(np.ascontiguousarray(small.particles.posR)).cuda(), out)
    assert got == [ref["pp"], ref["cnsv"]], (got, ref)


@pytest.mark.gpu
def test_noalloc_refuses_oversize(gpu_lib):
    case = beds.lattice_cloud_case(100, seed=63)
    cfg = cfg_from_case(case)
    with pytest.raises(SdemError) as e:
        count_contacts_noalloc(cfg, float(case.tables.radius.max()), NOALLOC_MAX_PARTICLES + 1, 256, 256)
    assert e.value.code == E_CAPACITY and "SDEM_NOALLOC_MAX_PARTICLES" in str(e.value)
    big = beds.scaled(case, maxpoint=(1.0, 1.0, 1.0))
    with pytest.raises(SdemError) as e:
        count_contacts_noalloc(cfg_from_case(big), float(case.tables.radius.max()), 10, 256, 256)
    assert e.value.code == E_CAPACITY and "SDEM_NOALLOC_MAX_CELLS" in str(e.value)


# The refusals below return before any CUDA call, so they also run without a GPU
# (the library is built and loaded, nothing is launched).
def test_noalloc_refuses_what_it_does_not_restate(gpu_lib):
    case = beds.lattice_cloud_case(100, seed=66)
    r = float(case.tables.radius.max())
    for opts in (replace(case.opts, periodic=(1, 0, 0)), replace(case.opts, periodic=(0, 0, 1)),
                 replace(case.opts, cs_method=2)):
        with pytest.raises(SdemError) as e:
            count_contacts_noalloc(cfg_from_case(replace(case, opts=opts)), r, 100, 256, 256)
        assert e.value.code == E_UNSUPPORTED, str(e.value)
    fixed = beds.fixed_floor_case(200, seed=67)
    with pytest.raises(SdemError) as e:
        count_contacts_noalloc(cfg_from_case(fixed), r, 100, 256, 256)
    assert e.value.code == E_UNSUPPORTED and "fixed spheres" in str(e.value)


def test_noalloc_names_the_misaligned_pointer(gpu_lib):
    case = beds.lattice_cloud_case(100, seed=68)
    cfg, r = cfg_from_case(case), float(case.tables.radius.max())
    with pytest.raises(SdemError) as e:
        count_contacts_noalloc(cfg, r, 100, 256 + 8, 256)
    assert e.value.code == E_ARG and "d_posR" in str(e.value)
    with pytest.raises(SdemError) as e:
        count_contacts_noalloc(cfg, r, 100, 256, 256 + 4)
    assert e.value.code == E_ARG and "d_counts" in str(e.value)


def test_noalloc_refuses_degenerate_grids(gpu_lib):
    case = beds.lattice_cloud_case(100, seed=69)
    cfg = cfg_from_case(case)
    for radius in (1e-300, float("inf")):
        with pytest.raises(SdemError) as e:
            count_contacts_noalloc(cfg, radius, 100, 256, 256)
        assert e.value.code in (E_ARG, E_CAPACITY), str(e.value)
    nan_dom = cfg_from_case(beds.scaled(case, maxpoint=(float("nan"), 1.0, 1.0)))
    with pytest.raises(SdemError) as e:
        count_contacts_noalloc(nan_dom, float(case.tables.radius.max()), 100, 256, 256)
    assert e.value.code == E_ARG, str(e.value)
