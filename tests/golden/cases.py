"""The beds of the golden fixtures in this folder.

Each fixture is a restart chain in the reference's restart-file layout
(sdem_gb300/restart.py, Prtcl_IOAndVisu.f90:903-1025): the input state with its
contact list and spring history, the state after one step from that file, and
the state after ten steps, plus the forces and torques of the first step.  The
beds come from the seeded makers of sdem_gb300.beds, so a test rebuilds the
material tables, walls and options from the name and takes the particles and
contacts from the input file (the reference's own restart workflow:
RestartFlag=T, ifirstDEM = itime + 1).
"""
from sdem_gb300 import beds, props

# name -> (maker of the case, steps the oracle runs before the input file)
GOLDEN = {
    # polydisperse Hertz, box walls, AB2 (the 1M configuration's contact law)
    "hertz_poly": (lambda: beds.lattice_cloud_case(400, seed=201, ntypes=7), 40),
    # monodisperse linear spring-dashpot, AB2 (the 20k configuration's law)
    "lsd_mono": (lambda: beds.lattice_cloud_case(400, seed=202, ntypes=1, nn=0.995e-3, cf_type=props.CFT_LSD), 40),
    # bidisperse 1:3 spheres in a hopper of finite walls with an outlet
    "hopper": (lambda: beds.hopper_case(600, 203), 60),
    # periodic in x and z (ghost images, image contacts, the wrap)
    "periodic_xz": (lambda: beds.periodic_lattice_case(400, 204, (1, 0, 1)), 30),
    # hierarchical search over three levels of cells
    "hrchl_poly3": (lambda: beds.scaled(beds.lattice_cloud_case(400, seed=205, ntypes=9, d_lo=0.3e-3, d_hi=1.2e-3,
                                                                nn=0.9e-3), cs_method=2), 30),
    # a rough floor of fixed spheres, linear spring-dashpot, forward Euler
    "lsd_fe_fixed": (lambda: beds.fixed_floor_case(400, 206, cf_type=props.CFT_LSD, ntypes=3, pi=1, pri=1), 30),
    # Adams-Bashforth 3, rolling resistance scaled by the relative speed
    # (CT_Model 2), the rotation update from the angular velocity (no quirk)
    "hertz_ab3_ct2": (lambda: beds.scaled(beds.lattice_cloud_case(400, seed=207, pi=3, pri=3), ct_model=2,
                                          quirk_ab2_rot=0), 30),
}

CHAIN = (1, 10)   # steps after the input file whose state is stored


def file_name(name: str, itime: int) -> str:
    """RestartFor<RunName><itime I10.10> (Prtcl_IOAndVisu.f90:889-891), gzip-compressed."""
    return f"RestartFor{name}{itime:010d}.gz"


def forces_name(name: str, itime: int) -> str:
    """Forces and torques of step itime, (n, 6) float64 in the file's particle order."""
    return f"Forces{name}{itime:010d}.npy"
