! Prtcl_GPU_Driver.f90 -- the reference's side of the GPU drop-in.
!
! Packs the reference's global arrays and options into the C ABI of
! include/sdem_gpu.h (bound by Prtcl_GPU.f90) and back.  Built only with
! -DSDEM_GPU, after the reference's modules it uses.  DEMS_iterate
! (src/DEM/Prtcl_DEMSystem.f90:201-317) calls:
!
!   gpu_initialize()         once, after DEMS_Initialize's step 7 (:181-182)
!                            and, on a restart, after PIO_RestartCL filled the
!                            contact list (contacts passed with gpu_upload_contacts)
!   gpu_iterate()            in place of :214-247 (preIteration .. RemvReleased)
!   gpu_sync_state(with_F)   before dump_visu (:254) and Write_Restart (:261),
!                            only on the steps where they fire
!   gpu_sync_contacts()      before Write_Restart (:261): the device's contact
!                            list rebuilt in GPPW_CntctList, which the
!                            reference's restart writer then walks
!   gpu_log_counters(...)    before the log block (:273-313)
!   gpu_finalize()           at the end of the run
!
! Error statuses become the reference's own abort (DEMLogInfo%CheckForError
! with ErrT_Abort), so a failure stops the run as the CPU path would.
!
! The reference's type(real3) and type(real4) arrays are sequences of
! real(RK) = real(c_double); they are copied into contiguous real(c_double)
! scratch arrays of the ABI's layouts (no dependence on how the compiler lays
! out derived types).
module Prtcl_GPU_Driver
  use iso_c_binding
  use Prtcl_GPU
  use Prtcl_TypeDef
  use Prtcl_LogInfo
  use Prtcl_Parameters
  use Prtcl_Property
  use Prtcl_Variables
  use prtcl_Geometry
  use Prtcl_CL_and_CF
  implicit none
  private

  real(c_double), allocatable, save :: s_posR(:), s_lin(:), s_linA(:), s_theta(:), s_rot(:), s_rotA(:)
  integer(c_int), allocatable, save :: s_id(:), s_ptype(:), s_mark(:)

  public :: gpu_initialize, gpu_upload_contacts, gpu_iterate, gpu_sync_state, gpu_sync_contacts, gpu_log_counters, &
            gpu_finalize

contains

  subroutine gpu_check(ierr, where)
    integer(c_int), intent(in) :: ierr
    character(*), intent(in) :: where
    if (ierr /= SDEM_OK) call DEMLogInfo%CheckForError(ErrT_Abort, "sdem_gpu: "//where, sdem_message(gpu_h))
  end subroutine gpu_check

  subroutine alloc_scratch()
    integer :: m
    m = max(GPrtcl_list%mlocal, 1)
    if (allocated(s_posR)) return
    allocate(s_posR(4*m), s_lin(3*GPrtcl_list%tsize*m), s_linA(3*GPrtcl_list%tsize*m), s_theta(3*m), &
             s_rot(3*GPrtcl_list%rsize*m), s_rotA(3*GPrtcl_list%rsize*m), s_id(m), s_ptype(m), s_mark(m))
  end subroutine alloc_scratch

  ! GPrtcl_* (1:nlocal) -> the ABI's layouts: posR 4 per particle, the AB
  ! levels of a vector field in Fortran (k,i) order, 3 components each
  subroutine pack_state(n)
    integer, intent(in) :: n
    integer :: i, k, o
    do i = 1, n
      s_id(i) = GPrtcl_id(i); s_ptype(i) = GPrtcl_pType(i); s_mark(i) = GPrtcl_usrMark(i)
      s_posR(4*i-3:4*i) = [GPrtcl_PosR(i)%x, GPrtcl_PosR(i)%y, GPrtcl_PosR(i)%z, GPrtcl_PosR(i)%w]
      s_theta(3*i-2:3*i) = [GPrtcl_theta(i)%x, GPrtcl_theta(i)%y, GPrtcl_theta(i)%z]
      do k = 1, GPrtcl_list%tsize
        o = ((i-1)*GPrtcl_list%tsize + (k-1))*3
        s_lin(o+1:o+3) = [GPrtcl_linVel(k,i)%x, GPrtcl_linVel(k,i)%y, GPrtcl_linVel(k,i)%z]
        s_linA(o+1:o+3) = [GPrtcl_linAcc(k,i)%x, GPrtcl_linAcc(k,i)%y, GPrtcl_linAcc(k,i)%z]
      end do
      do k = 1, GPrtcl_list%rsize
        o = ((i-1)*GPrtcl_list%rsize + (k-1))*3
        s_rot(o+1:o+3) = [GPrtcl_rotVel(k,i)%x, GPrtcl_rotVel(k,i)%y, GPrtcl_rotVel(k,i)%z]
        s_rotA(o+1:o+3) = [GPrtcl_rotAcc(k,i)%x, GPrtcl_rotAcc(k,i)%y, GPrtcl_rotAcc(k,i)%z]
      end do
    end do
  end subroutine pack_state

  subroutine unpack_state(n)
    integer, intent(in) :: n
    integer :: i, k, o
    do i = 1, n
      GPrtcl_id(i) = s_id(i); GPrtcl_pType(i) = s_ptype(i); GPrtcl_usrMark(i) = s_mark(i)
      GPrtcl_PosR(i) = real4(s_posR(4*i-3), s_posR(4*i-2), s_posR(4*i-1), s_posR(4*i))
      GPrtcl_theta(i) = real3(s_theta(3*i-2), s_theta(3*i-1), s_theta(3*i))
      do k = 1, GPrtcl_list%tsize
        o = ((i-1)*GPrtcl_list%tsize + (k-1))*3
        GPrtcl_linVel(k,i) = real3(s_lin(o+1), s_lin(o+2), s_lin(o+3))
        GPrtcl_linAcc(k,i) = real3(s_linA(o+1), s_linA(o+2), s_linA(o+3))
      end do
      do k = 1, GPrtcl_list%rsize
        o = ((i-1)*GPrtcl_list%rsize + (k-1))*3
        GPrtcl_rotVel(k,i) = real3(s_rot(o+1), s_rot(o+2), s_rot(o+3))
        GPrtcl_rotAcc(k,i) = real3(s_rotA(o+1), s_rotA(o+2), s_rotA(o+3))
      end do
    end do
  end subroutine unpack_state

  ! one BinaryProperty as the ABI's 11 doubles (SDEM_BP_*)
  subroutine pack_bnry(b, out)
    type(BinaryProperty), intent(in) :: b
    real(c_double), intent(out) :: out(11)
    out = [b%RadEff, b%MassEff, b%StiffnessCoe_n, b%StiffnessCoe_t, b%DampingCoe_n, b%DampingCoe_t, &
           b%RestitutionCoe_n, b%RestitutionCoe_t, b%FrictionCoe_s, b%FrictionCoe_k, b%FrictionCoe_Roll]
  end subroutine pack_bnry

  subroutine gpu_initialize()
    type(sdem_cfg) :: cfg
    integer :: nT, nWT, i, j, k, nw
    real(c_double), allocatable :: rad(:), mass(:), inert(:), bpp(:), bpw(:), walls(:), fixpos(:)
    integer(c_int), allocatable :: wflags(:)
    integer(c_int) :: ierr

    call sdem_default_cfg(cfg)
    cfg%n_capacity = GPrtcl_list%mlocal
    cfg%max_gid = DEM_opt%numPrtcl
    cfg%tsize = GPrtcl_list%tsize
    cfg%rsize = GPrtcl_list%rsize
    cfg%cf_type = DEM_opt%CF_Type
    cfg%ct_model = DEM_opt%CT_Model
    cfg%pi_method = DEM_opt%PI_Method
    cfg%pri_method = DEM_opt%PRI_Method
    cfg%cs_method = DEM_opt%CS_Method
    cfg%cntct_list_size = DEM_opt%CntctList_Size
    cfg%base_wall_id = DEM_opt%Base_wall_id
    cfg%wall_max_update_iter = DEM_opt%Wall_max_update_iter
    cfg%periodic = merge(1, 0, DEM_opt%IsPeriodic)
    cfg%dt = DEM_opt%dt
    cfg%gravity = [DEM_opt%gravity%x, DEM_opt%gravity%y, DEM_opt%gravity%z]
    cfg%dom_min = [DEM_opt%SimDomain_min%x, DEM_opt%SimDomain_min%y, DEM_opt%SimDomain_min%z]
    cfg%dom_max = [DEM_opt%SimDomain_max%x, DEM_opt%SimDomain_max%y, DEM_opt%SimDomain_max%z]
    cfg%cs_ratio = DEM_opt%Prtcl_cs_ratio
    cfg%wall_neighbor_ratio = DEM_opt%Wall_neighbor_ratio
    cfg%n_fixed_capacity = DEM_opt%numPrtclFix
    cfg%cs_num_levels = DEM_opt%CS_numlvls
    ! row capacity: room for the spheres that can touch the largest one
    nT = DEM_opt%numPrtcl_Type
    allocate(rad(nT), mass(nT), inert(nT))
    do i = 1, nT
      rad(i) = DEMProperty%Prtcl_PureProp(i)%Radius
      mass(i) = DEMProperty%Prtcl_PureProp(i)%Mass
      inert(i) = DEMProperty%Prtcl_PureProp(i)%Inertia
    end do
    cfg%max_contacts_per_particle = min(64, max(24, ceiling(3.63d0 * (1.0d0 + maxval(rad)/minval(rad))**2)))
    ierr = sdem_create(cfg, gpu_h);  call gpu_check(ierr, "sdem_create")

    nWT = DEM_opt%numWall_type
    allocate(bpp(11*nT*nT), bpw(11*nT*nWT))
    do j = 1, nT
      do i = 1, nT
        call pack_bnry(DEMProperty%Prtcl_BnryProp(i,j), bpp(11*((j-1)*nT+(i-1))+1 : 11*((j-1)*nT+i)))
      end do
    end do
    do j = 1, nWT
      do i = 1, nT
        call pack_bnry(DEMProperty%PrtclWall_BnryProp(i,j), bpw(11*((j-1)*nT+(i-1))+1 : 11*((j-1)*nT+i)))
      end do
    end do
    ierr = sdem_set_types(gpu_h, nT, rad, mass, inert, bpp, nWT, bpw);  call gpu_check(ierr, "sdem_set_types")

    nw = DEMGeometry%num_pWall
    allocate(walls(25*max(nw,1)), wflags(4*max(nw,1)))
    do k = 1, nw
      associate(w => DEMGeometry%pWall(k))
        walls(25*(k-1)+1 : 25*k) = [w%P1%x, w%P1%y, w%P1%z, w%P2%x, w%P2%y, w%P2%z, w%P3%x, w%P3%y, w%P3%z, &
                                    w%P4%x, w%P4%y, w%P4%z, w%n%x, w%n%y, w%n%z, w%d, &
                                    w%trans_vel%x, w%trans_vel%y, w%trans_vel%z, &
                                    w%min_point%x, w%min_point%y, w%min_point%z, &
                                    w%max_point%x, w%max_point%y, w%max_point%z]
        wflags(4*(k-1)+1 : 4*k) = [merge(1,0,w%bothSide), merge(1,0,w%isInfinite), w%wall_id, w%wall_Type]
      end associate
    end do
    ierr = sdem_set_walls(gpu_h, nw, walls, wflags);  call gpu_check(ierr, "sdem_set_walls")

    if (DEM_opt%numPrtclFix > 0 .and. GPrtcl_list%mlocalFix > 0) then
      allocate(fixpos(3*GPrtcl_list%mlocalFix))
      do i = 1, GPrtcl_list%mlocalFix
        fixpos(3*i-2:3*i) = [GPFix_PosR(i)%x, GPFix_PosR(i)%y, GPFix_PosR(i)%z]
      end do
      ierr = sdem_set_fixed(gpu_h, GPrtcl_list%mlocalFix, GPFix_id, GPFix_pType, fixpos)
      call gpu_check(ierr, "sdem_set_fixed")
    end if

    call alloc_scratch()
    call pack_state(GPrtcl_list%nlocal)
    ierr = sdem_upload_particles(gpu_h, GPrtcl_list%nlocal, s_id, s_ptype, s_mark, s_posR, s_lin, s_linA, &
                                 s_theta, s_rot, s_rotA)
    call gpu_check(ierr, "sdem_upload_particles")
  end subroutine gpu_initialize

  ! the contact list of a restart: owner particle index (1-based here),
  ! partner id, TanDelta, VelRel_Init, as PIO_RestartCL reads them
  subroutine gpu_upload_contacts(nc, owner, partner, tandelta, velrel)
    integer, intent(in) :: nc
    integer, intent(in) :: owner(nc), partner(nc)
    real(RK), intent(in) :: tandelta(3,nc), velrel(nc)
    integer(c_int), allocatable :: o0(:), p0(:)
    real(c_double), allocatable :: t0(:), v0(:)
    integer(c_int) :: ierr
    allocate(o0(max(nc,1)), p0(max(nc,1)), t0(3*max(nc,1)), v0(max(nc,1)))
    o0(1:nc) = owner - 1
    p0(1:nc) = partner
    t0(1:3*nc) = reshape(tandelta, [3*nc])
    v0(1:nc) = velrel
    ierr = sdem_upload_contacts(gpu_h, nc, o0, p0, t0, v0);  call gpu_check(ierr, "sdem_upload_contacts")
  end subroutine gpu_upload_contacts

  ! one step; GPrtcl_list%nlocal follows the device's deletes
  subroutine gpu_iterate()
    integer(c_int) :: ierr, out(SDEM_CNT_SIZE)
    ierr = sdem_step(gpu_h, 1);  call gpu_check(ierr, "sdem_step")
    ierr = sdem_counters(gpu_h, out);  call gpu_check(ierr, "sdem_counters")
    GPrtcl_list%nlocal = out(6)
  end subroutine gpu_iterate

  ! The contact list as the restart writer lists it (every particle-particle
  ! contact under both particles, wall contacts under their particle),
  ! rebuilt in GPPW_CntctList through the reference's own
  ! Add_RestartCntctlink, after the list is emptied (every link released).
  ! sdem_check_restart_limit first raises the writer's own abort for more than
  ! 20 contacts on one particle (Prtcl_CL_and_CF.f90:641,648).
  subroutine gpu_sync_contacts()
    integer(c_int) :: ierr, nc, cap
    integer(c_int), allocatable :: owner(:), partner(:)
    real(c_double), allocatable :: td(:), vr(:)
    integer :: k, a, b, m
    integer :: vec(20)
    type(real4) :: tan(20)
    ierr = sdem_check_restart_limit(gpu_h);  call gpu_check(ierr, "sdem_check_restart_limit")
    allocate(owner(1), partner(1), td(3), vr(1))
    ierr = sdem_download_contacts(gpu_h, 0, nc, owner, partner, td, vr)
    call gpu_check(ierr, "sdem_download_contacts")
    cap = max(nc, 1)
    deallocate(owner, partner, td, vr)
    allocate(owner(cap), partner(cap), td(3*cap), vr(cap))
    ierr = sdem_download_contacts(gpu_h, cap, nc, owner, partner, td, vr)
    call gpu_check(ierr, "sdem_download_contacts")
    call GPPW_CntctList%PreIteration()
    call GPPW_CntctList%RemvReleased()
    a = 1
    do while (a <= nc)          ! records come grouped by owner index
      b = a
      do while (b < nc)
        if (owner(b+1) /= owner(a)) exit
        b = b + 1
      end do
      m = b - a + 1
      do k = 1, m
        vec(k) = partner(a+k-1)
        tan(k) = real4(td(3*(a+k-2)+1), td(3*(a+k-2)+2), td(3*(a+k-2)+3), vr(a+k-1))
      end do
      call GPPW_CntctList%Add_RestartCntctlink(owner(a)+1, m, vec, tan)
      a = b + 1
    end do
  end subroutine gpu_sync_contacts

  ! the device state back into GPrtcl_* (and the contact force and torque
  ! when with_forces), for dump_visu and Write_Restart
  subroutine gpu_sync_state(with_forces)
    logical, intent(in) :: with_forces
    integer(c_int) :: ierr, n
    real(c_double), allocatable :: F(:), T(:)
    integer :: i
    ierr = sdem_download_particles(gpu_h, n, s_id, s_ptype, s_mark, s_posR, s_lin, s_linA, s_theta, s_rot, &
                                   s_rotA)
    call gpu_check(ierr, "sdem_download_particles")
    GPrtcl_list%nlocal = n
    call unpack_state(n)
    if (with_forces) then
      allocate(F(3*max(n,1)), T(3*max(n,1)))
      ierr = sdem_download_forces(gpu_h, F, T);  call gpu_check(ierr, "sdem_download_forces")
      do i = 1, n
        GPrtcl_cntctForce(i) = real3(F(3*i-2), F(3*i-1), F(3*i))
        GPrtcl_torque(i) = real3(T(3*i-2), T(3*i-1), T(3*i))
      end do
    end if
  end subroutine gpu_sync_state

  ! numCntcts(1:4) and the conservative candidates (same level, cross level)
  ! of the last step, for the log lines
  subroutine gpu_log_counters(numCntcts, consv)
    integer, intent(out) :: numCntcts(4), consv(2)
    integer(c_int) :: out(SDEM_CNT_SIZE), ierr
    ierr = sdem_counters(gpu_h, out);  call gpu_check(ierr, "sdem_counters")
    numCntcts = out(1:4)
    consv = [out(5), out(9)]
  end subroutine gpu_log_counters

  subroutine gpu_finalize()
    call sdem_destroy(gpu_h)
    gpu_h = c_null_ptr
  end subroutine gpu_finalize

end module Prtcl_GPU_Driver
