! Prtcl_GPU.f90 -- ISO_C_BINDING interfaces of include/sdem_gpu.h for the
! reference's Fortran driver (GongZheng-Justin/sDEM, Fortran 2003).
!
! Compiled with the reference's sources when it is built with -DSDEM_GPU
! (before Prtcl_DEMSystem.o) and linked with -lsdem_gpu -lcudart.  It depends
! on no module of the reference: the driver code that packs the reference's
! arrays into these calls is Prtcl_GPU_Driver.f90 (next to this file).
!
! Conventions (those of sdem_gpu.h):
!   - a handle (sdem_h*, sdem_batch*) and a device or stream address (void*,
!     the device arrays of sdem_count_contacts_noalloc) are type(c_ptr),
!     passed by value;
!   - C scalars (int, long long, double) are passed by value;
!   - every other C pointer is a Fortran array or scalar passed by reference;
!   - vector fields are real(c_double) arrays of the layouts the header
!     documents; the reference's type(real3)/type(real4) arrays have the same
!     memory layout, so c_loc of a contiguous array may be passed instead.
module Prtcl_GPU
  use iso_c_binding
  implicit none

  ! struct sdem_cfg, field for field
  type, bind(C) :: sdem_cfg
    integer(c_int) :: n_capacity, max_gid, tsize, rsize, cf_type, ct_model
    integer(c_int) :: pi_method, pri_method, cs_method, cntct_list_size
    integer(c_int) :: base_wall_id, wall_max_update_iter, periodic(3)
    integer(c_int) :: quirk_ab2_rot, max_contacts_per_particle
    real(c_double) :: dt, gravity(3), dom_min(3), dom_max(3), cs_ratio, wall_neighbor_ratio
    integer(c_int) :: n_fixed_capacity, cs_num_levels
  end type sdem_cfg

  integer(c_int), parameter :: SDEM_OK = 0, SDEM_E_ARG = 1, SDEM_E_CUDA = 2, SDEM_E_CL_FULL = 3, &
                               SDEM_E_BAD_ID = 4, SDEM_E_NCV20 = 5, SDEM_E_GRID = 6, SDEM_E_TIMEOUT = 7, &
                               SDEM_E_CAPACITY = 8, SDEM_E_NOMEM = 9, SDEM_E_UNSUPPORTED = 10
  integer(c_int), parameter :: SDEM_CNT_SIZE = 9

  type(c_ptr), save :: gpu_h = c_null_ptr

  interface
    subroutine sdem_default_cfg(cfg) bind(C, name="sdem_default_cfg")
      import :: sdem_cfg
      type(sdem_cfg), intent(out) :: cfg
    end subroutine sdem_default_cfg

    integer(c_int) function sdem_create(cfg, h) bind(C, name="sdem_create")
      import :: c_int, c_ptr, sdem_cfg
      type(sdem_cfg), intent(in) :: cfg
      type(c_ptr), intent(out) :: h
    end function sdem_create

    integer(c_int) function sdem_set_types(h, nT, radius, mass, inertia, bnry_pp, nWT, bnry_pw) &
        bind(C, name="sdem_set_types")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: nT
      real(c_double), intent(in) :: radius(*), mass(*), inertia(*), bnry_pp(*)
      integer(c_int), value :: nWT
      real(c_double), intent(in) :: bnry_pw(*)
    end function sdem_set_types

    integer(c_int) function sdem_set_walls(h, nw, wall, flags) bind(C, name="sdem_set_walls")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: nw
      real(c_double), intent(in) :: wall(*)
      integer(c_int), intent(in) :: flags(*)
    end function sdem_set_walls

    integer(c_int) function sdem_upload_particles(h, n, id, ptype, usrmark, posR, linVel, linAcc, &
        theta, rotVel, rotAcc) bind(C, name="sdem_upload_particles")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: n
      integer(c_int), intent(in) :: id(*), ptype(*), usrmark(*)
      real(c_double), intent(in) :: posR(*), linVel(*), linAcc(*), theta(*), rotVel(*), rotAcc(*)
    end function sdem_upload_particles

    integer(c_int) function sdem_upload_contacts(h, nc, owner_idx, partner_id, tandelta, velrel) &
        bind(C, name="sdem_upload_contacts")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: nc
      integer(c_int), intent(in) :: owner_idx(*), partner_id(*)
      real(c_double), intent(in) :: tandelta(*), velrel(*)
    end function sdem_upload_contacts

    integer(c_int) function sdem_step(h, nsteps) bind(C, name="sdem_step")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
    end function sdem_step

    integer(c_int) function sdem_step_async(h, nsteps) bind(C, name="sdem_step_async")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
    end function sdem_step_async

    integer(c_int) function sdem_get_stream(h, stream) bind(C, name="sdem_get_stream")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      type(c_ptr), intent(out) :: stream
    end function sdem_get_stream

    integer(c_int) function sdem_download_particles(h, n, id, ptype, usrmark, posR, linVel, linAcc, &
        theta, rotVel, rotAcc) bind(C, name="sdem_download_particles")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), intent(out) :: n
      integer(c_int), intent(out) :: id(*), ptype(*), usrmark(*)
      real(c_double), intent(out) :: posR(*), linVel(*), linAcc(*), theta(*), rotVel(*), rotAcc(*)
    end function sdem_download_particles

    integer(c_int) function sdem_download_contacts(h, cap, nc, owner_idx, partner_id, tandelta, velrel) &
        bind(C, name="sdem_download_contacts")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: cap
      integer(c_int), intent(out) :: nc
      integer(c_int), intent(out) :: owner_idx(*), partner_id(*)
      real(c_double), intent(out) :: tandelta(*), velrel(*)
    end function sdem_download_contacts

    integer(c_int) function sdem_check_restart_limit(h) bind(C, name="sdem_check_restart_limit")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function sdem_check_restart_limit

    integer(c_int) function sdem_download_forces(h, F, T) bind(C, name="sdem_download_forces")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), intent(out) :: F(*), T(*)
    end function sdem_download_forces

    integer(c_int) function sdem_set_fixed(h, nfix, id, ptype, pos) bind(C, name="sdem_set_fixed")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: nfix
      integer(c_int), intent(in) :: id(*), ptype(*)
      real(c_double), intent(in) :: pos(*)
    end function sdem_set_fixed

    integer(c_int) function sdem_counters(h, out) bind(C, name="sdem_counters")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), intent(out) :: out(*)
    end function sdem_counters

    integer(c_int) function sdem_counters_lagged(h, out) bind(C, name="sdem_counters_lagged")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), intent(out) :: out(*)
    end function sdem_counters_lagged

    integer(c_int) function sdem_snapshot_begin(h, id, ptype, usrmark, posR, linVel, linAcc, theta, &
        rotVel, rotAcc, F, T, want_contacts) bind(C, name="sdem_snapshot_begin")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int) :: id(*), ptype(*), usrmark(*)
      real(c_double) :: posR(*), linVel(*), linAcc(*), theta(*), rotVel(*), rotAcc(*), F(*), T(*)
      integer(c_int), value :: want_contacts
    end function sdem_snapshot_begin

    integer(c_int) function sdem_snapshot_end(h, n_out) bind(C, name="sdem_snapshot_end")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), intent(out) :: n_out
    end function sdem_snapshot_end

    integer(c_int) function sdem_snapshot_contacts(h, cap, nc, owner_idx, partner_id, tandelta, velrel) &
        bind(C, name="sdem_snapshot_contacts")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: cap
      integer(c_int), intent(out) :: nc
      integer(c_int), intent(out) :: owner_idx(*), partner_id(*)
      real(c_double), intent(out) :: tandelta(*), velrel(*)
    end function sdem_snapshot_contacts

    integer(c_int) function sdem_counter_sums(h, out) bind(C, name="sdem_counter_sums")
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: h
      integer(c_long_long), intent(out) :: out(*)
    end function sdem_counter_sums

    integer(c_int) function sdem_launch_count(h, n) bind(C, name="sdem_launch_count")
      import :: c_int, c_ptr, c_long_long
      type(c_ptr), value :: h
      integer(c_long_long), intent(out) :: n
    end function sdem_launch_count

    integer(c_int) function sdem_profile_begin(h, max_steps) bind(C, name="sdem_profile_begin")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: max_steps
    end function sdem_profile_begin

    integer(c_int) function sdem_profile_end(h, cap, ms, nsteps) bind(C, name="sdem_profile_end")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: cap
      real(c_double), intent(out) :: ms(*)
      integer(c_int), intent(out) :: nsteps
    end function sdem_profile_end

    type(c_ptr) function sdem_profile_phase_name(i) bind(C, name="sdem_profile_phase_name")
      import :: c_int, c_ptr
      integer(c_int), value :: i
    end function sdem_profile_phase_name

    integer(c_int) function sdem_selftest_fp64(n, seed, mismatches) bind(C, name="sdem_selftest_fp64")
      import :: c_int, c_long_long
      integer(c_long_long), value :: n, seed
      integer(c_long_long), intent(out) :: mismatches
    end function sdem_selftest_fp64

    integer(c_int) function sdem_probe_fp64_peak(iters, dfma_per_s, ms) bind(C, name="sdem_probe_fp64_peak")
      import :: c_int, c_long_long, c_double
      integer(c_long_long), value :: iters
      real(c_double), intent(out) :: dfma_per_s, ms
    end function sdem_probe_fp64_peak

    integer(c_int) function sdem_set_launch(h, pipeline_chunks, force_blocks_per_sm, first_chunk_percent) &
        bind(C, name="sdem_set_launch")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: pipeline_chunks, force_blocks_per_sm, first_chunk_percent
    end function sdem_set_launch

    integer(c_int) function sdem_get_launch(h, pipeline_chunks, force_blocks_per_sm, first_chunk_percent) &
        bind(C, name="sdem_get_launch")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), intent(out) :: pipeline_chunks, force_blocks_per_sm, first_chunk_percent
    end function sdem_get_launch

    integer(c_int) function sdem_count_contacts_noalloc(cfg, max_radius, n, d_posR, d_counts, stream) &
        bind(C, name="sdem_count_contacts_noalloc")
      import :: c_int, c_ptr, c_double, sdem_cfg
      type(sdem_cfg), intent(in) :: cfg
      real(c_double), value :: max_radius
      integer(c_int), value :: n
      type(c_ptr), value :: d_posR, d_counts, stream
    end function sdem_count_contacts_noalloc

    type(c_ptr) function sdem_last_error(h) bind(C, name="sdem_last_error")
      import :: c_ptr
      type(c_ptr), value :: h
    end function sdem_last_error

    subroutine sdem_destroy(h) bind(C, name="sdem_destroy")
      import :: c_ptr
      type(c_ptr), value :: h
    end subroutine sdem_destroy

    integer(c_int) function sdem_batch_create(n, members, b) bind(C, name="sdem_batch_create")
      import :: c_int, c_ptr
      integer(c_int), value :: n
      type(c_ptr), intent(in) :: members(*)
      type(c_ptr), intent(out) :: b
    end function sdem_batch_create

    integer(c_int) function sdem_batch_create_grouped(n, members, group_size, b) &
        bind(C, name="sdem_batch_create_grouped")
      import :: c_int, c_ptr
      integer(c_int), value :: n
      type(c_ptr), intent(in) :: members(*)
      integer(c_int), value :: group_size
      type(c_ptr), intent(out) :: b
    end function sdem_batch_create_grouped

    integer(c_int) function sdem_batch_step_async(b, nsteps) bind(C, name="sdem_batch_step_async")
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int), value :: nsteps
    end function sdem_batch_step_async

    integer(c_int) function sdem_batch_sync(b) bind(C, name="sdem_batch_sync")
      import :: c_int, c_ptr
      type(c_ptr), value :: b
    end function sdem_batch_sync

    integer(c_int) function sdem_batch_step(b, nsteps) bind(C, name="sdem_batch_step")
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int), value :: nsteps
    end function sdem_batch_step

    type(c_ptr) function sdem_batch_last_error(b) bind(C, name="sdem_batch_last_error")
      import :: c_ptr
      type(c_ptr), value :: b
    end function sdem_batch_last_error

    subroutine sdem_batch_destroy(b) bind(C, name="sdem_batch_destroy")
      import :: c_ptr
      type(c_ptr), value :: b
    end subroutine sdem_batch_destroy
  end interface

contains

  ! The message of a failed call as a Fortran string ("" when none).
  function sdem_message(h) result(msg)
    type(c_ptr), value :: h
    character(len=:), allocatable :: msg
    character(kind=c_char), pointer :: c(:)
    type(c_ptr) :: p
    integer :: k
    p = sdem_last_error(h)
    msg = ""
    if (.not. c_associated(p)) return
    call c_f_pointer(p, c, [1024])
    do k = 1, 1024
      if (c(k) == c_null_char) exit
      msg = msg // c(k)
    end do
  end function sdem_message

end module Prtcl_GPU
