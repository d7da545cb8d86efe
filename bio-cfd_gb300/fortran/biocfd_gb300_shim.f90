! ISO_C_BINDING shim: the reference's hot-path module subroutines, same
! names and dummy arguments, forwarding to libbiocfd_gb300.so.
!
! Link order: compile this file instead of src/NavierStokes.f90,
! src/PcorVcor.F90, src/BoundaryConditions.f90, src/Forcing.f90 and
! src/CoefficientMatrix.f90, and instead of the hot-path routines of
! src/Search.F90 / src/FineInterp_bound.f90 / src/CoarseInterp.f90; add the
! component `integer(int64) :: bcfd = 0` to Block_t (src/Blocks.f90) so that
! each block carries its device handle.  app/main.F90 relinks unchanged.
!
! Data ownership: the device arrays are authoritative.  Each routine here
! registers a block on first sight (uploading grids, surface, fields and
! tags), calls the C entry point and, when bcfd_host_mirror is .true. (the
! default), copies the fields back so that host-side code (output, restart,
! kinematics) sees current values.  Setting bcfd_host_mirror = .false. keeps
! the data on the GPU between calls; call bcfd_pull(blk) before host reads.
module biocfd_gb300_c
  use, intrinsic :: iso_c_binding
  implicit none
  interface
    integer(c_int) function bcfd_init(device) bind(C, name="bcfd_init")
      import :: c_int
      integer(c_int), value :: device
    end function
    integer(c_int) function bcfd_block_create(nx, ny, nz, x1, y1, z1, dx, dy, dz, h) &
         bind(C, name="bcfd_block_create")
      import :: c_int, c_int64_t, c_double
      integer(c_int64_t), value :: nx, ny, nz
      real(c_double), intent(in) :: x1(*), y1(*), z1(*), dx(*), dy(*), dz(*)
      integer(c_int64_t), intent(out) :: h
    end function
    integer(c_int) function bcfd_block_set_scalars(h, dx, dy, dz, omega) &
         bind(C, name="bcfd_block_set_scalars")
      import :: c_int, c_int64_t, c_double
      integer(c_int64_t), value :: h
      real(c_double), value :: dx, dy, dz, omega
    end function
    integer(c_int) function bcfd_block_set_search_box(h, i0, i1, j0, j1, k0, k1) &
         bind(C, name="bcfd_block_set_search_box")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h, i0, i1, j0, j1, k0, k1
    end function
    integer(c_int) function bcfd_block_set_surface(h, ne, nn, e1, e2, e3, sid, x, y, z) &
         bind(C, name="bcfd_block_set_surface")
      import :: c_int, c_int64_t, c_double
      integer(c_int64_t), value :: h, ne, nn
      integer(c_int64_t), intent(in) :: e1(*), e2(*), e3(*), sid(*)
      real(c_double), intent(in) :: x(*), y(*), z(*)
    end function
    integer(c_int) function bcfd_block_set_nodes(h, x, y, z) bind(C, name="bcfd_block_set_nodes")
      import :: c_int, c_int64_t, c_double
      integer(c_int64_t), value :: h
      real(c_double), intent(in) :: x(*), y(*), z(*)
    end function
    integer(c_int) function bcfd_block_set_kinematics(h, kin) bind(C, name="bcfd_block_set_kinematics")
      import :: c_int, c_int64_t, c_double
      integer(c_int64_t), value :: h
      real(c_double), intent(in) :: kin(11)
    end function
    integer(c_int) function bcfd_block_set_flags(h, mc, tag) bind(C, name="bcfd_block_set_flags")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h, mc, tag
    end function
    integer(c_int) function bcfd_block_upload_fields(h, u, v, w, p, ut, vt, wt) &
         bind(C, name="bcfd_block_upload_fields")
      import :: c_int, c_int64_t, c_double
      integer(c_int64_t), value :: h
      real(c_double), intent(in) :: u(*), v(*), w(*), p(*), ut(*), vt(*), wt(*)
    end function
    integer(c_int) function bcfd_block_download_fields(h, u, v, w, p, ut, vt, wt) &
         bind(C, name="bcfd_block_download_fields")
      import :: c_int, c_int64_t, c_double
      integer(c_int64_t), value :: h
      real(c_double), intent(out) :: u(*), v(*), w(*), p(*), ut(*), vt(*), wt(*)
    end function
    integer(c_int) function bcfd_block_upload_tags(h, cell, cell2, nid, celln, cellpr) &
         bind(C, name="bcfd_block_upload_tags")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
      integer(c_int64_t), intent(in) :: cell(*), cell2(*), nid(*), celln(*), cellpr(*)
    end function
    integer(c_int) function bcfd_block_get_counts(h, c) bind(C, name="bcfd_block_get_counts")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
      integer(c_int64_t), intent(out) :: c(6)
    end function
    integer(c_int) function bcfd_block_get_sor_stats(h, n, d2, dss) bind(C, name="bcfd_block_get_sor_stats")
      import :: c_int, c_int64_t, c_double
      integer(c_int64_t), value :: h
      integer(c_int64_t), intent(out) :: n
      real(c_double), intent(out) :: d2, dss
    end function
    integer(c_int) function bcfd_h(h) bind(C, name="bcfd_non_uni_coeff")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
    integer(c_int) function bcfd_coefficient_matrix(h, is_coarse) bind(C, name="bcfd_coefficient_matrix")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
      integer(c_int), value :: is_coarse
    end function
    integer(c_int) function bcfd_ns_momentum_2order(h, dt, re) bind(C, name="bcfd_ns_momentum_2order")
      import :: c_int, c_int64_t, c_double
      integer(c_int64_t), value :: h
      real(c_double), value :: dt, re
    end function
    integer(c_int) function bcfd_velocity_bc(h, dt, uc) bind(C, name="bcfd_velocity_bc")
      import :: c_int, c_int64_t, c_double
      integer(c_int64_t), value :: h
      real(c_double), value :: dt, uc
    end function
    integer(c_int) function bcfd_by_handle(h) bind(C, name="bcfd_solid_cell_bc")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
    integer(c_int) function bcfd_poisson_solver(itmax, epsi, ita, dt, totime, uc, total, s, f, st) &
         bind(C, name="bcfd_poisson_solver")
      import :: c_int, c_int64_t, c_double
      integer(c_int64_t), value :: itmax, ita
      real(c_double), value :: epsi, dt, totime, uc
      real(c_double), intent(inout) :: total
      integer(c_int), value :: s, f, st
    end function
  end interface

  ! one-argument routines share this C signature: int f(bcfd_handle)
  abstract interface
    integer(c_int) function h_routine(h) bind(C)
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
  end interface
end module biocfd_gb300_c

module biocfd_gb300_glue
  use, intrinsic :: iso_c_binding
  use, intrinsic :: iso_fortran_env, only: int64, dp => real64
  use biocfd_gb300_c
  use biocfd_block_type, only: Block_t
  implicit none
  logical :: bcfd_host_mirror = .true.
  logical, private :: ready = .false.
contains
  subroutine bcfd_check(st, what)
    integer(c_int), intent(in) :: st
    character(*), intent(in) :: what
    if (st /= 0) then
      write(*, '(A,A,A,I0)') 'biocfd_gb300: ', what, ' failed with status ', st
      error stop 1
    end if
  end subroutine

  ! register a block on first sight: grids, scalars, surface, tags, fields
  subroutine bcfd_ensure(blk)
    type(Block_t), intent(inout) :: blk
    integer(c_int64_t) :: h
    if (.not. ready) then
      call bcfd_check(bcfd_init(0_c_int), 'bcfd_init')
      ready = .true.
    end if
    if (blk%bcfd /= 0) return
    call bcfd_check(bcfd_block_create(blk%nx, blk%ny, blk%nz, blk%x1, blk%y1, blk%z1, &
         blk%deltax, blk%deltay, blk%deltaz, h), 'block_create')
    blk%bcfd = h
    call bcfd_check(bcfd_block_set_scalars(h, blk%dx, blk%dy, blk%dz, blk%omega), 'set_scalars')
    call bcfd_check(bcfd_block_set_search_box(h, blk%i_startSearch, blk%i_endSearch, &
         blk%j_startSearch, blk%j_endSearch, blk%k_startSearch, blk%k_endSearch), 'set_search_box')
    if (allocated(blk%ibElP1)) then
      call bcfd_check(bcfd_block_set_surface(h, blk%ibElems, blk%ibNodes, blk%ibElP1, blk%ibElP2, &
           blk%ibElP3, blk%ibSurfId, blk%xnode1, blk%ynode1, blk%znode1), 'set_surface')
    end if
    if (allocated(blk%cell2)) then
      call bcfd_check(bcfd_block_upload_tags(h, blk%cell, blk%cell2, blk%nodeIdTag, blk%cell_n, &
           blk%cell_pr), 'upload_tags')
    end if
    call bcfd_push(blk)
  end subroutine

  subroutine bcfd_push(blk)
    type(Block_t), intent(inout) :: blk
    real(dp) :: kin(11)
    kin = [blk%xdot, blk%ydot, blk%yddot, blk%thetaDot1, blk%thetaDDot1, blk%thetaDot2, &
           blk%thetaDDot2, blk%alphaDot, blk%piv_x, blk%piv_y, blk%piv_z]
    call bcfd_check(bcfd_block_set_kinematics(blk%bcfd, kin), 'set_kinematics')
    call bcfd_check(bcfd_block_set_flags(blk%bcfd, blk%move_check, int(blk%blk_mv_tag, int64)), 'set_flags')
    call bcfd_check(bcfd_block_upload_fields(blk%bcfd, blk%u, blk%v, blk%w, blk%p, blk%ut, blk%vt, &
         blk%wt), 'upload_fields')
  end subroutine

  subroutine bcfd_pull(blk)
    type(Block_t), intent(inout) :: blk
    integer(c_int64_t) :: c(6)
    call bcfd_check(bcfd_block_download_fields(blk%bcfd, blk%u, blk%v, blk%w, blk%p, blk%ut, blk%vt, &
         blk%wt), 'download_fields')
    call bcfd_check(bcfd_block_get_counts(blk%bcfd, c), 'get_counts')
    blk%ibCellCount = c(1); blk%solidCellCount = c(2); blk%fluidCellCount = c(3)
    blk%redCellCount = c(4); blk%blackCellCount = c(5); blk%TSCellCount = c(6)
    call bcfd_check(bcfd_block_get_sor_stats(blk%bcfd, blk%nIterPcor, blk%derr2, blk%derrStdSt), 'sor_stats')
  end subroutine

  ! call a one-handle routine by name and keep the host mirror current
  subroutine bcfd_call(blk, fn, what)
    type(Block_t), intent(inout) :: blk
    procedure(h_routine) :: fn
    character(*), intent(in) :: what
    call bcfd_ensure(blk)
    call bcfd_check(fn(blk%bcfd), what)
    if (bcfd_host_mirror) call bcfd_pull(blk)
  end subroutine
end module biocfd_gb300_glue

! --------------------------------------------------------------------------
! drop-in replacements keeping the reference's module and routine names
! --------------------------------------------------------------------------
module biocfd_navier_stokes
  use, intrinsic :: iso_fortran_env, only: dp => real64
  use biocfd_block_type, only: Block_t
  use biocfd_gb300_c
  use biocfd_gb300_glue
  implicit none
  private
  public :: non_uni_coeff, nsMomentum2order
contains
  subroutine non_uni_coeff(blk)                    ! src/NavierStokes.f90:13-250
    type(Block_t), intent(inout) :: blk
    call bcfd_ensure(blk)
    call bcfd_check(bcfd_h(blk%bcfd), 'non_uni_coeff')
  end subroutine
  subroutine nsMomentum2order(blk, deltat, re)     ! src/NavierStokes.f90:252-912
    type(Block_t), intent(inout) :: blk
    real(dp), intent(in) :: deltat, re
    call bcfd_ensure(blk)
    if (bcfd_host_mirror) call bcfd_push(blk)
    call bcfd_check(bcfd_ns_momentum_2order(blk%bcfd, deltat, re), 'nsMomentum2order')
    if (bcfd_host_mirror) call bcfd_pull(blk)
  end subroutine
end module biocfd_navier_stokes

module biocfd_boundary_conditions
  use, intrinsic :: iso_fortran_env, only: dp => real64
  use biocfd_block_type, only: Block_t
  use biocfd_gb300_c
  use biocfd_gb300_glue
  implicit none
  private
  public :: velocityBC, solidCellBC, solidCellBC_move
  interface
    integer(c_int) function c_solid_move(h) bind(C, name="bcfd_solid_cell_bc_move")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
  end interface
contains
  subroutine velocityBC(blk, deltat, uc)            ! src/BoundaryConditions.f90:11-74
    type(Block_t), intent(inout) :: blk
    real(dp), intent(in) :: deltat, uc
    call bcfd_ensure(blk)
    call bcfd_check(bcfd_velocity_bc(blk%bcfd, deltat, uc), 'velocityBC')
    if (bcfd_host_mirror) call bcfd_pull(blk)
  end subroutine
  subroutine solidCellBC(blk)                       ! :76-92
    type(Block_t), intent(inout) :: blk
    call bcfd_call(blk, bcfd_by_handle, 'solidCellBC')
  end subroutine
  subroutine solidCellBC_move(blk)                  ! :94-115
    type(Block_t), intent(inout) :: blk
    call bcfd_call(blk, c_solid_move, 'solidCellBC_move')
  end subroutine
end module biocfd_boundary_conditions

module biocfd_pcor_vcor
  use, intrinsic :: iso_fortran_env, only: dp => real64, int64
  use global, only: block
  use biocfd_block_type, only: Block_t
  use biocfd_gb300_c
  use biocfd_gb300_glue
  implicit none
  private
  public :: poissonSolver, updateVelocity_newv
  interface
    integer(c_int) function c_update_newv(h) bind(C, name="bcfd_update_velocity_newv")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
  end interface
contains
  subroutine poissonSolver(pcItaMax, epsi, ita, deltat, totime, uc, totalTime, start, finish, step)
    ! src/PcorVcor.F90:22-220 over all registered blocks (registration order =
    ! block number, block 1 coarse)
    integer(int64), intent(in) :: pcItaMax, ita
    real(dp), intent(in) :: epsi, deltat, totime, uc
    real(dp), intent(inout) :: totalTime
    integer, intent(in) :: start, finish, step
    integer :: g
    do g = start, finish, step
      call bcfd_ensure(block(g))
      if (bcfd_host_mirror) call bcfd_push(block(g))
    end do
    call bcfd_check(bcfd_poisson_solver(pcItaMax, epsi, ita, deltat, totime, uc, totalTime, &
         int(start, c_int), int(finish, c_int), int(step, c_int)), 'poissonSolver')
    if (bcfd_host_mirror) then
      do g = start, finish, step
        call bcfd_pull(block(g))
      end do
    end if
  end subroutine
  subroutine updateVelocity_newv(blk)               ! src/PcorVcor.F90:379-397
    type(Block_t), intent(inout) :: blk
    call bcfd_call(blk, c_update_newv, 'updateVelocity_newv')
  end subroutine
end module biocfd_pcor_vcor

module biocfd_forcing
  use biocfd_block_type, only: Block_t
  use biocfd_gb300_c
  use biocfd_gb300_glue
  implicit none
  private
  public :: velocityForcing1, pressureForcing1, velocityForcingField, pressureForcingField, &
            velocityForcingGhost, pressureForcingGhost
  interface
    integer(c_int) function c_vf1(h) bind(C, name="bcfd_velocity_forcing1")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
    integer(c_int) function c_pf1(h) bind(C, name="bcfd_pressure_forcing1")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
    integer(c_int) function c_vff(h) bind(C, name="bcfd_velocity_forcing_field")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
    integer(c_int) function c_pff(h) bind(C, name="bcfd_pressure_forcing_field")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
    integer(c_int) function c_vfg(h) bind(C, name="bcfd_velocity_forcing_ghost")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
    integer(c_int) function c_pfg(h) bind(C, name="bcfd_pressure_forcing_ghost")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
  end interface
contains
  subroutine velocityForcing1(blk)                  ! src/Forcing.f90:92-360
    type(Block_t), intent(inout) :: blk
    call bcfd_call(blk, c_vf1, 'velocityForcing1')
  end subroutine
  subroutine pressureForcing1(blk)                  ! src/Forcing.f90:14-90
    type(Block_t), intent(inout) :: blk
    call bcfd_call(blk, c_pf1, 'pressureForcing1')
  end subroutine
  subroutine velocityForcingField(blk)              ! src/Forcing.f90:813-1075
    type(Block_t), intent(inout) :: blk
    call bcfd_call(blk, c_vff, 'velocityForcingField')
  end subroutine
  subroutine pressureForcingField(blk)              ! src/Forcing.f90:737-811
    type(Block_t), intent(inout) :: blk
    call bcfd_call(blk, c_pff, 'pressureForcingField')
  end subroutine
  subroutine velocityForcingGhost(blk)              ! src/Forcing.f90:450-734
    type(Block_t), intent(inout) :: blk
    call bcfd_call(blk, c_vfg, 'velocityForcingGhost')
  end subroutine
  subroutine pressureForcingGhost(blk)              ! src/Forcing.f90:362-448
    type(Block_t), intent(inout) :: blk
    call bcfd_call(blk, c_pfg, 'pressureForcingGhost')
  end subroutine
end module biocfd_forcing

! Search routines of app/main.F90:169-263.  The fine-block move runs whole in
! block_move_check (bcfd_block_move_stage); change_block_coords,
! change_block_coords_interfaces, change_block_interface and
! cellCount_solid_coarse_mv then only refresh the host mirrors.
module biocfd_search
  use, intrinsic :: iso_fortran_env, only: dp => real64, int64
  use global, only: block
  use biocfd_block_type, only: Block_t
  use biocfd_gb300_c
  use biocfd_gb300_glue
  implicit none
  private
  public :: computeSurfaceVariables, computeSurfaceNorm, block_move_check, change_block_coords, &
            change_block_coords_interfaces, change_block_interface, fine_block_cell, &
            cellCount_solid_coarse_mv, tagging_th_move, selectiveRetagging_th, cellCount_solid, &
            computeNormDistance, findTScells
  interface
    integer(c_int) function c_csv(h, phase, piv, ita, dt, dxmin, freq, totime) &
         bind(C, name="bcfd_compute_surface_variables")
      import :: c_int, c_int64_t, c_double
      integer(c_int64_t), value :: h, ita
      real(c_double), value :: phase, piv, dt, dxmin, freq, totime
    end function
    integer(c_int) function c_csn(h, inor) bind(C, name="bcfd_compute_surface_norm")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h, inor
    end function
    integer(c_int) function c_move(moved) bind(C, name="bcfd_block_move_stage")
      import :: c_int, c_int64_t
      integer(c_int64_t), intent(out) :: moved
    end function
    integer(c_int) function c_tag_move(h) bind(C, name="bcfd_tagging_th_move")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
    integer(c_int) function c_retag(h) bind(C, name="bcfd_selective_retagging_th")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
    integer(c_int) function c_count(h) bind(C, name="bcfd_cellcount_solid")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
    integer(c_int) function c_nd(h) bind(C, name="bcfd_compute_norm_distance")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
    integer(c_int) function c_ts(h) bind(C, name="bcfd_find_ts_cells")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
    integer(c_int) function c_read(h, name, out, n, written) bind(C, name="bcfd_block_read")
      import :: c_int, c_int64_t, c_char, c_ptr
      integer(c_int64_t), value :: h, n
      character(kind=c_char), intent(in) :: name(*)
      type(c_ptr), value :: out
      integer(c_int64_t), intent(out) :: written
    end function
  end interface
contains
  subroutine computeSurfaceVariables(blk, g, phase_angle, piv_pt, ita, deltat, dxmin, freq, re, totime)
    ! src/Search.F90:126-208 (re is not used by the routine)
    type(Block_t), intent(inout) :: blk
    integer(int64), intent(in) :: g, ita
    real(dp), intent(in) :: phase_angle, piv_pt, deltat, dxmin, freq, re, totime
    call bcfd_ensure(blk)
    call bcfd_check(bcfd_block_set_flags(blk%bcfd, -1_c_int64_t, int(blk%blk_mv_tag, c_int64_t)), 'set_flags')
    call bcfd_check(c_csv(blk%bcfd, phase_angle, piv_pt, ita, deltat, dxmin, freq, totime), &
         'computeSurfaceVariables')
  end subroutine
  subroutine computeSurfaceNorm(blk, inor)          ! src/Search.F90:210-258
    type(Block_t), intent(inout) :: blk
    integer(int64), intent(in) :: inor
    call bcfd_ensure(blk)
    call bcfd_check(c_csn(blk%bcfd, inor), 'computeSurfaceNorm')
  end subroutine
  subroutine block_move_check(coarse_flcnt_check)   ! src/Search.F90:997-1203, with :1208-1461
    integer(int64), intent(inout) :: coarse_flcnt_check
    integer(c_int64_t) :: moved, w
    integer(int64), target :: f(1)
    integer :: g
    call bcfd_check(c_move(moved), 'block_move_check')
    coarse_flcnt_check = moved
    ! the switches a moved block carries into the re-tagging (Block_t copies)
    do g = 2, size(block)
      if (block(g)%bcfd == 0) cycle
      call bcfd_check(c_read(block(g)%bcfd, 'move_check'//char(0), c_loc(f), 1_c_int64_t, w), 'read')
      block(g)%move_check = f(1)
      call bcfd_check(c_read(block(g)%bcfd, 'blk_mv_tag'//char(0), c_loc(f), 1_c_int64_t, w), 'read')
      block(g)%blk_mv_tag = real(f(1), dp)
    end do
  end subroutine
  subroutine change_block_coords(blk)               ! src/Search.F90:1208-1264 (done in block_move_check)
    type(Block_t), intent(inout), target :: blk
    integer(c_int64_t) :: w
    if (blk%bcfd == 0 .or. blk%move_check /= 1) return
    call bcfd_check(c_read(blk%bcfd, 'x1'//char(0), c_loc(blk%x1), size(blk%x1, kind=c_int64_t), w), 'x1')
    call bcfd_check(c_read(blk%bcfd, 'y1'//char(0), c_loc(blk%y1), size(blk%y1, kind=c_int64_t), w), 'y1')
    call bcfd_check(c_read(blk%bcfd, 'z1'//char(0), c_loc(blk%z1), size(blk%z1, kind=c_int64_t), w), 'z1')
  end subroutine
  subroutine change_block_coords_interfaces(intf, blk)  ! :1269-1370 (done in block_move_check)
    class(*), intent(inout) :: intf
    type(Block_t), intent(inout) :: blk
    if (blk%bcfd /= 0 .and. blk%move_check == 1 .and. bcfd_host_mirror) call bcfd_pull(blk)
  end subroutine
  subroutine change_block_interface(intf, a, b)    ! :1372-1461 (done in block_move_check)
    class(*), intent(inout) :: intf
    type(Block_t), intent(inout) :: a, b
  end subroutine
  subroutine fine_block_cell                       ! :863-914 (done in block_move_check)
  end subroutine
  subroutine cellCount_solid_coarse_mv(coarse_flcnt_check)  ! :916-995 (done in block_move_check)
    integer(int64), intent(inout) :: coarse_flcnt_check
    coarse_flcnt_check = 0
  end subroutine
  subroutine tagging_th_move(blk, id)               ! src/Search.F90:415-432
    type(Block_t), intent(inout) :: blk
    integer(int64), intent(in) :: id
    call bcfd_call(blk, c_tag_move, 'tagging_th_move')
  end subroutine
  subroutine selectiveRetagging_th(blk)             ! src/Search.F90:520-651
    type(Block_t), intent(inout) :: blk
    call bcfd_call(blk, c_retag, 'selectiveRetagging_th')
  end subroutine
  subroutine cellCount_solid(blk, g)                ! src/Search.F90:653-741
    type(Block_t), intent(inout) :: blk
    integer(int64), intent(in) :: g
    ! main.F90 has cleared blk_mv_tag on the host by now
    call bcfd_ensure(blk)
    call bcfd_check(bcfd_block_set_flags(blk%bcfd, -1_c_int64_t, int(blk%blk_mv_tag, c_int64_t)), 'set_flags')
    call bcfd_call(blk, c_count, 'cellCount_solid')
  end subroutine
  subroutine computeNormDistance(blk)               ! src/Search.F90:743-861
    type(Block_t), intent(inout) :: blk
    ! main.F90 has cleared move_check on the host by now
    call bcfd_ensure(blk)
    call bcfd_check(bcfd_block_set_flags(blk%bcfd, blk%move_check, -1_c_int64_t), 'set_flags')
    call bcfd_call(blk, c_nd, 'computeNormDistance')
  end subroutine
  subroutine findTScells(blk)                       ! src/Search.F90:434-518
    type(Block_t), intent(inout) :: blk
    call bcfd_call(blk, c_ts, 'findTScells')
  end subroutine
end module biocfd_search
