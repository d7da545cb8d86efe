! ISO_C_BINDING shim: the reference's hot-path module subroutines, same
! names and dummy arguments, forwarding to libbiocfd_gb300.so.
!
! Link order: compile this file instead of src/NavierStokes.f90,
! src/PcorVcor.F90, src/BoundaryConditions.f90, src/Forcing.f90 and
! src/CoefficientMatrix.f90, and instead of the hot-path routines of
! src/Search.F90 / src/FineInterp_bound.f90 / src/CoarseInterp.f90; add the
! component `integer(int64) :: bcfd = 0` to Block_t (src/Blocks.f90) so that
! each block carries its device handle.  app/main.F90 relinks unchanged: every
! name it imports from biocfd_search, biocfd_pcor_vcor,
! biocfd_boundary_conditions, biocfd_coefficient_matrix,
! biocfd_navier_stokes and biocfd_forcing is public here.
!
! Registration: the first call of any routine here registers every block of
! `block` in block-number order (the library's block 1 is the coarse block)
! with its grids, scalars, search box, surface, tags, kinematics and fields,
! then every interface of `intfr` (the boxes read by readBlockInterface).  A
! surface is registered with the placed nodes xnode1 when they exist, else
! with the body-frame nodes xnode (findDistnode runs before
! shiftSurfaceNodesInitial allocates xnode1).
!
! Data ownership: the device arrays are authoritative.  When bcfd_host_mirror
! is .true. (the default) each routine uploads the block's fields before its
! C call and downloads them after it, so host-side code (initial and restart
! conditions, output, kinematics) and the device stay in step.  Setting
! bcfd_host_mirror = .false. keeps the data on the GPU between calls; call
! bcfd_push(blk) after host writes and bcfd_pull(blk) before host reads.
! Kinematic scalars and the body's nodes belong to the library once
! registered (computeSurfaceVariables runs there); the routines that change
! them copy them back to the Block_t members.
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
    integer(c_int) function bcfd_block_download_tags(h, cell, cell2, nid, celln, cellpr) &
         bind(C, name="bcfd_block_download_tags")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
      integer(c_int64_t), intent(out) :: cell(*), cell2(*), nid(*), celln(*), cellpr(*)
    end function
    integer(c_int) function bcfd_block_read(h, name, out, n, written) bind(C, name="bcfd_block_read")
      import :: c_int, c_int64_t, c_char, c_ptr
      integer(c_int64_t), value :: h, n
      character(kind=c_char), intent(in) :: name(*)
      type(c_ptr), value :: out
      integer(c_int64_t), intent(out) :: written
    end function
    integer(c_int) function bcfd_block_set_body_motion(h, p) bind(C, name="bcfd_block_set_body_motion")
      import :: c_int, c_int64_t, c_double
      integer(c_int64_t), value :: h
      real(c_double), intent(in) :: p(6)
    end function
    integer(c_int) function bcfd_interface_create(a, b, a_msh, b_msh, box, h) &
         bind(C, name="bcfd_interface_create")
      import :: c_int, c_int64_t, c_double
      integer(c_int64_t), value :: a, b, a_msh, b_msh
      real(c_double), intent(in) :: box(6)
      integer(c_int64_t), intent(out) :: h
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
  use global, only: block, intfr
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

  ! first call: the library, every block in block-number order, every interface
  subroutine bcfd_ensure(blk)
    type(Block_t), intent(inout) :: blk
    integer :: g
    integer(c_int64_t) :: hi
    real(c_double) :: box(6)
    if (.not. ready) then
      call bcfd_check(bcfd_init(0_c_int), 'bcfd_init')
      ready = .true.
      do g = 1, size(block)
        call bcfd_register(block(g))
      end do
      if (allocated(intfr)) then
        do g = 1, size(intfr)
          box = [intfr(g)%xintf_start, intfr(g)%xintf_end, intfr(g)%yintf_start, &
                 intfr(g)%yintf_end, intfr(g)%zintf_start, intfr(g)%zintf_end]
          call bcfd_check(bcfd_interface_create(block(intfr(g)%a_blk)%bcfd, &
               block(intfr(g)%b_blk)%bcfd, intfr(g)%a_msh, intfr(g)%b_msh, box, hi), &
               'interface_create')
        end do
      end if
    end if
    if (blk%bcfd == 0) call bcfd_register(blk)
  end subroutine

  ! one block: grids, scalars, search box, surface, tags, kinematics, fields
  subroutine bcfd_register(blk)
    type(Block_t), intent(inout) :: blk
    integer(c_int64_t) :: h
    real(dp) :: kin(11)
    if (blk%bcfd /= 0) return
    call bcfd_check(bcfd_block_create(blk%nx, blk%ny, blk%nz, blk%x1, blk%y1, blk%z1, &
         blk%deltax, blk%deltay, blk%deltaz, h), 'block_create')
    blk%bcfd = h
    call bcfd_check(bcfd_block_set_scalars(h, blk%dx, blk%dy, blk%dz, blk%omega), 'set_scalars')
    call bcfd_check(bcfd_block_set_search_box(h, blk%i_startSearch, blk%i_endSearch, &
         blk%j_startSearch, blk%j_endSearch, blk%k_startSearch, blk%k_endSearch), 'set_search_box')
    if (allocated(blk%ibElP1)) then
      if (allocated(blk%xnode1)) then
        call bcfd_check(bcfd_block_set_surface(h, blk%ibElems, blk%ibNodes, blk%ibElP1, blk%ibElP2, &
             blk%ibElP3, blk%ibSurfId, blk%xnode1, blk%ynode1, blk%znode1), 'set_surface')
      else
        call bcfd_check(bcfd_block_set_surface(h, blk%ibElems, blk%ibNodes, blk%ibElP1, blk%ibElP2, &
             blk%ibElP3, blk%ibSurfId, blk%xnode, blk%ynode, blk%znode), 'set_surface')
      end if
    end if
    if (allocated(blk%cell2)) then
      call bcfd_check(bcfd_block_upload_tags(h, blk%cell, blk%cell2, blk%nodeIdTag, blk%cell_n, &
           blk%cell_pr), 'upload_tags')
    end if
    kin = [blk%xdot, blk%ydot, blk%yddot, blk%thetaDot1, blk%thetaDDot1, blk%thetaDot2, &
           blk%thetaDDot2, blk%alphaDot, blk%piv_x, blk%piv_y, blk%piv_z]
    call bcfd_check(bcfd_block_set_kinematics(h, kin), 'set_kinematics')
    call bcfd_check(bcfd_block_set_flags(h, blk%move_check, int(blk%blk_mv_tag, int64)), 'set_flags')
    call bcfd_push(blk)
  end subroutine

  ! host fields -> device
  subroutine bcfd_push(blk)
    type(Block_t), intent(inout) :: blk
    call bcfd_check(bcfd_block_upload_fields(blk%bcfd, blk%u, blk%v, blk%w, blk%p, blk%ut, blk%vt, &
         blk%wt), 'upload_fields')
  end subroutine

  ! device fields, counts and Poisson statistics -> host
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
    if (bcfd_host_mirror) call bcfd_push(blk)
    call bcfd_check(fn(blk%bcfd), what)
    if (bcfd_host_mirror) call bcfd_pull(blk)
  end subroutine

  ! one real array of the block, read back by name (bcfd_block_read)
  subroutine bcfd_read_real(h, name, arr)
    integer(c_int64_t), intent(in) :: h
    character(*), intent(in) :: name
    real(dp), intent(inout), target, contiguous :: arr(:)
    integer(c_int64_t) :: w
    call bcfd_check(bcfd_block_read(h, name//char(0), c_loc(arr), size(arr, kind=c_int64_t), w), name)
  end subroutine

  ! kinematic scalars and placed nodes of a moving body -> Block_t members
  subroutine bcfd_pull_motion(blk)
    type(Block_t), intent(inout) :: blk
    real(dp) :: k(1)
    integer(c_int64_t) :: h
    h = blk%bcfd
    if (.not. allocated(blk%xnode1)) then
      allocate(blk%xnode1(blk%ibNodes), blk%ynode1(blk%ibNodes), blk%znode1(blk%ibNodes))
    end if
    call bcfd_read_real(h, 'xnode1', blk%xnode1)
    call bcfd_read_real(h, 'ynode1', blk%ynode1)
    call bcfd_read_real(h, 'znode1', blk%znode1)
    call bcfd_read_real(h, 'xdot', k); blk%xdot = k(1)
    call bcfd_read_real(h, 'ydot', k); blk%ydot = k(1)
    call bcfd_read_real(h, 'yddot', k); blk%yddot = k(1)
    call bcfd_read_real(h, 'thetaDot1', k); blk%thetaDot1 = k(1)
    call bcfd_read_real(h, 'thetaDDot1', k); blk%thetaDDot1 = k(1)
    call bcfd_read_real(h, 'thetaDot2', k); blk%thetaDot2 = k(1)
    call bcfd_read_real(h, 'thetaDDot2', k); blk%thetaDDot2 = k(1)
    call bcfd_read_real(h, 'piv_x', k); blk%piv_x = k(1)
    call bcfd_read_real(h, 'piv_y', k); blk%piv_y = k(1)
    call bcfd_read_real(h, 'piv_z', k); blk%piv_z = k(1)
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
    if (bcfd_host_mirror) call bcfd_push(blk)
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
  public :: findDistnode, shiftSurfaceNodesInitial, computeSurfaceVariables, computeSurfaceNorm, &
            tagging_th, block_move_check, change_block_coords, change_block_coords_interfaces, &
            change_block_interface, fine_block_cell, cellCount_solid_coarse, cellCount_solid_coarse_mv, &
            tagging_th_move, selectiveRetagging_th, cellCount_solid, computeNormDistance, findTScells
  ! the coarse cells under the fine blocks are marked (set-up call of
  ! fine_block_cell, or a fine-block move inside block_move_check)
  logical :: marks_current = .false.
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
    integer(c_int) function c_ssni(h, aoa, piv, ita, dt, dxmin, totime) &
         bind(C, name="bcfd_shift_surface_nodes_initial")
      import :: c_int, c_int64_t, c_double
      integer(c_int64_t), value :: h, ita
      real(c_double), value :: aoa, piv, dt, dxmin, totime
    end function
    integer(c_int) function c_tag(h) bind(C, name="bcfd_tagging_th")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
    integer(c_int) function c_count_coarse(h) bind(C, name="bcfd_cellcount_solid_coarse")
      import :: c_int, c_int64_t
      integer(c_int64_t), value :: h
    end function
    integer(c_int) function c_fbc() bind(C, name="bcfd_fine_block_cell")
      import :: c_int
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
  subroutine findDistnode(blk)                      ! src/Search.F90:21-47
    ! The library finds the extreme surface-51 nodes mk, mkx1, mkx2 of the
    ! body frame when the block's body motion is set; the block's nodes are
    ! the body frame here (xnode), and the motion members (a0 in degrees, as
    ! read) are handed over with them.
    type(Block_t), intent(inout), target :: blk
    real(dp) :: p(6)
    integer(int64), target :: f(1)
    integer(c_int64_t) :: w
    call bcfd_ensure(blk)
    call bcfd_check(bcfd_block_set_nodes(blk%bcfd, blk%xnode, blk%ynode, blk%znode), 'set_nodes')
    p = [blk%a0, blk%bfreq, blk%yamp, blk%xshift, blk%yshift, blk%zshift]
    call bcfd_check(bcfd_block_set_body_motion(blk%bcfd, p), 'set_body_motion')
    call bcfd_check(c_read(blk%bcfd, 'mk'//char(0), c_loc(f), 1_c_int64_t, w), 'mk')
    blk%mk = f(1)
    call bcfd_check(c_read(blk%bcfd, 'mkx1'//char(0), c_loc(f), 1_c_int64_t, w), 'mkx1')
    blk%mkx1 = f(1)
    call bcfd_check(c_read(blk%bcfd, 'mkx2'//char(0), c_loc(f), 1_c_int64_t, w), 'mkx2')
    blk%mkx2 = f(1)
  end subroutine
  subroutine shiftSurfaceNodesInitial(blk, aoa, piv_pt, ita, deltat, dxmin, totime)  ! src/Search.F90:49-124
    type(Block_t), intent(inout) :: blk
    real(dp), intent(in) :: aoa, piv_pt, deltat, dxmin, totime
    integer(int64), intent(in) :: ita
    real(dp), parameter :: pi_ = 4.0_dp * atan(1.0_dp)
    call bcfd_ensure(blk)
    call bcfd_check(c_ssni(blk%bcfd, aoa, piv_pt, ita, deltat, dxmin, totime), 'shiftSurfaceNodesInitial')
    ! the Block_t members the routine changes: the placed nodes (allocated
    ! here, as the reference does), the kinematics and a0 in radians
    call bcfd_pull_motion(blk)
    blk%a0 = blk%a0 * pi_ / 180.0_dp
  end subroutine
  subroutine tagging_th(blk, blk_no)                ! src/Search.F90:388-413
    ! tagging_th_core on the device, then the reference's two record files
    ! butter_f.NNN.dat (cell, nodeIdTag per point) and butter_cellcount_f.NNN.dat
    type(Block_t), intent(inout) :: blk
    integer(int64), intent(in) :: blk_no
    character(len=120) :: filename1
    integer(int64) :: i, j, k
    integer :: u
    call bcfd_call(blk, c_tag, 'tagging_th')
    call bcfd_check(bcfd_block_download_tags(blk%bcfd, blk%cell, blk%cell2, blk%nodeIdTag, blk%cell_n, &
         blk%cell_pr), 'download_tags')
    write(filename1, '("butter_f.",i3.3,".dat")') blk_no
    open(newunit=u, file=filename1, status="unknown")
    do k = 1, blk%nz + 2
      do j = 1, blk%ny + 2
        do i = 1, blk%nx + 2
          write(u, *) blk%cell(i, j, k), blk%nodeIdTag(i, j, k)
        end do
      end do
    end do
    close(u)
    write(filename1, '("butter_cellcount_f.",i3.3,".dat")') blk_no
    open(newunit=u, file=filename1, form="formatted")
    write(u, *) blk%solidCellCount, blk%fluidCellCount, blk%ibCellCount
    close(u)
  end subroutine
  subroutine cellCount_solid_coarse(blk)            ! src/Search.F90:1463-1532
    type(Block_t), intent(inout) :: blk
    call bcfd_call(blk, c_count_coarse, 'cellCount_solid_coarse')
  end subroutine
  subroutine computeSurfaceVariables(blk, g, phase_angle, piv_pt, ita, deltat, dxmin, freq, re, totime)
    ! src/Search.F90:126-208 (re is not used by the routine)
    type(Block_t), intent(inout) :: blk
    integer(int64), intent(in) :: g, ita
    real(dp), intent(in) :: phase_angle, piv_pt, deltat, dxmin, freq, re, totime
    call bcfd_ensure(blk)
    call bcfd_check(bcfd_block_set_flags(blk%bcfd, -1_c_int64_t, int(blk%blk_mv_tag, c_int64_t)), 'set_flags')
    call bcfd_check(c_csv(blk%bcfd, phase_angle, piv_pt, ita, deltat, dxmin, freq, totime), &
         'computeSurfaceVariables')
    if (bcfd_host_mirror) call bcfd_pull_motion(blk)
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
    if (moved /= 0) marks_current = .true.  ! re-marked with the move
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
  subroutine fine_block_cell                       ! src/Search.F90:863-914
    ! the set-up call marks the coarse cells under the fine blocks; later calls
    ! find them current (a fine-block move re-marks inside block_move_check),
    ! and marking them again would change nothing
    if (marks_current) return
    call bcfd_check(c_fbc(), 'fine_block_cell')
    marks_current = .true.
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

! coefficientMatrix of src/CoefficientMatrix.f90:10-71: the 3-point Poisson
! line tables Acx/Acy/Acz (coarse-block boundary folding when is_coarse)
module biocfd_coefficient_matrix
  use biocfd_block_type, only: Block_t
  use biocfd_gb300_c
  use biocfd_gb300_glue
  implicit none
  private
  public :: coefficientMatrix
contains
  subroutine coefficientMatrix(blk, is_coarse)      ! src/CoefficientMatrix.f90:10-71
    type(Block_t), intent(inout) :: blk
    logical, intent(in) :: is_coarse
    integer(c_int) :: c
    c = 0
    if (is_coarse) c = 1
    call bcfd_ensure(blk)
    call bcfd_check(bcfd_coefficient_matrix(blk%bcfd, c), 'coefficientMatrix')
  end subroutine
end module biocfd_coefficient_matrix
