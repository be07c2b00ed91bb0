! rhyme_gpu_drop_in.f90 -- state of the GPU drop-in for Rhyme's driver.
!
! Holds the librhyme_gpu context and the handle of every registered SAMR box.
! rhyme_gpu_drop_in_init is the one call added to src/main.f90, after the
! modules are initialised (after rhyme_cfl_init, main.f90:91); it copies the
! run parameters the reference's modules hold into rhyme_gpu_params_t and
! registers the boxes of every level (their cells arrays stay owned by
! Rhyme and must not be reallocated while registered).
!
! Two modes:
!  * host-authoritative (default): box%cells is the truth between calls;
!    the replacement rhyme_muscl_hancock_solve uploads the box (with the
!    ghosts rhyme_samr_bc_set_boundaries just filled), solves on the GPU and
!    downloads the result, so every host reader of box%cells (Chombo output,
!    reports, sanity checks, stabilizer) sees the reference's state.
!  * device-resident (rhyme_gpu_device_resident = .true.): the CFL time step,
!    the ghost fill and the solve all run on the device and box%cells is
!    refreshed only by rhyme_gpu_drop_in_sync_to_host, which the driver
!    calls before a host reader needs the state.
module rhyme_gpu_drop_in
   use, intrinsic :: iso_c_binding
   use rhyme_gpu_c
   use rhyme_units
   use rhyme_samr
   use rhyme_samr_bc
   use rhyme_cfl
   use rhyme_thermo_base
   use rhyme_riemann_problem
   use rhyme_slope_limiter
   use rhyme_muscl_hancock
   use rhyme_logger

   implicit none

   integer, parameter :: rhyme_gpu_max_boxes = 4096

   type(c_ptr), save :: rhyme_gpu_ctx_ptr = c_null_ptr
   integer(c_int), save :: rhyme_gpu_handles(0:23, rhyme_gpu_max_boxes) = -1
   logical, save :: rhyme_gpu_device_resident = .false.

contains

   subroutine rhyme_gpu_drop_in_init(units, thermo, cfl, bc, rp, sl, mh, samr, logger, mixed)
      type(units_t), intent(in) :: units
      type(thermo_base_t), intent(in) :: thermo
      type(cfl_t), intent(in) :: cfl
      type(samr_bc_t), intent(in) :: bc
      type(riemann_problem_t), intent(in) :: rp
      type(slope_limiter_t), intent(in) :: sl
      type(muscl_hancock_t), intent(in) :: mh
      type(samr_t), intent(inout) :: samr
      type(logger_t), intent(inout) :: logger
      logical, intent(in), optional :: mixed

      type(rhyme_gpu_params_t) :: params
      integer :: l, b
      integer(c_int) :: rc

      call logger%begin_section('rhyme_gpu')

      params%ndim = NDIM
      params%limiter = sl%type
      params%n_iteration = rp%irs%n_iteration
      params%solver_type = mh%solver_type
      params%bc(1:2*NDIM) = bc%types(1:2*NDIM)
      params%precision = rhyme_gpu_fp64
      if (present(mixed)) then
         if (mixed) params%precision = rhyme_gpu_mixed
      end if
      params%gamma = get_gamma()
      params%kb_amu = units%kb%v/units%amu%v
      params%courant = cfl%courant_number
      params%omega = sl%w
      params%vacuum_density = rp%w_vacuum(cid%rho)
      params%vacuum_pressure = rp%w_vacuum(cid%p)
      params%tolerance = rp%irs%tolerance
      params%inflow(1:NDIM + 2, 1:2*NDIM) = bc%cons_inflows(cid%rho:cid%e_tot, 1:2*NDIM)

      rc = rhyme_gpu_create(rhyme_gpu_ctx_ptr, params)
      if (rc /= rhyme_gpu_ok) then
         call logger%err('rhyme_gpu_create failed')
         call logger%end_section
         return
      end if

      do l = 0, samr%nlevels - 1
         do b = 1, samr%levels(l)%nboxes
            call rhyme_gpu_drop_in_register(samr%levels(l)%boxes(b), logger)
         end do
      end do

      call logger%end_section
   end subroutine rhyme_gpu_drop_in_init

   subroutine rhyme_gpu_drop_in_register(box, logger)
      type(samr_box_t), intent(inout) :: box
      type(logger_t), intent(inout) :: logger

      integer(c_int) :: dims(3), h, rc

      if (box%level < lbound(rhyme_gpu_handles, 1) .or. box%level > ubound(rhyme_gpu_handles, 1) &
          .or. box%number < 1 .or. box%number > rhyme_gpu_max_boxes) then
         call logger%err('box level or number outside the GPU handle table')
         return
      end if

      dims = 1
      dims(1:NDIM) = box%dims
      rc = rhyme_gpu_register_box(rhyme_gpu_ctx_ptr, box%level, box%number, box%cells, dims, &
                                  2_c_int, size(box%cells, NDIM + 1), h)
      if (rc /= rhyme_gpu_ok) then
         call logger%err('rhyme_gpu_register_box failed')
         return
      end if
      rhyme_gpu_handles(box%level, box%number) = h
      ! host-authoritative: each solve copies its result back while it runs
      if (.not. rhyme_gpu_device_resident) then
         rc = rhyme_gpu_set_host_writeback(rhyme_gpu_ctx_ptr, h, 1_c_int)
         if (rc /= rhyme_gpu_ok) call logger%err('rhyme_gpu_set_host_writeback failed')
      end if
   end subroutine rhyme_gpu_drop_in_register

   pure integer(c_int) function rhyme_gpu_handle_of(box) result(h)
      type(samr_box_t), intent(in) :: box
      ! a box outside the table was never registered: -1 makes every call
      ! on it return RHYME_GPU_EINVAL
      h = -1
      if (box%level < lbound(rhyme_gpu_handles, 1) .or. box%level > ubound(rhyme_gpu_handles, 1)) return
      if (box%number < 1 .or. box%number > rhyme_gpu_max_boxes) return
      h = rhyme_gpu_handles(box%level, box%number)
   end function rhyme_gpu_handle_of

   ! Device-resident mode: refresh box%cells of every registered box.
   subroutine rhyme_gpu_drop_in_sync_to_host(samr, logger)
      type(samr_t), intent(inout) :: samr
      type(logger_t), intent(inout) :: logger
      integer :: l, b
      integer(c_int) :: rc
      do l = 0, samr%nlevels - 1
         do b = 1, samr%levels(l)%nboxes
            rc = rhyme_gpu_sync_to_host(rhyme_gpu_ctx_ptr, rhyme_gpu_handle_of(samr%levels(l)%boxes(b)))
            if (rc /= rhyme_gpu_ok) call logger%err('rhyme_gpu_sync_to_host failed')
         end do
      end do
   end subroutine rhyme_gpu_drop_in_sync_to_host
end module rhyme_gpu_drop_in
