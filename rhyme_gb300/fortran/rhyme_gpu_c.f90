! rhyme_gpu_c.f90 -- ISO_C_BINDING interfaces of librhyme_gpu.so
! (include/rhyme_gpu.h) for Rhyme's Fortran 2008 code.
!
! The C structure rhyme_gpu_params maps onto rhyme_gpu_params_t field by
! field; inflow(rho:e_tot, side) is bc%cons_inflows(1:NDIM+2, side).
! Axis arguments are 0-based on the C side.
module rhyme_gpu_c
   use, intrinsic :: iso_c_binding

   implicit none

   integer(c_int), parameter :: rhyme_gpu_ok = 0
   integer(c_int), parameter :: rhyme_gpu_einval = -1
   integer(c_int), parameter :: rhyme_gpu_enomem = -2
   integer(c_int), parameter :: rhyme_gpu_ecuda = -3
   integer(c_int), parameter :: rhyme_gpu_etimedout = -4
   integer(c_int), parameter :: rhyme_gpu_enanstate = -5
   integer(c_int), parameter :: rhyme_gpu_enotfound = -6

   integer(c_int), parameter :: rhyme_gpu_fp64 = 0
   integer(c_int), parameter :: rhyme_gpu_mixed = 1
   integer(c_int), parameter :: rhyme_gpu_tune_auto = 0
   integer(c_int), parameter :: rhyme_gpu_tune_fixed = 1
   ! boundary type of a face whose ghost rows the caller fills (a slab of a
   ! box decomposed over several GPUs); the others are bcid's values
   integer(c_int), parameter :: rhyme_gpu_halo = 5

   type, bind(c) :: rhyme_gpu_params_t
      integer(c_int) :: ndim = 0
      integer(c_int) :: limiter = 0
      integer(c_int) :: n_iteration = 0
      integer(c_int) :: solver_type = 0
      integer(c_int) :: bc(6) = 0
      integer(c_int) :: precision = 0
      integer(c_int) :: sweep_tuning = 0
      real(c_double) :: gamma = 0d0
      real(c_double) :: kb_amu = 0d0
      real(c_double) :: courant = 0d0
      real(c_double) :: omega = 0d0
      real(c_double) :: vacuum_density = 0d0
      real(c_double) :: vacuum_pressure = 0d0
      real(c_double) :: tolerance = 0d0
      real(c_double) :: inflow(5, 6) = 0d0
   end type rhyme_gpu_params_t

   interface
      integer(c_int) function rhyme_gpu_abi_version() bind(c, name='rhyme_gpu_abi_version')
         import :: c_int
      end function rhyme_gpu_abi_version

      integer(c_int) function rhyme_gpu_create(ctx, params) bind(c, name='rhyme_gpu_create')
         import :: c_int, c_ptr, rhyme_gpu_params_t
         type(c_ptr), intent(out) :: ctx
         type(rhyme_gpu_params_t), intent(in) :: params
      end function rhyme_gpu_create

      integer(c_int) function rhyme_gpu_destroy(ctx) bind(c, name='rhyme_gpu_destroy')
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
      end function rhyme_gpu_destroy

      type(c_ptr) function rhyme_gpu_last_error(ctx) bind(c, name='rhyme_gpu_last_error')
         import :: c_ptr
         type(c_ptr), value :: ctx
      end function rhyme_gpu_last_error

      integer(c_int) function rhyme_gpu_register_box(ctx, level, number, cells, dims, ghost, ncmp, handle) &
         bind(c, name='rhyme_gpu_register_box')
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx
         integer(c_int), value :: level, number, ghost, ncmp
         real(c_double), intent(inout) :: cells(*)
         integer(c_int), intent(in) :: dims(3)
         integer(c_int), intent(out) :: handle
      end function rhyme_gpu_register_box

      integer(c_int) function rhyme_gpu_unregister_box(ctx, handle) bind(c, name='rhyme_gpu_unregister_box')
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
         integer(c_int), value :: handle
      end function rhyme_gpu_unregister_box

      integer(c_int) function rhyme_gpu_sync_to_device(ctx, handle) bind(c, name='rhyme_gpu_sync_to_device')
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
         integer(c_int), value :: handle
      end function rhyme_gpu_sync_to_device

      integer(c_int) function rhyme_gpu_sync_to_host(ctx, handle) bind(c, name='rhyme_gpu_sync_to_host')
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
         integer(c_int), value :: handle
      end function rhyme_gpu_sync_to_host

      integer(c_int) function rhyme_gpu_set_host_writeback(ctx, handle, on) bind(c, name='rhyme_gpu_set_host_writeback')
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
         integer(c_int), value :: handle, on
      end function rhyme_gpu_set_host_writeback

      ! rows row0 .. row0+nrows-1 (0-based, ghost rows included) of the
      ! outermost axis of the hydro components: the halo of a slab
      integer(c_int) function rhyme_gpu_get_rows(ctx, handle, row0, nrows, rows) bind(c, name='rhyme_gpu_get_rows')
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx
         integer(c_int), value :: handle, row0, nrows
         real(c_double), intent(out) :: rows(*)
      end function rhyme_gpu_get_rows

      integer(c_int) function rhyme_gpu_set_rows(ctx, handle, row0, nrows, rows) bind(c, name='rhyme_gpu_set_rows')
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx
         integer(c_int), value :: handle, row0, nrows
         real(c_double), intent(in) :: rows(*)
      end function rhyme_gpu_set_rows

      integer(c_int) function rhyme_gpu_box_status(ctx, handle, flags) bind(c, name='rhyme_gpu_box_status')
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
         integer(c_int), value :: handle
         integer(c_int), intent(out) :: flags
      end function rhyme_gpu_box_status

      integer(c_int) function rhyme_gpu_cfl_time_step(ctx, handle, dx, dt) &
         bind(c, name='rhyme_gpu_cfl_time_step')
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx
         integer(c_int), value :: handle
         real(c_double), intent(in) :: dx(3)
         real(c_double), intent(out) :: dt
      end function rhyme_gpu_cfl_time_step

      ! Declared pure so that the pure rhyme_cfl_time_step and
      ! rhyme_samr_bc_set_boundaries of the reference can call them.
      pure real(c_double) function rhyme_gpu_cfl_dt(ctx, handle, dx) bind(c, name='rhyme_gpu_cfl_dt')
         import :: c_int, c_ptr, c_double
         type(c_ptr), value, intent(in) :: ctx
         integer(c_int), value, intent(in) :: handle
         real(c_double), intent(in) :: dx(3)
      end function rhyme_gpu_cfl_dt

      pure integer(c_int) function rhyme_gpu_set_boundaries(ctx, handle) bind(c, name='rhyme_gpu_set_boundaries')
         import :: c_int, c_ptr
         type(c_ptr), value, intent(in) :: ctx
         integer(c_int), value, intent(in) :: handle
      end function rhyme_gpu_set_boundaries

      integer(c_int) function rhyme_gpu_mh_solve(ctx, handle, dx, dt) bind(c, name='rhyme_gpu_mh_solve')
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx
         integer(c_int), value :: handle
         real(c_double), intent(in) :: dx(3)
         real(c_double), value :: dt
      end function rhyme_gpu_mh_solve

      integer(c_int) function rhyme_gpu_run(ctx, handle, dx, nsteps, dt_trace) bind(c, name='rhyme_gpu_run')
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx
         integer(c_int), value :: handle, nsteps
         real(c_double), intent(in) :: dx(3)
         real(c_double), intent(out) :: dt_trace(*)
      end function rhyme_gpu_run

      integer(c_int) function rhyme_gpu_synchronize(ctx) bind(c, name='rhyme_gpu_synchronize')
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
      end function rhyme_gpu_synchronize

      integer(c_int) function rhyme_gpu_riemann_solve(ctx, l, r, n, dx, dt, axis, u) &
         bind(c, name='rhyme_gpu_riemann_solve')
         import :: c_int, c_ptr, c_double, c_long_long
         type(c_ptr), value :: ctx
         real(c_double), intent(in) :: l(*), r(*)
         integer(c_long_long), value :: n
         real(c_double), value :: dx, dt
         integer(c_int), value :: axis
         real(c_double), intent(out) :: u(*)
      end function rhyme_gpu_riemann_solve

      integer(c_int) function rhyme_gpu_irs_exec(ctx, states, n, out) bind(c, name='rhyme_gpu_irs_exec')
         import :: c_int, c_ptr, c_double, c_long_long
         type(c_ptr), value :: ctx
         real(c_double), intent(in) :: states(*)
         integer(c_long_long), value :: n
         real(c_double), intent(out) :: out(*)
      end function rhyme_gpu_irs_exec

      integer(c_int) function rhyme_gpu_slope_limiter(ctx, ul, u, ur, n, delta) &
         bind(c, name='rhyme_gpu_slope_limiter')
         import :: c_int, c_ptr, c_double, c_long_long
         type(c_ptr), value :: ctx
         real(c_double), intent(in) :: ul(*), u(*), ur(*)
         integer(c_long_long), value :: n
         real(c_double), intent(out) :: delta(*)
      end function rhyme_gpu_slope_limiter

      integer(c_int) function rhyme_gpu_half_step(ctx, u, delta, n, axis, dx, dt, l, r) &
         bind(c, name='rhyme_gpu_half_step')
         import :: c_int, c_ptr, c_double, c_long_long
         type(c_ptr), value :: ctx
         real(c_double), intent(in) :: u(*), delta(*)
         integer(c_long_long), value :: n
         integer(c_int), value :: axis
         real(c_double), value :: dx, dt
         real(c_double), intent(out) :: l(*), r(*)
      end function rhyme_gpu_half_step
   end interface
end module rhyme_gpu_c
