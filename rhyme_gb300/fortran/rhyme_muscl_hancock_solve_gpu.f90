! rhyme_muscl_hancock_solve_gpu.f90 -- replaces
! src/rhyme_muscl_hancock/src/rhyme_muscl_hancock_solve.f90 in the module's
! source list. Same interface (rhyme_muscl_hancock.f90:47-56); the solve runs
! on the GPU through librhyme_gpu (both solver types, by mh%solver_type).
submodule(rhyme_muscl_hancock) rhyme_mh_solve_submodule
   use, intrinsic :: iso_c_binding
   use rhyme_gpu_c
   use rhyme_gpu_drop_in
contains
   module subroutine rhyme_muscl_hancock_solve( &
      mh, box, dx, dt, rp, sl, ws, logger)
      implicit none

      type(muscl_hancock_t), intent(inout) :: mh
      type(samr_box_t), intent(inout) :: box
      real(kind=8), intent(in) :: dx(NDIM), dt
      type(riemann_problem_t), intent(inout) :: rp
      type(slope_limiter_t), intent(in) :: sl
      type(mh_workspace_t), intent(inout) :: ws
      type(logger_t), intent(inout) :: logger

      real(c_double) :: dx3(3)
      integer(c_int) :: h, rc

      call logger%begin_section('solver')

      if (mh%solver_type /= mhid%cpu_intensive .and. mh%solver_type /= mhid%memory_intensive) then
         call logger%err('Unknown solver type')
         return
      end if

      h = rhyme_gpu_handle_of(box)
      if (h < 0) then
         call rhyme_gpu_drop_in_register(box, logger)
         h = rhyme_gpu_handle_of(box)
      end if

      dx3 = 1d0
      dx3(1:NDIM) = dx

      rc = rhyme_gpu_ok
      if (.not. rhyme_gpu_device_resident) rc = rhyme_gpu_sync_to_device(rhyme_gpu_ctx_ptr, h)
      if (rc == rhyme_gpu_ok) rc = rhyme_gpu_mh_solve(rhyme_gpu_ctx_ptr, h, dx3, dt)
      if (rc == rhyme_gpu_ok .and. .not. rhyme_gpu_device_resident) &
         rc = rhyme_gpu_sync_to_host(rhyme_gpu_ctx_ptr, h)
      if (rc /= rhyme_gpu_ok) call logger%err('rhyme_gpu: MUSCL-Hancock solve failed')

      call logger%end_section
   end subroutine rhyme_muscl_hancock_solve
end submodule rhyme_mh_solve_submodule
