! rhyme_cfl_time_step_gpu.f90 -- device-resident mode only: replaces
! src/rhyme_cfl/src/rhyme_cfl_time_step.f90 (same pure interface,
! rhyme_cfl.f90:19-23). In host-authoritative mode keep the reference file.
submodule(rhyme_cfl) rhyme_cfl_time_step_smod
   use, intrinsic :: iso_c_binding
   use rhyme_gpu_c
   use rhyme_gpu_drop_in
contains
   pure module function rhyme_cfl_time_step(c, samr) result(dt)
      implicit none

      real(kind=8), intent(in) :: c
      type(samr_t), intent(in) :: samr
      real(kind=8) :: dt

      real(c_double) :: dx3(3)

      ! the courant number is a run parameter of the context (equal to c)
      dx3 = 1d0
      dx3(1:NDIM) = samr%levels(0)%dx
      dt = rhyme_gpu_cfl_dt(rhyme_gpu_ctx_ptr, rhyme_gpu_handle_of(samr%levels(0)%boxes(1)), dx3)
   end function rhyme_cfl_time_step
end submodule rhyme_cfl_time_step_smod
