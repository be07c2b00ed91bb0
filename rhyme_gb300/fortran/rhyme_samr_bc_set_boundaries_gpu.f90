! rhyme_samr_bc_set_boundaries_gpu.f90 -- device-resident mode only:
! replaces src/rhyme_samr_bc/src/rhyme_samr_bc_set_boundaries.f90 (same pure
! interface, rhyme_samr_bc.f90:38-41). In host-authoritative mode keep the
! reference file.
submodule(rhyme_samr_bc) set_boundaries_smod
   use, intrinsic :: iso_c_binding
   use rhyme_gpu_c
   use rhyme_gpu_drop_in
contains
   pure module subroutine rhyme_samr_bc_set_boundaries(bc, samr)
      implicit none

      type(samr_bc_t), intent(in) :: bc
      type(samr_t), intent(inout) :: samr

      integer(c_int) :: rc

      ! the boundary types are run parameters of the context (equal to bc%types)
      rc = rhyme_gpu_set_boundaries(rhyme_gpu_ctx_ptr, rhyme_gpu_handle_of(samr%levels(0)%boxes(1)))
   end subroutine rhyme_samr_bc_set_boundaries
end submodule set_boundaries_smod
