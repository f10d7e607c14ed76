! solver_gpu -- drop-in replacement of module solver (src/solver.f90) that runs
! pcg_solver on a GB300 through the C ABI of libsg.so (include/sg_solver.h).
!
! A host build selects it exactly as it selects solver_mpi: the drivers
! `use solver` / `use solver_mpi` (src/slope.F90:25-35, src/excavation.F90:28-37)
! become `use solver_gpu`, and the executable links libsg.so.  The subroutine
! keeps the reference signature, reads cg_maxiter and cg_tol from module
! global, and returns errcode 0 / -1 with the reference's errtag text.
!
! Build (where a Fortran compiler exists):
!   gfortran -c solver_gpu.f90   (after global.f90 / set_precision)
!   link with -L<path>/_lib -lsg -Wl,-rpath,<path>/_lib
module solver_gpu
use, intrinsic :: iso_c_binding
use set_precision
use global, only : cg_maxiter, cg_tol, nedof
implicit none
private
public :: pcg_solver

type(c_ptr), save :: ctx = c_null_ptr

interface
  function sg_create(device, hbm_budget) bind(c, name="sg_create")
    import :: c_ptr, c_int, c_size_t
    integer(c_int), value :: device
    integer(c_size_t), value :: hbm_budget
    type(c_ptr) :: sg_create
  end function sg_create

  function sg_pcg_solve(ctx, neq, nelmt, nedof, k, u, f, dprecon, gdof_elmt, cg_maxiter, cg_tol, &
                        cg_iter, errtag) bind(c, name="sg_pcg_solve")
    import :: c_ptr, c_int, c_double, c_char
    type(c_ptr), value :: ctx
    integer(c_int), value :: neq, nelmt, nedof, cg_maxiter
    real(c_double), intent(in) :: k(*), f(*), dprecon(*)
    real(c_double), intent(inout) :: u(*)
    integer(c_int), intent(in) :: gdof_elmt(*)
    real(c_double), value :: cg_tol
    integer(c_int), intent(out) :: cg_iter
    character(kind=c_char), intent(out) :: errtag(250)
    integer(c_int) :: sg_pcg_solve
  end function sg_pcg_solve
end interface

contains

! same signature as pcg_solver in src/solver.f90:14-27
subroutine pcg_solver(neq, nelmt, k, u, f, dprecon, gdof_elmt, cg_iter, errcode, errtag)
implicit none
integer, intent(in) :: neq, nelmt
real(kind=kreal), dimension(nedof,nedof,nelmt), intent(in), target :: k
real(kind=kreal), dimension(0:neq), intent(inout), target :: u
real(kind=kreal), dimension(0:neq), intent(in), target :: f, dprecon
integer, dimension(:,:), intent(in) :: gdof_elmt
integer, intent(out) :: cg_iter
integer, intent(out) :: errcode
character(len=250), intent(out) :: errtag

integer(c_int), allocatable :: ge(:,:)
character(kind=c_char) :: tag(250)
integer(c_int) :: it, rc
integer :: i

if (.not. c_associated(ctx)) ctx = sg_create(0_c_int, 0_c_size_t)
if (.not. c_associated(ctx)) then
  errcode = -1
  errtag = 'ERROR: no CUDA device for solver_gpu!'
  return
endif
! gdof_elmt may be a vector-subscripted section (src/excavation.F90:525-526):
! pass a contiguous copy, as the reference's copy-in does.
allocate(ge(nedof, nelmt))
ge = int(gdof_elmt, c_int)
rc = sg_pcg_solve(ctx, int(neq, c_int), int(nelmt, c_int), int(nedof, c_int), k, u, f, dprecon, ge, &
                  int(cg_maxiter, c_int), real(cg_tol, c_double), it, tag)
deallocate(ge)
cg_iter = it
errcode = rc
do i = 1, 250
  errtag(i:i) = tag(i)
enddo
end subroutine pcg_solver

end module solver_gpu
