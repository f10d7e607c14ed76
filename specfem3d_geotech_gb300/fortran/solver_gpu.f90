! solver_gpu -- drop-in replacement of module solver (src/solver.f90) that runs
! pcg_solver on a GB300 through the C ABI of libsg.so (include/sg_solver.h),
! plus stress_bodyload_gpu, the GPU form of the stress / yield / flow /
! body-load block that slope3d and excavation3d inline after each solve
! (src/slope.F90:311-383, src/excavation.F90:546-616).
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
public :: pcg_solver, stress_bodyload_gpu

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

  function sg_stress_bodyload(ctx, neq, nelmt, nnode, g_coord, g_num, gdof_elmt, mat_id, nmatblk, ym_blk, &
                              nuf_blk, phif_blk, cohf_blk, psif_blk, dt, nl_isconv, last, elmt_list, nel,  &
                              wpressure, form, x, evpt, stress_elmt, bodyload, vmeps, scf, fmax, errtag)   &
                              bind(c, name="sg_stress_bodyload")
    import :: c_ptr, c_int, c_double, c_char
    type(c_ptr), value :: ctx
    integer(c_int), value :: neq, nelmt, nnode, nmatblk, nl_isconv, last, nel, form
    type(c_ptr), value :: g_coord, g_num, gdof_elmt, mat_id, ym_blk, nuf_blk, phif_blk, cohf_blk, psif_blk
    type(c_ptr), value :: elmt_list, wpressure, x, evpt, stress_elmt, bodyload, vmeps, scf
    real(c_double), value :: dt
    real(c_double), intent(out) :: fmax
    character(kind=c_char), intent(out) :: errtag(250)
    integer(c_int) :: sg_stress_bodyload
  end function sg_stress_bodyload
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

! In place of the element loop of src/slope.F90:311-383 (form = 0, all
! elements) or src/excavation.F90:546-616 (form = 1 over elmt_intact, with
! vmeps/scf accumulated when last):
!   call stress_bodyload_gpu(neq, nelmt, nnode, g_coord, g_num, gdof_elmt, mat_id, ym_blk, nuf_blk, &
!        phif_blk, cohf_blk, psif_blk, dt, nl_isconv, nl_isconv .or. nl_iter == nl_maxiter, x, evpt, &
!        stress_elmt, bodyload, fmax, errcode, errtag [, elmt_list, wpressure, form, vmeps, scf])
! evpt, stress_elmt and bodyload are updated as the loop updates them.
subroutine stress_bodyload_gpu(neq, nelmt, nnode, g_coord, g_num, gdof_elmt, mat_id, ym_blk, nuf_blk, &
                               phif_blk, cohf_blk, psif_blk, dt, nl_isconv, last, x, evpt, stress_elmt,  &
                               bodyload, fmax, errcode, errtag, elmt_list, wpressure, form, vmeps, scf)
implicit none
integer, intent(in) :: neq, nelmt, nnode
real(kind=kreal), intent(in), target :: g_coord(:,:), ym_blk(:), nuf_blk(:), phif_blk(:), cohf_blk(:), &
                                        psif_blk(:)
integer, intent(in) :: g_num(:,:), gdof_elmt(:,:), mat_id(:)
real(kind=kreal), intent(in) :: dt
logical, intent(in) :: nl_isconv, last
real(kind=kreal), dimension(0:neq), intent(in), target :: x
real(kind=kreal), intent(inout), target :: evpt(:,:,:), stress_elmt(:,:,:)
real(kind=kreal), dimension(0:neq), intent(inout), target :: bodyload
real(kind=kreal), intent(out) :: fmax
integer, intent(out) :: errcode
character(len=250), intent(out) :: errtag
integer, intent(in), optional :: elmt_list(:)
real(kind=kreal), intent(in), optional, target :: wpressure(:)
integer, intent(in), optional :: form
real(kind=kreal), intent(inout), optional, target :: vmeps(:), scf(:)

integer(c_int), allocatable, target :: gn(:,:), ge(:,:), mid(:), el(:)
type(c_ptr) :: p_el, p_wp, p_vm, p_sf
character(kind=c_char) :: tag(250)
real(c_double) :: fm
integer(c_int) :: rc, nel, frm, iconv, ilast
integer :: i

if (.not. c_associated(ctx)) ctx = sg_create(0_c_int, 0_c_size_t)
if (.not. c_associated(ctx)) then
  errcode = -1
  errtag = 'ERROR: no CUDA device for solver_gpu!'
  return
endif
! contiguous C-int copies of the integer maps (they may be sections)
allocate(gn(size(g_num,1), nelmt), ge(size(gdof_elmt,1), nelmt), mid(nelmt))
gn = int(g_num(:,1:nelmt), c_int)
ge = int(gdof_elmt(:,1:nelmt), c_int)
mid = int(mat_id(1:nelmt), c_int)
p_el = c_null_ptr; nel = int(nelmt, c_int)
if (present(elmt_list)) then
  allocate(el(size(elmt_list)))
  el = int(elmt_list, c_int)
  nel = int(size(elmt_list), c_int)
  p_el = c_loc(el)
endif
p_wp = c_null_ptr; p_vm = c_null_ptr; p_sf = c_null_ptr
if (present(wpressure)) p_wp = c_loc(wpressure)
if (present(vmeps)) p_vm = c_loc(vmeps)
if (present(scf)) p_sf = c_loc(scf)
frm = 0_c_int
if (present(form)) frm = int(form, c_int)
iconv = 0_c_int; if (nl_isconv) iconv = 1_c_int
ilast = 0_c_int; if (last) ilast = 1_c_int
rc = sg_stress_bodyload(ctx, int(neq, c_int), int(nelmt, c_int), int(nnode, c_int), c_loc(g_coord), c_loc(gn), &
                        c_loc(ge), c_loc(mid), int(size(ym_blk), c_int), c_loc(ym_blk), c_loc(nuf_blk),        &
                        c_loc(phif_blk), c_loc(cohf_blk), c_loc(psif_blk), real(dt, c_double), iconv, ilast,   &
                        p_el, nel, p_wp, frm, c_loc(x), c_loc(evpt), c_loc(stress_elmt), c_loc(bodyload),      &
                        p_vm, p_sf, fm, tag)
deallocate(gn, ge, mid)
if (allocated(el)) deallocate(el)
fmax = fm
errcode = rc
do i = 1, 250
  errtag(i:i) = tag(i)
enddo
end subroutine stress_bodyload_gpu

end module solver_gpu
