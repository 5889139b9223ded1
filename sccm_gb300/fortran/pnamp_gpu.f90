! pnamp_gpu.f90 -- ISO_C_BINDING interface to the GB300 PNAMP library
! (include/pnamp_gpu.h, sccm_gb300/_lib/libpnamp_gb300.so).
!
! The derived types mirror the C structs field for field (bind(C) gives them the
! C layout); matrices are column-major like the Fortran arrays they come from,
! complex numbers are complex(c_double_complex), i.e. complex*16. Return codes:
! 0 = success, otherwise pnamp_strerror(code) gives the text.
!
! Build (with the PNAMP objects, next to VAPHFB_Par.f90):
!   gfortran -c pnamp_gpu.f90 kernel4triaxial_gpu.f90
!   ... -L<repo>/sccm_gb300/_lib -lpnamp_gb300 -Wl,-rpath,<repo>/sccm_gb300/_lib
module pnamp_gpu
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: PNAMP_NOBS = 19, PNAMP_JJMAX = 6
  integer(c_int), parameter :: PNAMP_FORM_FP64 = 0, PNAMP_FORM_DF64 = 1
  integer(c_int), parameter :: PNAMP_ERR_SMALL_NORM = 8

  type, bind(C) :: pnamp_space
     integer(c_int) :: nlev, nprot, nneut, core_prot, core_neut
     type(c_ptr)    :: t, n, l, twoj, twom
  end type pnamp_space

  type, bind(C) :: pnamp_hamiltonian
     real(c_double) :: e0
     type(c_ptr)    :: t1b
     integer(c_int) :: nrec
     type(c_ptr)    :: ka, kb, kc, kd, vbar, q2
  end type pnamp_hamiltonian

  type, bind(C) :: pnamp_mesh
     integer(c_int) :: nalp, nbet, ngam, nfom, ncosbet
     type(c_ptr)    :: alpha, walp, beta, wbet, gamma, wgam
     real(c_double) :: cscale
     integer(c_int) :: iscale
  end type pnamp_mesh

  type, bind(C) :: pnamp_kernels
     type(c_ptr) :: njkk, hjkk, nn, zz, j2
  end type pnamp_kernels

  interface
     integer(c_int) function pnamp_init(sp, h, m, ctx) bind(C, name="pnamp_init")
       import :: c_int, c_ptr, pnamp_space, pnamp_hamiltonian, pnamp_mesh
       type(pnamp_space), intent(in) :: sp
       type(pnamp_hamiltonian), intent(in) :: h
       type(pnamp_mesh), intent(in) :: m
       type(c_ptr), intent(out) :: ctx
     end function pnamp_init

     integer(c_int) function pnamp_set_form(ctx, form) bind(C, name="pnamp_set_form")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: form
     end function pnamp_set_form

     integer(c_int) function pnamp_n_euler(ctx) bind(C, name="pnamp_n_euler")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function pnamp_n_euler

     integer(c_int) function pnamp_pair(ctx, u0, v0, u1, v1, zres, st) bind(C, name="pnamp_pair")
       import :: c_int, c_ptr, c_double, c_double_complex
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: u0(*), v0(*), u1(*), v1(*)
       complex(c_double_complex), intent(out) :: zres(*)
       integer(c_int), intent(out) :: st(*)
     end function pnamp_pair

     integer(c_int) function pnamp_project(ctx, zres, chop, k) bind(C, name="pnamp_project")
       import :: c_int, c_ptr, c_double_complex, pnamp_kernels
       type(c_ptr), value :: ctx
       complex(c_double_complex), intent(in) :: zres(*)
       integer(c_int), value :: chop
       type(pnamp_kernels), intent(in) :: k
     end function pnamp_project

     integer(c_int) function pnamp_batch_rho1b(ctx, npairs, uv, zres, st, r1) bind(C, name="pnamp_batch_rho1b")
       import :: c_int, c_ptr, c_double, c_double_complex
       type(c_ptr), value :: ctx
       integer(c_int), value :: npairs
       real(c_double), intent(in) :: uv(*)
       complex(c_double_complex), intent(out) :: zres(*), r1(*)
       integer(c_int), intent(out) :: st(*)
     end function pnamp_batch_rho1b

     integer(c_int) function pnamp_rho1b_blocks(ctx, it, lj, n1, n2, twoj) bind(C, name="pnamp_rho1b_blocks")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), intent(out) :: it(*), lj(*), n1(*), n2(*), twoj(*)
     end function pnamp_rho1b_blocks

     integer(c_int) function pnamp_project_rho1b(ctx, zres, r1, out) bind(C, name="pnamp_project_rho1b")
       import :: c_int, c_ptr, c_double, c_double_complex
       type(c_ptr), value :: ctx
       complex(c_double_complex), intent(in) :: zres(*), r1(*)
       real(c_double), intent(out) :: out(*)
     end function pnamp_project_rho1b

     type(c_ptr) function pnamp_strerror(code) bind(C, name="pnamp_strerror")
       import :: c_ptr, c_int
       integer(c_int), value :: code
     end function pnamp_strerror

     subroutine pnamp_free(ctx) bind(C, name="pnamp_free")
       import :: c_ptr
       type(c_ptr), value :: ctx
     end subroutine pnamp_free
  end interface

contains

  ! Text of a return code as a Fortran string (for `stop` messages).
  function pnamp_message(code) result(msg)
    integer(c_int), intent(in) :: code
    character(len=:), allocatable :: msg
    character(kind=c_char), pointer :: p(:)
    integer :: k
    call c_f_pointer(pnamp_strerror(code), p, [256])
    k = 0
    do while (k < 256)
       if (p(k + 1) == c_null_char) exit
       k = k + 1
    end do
    allocate(character(len=k) :: msg)
    msg = transfer(p(1:k), msg)
  end function pnamp_message

end module pnamp_gpu
