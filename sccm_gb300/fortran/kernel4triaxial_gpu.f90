! kernel4triaxial_gpu.f90 -- drop-in replacement of SCCM's per-pair subroutine
!   subroutine Kernel4Triaxial(lpr, Nphi1, Nphi2, NLEV)   (Codes/PNAMP/PNAMP_Kernel3D.f90:1)
! with the same name and signature, so the call at Codes/PNAMP/PNAMP_Main.f90:113 and the
! writer post_general (PNAMP_IO.f90:39-96) stay as they are. It reads the pair's vacua
! exactly as the reference does (PNAMP_Kernel3D.f90:88-122), hands the mesh loop and the
! J/K projection to the GB300 library through the C ABI (module pnamp_gpu), and fills
! Kernel%njkk, hjkk, nn, zz and J2 (VAPHFB_Par.f90:281-290).
!
! Compile it in place of PNAMP_Kernel3D(_triaxial).f90 with the PNAMP objects (it uses the
! reference's module VAPHFB_PAR) and link libpnamp_gb300.so. The library context (model
! space, Hamiltonian, one-body operators, mesh) is built on the first call of the process
! and reused for every later pair, as the module state it copies does not change between
! pairs; one context per MPI rank, one GPU per rank.
subroutine Kernel4Triaxial(lpr, Nphi1, Nphi2, NLEV)
  use iso_c_binding
  use vaphfb_par
  use pnamp_gpu
  implicit none
  logical, intent(in) :: lpr
  integer, intent(in) :: Nphi1, Nphi2, NLEV

  type(c_ptr), save :: ctx = c_null_ptr
  ! copies of the module state with the TARGET attribute that c_loc needs
  integer(c_int), allocatable, target, save :: t(:), n(:), l(:), twoj(:), twom(:)
  integer(c_int), allocatable, target, save :: ka(:), kb(:), kc(:), kd(:)
  real(c_double), allocatable, target, save :: t1b(:,:), vbar(:), q2(:,:)
  real(c_double), allocatable, target, save :: alp(:), walp(:), bet(:), wbet(:), gam(:), wgam(:)
  complex(c_double_complex), target, save :: nj(-PNAMP_JJMAX:PNAMP_JJMAX, -PNAMP_JJMAX:PNAMP_JJMAX, 0:PNAMP_JJMAX)
  complex(c_double_complex), target, save :: hj(-PNAMP_JJMAX:PNAMP_JJMAX, -PNAMP_JJMAX:PNAMP_JJMAX, 0:PNAMP_JJMAX)
  complex(c_double_complex), target, save :: xn(-PNAMP_JJMAX:PNAMP_JJMAX, -PNAMP_JJMAX:PNAMP_JJMAX, 0:PNAMP_JJMAX)
  complex(c_double_complex), target, save :: xz(-PNAMP_JJMAX:PNAMP_JJMAX, -PNAMP_JJMAX:PNAMP_JJMAX, 0:PNAMP_JJMAX)
  complex(c_double_complex), target, save :: xj(-PNAMP_JJMAX:PNAMP_JJMAX, -PNAMP_JJMAX:PNAMP_JJMAX, 0:PNAMP_JJMAX)
  complex(c_double_complex), allocatable :: zres(:,:)
  integer(c_int), allocatable :: st(:)
  type(pnamp_space) :: sp
  type(pnamp_hamiltonian) :: hc
  type(pnamp_mesh) :: mc
  type(pnamp_kernels) :: kc5
  integer(c_int) :: rc, ne
  integer :: ii, jj, J, K1, K2

  ! ---- the pair's vacua, as PNAMP_Kernel3D.f90:88-122 reads them
  if (.not. allocated(HFB%U0)) allocate(HFB%U0(NLEV, NLEV), HFB%V0(NLEV, NLEV))
  if (.not. allocated(HFB%U1)) allocate(HFB%U1(NLEV, NLEV), HFB%V1(NLEV, NLEV))
  open(unit=10, file=File%cwf(Nphi1), status='old')
  read(10, *) HFB%ide0(0), HFB%ide0(1)
  do ii = 1, NLEV
     do jj = 1, NLEV
        read(10, *) HFB%U0(ii, jj), HFB%V0(ii, jj)
     end do
  end do
  close(10)
  open(unit=11, file=File%cwf(Nphi2), status='old')
  read(11, *) HFB%ide1(0), HFB%ide1(1)
  do ii = 1, NLEV
     do jj = 1, NLEV
        read(11, *) HFB%U1(ii, jj), HFB%V1(ii, jj)
     end do
  end do
  close(11)

  ! ---- one library context per process: model space, H, cME1B, mesh
  if (.not. c_associated(ctx)) then
     allocate(t(NLEV), n(NLEV), l(NLEV), twoj(NLEV), twom(NLEV))
     t = tnljm%t(1:NLEV); n = tnljm%n(1:NLEV); l = tnljm%l(1:NLEV)
     twoj = tnljm%twoj(1:NLEV); twom = tnljm%twom(1:NLEV)
     sp%nlev = NLEV; sp%nprot = Input%nprot; sp%nneut = Input%nneut
     sp%core_prot = Nucl%ncore(1); sp%core_neut = Nucl%ncore(0)
     sp%t = c_loc(t); sp%n = c_loc(n); sp%l = c_loc(l); sp%twoj = c_loc(twoj); sp%twom = c_loc(twom)

     allocate(ka(H%iabcd_max), kb(H%iabcd_max), kc(H%iabcd_max), kd(H%iabcd_max), vbar(H%iabcd_max))
     ka = H%ka(1:H%iabcd_max); kb = H%kb(1:H%iabcd_max)
     kc = H%kc(1:H%iabcd_max); kd = H%kd(1:H%iabcd_max)
     vbar = H%ME2BM(1:H%iabcd_max)
     allocate(t1b(NLEV, NLEV), q2(NLEV * NLEV, 5))
     t1b = H%ME1BM(1:NLEV, 1:NLEV)
     q2(:, 1) = cME1B%Q2_2t(1:NLEV * NLEV); q2(:, 2) = cME1B%Q2_1t(1:NLEV * NLEV)
     q2(:, 3) = cME1B%Q20t(1:NLEV * NLEV);  q2(:, 4) = cME1B%Q21t(1:NLEV * NLEV)
     q2(:, 5) = cME1B%Q22t(1:NLEV * NLEV)
     hc%e0 = H%E0; hc%t1b = c_loc(t1b); hc%nrec = H%iabcd_max
     hc%ka = c_loc(ka); hc%kb = c_loc(kb); hc%kc = c_loc(kc); hc%kd = c_loc(kd)
     hc%vbar = c_loc(vbar)
     hc%q2 = c_null_ptr
     if (Input%iE2 .ne. 0) hc%q2 = c_loc(q2)

     allocate(alp(AMP%NLEG_ALP), walp(AMP%NLEG_ALP), bet(AMP%NLEG_BET), wbet(AMP%NLEG_BET))
     allocate(gam(AMP%NLEG_GAM), wgam(AMP%NLEG_GAM))
     alp = AMP%alpha(1:AMP%NLEG_ALP); walp = AMP%wwalp(1:AMP%NLEG_ALP)
     bet = AMP%beta(1:AMP%NLEG_BET);  wbet = AMP%wwbet(1:AMP%NLEG_BET)
     gam = AMP%gamma(1:AMP%NLEG_GAM); wgam = AMP%wwgam(1:AMP%NLEG_GAM)
     mc%nalp = AMP%NLEG_ALP; mc%nbet = AMP%NLEG_BET; mc%ngam = AMP%NLEG_GAM
     mc%nfom = PNP%NFOM; mc%ncosbet = 1
     mc%alpha = c_loc(alp); mc%walp = c_loc(walp); mc%beta = c_loc(bet); mc%wbet = c_loc(wbet)
     mc%gamma = c_loc(gam); mc%wgam = c_loc(wgam)
     mc%cscale = Input%Cscale; mc%iscale = Input%iscale

     rc = pnamp_init(sp, hc, mc, ctx)
     if (rc /= 0) then
        write(*, *) ' pnamp_init: ', pnamp_message(rc)
        stop
     end if
  end if

  ! ---- mesh loop (ZRES) and J/K projection on the GPU
  ne = pnamp_n_euler(ctx)
  allocate(zres(ne, PNAMP_NOBS), st(ne))
  rc = pnamp_pair(ctx, HFB%U0, HFB%V0, HFB%U1, HFB%V1, zres, st)
  if (rc /= 0) then
     write(*, *) ' pnamp_pair: ', pnamp_message(rc)
     stop
  end if
  kc5%njkk = c_loc(nj); kc5%hjkk = c_loc(hj); kc5%nn = c_loc(xn); kc5%zz = c_loc(xz); kc5%j2 = c_loc(xj)
  rc = pnamp_project(ctx, zres, 1_c_int, kc5)
  if (rc /= 0) then
     write(*, *) ' pnamp_project: ', pnamp_message(rc)
     stop
  end if

  ! the library's [J][K1][K2] arrays, seen from Fortran as (K2, K1, J)
  do J = 0, JJmax
     do K1 = -JJmax, JJmax
        do K2 = -JJmax, JJmax
           Kernel%njkk(J, K1, K2) = nj(K2, K1, J)
           Kernel%hjkk(J, K1, K2) = hj(K2, K1, J)
           Kernel%nn(J, K1, K2) = xn(K2, K1, J)
           Kernel%zz(J, K1, K2) = xz(K2, K1, J)
           Kernel%J2(J, K1, K2) = xj(K2, K1, J)
        end do
     end do
  end do
  if (lpr) write(*, '(a, i6, a, 2es16.8)') ' Kernel4Triaxial (GB300): ', ne, ' Euler points, N^0_00 =', &
       Kernel%njkk(0, 0, 0)
  deallocate(zres, st)
end subroutine Kernel4Triaxial
