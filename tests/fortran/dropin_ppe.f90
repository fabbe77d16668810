! Drop-in check of the Fortran binding (include/gbmg.f90).
!
! Reads a case written by tests/test_gpu_fortran.py -- grid, density, face
! velocities u*, v*, w*, dt, tol -- into arrays laid out as the reference's
! solvers allocate them (ghc = 3 ghost cells per side, u(i,j,k) on face i+1/2
! so u(0,1,1) is the low wall face), then makes the two calls that replace
! "call ppe_sor_init" and "call ppe_sor_solver(p%glb%p_tol)" in ns_ab_solver_SOR
! ("Two phase flows/newOpenMP/3D+IBM/src/ns_solver/admas_bashforth_solver.f90:50,62"),
! checks the divergence as ns_check_convergence_div does, and writes the
! pressure and the corrected velocities (interior) back.
!
! usage: dropin_ppe <case file> <result file>
program dropin_ppe
  use iso_c_binding
  use gbmg
  implicit none
  integer, parameter :: ghc = 3
  real(c_double), parameter :: sentinel = -777.0d0
  character(len=1024) :: fin, fout
  integer(c_int32_t) :: hdr(4)
  integer :: nx, ny, nz, lx, ly, ghosts_ok
  real(c_double) :: sp(5), dt, tol, mx, mean
  real(c_double), allocatable, target :: rho(:,:,:), p(:,:,:), u(:,:,:), v(:,:,:), w(:,:,:)
  real(c_double), allocatable :: buf(:,:,:)
  type(c_ptr) :: h
  type(gbmg_grid) :: g
  type(gbmg_params) :: prm
  type(gbmg_stats) :: st
  type(gbmg_field) :: fu, fv, fw, fp
  integer(c_int) :: rc, rc_div

  call get_command_argument(1, fin)
  call get_command_argument(2, fout)
  open(10, file=trim(fin), access='stream', form='unformatted', status='old')
  read(10) hdr
  read(10) sp
  nx = hdr(1); ny = hdr(2); nz = hdr(3)
  dt = sp(4); tol = sp(5)
  lx = nx + 2 * ghc
  ly = ny + 2 * ghc
  allocate(rho(1-ghc:nx+ghc, 1-ghc:ny+ghc, 1-ghc:nz+ghc))
  allocate(p(1-ghc:nx+ghc, 1-ghc:ny+ghc, 1-ghc:nz+ghc))
  allocate(u(1-ghc:nx+ghc, 1-ghc:ny+ghc, 1-ghc:nz+ghc))
  allocate(v(1-ghc:nx+ghc, 1-ghc:ny+ghc, 1-ghc:nz+ghc))
  allocate(w(1-ghc:nx+ghc, 1-ghc:ny+ghc, 1-ghc:nz+ghc))
  rho = sentinel; p = sentinel; u = sentinel; v = sentinel; w = sentinel
  allocate(buf(nx, ny, nz))
  read(10) buf
  rho(1:nx, 1:ny, 1:nz) = buf
  deallocate(buf)
  allocate(buf(0:nx, 1:ny, 1:nz))
  read(10) buf
  u(0:nx, 1:ny, 1:nz) = buf
  deallocate(buf)
  allocate(buf(1:nx, 0:ny, 1:nz))
  read(10) buf
  v(1:nx, 0:ny, 1:nz) = buf
  deallocate(buf)
  allocate(buf(1:nx, 1:ny, 0:nz))
  read(10) buf
  w(1:nx, 1:ny, 0:nz) = buf
  deallocate(buf)
  close(10)
  p(1:nx, 1:ny, 1:nz) = 0.0d0

  ! once, after the grid is known
  call gbmg_default_params(prm)
  prm%precision = hdr(4)
  g = gbmg_grid(int(nx, c_int32_t), int(ny, c_int32_t), int(nz, c_int32_t), sp(1), sp(2), sp(3))
  rc = gbmg_create(g, prm, h)
  if (rc /= GBMG_OK) then
    write(*, '(a, a)') 'gbmg_create: ', gbmg_strerror(rc)
    stop 2
  end if

  ! replaces "call ppe_sor_init"
  rc = gbmg_set_rho(h, gbmg_field_of(rho(1,1,1), lx, ly), GBMG_MEM_HOST)
  if (rc /= GBMG_OK) then
    write(*, '(a, a)') 'gbmg_set_rho: ', gbmg_last_error(h)
    stop 3
  end if

  ! replaces "call ppe_sor_solver(p%glb%p_tol)": right-hand side, iteration
  ! and ns_momentum_correction
  fu = gbmg_field_of(u(0,1,1), lx, ly)
  fv = gbmg_field_of(v(1,0,1), lx, ly)
  fw = gbmg_field_of(w(1,1,0), lx, ly)
  fp = gbmg_field_of(p(1,1,1), lx, ly)
  rc = gbmg_project(h, fu, fv, fw, fp, dt, tol, GBMG_MEM_HOST, st)
  if (rc /= GBMG_OK) write(*, '(a, a, es12.4)') 'gbmg_project: ', gbmg_strerror(rc), st%rel_residual
  rc_div = gbmg_div_stats(h, fu, fv, fw, mx, mean, GBMG_MEM_HOST)
  rc = gbmg_destroy(h)

  ghosts_ok = 1
  if (any(p(1-ghc:0, :, :) /= sentinel) .or. any(p(nx+1:, :, :) /= sentinel)) ghosts_ok = 0
  if (any(p(:, 1-ghc:0, :) /= sentinel) .or. any(p(:, ny+1:, :) /= sentinel)) ghosts_ok = 0
  if (any(p(:, :, 1-ghc:0) /= sentinel) .or. any(p(:, :, nz+1:) /= sentinel)) ghosts_ok = 0
  if (any(u(1-ghc:-1, :, :) /= sentinel) .or. any(u(nx+1:, :, :) /= sentinel)) ghosts_ok = 0

  open(11, file=trim(fout), access='stream', form='unformatted', status='replace')
  write(11) int(st%status, c_int32_t), int(st%cycles, c_int32_t), int(rc_div, c_int32_t), &
            int(ghosts_ok, c_int32_t)
  write(11) st%rel_residual, mx, mean
  write(11) p(1:nx, 1:ny, 1:nz)
  write(11) u(0:nx, 1:ny, 1:nz)
  write(11) v(1:nx, 0:ny, 1:nz)
  write(11) w(1:nx, 1:ny, 0:nz)
  close(11)
  write(*, '(a, i0, a, es10.3, a, es10.3)') 'cycles ', st%cycles, '  rel_residual ', &
      st%rel_residual, '  max|div u| ', mx
end program dropin_ppe
