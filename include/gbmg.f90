! gbmg.f90 -- ISO_C_BINDING interface to the C ABI of gbmg.h.
!
! A Fortran host of the reference's two-phase solvers binds the GB300
! pressure-Poisson multigrid through this module: the types mirror the C
! structs field for field and every entry point of gbmg.h has an interface
! here.  Structs are passed by value where the C prototype takes them by
! value (gbmg_field) and by reference where it takes a pointer.
!
! Compile together with the host code, e.g.
!     gfortran -c gbmg.f90 && gfortran host.f90 gbmg.o -L<dir> -lgbmg
module gbmg
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: GBMG_OK = 0, GBMG_NOT_CONVERGED = 1, GBMG_DIVERGED = 2
  integer(c_int), parameter :: GBMG_INVALID_ARG = 3, GBMG_CUDA_ERROR = 4, GBMG_NO_DEVICE = 5
  integer(c_int), parameter :: GBMG_OUT_OF_MEMORY = 6, GBMG_STATE_ERROR = 7
  integer(c_int), parameter :: GBMG_PREC_FP64 = 0, GBMG_PREC_MIXED = 1
  integer(c_int), parameter :: GBMG_STOP_RELATIVE = 0, GBMG_STOP_RMS = 1, GBMG_STOP_INCREMENT = 2
  integer(c_int), parameter :: GBMG_MEM_HOST = 0, GBMG_MEM_DEVICE = 1
  integer(c_int), parameter :: GBMG_PROF_CLASSES = 12

  type, bind(c) :: gbmg_grid
    integer(c_int32_t) :: nx, ny, nz
    real(c_double)     :: dx, dy, dz
  end type

  type, bind(c) :: gbmg_params
    integer(c_int32_t) :: precision, nu1, nu2, levels, coarse_max, max_cycles
    integer(c_int32_t) :: krylov, use_graph, remove_rhs_mean, certify, device
    type(c_ptr)        :: stream
    integer(c_int32_t) :: stop_rule, zero_wall_faces, inner_cycles, split_restarts
  end type

  type, bind(c) :: gbmg_stats
    integer(c_int32_t) :: status, cycles, levels, coarse_n
    real(c_double)     :: rel_residual, rms_residual, res0, ms, bytes, increment
    integer(c_int32_t) :: device_loop, restarts
  end type

  type, bind(c) :: gbmg_field
    type(c_ptr)        :: data
    integer(c_int64_t) :: sy, sz
  end type

  ! the Adams-Bashforth momentum step (gbmg_ns_ab_step)
  type, bind(c) :: gbmg_ns_params
    integer(c_int32_t) :: ghost
    integer(c_int32_t) :: bc(6)        ! ubc(1:2), vbc(1:2), wbc(1:2)
    integer(c_int32_t) :: iterations
    integer(c_int32_t) :: adv_scheme   ! 0 second-order upwind, 1 QUICK
    real(c_double)     :: dt, re, fr, we, mu_12, gx, gy, gz, btn_g, btn_sf, p_tol
  end type

  type, bind(c) :: gbmg_ns_fields
    type(gbmg_field) :: u, v, w, u_old, v_old, w_old, su, sv, sw, su_old, sv_old, sw_old
    type(gbmg_field) :: rho, mu, delta, phi, nrm_x, nrm_y, nrm_z, curv, p
  end type

  type, bind(c) :: gbmg_ns_stats
    integer(c_int32_t) :: status, cycles
    real(c_double)     :: max_rel_residual, linf, l2f, ms
  end type

  interface
    subroutine gbmg_default_params(prm) bind(c, name="gbmg_default_params")
      import :: gbmg_params
      type(gbmg_params), intent(out) :: prm
    end subroutine

    integer(c_int) function gbmg_create(grid, prm, h) bind(c, name="gbmg_create")
      import :: c_int, c_ptr, gbmg_grid, gbmg_params
      type(gbmg_grid), intent(in)    :: grid
      type(gbmg_params), intent(in)  :: prm
      type(c_ptr), intent(out)       :: h
    end function

    integer(c_int) function gbmg_destroy(h) bind(c, name="gbmg_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_int) function gbmg_set_rho(h, rho, mem) bind(c, name="gbmg_set_rho")
      import :: c_int, c_ptr, gbmg_field
      type(c_ptr), value      :: h
      type(gbmg_field), value :: rho
      integer(c_int), value   :: mem
    end function

    integer(c_int) function gbmg_set_phi(h, phi, eps, rho_pos, rho_neg, mem) &
        bind(c, name="gbmg_set_phi")
      import :: c_int, c_ptr, c_double, gbmg_field
      type(c_ptr), value      :: h
      type(gbmg_field), value :: phi
      real(c_double), value   :: eps, rho_pos, rho_neg
      integer(c_int), value   :: mem
    end function

    integer(c_int) function gbmg_set_coef(h, cx, cy, cz, mem) bind(c, name="gbmg_set_coef")
      import :: c_int, c_ptr, gbmg_field
      type(c_ptr), value      :: h
      type(gbmg_field), value :: cx, cy, cz
      integer(c_int), value   :: mem
    end function

    integer(c_int) function gbmg_solve(h, b, p, tol, mem, st) bind(c, name="gbmg_solve")
      import :: c_int, c_ptr, c_double, gbmg_field, gbmg_stats
      type(c_ptr), value      :: h
      type(gbmg_field), value :: b, p
      real(c_double), value   :: tol
      integer(c_int), value   :: mem
      type(gbmg_stats), intent(out) :: st
    end function

    integer(c_int) function gbmg_project(h, u, v, w, p, dt, tol, mem, st) &
        bind(c, name="gbmg_project")
      import :: c_int, c_ptr, c_double, gbmg_field, gbmg_stats
      type(c_ptr), value      :: h
      type(gbmg_field), value :: u, v, w, p
      real(c_double), value   :: dt, tol
      integer(c_int), value   :: mem
      type(gbmg_stats), intent(out) :: st
    end function

    integer(c_int) function gbmg_set_split(h, rho, rho_12, mem) bind(c, name="gbmg_set_split")
      import :: c_int, c_ptr, c_double, gbmg_field
      type(c_ptr), value      :: h
      type(gbmg_field), value :: rho
      real(c_double), value   :: rho_12
      integer(c_int), value   :: mem
    end function

    integer(c_int) function gbmg_project_split(h, u, v, w, p_hat, p, dt, tol, mem, st) &
        bind(c, name="gbmg_project_split")
      import :: c_int, c_ptr, c_double, gbmg_field, gbmg_stats
      type(c_ptr), value      :: h
      type(gbmg_field), value :: u, v, w, p_hat, p
      real(c_double), value   :: dt, tol
      integer(c_int), value   :: mem
      type(gbmg_stats), intent(out) :: st
    end function

    integer(c_int) function gbmg_divergence(h, u, v, w, dt, b, mem) &
        bind(c, name="gbmg_divergence")
      import :: c_int, c_ptr, c_double, gbmg_field
      type(c_ptr), value      :: h
      type(gbmg_field), value :: u, v, w
      real(c_double), value   :: dt
      type(gbmg_field), value :: b
      integer(c_int), value   :: mem
    end function

    integer(c_int) function gbmg_residual(h, b, p, r, norm2, mem) bind(c, name="gbmg_residual")
      import :: c_int, c_ptr, c_double, gbmg_field
      type(c_ptr), value      :: h
      type(gbmg_field), value :: b, p, r
      real(c_double), intent(out) :: norm2
      integer(c_int), value   :: mem
    end function

    integer(c_int) function gbmg_div_stats(h, u, v, w, max_div, mean_div, mem) &
        bind(c, name="gbmg_div_stats")
      import :: c_int, c_ptr, c_double, gbmg_field
      type(c_ptr), value      :: h
      type(gbmg_field), value :: u, v, w
      real(c_double), intent(out) :: max_div, mean_div
      integer(c_int), value   :: mem
    end function

    integer(c_int) function gbmg_div_stats_noalloc(grid, u, v, w, max_div, mean_div, device, &
        stream, err, err_len) bind(c, name="gbmg_div_stats_noalloc")
      import :: c_int, c_ptr, c_double, c_char, c_size_t, gbmg_grid, gbmg_field
      type(gbmg_grid), intent(in) :: grid
      type(gbmg_field), value :: u, v, w
      real(c_double), intent(out) :: max_div, mean_div
      integer(c_int), value   :: device
      type(c_ptr), value      :: stream
      character(kind=c_char)  :: err(*)
      integer(c_size_t), value :: err_len
    end function

    integer(c_int) function gbmg_adjoint(h, p, lam, phi, eps, rho_pos, rho_neg, grad_rho, &
        grad_phi, mem) bind(c, name="gbmg_adjoint")
      import :: c_int, c_ptr, c_double, gbmg_field
      type(c_ptr), value      :: h
      type(gbmg_field), value :: p, lam, phi
      real(c_double), value   :: eps, rho_pos, rho_neg
      type(gbmg_field), value :: grad_rho, grad_phi
      integer(c_int), value   :: mem
    end function

    integer(c_int) function gbmg_level_coef(h, level, cx, cy, cz, mem) &
        bind(c, name="gbmg_level_coef")
      import :: c_int, c_ptr, gbmg_field
      type(c_ptr), value      :: h
      integer(c_int), value   :: level
      type(gbmg_field), value :: cx, cy, cz
      integer(c_int), value   :: mem
    end function

    integer(c_int) function gbmg_level_dims(h, levels, dims, max_levels) &
        bind(c, name="gbmg_level_dims")
      import :: c_int, c_int32_t, c_ptr
      type(c_ptr), value        :: h
      integer(c_int32_t), intent(out) :: levels
      integer(c_int32_t)        :: dims(*)
      integer(c_int32_t), value :: max_levels
    end function

    integer(c_int64_t) function gbmg_kernel_launches(h) bind(c, name="gbmg_kernel_launches")
      import :: c_int64_t, c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_int) function gbmg_set_profiling(h, on) bind(c, name="gbmg_set_profiling")
      import :: c_int, c_ptr
      type(c_ptr), value    :: h
      integer(c_int), value :: on
    end function

    integer(c_int) function gbmg_profile(h, ms, launches, n) bind(c, name="gbmg_profile")
      import :: c_int, c_int32_t, c_int64_t, c_double, c_ptr
      type(c_ptr), value        :: h
      real(c_double)            :: ms(*)
      integer(c_int64_t)        :: launches(*)
      integer(c_int32_t), value :: n
    end function

    ! level-set transport (a separate handle, gbmg_ls)
    integer(c_int) function gbmg_ls_create(grid, device, stream, ls) bind(c, name="gbmg_ls_create")
      import :: c_int, c_ptr, gbmg_grid
      type(gbmg_grid), intent(in) :: grid
      integer(c_int), value   :: device
      type(c_ptr), value      :: stream
      type(c_ptr), intent(out) :: ls
    end function

    integer(c_int) function gbmg_ls_destroy(ls) bind(c, name="gbmg_ls_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: ls
    end function

    integer(c_int) function gbmg_ls_advect(ls, phi, u, v, w, dt, steps, mem) &
        bind(c, name="gbmg_ls_advect")
      import :: c_int, c_ptr, c_double, gbmg_field
      type(c_ptr), value      :: ls
      type(gbmg_field), value :: phi, u, v, w
      real(c_double), value   :: dt
      integer(c_int), value   :: steps, mem
    end function

    integer(c_int) function gbmg_ls_redistance(ls, phi, ls_wid, rdt, rho_12, btn, max_iter, mem, &
        iters, last_change) bind(c, name="gbmg_ls_redistance")
      import :: c_int, c_int32_t, c_ptr, c_double, gbmg_field
      type(c_ptr), value      :: ls
      type(gbmg_field), value :: phi
      real(c_double), value   :: ls_wid, rdt, rho_12
      integer(c_int), value   :: btn, max_iter, mem
      integer(c_int32_t), intent(out) :: iters
      real(c_double), intent(out) :: last_change
    end function

    integer(c_int) function gbmg_ns_ab_step(h, prm, f, mem, st) bind(c, name="gbmg_ns_ab_step")
      import :: c_int, c_ptr, gbmg_ns_params, gbmg_ns_fields, gbmg_ns_stats
      type(c_ptr), value :: h
      type(gbmg_ns_params), intent(in) :: prm
      type(gbmg_ns_fields), intent(in) :: f
      integer(c_int), value :: mem
      type(gbmg_ns_stats), intent(out) :: st
    end function

    integer(c_int) function gbmg_ns_ab_predict(h, prm, f, mem) bind(c, name="gbmg_ns_ab_predict")
      import :: c_int, c_ptr, gbmg_ns_params, gbmg_ns_fields
      type(c_ptr), value :: h
      type(gbmg_ns_params), intent(in) :: prm
      type(gbmg_ns_fields), intent(in) :: f
      integer(c_int), value :: mem
    end function

    integer(c_int) function gbmg_ns_velbc(h, prm, u, v, w, mem) bind(c, name="gbmg_ns_velbc")
      import :: c_int, c_ptr, gbmg_ns_params, gbmg_field
      type(c_ptr), value :: h
      type(gbmg_ns_params), intent(in) :: prm
      type(gbmg_field), value :: u, v, w
      integer(c_int), value :: mem
    end function

    integer(c_int) function gbmg_ns_curvature(h, prm, phi, nrm_x, nrm_y, nrm_z, curv, mem) &
        bind(c, name="gbmg_ns_curvature")
      import :: c_int, c_ptr, gbmg_ns_params, gbmg_field
      type(c_ptr), value :: h
      type(gbmg_ns_params), intent(in) :: prm
      type(gbmg_field), value :: phi, nrm_x, nrm_y, nrm_z, curv
      integer(c_int), value :: mem
    end function

    integer(c_int) function gbmg_ns_rho_mu(h, prm, phi, ls_wid, rho_12, rho, mu, delta, mem) &
        bind(c, name="gbmg_ns_rho_mu")
      import :: c_int, c_ptr, c_double, gbmg_ns_params, gbmg_field
      type(c_ptr), value :: h
      type(gbmg_ns_params), intent(in) :: prm
      type(gbmg_field), value :: phi, rho, mu, delta
      real(c_double), value :: ls_wid, rho_12
      integer(c_int), value :: mem
    end function

    integer(c_int) function gbmg_ns_mass_correct(h, prm, phi, ls_wid, rho_12, imass, iterations, &
        mem, mass) bind(c, name="gbmg_ns_mass_correct")
      import :: c_int, c_ptr, c_double, gbmg_ns_params, gbmg_field
      type(c_ptr), value :: h
      type(gbmg_ns_params), intent(in) :: prm
      type(gbmg_field), value :: phi
      real(c_double), value :: ls_wid, rho_12, imass
      integer(c_int), value :: iterations, mem
      real(c_double), intent(out) :: mass
    end function

    integer(c_int) function gbmg_ns_vof_advect(h, prm, vof, vof_old, u_old, v_old, w_old, phi, &
        mem) bind(c, name="gbmg_ns_vof_advect")
      import :: c_int, c_ptr, gbmg_ns_params, gbmg_field
      type(c_ptr), value :: h
      type(gbmg_ns_params), intent(in) :: prm
      type(gbmg_field), value :: vof, vof_old, u_old, v_old, w_old, phi
      integer(c_int), value :: mem
    end function

    integer(c_int) function gbmg_ns_ibm(h, prm, solid, w_body, u, v, w, mem) &
        bind(c, name="gbmg_ns_ibm")
      import :: c_int, c_ptr, c_double, gbmg_ns_params, gbmg_field
      type(c_ptr), value :: h
      type(gbmg_ns_params), intent(in) :: prm
      type(gbmg_field), value :: solid, u, v, w
      real(c_double), value :: w_body
      integer(c_int), value :: mem
    end function

    integer(c_int) function gbmg_ns_bc(h, prm, a, mem) bind(c, name="gbmg_ns_bc")
      import :: c_int, c_ptr, gbmg_ns_params, gbmg_field
      type(c_ptr), value :: h
      type(gbmg_ns_params), intent(in) :: prm
      type(gbmg_field), value :: a
      integer(c_int), value :: mem
    end function

    integer(c_int64_t) function gbmg_ls_kernel_launches(ls) bind(c, name="gbmg_ls_kernel_launches")
      import :: c_int64_t, c_ptr
      type(c_ptr), value :: ls
    end function

    type(c_ptr) function gbmg_ls_last_error_c(ls) bind(c, name="gbmg_ls_last_error")
      import :: c_ptr
      type(c_ptr), value :: ls
    end function

    type(c_ptr) function gbmg_strerror_c(status) bind(c, name="gbmg_strerror")
      import :: c_int, c_ptr
      integer(c_int), value :: status
    end function

    type(c_ptr) function gbmg_last_error_c(h) bind(c, name="gbmg_last_error")
      import :: c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_size_t) function gbmg_c_strlen(s) bind(c, name="strlen")
      import :: c_size_t, c_ptr
      type(c_ptr), value :: s
    end function
  end interface

contains

  ! A cell or face array of the reference's ghost-padded layout as a
  ! gbmg_field: first is element (1,1,1) of a cell array (or (0,1,1), (1,0,1),
  ! (1,1,0) of the u, v, w face arrays), lx and ly the padded extents of the
  ! first two dimensions (nx + 2*ghc, ny + 2*ghc).  The array must stay
  ! allocated (and should have the TARGET attribute) for as long as the field
  ! is used; the library keeps no pointer after a call returns.
  function gbmg_field_of(first, lx, ly) result(f)
    real(c_double), target, intent(in) :: first
    integer, intent(in) :: lx, ly
    type(gbmg_field) :: f
    f%data = c_loc(first)
    f%sy = int(lx, c_int64_t)
    f%sz = int(lx, c_int64_t) * int(ly, c_int64_t)
  end function

  ! The unused field (data = NULL), e.g. w of a 2D grid or phi of gbmg_adjoint.
  function gbmg_no_field() result(f)
    type(gbmg_field) :: f
    f%data = c_null_ptr
    f%sy = 1_c_int64_t
    f%sz = 1_c_int64_t
  end function

  function gbmg_c_string(s) result(text)
    type(c_ptr), intent(in) :: s
    character(len=:), allocatable :: text
    character(kind=c_char), pointer :: chars(:)
    integer :: i, n
    if (.not. c_associated(s)) then
      text = ""
      return
    end if
    n = int(gbmg_c_strlen(s))
    call c_f_pointer(s, chars, [n])
    allocate(character(len=n) :: text)
    do i = 1, n
      text(i:i) = chars(i)
    end do
  end function

  function gbmg_strerror(status) result(text)
    integer(c_int), intent(in) :: status
    character(len=:), allocatable :: text
    text = gbmg_c_string(gbmg_strerror_c(status))
  end function

  function gbmg_last_error(h) result(text)
    type(c_ptr), intent(in) :: h
    character(len=:), allocatable :: text
    text = gbmg_c_string(gbmg_last_error_c(h))
  end function

end module gbmg
