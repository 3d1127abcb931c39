!> FLINT_GPU -- ISO_C_BINDING interface to the GB300 chemistry library (flint_gpu.h).
!>
!> A FLINT caller replaces
!>   read_idealgas_thermo / read_chemistry / Assign_Mechanism  -> flint_mech_create
!>   the same readers on a folder of tabulated input files     -> flint_mech_create_from_files
!>   a mechanism held as one IR byte string                    -> flint_mech_create_from_ir
!>   loop over cells of chemistry_source(roi, T, omegadot)    -> flint_chemistry_source_batch
!>   loop over cells of run_odesolver(neq, tin, tout, Z, rhs_native, err)
!>                                                            -> flint_reactor_advance_host
!>   free_chemistry_data                                       -> flint_mech_destroy
!> Arrays are Fortran column-major: roi(ns, ncells), Y(ns, ncells),
!> jac(ns+1, ns+1, ncells) -- the library's FLINT_CELL_MAJOR layout.
!> No Fortran compiler exists in the build images of this project, so this
!> module is checked only by the symbol test (tests/test_abi_cpu.py).
module FLINT_GPU
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: FLINT_OK = 0
  integer(c_int), parameter :: FLINT_CELL_MAJOR = 0, FLINT_SPECIES_MAJOR = 1

  type, bind(C) :: flint_mech_desc
    integer(c_int) :: ns, nr
    type(c_ptr) :: mw, nasa7, rtype, reversible, arrh, arrh0, troe
    type(c_ptr) :: rsp, rnu, rord, psp, pnu, eff
    real(c_double) :: r_eos, r_thermo, p_ref
    type(c_ptr) :: nasa9 = c_null_ptr   ! optional NASA-9 rows (ns, 32)
  end type flint_mech_desc

  ! mirror of flint_table_desc: FLINT's module arrays by c_loc, in their own layout
  type, bind(C) :: flint_table_desc
    integer(c_int) :: ns, nr_arrh, nr_troe, nr_lind, tmin, tmax, ti1, ti2
    type(c_ptr) :: wm, cp_tab, h_tab, kf_tab, kb_tab
    type(c_ptr) :: kinf_troe, k0_troe, kc_troe, fcent_troe, kinf_lind, k0_lind, kc_lind
    type(c_ptr) :: ni1_arrh, ni2_arrh, eps_arrh, ni1_troe, ni2_troe, eps_troe
    type(c_ptr) :: ni1_lind, ni2_lind, eps_lind
    real(c_double) :: runiv
    type(c_ptr) :: mi_tab = c_null_ptr, k_tab = c_null_ptr   ! optional transport tables
  end type flint_table_desc

  type, bind(C) :: flint_reactor_opts
    real(c_double) :: rtol, atol
    integer(c_int) :: max_steps, max_order, constant_volume, reserved
    real(c_double) :: tmin, tmax
  end type flint_reactor_opts

  interface
    integer(c_int) function flint_mech_create(desc, mech) bind(C, name='flint_mech_create')
      import :: c_int, c_ptr, flint_mech_desc
      type(flint_mech_desc), intent(in) :: desc
      type(c_ptr), intent(out) :: mech
    end function

    integer(c_int) function flint_mech_create_tables(desc, mech) bind(C, name='flint_mech_create_tables')
      import :: c_int, c_ptr, flint_table_desc
      type(flint_table_desc), intent(in) :: desc
      type(c_ptr), intent(out) :: mech
    end function

    ! folder and prefix: NUL-terminated, e.g. trim(dir)//c_null_char
    integer(c_int) function flint_mech_create_from_files(folder, prefix, mech) &
        bind(C, name='flint_mech_create_from_files')
      import :: c_int, c_char, c_ptr
      character(kind=c_char), dimension(*), intent(in) :: folder, prefix
      type(c_ptr), intent(out) :: mech
    end function

    ! blob: the mechanism IR bytes (layout in flint_gpu.h), nbytes its length
    integer(c_int) function flint_mech_create_from_ir(blob, nbytes, mech) &
        bind(C, name='flint_mech_create_from_ir')
      import :: c_int, c_int8_t, c_int64_t, c_ptr
      integer(c_int8_t), dimension(*), intent(in) :: blob
      integer(c_int64_t), value :: nbytes
      type(c_ptr), intent(out) :: mech
    end function

    integer(c_int) function flint_mech_destroy(mech) bind(C, name='flint_mech_destroy')
      import :: c_int, c_ptr
      type(c_ptr), value :: mech
    end function

    type(c_ptr) function flint_last_error() bind(C, name='flint_last_error')
      import :: c_ptr
    end function

    integer(c_int) function flint_chemistry_source_batch(mech, n, roi, temp, omegadot, stream) &
        bind(C, name='flint_chemistry_source_batch')
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: mech, roi, temp, omegadot, stream
      integer(c_int64_t), value :: n
    end function

    ! Wilke viscosity and conductivity over ncells on device arrays (rhoi: (ns, ncells))
    ! device arrays below (c_ptr by value); stream: a cudaStream_t or c_null_ptr
    integer(c_int) function flint_rhs_native_batch(mech, n, Z, F, stream) &
        bind(C, name='flint_rhs_native_batch')
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: mech, Z, F, stream
      integer(c_int64_t), value :: n
    end function

    integer(c_int) function flint_thermo_batch(mech, n, layout, temp, Y, cp, h, stream) &
        bind(C, name='flint_thermo_batch')
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: mech, temp, Y, cp, h, stream
      integer(c_int64_t), value :: n
      integer(c_int), value :: layout
    end function

    integer(c_int) function flint_species_thermo_batch(mech, n, temp, cp, h, s, g, stream) &
        bind(C, name='flint_species_thermo_batch')
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: mech, temp, cp, h, s, g, stream
      integer(c_int64_t), value :: n
    end function

    integer(c_int) function flint_wdot_batch(mech, n, layout, temp, p, Y, wdot, cp, h, stream) &
        bind(C, name='flint_wdot_batch')
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: mech, temp, p, Y, wdot, cp, h, stream
      integer(c_int64_t), value :: n
      integer(c_int), value :: layout
    end function

    integer(c_int) function flint_wdot_jac_batch(mech, n, layout, temp, p, Y, wdot, jac, stream) &
        bind(C, name='flint_wdot_jac_batch')
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: mech, temp, p, Y, wdot, jac, stream
      integer(c_int64_t), value :: n
      integer(c_int), value :: layout
    end function

    integer(c_int) function flint_reactor_advance(mech, n, temp, p, Y, dt, opts, status, nsteps, stream) &
        bind(C, name='flint_reactor_advance')
      import :: c_int, c_int64_t, c_ptr, flint_reactor_opts
      type(c_ptr), value :: mech, temp, p, Y, dt, status, nsteps, stream
      integer(c_int64_t), value :: n
      type(flint_reactor_opts), intent(in) :: opts
    end function

    ! flint_reactor_advance without any device allocation (scratch in a static
    ! 10 MiB + 256 B device array, up to 31 species, one call at a time on the
    ! GPU).  Call it once with n = 0 before the solver's pool reserves its
    ! device memory and before any stream capture: that call does the set-up.
    integer(c_int) function flint_reactor_advance_noalloc(mech, n, temp, p, Y, dt, opts, status, nsteps, &
        stream) bind(C, name='flint_reactor_advance_noalloc')
      import :: c_int, c_int64_t, c_ptr, flint_reactor_opts
      type(c_ptr), value :: mech, temp, p, Y, dt, status, nsteps, stream
      integer(c_int64_t), value :: n
      type(flint_reactor_opts), intent(in) :: opts
    end function

    integer(c_int) function flint_transport_batch(mech, n, rhoi, temp, mu, lambda, stream) &
        bind(C, name='flint_transport_batch')
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: mech, rhoi, temp, mu, lambda, stream
      integer(c_int64_t), value :: n
    end function

    ! cons2prim over ncells on device arrays (cons, prim: (ns+ndim+1, ncells))
    integer(c_int) function flint_cons2prim_batch(mech, n, ndim, cons, temp, prim, temp_out, stream) &
        bind(C, name='flint_cons2prim_batch')
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: mech, cons, temp, prim, temp_out, stream
      integer(c_int64_t), value :: n
      integer(c_int), value :: ndim
    end function

    integer(c_int) function flint_wdot_batch_host(mech, n, layout, temp, p, Y, wdot, cp, h) &
        bind(C, name='flint_wdot_batch_host')
      import :: c_int, c_int64_t, c_double, c_ptr
      type(c_ptr), value :: mech
      integer(c_int64_t), value :: n
      integer(c_int), value :: layout
      real(c_double), intent(in) :: temp(*), p(*), Y(*)
      real(c_double), intent(out) :: wdot(*), cp(*), h(*)
    end function

    integer(c_int) function flint_wdot_jac_batch_host(mech, n, layout, temp, p, Y, wdot, jac) &
        bind(C, name='flint_wdot_jac_batch_host')
      import :: c_int, c_int64_t, c_double, c_ptr
      type(c_ptr), value :: mech
      integer(c_int64_t), value :: n
      integer(c_int), value :: layout
      real(c_double), intent(in) :: temp(*), p(*), Y(*)
      real(c_double), intent(out) :: wdot(*), jac(*)
    end function

    integer(c_int) function flint_reactor_advance_host(mech, n, temp, p, Y, dt, opts, status, nsteps) &
        bind(C, name='flint_reactor_advance_host')
      import :: c_int, c_int64_t, c_double, c_ptr, flint_reactor_opts
      type(c_ptr), value :: mech
      integer(c_int64_t), value :: n
      real(c_double), intent(inout) :: temp(*), Y(*)
      real(c_double), intent(in) :: p(*), dt(*)
      type(flint_reactor_opts), intent(in) :: opts
      integer(c_int), intent(out) :: status(*), nsteps(*)
    end function

    subroutine flint_reactor_default_opts(opts) bind(C, name='flint_reactor_default_opts')
      import :: flint_reactor_opts
      type(flint_reactor_opts), intent(out) :: opts
    end subroutine
  end interface
end module FLINT_GPU
