! mo_ed_bind.f90 -- Fortran 2008 bindings of the GB300 ED solver's C-ABI.
!
! Two modules:
!   mo_ed_bind  -- one bind(C) interface per entry point of include/mo_ed.h,
!                  plus the bind(C) options record.
!   mo_ed_gpu   -- procedures with the argument lists of the MO-DMFT routines
!                  they replace, on one module-level context.  A nonzero
!                  status prints the library message and stops, as the
!                  reference's die does.
!
! External procedures FUNC, dfunc and minimization (func.f90:1, :47, :144)
! keep the reference's implicit interfaces and argument order (nwloc and Ns
! are swapped between FUNC and dfunc there, and here).  The MPI communicator
! argument is accepted and ignored: the solver runs on one GPU.
!
! Arrays are passed as the reference holds them: column-major, 1-based,
! double complex as interleaved (re, im) pairs.

module mo_ed_bind
    use iso_c_binding
    implicit none

    integer(c_int), parameter :: MO_ED_OK = 0
    integer(c_int), parameter :: MO_ED_FP64 = 0
    integer(c_int), parameter :: MO_ED_FP32 = 1

    type, bind(C) :: mo_ed_options
        integer(c_int) :: nstep
        integer(c_int) :: nev
        real(c_double) :: beta
        integer(c_int) :: precision
        integer(c_int) :: fortran_cmplx
        integer(c_int) :: gs_ncv
        integer(c_int) :: gs_maxcycles
        real(c_double) :: gs_tol
        integer(c_int) :: green_reorth
        integer(c_int) :: green_fp64
        integer(c_int) :: solve_threads
        integer(c_int) :: fit_quantum
        integer(c_int) :: reserved(5)
    end type mo_ed_options

    interface
        integer(c_int) function mo_ed_create(ctx, device, stream) bind(C, name="mo_ed_create")
            import :: c_int, c_ptr
            type(c_ptr), intent(out) :: ctx
            integer(c_int), value :: device
            type(c_ptr), value :: stream
        end function
        integer(c_int) function mo_ed_destroy(ctx) bind(C, name="mo_ed_destroy")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        type(c_ptr) function mo_ed_last_error(ctx) bind(C, name="mo_ed_last_error")
            import :: c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function mo_ed_default_options(opt) bind(C, name="mo_ed_default_options")
            import :: c_int, mo_ed_options
            type(mo_ed_options), intent(out) :: opt
        end function
        integer(c_int) function mo_ed_set_options(ctx, opt) bind(C, name="mo_ed_set_options")
            import :: c_int, c_ptr, mo_ed_options
            type(c_ptr), value :: ctx
            type(mo_ed_options), intent(in) :: opt
        end function
        integer(c_int) function mo_ed_set_model(ctx, norb, nbath, u, jex, ek, vk) &
                bind(C, name="mo_ed_set_model")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: norb, nbath
            real(c_double), value :: u, jex
            real(c_double), intent(in) :: ek(*), vk(*)
        end function
        integer(c_int) function mo_ed_set_sectors(ctx, nsector, nelec, nup) &
                bind(C, name="mo_ed_set_sectors")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), value :: nsector
            integer(c_int), intent(in) :: nelec(*), nup(*)
        end function
        integer(c_int) function mo_ed_set_omega(ctx, nw, omega) bind(C, name="mo_ed_set_omega")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: nw
            real(c_double), intent(in) :: omega(*)
        end function
        integer(c_long_long) function mo_ed_icom(n, m) bind(C, name="mo_ed_icom")
            import :: c_int, c_long_long
            integer(c_int), value :: n, m
        end function
        integer(c_int) function mo_ed_sector_dims(ctx, ne_up, ne_down, nup, ndown, ntot) &
                bind(C, name="mo_ed_sector_dims")
            import :: c_int, c_ptr, c_long_long
            type(c_ptr), value :: ctx
            integer(c_int), value :: ne_up, ne_down
            integer(c_int), intent(out) :: nup, ndown
            integer(c_long_long), intent(out) :: ntot
        end function
        integer(c_int) function mo_ed_generate_basis(ctx, ne_up, ne_down, up, down, idx_up, idx_down) &
                bind(C, name="mo_ed_generate_basis")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), value :: ne_up, ne_down
            integer(c_int), intent(out) :: up(*), down(*), idx_up(*), idx_down(*)
        end function
        integer(c_int) function mo_ed_basis_get(ctx, ne_up, ne_down, n, idx, state) &
                bind(C, name="mo_ed_basis_get")
            import :: c_int, c_ptr, c_long_long
            type(c_ptr), value :: ctx
            integer(c_int), value :: ne_up, ne_down
            integer(c_long_long), value :: n
            integer(c_long_long), intent(in) :: idx(*)
            integer(c_int), intent(out) :: state(*)
        end function
        integer(c_int) function mo_ed_basis_idx(ctx, ne_up, ne_down, n, state, idx) &
                bind(C, name="mo_ed_basis_idx")
            import :: c_int, c_ptr, c_long_long
            type(c_ptr), value :: ctx
            integer(c_int), value :: ne_up, ne_down
            integer(c_long_long), value :: n
            integer(c_int), intent(in) :: state(*)
            integer(c_long_long), intent(out) :: idx(*)
        end function
        integer(c_int) function mo_ed_multiply_h(ctx, ne_up, ne_down, a, b) &
                bind(C, name="mo_ed_multiply_h")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: ne_up, ne_down
            real(c_double), intent(in) :: a(*)
            real(c_double), intent(out) :: b(*)
        end function
        integer(c_int) function mo_ed_apply_c(ctx, ne_up, ne_down, vec, pm, iorb, ispin, vec_out, &
                capacity, ntot_out) bind(C, name="mo_ed_apply_c")
            import :: c_int, c_ptr, c_double, c_long_long
            type(c_ptr), value :: ctx
            integer(c_int), value :: ne_up, ne_down, pm, iorb, ispin
            real(c_double), intent(in) :: vec(*)
            real(c_double), intent(out) :: vec_out(*)
            integer(c_long_long), value :: capacity
            integer(c_long_long), intent(out) :: ntot_out
        end function
        integer(c_int) function mo_ed_lanczos_iteration(ctx, ne_up, ne_down, vec, nstep_calc, a, b) &
                bind(C, name="mo_ed_lanczos_iteration")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: ne_up, ne_down
            real(c_double), intent(in) :: vec(*)
            integer(c_int), intent(out) :: nstep_calc
            real(c_double), intent(out) :: a(*), b(*)
        end function
        integer(c_int) function mo_ed_diag(ctx, ne_up, ne_down, nev, eigval, eigvec) &
                bind(C, name="mo_ed_diag")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: ne_up, ne_down, nev
            real(c_double), intent(out) :: eigval(*), eigvec(*)
        end function
        integer(c_int) function mo_ed_solve(ctx, nev_calc, val, prob, sector, level, capacity) &
                bind(C, name="mo_ed_solve")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), intent(out) :: nev_calc
            real(c_double), intent(out) :: val(*), prob(*)
            integer(c_int), intent(out) :: sector(*), level(*)
            integer(c_int), value :: capacity
        end function
        integer(c_int) function mo_ed_calc_green_ftn(ctx, gr) bind(C, name="mo_ed_calc_green_ftn")
            import :: c_int, c_ptr, c_double_complex
            type(c_ptr), value :: ctx
            complex(c_double_complex), intent(out) :: gr(*)
        end function
        integer(c_int) function mo_ed_func(ctx, x, ns, nwloc, nxsize, omega, d_ev, nbath, norb, f) &
                bind(C, name="mo_ed_func")
            import :: c_int, c_ptr, c_double, c_double_complex
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: x(*), omega(*)
            integer(c_int), value :: ns, nwloc, nxsize, nbath, norb
            complex(c_double_complex), intent(in) :: d_ev(*)
            real(c_double), intent(out) :: f
        end function
        integer(c_int) function mo_ed_dfunc(ctx, x, p, nwloc, ns, nxsize, omega, d_ev, nbath, norb) &
                bind(C, name="mo_ed_dfunc")
            import :: c_int, c_ptr, c_double, c_double_complex
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: x(*), omega(*)
            real(c_double), intent(out) :: p(*)
            integer(c_int), value :: nwloc, ns, nxsize, nbath, norb
            complex(c_double_complex), intent(in) :: d_ev(*)
        end function
        integer(c_int) function mo_ed_minimization(ctx, x, nwloc, ns, nxsize, omega, d_ev, nbath, &
                norb, fret, iter) bind(C, name="mo_ed_minimization")
            import :: c_int, c_ptr, c_double, c_double_complex
            type(c_ptr), value :: ctx
            real(c_double), intent(inout) :: x(*)
            integer(c_int), value :: nwloc, ns, nxsize, nbath, norb
            real(c_double), intent(in) :: omega(*)
            complex(c_double_complex), intent(in) :: d_ev(*)
            real(c_double), intent(out) :: fret
            integer(c_int), intent(out) :: iter
        end function
        integer(c_int) function mo_ed_calc_dev(ctx, norb, nsite, nwloc, omega, ek, vk, ef, d_ev) &
                bind(C, name="mo_ed_calc_dev")
            import :: c_int, c_ptr, c_double, c_double_complex
            type(c_ptr), value :: ctx
            integer(c_int), value :: norb, nsite, nwloc
            real(c_double), intent(in) :: omega(*), ek(*), vk(*), ef(*)
            complex(c_double_complex), intent(out) :: d_ev(*)
        end function
        integer(c_int) function mo_ed_set_band_structure(ctx, nq, ef) &
                bind(C, name="mo_ed_set_band_structure")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: nq
            real(c_double), intent(out) :: ef(*)
        end function
        integer(c_int) function mo_ed_delta_new(ctx, nwloc, rmu, gr, d_ev, gksum) &
                bind(C, name="mo_ed_delta_new")
            import :: c_int, c_ptr, c_double, c_double_complex
            type(c_ptr), value :: ctx
            integer(c_int), value :: nwloc
            real(c_double), value :: rmu
            complex(c_double_complex), intent(in) :: gr(*)
            complex(c_double_complex), intent(inout) :: d_ev(*)
            complex(c_double_complex), intent(out) :: gksum(*)
        end function
        integer(c_int) function mo_ed_n_from_gksum(ctx, nw, gksum, beta, nocc) &
                bind(C, name="mo_ed_n_from_gksum")
            import :: c_int, c_ptr, c_double, c_double_complex
            type(c_ptr), value :: ctx
            integer(c_int), value :: nw
            complex(c_double_complex), intent(in) :: gksum(*)
            real(c_double), value :: beta
            real(c_double), intent(out) :: nocc(*)
        end function
        integer(c_int) function mo_ed_dos(ctx, nw, omega_real, small, weighted, aff) &
                bind(C, name="mo_ed_dos")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: nw, weighted
            real(c_double), intent(in) :: omega_real(*)
            real(c_double), value :: small
            real(c_double), intent(out) :: aff(*)
        end function
        integer(c_int) function mo_ed_export_eigvec(ctx, dir) bind(C, name="mo_ed_export_eigvec")
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: dir(*)
        end function
        integer(c_int) function mo_ed_import_eigvec(ctx, dir, nev_calc) bind(C, name="mo_ed_import_eigvec")
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: dir(*)
            integer(c_int), intent(out) :: nev_calc
        end function
        integer(c_int) function mo_ed_write_apbpanbn(ctx, path) bind(C, name="mo_ed_write_apbpanbn")
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: path(*)
        end function
        integer(c_int) function mo_ed_read_apbpanbn(ctx, path, nrec) bind(C, name="mo_ed_read_apbpanbn")
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: path(*)
            integer(c_int), intent(out) :: nrec
        end function
        integer(c_int) function mo_ed_ev_to_x(ek, vk, ef, ns, nbath, nxsize, x) &
                bind(C, name="mo_ed_ev_to_x")
            import :: c_int, c_double
            real(c_double), intent(in) :: ek(*), vk(*), ef(*)
            integer(c_int), value :: ns, nbath, nxsize
            real(c_double), intent(out) :: x(*)
        end function
        integer(c_int) function mo_ed_x_to_ev(x, nxsize, ns, nbath, norb, ef, ek, vk) &
                bind(C, name="mo_ed_x_to_ev")
            import :: c_int, c_double
            real(c_double), intent(in) :: x(*)
            integer(c_int), value :: nxsize, ns, nbath, norb
            real(c_double), intent(out) :: ef(*), ek(*), vk(*)
        end function
    end interface
end module mo_ed_bind


module mo_ed_gpu
    use iso_c_binding
    use mo_ed_bind
    implicit none
    private
    type(c_ptr), save :: ctx = c_null_ptr
    public :: mo_ed_gpu_init, mo_ed_gpu_finalize, mo_ed_gpu_context, mo_ed_gpu_check
    public :: mo_ed_gpu_set_problem, mo_ed_gpu_solve, mo_ed_gpu_green
    public :: mo_ed_gpu_multiply_h, mo_ed_gpu_lanczos, mo_ed_gpu_diag
    public :: mo_ed_gpu_set_band_structure, mo_ed_gpu_delta_new, mo_ed_gpu_dos
    public :: mo_ed_gpu_export_eigvec, mo_ed_gpu_import_eigvec, mo_ed_gpu_write_apbpanbn
contains

    ! Stop with the library's message on a nonzero status (the reference's die).
    subroutine mo_ed_gpu_check(status, where)
        integer(c_int), intent(in) :: status
        character(len=*), intent(in) :: where
        character(kind=c_char), pointer :: msg(:)
        integer :: n
        if (status == MO_ED_OK) return
        call c_f_pointer(mo_ed_last_error(ctx), msg, [4096])
        n = 0
        do while (n < 4096)
            if (msg(n + 1) == c_null_char) exit
            n = n + 1
        end do
        write(0, '(a, a, i0, a, 4096a1)') where, ': mo_ed status ', status, ': ', msg(1:n)
        error stop 1
    end subroutine

    subroutine mo_ed_gpu_init(device)
        integer, intent(in) :: device
        if (c_associated(ctx)) return
        call mo_ed_gpu_check(mo_ed_create(ctx, int(device, c_int), c_null_ptr), 'mo_ed_gpu_init')
    end subroutine

    subroutine mo_ed_gpu_finalize()
        integer(c_int) :: rc
        if (.not. c_associated(ctx)) return
        rc = mo_ed_destroy(ctx)
        ctx = c_null_ptr
    end subroutine

    type(c_ptr) function mo_ed_gpu_context()
        mo_ed_gpu_context = ctx
    end function

    ! ed_config globals (ed_config.f90:11-36) and the Matsubara grid
    ! (ed_green.F90:41-52): call once per DMFT iteration, after the bath
    ! parameters ek, vk changed.  vk is vk(1:Norb, Norb+1:Nsite).
    subroutine mo_ed_gpu_set_problem(Norb, Nbath, U, Jex, ek, vk, Nsector, Nelec, Nup, &
                                     Nstep, Nev, beta, nwloc, omega, use_fp64)
        integer, intent(in) :: Norb, Nbath, Nsector, Nelec(Nsector), Nup(Nsector)
        integer, intent(in) :: Nstep, Nev, nwloc
        double precision, intent(in) :: U, Jex, beta, ek(Norb + Nbath), vk(Norb, Nbath), omega(nwloc)
        logical, intent(in) :: use_fp64
        type(mo_ed_options) :: opt
        integer(c_int) :: ne(Nsector), nu(Nsector)
        call mo_ed_gpu_check(mo_ed_default_options(opt), 'mo_ed_default_options')
        opt%nstep = Nstep
        opt%nev = Nev
        opt%beta = beta
        if (use_fp64) then
            opt%precision = MO_ED_FP64
        else
            opt%precision = MO_ED_FP32
        end if
        call mo_ed_gpu_check(mo_ed_set_options(ctx, opt), 'mo_ed_set_options')
        call mo_ed_gpu_check(mo_ed_set_model(ctx, int(Norb, c_int), int(Nbath, c_int), U, Jex, ek, vk), &
                             'mo_ed_set_model')
        ne = int(Nelec, c_int)
        nu = int(Nup, c_int)
        call mo_ed_gpu_check(mo_ed_set_sectors(ctx, int(Nsector, c_int), ne, nu), 'mo_ed_set_sectors')
        call mo_ed_gpu_check(mo_ed_set_omega(ctx, int(nwloc, c_int), omega), 'mo_ed_set_omega')
    end subroutine

    ! ed_solve (ed_solver.F90:28-105): fills the fields of eigval_t and nev_calc.
    subroutine mo_ed_gpu_solve(capacity, val, prob, sector, level, nev_calc)
        integer, intent(in) :: capacity
        double precision, intent(out) :: val(capacity), prob(capacity)
        integer, intent(out) :: sector(capacity), level(capacity), nev_calc
        integer(c_int) :: nc, isec(capacity), ilev(capacity)
        call mo_ed_gpu_check(mo_ed_solve(ctx, nc, val, prob, isec, ilev, int(capacity, c_int)), 'ed_solve')
        nev_calc = nc
        sector = isec
        level = ilev
    end subroutine

    ! ed_calc_green_ftn (ed_green.F90:60-134): Gr(Norb, nwloc) of the last solve.
    subroutine mo_ed_gpu_green(Norb, nwloc, Gr)
        integer, intent(in) :: Norb, nwloc
        double complex, intent(out) :: Gr(Norb, nwloc)
        call mo_ed_gpu_check(mo_ed_calc_green_ftn(ctx, Gr), 'ed_calc_green_ftn')
    end subroutine

    ! ed_set_band_structure (ed_hamiltonian.F90:29-85): ef(Norb); the caller
    ! copies ef into ek(1:Norb) as the reference does.
    subroutine mo_ed_gpu_set_band_structure(Nq, Norb, ef)
        integer, intent(in) :: Nq, Norb
        double precision, intent(out) :: ef(Norb)
        call mo_ed_gpu_check(mo_ed_set_band_structure(ctx, int(Nq, c_int), ef), 'ed_set_band_structure')
    end subroutine

    ! ed_delta_new + n_from_gksum (ed_green.F90:187-253): D_ev updated in place,
    ! Gksum and the occupations returned.
    subroutine mo_ed_gpu_delta_new(Norb, nwloc, rMu, beta, Gr, D_ev, Gksum, nocc)
        integer, intent(in) :: Norb, nwloc
        double precision, intent(in) :: rMu, beta
        double complex, intent(in) :: Gr(Norb, nwloc)
        double complex, intent(inout) :: D_ev(Norb, nwloc)
        double complex, intent(out) :: Gksum(Norb, nwloc)
        double precision, intent(out) :: nocc(Norb)
        call mo_ed_gpu_check(mo_ed_delta_new(ctx, int(nwloc, c_int), rMu, Gr, D_ev, Gksum), 'ed_delta_new')
        call mo_ed_gpu_check(mo_ed_n_from_gksum(ctx, int(nwloc, c_int), Gksum, beta, nocc), 'n_from_gksum')
    end subroutine

    ! dos (dos.f90:1-106) from the last Green's function's records, without
    ! re-reading apbpanbn.dat; weighted = 0 is the reference's assignment.
    subroutine mo_ed_gpu_dos(Norb, Nw, omega_real, small, weighted, Aff)
        integer, intent(in) :: Norb, Nw, weighted
        double precision, intent(in) :: omega_real(Nw), small
        double precision, intent(out) :: Aff(Norb, Nw)
        call mo_ed_gpu_check(mo_ed_dos(ctx, int(Nw, c_int), omega_real, small, int(weighted, c_int), Aff), 'dos')
    end subroutine

    ! export_eigval + export_eigvec (ed_io.F90:13-56) of the kept states, in
    ! the current directory, file names as eigvec_filename.
    subroutine mo_ed_gpu_export_eigvec()
        call mo_ed_gpu_check(mo_ed_export_eigvec(ctx, c_null_char), 'export_eigvec')
    end subroutine

    ! import_eigval + import_eigvec (ed_io.F90:58-138): kept states read back.
    subroutine mo_ed_gpu_import_eigvec(nev_calc)
        integer, intent(out) :: nev_calc
        integer(c_int) :: n
        call mo_ed_gpu_check(mo_ed_import_eigvec(ctx, c_null_char, n), 'import_eigvec')
        nev_calc = n
    end subroutine

    ! apbpanbn.dat (ed_green.F90:112-115,125-128) of the last mo_ed_gpu_green.
    subroutine mo_ed_gpu_write_apbpanbn()
        call mo_ed_gpu_check(mo_ed_write_apbpanbn(ctx, 'apbpanbn.dat' // c_null_char), 'apbpanbn.dat')
    end subroutine

    ! multiply_H (ed_hamiltonian.F90:88-191) on a whole sector vector.
    subroutine mo_ed_gpu_multiply_h(ne_up, ne_down, ntot, A, B)
        integer, intent(in) :: ne_up, ne_down
        integer(c_long_long), intent(in) :: ntot
        double precision, intent(in) :: A(ntot)
        double precision, intent(out) :: B(ntot)
        call mo_ed_gpu_check(mo_ed_multiply_h(ctx, int(ne_up, c_int), int(ne_down, c_int), A, B), 'multiply_H')
    end subroutine

    ! lanczos_iteration (ed_lanczos.F90:14-68): a(0:Nstep), b(0:Nstep).
    subroutine mo_ed_gpu_lanczos(ne_up, ne_down, ntot, vec, Nstep, nstep_calc, a, b)
        integer, intent(in) :: ne_up, ne_down, Nstep
        integer(c_long_long), intent(in) :: ntot
        double precision, intent(in) :: vec(ntot)
        integer, intent(out) :: nstep_calc
        double precision, intent(out) :: a(0:Nstep), b(0:Nstep)
        integer(c_int) :: nc
        call mo_ed_gpu_check(mo_ed_lanczos_iteration(ctx, int(ne_up, c_int), int(ne_down, c_int), vec, nc, a, b), &
                             'lanczos_iteration')
        nstep_calc = nc
    end subroutine

    ! diag (ed_solver.F90:107-191): nev lowest eigenpairs of one sector.
    subroutine mo_ed_gpu_diag(ne_up, ne_down, ntot, nev, eigval, eigvec)
        integer, intent(in) :: ne_up, ne_down, nev
        integer(c_long_long), intent(in) :: ntot
        double precision, intent(out) :: eigval(nev), eigvec(ntot, nev)
        call mo_ed_gpu_check(mo_ed_diag(ctx, int(ne_up, c_int), int(ne_down, c_int), int(nev, c_int), &
                                        eigval, eigvec), 'diag')
    end subroutine
end module mo_ed_gpu


! ---- bath fit: the reference's external procedures, same argument lists -----

! FUNC (func.f90:1-45)
double precision function FUNC(x, Ns, nwloc, nxsize, omega, D_ev, Nbath, Norb, comm)
    use iso_c_binding
    use mo_ed_bind
    use mo_ed_gpu
    implicit none
    integer :: Ns, nwloc, nxsize, Nbath, Norb, comm
    double precision :: x(nxsize), omega(nwloc)
    double complex :: D_ev(Norb, nwloc)
    real(c_double) :: f
    call mo_ed_gpu_check(mo_ed_func(mo_ed_gpu_context(), x, int(Ns, c_int), int(nwloc, c_int), &
                                    int(nxsize, c_int), omega, D_ev, int(Nbath, c_int), &
                                    int(Norb, c_int), f), 'FUNC')
    FUNC = f
end function FUNC

! dfunc (func.f90:47-142): note nwloc before Ns, as in the reference
subroutine dfunc(x, p, nwloc, Ns, nxsize, omega, D_ev, Nbath, Norb, comm)
    use iso_c_binding
    use mo_ed_bind
    use mo_ed_gpu
    implicit none
    integer :: nwloc, Ns, nxsize, Nbath, Norb, comm
    double precision :: x(nxsize), p(nxsize), omega(nwloc)
    double complex :: D_ev(Norb, nwloc)
    call mo_ed_gpu_check(mo_ed_dfunc(mo_ed_gpu_context(), x, p, int(nwloc, c_int), int(Ns, c_int), &
                                     int(nxsize, c_int), omega, D_ev, int(Nbath, c_int), &
                                     int(Norb, c_int)), 'dfunc')
end subroutine dfunc

! minimization (func.f90:144-163): frprmn with FTOL = 1e-7; dab = final chi^2
subroutine minimization(x, nwloc, Ns, nxsize, omega, D_ev, Nbath, Norb, comm, dab)
    use iso_c_binding
    use mo_ed_bind
    use mo_ed_gpu
    implicit none
    integer :: nwloc, Ns, nxsize, Nbath, Norb, comm
    double precision :: x(nxsize), omega(nwloc), dab
    double complex :: D_ev(Norb, nwloc)
    real(c_double) :: fret
    integer(c_int) :: iter
    call mo_ed_gpu_check(mo_ed_minimization(mo_ed_gpu_context(), x, int(nwloc, c_int), int(Ns, c_int), &
                                            int(nxsize, c_int), omega, D_ev, int(Nbath, c_int), &
                                            int(Norb, c_int), fret, iter), 'minimization')
    dab = fret
end subroutine minimization
