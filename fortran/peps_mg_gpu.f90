!>
!> @file        peps_mg_gpu.f90
!> @brief       iso_c_binding interface of the GB300 multigrid library (libpeps_mg.so) for
!>              the PEPS_MG Fortran host.
!> @details     Two layers:
!>              (1) bind(C) interfaces for every entry point of include/peps_mg.h, with
!>                  the C structs pmg_config_t and pmg_report_t as bind(C) derived types;
!>              (2) wrapper subroutines with the argument lists of the reference routines
!>                  they replace (src/multigrid.f90:75,1864,1320,1345,1516,1782;
!>                  src/rbgs_poisson_matrix.f90:47,191; src/cg_poisson_matrix.f90:47,157;
!>                  src/poisson_matrix_operator.f90:40,110), so a caller swaps
!>                  `use multigrid` for `use peps_mg_gpu` and renames the calls.
!>              The wrappers keep one library context in a module variable, as the
!>              reference keeps its level hierarchy in module globals between
!>              multigrid_create and multigrid_destroy (src/multigrid.f90:54-55).  A
!>              lower-level wrapper finds the level of its subdomain argument by its
!>              sizes (levels of one hierarchy have distinct sizes).  Grid arrays are
!>              passed as c_loc of element (0,0,0); host arrays are staged through the
!>              GPU by pmg_solve_vcycle, the lower-level routines need device arrays
!>              (CUDA Fortran `device`, or OpenACC `host_data use_device`).
!>              Errors: where the reference prints and stops, a wrapper prints the
!>              library's message and stops, unless the caller passes the optional
!>              `status` argument, which then receives the code.
!>              The module uses only standard interoperable types (Fortran 2008).  No
!>              Fortran compiler exists where this library is built, so it has not been
!>              compiled here; tests/test_host_abi.py checks the C layouts its bind(C)
!>              types assume.
!>
module peps_mg_gpu

    use, intrinsic :: iso_c_binding

    implicit none

    private

    ! ---- status codes, options (include/peps_mg.h) ----------------------------------
    integer(c_int), parameter, public :: PMG_OK = 0, PMG_EINVAL = 1, PMG_ENOMEM = 2, PMG_EDIVERGED = 3
    integer(c_int), parameter, public :: PMG_ETIMEOUT = 4, PMG_ECUDA = 5
    integer(c_int), parameter, public :: PMG_CGS = 0, PMG_CGA = 1, PMG_CGPSA = 2
    integer(c_int), parameter, public :: PMG_COARSE_RBGS = 0, PMG_COARSE_CG = 1
    integer(c_int), parameter, public :: PMG_FP64 = 0, PMG_MIXED = 1, PMG_FP64_FAST = 2

    !> pmg_config_t: 3 ints, 9 pointers, 10 ints (C layout: the pointers start at byte
    !> 16 on an LP64 target, 4 bytes of padding after nz; 112 bytes in all)
    type, bind(C), public :: pmg_config_t
        integer(c_int) :: nx, ny, nz
        type(c_ptr)    :: dxm, dxg, xg
        type(c_ptr)    :: dym, dyg, yg
        type(c_ptr)    :: dzm, dzg, zg
        integer(c_int) :: number_of_levels
        integer(c_int) :: number_of_vcycles
        integer(c_int) :: aggregation_method
        integer(c_int) :: cga_level
        integer(c_int) :: cgpsa_level(3)
        integer(c_int) :: coarse_solver
        integer(c_int) :: precision
        integer(c_int) :: mixed_inner_cycles
    end type pmg_config_t

    !> pmg_report_t: 2 ints, 2 doubles, 2 pointers, 1 float, 1 int (48 bytes)
    type, bind(C), public :: pmg_report_t
        integer(c_int) :: cycles
        integer(c_int) :: converged
        real(c_double) :: res0
        real(c_double) :: final_ratio
        type(c_ptr)    :: history             !< 3*number_of_vcycles doubles, or c_null_ptr
        type(c_ptr)    :: coarse_iterations   !< number_of_vcycles ints, or c_null_ptr
        real(c_float)  :: elapsed_ms
        integer(c_int) :: inner_cycles
    end type pmg_report_t

    public :: pmg_create, pmg_solve_vcycle, pmg_destroy, pmg_level_sizes, pmg_level_dims, pmg_level_mesh
    public :: pmg_coarsest_levels, pmg_mv_mul, pmg_vv_dot, pmg_residual, pmg_rbgs_iterator, pmg_rbgs_solver
    public :: pmg_cg_iterator, pmg_cg_solver, pmg_restriction, pmg_prolongation, pmg_prolong_add
    public :: pmg_adjoint, pmg_batch_create, pmg_batch_layout, pmg_batch_solve, pmg_batch_destroy
    public :: pmg_vv_dot_static, pmg_profile, pmg_profile_read, pmg_launch_count, pmg_sync
    public :: pmg_dd_create, pmg_dd_solve, pmg_dd_destroy, pmg_dd_partition
    public :: pmg_set_abort, pmg_inject_alloc_failure, pmg_selftest_convert, pmg_selftest_smooth32
    public :: pmg_selftest_wait_timeout
    public :: pmg_last_error_c, pmg_status_string_c, pmg_error_message

    public :: multigrid_gpu_create, multigrid_gpu_solve_vcycle, multigrid_gpu_destroy
    public :: multigrid_gpu_context, multigrid_gpu_level_of
    public :: mv_mul_gpu_poisson_matrix, vv_dot_gpu_3d_matrix, multigrid_gpu_residual
    public :: rbgs_gpu_iterator_poisson_matrix, rbgs_gpu_solver_poisson_matrix
    public :: cg_gpu_iterator_poisson_matrix, cg_gpu_solver_poisson_matrix
    public :: multigrid_gpu_restriction, multigrid_gpu_prolongation

    !> the context of the wrappers (the reference's module-level hierarchy)
    type(c_ptr), save :: g_ctx = c_null_ptr

    interface

        ! multigrid_create (src/multigrid.f90:75)
        integer(c_int) function pmg_create(ctx, cfg, stream) bind(C, name="pmg_create")
            import :: c_int, c_ptr, pmg_config_t
            type(c_ptr), intent(out)        :: ctx
            type(pmg_config_t), intent(in)  :: cfg
            type(c_ptr), value              :: stream     !< cudaStream_t, c_null_ptr: default stream
        end function pmg_create

        ! multigrid_solve_vcycle (src/multigrid.f90:1864)
        integer(c_int) function pmg_solve_vcycle(ctx, sol, rsd, rhs, maxiteration, tolerance, omega_sor, report) &
                bind(C, name="pmg_solve_vcycle")
            import :: c_int, c_ptr, c_double, pmg_report_t
            type(c_ptr), value                  :: ctx, sol, rsd, rhs
            integer(c_int), value               :: maxiteration
            real(c_double), value               :: tolerance, omega_sor
            type(pmg_report_t), intent(inout)   :: report
        end function pmg_solve_vcycle

        ! multigrid_destroy (src/multigrid.f90:1320)
        integer(c_int) function pmg_destroy(ctx) bind(C, name="pmg_destroy")
            import :: c_int, c_ptr
            type(c_ptr), value  :: ctx
        end function pmg_destroy

        ! level-size rules of multigrid_subdomain_create_CGS/_CGA/_CGPSA (host only)
        integer(c_int) function pmg_level_sizes(nx, ny, nz, n_levels, aggregation_method, cga_level, sizes, &
                                                lv_coarsest) bind(C, name="pmg_level_sizes")
            import :: c_int
            integer(c_int), value           :: nx, ny, nz, n_levels, aggregation_method, cga_level
            integer(c_int), intent(out)     :: sizes(*)          !< 3*(n_levels+1)
            integer(c_int), intent(out)     :: lv_coarsest(3)
        end function pmg_level_sizes

        integer(c_int) function pmg_level_dims(ctx, level, dims) bind(C, name="pmg_level_dims")
            import :: c_int, c_ptr
            type(c_ptr), value              :: ctx
            integer(c_int), value           :: level
            integer(c_int), intent(out)     :: dims(3)
        end function pmg_level_dims

        integer(c_int) function pmg_level_mesh(ctx, level, axis, dm, dg, xg) bind(C, name="pmg_level_mesh")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value              :: ctx
            integer(c_int), value           :: level, axis
            real(c_double), intent(out)     :: dm(*), dg(*), xg(*)   !< n+2 values each
        end function pmg_level_mesh

        integer(c_int) function pmg_coarsest_levels(ctx, lv_coarsest) bind(C, name="pmg_coarsest_levels")
            import :: c_int, c_ptr
            type(c_ptr), value              :: ctx
            integer(c_int), intent(out)     :: lv_coarsest(3)
        end function pmg_coarsest_levels

        ! mv_mul_poisson_matrix (src/poisson_matrix_operator.f90:110)
        integer(c_int) function pmg_mv_mul(ctx, level, y, x) bind(C, name="pmg_mv_mul")
            import :: c_int, c_ptr
            type(c_ptr), value      :: ctx, y, x
            integer(c_int), value   :: level
        end function pmg_mv_mul

        ! vv_dot_3d_matrix (src/poisson_matrix_operator.f90:40)
        integer(c_int) function pmg_vv_dot(ctx, level, x, y, result) bind(C, name="pmg_vv_dot")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value          :: ctx, x, y
            integer(c_int), value       :: level
            real(c_double), intent(out) :: result
        end function pmg_vv_dot

        ! multigrid_residual (src/multigrid.f90:1782)
        integer(c_int) function pmg_residual(ctx, level, r, x, b) bind(C, name="pmg_residual")
            import :: c_int, c_ptr
            type(c_ptr), value      :: ctx, r, x, b
            integer(c_int), value   :: level
        end function pmg_residual

        ! rbgs_iterator_poisson_matrix (src/rbgs_poisson_matrix.f90:191)
        integer(c_int) function pmg_rbgs_iterator(ctx, level, x, b, maxiteration, omega) &
                bind(C, name="pmg_rbgs_iterator")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value      :: ctx, x, b
            integer(c_int), value   :: level, maxiteration
            real(c_double), value   :: omega
        end function pmg_rbgs_iterator

        ! rbgs_solver_poisson_matrix (src/rbgs_poisson_matrix.f90:47)
        integer(c_int) function pmg_rbgs_solver(ctx, level, x, b, maxiteration, tolerance, omega, iterations, ratio) &
                bind(C, name="pmg_rbgs_solver")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value          :: ctx, x, b
            integer(c_int), value       :: level, maxiteration
            real(c_double), value       :: tolerance, omega
            integer(c_int), intent(out) :: iterations
            real(c_double), intent(out) :: ratio
        end function pmg_rbgs_solver

        ! cg_iterator_poisson_matrix (src/cg_poisson_matrix.f90:157)
        integer(c_int) function pmg_cg_iterator(ctx, level, x, b, maxiteration) bind(C, name="pmg_cg_iterator")
            import :: c_int, c_ptr
            type(c_ptr), value      :: ctx, x, b
            integer(c_int), value   :: level, maxiteration
        end function pmg_cg_iterator

        ! cg_solver_poisson_matrix (src/cg_poisson_matrix.f90:47)
        integer(c_int) function pmg_cg_solver(ctx, level, x, b, maxiteration, tolerance, iterations, ratio) &
                bind(C, name="pmg_cg_solver")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value          :: ctx, x, b
            integer(c_int), value       :: level, maxiteration
            real(c_double), value       :: tolerance
            integer(c_int), intent(out) :: iterations
            real(c_double), intent(out) :: ratio
        end function pmg_cg_solver

        ! multigrid_restriction (src/multigrid.f90:1345); level = the fine level
        integer(c_int) function pmg_restriction(ctx, level, val_c, val_f) bind(C, name="pmg_restriction")
            import :: c_int, c_ptr
            type(c_ptr), value      :: ctx, val_c, val_f
            integer(c_int), value   :: level
        end function pmg_restriction

        ! multigrid_prolongation_linear_on_nonuniform_grid (src/multigrid.f90:1516)
        integer(c_int) function pmg_prolongation(ctx, level, val_f, val_c) bind(C, name="pmg_prolongation")
            import :: c_int, c_ptr
            type(c_ptr), value      :: ctx, val_f, val_c
            integer(c_int), value   :: level
        end function pmg_prolongation

        ! prolongation + correction x_f = x_f + P x_c (src/multigrid.f90:1957-1958)
        integer(c_int) function pmg_prolong_add(ctx, level, x_f, x_c) bind(C, name="pmg_prolong_add")
            import :: c_int, c_ptr
            type(c_ptr), value      :: ctx, x_f, x_c
            integer(c_int), value   :: level
        end function pmg_prolong_add

        ! adjoint of the last solve (no counterpart in the reference)
        integer(c_int) function pmg_adjoint(ctx, dLdu, dLdb, dLdg, maxiteration, tolerance, omega_sor, report) &
                bind(C, name="pmg_adjoint")
            import :: c_int, c_ptr, c_double, pmg_report_t
            type(c_ptr), value                  :: ctx, dLdu, dLdb   !< device arrays of the finest level
            real(c_double), intent(out)         :: dLdg(6)           !< x-, x+, y-, y+, z-, z+
            integer(c_int), value               :: maxiteration
            real(c_double), value               :: tolerance, omega_sor
            type(pmg_report_t), intent(inout)   :: report
        end function pmg_adjoint

        ! batched solver (no counterpart in the reference)
        integer(c_int) function pmg_batch_create(batch, n_problems, dims, meshes, mixed_inner_cycles, stream) &
                bind(C, name="pmg_batch_create")
            import :: c_int, c_ptr
            type(c_ptr), intent(out)    :: batch
            integer(c_int), value       :: n_problems, mixed_inner_cycles
            integer(c_int), intent(in)  :: dims(3, *)
            type(c_ptr), value          :: meshes      !< c_null_ptr (uniform cubic cells) or 6 pointers per problem
            type(c_ptr), value          :: stream
        end function pmg_batch_create

        integer(c_int) function pmg_batch_layout(batch, offsets, levels) bind(C, name="pmg_batch_layout")
            import :: c_int, c_ptr, c_long_long
            type(c_ptr), value                  :: batch
            integer(c_long_long), intent(out)   :: offsets(*)   !< n_problems + 1 element offsets
            integer(c_int), intent(out)         :: levels(*)
        end function pmg_batch_layout

        integer(c_int) function pmg_batch_solve(batch, sol, rhs, maxiteration, tolerance, omega_sor, max_cycles, &
                                                cycles, ratio, elapsed_ms) bind(C, name="pmg_batch_solve")
            import :: c_int, c_ptr, c_double, c_float
            type(c_ptr), value          :: batch, sol, rhs   !< packed device arrays
            integer(c_int), value       :: maxiteration, max_cycles
            real(c_double), value       :: tolerance, omega_sor
            integer(c_int), intent(out) :: cycles(*)
            real(c_double), intent(out) :: ratio(*)
            real(c_float), intent(out)  :: elapsed_ms
        end function pmg_batch_solve

        integer(c_int) function pmg_batch_destroy(batch) bind(C, name="pmg_batch_destroy")
            import :: c_int, c_ptr
            type(c_ptr), value  :: batch
        end function pmg_batch_destroy

        ! the CGS V-cycle on a procs(1) x procs(2) x procs(3) decomposition of one grid, every
        ! subdomain on this process's GPU (the reference's multi-rank execution)
        integer(c_int) function pmg_dd_create(dd, cfg, procs, stream) bind(C, name="pmg_dd_create")
            import :: c_int, c_ptr, pmg_config_t
            type(c_ptr), intent(out)        :: dd
            type(pmg_config_t), intent(in)  :: cfg      !< the global problem
            integer(c_int), intent(in)      :: procs(3)
            type(c_ptr), value              :: stream
        end function pmg_dd_create

        integer(c_int) function pmg_dd_solve(dd, sol, rsd, rhs, maxiteration, tolerance, omega_sor, report) &
                bind(C, name="pmg_dd_solve")
            import :: c_int, c_ptr, c_double, pmg_report_t
            type(c_ptr), value                  :: dd, sol, rsd, rhs   !< global device arrays
            integer(c_int), value               :: maxiteration
            real(c_double), value               :: tolerance, omega_sor
            type(pmg_report_t), intent(inout)   :: report
        end function pmg_dd_solve

        integer(c_int) function pmg_dd_destroy(dd) bind(C, name="pmg_dd_destroy")
            import :: c_int, c_ptr
            type(c_ptr), value  :: dd
        end function pmg_dd_destroy

        ! one rank's subdomain (host only): sizes, mesh and RBGS colour offset on a level
        integer(c_int) function pmg_dd_partition(cfg, procs, coords, level, dims, mesh, offset) &
                bind(C, name="pmg_dd_partition")
            import :: c_int, c_ptr, pmg_config_t
            type(pmg_config_t), intent(in)  :: cfg
            integer(c_int), intent(in)      :: procs(3), coords(3)
            integer(c_int), value           :: level
            integer(c_int), intent(out)     :: dims(3)
            type(c_ptr), intent(in)         :: mesh(9)     !< dxm, dxg, xg, dym, ..., zg (c_null_ptr allowed)
            integer(c_int), intent(out)     :: offset
        end function pmg_dd_partition

        ! interior dot product with no device allocation (no counterpart in the reference)
        integer(c_int) function pmg_vv_dot_static(x, y, nx, ny, nz, stream, result) &
                bind(C, name="pmg_vv_dot_static")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value          :: x, y, stream
            integer(c_int), value       :: nx, ny, nz
            real(c_double), intent(out) :: result
        end function pmg_vv_dot_static

        ! telemetry (no counterpart in the reference, which only prints MPI_Wtime)
        integer(c_int) function pmg_profile(ctx, enable) bind(C, name="pmg_profile")
            import :: c_int, c_ptr
            type(c_ptr), value      :: ctx
            integer(c_int), value   :: enable
        end function pmg_profile

        integer(c_int) function pmg_profile_read(ctx, kernel_class, total_ms, launches, bytes) &
                bind(C, name="pmg_profile_read")
            import :: c_int, c_ptr, c_double, c_long_long
            type(c_ptr), value                  :: ctx
            integer(c_int), value               :: kernel_class
            real(c_double), intent(out)         :: total_ms, bytes
            integer(c_long_long), intent(out)   :: launches
        end function pmg_profile_read

        integer(c_int) function pmg_launch_count(count) bind(C, name="pmg_launch_count")
            import :: c_int, c_long_long
            integer(c_long_long), intent(out)   :: count
        end function pmg_launch_count

        ! host-set abort flag polled by the solver's device loops
        integer(c_int) function pmg_set_abort(ctx, flag) bind(C, name="pmg_set_abort")
            import :: c_int, c_ptr
            type(c_ptr), value      :: ctx
            integer(c_int), value   :: flag
        end function pmg_set_abort

        ! self-tests of the mixed-precision kernels
        integer(c_int) function pmg_selftest_convert(in64, out32, in32, out64, n) &
                bind(C, name="pmg_selftest_convert")
            import :: c_int, c_ptr
            type(c_ptr), value      :: in64, out32, in32, out64
            integer(c_int), value   :: n
        end function pmg_selftest_convert

        integer(c_int) function pmg_selftest_smooth32(ctx, level, impl, variant, kchunk, zero_in, omega, e_in, b, &
                                                      e_out) bind(C, name="pmg_selftest_smooth32")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value      :: ctx
            integer(c_int), value   :: level, impl, variant, kchunk, zero_in
            real(c_double), value   :: omega
            real(c_double), intent(in)  :: e_in(*), b(*)
            real(c_double), intent(out) :: e_out(*)
        end function pmg_selftest_smooth32

        ! timeout path of the TMA-fed smoother (waits run out with no copy in flight)
        integer(c_int) function pmg_selftest_wait_timeout(ctx, level) bind(C, name="pmg_selftest_wait_timeout")
            import :: c_int, c_ptr
            type(c_ptr), value      :: ctx
            integer(c_int), value   :: level
        end function pmg_selftest_wait_timeout

        ! host-side fault injection: the n-th next device allocation fails (n < 0: off)
        integer(c_int) function pmg_inject_alloc_failure(n) bind(C, name="pmg_inject_alloc_failure")
            import :: c_int, c_long_long
            integer(c_long_long), value :: n
        end function pmg_inject_alloc_failure

        integer(c_int) function pmg_sync(ctx) bind(C, name="pmg_sync")
            import :: c_int, c_ptr
            type(c_ptr), value  :: ctx
        end function pmg_sync

        type(c_ptr) function pmg_last_error_c() bind(C, name="pmg_last_error")
            import :: c_ptr
        end function pmg_last_error_c

        type(c_ptr) function pmg_status_string_c(status) bind(C, name="pmg_status_string")
            import :: c_ptr, c_int
            integer(c_int), value   :: status
        end function pmg_status_string_c

        integer(c_size_t) function c_strlen(s) bind(C, name="strlen")
            import :: c_size_t, c_ptr
            type(c_ptr), value  :: s
        end function c_strlen

    end interface

contains

    !> The library's message for the last error of the calling thread.
    function pmg_error_message() result(msg)
        character(len=:), allocatable   :: msg
        type(c_ptr)                     :: p
        character(kind=c_char), pointer :: chars(:)
        integer                         :: n, i

        msg = ''
        p = pmg_last_error_c()
        if (.not. c_associated(p)) return
        n = int(c_strlen(p))
        if (n <= 0) return
        call c_f_pointer(p, chars, [n])
        deallocate(msg)
        allocate(character(len=n) :: msg)
        do i = 1, n
            msg(i:i) = chars(i)
        enddo
    end function pmg_error_message

    !> Hands a status to the caller's optional argument, or prints the library's message
    !> and stops where the reference stops (e.g. src/multigrid.f90:101-107).
    subroutine handle_status(rc, what, status)
        integer(c_int), intent(in)              :: rc
        character(len=*), intent(in)            :: what
        integer(kind=4), intent(out), optional  :: status

        if (present(status)) then
            status = rc
            return
        endif
        if (rc /= PMG_OK) then
            print '(a,a,a,i2,a,a)', '[Error] ', what, ' failed (status ', rc, '): ', pmg_error_message()
            error stop 301
        endif
    end subroutine handle_status

    !> The wrappers' context (c_null_ptr before multigrid_gpu_create).
    function multigrid_gpu_context() result(ctx)
        type(c_ptr) :: ctx
        ctx = g_ctx
    end function multigrid_gpu_context

    !> Level of the hierarchy whose interior sizes are nx, ny, nz (-1 if none).
    function multigrid_gpu_level_of(nx, ny, nz) result(level)
        integer(kind=4), intent(in) :: nx, ny, nz
        integer(kind=4)             :: level
        integer(c_int)              :: dims(3), l

        level = -1
        if (.not. c_associated(g_ctx)) return
        l = 0
        do while (pmg_level_dims(g_ctx, l, dims) == PMG_OK)
            if (dims(1) == nx .and. dims(2) == ny .and. dims(3) == nz) then
                level = l
                return
            endif
            l = l + 1
        enddo
    end function multigrid_gpu_level_of

    !> multigrid_create(sdm, nlevel, ncycle, aggr_method, single_aggr_level,
    !> adaptive_aggr_level) -- src/multigrid.f90:75.  Optional: precision (PMG_FP64, the
    !> default, PMG_MIXED or PMG_FP64_FAST), coarse_solver (PMG_COARSE_RBGS, the default, or
    !> PMG_COARSE_CG), mixed_inner_cycles, stream (a cudaStream_t), status.
    subroutine multigrid_gpu_create(sdm, nlevel, ncycle, aggr_method, single_aggr_level, adaptive_aggr_level, &
                                    precision, coarse_solver, mixed_inner_cycles, stream, status)
        use geometry, only : subdomain

        type(subdomain), intent(in), target     :: sdm
        integer(kind=4), intent(in)             :: nlevel, ncycle, aggr_method, single_aggr_level
        integer(kind=4), intent(in)             :: adaptive_aggr_level(3)
        integer(kind=4), intent(in), optional   :: precision, coarse_solver, mixed_inner_cycles
        type(c_ptr), intent(in), optional       :: stream
        integer(kind=4), intent(out), optional  :: status

        type(pmg_config_t)  :: cfg
        type(c_ptr)         :: s
        integer(c_int)      :: rc

        if (c_associated(g_ctx)) rc = pmg_destroy(g_ctx)
        g_ctx = c_null_ptr
        cfg%nx = sdm%nx
        cfg%ny = sdm%ny
        cfg%nz = sdm%nz
        cfg%dxm = c_loc(sdm%dxm(0))
        cfg%dxg = c_loc(sdm%dxg(0))
        cfg%xg  = c_loc(sdm%xg(0))
        cfg%dym = c_loc(sdm%dym(0))
        cfg%dyg = c_loc(sdm%dyg(0))
        cfg%yg  = c_loc(sdm%yg(0))
        cfg%dzm = c_loc(sdm%dzm(0))
        cfg%dzg = c_loc(sdm%dzg(0))
        cfg%zg  = c_loc(sdm%zg(0))
        cfg%number_of_levels = nlevel
        cfg%number_of_vcycles = ncycle
        cfg%aggregation_method = aggr_method
        cfg%cga_level = single_aggr_level
        cfg%cgpsa_level = adaptive_aggr_level
        cfg%coarse_solver = PMG_COARSE_RBGS
        if (present(coarse_solver)) cfg%coarse_solver = coarse_solver
        cfg%precision = PMG_FP64
        if (present(precision)) cfg%precision = precision
        cfg%mixed_inner_cycles = 0
        if (present(mixed_inner_cycles)) cfg%mixed_inner_cycles = mixed_inner_cycles
        s = c_null_ptr
        if (present(stream)) s = stream
        rc = pmg_create(g_ctx, cfg, s)
        if (rc /= PMG_OK) g_ctx = c_null_ptr
        call handle_status(rc, 'multigrid_create', status)
    end subroutine multigrid_gpu_create

    !> multigrid_solve_vcycle(sol, rsd, a_poisson, rhs, sdm, maxiteration, tolerance,
    !> omega_sor) -- src/multigrid.f90:1864.  a_poisson and sdm are accepted for the
    !> reference's argument list; the library built the operator of every level from the
    !> mesh at multigrid_gpu_create.  Host or device arrays (all three alike).  Optional:
    !> report (cycles, history, timing), status.
    subroutine multigrid_gpu_solve_vcycle(sol, rsd, a_poisson, rhs, sdm, maxiteration, tolerance, omega_sor, &
                                          report, status)
        use geometry, only : subdomain
        use matrix, only : matrix_heptadiagonal

        real(c_double), intent(inout), target, contiguous   :: sol(0:,0:,0:), rsd(0:,0:,0:)
        type(matrix_heptadiagonal), intent(in)              :: a_poisson
        real(c_double), intent(in), target, contiguous      :: rhs(0:,0:,0:)
        type(subdomain), intent(in)                         :: sdm
        integer(kind=4), intent(in)                         :: maxiteration
        real(kind=8), intent(in)                            :: tolerance, omega_sor
        type(pmg_report_t), intent(inout), optional         :: report
        integer(kind=4), intent(out), optional              :: status

        type(pmg_report_t)  :: rep
        integer(c_int)      :: rc

        rep%history = c_null_ptr
        rep%coarse_iterations = c_null_ptr
        if (present(report)) rep = report
        rc = pmg_solve_vcycle(g_ctx, c_loc(sol(0,0,0)), c_loc(rsd(0,0,0)), c_loc(rhs(0,0,0)), &
                              maxiteration, tolerance, omega_sor, rep)
        if (present(report)) report = rep
        call handle_status(rc, 'multigrid_solve_vcycle', status)
    end subroutine multigrid_gpu_solve_vcycle

    !> multigrid_destroy -- src/multigrid.f90:1320
    subroutine multigrid_gpu_destroy(status)
        integer(kind=4), intent(out), optional  :: status
        integer(c_int)                          :: rc

        rc = PMG_OK
        if (c_associated(g_ctx)) rc = pmg_destroy(g_ctx)
        g_ctx = c_null_ptr
        call handle_status(rc, 'multigrid_destroy', status)
    end subroutine multigrid_gpu_destroy

    ! ---- lower-level wrappers (device arrays of one level of the hierarchy) ------------

    !> level of a subdomain of the wrappers' hierarchy; stops (or returns PMG_EINVAL in
    !> status) when no level has its sizes
    function level_or_fail(nx, ny, nz, what, status) result(level)
        integer(kind=4), intent(in)             :: nx, ny, nz
        character(len=*), intent(in)            :: what
        integer(kind=4), intent(out), optional  :: status
        integer(kind=4)                         :: level

        level = multigrid_gpu_level_of(nx, ny, nz)
        if (level < 0) then
            if (present(status)) then
                status = PMG_EINVAL
            else
                print '(a,a,a,3i6)', '[Error] ', what, ': no level of the hierarchy has the sizes ', nx, ny, nz
                error stop 301
            endif
        endif
    end function level_or_fail

    !> mv_mul_poisson_matrix(y, a_poisson, x, dm, is_serial) -- src/poisson_matrix_operator.f90:110
    subroutine mv_mul_gpu_poisson_matrix(y, a_poisson, x, dm, is_serial, status)
        use geometry, only : subdomain
        use matrix, only : matrix_heptadiagonal

        real(c_double), intent(inout), target, contiguous   :: y(0:,0:,0:)
        type(matrix_heptadiagonal), intent(in)              :: a_poisson
        real(c_double), intent(in), target, contiguous      :: x(0:,0:,0:)
        type(subdomain), intent(in)                         :: dm
        logical, intent(in)                                 :: is_serial(0:2)
        integer(kind=4), intent(out), optional              :: status
        integer(kind=4)                                     :: l

        l = level_or_fail(dm%nx, dm%ny, dm%nz, 'mv_mul_poisson_matrix', status)
        if (l < 0) return
        call handle_status(pmg_mv_mul(g_ctx, l, c_loc(y(0,0,0)), c_loc(x(0,0,0))), 'mv_mul_poisson_matrix', status)
    end subroutine mv_mul_gpu_poisson_matrix

    !> vv_dot_3d_matrix(result, x, y, nx, ny, nz, is_serial) -- src/poisson_matrix_operator.f90:40
    subroutine vv_dot_gpu_3d_matrix(result, x, y, nx, ny, nz, is_serial, status)
        real(kind=8), intent(out)                           :: result
        real(c_double), intent(in), target, contiguous      :: x(0:,0:,0:), y(0:,0:,0:)
        integer(kind=4), intent(in)                         :: nx, ny, nz
        logical, intent(in)                                 :: is_serial(0:2)
        integer(kind=4), intent(out), optional              :: status
        integer(kind=4)                                     :: l

        l = level_or_fail(nx, ny, nz, 'vv_dot_3d_matrix', status)
        if (l < 0) return
        call handle_status(pmg_vv_dot(g_ctx, l, c_loc(x(0,0,0)), c_loc(y(0,0,0)), result), 'vv_dot_3d_matrix', status)
    end subroutine vv_dot_gpu_3d_matrix

    !> multigrid_residual(rsd, a_poisson, x, rhs, dm, is_aggregated) -- src/multigrid.f90:1782
    subroutine multigrid_gpu_residual(rsd, a_poisson, x, rhs, dm, is_aggregated, status)
        use geometry, only : subdomain
        use matrix, only : matrix_heptadiagonal

        real(c_double), intent(inout), target, contiguous   :: rsd(0:,0:,0:)
        type(matrix_heptadiagonal), intent(in)              :: a_poisson
        real(c_double), intent(in), target, contiguous      :: x(0:,0:,0:), rhs(0:,0:,0:)
        type(subdomain), intent(in)                         :: dm
        logical, intent(in)                                 :: is_aggregated(0:2)
        integer(kind=4), intent(out), optional              :: status
        integer(kind=4)                                     :: l

        l = level_or_fail(dm%nx, dm%ny, dm%nz, 'multigrid_residual', status)
        if (l < 0) return
        call handle_status(pmg_residual(g_ctx, l, c_loc(rsd(0,0,0)), c_loc(x(0,0,0)), c_loc(rhs(0,0,0))), &
                           'multigrid_residual', status)
    end subroutine multigrid_gpu_residual

    !> rbgs_iterator_poisson_matrix(sol, a_poisson, rhs, dm, maxiteration, omega,
    !> is_aggregated) -- src/rbgs_poisson_matrix.f90:191
    subroutine rbgs_gpu_iterator_poisson_matrix(sol, a_poisson, rhs, dm, maxiteration, omega, is_aggregated, status)
        use geometry, only : subdomain
        use matrix, only : matrix_heptadiagonal

        real(c_double), intent(inout), target, contiguous   :: sol(0:,0:,0:)
        type(matrix_heptadiagonal), intent(in)              :: a_poisson
        real(c_double), intent(in), target, contiguous      :: rhs(0:,0:,0:)
        type(subdomain), intent(in)                         :: dm
        integer(kind=4), intent(in)                         :: maxiteration
        real(kind=8), intent(in)                            :: omega
        logical, intent(in)                                 :: is_aggregated(0:2)
        integer(kind=4), intent(out), optional              :: status
        integer(kind=4)                                     :: l

        l = level_or_fail(dm%nx, dm%ny, dm%nz, 'rbgs_iterator_poisson_matrix', status)
        if (l < 0) return
        call handle_status(pmg_rbgs_iterator(g_ctx, l, c_loc(sol(0,0,0)), c_loc(rhs(0,0,0)), maxiteration, omega), &
                           'rbgs_iterator_poisson_matrix', status)
    end subroutine rbgs_gpu_iterator_poisson_matrix

    !> rbgs_solver_poisson_matrix(sol, a_poisson, rhs, dm, maxiteration, tolerance, omega,
    !> is_aggregated) -- src/rbgs_poisson_matrix.f90:47.  Optional: iterations, ratio.
    subroutine rbgs_gpu_solver_poisson_matrix(sol, a_poisson, rhs, dm, maxiteration, tolerance, omega, is_aggregated, &
                                              iterations, ratio, status)
        use geometry, only : subdomain
        use matrix, only : matrix_heptadiagonal

        real(c_double), intent(inout), target, contiguous   :: sol(0:,0:,0:)
        type(matrix_heptadiagonal), intent(in)              :: a_poisson
        real(c_double), intent(in), target, contiguous      :: rhs(0:,0:,0:)
        type(subdomain), intent(in)                         :: dm
        integer(kind=4), intent(in)                         :: maxiteration
        real(kind=8), intent(in)                            :: tolerance, omega
        logical, intent(in)                                 :: is_aggregated(0:2)
        integer(kind=4), intent(out), optional              :: iterations
        real(kind=8), intent(out), optional                 :: ratio
        integer(kind=4), intent(out), optional              :: status
        integer(kind=4)                                     :: l
        integer(c_int)                                      :: it
        real(c_double)                                      :: rt

        l = level_or_fail(dm%nx, dm%ny, dm%nz, 'rbgs_solver_poisson_matrix', status)
        if (l < 0) return
        call handle_status(pmg_rbgs_solver(g_ctx, l, c_loc(sol(0,0,0)), c_loc(rhs(0,0,0)), maxiteration, tolerance, &
                                           omega, it, rt), 'rbgs_solver_poisson_matrix', status)
        if (present(iterations)) iterations = it
        if (present(ratio)) ratio = rt
    end subroutine rbgs_gpu_solver_poisson_matrix

    !> cg_iterator_poisson_matrix(sol, a_poisson, rhs, dm, maxiteration, is_aggregated)
    !> -- src/cg_poisson_matrix.f90:157
    subroutine cg_gpu_iterator_poisson_matrix(sol, a_poisson, rhs, dm, maxiteration, is_aggregated, status)
        use geometry, only : subdomain
        use matrix, only : matrix_heptadiagonal

        real(c_double), intent(inout), target, contiguous   :: sol(0:,0:,0:)
        type(matrix_heptadiagonal), intent(in)              :: a_poisson
        real(c_double), intent(in), target, contiguous      :: rhs(0:,0:,0:)
        type(subdomain), intent(in)                         :: dm
        integer(kind=4), intent(in)                         :: maxiteration
        logical, intent(in)                                 :: is_aggregated(0:2)
        integer(kind=4), intent(out), optional              :: status
        integer(kind=4)                                     :: l

        l = level_or_fail(dm%nx, dm%ny, dm%nz, 'cg_iterator_poisson_matrix', status)
        if (l < 0) return
        call handle_status(pmg_cg_iterator(g_ctx, l, c_loc(sol(0,0,0)), c_loc(rhs(0,0,0)), maxiteration), &
                           'cg_iterator_poisson_matrix', status)
    end subroutine cg_gpu_iterator_poisson_matrix

    !> cg_solver_poisson_matrix(sol, a_poisson, rhs, dm, maxiteration, tolerance,
    !> is_aggregated) -- src/cg_poisson_matrix.f90:47.  Optional: iterations, ratio.
    subroutine cg_gpu_solver_poisson_matrix(sol, a_poisson, rhs, dm, maxiteration, tolerance, is_aggregated, &
                                            iterations, ratio, status)
        use geometry, only : subdomain
        use matrix, only : matrix_heptadiagonal

        real(c_double), intent(inout), target, contiguous   :: sol(0:,0:,0:)
        type(matrix_heptadiagonal), intent(in)              :: a_poisson
        real(c_double), intent(in), target, contiguous      :: rhs(0:,0:,0:)
        type(subdomain), intent(in)                         :: dm
        integer(kind=4), intent(in)                         :: maxiteration
        real(kind=8), intent(in)                            :: tolerance
        logical, intent(in)                                 :: is_aggregated(0:2)
        integer(kind=4), intent(out), optional              :: iterations
        real(kind=8), intent(out), optional                 :: ratio
        integer(kind=4), intent(out), optional              :: status
        integer(kind=4)                                     :: l
        integer(c_int)                                      :: it
        real(c_double)                                      :: rt

        l = level_or_fail(dm%nx, dm%ny, dm%nz, 'cg_solver_poisson_matrix', status)
        if (l < 0) return
        call handle_status(pmg_cg_solver(g_ctx, l, c_loc(sol(0,0,0)), c_loc(rhs(0,0,0)), maxiteration, tolerance, &
                                         it, rt), 'cg_solver_poisson_matrix', status)
        if (present(iterations)) iterations = it
        if (present(ratio)) ratio = rt
    end subroutine cg_gpu_solver_poisson_matrix

    !> multigrid_restriction(val_c, val_f, dm_c, dm_f, level) -- src/multigrid.f90:1345
    !> (level: the fine level, as in the reference)
    subroutine multigrid_gpu_restriction(val_c, val_f, dm_c, dm_f, level, status)
        use geometry, only : subdomain

        real(c_double), intent(inout), target, contiguous   :: val_c(0:,0:,0:)
        real(c_double), intent(in), target, contiguous      :: val_f(0:,0:,0:)
        type(subdomain), intent(in)                         :: dm_c, dm_f
        integer(kind=4), intent(in)                         :: level
        integer(kind=4), intent(out), optional              :: status

        call handle_status(pmg_restriction(g_ctx, level, c_loc(val_c(0,0,0)), c_loc(val_f(0,0,0))), &
                           'multigrid_restriction', status)
    end subroutine multigrid_gpu_restriction

    !> multigrid_prolongation_linear_on_nonuniform_grid(val_f, val_c, dm_f, dm_c, level)
    !> -- src/multigrid.f90:1516 (level: the fine level)
    subroutine multigrid_gpu_prolongation(val_f, val_c, dm_f, dm_c, level, status)
        use geometry, only : subdomain

        real(c_double), intent(inout), target, contiguous   :: val_f(0:,0:,0:)
        real(c_double), intent(in), target, contiguous      :: val_c(0:,0:,0:)
        type(subdomain), intent(in)                         :: dm_f, dm_c
        integer(kind=4), intent(in)                         :: level
        integer(kind=4), intent(out), optional              :: status

        call handle_status(pmg_prolongation(g_ctx, level, c_loc(val_f(0,0,0)), c_loc(val_c(0,0,0))), &
                           'multigrid_prolongation_linear_on_nonuniform_grid', status)
    end subroutine multigrid_gpu_prolongation

end module peps_mg_gpu
