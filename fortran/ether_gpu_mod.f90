! ether_gpu_mod.f90 -- ISO_C_BINDING interface of libether_gpu.so (include/ether_gpu.h)
! for ETHER's Fortran driver.  It replaces, call for call, the routines that the MCS loop
! of src/ether.f90:152-214 invokes on `module init` state:
!   fresh_spins             -> ether_fresh_spins
!   overrelaxation          -> ether_overrelaxation
!   Metropolis              -> ether_metropolis
!   get_tot_energy          -> ether_tot_energy
!   parallel_tempering      -> ether_parallel_tempering
!   observable              -> ether_observable
!   get_eng/get_mag('avg')  -> ether_avg
!   observables_per_repeat  -> ether_per_repeat
! All arrays keep the layouts of module init (ion(0:8,N), nn(nsh,N,0:cap,0:1),
! j_exc(nsh,nsp,nsp,3), sia_vec(3,nsp)); they are passed by address and are not retained.
module ether_gpu_mod
    use iso_c_binding
    implicit none

    integer(c_int), parameter :: ETHER_OK = 0
    integer(c_int), parameter :: ETHER_MODEL_ISING = 0, ETHER_MODEL_XYZ = 1
    integer(c_int), parameter :: ETHER_FLAG_FORCE_GENERAL = 1
    integer(c_int), parameter :: ETHER_FLAG_PT_TRUE_ENERGY = 2
    integer(c_int), parameter :: ETHER_FLAG_PT_REFERENCE_COPY = 4
    integer(c_int), parameter :: ETHER_FLAG_NO_GRAPHS = 8, ETHER_FLAG_NO_RESIDENT = 16
    integer(c_int), parameter :: ETHER_FLAG_STAGED_SPINS = 32

    type, bind(C) :: ether_desc
        integer(c_int32_t) :: n_sites, n_species, n_shells, nbd_capacity, model, angle
        real(c_double)     :: dphi
        integer(c_int32_t) :: zeeman
        real(c_double)     :: h(3), g_factor, mb
        integer(c_int32_t) :: sia
        type(c_ptr)        :: ion, nn, j_exc, sia_vec, s, stgg
        integer(c_int32_t) :: n_replicas
        integer(c_int32_t) :: seed          ! uint32_t in C
        integer(c_int32_t) :: sc(3), basis, flags
        type(c_ptr)        :: sia_local     ! sia_local(4, N) or c_null_ptr
    end type ether_desc

    integer(c_int), parameter :: ETHER_RUN_PARSE_ONLY = 1, ETHER_RUN_QUIET = 2, ETHER_RUN_RESUME = 4

    type, bind(C) :: ether_run_info
        integer(c_int32_t) :: ranks, model, n_sites, n_species, n_shells, n_temperatures, &
                              repeat, n_rounds
        integer(c_int64_t) :: site_updates     ! uint64_t in C
        real(c_double)     :: seconds
    end type ether_run_info

    type, bind(C) :: ether_schedule
        integer(c_int32_t) :: tmcs_eq, coa, ovrr
        real(c_double)     :: ovrr_para
        integer(c_int32_t) :: ovrr_mcs, pt, exchange_interval
    end type ether_schedule

    type, bind(C) :: ether_learn_desc
        integer(c_int32_t) :: patch, hidden
        integer(c_int32_t) :: seed       ! uint32_t in C
        integer(c_int64_t) :: capacity
    end type ether_learn_desc

    interface
        integer(c_int) function ether_create(desc, ctx) bind(C, name="ether_create")
            import :: c_int, c_ptr, ether_desc
            type(ether_desc), intent(in) :: desc
            type(c_ptr), intent(out) :: ctx
        end function
        integer(c_int) function ether_destroy(ctx) bind(C, name="ether_destroy")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        type(c_ptr) function ether_last_error() bind(C, name="ether_last_error")
            import :: c_ptr
        end function
        integer(c_int) function ether_set_beta(ctx, beta) bind(C, name="ether_set_beta")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: beta(*)
        end function
        integer(c_int) function ether_set_ladder(ctx, n_slots, beta) bind(C, name="ether_set_ladder")
            import :: c_int, c_ptr, c_double, c_int32_t
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: n_slots
            real(c_double), intent(in) :: beta(*)
        end function
        integer(c_int) function ether_set_streams(ctx, stream, step) bind(C, name="ether_set_streams")
            import :: c_int, c_ptr, c_int32_t
            type(c_ptr), value :: ctx
            integer(c_int32_t), intent(in) :: stream(*), step(*)
        end function
        integer(c_int) function ether_set_spins(ctx, replica, ion) bind(C, name="ether_set_spins")
            import :: c_int, c_ptr, c_double, c_int32_t
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: replica
            real(c_double), intent(in) :: ion(0:8, *)
        end function
        integer(c_int) function ether_get_spins(ctx, replica, ion) bind(C, name="ether_get_spins")
            import :: c_int, c_ptr, c_double, c_int32_t
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: replica
            real(c_double), intent(inout) :: ion(0:8, *)
        end function
        integer(c_int) function ether_set_spins_batch(ctx, r0, n, ion) bind(C, name="ether_set_spins_batch")
            import :: c_int, c_ptr, c_double, c_int32_t
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: r0, n
            real(c_double), intent(in) :: ion(0:8, *)
        end function
        integer(c_int) function ether_get_spins_batch(ctx, r0, n, ion) bind(C, name="ether_get_spins_batch")
            import :: c_int, c_ptr, c_double, c_int32_t
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: r0, n
            real(c_double), intent(inout) :: ion(0:8, *)
        end function
        integer(c_int) function ether_spins_batch_split(ctx, get_kernel, set_kernel) &
                bind(C, name="ether_spins_batch_split")
            import :: c_int, c_ptr, c_int32_t
            type(c_ptr), value :: ctx
            integer(c_int32_t), intent(out) :: get_kernel, set_kernel
        end function
        integer(c_int) function ether_fresh_spins(ctx) bind(C, name="ether_fresh_spins")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function ether_metropolis(ctx, nsweeps, accept) bind(C, name="ether_metropolis")
            import :: c_int, c_ptr, c_double, c_int32_t
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: nsweeps
            real(c_double), intent(out) :: accept(*)
        end function
        integer(c_int) function ether_overrelaxation(ctx, ovrr_para) bind(C, name="ether_overrelaxation")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), value :: ovrr_para
        end function
        integer(c_int) function ether_tot_energy(ctx, e) bind(C, name="ether_tot_energy")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: e(*)
        end function
        integer(c_int) function ether_tot_magnetisation(ctx, m) bind(C, name="ether_tot_magnetisation")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: m(3, *)
        end function
        integer(c_int) function ether_observable(ctx, step, tmcs_eq, coa) bind(C, name="ether_observable")
            import :: c_int, c_ptr, c_int32_t
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: step, tmcs_eq, coa
        end function
        integer(c_int) function ether_zero_avg(ctx) bind(C, name="ether_zero_avg")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function ether_avg(ctx, out) bind(C, name="ether_avg")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: out(6, *)
        end function
        integer(c_int) function ether_per_repeat(ctx, mean, err) bind(C, name="ether_per_repeat")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: mean(6, *), err(6, *)
        end function
        integer(c_int) function ether_parallel_tempering(ctx, swap_count, accepted) &
                bind(C, name="ether_parallel_tempering")
            import :: c_int, c_ptr, c_int32_t
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: swap_count
            integer(c_int32_t), intent(out) :: accepted
        end function
        integer(c_int) function ether_mcs(ctx, sch, step0, nsteps, swap_count) bind(C, name="ether_mcs")
            import :: c_int, c_ptr, c_int32_t, ether_schedule
            type(c_ptr), value :: ctx
            type(ether_schedule), intent(in) :: sch
            integer(c_int32_t), value :: step0, nsteps
            integer(c_int32_t), intent(inout) :: swap_count
        end function
        integer(c_int) function ether_build_lattice(nbasis, basis_cart, basis_species, abc, sc, bc, &
                checkerboard, n_shells, nbd_dis, tol, cap, ion, stgg, nn) bind(C, name="ether_build_lattice")
            import :: c_int, c_int32_t, c_double, c_char
            integer(c_int32_t), value :: nbasis, checkerboard, n_shells, cap
            real(c_double), intent(in) :: basis_cart(3, *), abc(3, 3), nbd_dis(*)
            integer(c_int32_t), intent(in) :: basis_species(*), sc(3)
            character(kind=c_char), intent(in) :: bc(3)
            real(c_double), value :: tol
            real(c_double), intent(out) :: ion(0:8, *), stgg(*)
            integer(c_int32_t), intent(out) :: nn(*)
        end function
        ! batched sweeps over several contexts (no counterpart in the reference)
        integer(c_int) function ether_batch_create(members, n_members, batch) bind(C, name="ether_batch_create")
            import :: c_int, c_ptr, c_int32_t
            type(c_ptr), intent(in) :: members(*)
            integer(c_int32_t), value :: n_members
            type(c_ptr), intent(out) :: batch
        end function
        integer(c_int) function ether_batch_destroy(batch) bind(C, name="ether_batch_destroy")
            import :: c_int, c_ptr
            type(c_ptr), value :: batch
        end function
        integer(c_int) function ether_batch_metropolis(batch, nsweeps) bind(C, name="ether_batch_metropolis")
            import :: c_int, c_ptr, c_int32_t
            type(c_ptr), value :: batch
            integer(c_int32_t), value :: nsweeps
        end function
        integer(c_int) function ether_batch_mcs(batch, sch, step0, nsteps, swap_counts) bind(C, name="ether_batch_mcs")
            import :: c_int, c_ptr, c_int32_t, ether_schedule
            type(c_ptr), value :: batch
            type(ether_schedule), intent(in) :: sch
            integer(c_int32_t), value :: step0, nsteps
            integer(c_int32_t), intent(inout) :: swap_counts(*)
        end function
        integer(c_int) function ether_batch_autotune(batch, config, best_ms) bind(C, name="ether_batch_autotune")
            import :: c_int, c_ptr, c_int32_t, c_float
            type(c_ptr), value :: batch
            integer(c_int32_t), intent(out) :: config(4)
            real(c_float), intent(out) :: best_ms
        end function
        ! learned patch proposal (no counterpart in the reference)
        integer(c_int) function ether_learn_create(ctx, desc, learn) bind(C, name="ether_learn_create")
            import :: c_int, c_ptr, ether_learn_desc
            type(c_ptr), value :: ctx
            type(ether_learn_desc), intent(in) :: desc
            type(c_ptr), intent(out) :: learn
        end function
        integer(c_int) function ether_learn_destroy(learn) bind(C, name="ether_learn_destroy")
            import :: c_int, c_ptr
            type(c_ptr), value :: learn
        end function
        integer(c_int) function ether_learn_collect(learn, per_replica) bind(C, name="ether_learn_collect")
            import :: c_int, c_ptr, c_int32_t
            type(c_ptr), value :: learn
            integer(c_int32_t), value :: per_replica
        end function
        integer(c_int) function ether_learn_train(learn, steps, batch, lr, loss) bind(C, name="ether_learn_train")
            import :: c_int, c_ptr, c_int32_t, c_float, c_double
            type(c_ptr), value :: learn
            integer(c_int32_t), value :: steps, batch
            real(c_float), value :: lr
            real(c_double), intent(out) :: loss
        end function
        integer(c_int) function ether_learn_sweep(learn, nsweeps) bind(C, name="ether_learn_sweep")
            import :: c_int, c_ptr, c_int32_t
            type(c_ptr), value :: learn
            integer(c_int32_t), value :: nsweeps
        end function
        ! network widths (Ising 128, 32, 37152; Heisenberg 304, 96, 67936)
        integer(c_int) function ether_learn_batch_sweep(learns, n, nsweeps, plain_per_sweep) &
                bind(C, name="ether_learn_batch_sweep")
            import :: c_int, c_ptr, c_int32_t
            type(c_ptr), intent(in) :: learns(*)
            integer(c_int32_t), value :: n, nsweeps, plain_per_sweep
        end function
        integer(c_int) function ether_learn_get_shape(learn, n_inputs, n_outputs, n_params) &
                bind(C, name="ether_learn_get_shape")
            import :: c_int, c_ptr, c_int32_t
            type(c_ptr), value :: learn
            integer(c_int32_t), intent(out) :: n_inputs, n_outputs, n_params
        end function
        ! per-temperature acceptance (src/ether.f90:173) and the spiral-state averages
        ! (src/get_spiral_state.f90:127-140)
        integer(c_int) function ether_get_slot_accept_counts(ctx, counts) bind(C, name="ether_get_slot_accept_counts")
            import :: c_int, c_ptr, c_int64_t
            type(c_ptr), value :: ctx
            integer(c_int64_t), intent(out) :: counts(*)
        end function
        integer(c_int) function ether_spiral_avg(ctx, out) bind(C, name="ether_spiral_avg")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: out(3, *)
        end function
        ! get_moment_vectors (src/ether.f90:219) and get_spiral_state's setup (:69) and
        ! per-sample value (:207)
        integer(c_int) function ether_moment_vectors(ctx, mm) bind(C, name="ether_moment_vectors")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: mm(3, *)
        end function
        integer(c_int) function ether_spiral_setup(ctx, ss_dis, ss_direc, ss_latency, capacity, count) &
                bind(C, name="ether_spiral_setup")
            import :: c_int, c_ptr, c_double, c_int32_t, c_int64_t
            type(c_ptr), value :: ctx
            real(c_double), value :: ss_dis, ss_latency
            real(c_double), intent(in) :: ss_direc(3)
            integer(c_int32_t), value :: capacity
            integer(c_int64_t), intent(out) :: count
        end function
        integer(c_int) function ether_spiral_state(ctx, ss) bind(C, name="ether_spiral_state")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: ss(*)
        end function
        ! the structure factor of utility/Structure_Factor/structure_factor.f90:99-183, nq(1)
        ! a multiple of 64
        integer(c_int) function ether_structure_factor(ctx, abc, nq, q0, dq, sq, comp) &
                bind(C, name="ether_structure_factor")
            import :: c_int, c_ptr, c_double, c_float, c_int32_t
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: abc(3, 3), q0(3), dq(3)
            integer(c_int32_t), intent(in) :: nq(3)
            real(c_float), intent(out) :: sq(*), comp(3, *)
        end function
        ! accumulators, slots and the stream's end
        integer(c_int) function ether_get_sums(ctx, sums) bind(C, name="ether_get_sums")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: sums(7, *)
        end function
        integer(c_int) function ether_get_slots(ctx, slot_of_replica) bind(C, name="ether_get_slots")
            import :: c_int, c_ptr, c_int32_t
            type(c_ptr), value :: ctx
            integer(c_int32_t), intent(out) :: slot_of_replica(*)
        end function
        integer(c_int) function ether_sync(ctx) bind(C, name="ether_sync")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function ether_abi_version() bind(C, name="ether_abi_version")
            import :: c_int
        end function
        ! the whole program src/ether.f90 for one input directory; the directory names are
        ! C strings: trim(dir)//c_null_char
        integer(c_int) function ether_run(indir, outdir, flags, info) bind(C, name="ether_run")
            import :: c_int, c_char, c_int32_t, ether_run_info
            character(kind=c_char), intent(in) :: indir(*), outdir(*)
            integer(c_int32_t), value :: flags
            type(ether_run_info), intent(inout) :: info
        end function
    end interface
end module ether_gpu_mod
