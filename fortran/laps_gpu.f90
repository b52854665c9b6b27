! iso_c_binding interface to liblaps_gpu.so (include/laps_gpu.h) for a Fortran LAPS host.
! Not compile-checked in this repository (no Fortran compiler is installed here); the types
! and argument passing follow the C declarations one-for-one.
module laps_gpu
    use, intrinsic :: iso_c_binding
    implicit none

    integer(c_int), parameter :: LAPS_OK = 0
    integer(c_int), parameter :: LAPS_STATUS_NAN = 1, LAPS_STATUS_DT_FLOOR = 2, LAPS_STATUS_DEVICE_TIMEOUT = 4
    integer(c_int), parameter :: LAPS_VARIANT_3DC = 0, LAPS_VARIANT_3DI = 1, LAPS_VARIANT_2DC = 2
    integer(c_int), parameter :: LAPS_PREC_FP64 = 0, LAPS_PREC_DD = 1, LAPS_PREC_FP32 = 2, &
        LAPS_PREC_FP32_F64 = 3
    integer(c_int), parameter :: LAPS_LAYOUT_PRIMITIVE = 0, LAPS_LAYOUT_CONSERVED = 1

    type, bind(C) :: laps_params
        integer(c_int) :: variant, precision
        integer(c_int) :: nx, ny, nz
        real(c_double) :: Lx, Ly, Lz
        real(c_double) :: adiabatic_index
        integer(c_int) :: if_resis, if_resis_exp
        real(c_double) :: resistivity
        integer(c_int) :: if_visc, if_visc_exp
        real(c_double) :: viscosity
        integer(c_int) :: if_conserve_background
        integer(c_int) :: dealias_option
        real(c_double) :: afx, afy, afz
        real(c_double) :: cfl
        integer(c_int) :: if_AEB
        real(c_double) :: radius0, Ur0
        integer(c_int) :: if_corotating
        real(c_double) :: corotating_angle
        integer(c_int) :: if_Hall
        real(c_double) :: ion_inertial_length
        real(c_double) :: rho0
        integer(c_int) :: if_z_radial, if_limit_dt_increase, dstep_calcdt
        integer(c_int) :: device, timeout_ms
        integer(c_long_long) :: mem_cap_bytes
        integer(c_int) :: reserved(8)
    end type laps_params

    type, bind(C) :: laps_ic
        integer(c_int) :: ifield, ipert
        real(c_double) :: T0, rho0, B0, a0
        real(c_double) :: U_fast, U_slow, n_fast, n_slow, press0, shear_width
        real(c_double) :: bx0, by0, bz0, db0, in_out_ratio, dv0, drho0
        integer(c_int) :: nmodex, nmodey, nmodez, wave_number_jet
        real(c_double) :: jet_width, Vjet
        real(c_double) :: B0_SB, dB_SB, R0_SB, R1_SB, H_SB, Rm_SB, Rd_SB
    end type laps_ic

    type, bind(C) :: laps_diag
        real(c_double) :: time, dt, radius
        real(c_double) :: uu_ave(8), uu_rms(8), rho_u2(3)
        real(c_double) :: max_divB, max_divB_real, max_divV_real, e_kin, e_mag, h_cross, h_mag
    end type laps_diag

    type, bind(C) :: laps_info
        integer(c_long_long) :: device_bytes
        integer(c_int) :: kx_keep, ky_keep, kz_keep
        integer(c_int) :: kernels_per_step
        integer(c_int) :: graph
    end type laps_info

    interface
        integer(c_int) function laps_params_default(p) bind(C, name='laps_params_default')
            import :: c_int, laps_params
            type(laps_params), intent(out) :: p
        end function
        integer(c_int) function laps_create(p, ctx) bind(C, name='laps_create')
            import :: c_int, c_ptr, laps_params
            type(laps_params), intent(in) :: p
            type(c_ptr), intent(out) :: ctx
        end function
        subroutine laps_destroy(ctx) bind(C, name='laps_destroy')
            import :: c_ptr
            type(c_ptr), value :: ctx
        end subroutine
        integer(c_int) function laps_upload_state(ctx, uu, layout) bind(C, name='laps_upload_state')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: uu(*)
            integer(c_int), value :: layout
        end function
        integer(c_int) function laps_ic_default(ic) bind(C, name='laps_ic_default')
            import :: c_int, laps_ic
            type(laps_ic), intent(out) :: ic
        end function
        integer(c_long_long) function laps_ic_nphases(ic) bind(C, name='laps_ic_nphases')
            import :: c_long_long, laps_ic
            type(laps_ic), intent(in) :: ic
        end function
        ! in place of background_fields_initialize + perturbation_initialize +
        ! initial_calc_conserve_variable + transform_uu_real_to_fourier (mhd.f90:110-122);
        ! phs: the phases random_number drew (times 2 pi), laps_ic_nphases of them
        integer(c_int) function laps_init_fields(ctx, ic, phs, nphases) bind(C, name='laps_init_fields')
            import :: c_int, c_ptr, c_double, c_long_long, laps_ic
            type(c_ptr), value :: ctx
            type(laps_ic), intent(in) :: ic
            real(c_double), intent(in) :: phs(*)
            integer(c_long_long), value :: nphases
        end function
        integer(c_int) function laps_set_time(ctx, time) bind(C, name='laps_set_time')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), value :: time
        end function
        integer(c_int) function laps_vardt(ctx, dt) bind(C, name='laps_vardt')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: dt
        end function
        integer(c_int) function laps_step(ctx, nsteps, time, dt, status) bind(C, name='laps_step')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: nsteps
            real(c_double), intent(out) :: time, dt
            integer(c_int), intent(out) :: status
        end function
        integer(c_int) function laps_rk_stage(ctx, irk) bind(C, name='laps_rk_stage')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), value :: irk
        end function
        integer(c_int) function laps_download_state(ctx, uu, uu_prim) bind(C, name='laps_download_state')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: uu(*), uu_prim(*)
        end function
        integer(c_int) function laps_diagnostics(ctx, d) bind(C, name='laps_diagnostics')
            import :: c_int, c_ptr, laps_diag
            type(c_ptr), value :: ctx
            type(laps_diag), intent(out) :: d
        end function
        integer(c_int) function laps_spectrum(ctx, nshell, e_u, e_b) bind(C, name='laps_spectrum')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: nshell
            real(c_double), intent(out) :: e_u(*), e_b(*)
        end function
        integer(c_int) function laps_batch_create(members, n, batch) bind(C, name='laps_batch_create')
            import :: c_int, c_ptr, laps_params
            type(laps_params), intent(in) :: members(*)
            integer(c_int), value :: n
            type(c_ptr), intent(out) :: batch
        end function
        integer(c_int) function laps_batch_member(batch, i, ctx) bind(C, name='laps_batch_member')
            import :: c_int, c_ptr
            type(c_ptr), value :: batch
            integer(c_int), value :: i
            type(c_ptr), intent(out) :: ctx
        end function
        integer(c_int) function laps_batch_step(batch, nsteps, time, dt, status) bind(C, name='laps_batch_step')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: batch
            integer(c_int), value :: nsteps
            real(c_double), intent(out) :: time(*), dt(*)
            integer(c_int), intent(out) :: status(*)
        end function
        subroutine laps_batch_destroy(batch) bind(C, name='laps_batch_destroy')
            import :: c_ptr
            type(c_ptr), value :: batch
        end subroutine
        integer(c_int) function laps_write_output(ctx, path, layout) bind(C, name='laps_write_output')
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: path(*)   ! NUL-terminated, e.g. 'out007.dat'//c_null_char
            integer(c_int), value :: layout
        end function
        integer(c_int) function laps_read_restart(ctx, path, time) bind(C, name='laps_read_restart')
            import :: c_int, c_ptr, c_char, c_double
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: path(*)
            real(c_double), intent(out) :: time
        end function
        integer(c_int) function laps_calc_flux(ctx, flux) bind(C, name='laps_calc_flux')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: flux(*)
        end function
        integer(c_int) function laps_transform_flux(ctx, flux_fourier) bind(C, name='laps_transform_flux')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: flux_fourier(*)
        end function
        integer(c_int) function laps_calc_rhs(ctx, fnl) bind(C, name='laps_calc_rhs')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: fnl(*)
        end function
        integer(c_int) function laps_dealias(ctx) bind(C, name='laps_dealias')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function laps_wait(ctx, timeout_ms) bind(C, name='laps_wait')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), value :: timeout_ms
        end function
        ! the granular calls of the reference's stage, in its order (mhd.f90:303-325)
        integer(c_int) function laps_transform_uu_k2r(ctx, uu) bind(C, name='laps_transform_uu_k2r')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: uu(*)
        end function
        integer(c_int) function laps_update_prim(ctx, uu_prim) bind(C, name='laps_update_prim')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: uu_prim(*)
        end function
        ! uu_fourier(kx,ky,kz,1:8) as interleaved (re, im) pairs
        integer(c_int) function laps_download_spectral(ctx, uf) bind(C, name='laps_download_spectral')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: uf(*)
        end function
        integer(c_int) function laps_upload_spectral(ctx, uf) bind(C, name='laps_upload_spectral')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: uf(*)
        end function
        integer(c_int) function laps_get_time(ctx, time, dt) bind(C, name='laps_get_time')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: time, dt
        end function
        integer(c_int) function laps_get_info(ctx, info) bind(C, name='laps_get_info')
            import :: c_int, c_ptr, laps_info
            type(c_ptr), value :: ctx
            type(laps_info), intent(out) :: info
        end function
        integer(c_int) function laps_step_profiled(ctx, nsteps, pass_ms, total_ms, status) &
                bind(C, name='laps_step_profiled')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: nsteps
            real(c_double), intent(out) :: pass_ms(6), total_ms
            integer(c_int), intent(out) :: status
        end function
        ! data_process/3D_C/statistics.c on the device: out(n_axis, 4)
        integer(c_int) function laps_angle_statistics(ctx, axis, out) bind(C, name='laps_angle_statistics')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: axis
            real(c_double), intent(out) :: out(*)
        end function
        integer(c_int) function laps_set_schedule(ctx, bits) bind(C, name='laps_set_schedule')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), value :: bits
        end function
        integer(c_int) function laps_get_schedule(ctx, bits) bind(C, name='laps_get_schedule')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), intent(out) :: bits
        end function
        integer(c_int) function laps_batch_size(batch) bind(C, name='laps_batch_size')
            import :: c_int, c_ptr
            type(c_ptr), value :: batch
        end function
        ! device arrays (c_loc of a CUDA Fortran / OpenACC device array, or a cudaMalloc pointer)
        integer(c_int) function laps_transform_uu_real_to_fourier_noalloc(uu, uf, nx, ny, nz, nfields, stream) &
                bind(C, name='laps_transform_uu_real_to_fourier_noalloc')
            import :: c_int, c_ptr
            type(c_ptr), value :: uu, uf
            integer(c_int), value :: nx, ny, nz, nfields
            type(c_ptr), value :: stream
        end function
        integer(c_int) function laps_state_real_device(ctx, uu_dev) bind(C, name='laps_state_real_device')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx, uu_dev
        end function
        integer(c_int) function laps_add_spectral_device(ctx, duf_dev, scale) bind(C, name='laps_add_spectral_device')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx, duf_dev
            real(c_double), value :: scale
        end function
        type(c_ptr) function laps_batch_last_error(batch) bind(C, name='laps_batch_last_error')
            import :: c_ptr
            type(c_ptr), value :: batch
        end function
        type(c_ptr) function laps_last_error(ctx) bind(C, name='laps_last_error')
            import :: c_ptr
            type(c_ptr), value :: ctx
        end function
    end interface
end module laps_gpu
