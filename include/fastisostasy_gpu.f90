! fastisostasy_gpu.f90 — iso_c_binding interface to libfigpu.so (fi_gpu.h).
!
! The Fortran side of the drop-in boundary: module fastisostasy's routines
! (src/fastisostasy.f90) call these functions in place of their CPU bodies;
! the caller keeps isos_class / bsl_class and stores the GPU handle in one
! type(c_ptr) component.  Every bind(C) type below has the field order and
! kinds of its C struct in fi_gpu.h; every function of fi_gpu.h has an
! interface here with the same argument order.
!
! Arrays: pass the caller's contiguous real(c_double) arrays as assumed-size
! dummies (x fastest, the reference's own layout) or as c_loc pointers where
! the C side takes NULL for "absent".  Masks are integer(c_int8_t) 0/1.
!
! Status: every function returns FI_OK (0) or an FI_E_* code; fi_check
! turns a nonzero status into the reference's behaviour (write the message
! and stop, as src/fastisostasy.f90:197, 853, 868, 897 do).
module fastisostasy_gpu
    use iso_c_binding
    implicit none

    integer(c_int), parameter :: FI_OK = 0, FI_E_NAN = 1, FI_E_LARGE = 2, FI_E_STEP = 3, FI_E_OOM = 4
    integer(c_int), parameter :: FI_E_CONFIG = 5, FI_E_CUDA = 6, FI_E_TIMEOUT = 7, FI_E_ARG = 8
    integer(c_int), parameter :: FI_E_STATE = 9, FI_E_SIZE = 10, FI_E_CANCELLED = 11
    integer(c_int), parameter :: FI_PREC_FP64 = 0, FI_PREC_MIXED = 1
    integer(c_int), parameter :: FI_STATIC_MAX_N = 256

    ! fi_get_field selectors (padded grid)
    integer(c_int), parameter :: FI_FIELD_Z_BED = 0, FI_FIELD_DWDT = 1, FI_FIELD_W = 2, FI_FIELD_WE = 3
    integer(c_int), parameter :: FI_FIELD_HAF = 4, FI_FIELD_HICE = 5, FI_FIELD_Z_SS = 6, FI_FIELD_DZ_SS = 7
    integer(c_int), parameter :: FI_FIELD_CANOM_LOAD = 8, FI_FIELD_CANOM_FULL = 9, FI_FIELD_MASS_ANOM = 10
    integer(c_int), parameter :: FI_FIELD_MASKOCEAN = 11, FI_FIELD_MASKGROUNDED = 12, FI_FIELD_MASKCONTINENT = 13
    integer(c_int), parameter :: FI_FIELD_CANOM_MANTLE = 14, FI_FIELD_CANOM_LITHO = 15
    integer(c_int), parameter :: FI_FIELD_CANOM_SEAWATER = 16, FI_FIELD_CANOM_ICE = 17, FI_FIELD_X = 18
    integer(c_int), parameter :: FI_FIELD_KAPPA = 19, FI_FIELD_D_LITH = 20, FI_FIELD_ETA_EFF = 21
    integer(c_int), parameter :: FI_FIELD_R = 22, FI_FIELD_MASKACTIVE = 23, FI_FIELD_GE = 24, FI_FIELD_GN = 25

    ! isos_param_class (src/isostasy_defs.f90:34-100) after isos_par_load's
    ! unit conversion; string options as the integer codes of fi_gpu.h
    type, bind(C) :: fi_params
        integer(c_int32_t) :: method, interactive_sealevel, include_elastic, heterogeneous_ssh
        integer(c_int32_t) :: correct_compression, lithosphere, mantle, layering, lumping
        integer(c_int32_t) :: visc_scaling_method, nl, dt_method, stage_mode
        integer(c_int32_t) :: nx_target, ny_target, precision
        real(c_double) :: dt_diagnostics, min_pad, viscosity_scaling
        real(c_double) :: zl(8), viscosities(8), dl, eta_ref
        real(c_double) :: E, nu, rho_water, rho_ice, rho_seawater, rho_uppermantle, rho_litho, g
        real(c_double) :: r_earth, m_earth
        real(c_double) :: atol, rtol, dt_min, dt_max, dt_init, q
        real(c_double) :: tau
    end type

    ! bsl_class (src/barysealevel.f90:16-29); the series tables are the
    ! caller's arrays (c_loc), replacing the reference's file readers
    type, bind(C) :: fi_bsl
        integer(c_int32_t) :: method, constant_ocean_surface, n_series, n_aocean
        real(c_double) :: bsl_init, bsl_now, A_ocean_now, A_ocean_pd, time
        type(c_ptr) :: series_t, series_v, bsl_vec, aocean_vec
    end type

    ! isos_out_class (src/isostasy_defs.f90:185-200): c_loc of the ice-grid
    ! outputs, c_null_ptr for fields not wanted
    type, bind(C) :: fi_out
        type(c_ptr) :: z_bed, z_ss, dz_ss, w, we, dwdt, canom_full, Hice
        type(c_ptr) :: maskocean, maskgrounded, maskcontinent
    end type

    ! the arrays of a rheology file as nc_read_and_scale_* returns them
    type, bind(C) :: fi_rheology
        integer(c_int32_t) :: nx, ny, nz
        type(c_ptr) :: xc, yc, zc
        type(c_ptr) :: litho_thickness
        real(c_double) :: litho_thickness_scaling
        type(c_ptr) :: log10_viscosity
        type(c_ptr) :: stddev_log10_viscosity
        integer(c_int32_t) :: stddev_scaling
        real(c_double) :: rheo_smoothing_radius
    end type

    ! one solve for the request server
    type, bind(C) :: fi_request
        type(fi_params) :: p
        integer(c_int32_t) :: nx_ice, ny_ice
        real(c_double) :: dx, dy
        type(c_ptr) :: z_bed, H_ref, H_ice, D_lith, eta_eff, R, maskactive
        real(c_double) :: t0, t_end, dtt, bsl
    end type

    type, bind(C) :: fi_request_info
        integer(c_int32_t) :: state, status
        integer(c_int64_t) :: updates
        real(c_double) :: t_submit, t_admit, t_done
        character(kind=c_char) :: error(128)
    end type

    interface
        ! ---- isos_init / isos_end (src/fastisostasy.f90:64-473, 911-923)
        integer(c_int) function fi_create(p, nx_ice, ny_ice, dx, dy, K, h) bind(C, name="fi_create")
            import
            type(fi_params), intent(in) :: p
            integer(c_int), value :: nx_ice, ny_ice
            real(c_double), value :: dx, dy
            type(c_ptr), value :: K                  ! c_null_ptr, or c_loc of the padded K field
            type(c_ptr), intent(out) :: h
        end function
        integer(c_int) function fi_padded_dims(p, nx_ice, ny_ice, dx, dy, out6) bind(C, name="fi_padded_dims")
            import
            type(fi_params), intent(in) :: p
            integer(c_int), value :: nx_ice, ny_ice
            real(c_double), value :: dx, dy
            integer(c_int32_t), intent(out) :: out6(6)
        end function
        integer(c_int) function fi_destroy(h) bind(C, name="fi_destroy")
            import
            type(c_ptr), value :: h
        end function
        integer(c_int) function fi_dims(h, out8) bind(C, name="fi_dims")
            import
            type(c_ptr), value :: h
            integer(c_int32_t), intent(out) :: out8(8)
        end function
        integer(c_int) function fi_set_fields(h, D_lith, eta_eff, R, maskactive) bind(C, name="fi_set_fields")
            import
            type(c_ptr), value :: h, D_lith, eta_eff, R, maskactive
        end function
        integer(c_int) function fi_set_rheology(h, r) bind(C, name="fi_set_rheology")
            import
            type(c_ptr), value :: h
            type(fi_rheology), intent(in) :: r
        end function
        integer(c_int) function fi_set_kernels(h, GE, GN) bind(C, name="fi_set_kernels")
            import
            type(c_ptr), value :: h, GE, GN
        end function

        ! ---- isos_init_ref, isos_init_state, isos_update (:550-872)
        integer(c_int) function fi_init_ref(h, z_bed, H_ice, bsl, dz_ss) bind(C, name="fi_init_ref")
            import
            type(c_ptr), value :: h
            real(c_double), intent(in) :: z_bed(*), H_ice(*)
            real(c_double), value :: bsl
            type(c_ptr), value :: dz_ss              ! c_null_ptr when absent
        end function
        integer(c_int) function fi_init_state(h, z_bed, H_ice, time, bsl) bind(C, name="fi_init_state")
            import
            type(c_ptr), value :: h
            real(c_double), intent(in) :: z_bed(*), H_ice(*)
            real(c_double), value :: time
            type(fi_bsl), intent(inout) :: bsl
        end function
        integer(c_int) function fi_update(h, H_ice, time, bsl, out) bind(C, name="fi_update")
            import
            type(c_ptr), value :: h
            real(c_double), intent(in) :: H_ice(*)
            real(c_double), value :: time
            type(fi_bsl), intent(inout) :: bsl
            type(fi_out), intent(in) :: out
        end function
        integer(c_int) function fi_update_async(h, d_H_ice, time, bsl) bind(C, name="fi_update_async")
            import
            type(c_ptr), value :: h, d_H_ice         ! device pointer, or c_null_ptr to keep the load
            real(c_double), value :: time
            type(fi_bsl), intent(inout) :: bsl
        end function
        integer(c_int) function fi_synchronize(h) bind(C, name="fi_synchronize")
            import
            type(c_ptr), value :: h
        end function
        integer(c_int) function fi_set_max_rejections(h, max_per_update) bind(C, name="fi_set_max_rejections")
            import
            type(c_ptr), value :: h
            integer(c_int64_t), value :: max_per_update
        end function
        integer(c_int) function fi_metrics_json(h, buf, len) bind(C, name="fi_metrics_json")
            import
            type(c_ptr), value :: h
            character(kind=c_char), intent(out) :: buf(*)   ! NUL-terminated JSON line
            integer(c_size_t), value :: len
        end function

        ! ---- bsl_update (src/barysealevel.f90:195-252)
        integer(c_int) function fi_bsl_update(bsl, year_bp) bind(C, name="fi_bsl_update")
            import
            type(fi_bsl), intent(inout) :: bsl
            real(c_double), value :: year_bp
        end function

        ! ---- asynchronous output of isos%out
        integer(c_int64_t) function fi_output_bytes(h) bind(C, name="fi_output_bytes")
            import
            type(c_ptr), value :: h
        end function
        integer(c_int) function fi_output_async(h, dst) bind(C, name="fi_output_async")
            import
            type(c_ptr), value :: h, dst
        end function
        integer(c_int) function fi_output_wait(h) bind(C, name="fi_output_wait")
            import
            type(c_ptr), value :: h
        end function

        ! ---- inspection, parity entry points
        integer(c_int) function fi_get_field(h, which, out_padded) bind(C, name="fi_get_field")
            import
            type(c_ptr), value :: h
            integer(c_int), value :: which
            real(c_double), intent(out) :: out_padded(*)
        end function
        integer(c_int) function fi_get_scalars(h, out16) bind(C, name="fi_get_scalars")
            import
            type(c_ptr), value :: h
            real(c_double), intent(out) :: out16(16)
        end function
        integer(c_int) function fi_lvelva(h, w, canom_full, dwdt) bind(C, name="fi_lvelva")
            import
            type(c_ptr), value :: h
            real(c_double), intent(in) :: w(*), canom_full(*)
            real(c_double), intent(out) :: dwdt(*)
        end function
        integer(c_int) function fi_convolve(h, kernel, in_padded, out_padded) bind(C, name="fi_convolve")
            import
            type(c_ptr), value :: h
            integer(c_int), value :: kernel
            real(c_double), intent(in) :: in_padded(*)
            real(c_double), intent(out) :: out_padded(*)
        end function
        integer(c_int) function fi_lvelva_static(d_w, d_canom_full, d_maskactive, d_D_lith, d_eta_eff, d_kappa, &
                                                 d_R, d_dx_matrix, d_dy_matrix, nx, ny, dx, dy, g, nu, &
                                                 sec_per_year, d_dwdt, stream) bind(C, name="fi_lvelva_static")
            import
            type(c_ptr), value :: d_w, d_canom_full, d_maskactive, d_D_lith, d_eta_eff, d_kappa, d_R
            type(c_ptr), value :: d_dx_matrix, d_dy_matrix
            integer(c_int), value :: nx, ny
            real(c_double), value :: dx, dy, g, nu, sec_per_year
            type(c_ptr), value :: d_dwdt, stream
        end function

        ! ---- request server
        integer(c_int) function fi_serve_create(max_inflight, reserve_gb, s) bind(C, name="fi_serve_create")
            import
            integer(c_int), value :: max_inflight
            real(c_double), value :: reserve_gb
            type(c_ptr), intent(out) :: s
        end function
        integer(c_int) function fi_serve_submit(s, r, id) bind(C, name="fi_serve_submit")
            import
            type(c_ptr), value :: s
            type(fi_request), intent(in) :: r
            integer(c_int64_t), intent(out) :: id
        end function
        integer(c_int) function fi_serve_info(s, id, info) bind(C, name="fi_serve_info")
            import
            type(c_ptr), value :: s
            integer(c_int64_t), value :: id
            type(fi_request_info), intent(out) :: info
        end function
        integer(c_int) function fi_serve_wait(s, id, timeout_s, info) bind(C, name="fi_serve_wait")
            import
            type(c_ptr), value :: s
            integer(c_int64_t), value :: id
            real(c_double), value :: timeout_s
            type(fi_request_info), intent(out) :: info
        end function
        integer(c_int) function fi_serve_result(s, id, w_ice, z_bed_ice) bind(C, name="fi_serve_result")
            import
            type(c_ptr), value :: s
            integer(c_int64_t), value :: id
            type(c_ptr), value :: w_ice, z_bed_ice
        end function
        real(c_double) function fi_serve_clock(s) bind(C, name="fi_serve_clock")
            import
            type(c_ptr), value :: s
        end function
        integer(c_int) function fi_serve_cancel(s, id) bind(C, name="fi_serve_cancel")
            import
            type(c_ptr), value :: s
            integer(c_int64_t), value :: id
        end function
        integer(c_int) function fi_serve_destroy(s) bind(C, name="fi_serve_destroy")
            import
            type(c_ptr), value :: s
        end function

        ! ---- ensembles
        integer(c_int) function fi_batch_update(hs, n, time, bsl) bind(C, name="fi_batch_update")
            import
            type(c_ptr), intent(in) :: hs(*)
            integer(c_int), value :: n
            real(c_double), value :: time
            type(fi_bsl), intent(inout) :: bsl(*)
        end function
        integer(c_int) function fi_batch_synchronize(hs, n, status) bind(C, name="fi_batch_synchronize")
            import
            type(c_ptr), intent(in) :: hs(*)
            integer(c_int), value :: n
            integer(c_int32_t), intent(out) :: status(*)
        end function
        integer(c_int) function fi_batch_create(hs, n, b) bind(C, name="fi_batch_create")
            import
            type(c_ptr), intent(in) :: hs(*)
            integer(c_int), value :: n
            type(c_ptr), intent(out) :: b
        end function
        integer(c_int) function fi_batch_set_priority(b, level) bind(C, name="fi_batch_set_priority")
            import
            type(c_ptr), value :: b
            integer(c_int), value :: level
        end function
        integer(c_int) function fi_batch_autotune(b, chosen4) bind(C, name="fi_batch_autotune")
            import
            type(c_ptr), value :: b
            integer(c_int32_t), intent(out) :: chosen4(4)
        end function
        integer(c_int) function fi_batch_step(b, time, bsl) bind(C, name="fi_batch_step")
            import
            type(c_ptr), value :: b
            real(c_double), value :: time
            type(fi_bsl), intent(inout) :: bsl(*)
        end function
        integer(c_int) function fi_batch_wait(b, status) bind(C, name="fi_batch_wait")
            import
            type(c_ptr), value :: b
            integer(c_int32_t), intent(out) :: status(*)
        end function
        integer(c_int) function fi_batch_destroy(b) bind(C, name="fi_batch_destroy")
            import
            type(c_ptr), value :: b
        end function

        ! ---- analytical ELVA disc (src/isostasy_benchmarks.f90:74-280)
        integer(c_int) function fi_elva_disk(nx, ny, dx, r0, h0, eta, D, rho_ice, rho_m, g, time_yr, out) &
                bind(C, name="fi_elva_disk")
            import
            integer(c_int), value :: nx, ny
            real(c_double), value :: dx, r0, h0, eta, D, rho_ice, rho_m, g, time_yr
            real(c_double), intent(out) :: out(*)
        end function

        ! ---- restart state
        integer(c_size_t) function fi_state_size(h) bind(C, name="fi_state_size")
            import
            type(c_ptr), value :: h
        end function
        integer(c_int) function fi_state_export(h, buf) bind(C, name="fi_state_export")
            import
            type(c_ptr), value :: h
            real(c_double), intent(out) :: buf(*)
        end function
        integer(c_int) function fi_state_import(h, buf) bind(C, name="fi_state_import")
            import
            type(c_ptr), value :: h
            real(c_double), intent(in) :: buf(*)
        end function

        ! ---- streams, counters, profiling, errors
        type(c_ptr) function fi_stream(h) bind(C, name="fi_stream")
            import
            type(c_ptr), value :: h
        end function
        integer(c_int) function fi_set_stream(h, stream) bind(C, name="fi_set_stream")
            import
            type(c_ptr), value :: h, stream
        end function
        integer(c_long_long) function fi_launch_count(h) bind(C, name="fi_launch_count")
            import
            type(c_ptr), value :: h
        end function
        integer(c_int) function fi_profile(h, enable) bind(C, name="fi_profile")
            import
            type(c_ptr), value :: h
            integer(c_int), value :: enable
        end function
        integer(c_int) function fi_engine_trace(h, out, n) bind(C, name="fi_engine_trace")
            import
            type(c_ptr), value :: h
            integer(c_long_long), intent(out) :: out(*)
            integer(c_int), value :: n
        end function
        integer(c_int) function fi_profile_read(h, ms, counts, n) bind(C, name="fi_profile_read")
            import
            type(c_ptr), value :: h
            real(c_double), intent(out) :: ms(*)
            integer(c_long_long), intent(out) :: counts(*)
            integer(c_int), value :: n
        end function
        type(c_ptr) function fi_last_error(h) bind(C, name="fi_last_error")
            import
            type(c_ptr), value :: h
        end function
        integer(c_int) function fi_version() bind(C, name="fi_version")
            import
        end function
    end interface

contains

    ! fi_last_error as a Fortran string
    function fi_error_text(h) result(msg)
        type(c_ptr), intent(in) :: h
        character(len=256) :: msg
        character(kind=c_char), pointer :: s(:)
        type(c_ptr) :: p
        integer :: i
        msg = ""
        p = fi_last_error(h)
        if (.not. c_associated(p)) return
        call c_f_pointer(p, s, [256])
        do i = 1, 256
            if (s(i) == c_null_char) exit
            msg(i:i) = s(i)
        end do
    end function

    ! The reference stops on every failure; so does this, unless the caller
    ! asks for the status.
    subroutine fi_check(h, stat, where, status_out)
        type(c_ptr), intent(in) :: h
        integer(c_int), intent(in) :: stat
        character(len=*), intent(in) :: where
        integer(c_int), intent(out), optional :: status_out
        if (present(status_out)) then
            status_out = stat
            return
        end if
        if (stat /= FI_OK) then
            write(*, *) trim(where), ": status ", stat, ": ", trim(fi_error_text(h))
            stop
        end if
    end subroutine

end module fastisostasy_gpu
