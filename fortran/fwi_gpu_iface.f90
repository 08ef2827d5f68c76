!! fwi_gpu_iface.f90 -- iso_c_binding interface to libfwi_gb300.so
!!
!! The reference driver keeps its call signatures; each routine on the hot
!! path gains a GPU twin with the same arguments.  Fortran passes everything
!! by reference, which is exactly the C ABI of include/fwi_gb300.h, so the
!! dummies below carry no VALUE attribute except where the C side takes a
!! scalar by value.  Default INTEGER and REAL must be 4 bytes (c_int,
!! c_float), as in the reference build (mpif90 -O3, no -fdefault-real-8).
module fwi_gpu_iface
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: FWI_OK = 0
  ! fwi_survey_desc%flags bits
  integer(c_int), parameter :: FWI_SURVEY_NO_GRAPH = 1, FWI_SURVEY_RECOMPUTE = 2, FWI_SURVEY_SINGLE_STEP = 4, &
                                FWI_SURVEY_FUSED_STEP = 8, FWI_SURVEY_GRAPH = 16

  type, bind(C) :: fwi_shot
     integer(c_int) :: x0, nx, num_sou, num_rec
     type(c_ptr)    :: nxSou, nySou, nxRec, nyRec
     type(c_ptr)    :: src, obs
     real(c_double) :: grad_weight, misfit_weight
  end type fwi_shot

  type, bind(C) :: fwi_survey_desc
     integer(c_int)    :: ny, nx_model
     real(c_float)     :: d, dt
     integer(c_int)    :: nt, store_snap, acc, dpml, numtasks
     integer(c_int)    :: snap_form, grad_form, nshots
     type(c_ptr)       :: shots, water_rows
     integer(c_size_t) :: hbm_budget
     integer(c_int)    :: wave_shots, band_rows, flags
     integer(c_int)    :: tile_kernel, tile_rows, tile_edge_rows
  end type fwi_survey_desc

  interface
     integer(c_int) function fwi_init(device) bind(C, name="fwi_init")
       import :: c_int
       integer(c_int), value :: device
     end function fwi_init

     integer(c_int) function fwi_set_solver_options(acc, dpml) bind(C, name="fwi_set_solver_options")
       import :: c_int
       integer(c_int), value :: acc, dpml
     end function fwi_set_solver_options

     !! solver_acoustic_SS (src/solver_acoustic_SS.f90:9-11), same 21 arguments
     integer(c_int) function fwi_solver_acoustic_ss(rank, iprop, NumSou, NumRec, nxSou, nySou, &
          nxRec, nyRec, S, Sadj, d, dt, ny, nx, ctmp, store_snap, nt_Store, nt, kernel, Fields, &
          Rec_point) bind(C, name="fwi_solver_acoustic_ss")
       import :: c_int, c_float
       integer(c_int) :: rank, iprop, NumSou, NumRec, ny, nx, store_snap, nt_Store, nt
       integer(c_int) :: nxSou(*), nySou(*), nxRec(*), nyRec(*)
       real(c_float)  :: S(*), Sadj(*), d, dt, ctmp(*), kernel(*), Fields(*), Rec_point(*)
     end function fwi_solver_acoustic_ss

     !! Misfit_function (src/Misfit.f90:1), misfit_type = 1
     integer(c_int) function fwi_misfit_function(rank, freq, Data_Synth, Data_trace, NumRec, nt, dt, &
          Misfit, AdjSource, misfit64) bind(C, name="fwi_misfit_function")
       import :: c_int, c_float, c_double
       integer(c_int) :: rank, NumRec, nt
       real(c_float)  :: freq, dt, Misfit
       real(c_float)  :: Data_Synth(*), Data_trace(*), AdjSource(*)
       real(c_double) :: misfit64
     end function fwi_misfit_function

     !! Beta_calculous (src/Beta_calculous.f90:1)
     integer(c_int) function fwi_beta_calculous(Grad, OldGrad, nx, ny, Beta, num64, den64) &
          bind(C, name="fwi_beta_calculous")
       import :: c_int, c_float, c_double
       real(c_float)  :: Grad(*), OldGrad(*), Beta
       integer(c_int) :: nx, ny
       real(c_double) :: num64, den64
     end function fwi_beta_calculous

     !! calculate_misfit_gradient (src/calculate_misfit_gradient.f90:1) for all shots at once
     integer(c_int) function fwi_misfit_gradient_batch(desc, lambda, step, Misfit, Grad) &
          bind(C, name="fwi_misfit_gradient_batch")
       import :: c_int, c_float, fwi_survey_desc
       type(fwi_survey_desc) :: desc
       real(c_float)         :: lambda(*), Misfit, Grad(*)
       integer(c_int), value :: step
     end function fwi_misfit_gradient_batch

     !! time_filter (src/time_filter.f90:1): Butterworth filter of Data_trace(nt,Num) in place
     integer(c_int) function fwi_time_filter(Data_trace, nt, dt, Num, typef, f1, fc) &
          bind(C, name="fwi_time_filter")
       import :: c_int, c_float
       real(c_float)  :: Data_trace(*), dt, f1, fc
       integer(c_int) :: nt, Num, typef
     end function fwi_time_filter

     !! interpolation_akima (src/interpolation_akima.f90:1)
     integer(c_int) function fwi_interpolation_akima(Data_tmp, dt_Data, nt_Data, Data_trace, NumRec, dt, nt) &
          bind(C, name="fwi_interpolation_akima")
       import :: c_int, c_float
       real(c_float)  :: Data_tmp(*), Data_trace(*), dt_Data, dt
       integer(c_int) :: nt_Data, NumRec, nt
     end function fwi_interpolation_akima

     !! device-resident survey: create once per band, run once per gradient or
     !! line-search trial (the driver loop of FWI.f90), destroy at the end
     integer(c_int) function fwi_survey_create(desc, s) bind(C, name="fwi_survey_create")
       import :: c_int, c_ptr, fwi_survey_desc
       type(fwi_survey_desc) :: desc
       type(c_ptr)           :: s
     end function fwi_survey_create

     integer(c_int) function fwi_survey_destroy(s) bind(C, name="fwi_survey_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: s
     end function fwi_survey_destroy

     integer(c_int) function fwi_survey_set_lambda(s, lambda) bind(C, name="fwi_survey_set_lambda")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: s
       real(c_float)      :: lambda(*)
     end function fwi_survey_set_lambda

     integer(c_int) function fwi_survey_set_observed(s, obs_packed) bind(C, name="fwi_survey_set_observed")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: s
       real(c_float)      :: obs_packed(*)
     end function fwi_survey_set_observed

     !! the per-trial time axis (FWI.f90:225-230): resampled sources and observed traces
     integer(c_int) function fwi_survey_set_time(s, dt, nt, src, obs) bind(C, name="fwi_survey_set_time")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value    :: s
       real(c_float), value  :: dt
       integer(c_int), value :: nt
       real(c_float)         :: src(*), obs(*)
     end function fwi_survey_set_time

     !! calculate_misfit_gradient: step 1 gradient, step 2 line-search trial
     integer(c_int) function fwi_survey_run(s, step, misfit, grad) bind(C, name="fwi_survey_run")
       import :: c_int, c_ptr, c_float, c_double
       type(c_ptr), value    :: s
       integer(c_int), value :: step
       real(c_double)        :: misfit
       real(c_float)         :: grad(*)
     end function fwi_survey_run

     !! the FP64 gradient stack of the last run (the rank's term of the MPI_REDUCE of Grad)
     integer(c_int) function fwi_survey_get_stack(s, stack) bind(C, name="fwi_survey_get_stack")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: s
       real(c_double)     :: stack(*)
     end function fwi_survey_get_stack

     !! the plan fwi_misfit_gradient_batch keeps: how many were built, free it
     integer(c_int64_t) function fwi_batch_plans() bind(C, name="fwi_batch_plans")
       import :: c_int64_t
     end function fwi_batch_plans

     integer(c_int) function fwi_batch_release() bind(C, name="fwi_batch_release")
       import :: c_int
     end function fwi_batch_release

     !! FWI.f90:175: nut = 1/100/maxval(abs(Search/log(var_orig)))
     integer(c_int) function fwi_first_step(Search, var_orig, nx, ny, nut) bind(C, name="fwi_first_step")
       import :: c_int, c_float
       real(c_float)  :: Search(*), var_orig(*), nut
       integer(c_int) :: nx, ny
     end function fwi_first_step

     !! FWI.f90:227, :315: lambda = exp(Search*step)*var_orig
     integer(c_int) function fwi_model_update(Search, var_orig, step, nx, ny, lambda) &
          bind(C, name="fwi_model_update")
       import :: c_int, c_float
       real(c_float)  :: Search(*), var_orig(*), step, lambda(*)
       integer(c_int) :: nx, ny
     end function fwi_model_update

     !! get_mcs_data.f90:113-114,147-155,503-512 (scalars by value)
     integer(c_int) function fwi_mcs_geometry(xs, shot_depth, streamer_depth, near_offset, drec, dmodel, &
          num_rec, nxSou, nySou, nxRec, nyRec) bind(C, name="fwi_mcs_geometry")
       import :: c_int, c_float
       real(c_float), value  :: xs, shot_depth, streamer_depth, near_offset, drec, dmodel
       integer(c_int), value :: num_rec
       integer(c_int)        :: nxSou, nySou, nxRec(*), nyRec(*)
     end function fwi_mcs_geometry

     !! get_was_data.f90:112-115,155-159,201-205,223-231,584-613
     integer(c_int) function fwi_was_geometry(num_obs, xobs, zobs, num_shots, xshot, bat, shot_depth, dmodel, &
          nxmodel, relocate, nxSou, nySou, nxRec, nyRec, bat_model, bat_model_grid) bind(C, name="fwi_was_geometry")
       import :: c_int, c_float
       integer(c_int), value :: num_obs, num_shots, nxmodel, relocate
       real(c_float), value  :: shot_depth, dmodel
       real(c_float)         :: xobs(*), zobs(*), xshot(*), bat(*), bat_model(*)
       integer(c_int)        :: nxSou(*), nySou(*), nxRec(*), nyRec, bat_model_grid(*)
     end function fwi_was_geometry

     !! Ricker_mcs (get_mcs_data.f90:331)
     integer(c_int) function fwi_ricker(freq, dt, nt, out) bind(C, name="fwi_ricker")
       import :: c_int, c_float
       real(c_float), value  :: freq, dt
       integer(c_int), value :: nt
       real(c_float)         :: out(*)
     end function fwi_ricker

     !! calculate_misfit_gradient.f90:198-203
     integer(c_int) function fwi_time_rules(lambda, ny, nx, dmodel, tfin, store_snap, dt, nt, nt_Store) &
          bind(C, name="fwi_time_rules")
       import :: c_int, c_float
       real(c_float)         :: lambda(*), dt
       integer(c_int), value :: ny, nx, store_snap
       real(c_float), value  :: dmodel, tfin
       integer(c_int)        :: nt, nt_Store
     end function fwi_time_rules

     !! Butterworth order of fwi_time_filter (the reference's n = 6)
     integer(c_int) function fwi_set_filter_order(order) bind(C, name="fwi_set_filter_order")
       import :: c_int
       integer(c_int), value :: order
     end function fwi_set_filter_order

     !! SU files (paths: null-terminated character strings)
     integer(c_int) function fwi_su_info(path, big_endian, ns, dt, ntraces) bind(C, name="fwi_su_info")
       import :: c_int, c_float, c_char
       character(kind=c_char) :: path(*)
       integer(c_int), value  :: big_endian
       integer(c_int)         :: ns, ntraces
       real(c_float)          :: dt
     end function fwi_su_info

     integer(c_int) function fwi_su_read(path, nt, ntr, big_endian, out) bind(C, name="fwi_su_read")
       import :: c_int, c_float, c_char
       character(kind=c_char) :: path(*)
       integer(c_int), value  :: nt, ntr, big_endian
       real(c_float)          :: out(*)
     end function fwi_su_read

     !! get_obs_data (get_was_data.f90:241-288): paths(k) = c_loc of each OBS file name
     integer(c_int) function fwi_su_supershot(paths, nsrc, coding, nt, ntr, big_endian, raw_data) &
          bind(C, name="fwi_su_supershot")
       import :: c_int, c_float, c_ptr
       type(c_ptr)           :: paths(*)
       integer(c_int), value :: nsrc, nt, ntr, big_endian
       real(c_float)         :: coding(*), raw_data(*)
     end function fwi_su_supershot

     !! write_new_data (auxiliar.f90:433)
     integer(c_int) function fwi_su_write(path, data, nt, ntr, dt, big_endian) bind(C, name="fwi_su_write")
       import :: c_int, c_float, c_char
       character(kind=c_char) :: path(*)
       real(c_float)          :: data(*)
       integer(c_int), value  :: nt, ntr, big_endian
       real(c_float), value   :: dt
     end function fwi_su_write

     !! navigation lists (read_nav_shot_mcs, read_nav_shot_was, read_nav_obs)
     integer(c_int) function fwi_read_nav(path, max_records, shot_id, xs, bat, nrecords) bind(C, name="fwi_read_nav")
       import :: c_int, c_float, c_char
       character(kind=c_char) :: path(*)
       integer(c_int), value  :: max_records
       integer(c_int)         :: shot_id(*), nrecords
       real(c_float)          :: xs(*), bat(*)
     end function fwi_read_nav

     integer(c_int) function fwi_finalize() bind(C, name="fwi_finalize")
       import :: c_int
     end function fwi_finalize

     type(c_ptr) function fwi_last_error() bind(C, name="fwi_last_error")
       import :: c_ptr
     end function fwi_last_error
  end interface

contains

  !! Stop like the reference does on an error, with the library's message.
  subroutine fwi_check(rc)
    integer(c_int), intent(in) :: rc
    character(kind=c_char), pointer :: msg(:)
    integer :: n
    if (rc == FWI_OK) return
    call c_f_pointer(fwi_last_error(), msg, [512])
    n = 0
    do while (n < 512)
       if (msg(n + 1) == c_null_char) exit
       n = n + 1
    end do
    write(*,*) 'fwi_gb300 error ', rc, ': ', msg(1:n)
    stop
  end subroutine fwi_check

end module fwi_gpu_iface
