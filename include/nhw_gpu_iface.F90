! nhw_gpu_iface.F90 -- Fortran 2003 (ISO_C_BINDING) interface to libnhw_gpu,
! the C-ABI declared in include/nhwave_gb300.h.
!
! A patched `program NHWAVE` (src/nhwave.F:1-330) adds `use nhw_gpu_iface`,
! fills a `type(nhw_params)` from its input.txt values and calls the entry
! points below in place of the subroutines of its time loop
! (src/nhwave.F:119-258).  Every derived type is `bind(C)` with the members of
! the C struct of the same name, in the same order and of the same kinds, so
! that the two have the same layout; nhw_abi_sizes returns the library's
! sizeof of nhw_params and nhw_scalars for a start-up check.  The parameters
! below mirror the header's enums value for value.  tests/test_fortran_iface.py
! checks this file against the header: members, order, kinds, enum values and
! the list of entry points.
!
! Arrays cross as the reference's own ghosted, column-major module arrays,
! passed with c_loc: Eta(Mloc,Nloc), U(Mloc,Nloc,Kloc), Ex(Mloc1,Nloc,Kloc) ...
! (src/initialize.F:1423-1643).  The library never keeps a host pointer after
! a call returns.
module nhw_gpu_iface
  use iso_c_binding
  implicit none

  ! ------------------------------------------------------------ enum nhw_status
  integer(c_int), parameter :: NHW_OK = 0
  integer(c_int), parameter :: NHW_ERR_ARG = 1
  integer(c_int), parameter :: NHW_ERR_UNSUPPORTED = 2
  integer(c_int), parameter :: NHW_ERR_CUDA = 3
  integer(c_int), parameter :: NHW_ERR_NOMEM = 4
  integer(c_int), parameter :: NHW_ERR_DT_MIN = 5
  integer(c_int), parameter :: NHW_ERR_KRYLOV_NOCONV = 6
  integer(c_int), parameter :: NHW_ERR_NAN = 7
  integer(c_int), parameter :: NHW_ERR_TIMEOUT = 8
  integer(c_int), parameter :: NHW_ERR_STATE = 9
  integer(c_int), parameter :: NHW_ERR_CAPACITY = 10
  integer(c_int), parameter :: NHW_ERR_NOT_FOUND = 11

  ! --------------------------------------------------------- enum nhw_precision
  integer(c_int), parameter :: NHW_FP64 = 0
  integer(c_int), parameter :: NHW_FP32_IR = 1

  ! --------------------------------------------------------- enum nhw_wavemaker
  integer(c_int), parameter :: NHW_WM_NONE = 0
  integer(c_int), parameter :: NHW_WM_INT_LIN = 1
  integer(c_int), parameter :: NHW_WM_INT_SOL = 2
  integer(c_int), parameter :: NHW_WM_LEF_LIN = 3
  integer(c_int), parameter :: NHW_WM_LEF_SOL = 4
  integer(c_int), parameter :: NHW_WM_LEF_STK = 5
  integer(c_int), parameter :: NHW_WM_LEF_CON = 6
  integer(c_int), parameter :: NHW_WM_WAV_CUR = 7
  integer(c_int), parameter :: NHW_WM_FOCUSED = 8
  integer(c_int), parameter :: NHW_WM_LEF_TID = 9
  integer(c_int), parameter :: NHW_WM_RIG_LIN = 10
  integer(c_int), parameter :: NHW_WM_FLUX_LR = 11
  integer(c_int), parameter :: NHW_WM_LEF_JON = 12
  integer(c_int), parameter :: NHW_WM_LEF_TMA = 13
  integer(c_int), parameter :: NHW_WM_LEF_SPC = 14
  integer(c_int), parameter :: NHW_WM_INT_CON = 15
  integer(c_int), parameter :: NHW_WM_INT_JON = 16
  integer(c_int), parameter :: NHW_WM_INT_TMA = 17
  integer(c_int), parameter :: NHW_WM_INT_SPC = 18
  integer(c_int), parameter :: NHW_WM_INT_IRR = 19

  ! ------------------------------------------- enum nhw_slide, nhw_depth_type
  integer(c_int), parameter :: NHW_SLIDE_NONE = 0
  integer(c_int), parameter :: NHW_SLIDE_RIGID_3D = 1
  integer(c_int), parameter :: NHW_DEPTH_CELL_CENTER = 0
  integer(c_int), parameter :: NHW_DEPTH_CELL_GRID = 1

  ! ------------------------------------------------------------- enum nhw_field
  ! 2-D cell (Mloc,Nloc)
  integer(c_int), parameter :: NHW_F_D = 0
  integer(c_int), parameter :: NHW_F_D0 = 1
  integer(c_int), parameter :: NHW_F_ETA = 2
  integer(c_int), parameter :: NHW_F_ETA0 = 3
  integer(c_int), parameter :: NHW_F_HC = 4
  integer(c_int), parameter :: NHW_F_HC0 = 5
  integer(c_int), parameter :: NHW_F_DELXH = 6
  integer(c_int), parameter :: NHW_F_DELYH = 7
  integer(c_int), parameter :: NHW_F_DELXETA = 8
  integer(c_int), parameter :: NHW_F_DELYETA = 9
  integer(c_int), parameter :: NHW_F_DELTH = 10
  integer(c_int), parameter :: NHW_F_DELT2H = 11
  integer(c_int), parameter :: NHW_F_SOURCEX = 12
  integer(c_int), parameter :: NHW_F_SOURCEY = 13
  integer(c_int), parameter :: NHW_F_SOURCEC = 14
  integer(c_int), parameter :: NHW_F_SPONGE = 15
  integer(c_int), parameter :: NHW_F_R1 = 16
  ! 2-D x faces (Mloc1,Nloc)
  integer(c_int), parameter :: NHW_F_HFX = 17
  integer(c_int), parameter :: NHW_F_HFX0 = 18
  integer(c_int), parameter :: NHW_F_ETAXL = 19
  integer(c_int), parameter :: NHW_F_ETAXR = 20
  ! 2-D y faces (Mloc,Nloc1)
  integer(c_int), parameter :: NHW_F_HFY = 21
  integer(c_int), parameter :: NHW_F_HFY0 = 22
  integer(c_int), parameter :: NHW_F_ETAYL = 23
  integer(c_int), parameter :: NHW_F_ETAYR = 24
  ! 2-D integer (Mloc,Nloc)
  integer(c_int), parameter :: NHW_F_MASK = 25
  integer(c_int), parameter :: NHW_F_MASK_STRUCT = 26
  integer(c_int), parameter :: NHW_F_MASK9 = 27
  ! 3-D cell (Mloc,Nloc,Kloc)
  integer(c_int), parameter :: NHW_F_U = 28
  integer(c_int), parameter :: NHW_F_V = 29
  integer(c_int), parameter :: NHW_F_W = 30
  integer(c_int), parameter :: NHW_F_DU = 31
  integer(c_int), parameter :: NHW_F_DV = 32
  integer(c_int), parameter :: NHW_F_DW = 33
  integer(c_int), parameter :: NHW_F_DU0 = 34
  integer(c_int), parameter :: NHW_F_DV0 = 35
  integer(c_int), parameter :: NHW_F_DW0 = 36
  integer(c_int), parameter :: NHW_F_P = 37
  ! 3-D z faces (Mloc,Nloc,Kloc1)
  integer(c_int), parameter :: NHW_F_OMEGA = 38
  ! 3-D x faces (Mloc1,Nloc,Kloc)
  integer(c_int), parameter :: NHW_F_EX = 39
  integer(c_int), parameter :: NHW_F_FX = 40
  integer(c_int), parameter :: NHW_F_GX = 41
  integer(c_int), parameter :: NHW_F_HX = 42
  ! 3-D y faces (Mloc,Nloc1,Kloc)
  integer(c_int), parameter :: NHW_F_EY = 43
  integer(c_int), parameter :: NHW_F_FY = 44
  integer(c_int), parameter :: NHW_F_GY = 45
  integer(c_int), parameter :: NHW_F_HY = 46
  ! 3-D z faces (Mloc,Nloc,Kloc1)
  integer(c_int), parameter :: NHW_F_FZ = 47
  integer(c_int), parameter :: NHW_F_GZ = 48
  integer(c_int), parameter :: NHW_F_HZ = 49
  integer(c_int), parameter :: NHW_F_CMUVT = 50
  integer(c_int), parameter :: NHW_F_CMUHT = 51
  integer(c_int), parameter :: NHW_F_TKE = 52
  integer(c_int), parameter :: NHW_F_EPS = 53
  integer(c_int), parameter :: NHW_F_DTKE = 54
  integer(c_int), parameter :: NHW_F_DEPS = 55
  integer(c_int), parameter :: NHW_F_COUNT = 56

  ! ------------------------------------------------------------- nhw_params
  ! The input.txt keys the path reads (src/initialize.F:141-1321), in the C
  ! struct's order.  Fill every member: zero is the default of the multigrid
  ! settings and test hooks (precond ... test_barrier_extra).
  type, bind(C) :: nhw_params
     integer(c_int32_t) :: Mglob, Nglob, Kglob
     real(c_double)     :: dx, dy
     integer(c_int32_t) :: ivgrd
     real(c_double)     :: grd_r
     real(c_double)     :: dt_ini, dt_min, dt_max
     real(c_double)     :: total_time
     integer(c_int32_t) :: sim_steps
     real(c_double)     :: cfl
     integer(c_int32_t) :: froude_cap_on
     real(c_double)     :: froude_cap
     real(c_double)     :: min_dep
     integer(c_int32_t) :: non_hydro
     integer(c_int32_t) :: time_order
     integer(c_int32_t) :: hllc
     integer(c_int32_t) :: viscous_flow
     integer(c_int32_t) :: barotropic
     integer(c_int32_t) :: itmax
     real(c_double)     :: tol
     integer(c_int32_t) :: bc_x0, bc_xn, bc_y0, bc_yn
     integer(c_int32_t) :: bc_z0
     real(c_double)     :: visc
     real(c_double)     :: slat
     real(c_double)     :: wind_u, wind_v
     integer(c_int32_t) :: depth_type
     integer(c_int32_t) :: wavemaker
     real(c_double)     :: amp_wave, per_wave, dep_wave, theta_wave, cur_wave
     real(c_double)     :: xsource_west, xsource_east, ysource_suth, ysource_nrth
     integer(c_int32_t) :: sponge_on
     real(c_double)     :: sponge_west_width, sponge_east_width, sponge_south_width, sponge_north_width
     real(c_double)     :: tramp
     integer(c_int32_t) :: slide_type
     real(c_double)     :: slide_t, slide_l, slide_w, slide_angle, slope_angle, slide_x0, slide_y0
     real(c_double)     :: slide_ut, slide_a0
     integer(c_int32_t) :: precision
     integer(c_int32_t) :: device
     integer(c_int32_t) :: precond
     real(c_float)      :: mg_weight
     integer(c_int32_t) :: krylov_kernel
     integer(c_int32_t) :: mg_coarse_sweeps
     integer(c_int32_t) :: mg_cta_columns
     integer(c_int32_t) :: mg_aggregate
     integer(c_int32_t) :: test_barrier_extra
     integer(c_int32_t) :: ivturb, ihturb
     integer(c_int32_t) :: rng
     real(c_double)     :: cvs, chs
     real(c_double)     :: schmidt
     real(c_double)     :: viscous_number
     integer(c_int32_t) :: ibot
     real(c_double)     :: cd0, zob
     integer(c_int32_t) :: nwave, component_amp_type
     real(c_double)     :: k_center, f_center, x_breaking, t_breaking, slope_group, normalized_delta_f, depth_comp
     real(c_double)     :: sd_return
     real(c_double)     :: hm0, tp, freq_min, freq_max
     integer(c_int32_t) :: numfreq, wave_seed
     integer(c_int32_t) :: prod_type
  end type nhw_params

  ! ------------------------------------------------------------ nhw_scalars
  type, bind(C) :: nhw_scalars
     real(c_double)     :: time
     real(c_double)     :: dt
     real(c_double)     :: dt_old
     integer(c_int32_t) :: run_step
     integer(c_int32_t) :: last_krylov_iters
     integer(c_int64_t) :: total_krylov_iters
     integer(c_int64_t) :: poisson_solves
     real(c_double)     :: last_rel_residual
     integer(c_int32_t) :: last_refinements
     integer(c_int32_t) :: status
  end type nhw_scalars

  ! -------------------------------------------------------------- nhw_stats
  ! the figures statistics prints (src/nhwave.F:3118-3160)
  type, bind(C) :: nhw_stats
     real(c_double)     :: mass_volume, energy, max_eta, min_eta, max_u, max_v, max_w
  end type nhw_stats

  ! ------------------------------------------------------ ensembles (no counterpart)
  type, bind(C) :: nhw_ensemble_opts
     integer(c_int32_t) :: cells_per_block
     integer(c_int32_t) :: block_rows
     integer(c_int32_t) :: coarse_sweeps
     integer(c_int32_t) :: solver
     integer(c_int32_t) :: reserved(4)
  end type nhw_ensemble_opts

  type, bind(C) :: nhw_ensemble_info
     integer(c_int32_t) :: members
     integer(c_int32_t) :: solve_launches_per_stage
     integer(c_int32_t) :: blocks_per_launch
     integer(c_int32_t) :: max_resident_blocks
     integer(c_int64_t) :: kernels_per_step
     integer(c_int64_t) :: cells
     type(nhw_ensemble_opts) :: opts
     integer(c_int64_t) :: kernels_launched
  end type nhw_ensemble_info

  interface
     ! ---------------------------------------------------------- lifecycle
     integer(c_int) function nhw_create(params, h) bind(C, name="nhw_create")
       import :: c_int, c_ptr, nhw_params
       type(nhw_params), intent(in) :: params
       type(c_ptr), intent(out) :: h
     end function nhw_create
     integer(c_int) function nhw_destroy(h) bind(C, name="nhw_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function nhw_destroy
     integer(c_int) function nhw_device_bytes(params, bytes) bind(C, name="nhw_device_bytes")
       import :: c_int, c_int64_t, nhw_params
       type(nhw_params), intent(in) :: params
       integer(c_int64_t), intent(out) :: bytes
     end function nhw_device_bytes
     ! depth: Mglob x Nglob interior values (CELL_CENTER; (Mglob+1) x (Nglob+1)
     ! for CELL_GRID) in depth.txt's row order -- not the ghosted Hc; eta0 and
     ! uvw0 interior values as eta0.txt / uvw0.txt, or c_null_ptr for rest
     integer(c_int) function nhw_setup(h, depth, eta0, uvw0) bind(C, name="nhw_setup")
       import :: c_int, c_ptr
       type(c_ptr), value :: h, depth, eta0, uvw0
     end function nhw_setup
     integer(c_int) function nhw_get_field(h, field, host) bind(C, name="nhw_get_field")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: field
       type(c_ptr), value :: host
     end function nhw_get_field
     integer(c_int) function nhw_set_field(h, field, host) bind(C, name="nhw_set_field")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: field
       type(c_ptr), value :: host
     end function nhw_set_field
     integer(c_int) function nhw_field_shape(h, field, dims, elem_bytes) bind(C, name="nhw_field_shape")
       import :: c_int, c_int32_t, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: field
       integer(c_int32_t), intent(out) :: dims(3)
       integer(c_int32_t), intent(out) :: elem_bytes
     end function nhw_field_shape
     integer(c_int) function nhw_get_scalars(h, out) bind(C, name="nhw_get_scalars")
       import :: c_int, c_ptr, nhw_scalars
       type(c_ptr), value :: h
       type(nhw_scalars), intent(out) :: out
     end function nhw_get_scalars
     integer(c_int) function nhw_set_time(h, time, dt, run_step) bind(C, name="nhw_set_time")
       import :: c_int, c_ptr, c_double, c_int32_t
       type(c_ptr), value :: h
       real(c_double), value :: time, dt
       integer(c_int32_t), value :: run_step
     end function nhw_set_time
     integer(c_int) function nhw_set_wave_phases(h, n, phases) bind(C, name="nhw_set_wave_phases")
       import :: c_int, c_int32_t, c_double, c_ptr
       type(c_ptr), value :: h
       integer(c_int32_t), value :: n
       real(c_double), intent(in) :: phases(*)
     end function nhw_set_wave_phases
     ! Wave_Spc2d(NumDir, NumFreq) and Random_Phs(NumDir, NumFreq) as the
     ! reference holds them; phases may be c_null_ptr (seeded phases)
     integer(c_int) function nhw_set_wave_spectrum(h, numfreq, numdir, freq, dire, spc2d, phases) &
                                                   bind(C, name="nhw_set_wave_spectrum")
       import :: c_int, c_int32_t, c_double, c_ptr
       type(c_ptr), value :: h
       integer(c_int32_t), value :: numfreq, numdir
       real(c_double), intent(in) :: freq(*), dire(*), spc2d(*)
       type(c_ptr), value :: phases
     end function nhw_set_wave_spectrum

     ! ------------------------------------------ the reference's subroutines
     integer(c_int) function nhw_estimate_dt(h) bind(C, name="nhw_estimate_dt")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function nhw_estimate_dt
     integer(c_int) function nhw_update_bathymetry(h) bind(C, name="nhw_update_bathymetry")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function nhw_update_bathymetry
     integer(c_int) function nhw_update_wave_bc(h) bind(C, name="nhw_update_wave_bc")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function nhw_update_wave_bc
     integer(c_int) function nhw_update_mask(h) bind(C, name="nhw_update_mask")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function nhw_update_mask
     integer(c_int) function nhw_update_vars(h) bind(C, name="nhw_update_vars")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function nhw_update_vars
     integer(c_int) function nhw_source_terms(h) bind(C, name="nhw_source_terms")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function nhw_source_terms
     integer(c_int) function nhw_fluxes(h) bind(C, name="nhw_fluxes")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function nhw_fluxes
     integer(c_int) function nhw_eval_duvw(h, istep) bind(C, name="nhw_eval_duvw")
       import :: c_int, c_int32_t, c_ptr
       type(c_ptr), value :: h
       integer(c_int32_t), value :: istep
     end function nhw_eval_duvw
     integer(c_int) function nhw_sponge_damping(h) bind(C, name="nhw_sponge_damping")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function nhw_sponge_damping
     integer(c_int) function nhw_eval_turb(h, istep) bind(C, name="nhw_eval_turb")
       import :: c_int, c_int32_t, c_ptr
       type(c_ptr), value :: h
       integer(c_int32_t), value :: istep
     end function nhw_eval_turb

     ! ------------------------------------------------------ whole steps
     ! time, dt, run_step: pass variables, or c_null_ptr through a c_ptr
     ! variant of this interface to skip them
     integer(c_int) function nhw_step(h, time, dt, run_step) bind(C, name="nhw_step")
       import :: c_int, c_int32_t, c_double, c_ptr
       type(c_ptr), value :: h
       real(c_double), intent(out) :: time, dt
       integer(c_int32_t), intent(out) :: run_step
     end function nhw_step
     integer(c_int) function nhw_run(h, nsteps, steps_done) bind(C, name="nhw_run")
       import :: c_int, c_int32_t, c_ptr
       type(c_ptr), value :: h
       integer(c_int32_t), value :: nsteps
       integer(c_int32_t), intent(out) :: steps_done
     end function nhw_run

     ! -------------------------------------------------- checkpoint / resume
     integer(c_int) function nhw_checkpoint_bytes(h, bytes) bind(C, name="nhw_checkpoint_bytes")
       import :: c_int, c_int64_t, c_ptr
       type(c_ptr), value :: h
       integer(c_int64_t), intent(out) :: bytes
     end function nhw_checkpoint_bytes
     integer(c_int) function nhw_save_state(h, host, bytes) bind(C, name="nhw_save_state")
       import :: c_int, c_int64_t, c_ptr
       type(c_ptr), value :: h, host
       integer(c_int64_t), value :: bytes
     end function nhw_save_state
     integer(c_int) function nhw_load_state(h, host, bytes) bind(C, name="nhw_load_state")
       import :: c_int, c_int64_t, c_ptr
       type(c_ptr), value :: h, host
       integer(c_int64_t), value :: bytes
     end function nhw_load_state

     ! ------------------------------------------------------------ statistics
     integer(c_int) function nhw_mass(h, mass) bind(C, name="nhw_mass")
       import :: c_int, c_double, c_ptr
       type(c_ptr), value :: h
       real(c_double), intent(out) :: mass
     end function nhw_mass
     integer(c_int) function nhw_statistics(h, out) bind(C, name="nhw_statistics")
       import :: c_int, c_ptr, nhw_stats
       type(c_ptr), value :: h
       type(nhw_stats), intent(out) :: out
     end function nhw_statistics

     ! ------------------------------------------------------ timing and misc
     integer(c_int) function nhw_synchronize(h) bind(C, name="nhw_synchronize")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function nhw_synchronize
     integer(c_int) function nhw_run_timed(h, nsteps, device_ms) bind(C, name="nhw_run_timed")
       import :: c_int, c_int32_t, c_double, c_ptr
       type(c_ptr), value :: h
       integer(c_int32_t), value :: nsteps
       real(c_double), intent(out) :: device_ms
     end function nhw_run_timed
     integer(c_int) function nhw_profile(h, on) bind(C, name="nhw_profile")
       import :: c_int, c_int32_t, c_ptr
       type(c_ptr), value :: h
       integer(c_int32_t), value :: on
     end function nhw_profile
     integer(c_int) function nhw_profile_report(h, buf, buflen) bind(C, name="nhw_profile_report")
       import :: c_int, c_int32_t, c_char, c_ptr
       type(c_ptr), value :: h
       character(kind=c_char), intent(out) :: buf(*)
       integer(c_int32_t), value :: buflen
     end function nhw_profile_report
     integer(c_int) function nhw_time_smoother(h, reps, flush_bytes, us_per_launch) bind(C, name="nhw_time_smoother")
       import :: c_int, c_int32_t, c_int64_t, c_double, c_ptr
       type(c_ptr), value :: h
       integer(c_int32_t), value :: reps
       integer(c_int64_t), value :: flush_bytes
       real(c_double), intent(out) :: us_per_launch
     end function nhw_time_smoother
     integer(c_int) function nhw_abi_sizes(params_bytes, scalars_bytes) bind(C, name="nhw_abi_sizes")
       import :: c_int, c_int32_t
       integer(c_int32_t), intent(out) :: params_bytes, scalars_bytes
     end function nhw_abi_sizes
     ! both return a NUL-terminated C string owned by the library
     type(c_ptr) function nhw_status_string(status) bind(C, name="nhw_status_string")
       import :: c_int, c_ptr
       integer(c_int), value :: status
     end function nhw_status_string
     type(c_ptr) function nhw_last_error() bind(C, name="nhw_last_error")
       import :: c_ptr
     end function nhw_last_error

     ! ------------------------------------------- allocation-free variant
     ! device arrays of the caller (c_ptr to device memory); stream: a
     ! cudaStream_t, or c_null_ptr for the default stream
     integer(c_int) function nhw_estimate_dt_noalloc(U, V, W, D, dsig, Mglob, Nglob, Kglob, dx, dy, cfl, &
                                                     dt_old, dt_max, dt_out, stream) &
                                                     bind(C, name="nhw_estimate_dt_noalloc")
       import :: c_int, c_int32_t, c_double, c_ptr
       type(c_ptr), value :: U, V, W, D, dsig
       integer(c_int32_t), value :: Mglob, Nglob, Kglob
       real(c_double), value :: dx, dy, cfl, dt_old, dt_max
       type(c_ptr), value :: dt_out, stream
     end function nhw_estimate_dt_noalloc

     ! ---------------------------------------------------------------- ensembles
     integer(c_int) function nhw_ensemble_create(members, n, opts, out) bind(C, name="nhw_ensemble_create")
       import :: c_int, c_int32_t, c_ptr, nhw_ensemble_opts
       type(c_ptr), intent(in) :: members(*)
       integer(c_int32_t), value :: n
       type(nhw_ensemble_opts), intent(in) :: opts
       type(c_ptr), intent(out) :: out
     end function nhw_ensemble_create
     integer(c_int) function nhw_ensemble_step(e, nsteps) bind(C, name="nhw_ensemble_step")
       import :: c_int, c_int32_t, c_ptr
       type(c_ptr), value :: e
       integer(c_int32_t), value :: nsteps
     end function nhw_ensemble_step
     integer(c_int) function nhw_ensemble_run_timed(e, nsteps, device_ms) bind(C, name="nhw_ensemble_run_timed")
       import :: c_int, c_int32_t, c_double, c_ptr
       type(c_ptr), value :: e
       integer(c_int32_t), value :: nsteps
       real(c_double), intent(out) :: device_ms
     end function nhw_ensemble_run_timed
     integer(c_int) function nhw_ensemble_tune(e, steps_per_trial, chosen) bind(C, name="nhw_ensemble_tune")
       import :: c_int, c_int32_t, c_ptr, nhw_ensemble_opts
       type(c_ptr), value :: e
       integer(c_int32_t), value :: steps_per_trial
       type(nhw_ensemble_opts), intent(out) :: chosen
     end function nhw_ensemble_tune
     integer(c_int) function nhw_ensemble_get_info(e, out) bind(C, name="nhw_ensemble_get_info")
       import :: c_int, c_ptr, nhw_ensemble_info
       type(c_ptr), value :: e
       type(nhw_ensemble_info), intent(out) :: out
     end function nhw_ensemble_get_info
     integer(c_int) function nhw_ensemble_destroy(e) bind(C, name="nhw_ensemble_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: e
     end function nhw_ensemble_destroy
  end interface
end module nhw_gpu_iface
