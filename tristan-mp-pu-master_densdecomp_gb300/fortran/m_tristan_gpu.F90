!
! m_tristan_gpu -- ISO_C_BINDING shim between the TRISTAN-MP main loop and
! the GB300 C-ABI (include/tristan_gpu.h).
!
! The reference main loop (code/tristanmainloop.F90:107-344) calls
! argument-less module subroutines. This module exports the same names
! (bc_b1, bc_e1, bc_b2, bc_e2, advance_Bhalfstep, advance_Efield,
! move_particles, reset_currents, deposit_particles, exchange_current,
! apply_filter1_opt, add_current, reorder_particles and the shock setup's
! particle_bc_user, field_bc_user, inject_particles_user) and forwards them
! to libtristan_gpu.so, so the lap body compiles unchanged: the module that
! holds mainloop adds `use m_tristan_gpu` and renames the CPU versions away
! on its existing use lines (e.g. `use m_fields, cpu_add_current =>
! add_current`). The module-global arrays of m_fields and m_particles are
! registered once with tg_bind_fields / tg_bind_particles and synchronised
! only around host-side work: reorder_particles, the last hot call of a
! lap, brings the device state home before a lap whose Diagnostics writes
! output (every gpu_sync_every laps, set by tg_start). Compile with the
! reference's -DtwoD/-Dddk flags and link -ltristan_gpu. Not compiled in
! this repository (no Fortran compiler).
!
! The CPU subroutines this module replaces are renamed away on its own use
! lines, so the local procedures below can carry their names.
#ifdef twoD
module m_tristan_gpu
  use m_globaldata
  use m_system
  use m_aux
  use m_communications
  use m_fields, cpu_advance_Efield => advance_Efield, cpu_advance_Bhalfstep => advance_Bhalfstep, &
                cpu_add_current => add_current, cpu_reset_currents => reset_currents
  use m_particles, cpu_reorder_particles => reorder_particles
#else
module m_tristan_gpu_3d
  use m_globaldata_3d
  use m_system_3d
  use m_aux_3d
  use m_communications_3d
  use m_fields_3d, cpu_advance_Efield => advance_Efield, cpu_advance_Bhalfstep => advance_Bhalfstep, &
                   cpu_add_current => add_current, cpu_reset_currents => reset_currents
  use m_particles_3d, cpu_reorder_particles => reorder_particles
#endif
  use iso_c_binding
  implicit none
  private

  type, bind(C) :: tg_config
     integer(c_int32_t) :: dims, order, mx, my, mz, nghost, nghostz
     integer(c_int32_t) :: periodic(3), ntimes, quirks
     real(c_float) :: c, corr, qi, qe, qmi, qme
     integer(c_int32_t) :: external_fields
     real(c_float) :: ext(6)
     real(c_double) :: x1in, x2in, y1in, y2in, z1in, z2in
     integer(c_int64_t) :: mxcum, mycum, mzcum
     integer(c_int32_t) :: deposit_mode, fx_shift
     integer(c_int64_t) :: maxhlf
     integer(c_int32_t) :: sort_every, tile(3), device, diag_every
  end type tg_config

  type, bind(C) :: tg_shock
     integer(c_int32_t) :: wall
     real(c_double) :: walloc
     real(c_float) :: gammawall, betawall
     integer(c_int32_t) :: cond_i1, cond_i2, edge_i1, edge_i2
     real(c_float) :: edge(6)
     integer(c_int32_t) :: inject
     real(c_double) :: xinject2
     real(c_float) :: betainj
     real(c_double) :: xinj_max
     real(c_float) :: ppc0, gamma_drift, weight, y1, y2, delgam_i, delgam_e, pcosthmult
     integer(c_int32_t) :: sigma_nonzero
     real(c_double) :: dseed
     integer(c_int32_t) :: totalpartnum
  end type tg_shock

  ! FP64 diagnostics (tg_diag of tristan_gpu.h)
  type, bind(C) :: tg_diag
     real(c_double) :: gauss_residual, gauss_abs, rho_norm, e_field, e_mag, e_kin_ions, e_kin_lecs
     real(c_double) :: p_part(3), p_field(3), charge_total
  end type tg_diag

  interface
     integer(c_int) function tg_init(cfg, ctx) bind(C, name="tg_init")
       import :: tg_config, c_int, c_ptr
       type(tg_config), intent(in) :: cfg
       type(c_ptr), intent(out) :: ctx
     end function
     subroutine tg_finalize(ctx) bind(C, name="tg_finalize")
       import :: c_ptr
       type(c_ptr), value :: ctx
     end subroutine
     type(c_ptr) function tg_last_error(ctx) bind(C, name="tg_last_error")
       import :: c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function tg_bind_fields(ctx, ex, ey, ez, bx, by, bz, cx, cy, cz) bind(C, name="tg_bind_fields")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx, ex, ey, ez, bx, by, bz, cx, cy, cz
     end function
     integer(c_int) function tg_bind_particles(ctx, p, ions, lecs) bind(C, name="tg_bind_particles")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx, p, ions, lecs
     end function
     integer(c_int) function tg_sync_from_host(ctx, mask) bind(C, name="tg_sync_from_host")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: mask
     end function
     integer(c_int) function tg_sync_to_host(ctx, mask) bind(C, name="tg_sync_to_host")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: mask
     end function
     integer(c_int) function tg_bc_b1(ctx) bind(C, name="tg_bc_b1")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function tg_bc_e1(ctx) bind(C, name="tg_bc_e1")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function tg_advance_b_half(ctx) bind(C, name="tg_advance_b_half")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function tg_advance_e(ctx) bind(C, name="tg_advance_e")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function tg_move(ctx) bind(C, name="tg_move")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function tg_reset_currents(ctx) bind(C, name="tg_reset_currents")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function tg_deposit(ctx) bind(C, name="tg_deposit")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function tg_fold_currents(ctx) bind(C, name="tg_fold_currents")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function tg_filter(ctx) bind(C, name="tg_filter")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function tg_add_current(ctx) bind(C, name="tg_add_current")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function tg_reorder(ctx, lap, force) bind(C, name="tg_reorder")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: lap, force
     end function
     integer(c_int) function tg_step(ctx, nsteps) bind(C, name="tg_step")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: nsteps
     end function
     integer(c_int) function tg_step_host(ctx, nsteps) bind(C, name="tg_step_host")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: nsteps
     end function
     integer(c_int) function tg_pin_host(ctx) bind(C, name="tg_pin_host")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function tg_set_host_parts(ctx, parts) bind(C, name="tg_set_host_parts")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: parts
     end function
     ! collisionless-shock hooks (user_pu/user_shock_pu.F90)
     integer(c_int) function tg_shock_init(ctx, k) bind(C, name="tg_shock_init")
       import :: c_int, c_ptr, tg_shock
       type(c_ptr), value :: ctx
       type(tg_shock), intent(in) :: k
     end function
     integer(c_int) function tg_shock_get(ctx, k) bind(C, name="tg_shock_get")
       import :: c_int, c_ptr, tg_shock
       type(c_ptr), value :: ctx
       type(tg_shock), intent(out) :: k
     end function
     integer(c_int) function tg_inject_region(ctx, x1, x2, y1, y2, ppc, weight) bind(C, name="tg_inject_region")
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: ctx
       real(c_float), value :: x1, x2, y1, y2, ppc, weight
     end function
     integer(c_int) function tg_particle_bc(ctx) bind(C, name="tg_particle_bc")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function tg_field_bc(ctx) bind(C, name="tg_field_bc")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function tg_inject(ctx) bind(C, name="tg_inject")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     ! restart files and output moments
     integer(c_int) function tg_write_restart(ctx, ffld, fprt, meta) bind(C, name="tg_write_restart")
       import :: c_int, c_ptr, c_char, tg_restart_meta
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(in) :: ffld(*), fprt(*)
       type(tg_restart_meta), intent(in) :: meta
     end function
     integer(c_int) function tg_read_restart(ctx, ffld, fprt, meta) bind(C, name="tg_read_restart")
       import :: c_int, c_ptr, c_char, tg_restart_meta
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(in) :: ffld(*), fprt(*)
       type(tg_restart_meta), intent(out) :: meta
     end function
     integer(c_int) function tg_moments(ctx, kind, idx, idy, idz, num, den) bind(C, name="tg_moments")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: kind, idx, idy, idz
       type(c_ptr), value :: num, den
     end function
     integer(c_int) function tg_output_var(ctx, var, istep, idx, idy, idz, out) bind(C, name="tg_output_var")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: var, istep, idx, idy, idz
       type(c_ptr), value :: out
     end function
     integer(c_int) function tg_output_particles(ctx, species, stride, cap, vals, ids, count) &
         bind(C, name="tg_output_particles")
       import :: c_int, c_ptr, c_int32_t, c_int64_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: species, stride
       integer(c_int64_t), value :: cap
       type(c_ptr), value :: vals, ids
       integer(c_int64_t), intent(out) :: count
     end function
     integer(c_int) function tg_spectrum_x_bins(ctx, nbins) bind(C, name="tg_spectrum_x_bins")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), intent(out) :: nbins
     end function
     integer(c_int) function tg_spectrum_x(ctx, gambins, si, se, sir, ser, xgamma, xslice, grange) &
         bind(C, name="tg_spectrum_x")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: gambins
       type(c_ptr), value :: si, se, sir, ser, xgamma, xslice, grange
     end function
     integer(c_int) function tg_spectrum_dims(ctx, gambins, nxbins, nybins) bind(C, name="tg_spectrum_dims")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: gambins
       integer(c_int32_t), intent(out) :: nxbins, nybins
     end function
     integer(c_int) function tg_spectrum(ctx, gambins, si, se, xgamma, xslice, yslice, grange) &
         bind(C, name="tg_spectrum")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: gambins
       type(c_ptr), value :: si, se, xgamma, xslice, yslice, grange
     end function
     integer(c_int) function tg_output_dims(ctx, istep, dims) bind(C, name="tg_output_dims")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: istep
       integer(c_int32_t), intent(out) :: dims(3)
     end function
     integer(c_int) function tg_diag_fp64(ctx, out) bind(C, name="tg_diag_fp64")
       import :: c_int, c_ptr, tg_diag
       type(c_ptr), value :: ctx
       type(tg_diag), intent(out) :: out
     end function
     integer(c_int) function tg_get_counts(ctx, ions, lecs) bind(C, name="tg_get_counts")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: ctx
       integer(c_int64_t), intent(out) :: ions, lecs
     end function
     integer(c_int) function tg_synchronize(ctx) bind(C, name="tg_synchronize")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
  end interface

  type, bind(C) :: tg_restart_meta
     real(c_double) :: dseed
     integer(c_int32_t) :: lap
     real(c_double) :: xinject, xinject2, xinject3
     real(c_float) :: leftwall
     real(c_double) :: walloc
     integer(c_int32_t) :: totalpartnum, maxptl
     integer(c_int64_t) :: max_subrecord
  end type tg_restart_meta

  type(c_ptr), save :: ctx = c_null_ptr
  integer(c_int), parameter :: SYNC_E = 1, SYNC_B = 2, SYNC_CUR = 4, SYNC_PARTICLES = 8, SYNC_ALL = 15

  ! laps between downloads of the device state (0: never), so that the
  ! host arrays are current when Diagnostics writes output
  integer, save :: gpu_sync_every = 0

  public :: tg_start, tg_stop, tg_download, tg_upload, tg_pin, tg_parts, gpu_sync_every, &
            bc_b1, bc_e1, bc_b2, bc_e2, advance_Bhalfstep, advance_Efield, move_particles, &
            reset_currents, deposit_particles, exchange_current, apply_filter1_opt, &
            add_current, reorder_particles, gpu_step, gpu_step_host, &
            particle_bc_user, field_bc_user, inject_particles_user, &
            gpu_write_restart, gpu_read_restart, gpu_meanq, gpu_spectrum_bins, gpu_spectrum, gpu_output_var, &
            gpu_output_particles, tg_diag, gpu_diagnostics, gpu_counts, gpu_synchronize, gpu_output_dims, &
            gpu_spectrum2d_bins, gpu_spectrum2d

contains

  subroutine check(rc, what)
    integer(c_int), intent(in) :: rc
    character(len=*), intent(in) :: what
    character(kind=c_char), pointer :: msg(:)
    integer :: n
    if (rc == 0) return
    call c_f_pointer(tg_last_error(ctx), msg, [512])
    n = 0
    do while (n < 512)
       if (msg(n + 1) == c_null_char) exit
       n = n + 1
    enddo
    print *, rank, ": ", what, " failed: ", msg(1:n)
    stop
  end subroutine check

  ! after read_input_* and allocate_*: the device mirror of one rank's domain
  subroutine tg_start(deposit_mode, sort_every, sync_every)
    integer, intent(in) :: deposit_mode, sort_every, sync_every
    type(tg_config) :: cfg
    cfg%dims = merge(2, 3, mz == 1)
#ifdef dd1
    cfg%order = 1
#endif
#ifdef dd2
    cfg%order = 2
#endif
#ifdef dd3
    cfg%order = 3
#endif
    cfg%mx = mx; cfg%my = my; cfg%mz = mz
    cfg%nghost = nghost; cfg%nghostz = nghostz
    cfg%periodic = [periodicx, periodicy, periodicz]
    cfg%ntimes = ntimes; cfg%quirks = 0
    cfg%c = c; cfg%corr = corr
    cfg%qi = qi; cfg%qe = qe; cfg%qmi = qmi; cfg%qme = qme
    cfg%external_fields = merge(1, 0, external_fields)
    cfg%ext = 0.
    cfg%x1in = x1in; cfg%x2in = x2in; cfg%y1in = y1in; cfg%y2in = y2in; cfg%z1in = z1in; cfg%z2in = z2in
    cfg%mxcum = mxcum; cfg%mycum = mycum; cfg%mzcum = mzcum
    cfg%deposit_mode = deposit_mode
    cfg%fx_shift = 30 - ceiling(log(max(abs(qi), abs(qe))) / log(2.))
    cfg%maxhlf = maxhlf
    cfg%sort_every = sort_every
    cfg%tile = 0; cfg%device = 0; cfg%diag_every = 0
    call check(tg_init(cfg, ctx), "tg_init")
    call check(tg_bind_fields(ctx, c_loc(ex), c_loc(ey), c_loc(ez), c_loc(bx), c_loc(by), c_loc(bz), &
               c_loc(curx), c_loc(cury), c_loc(curz)), "tg_bind_fields")
    call check(tg_bind_particles(ctx, c_loc(p), c_loc(ions), c_loc(lecs)), "tg_bind_particles")
    call check(tg_sync_from_host(ctx, SYNC_ALL), "tg_sync_from_host")
    gpu_sync_every = sync_every
  end subroutine tg_start

  subroutine tg_stop()
    call tg_finalize(ctx)
    ctx = c_null_ptr
  end subroutine tg_stop

  ! page-lock ex..curz and p (asynchronous DMA for gpu_step_host and the syncs)
  subroutine tg_pin()
    call check(tg_pin_host(ctx), "tg_pin_host")
  end subroutine tg_pin

  ! parts per species of gpu_step_host's transfers (0: by size)
  subroutine tg_parts(parts)
    integer, intent(in) :: parts
    call check(tg_set_host_parts(ctx, int(parts, c_int32_t)), "tg_set_host_parts")
  end subroutine tg_parts

  ! before Diagnostics / output / restart / host-side user hooks
  subroutine tg_download()
    call check(tg_sync_to_host(ctx, SYNC_ALL), "tg_sync_to_host")
  end subroutine tg_download

  ! after host-side injection or field_bc_user edits
  subroutine tg_upload()
    call check(tg_sync_from_host(ctx, SYNC_ALL), "tg_sync_from_host")
  end subroutine tg_upload

  ! the lap body's hot calls (code/tristanmainloop.F90:117-303)
  subroutine bc_b1()
    call check(tg_bc_b1(ctx), "bc_b1")
  end subroutine
  subroutine bc_e1()
    call check(tg_bc_e1(ctx), "bc_e1")
  end subroutine
  ! without radiation boundaries bc_b2 / bc_e2 are the periodic copies
  subroutine bc_b2()
    call check(tg_bc_b1(ctx), "bc_b2")
  end subroutine
  subroutine bc_e2()
    call check(tg_bc_e1(ctx), "bc_e2")
  end subroutine
  subroutine advance_Bhalfstep()
    call check(tg_advance_b_half(ctx), "advance_Bhalfstep")
  end subroutine
  subroutine advance_Efield()
    call check(tg_advance_e(ctx), "advance_Efield")
  end subroutine
  subroutine move_particles()
    call check(tg_move(ctx), "move_particles")
  end subroutine
  subroutine reset_currents()
    call check(tg_reset_currents(ctx), "reset_currents")
  end subroutine
  subroutine deposit_particles()
    call check(tg_deposit(ctx), "deposit_particles")
  end subroutine
  subroutine exchange_current()
    call check(tg_fold_currents(ctx), "exchange_current")
  end subroutine
  subroutine apply_filter1_opt()
    call check(tg_filter(ctx), "apply_filter1_opt")
  end subroutine
  subroutine add_current()
    call check(tg_add_current(ctx), "add_current")
  end subroutine
  ! the last hot call of a lap: the reorder on the reference's cadence, then
  ! the device state home when the next lap's Diagnostics writes output
  subroutine reorder_particles()
    call check(tg_reorder(ctx, int(lap, c_int32_t), 0_c_int32_t), "reorder_particles")
    if (gpu_sync_every > 0) then
       if (modulo(lap + 1, gpu_sync_every) == 0) call tg_download()
    endif
  end subroutine

  ! the shock's user hooks on the device (after tg_shock_init)
  subroutine particle_bc_user()
    call check(tg_particle_bc(ctx), "particle_bc_user")
  end subroutine
  subroutine field_bc_user()
    call check(tg_field_bc(ctx), "field_bc_user")
  end subroutine
  subroutine inject_particles_user()
    call check(tg_inject(ctx), "inject_particles_user")
  end subroutine

  ! write_restart / restart with the device state (frestartfld, frestartprt)
  subroutine gpu_write_restart(ffld, fprt)
    character(len=*), intent(in) :: ffld, fprt
    type(tg_restart_meta) :: m
    m%dseed = dseed; m%lap = lap; m%xinject = xinject; m%xinject2 = xinject2; m%xinject3 = xinject3
    m%leftwall = leftwall; m%walloc = walloc; m%totalpartnum = totalpartnum; m%maxptl = maxptl
    m%max_subrecord = 0
    call check(tg_write_restart(ctx, trim(ffld)//c_null_char, trim(fprt)//c_null_char, m), "write_restart")
  end subroutine
  subroutine gpu_read_restart(ffld, fprt)
    character(len=*), intent(in) :: ffld, fprt
    type(tg_restart_meta) :: m
    call check(tg_read_restart(ctx, trim(ffld)//c_null_char, trim(fprt)//c_null_char, m), "restart")
    dseed = m%dseed; lapst = m%lap + 1; xinject = m%xinject; xinject2 = m%xinject2; xinject3 = m%xinject3
    leftwall = m%leftwall; walloc = m%walloc; totalpartnum = m%totalpartnum
  end subroutine

  ! meanq_fld_cur on the device: kind 0..15 in the order of tg_moments
  subroutine gpu_meanq(kind, num, den)
    integer, intent(in) :: kind
    real, target, intent(out) :: num(:,:,:), den(:,:,:)
    call check(tg_moments(ctx, int(kind, c_int32_t), 2_c_int32_t, 2_c_int32_t, merge(0_c_int32_t, 2_c_int32_t, mz == 1), &
               c_loc(num), c_loc(den)), "meanq_fld_cur")
  end subroutine

  ! one .tot. variable of output_tot sampled on the device into its
  ! temporary1(mx1,my1,mz1) array (var: 0-5 ex..bz, 6-8 jx..jz, 16 + the
  ! meanq_fld_cur kind of tg_moments); the HDF5 write stays the reference's
  subroutine gpu_output_var(var, istep, out)
    integer, intent(in) :: var, istep
    real, target, intent(out) :: out(:,:,:)
    call check(tg_output_var(ctx, int(var, c_int32_t), int(istep, c_int32_t), 2_c_int32_t, 2_c_int32_t, &
               merge(0_c_int32_t, 2_c_int32_t, mz == 1), c_loc(out)), "output_tot")
  end subroutine

  ! output_tot's particle sample of one species (0 ions, 1 electrons): the
  ! particles with modulo(ind/2, stride) = 0; vals(:, 1:8) = x+mxcum,
  ! y+mycum, z+mzcum, u, v, w, ch, gamma and ids(:, 1:2) = ind, proc for
  ! the first count rows (count > size(vals, 1): only count is set)
  subroutine gpu_output_particles(species, stride, vals, ids, count)
    integer, intent(in) :: species, stride
    real, target, intent(out) :: vals(:,:)
    integer, target, intent(out) :: ids(:,:)
    integer(c_int64_t), intent(out) :: count
    call check(tg_output_particles(ctx, int(species, c_int32_t), int(stride, c_int32_t), &
               int(size(vals, 1), c_int64_t), c_loc(vals), c_loc(ids), count), "output_tot particles")
  end subroutine

  ! save_spectrum's arrays from the device (code/output.F90:380-785): nbins
  ! x slices, specp / spece and the flow-frame specprest / specerest
  ! (nbins, gambins), each divided by gamma - 1, xgamma, xslice, gmin, gmax;
  ! the HDF5 write stays the reference's
  integer function gpu_spectrum_bins()
    integer(c_int32_t) :: nb
    call check(tg_spectrum_x_bins(ctx, nb), "tg_spectrum_x_bins")
    gpu_spectrum_bins = nb
  end function

  subroutine gpu_spectrum(gambins, specp, spece, specprest, specerest, xgamma, xslice, gmin, gmax)
    integer, intent(in) :: gambins
    real, target, intent(out) :: specp(:,:), spece(:,:), specprest(:,:), specerest(:,:), xgamma(:), xslice(:)
    real, intent(out) :: gmin, gmax
    real, target :: gr(2)
    call check(tg_spectrum_x(ctx, int(gambins, c_int32_t), c_loc(specp), c_loc(spece), c_loc(specprest), &
               c_loc(specerest), c_loc(xgamma), c_loc(xslice), c_loc(gr)), "save_spectrum")
    gmin = gr(1)
    gmax = gr(2)
  end subroutine

  ! save_spectrum_2d (code/output.F90:794-1249): the slice counts for
  ! gambins bins, then the flow-frame spectra of both species,
  ! spec(nxbins, nybins, gambins), with the gamma and slice axes
  subroutine gpu_spectrum2d_bins(gambins, nxbins, nybins)
    integer, intent(in) :: gambins
    integer, intent(out) :: nxbins, nybins
    integer(c_int32_t) :: nx, ny
    call check(tg_spectrum_dims(ctx, int(gambins, c_int32_t), nx, ny), "save_spectrum_2d")
    nxbins = int(nx)
    nybins = int(ny)
  end subroutine

  subroutine gpu_spectrum2d(gambins, specp, spece, xgamma, xslice, yslice, gmin, gmax)
    integer, intent(in) :: gambins
    real, target, intent(out) :: specp(:,:,:), spece(:,:,:), xgamma(:), xslice(:), yslice(:)
    real, intent(out) :: gmin, gmax
    real, target :: gr(2)
    call check(tg_spectrum(ctx, int(gambins, c_int32_t), c_loc(specp), c_loc(spece), c_loc(xgamma), &
               c_loc(xslice), c_loc(yslice), c_loc(gr)), "save_spectrum_2d")
    gmin = gr(1)
    gmax = gr(2)
  end subroutine

  ! output_tot's sampled grid (mx1, my1, mz1) for the stride istep
  subroutine gpu_output_dims(istep, dims)
    integer, intent(in) :: istep
    integer, intent(out) :: dims(3)
    integer(c_int32_t) :: d(3)
    call check(tg_output_dims(ctx, int(istep, c_int32_t), d), "output_tot")
    dims = int(d)
  end subroutine

  ! FP64 Gauss residual, field and kinetic energies, momenta of the state
  subroutine gpu_diagnostics(d)
    type(tg_diag), intent(out) :: d
    call check(tg_diag_fp64(ctx, d), "tg_diag_fp64")
  end subroutine

  ! the particle counts on the device
  subroutine gpu_counts(nions, nlecs)
    integer, intent(out) :: nions, nlecs
    integer(c_int64_t) :: a, b
    call check(tg_get_counts(ctx, a, b), "tg_get_counts")
    nions = int(a)
    nlecs = int(b)
  end subroutine

  ! wait for the device (reports a device fault as an error)
  subroutine gpu_synchronize()
    call check(tg_synchronize(ctx), "tg_synchronize")
  end subroutine

  ! the whole periodic lap fused on the device (replaces lines 115-303)
  subroutine gpu_step(nsteps)
    integer, intent(in) :: nsteps
    call check(tg_step(ctx, int(nsteps, c_int32_t)), "tg_step")
  end subroutine

  ! one main-loop pass with the module's own arrays as the state: ex..bz and
  ! the particle records go to the device, the lap runs, ex..curz, the
  ! records and ions / lecs come back (tg_step_host)
  subroutine gpu_step_host(nsteps)
    integer, intent(in) :: nsteps
    call check(tg_step_host(ctx, int(nsteps, c_int32_t)), "tg_step_host")
  end subroutine

#ifdef twoD
end module m_tristan_gpu
#else
end module m_tristan_gpu_3d
#endif
