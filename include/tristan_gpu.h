/*
 * tristan_gpu.h -- C-ABI of the GB300 (sm_103a) TRISTAN-MP per-step hot path.
 *
 * Drop-in boundary for the argument-less module subroutines that the
 * reference main loop calls each lap (mrowan137/tristan-mp-pu-master_densdecomp,
 * code/tristanmainloop.F90:107-344). A Fortran ISO_C_BINDING shim keeps the
 * reference's subroutine names and forwards to these entry points, so the
 * main loop, the `input` file and the user_* hooks stay unchanged.
 *
 * Conventions
 *  - Plain C types only; every call returns an int status (TG_OK = 0).
 *  - Host arrays are the reference's own: fields are Fortran-ordered
 *    (mx,my,mz) float arrays, particles the 40-byte `type particle` records
 *    (code/particles.F90:51-55) with ions at p(1:ions) and electrons at
 *    p(maxhlf+1:maxhlf+lecs).
 *  - One context per process, one CUDA stream; calls are stream-ordered and
 *    return without a host synchronisation except tg_sync_to_host,
 *    tg_synchronize, tg_diag_fp64 and tg_get_counts. A context is not
 *    thread-safe.
 *  - Device-side faults (a particle outside the grid, a NaN, a capacity
 *    overflow) are recorded in a device status word, never trapped; the next
 *    synchronising call returns the matching TG_ERR_* code and
 *    tg_last_error() describes it.
 */
#ifndef TRISTAN_GPU_H
#define TRISTAN_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TG_OK 0
#define TG_ERR_ARG 1      /* bad argument or configuration */
#define TG_ERR_CUDA 2     /* a CUDA runtime call failed */
#define TG_ERR_OVERFLOW 3 /* particle count above maxhlf (check_overflow,
                             code/particles.F90:362-370) */
#define TG_ERR_BOUNDS 4   /* a particle or deposit left the local grid */
#define TG_ERR_NAN 5      /* non-finite particle coordinate */
#define TG_ERR_STATE 6    /* call made in the wrong order (e.g. unbound) */

/* quirk switches, tg_config.quirks */
#define TG_QUIRK_Q5_LHS 1 /* y-fold of cury reads curx(:,my) for row nghost,
                             the left-hand-side reading of the shape-mismatched
                             copy at code/fieldboundaries.F90:1938 */

/* deposit modes, tg_config.deposit_mode */
/* Both modes compute every Esirkepov contribution in FP32 in the
   reference's order and sum a tile's contributions exactly in a fixed-point
   shared-memory window; they differ in how the tile sums reach the global
   currents. */
#define TG_DEPOSIT_FP32 0  /* each tile sum rounded once to FP32 and added
                              with FP32 global atomics (the summation order
                              across tiles varies run to run) */
#define TG_DEPOSIT_FIXED 1 /* tile sums added to int64 fixed-point global
                              accumulators, converted to FP32 once per lap:
                              bit-reproducible currents */

/* sync masks */
#define TG_SYNC_E 1u
#define TG_SYNC_B 2u
#define TG_SYNC_CUR 4u
#define TG_SYNC_PARTICLES 8u
#define TG_SYNC_ALL 15u

/* Run configuration: the values the reference reads from `input` and
   derives at start-up (read_input_grid code/fields.F90:154-192,
   allocate_fields :207-360, read_input_particles code/particles.F90:189-233,
   allocate_particles :286-341, read_input_algorithm
   code/initialize.F90:293-305). */
typedef struct {
    int32_t dims;        /* 2 (twoD build) or 3 */
    int32_t order;       /* shape order 1, 2, 3 (-Ddd1/-Ddd2/-Ddd3) */
    int32_t mx, my, mz;  /* local extents including ghosts; 2D: mz = 1 */
    int32_t nghost, nghostz;
    int32_t periodic[3];
    int32_t ntimes;      /* filter passes */
    int32_t quirks;
    float c, corr;
    float qi, qe, qmi, qme;
    int32_t external_fields; /* add ext[] in the mover (get_external_fields) */
    float ext[6];            /* ex, ey, ez, bx, by, bz */
    double x1in, x2in, y1in, y2in, z1in, z2in; /* keep-window on open axes */
    int64_t mxcum, mycum, mzcum;               /* slab offsets (0 for one domain) */
    int32_t deposit_mode;
    int32_t fx_shift;    /* fixed-point scale 2^fx_shift */
    int64_t maxhlf;      /* particle capacity per species */
    int32_t sort_every;  /* re-sort particles into tiles every k laps (>= 1) */
    int32_t tile[3];     /* tile edge in cells (0 = automatic); a tile's shared
                            memory (its deposit window and field copy) must fit
                            in 227 KB, else tg_init fails with TG_ERR_ARG */
    int32_t device;      /* CUDA device ordinal */
    int32_t diag_every;  /* 1: FP64 diagnostics inside every tg_step lap */
} tg_config;

typedef struct tg_ctx tg_ctx;

/* FP64 diagnostics (reduced on the device) */
typedef struct {
    double gauss_residual; /* ||div E - F^ntimes(rho)|| / ||F^ntimes(rho)|| */
    double gauss_abs;
    double rho_norm;
    double e_field, e_mag;      /* sum E^2/2, sum B^2/2 over the interior */
    double e_kin_ions, e_kin_lecs;
    double p_part[3];           /* sum m u */
    double p_field[3];          /* sum E x B */
    double charge_total;
} tg_diag;

/* Allocate the device domain: replaces allocate_fields
   (code/fields.F90:207-360) and allocate_particles
   (code/particles.F90:286-341). TG_ERR_ARG for a domain with fewer than
   nghost/2 + 1 interior cells along an axis (mx - nghost, my - nghost, and
   in 3D mz - nghostz): 3 at order 1, 4 at orders 2 and 3. */
int tg_init(const tg_config *cfg, tg_ctx **out);
/* Release everything (finalize, code/tristan.F90:38). */
void tg_finalize(tg_ctx *ctx);
/* Text of the last error on this context (or of the last failed tg_init
   when ctx is NULL). */
const char *tg_last_error(tg_ctx *ctx);

/* Register the host Fortran arrays (module m_fields, code/fields.F90:81-86).
   Any pointer may be NULL. */
int tg_bind_fields(tg_ctx *ctx, float *ex, float *ey, float *ez, float *bx, float *by,
                   float *bz, float *curx, float *cury, float *curz);
/* Register the host particle array p (2*maxhlf records) and the species
   counters ions/lecs (module m_particles, code/particles.F90:80-100). */
int tg_bind_particles(tg_ctx *ctx, void *p, int32_t *ions, int32_t *lecs);
/* Host -> device for the masked groups (after host-side injection or
   field_bc_user edits). Particles are sorted into tiles on upload. */
int tg_sync_from_host(tg_ctx *ctx, unsigned mask);
/* Device -> host for the masked groups (before Diagnostics, output,
   restart, host-side user hooks). Synchronises. */
int tg_sync_to_host(tg_ctx *ctx, unsigned mask);

/* bc_b1 / bc_e1: periodic ghost-layer copies (code/fieldboundaries.F90:
   181-263, :306-392). bc_b2 / bc_e2 reduce to these without radiation
   boundaries. */
int tg_bc_b1(tg_ctx *ctx);
int tg_bc_e1(tg_ctx *ctx);
/* advance_Bhalfstep (code/fields.F90:1407-1415 -> advance_b_halfstep
   :586-728): B += corr*c/2 * (-curl E) on the update range. */
int tg_advance_b_half(tg_ctx *ctx);
/* advance_Efield (code/fields.F90:1425-1433 -> advance_e_fullstep
   :739-870): E += corr*c * curl B. */
int tg_advance_e(tg_ctx *ctx);
/* move_particles (code/particles_movedeposit.F90:63-88): Boris push with
   the shape-consistent gather, both species. */
int tg_move(tg_ctx *ctx);
/* reset_currents (code/fields.F90:499-506). */
int tg_reset_currents(tg_ctx *ctx);
/* deposit_particles (code/particles_movedeposit.F90:1281-2051): Esirkepov
   current of every particle from its reconstructed previous position, then
   the periodic wrap / open-boundary discard and compaction. */
int tg_deposit(tg_ctx *ctx);
/* exchange_current (code/fieldboundaries.F90:1768-2189): fold the current
   ghost layers into the interior. */
int tg_fold_currents(tg_ctx *ctx);
/* apply_filter1_opt (code/filter.F90:8-221): ntimes binomial passes. */
int tg_filter(tg_ctx *ctx);
/* add_current (code/fields.F90:1372-1395): E += cur over the array. */
int tg_add_current(tg_ctx *ctx);
/* reorder_particles (code/particles.F90:394-403): stable counting sort of
   each species by cell, on the reference's cadence (every 10 laps, not the
   lap after the previous reorder). force != 0 sorts now. */
int tg_reorder(tg_ctx *ctx, int32_t lap, int32_t force);

/* One or more complete laps of the main loop
   (code/tristanmainloop.F90:115-303 without output and domain moves; with
   the shock hooks set, also particle_bc_user, field_bc_user and
   inject_particles_user at their places), fused and replayed from a
   captured CUDA graph. */
int tg_step(tg_ctx *ctx, int32_t nsteps);
/* nsteps passes of the main loop (code/tristanmainloop.F90:115-303) with the
   bound host arrays as the state of record, as when the reference's loop
   keeps its own arrays between laps: per lap E, B and the particle records
   (tg_bind_fields / tg_bind_particles) go to the device, the lap runs, and
   E, B, the currents, the records and the counts come back before the call
   returns. With page-locked host records on an all-periodic domain each
   species travels in parts (tg_set_host_parts): a part is sorted and
   pushed as soon as its records are in, and sent home while later parts
   are still arriving; otherwise it is tg_sync_from_host + tg_step(1) +
   tg_sync_to_host per lap. The records come back in the device's order
   (each part grouped by tile), not in the order they went up. */
int tg_step_host(tg_ctx *ctx, int32_t nsteps);
/* Parts per species for the overlapped tg_step_host, 1..TG_HOST_PARTS_MAX;
   0 (the default) picks by size: about 512 records of the larger species
   per tile and part, at most TG_HOST_PARTS_MAX. No counterpart in the
   reference. */
#define TG_HOST_PARTS_MAX 8
int tg_set_host_parts(tg_ctx *ctx, int32_t parts);
/* Page-lock the bound host arrays (the nine fields and 2 * maxhlf particle
   records) so host transfers run as asynchronous DMA; arrays already
   page-locked are left as they are. Before locking a range it asks the
   kernel for transparent huge pages behind it (madvise MADV_HUGEPAGE, and
   MADV_COLLAPSE where the kernel has it): locked base pages sustain fewer
   bytes per second over the host link with both directions in flight.
   Undone by tg_finalize (the advice stays). No counterpart in the
   reference. */
int tg_pin_host(tg_ctx *ctx);
/* tg_step bracketed by CUDA events on the context's stream; *ms receives
   the device time of the nsteps laps. Synchronises. */
int tg_step_timed(tg_ctx *ctx, int32_t nsteps, float *ms);
/* Autotuner (no counterpart in the reference, which has no tunables of
   this kind): times `laps` sort cycles of the fused lap for each candidate
   tile shape (particles per tile follow from it) and re-sort cadence on the
   caller's particles (p, ions, lecs as for tg_bind_particles, not
   modified), and writes the fastest tile[] and sort_every into *cfg. If
   table is non-NULL it receives up to table_len rows of (tx, ty, tz,
   sort_every, ms per lap; -1 when the candidate failed). Returns the
   number of rows, or a negative TG_ERR code when no candidate ran. */
int tg_autotune(tg_config *cfg, void *p, int32_t ions, int32_t lecs, int32_t laps, float *best_ms,
                float *table, int32_t table_len);

/* FP64 Gauss-law residual, energies and momenta of the device state.
   Synchronises. */
int tg_diag_fp64(tg_ctx *ctx, tg_diag *out);

/* Per-lap FP64 diagnostics recorded by tg_step when diag_every = 1: the
   last n records, oldest first, 16 doubles each in the order
   |div E - F(rho)|^2, |F(rho)|^2, total charge, E energy, B energy, ion and
   electron kinetic energy, particle momentum x/y/z, field momentum x/y/z,
   2 unused. Returns the number of records written. Synchronises. */
int tg_diag_history(tg_ctx *ctx, double *out, int32_t n);

/* Phase timing with CUDA events recorded on the context's stream inside
   tg_step (and inside its captured graph). on != 0 enables it (graphs are
   re-captured; the last lap of each tg_step then runs outside the graph,
   since events recorded by graph nodes cannot be read back). tg_phase_times
   returns, for the last lap of the last tg_step, the milliseconds of up to
   TG_NPHASES phases, grouped as the reference's per-lap timers
   (print_timers, code/communications.F90:242-326): [0] field update before
   the push and [2] after it (with [5], "Field slv"), [1] the fused push +
   deposit kernel ("Mover" + "Deposit"), [3] current fold ("Currnt exch"),
   [4] filter passes ("Filter"), [5] add_current, with the shock's field
   reset and injection when set ("Inject"), [6] tile sort ("Reorder"),
   [7] FP64 diagnostics (no counterpart). A phase not run returns 0. */
#define TG_NPHASES 8
int tg_enable_timing(tg_ctx *ctx, int32_t on);
int tg_phase_times(tg_ctx *ctx, float *ms, int32_t nphases);

/* Binomial current filter (the ntimes passes of apply_filter1_opt) on three
   caller-owned device arrays of the Fortran (mx,my,mz) layout, allocating
   nothing. No counterpart in the reference: it exists for callers that
   cannot allocate device memory (a host whose own pool owns the whole
   device, or work issued where a cudaMalloc could synchronise the device).
   Its scratch is a fixed device array of 3 x TG_NOALLOC_MAX_CELLS floats
   held by every GPU that loads the library; larger grids are rejected with
   TG_ERR_ARG. The first call on a device looks the array up (make it before
   any stream capture) and keeps its address for the life of the process:
   after a cudaDeviceReset of that device the kept address is stale, so do
   not call this entry point on a device that was reset. Calls that overlap
   on the GPU race on the shared scratch. `stream` is a cudaStream_t (NULL:
   the default stream). Errors are described by tg_last_error(NULL), whose
   text is kept per host thread. */
#define TG_NOALLOC_MAX_CELLS 1310720
int tg_filter_noalloc(int32_t dims, int32_t mx, int32_t my, int32_t mz, int32_t nghost, int32_t nghostz,
                      const int32_t *periodic, int32_t ntimes, float *curx, float *cury, float *curz,
                      void *stream);

/* Wait for all work on the context's stream; returns any device status. */
int tg_synchronize(tg_ctx *ctx);
/* Current particle counts per species (synchronises). */
int tg_get_counts(tg_ctx *ctx, int64_t *ions, int64_t *lecs);
/* Raw device pointers of the field arrays in the order ex, ey, ez, bx, by,
   bz, curx, cury, curz (for zero-copy coupling; valid until tg_finalize). */
int tg_device_fields(tg_ctx *ctx, float **ptrs9);
/* The CUDA stream the context launches on (as a cudaStream_t). */
void *tg_stream(tg_ctx *ctx);
/* Number of kernels launched by the last tg_step lap (for accounting). */
int32_t tg_kernels_per_step(tg_ctx *ctx);

/* ---------------------------------------------------------------------
   Collisionless-shock hooks (2D): the user_* routines of
   user_pu/user_shock_pu.F90 run as device kernels, so the main loop stays
   on the GPU. Replaces particle_bc_user (:514-611, the left reflecting
   wall with its zigzag partial deposits, code/particles.F90:550-669),
   field_bc_user (:460-488, conductor behind the wall and upstream fields
   at the right edge) and inject_particles_user (:364-395, the moving
   injector with rightclean = 0 and rightwall = 0) with
   inject_from_wall / inject_plasma_region (code/particles.F90:2439-2938)
   and the Park-Miller generator and Maxwell-Juttner loader
   (code/aux.F90:82-134, code/particles.F90:2126-2273). Random draws follow
   the reference's sequence: pair k of an injection starts 13k draws (plus
   any gamma redraws before it) after the call's first draw, so ind, counts
   and positions are the reference's. With the hooks set, tg_step runs them
   at their places in the lap and sorts every lap (sort_every must be 1).
   --------------------------------------------------------------------- */
typedef struct {
    int32_t wall;                 /* left wall on */
    double walloc;                /* wall position, global x */
    float gammawall, betawall;    /* wallgam and its beta */
    int32_t cond_i1, cond_i2;     /* ey = ez = 0 on local i in [cond_i1, cond_i2] (if different) */
    int32_t edge_i1, edge_i2;     /* upstream fields on i in [edge_i1, edge_i2] (if different) */
    float edge[6];                /* ex ey ez bx by bz written there */
    int32_t inject;               /* moving injector on */
    double xinject2;              /* injector position, global x */
    float betainj;                /* injector speed / c */
    double xinj_max;              /* mx0 - 15: the injector stops there */
    float ppc0, gamma_drift, weight;
    float y1, y2;                 /* injection band, global y */
    float delgam_i, delgam_e;     /* kT / m c^2 of ions and electrons */
    float pcosthmult;             /* 1: 3D Maxwellians (table and angles) */
    int32_t sigma_nonzero;        /* magnetised: one more pcosth draw */
    double dseed;                 /* generator state (an integer in a double) */
    int32_t totalpartnum;         /* last ind handed out */
} tg_shock;
/* Set (or replace) the hooks; builds the Maxwell-Juttner tables on the
   host. Errors: TG_ERR_ARG (3D domain, sort_every != 1). */
int tg_shock_init(tg_ctx *ctx, const tg_shock *shock);
/* Current injector / wall / generator state (synchronises). */
int tg_shock_get(tg_ctx *ctx, tg_shock *out);
/* inject_plasma_region over [x1, x2] x [y1, y2] (global coordinates),
   drift along x, with the hooks' plasma (the initial load). */
int tg_inject_region(tg_ctx *ctx, float x1, float x2, float y1, float y2, float ppc, float weight);
/* The three hooks as separate calls (the reference's order is tg_move,
   tg_reset_currents, tg_particle_bc, tg_deposit, ... tg_field_bc ...,
   tg_inject). */
int tg_particle_bc(tg_ctx *ctx);
int tg_field_bc(tg_ctx *ctx);
int tg_inject(tg_ctx *ctx);

/* ---------------------------------------------------------------------
   Restart files in the reference's format: the fields file of
   write_restart (code/output.F90:2192-2201: one unformatted record of
   mx, my, mz, ex, ey, ez, bx, by, bz, dseed, lap, xinject, xinject2,
   xinject3, leftwall, walloc) and its particle file (:2202-2218: ions,
   lecs, maxptl, maxhlf, totalpartnum, then x of the ions and of the
   electrons, y, z, u, v, w, ch, ind, proc, splitlev), read back as
   restart() does (code/restart.F90:209-255). Records follow gfortran's
   unformatted sequential layout (4-byte signed markers, subrecords of at
   most 2147483639 bytes).
   --------------------------------------------------------------------- */
typedef struct {
    double dseed;
    int32_t lap;
    double xinject, xinject2, xinject3;
    float leftwall;
    double walloc;
    int32_t totalpartnum;
    int32_t maxptl;           /* written as is (0: 2 maxhlf) */
    int64_t max_subrecord;    /* 0: gfortran's 2147483639 bytes */
} tg_restart_meta;
/* Write the device state (synchronises). With the shock hooks set, dseed,
   xinject2, walloc and totalpartnum come from the device. */
int tg_write_restart(tg_ctx *ctx, const char *fields_path, const char *particles_path,
                     const tg_restart_meta *meta);
/* Load a restart into the context (the grid must match); *out receives the
   scalars (the shock hooks, when set, take dseed, xinject2, walloc and
   totalpartnum). Currents are not part of the files. */
int tg_read_restart(tg_ctx *ctx, const char *fields_path, const char *particles_path, tg_restart_meta *out);

/* Grid moments of the particles for output_tot (meanq_fld_cur,
   code/output.F90:5222-5482): each particle adds its quantity and its
   weight to the cells of the box (i +- idx, j +- idy, k +- idz) around its
   cell (2D: idz ignored); ghost layers are folded as exchange_current does,
   each cell is divided by its box size, and the velocity-like moments by
   the summed weight. kind: TG_MOMENT_* below, the reference's names.
   num and den are host arrays of mx*my*mz floats. Sums are FP64, rounded to
   single once (the reference sums in single, particle by particle), so
   densities of unit weights are exact. Synchronises. */
#define TG_MOMENT_TDENS 0
#define TG_MOMENT_IDENS 1
#define TG_MOMENT_TBETX 2
#define TG_MOMENT_TBETY 3
#define TG_MOMENT_TBETZ 4
#define TG_MOMENT_IBETX 5
#define TG_MOMENT_IBETY 6
#define TG_MOMENT_IBETZ 7
#define TG_MOMENT_TMOMX 8
#define TG_MOMENT_TMOMY 9
#define TG_MOMENT_TMOMZ 10
#define TG_MOMENT_IMOMX 11
#define TG_MOMENT_IMOMY 12
#define TG_MOMENT_IMOMZ 13
#define TG_MOMENT_EENER 14
#define TG_MOMENT_IENER 15
#define TG_MOMENT_KINDS 16
int tg_moments(tg_ctx *ctx, int32_t kind, int32_t idx, int32_t idy, int32_t idz, float *num, float *den);

/* One variable of the .tot. field output (output_tot,
   code/output.F90:2494-3884) sampled on the device every istep nodes: from
   the first to the last node i in [1, mx] with (i + mxcum) divisible by
   istep, likewise in y and (3D) z; tg_output_dims gives the counts
   (2D: dims[2] = 1). var: TG_OUT_EX..TG_OUT_BZ interpolate the staggered
   field to the node as interpolfld (code/output.F90:4995-5127) does and add
   the constant external field when it is on; TG_OUT_JX..TG_OUT_JZ sample
   the current as it is (the lap's filtered current; the reference re-reads
   a copy it saved); TG_OUT_MOMENT + TG_MOMENT_* sample meanq_fld_cur's
   moment with box half-widths idx, idy, idz as tg_moments (dens = TDENS,
   densi = IDENS, v3x..v3z = TBETX..TBETZ, v3xi.. = IBETX.., v4x.. =
   TMOMX.., v4xi.. = IMOMX.., keni = IENER; the reference's ken asks for
   "tener", a name meanq_fld_cur does not know, and so writes zeros). out
   receives dims[0]*dims[1]*dims[2] floats, x fastest. Synchronises. */
#define TG_OUT_EX 0
#define TG_OUT_EY 1
#define TG_OUT_EZ 2
#define TG_OUT_BX 3
#define TG_OUT_BY 4
#define TG_OUT_BZ 5
#define TG_OUT_JX 6
#define TG_OUT_JY 7
#define TG_OUT_JZ 8
#define TG_OUT_MOMENT 16
int tg_output_dims(tg_ctx *ctx, int32_t istep, int32_t *dims);
int tg_output_var(tg_ctx *ctx, int32_t var, int32_t istep, int32_t idx, int32_t idy, int32_t idz, float *out);
/* The particle sample of output_tot (prtl.tot, code/output.F90:3293-3884):
   the particles of one species (0 ions, 1 electrons) with
   modulo(ind / 2, stride) = 0, in the device's order (tile-sorted; the
   reference writes its array order; the set is the same). Per particle
   vals[k * cap + i] holds, for k = 0..7, x + mxcum, y + mycum, z + mzcum,
   u, v, w, ch and gamma = sqrt(1 + (u^2 + v^2 + w^2)) (the reference's
   xi, yi, zi, ui, vi, wi, chi, gammai), and ids[k * cap + i], k = 0..1,
   ind and proc. *count receives the number selected; when it exceeds cap
   only the count is set (cap = 0 sizes the arrays). Synchronises. */
int tg_output_particles(tg_ctx *ctx, int32_t species, int32_t stride, int64_t cap, float *vals, int32_t *ids,
                        int64_t *count);

/* Energy spectra in the local flow frame for the spectrum output
   (save_spectrum_2d, code/output.F90:794-1249): slices of 30 cells over
   x in [mx0/2 - 1200, mx0/2 + 400] and the interior in y; the gamma range
   over every particle; per species the slice-mean velocity, each
   particle's gamma in that frame, and gambins logarithmic bins of
   gamma - 1 counting the weights ch. tg_spectrum_dims gives nxbins and
   nybins; spec_* hold nxbins*nybins*gambins floats (x fastest), xgamma
   gambins, xslice nxbins, yslice nybins, gamma_range (may be NULL) the
   [gammin, gammax] used. log10 is evaluated in double and rounded once;
   slice means are FP64 sums rounded to single (the reference sums in
   single, particle by particle). Synchronises. */
int tg_spectrum_dims(tg_ctx *ctx, int32_t gambins, int32_t *nxbins, int32_t *nybins);
int tg_spectrum(tg_ctx *ctx, int32_t gambins, float *spec_ions, float *spec_lecs, float *xgamma, float *xslice,
                float *yslice, float *gamma_range);
/* Energy spectra per x slice for the spectrum output (save_spectrum,
   code/output.F90:380-785, the writer the reference's output calls):
   nbins = max((mx0 - 5) / 100, 1) slices of x in [3, mx0 - 2] (all y);
   gambins logarithmic bins of gamma - 1 over the gamma range of every
   particle; per species the lab-frame spectrum (spec_ions, spec_lecs:
   "specp", "spece") and the spectrum in each slice's mean-flow frame
   (spec_*_rest: "specprest", "specerest"), weights splitratio^(1 -
   splitlev) ch with the legacy splitratio = 10, every bin divided by its
   gamma - 1 (xgamma) as the reference does. tg_spectrum_x_bins gives
   nbins; spec_* hold nbins*gambins floats (slice fastest), xgamma gambins,
   xslice nbins, gamma_range (may be NULL) [gammin, gammax]. The
   reference's electron loops start one record early (p(maxhlf), the last
   ion slot, zero unless the ion array is full); that record is not
   counted. Synchronises. */
int tg_spectrum_x_bins(tg_ctx *ctx, int32_t *nbins);
int tg_spectrum_x(tg_ctx *ctx, int32_t gambins, float *spec_ions, float *spec_lecs, float *spec_ions_rest,
                  float *spec_lecs_rest, float *xgamma, float *xslice, float *gamma_range);

/* ---------------------------------------------------------------------
   Batched ensemble: many independent periodic 2D boxes of uneven size
   (seed or parameter ensembles) stepped together, one launch per phase for
   all boxes, the laps replayed from a captured CUDA graph. No counterpart
   in the reference, which runs one domain per job; each box is what one
   run of its main loop steps (code/tristanmainloop.F90:117-303), and the
   per-box entry points mirror the single-domain ones above (same
   arguments with a box index, same error codes). All boxes share the
   deposit mode, the sort cadence, ntimes and the device; boxes may differ
   in size, shape order, plasma and charges. In fixed-point mode every box
   evolves bit for bit as a single-domain context of the same
   configuration. Not thread-safe per ensemble. An ensemble of up to 72
   boxes keeps its boxes' tile arguments in a constant-memory table that is
   one per device and shared by every ensemble of the process: an ensemble
   stepped after another one on the same device waits for the other's
   laps first, so the laps of two such ensembles never overlap on the GPU.
   --------------------------------------------------------------------- */
typedef struct tg_ens tg_ens;
/* cfgs[0..nbox): one tg_config per box (dims 2, periodic x and y). */
int tg_ens_init(const tg_config *cfgs, int32_t nbox, tg_ens **out);
void tg_ens_finalize(tg_ens *ens);
/* Message of the last failure (ens NULL: of the last failed tg_ens_init). */
const char *tg_ens_last_error(tg_ens *ens);
int tg_ens_bind_fields(tg_ens *ens, int32_t box, float *ex, float *ey, float *ez, float *bx, float *by, float *bz,
                       float *curx, float *cury, float *curz);
int tg_ens_bind_particles(tg_ens *ens, int32_t box, void *p, int32_t *ions, int32_t *lecs);
/* Copies of the bound host arrays of every box, as tg_sync_from_host /
   tg_sync_to_host. */
int tg_ens_sync_from_host(tg_ens *ens, unsigned mask);
int tg_ens_sync_to_host(tg_ens *ens, unsigned mask);
/* nsteps laps of every box. */
int tg_ens_step(tg_ens *ens, int32_t nsteps);
int tg_ens_step_timed(tg_ens *ens, int32_t nsteps, float *ms);
/* FP64 diagnostics of one box (as tg_diag_fp64). Synchronises. */
int tg_ens_diag_fp64(tg_ens *ens, int32_t box, tg_diag *out);
int tg_ens_get_counts(tg_ens *ens, int32_t box, int64_t *ions, int64_t *lecs);
int tg_ens_synchronize(tg_ens *ens);
int32_t tg_ens_kernels_per_step(tg_ens *ens);
/* Autotuner of the ensemble: one tile shape and sort cadence for all boxes,
   timed on the given boxes (p[b], *ions[b], *lecs[b] as for
   tg_ens_bind_particles, not modified); writes tile[] and sort_every into
   every cfgs[b]. table rows and return value as tg_autotune. */
int tg_ens_autotune(tg_config *cfgs, int32_t nbox, void *const *p, int32_t *const *ions, int32_t *const *lecs,
                    int32_t laps, float *best_ms, float *table, int32_t table_len);

#ifdef __cplusplus
}
#endif
#endif
