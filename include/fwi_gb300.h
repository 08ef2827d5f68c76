/*
 * fwi_gb300.h -- C ABI of the GB300-native FWI hot path.
 *
 * Every entry point returns 0 on success or a negative FWI_ERR_* code; the
 * message of the last failure on the calling thread is fwi_last_error().
 * Arrays follow the reference's Fortran conventions (column-major, grid
 * indices 1-based and relative to the model, default REAL = float,
 * INTEGER = int32), so a Fortran caller binds them with iso_c_binding and
 * passes its arrays unchanged (see fortran/fwi_gpu_iface.f90).
 *
 * Reference interfaces replaced (paths inside ejimeneztejero/FWI):
 *   fwi_solver_acoustic_ss    src/solver_acoustic_SS.f90:9-11
 *   fwi_misfit_function       src/Misfit.f90:1 (Misfit_function, L2 path
 *                             src/Misfit_L2.f90:1)
 *   fwi_beta_calculous        src/Beta_calculous.f90:1
 *   fwi_misfit_gradient_batch src/calculate_misfit_gradient.f90:1 (all
 *                             shots of one call; the MPI shot loop
 *                             :73-360 becomes on-device batching)
 *   fwi_mcs_geometry          src/get_mcs_data.f90:113-114,147-155,503-512
 *   fwi_was_geometry          src/get_was_data.f90:112-115,155-159,201-205,223-231,584-613
 *   fwi_ricker                src/get_mcs_data.f90:331 (Ricker_mcs)
 *   fwi_time_rules            src/calculate_misfit_gradient.f90:198-203
 *   fwi_time_filter           src/time_filter.f90:1 (time_filter), src/filters.f90:1 (filters_function1D)
 *   fwi_interpolation_akima   src/interpolation_akima.f90:1 (interpolation_akima, INTRPL of akima433.f90:6)
 *   fwi_su_read / fwi_su_info src/get_mcs_data.f90:167 (get_shot_data)
 *   fwi_su_supershot          src/get_was_data.f90:241 (get_obs_data)
 *   fwi_su_write              src/auxiliar.f90:433 (write_new_data: the suaddhead/sushw pipeline)
 *   fwi_read_nav              src/get_mcs_data.f90:88 (read_nav_shot_mcs), src/get_was_data.f90:134
 *                             (read_nav_shot_was), :180 (read_nav_obs)
 */
#ifndef FWI_GB300_H
#define FWI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FWI_OK 0
#define FWI_ERR_ARG (-1)        /* invalid argument (size, index, order)        */
#define FWI_ERR_CUDA (-2)       /* CUDA runtime error                            */
#define FWI_ERR_NOMEM (-3)      /* device memory exhausted                       */
#define FWI_ERR_NONFINITE (-4)  /* NaN/Inf in a result (e.g. CFL-unstable dt)    */
#define FWI_ERR_STATE (-5)      /* library not initialised / bad handle          */

/* Snapshot storage forms for the forward wavefield time derivative. */
#define FWI_SNAP_F32 0
#define FWI_SNAP_BF16 1         /* bfloat16 + power-of-two scale per 128 values */
#define FWI_SNAP_F16 2          /* float16  + power-of-two scale per 128 values */

/* Gradient accumulation forms. */
#define FWI_GRAD_F32 0          /* per-shot FP32 accumulation, as the reference  */
#define FWI_GRAD_F64 1          /* per-shot and cross-shot FP64 accumulation     */

/* ---- library state ------------------------------------------------------ */

/* Select the CUDA device and create the library's stream.  Optional: every
 * other entry point initialises device 0 on first use.  The library serves
 * one device at a time: every entry point makes that device current on the
 * calling thread, and fwi_init with another device first releases everything
 * held on the previous one (as fwi_finalize). */
int fwi_init(int device);
/* Free every device buffer the library holds and destroy its stream. */
int fwi_finalize(void);
/* Message of the last failed call on this thread ("" if none). */
const char* fwi_last_error(void);
/* Run subsequent work on a caller-owned cudaStream_t (NULL = library stream). */
int fwi_set_stream(void* cuda_stream);
/* Solver order/CPML width used by fwi_solver_acoustic_ss.  The reference
 * hard-codes acc = 3, dPML = 20 (solver_acoustic_SS.f90:90-91); acc = 4 is
 * the reference's own 8th-order table (solver_FD_coeffs.f90:21-27,52-58). */
int fwi_set_solver_options(int acc, int dpml);
/* Number of step-kernel launches issued since the library was initialised. */
int64_t fwi_kernel_launch_count(void);

/* ---- drop-in single-shot solver ------------------------------------------ */

/* solver_acoustic_SS(rank,iprop,NumSou,NumRec,nxSou,nySou,nxRec,nyRec,S,Sadj,
 *                    d,dt,ny,nx,ctmp,store_snap,nt_Store,nt,kernel,Fields,
 *                    Rec_point)            -- src/solver_acoustic_SS.f90:9-11
 * All scalars by reference.  iprop = 1: forward; Fields(ny,nx*(nt_Store+1))
 * receives the snapshots (block s = 1..), Rec_point(nt,NumRec) the traces.
 * iprop = 2: adjoint driven by Sadj(nt,NumRec) at the receivers; Fields is
 * read and kernel(ny,nx) is accumulated (+=) with the imaging condition;
 * Rec_point is zeroed.  Host pointers; the copies are part of the call. */
int fwi_solver_acoustic_ss(const int* rank, const int* iprop, const int* NumSou, const int* NumRec,
                           const int* nxSou, const int* nySou, const int* nxRec, const int* nyRec,
                           const float* S, const float* Sadj, const float* d, const float* dt,
                           const int* ny, const int* nx, const float* ctmp, const int* store_snap,
                           const int* nt_Store, const int* nt, float* kernel, float* Fields,
                           float* Rec_point);

/* ---- misfit, adjoint source, Polak-Ribiere beta --------------------------- */

/* Misfit_function(rank,freq,Data_Synth,Data_trace,NumRec,nt,dt,Misfit,
 * AdjSource) with misfit_type = 1 (L2 of max-abs-normalised traces,
 * Misfit.f90:28-61, Misfit_L2.f90:8-14).  Misfit is overwritten with the sum
 * accumulated in FP64 and rounded to float; misfit64 (may be NULL) receives
 * the FP64 value.  AdjSource(nt,NumRec) = time-reversed negative residual. */
int fwi_misfit_function(const int* rank, const float* freq, const float* Data_Synth,
                        const float* Data_trace, const int* NumRec, const int* nt, const float* dt,
                        float* Misfit, float* AdjSource, double* misfit64);

/* Beta_calculous(Grad,OldGrad,nx,ny,Beta) (Beta_calculous.f90:1-25) with the
 * two dot products in FP64 on the device.  num64/den64 may be NULL. */
int fwi_beta_calculous(const float* Grad, const float* OldGrad, const int* nx, const int* ny,
                       float* Beta, double* num64, double* den64);

/* The NLCG model arithmetic of FWI.f90 on the device, in the reference's
 * FP32 operations with exp and log evaluated in FP64 and rounded once (the
 * correctly rounded FP32 value).  Arrays (ny, nx) column-major, host or device
 * pointers (the call detects which).
 *   fwi_first_step:   nut = 1/100/maxval(abs(Search/log(var_orig)))   FWI.f90:175
 *   fwi_model_update: lambda = exp(Search*step)*var_orig         FWI.f90:227, :315 */
int fwi_first_step(const float* Search, const float* var_orig, const int* nx, const int* ny, float* nut);
int fwi_model_update(const float* Search, const float* var_orig, const float* step, const int* nx,
                     const int* ny, float* lambda);

/* ---- geometry and wavelet (host arithmetic, bit-exact FP32) -------------- */

/* One MCS shot: shot x position xs (m), depths, near offset, channel
 * spacing, grid step -> 1-based grid indices, as read_nav_shot_mcs,
 * get_geometry_mcs and get_pos_channels (offset_header = 0) compute them. */
int fwi_mcs_geometry(float xs, float shot_depth, float streamer_depth, float near_offset, float drec,
                     float dmodel, int num_rec, int* nxSou, int* nySou, int* nxRec, int* nyRec);
/* WAS geometry (get_was_data.f90: read_nav_shot_was :155-159, read_nav_obs
 * :201-205, get_bathymetry_model_was :584-613, relocation_zOBS :112-115,
 * get_geometry_WAS :223-231), host FP32 in the reference's order: the OBS are
 * the sources, the shots the receivers.  Inputs: OBS x and z (m), shot x and
 * water depth bat (m), streamer/shot depth, grid step, model columns.
 * relocate = 1 moves every OBS to the bathymetry model (Akima through the
 * shots' water depths) at its column, as the reference does.  Outputs (any
 * may be NULL): nxSou, nySou (num_obs), nxRec (num_shots), *nyRec, and the
 * bathymetry model bat_model, bat_model_grid (nxmodel; bat may be NULL
 * when neither the model nor the relocation is asked for). */
int fwi_was_geometry(int num_obs, const float* xobs, const float* zobs, int num_shots, const float* xshot,
                     const float* bat, float shot_depth, float dmodel, int nxmodel, int relocate, int* nxSou,
                     int* nySou, int* nxRec, int* nyRec, float* bat_model, int* bat_model_grid);
/* Ricker_mcs: out(nt) for peak frequency freq and sampling dt. */
int fwi_ricker(float freq, float dt, int nt, float* out);
/* dt = dmodel/sqrt(max(lambda/1000))/2, nt = 1+ceil(tfin/dt) truncated to a
 * multiple of store_snap, nt_Store = nt/store_snap. lambda(ny,nx) host. */
int fwi_time_rules(const float* lambda, int ny, int nx, float dmodel, float tfin, int store_snap,
                   float* dt, int* nt, int* nt_Store);

/* ---- trace pre-processing on the device ----------------------------------- */

/* time_filter(Data_trace,nt,dt,Num,typef,f1,fc): every trace of
 * Data_trace(nt,Num) (column-major, host or device pointer, filtered in
 * place) is placed at the end of a 24x zero-padded buffer, transformed,
 * multiplied by the Butterworth response of filters_function1D (typef 1
 * low-pass at fc, 2 high-pass at 40 Hz, 3 band-pass f1..fc; order 6 unless
 * fwi_set_filter_order) and transformed back.  The FFT is cuFFT in FP32. */
int fwi_time_filter(float* Data_trace, const int* nt, const float* dt, const int* Num, const int* typef,
                    const float* f1, const float* fc);
/* Butterworth order of fwi_time_filter (the reference hard-codes n = 6,
 * filters.f90:21); 1..32. */
int fwi_set_filter_order(int order);
/* interpolation_akima(Data_tmp,dt_Data,nt_Data,Data_trace,NumRec,dt,nt):
 * Akima resampling (ACM Algorithm 433, as INTRPL) of every trace of
 * Data_tmp(nt_Data,NumRec) from the axis (i-1)*dt_Data to (i-1)*dt,
 * i = 1..nt, into Data_trace(nt,NumRec); host or device pointers.  FP32 in
 * the reference's evaluation order: bit-identical results. */
int fwi_interpolation_akima(const float* Data_tmp, const float* dt_Data, const int* nt_Data, float* Data_trace,
                            const int* NumRec, const float* dt, const int* nt);

/* ---- Seismic Unix trace files (host) -------------------------------------- */

/* ns, dt (s) from the first 240-byte SU header of `path` and the number of
 * traces from the file size; big_endian = byte order of the file. */
int fwi_su_info(const char* path, int big_endian, int* ns, float* dt, int* ntraces);
/* The first ntr traces of nt samples of an SU file into out(nt, ntr)
 * (column-major), skipping the headers, as get_shot_data reads a shot. */
int fwi_su_read(const char* path, int nt, int ntr, int big_endian, float* out);
/* data(nt, ntr) as an SU file: tracl (1-based trace number), ns = nt and
 * dt = int(dt*1e6) microseconds in each header, every other word 0 (what
 * `suaddhead ns= | sushw key=dt a=` writes in write_new_data). */
int fwi_su_write(const char* path, const float* data, int nt, int ntr, float dt, int big_endian);
/* Navigation lists: MCS shots (read_nav_shot_mcs, get_mcs_data.f90:88-117),
 * WAS shots (read_nav_shot_was, get_was_data.f90:148-164) and OBS
 * (read_nav_obs, get_was_data.f90:196-207): one record per line -- an
 * integer (shot or OBS number) and two reals (x in m, and water depth or OBS
 * depth in m) -- blanks or commas between values.  Fills up to max_records
 * entries and returns the number of records in the file in *nrecords. */
int fwi_read_nav(const char* path, int max_records, int* shot_id, float* xs, float* bat, int* nrecords);
/* get_obs_data(rank,iSS,NumSou_SS,NumRec_SS,Coding,raw_data)
 * (get_was_data.f90:241-288): the first ntr traces (nt samples) of each of the
 * nsrc OBS files paths[k] -- the reference's OBS number SourceNum(iSS,k,NumSS)
 * = iSS+NumSS*(k-1) (auxiliar.f90:73-88) -- summed into raw_data(nt,ntr)
 * (column-major, zeroed first) as raw_data = raw_data + Coding(k)*data, FP32. */
int fwi_su_supershot(const char* const* paths, int nsrc, const float* coding, int nt, int ntr, int big_endian,
                     float* raw_data);

/* ---- batched misfit + gradient over shots ------------------------------ */

typedef struct fwi_shot {
    int x0;               /* first model column of the shot's window (0-based)   */
    int nx;               /* window width in model columns                       */
    int num_sou, num_rec;
    const int* nxSou;     /* window-relative 1-based grid indices (num_sou)      */
    const int* nySou;
    const int* nxRec;     /* (num_rec)                                           */
    const int* nyRec;
    const float* src;     /* S(nt, num_sou), column-major                        */
    const float* obs;     /* observed Data_target(nt, num_rec), column-major     */
    double grad_weight;   /* weight of this shot's kernel in the stack (1.0)     */
    double misfit_weight; /* weight of this shot's misfit in the sum (1.0)       */
} fwi_shot;

typedef struct fwi_survey_desc {
    int ny;               /* model rows (depth)                                  */
    int nx_model;         /* model columns                                       */
    float d;              /* grid step (m)                                       */
    float dt;             /* time step (s)                                       */
    int nt;               /* time samples, common to all shots                   */
    int store_snap;       /* snapshot decimation (reference: 10)                 */
    int acc;              /* FD half-order: 3 (reference) or 4                   */
    int dpml;             /* CPML cells (reference: 20)                          */
    int numtasks;         /* gradient divisor of the reference's MPI reduction   */
    int snap_form;        /* FWI_SNAP_*                                          */
    int grad_form;        /* FWI_GRAD_*                                          */
    int nshots;
    const fwi_shot* shots;
    const int* water_rows;/* bat_model_grid(nx_model): rows 1..k zeroed, or NULL */
    size_t hbm_budget;    /* bytes the survey may hold on the device (0 = all)   */
    int wave_shots;       /* shots per concurrent wave (0 = chosen by the tuner) */
    int band_rows;        /* rows per warp work item (0 = chosen by the tuner)   */
    int flags;            /* FWI_SURVEY_* bits                                   */
    int tile_kernel;      /* two-step tile kernel: 0 = chosen by the tuner,
                             1 = register queues, 2 = shared-memory queue        */
    int tile_rows;        /* rows per two-step tile (0 = chosen by the tuner)    */
    int tile_edge_rows;   /* rows of the bottom edge band -- the last
                             two-step rows, next to the single-step rows above
                             the bottom pad -- (0 = chosen by the tuner; more
                             than the model's rows: the last core-height
                             band)                                            */
} fwi_survey_desc;

/* fwi_survey_desc.flags: launch every time step directly instead of
 * replaying the captured CUDA graph (the plain one-launch-per-step path). */
#define FWI_SURVEY_NO_GRAPH 1
/* fwi_survey_desc.flags: keep forward-state checkpoints and a small snapshot
 * ring and recompute forward segments during the adjoint (one more forward
 * pass, far less memory).  Chosen automatically when the HBM budget would
 * otherwise leave waves of fewer than 8 shots. */
#define FWI_SURVEY_RECOMPUTE 2
/* fwi_survey_desc.flags: advance every time step with the single-step
 * kernels.  By default, pairs of steps with no snapshot or imaging in them
 * run as two-step passes (the model-row interior advanced twice per sweep
 * over the wavefields); the results are bit-identical either way. */
#define FWI_SURVEY_SINGLE_STEP 4
/* fwi_survey_desc.flags: single steps, each one launch of the fused kernel
 * (interior, side strips and bottom tiles together) instead of three on
 * three streams; implies FWI_SURVEY_SINGLE_STEP.  The tuner picks this form
 * for a small wave where it is measured faster; results are bit-identical. */
#define FWI_SURVEY_FUSED_STEP 8
/* fwi_survey_desc.flags: replay the captured CUDA graph from the first run
 * on, without timing it against direct launches (FWI_SURVEY_NO_GRAPH wins
 * over it). */
#define FWI_SURVEY_GRAPH 16

typedef struct fwi_survey fwi_survey;

/* Plan a survey: validate the geometry, upload sources and observed data,
 * size the shot waves to the HBM budget and allocate device buffers. */
int fwi_survey_create(const fwi_survey_desc* desc, fwi_survey** out);
/* New time axis for an existing survey (the line search of FWI.f90:225-230
 * recomputes dt from the CFL rule and nt = 1+ceiling(tfin/dt) for every trial
 * model; calculate_misfit_gradient.f90:198-203 truncates nt to whole
 * snapshot blocks).  src: all shots' sources resampled to (dt, nt), shot after
 * shot, each (nt, num_sou) column-major; obs: all shots' observed traces,
 * (nt, num_rec) each, in shot order.  Host or device pointers; NULL = zeros.
 * The survey keeps its model, buffers (grown if nt grew) and band height; the
 * wave plan is redone when nt changes and the graphs are re-captured. */
int fwi_survey_set_time(fwi_survey* s, float dt, int nt, const float* src, const float* obs);
int fwi_survey_destroy(fwi_survey* s);
/* Model parameter: lambda(ny,nx_model) bulk modulus (rho = 1000), host or
 * device pointer (the call detects which).  Vp = sqrt(lambda/1000.) as in
 * calculate_misfit_gradient.f90:252. */
int fwi_survey_set_lambda(fwi_survey* s, const float* lambda);
/* Replace the observed data of every shot (host or device pointer to the
 * shots' obs blocks packed in shot order, each (nt, num_rec)). */
int fwi_survey_set_observed(fwi_survey* s, const float* obs_packed);
/* Replace every shot's source wavelets (packed like set_observed). */
int fwi_survey_set_sources(fwi_survey* s, const float* src_packed);
/* One calculate_misfit_gradient call: step = 1 forward + misfit + adjoint +
 * imaging + stack; step = 2 forward + misfit only (line-search trials).
 * misfit (may be NULL) += the weighted misfit sum (FP64); grad (may be NULL)
 * (ny, nx_model) host float is updated as Grad = Grad + stack/numtasks and
 * the water rows are zeroed, as calculate_misfit_gradient.f90:339-351. */
int fwi_survey_run(fwi_survey* s, int step, double* misfit, float* grad);
/* Device pointer to the FP64 gradient stack of the last run
 * ((ny, nx_model) column-major, before the numtasks divisor and mask). */
int fwi_survey_grad_device(fwi_survey* s, const double** ptr);
/* The same FP64 stack copied to host memory (ny*nx_model doubles, column-
 * major): the per-rank term of the reference's MPI_REDUCE of Grad
 * (calculate_misfit_gradient.f90:299-300) when shots are split over ranks. */
int fwi_survey_get_stack(fwi_survey* s, double* out);
/* Synthetic traces of shot i from the last run: Rec_point(nt, num_rec),
 * copied to host. */
int fwi_survey_get_synthetic(fwi_survey* s, int shot, float* out);
/* Algorithmic HBM bytes of one forward time step of the shots of the first
 * wave (the unit fwi_survey_time_steps advances). */
int fwi_survey_step_bytes(fwi_survey* s, double* bytes);
/* Algorithmic bytes of one time step of the first wave when the steps run as
 * two-step passes (the two-step tiles move 20 B per cell for two steps, the
 * single-step lists their usual bytes), and the tiles' bytes of one pass.
 * Without two-step tiles per_step equals fwi_survey_step_bytes. */
int fwi_survey_two_step_bytes(fwi_survey* s, double* per_step, double* tiles_per_pass);
/* Tuning chosen for the survey (wave size, band rows). */
int fwi_survey_tuning(fwi_survey* s, int* wave_shots, int* band_rows);
/* Two-step tiles chosen for the survey: kernel (1 = register queues, 2 =
 * shared-memory queue; 0 when the survey runs single steps only) and rows per
 * tile.  With times != NULL, also the tuner's measurements: times[k*ncand+c]
 * = ms per forward two-step pass of the first wave for kernel k+1 and tile
 * height cand[c] (-1 where not measured; cached or forced choices measure
 * nothing); *ncand receives the number of tile heights tried (at most 8). */
int fwi_survey_tiles(fwi_survey* s, int* tile_kernel, int* tile_rows, int* cand, float* times, int* ncand);
/* Rows of the bottom edge band chosen for the survey (0: the last core-height
 * band) and the tuner's measurements: times[c] = ms per forward two-step pass
 * of the first wave with a bottom edge band of cand[c] rows (-1 where not
 * measured; at most 8). */
int fwi_survey_edge_tiles(fwi_survey* s, int* edge_rows, int* cand, float* times, int* ncand);
/* Time stepping chosen for the survey: *form = 1 two-step passes; 0 single
 * steps, three launches on three streams each; 2 single steps, one launch
 * each.  Single steps run under FWI_SURVEY_SINGLE_STEP, without two-step
 * tiles, or where the tuner measured them faster (a small wave, whose time
 * step is latency-bound).  *two_step_ms, *single_ms, *fused_ms: the
 * tuner's timings of the first wave per two time steps (-1 where not
 * measured: a forced or cached choice). */
int fwi_survey_stepping(fwi_survey* s, int* form, float* two_step_ms, float* single_ms, float* fused_ms);
/* Launch form of the first wave's runs with this step (1 gradient, 2
 * forward and misfit): *form = 1 replays of a captured CUDA graph, 2 direct
 * launches, 0 not decided yet.  A time axis runs directly the first time and
 * as a graph replay the second; both runs are timed (*direct_ms, *graph_ms;
 * 0 where not measured), and a graph slower than the direct launches is
 * dropped; one that looks faster is kept only if the third run, launched
 * directly once more, does not beat it.  FWI_SURVEY_NO_GRAPH: always 2. */
int fwi_survey_launch_form(fwi_survey* s, int step, int* form, float* direct_ms, float* graph_ms);
/* Checkpointed recomputation plan: forward steps per segment and number of
 * segments (0, 0 when all snapshots are stored). */
int fwi_survey_recompute(fwi_survey* s, int* segment_steps, int* segments);
/* Run `steps` forward time steps of the first wave (for kernel timing; the
 * wavefields keep evolving, sources are injected). */
int fwi_survey_time_steps(fwi_survey* s, int steps);

/* calculate_misfit_gradient(iter,step,f1,f2,dt,nt,tfin,S0,Misfit,Grad) for
 * all shots in one call, with host buffers: uploads lambda, sources and
 * observed data, runs, and downloads Misfit (+=) and Grad (updated, masked).
 * src/calculate_misfit_gradient.f90:1-366
 * The library keeps the plan (device buffers, work lists, tuning, graphs) of
 * the last geometry it was called with -- sizes, grid indices, weights and
 * forms, not dt and nt: a call with a new dt/nt (the line search of
 * FWI.f90:225-227 derives them from every trial model) moves that plan to the
 * new time axis as fwi_survey_set_time does; a new geometry frees the old
 * plan before it plans. */
int fwi_misfit_gradient_batch(const fwi_survey_desc* desc, const float* lambda, int step,
                              float* Misfit, float* Grad);
/* Number of plans fwi_misfit_gradient_batch has built in this process. */
int64_t fwi_batch_plans(void);
/* The survey of fwi_misfit_gradient_batch's current plan (NULL before the
 * first call), owned by the library: for the query entries (fwi_survey_tiles,
 * fwi_survey_stepping, fwi_survey_launch_form ...); valid until the next
 * call with another geometry, fwi_batch_release or fwi_finalize. */
int fwi_batch_survey(fwi_survey** s);
/* Free the plan fwi_misfit_gradient_batch holds (its device memory). */
int fwi_batch_release(void);

/* ---- forward traces without device allocation --------------------------- */

/* No counterpart in the reference: an addition for callers that cannot call
 * cudaMalloc -- code inside a framework that owns the device memory pool (a
 * raw cudaMalloc synchronises the device and falls outside the pool's
 * budget) and code paths that must not allocate once they are set up.
 *
 * Forward propagation of one shot (the reference's solver_acoustic_SS with
 * iprop = 3: traces only, no snapshots) with the order and CPML width of
 * fwi_set_solver_options.  The caller passes its own DEVICE buffers for
 * S(nt,NumSou), ctmp(ny,nx) and the output Rec_point(nt,NumRec); the grid
 * indices are host arrays.  All working state (wavefields, c2, CPML memory
 * variables, work lists) lives in one fixed 16 MiB device array that every
 * GPU loading this library holds until the process exits; grids whose state
 * does not fit (about 8*(ny+2*dn)*(nx+2*dn+128)*4 bytes, dn = dpml+2*acc)
 * are rejected with FWI_ERR_ARG.  Nothing is allocated: no cudaMalloc,
 * cudaFree or allocating library call.
 *
 * The first call on a device looks up the array's device address (and, if
 * the library was not initialised, creates its streams); make that first
 * call before any stream capture.  Every call shares the one array, which
 * keeps the last call's contents (the call clears what must start at zero):
 * calls that overlap on the GPU -- from several host threads or streams --
 * race and must not be issued.  The call waits for its stream to finish
 * before it returns. */
int fwi_solver_forward_noalloc(int NumSou, int NumRec, const int* nxSou, const int* nySou,
                               const int* nxRec, const int* nyRec, const float* S_dev, float d, float dt,
                               int ny, int nx, const float* ctmp_dev, int nt, float* Rec_point_dev);

#ifdef __cplusplus
}
#endif

#endif /* FWI_GB300_H */
