/*
 * gbfdtd.h — C ABI of the GB300 FDTD solver core for gprMax models (libgbfdtd.so).
 *
 * The library replaces the time-stepping part of gprMax v3.1.7: the loop of solve_cpu /
 * solve_gpu (gprMax/model_build_run.py:408-474 and :477-716) and the kernels it calls
 * (gprMax/fields_updates_ext.pyx, gprMax/pml_updates/pml_updates_*_ext.pyx,
 * gprMax/sources.py update_* methods, gprMax/fields_outputs.py store_outputs,
 * gprMax/snapshots.py Snapshot.store). The host builds the model exactly as the reference
 * does (material IDs, fp32 update coefficients, PML coefficient rows, source waveform tables)
 * and hands the arrays over through this interface; every array crosses as a plain host
 * pointer with the reference's C-order layout.
 *
 * Conventions
 *  - Every call returns GBF_OK (0) or a negative GBF_E* status; the message of the last
 *    failure on a context is available from gbf_last_error. Nothing calls exit() or traps.
 *  - Host buffers are owned by the caller and copied; device memory is owned by the context.
 *    Every call has copied what it needs out of the caller's buffers when it returns; the small
 *    uploads (PML rows, sources, receivers) complete on the context's stream before its next
 *    run, and gbf_reset and gbf_synchronize wait for them.
 *  - One context per host thread; calls on one context are not re-entrant. The context owns
 *    one CUDA stream on which all of its work runs.
 *  - Grid sizes nx, ny, nz are cell counts; field and ID arrays have (nx+1)(ny+1)(nz+1) nodes
 *    per component, C order with k (z) fastest, exactly as gprMax/grid.py:157-178.
 */
#ifndef GBFDTD_H
#define GBFDTD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBF_OK 0
#define GBF_EINVAL (-1)      /* bad argument, size or layout */
#define GBF_ECUDA (-2)       /* CUDA runtime error (message has the CUDA error string) */
#define GBF_ENOMEM (-3)      /* device allocation failed */
#define GBF_ESTATE (-4)      /* call out of order (e.g. run before materials were uploaded) */
#define GBF_ENONFINITE (-5)  /* the NaN/Inf probe found a non-finite receiver sample */

/* PML formulations (gprMax/pml.py:156-159) */
#define GBF_PML_HORIPML 0
#define GBF_PML_MRIPML 1

/* source kinds (gprMax/sources.py) */
#define GBF_SRC_HERTZIAN 0          /* E -= ((srce*w[it])*s0)*s1        sources.py:163-193 */
#define GBF_SRC_VOLTAGE_RESISTIVE 1 /* E -= (srce*w[it])*s0             sources.py:81-120  */
#define GBF_SRC_VOLTAGE_HARD 2      /* E = (-w[it])/s0 while active     sources.py:81-120  */
#define GBF_SRC_MAGNETIC 3          /* H -= (srcm*w[it])*s0             sources.py:202-232 */
#define GBF_SRC_TRANSMISSION_LINE 4 /* E = -V(antpos)/d of the line      sources.py:396-424 */

/* gbf_run flags */
#define GBF_RUN_GRAPH 1u     /* replay the step sequence from a captured CUDA graph */
#define GBF_RUN_CHECK 2u     /* after the run, test receiver samples for NaN/Inf */

/* Model description. Mirrors the attributes of gprMax's FDTDGrid that the time loop reads. */
typedef struct gbf_grid_desc {
    int32_t nx, ny, nz;          /* cells (grid.py: G.nx, G.ny, G.nz) */
    int32_t iterations;          /* time steps (input_cmds_singleuse.py:184-207) */
    int32_t nmat;                /* rows of the coefficient tables (len(G.materials)) */
    int32_t maxpoles;            /* dispersive poles per material, 0 = none (Material.maxpoles) */
    int32_t pml_formulation;     /* GBF_PML_* (G.pmlformulation) */
    int32_t pml_order;           /* CFS terms per slab, 1 or 2 (len(G.cfs)) */
    int32_t pml_thickness[6];    /* cells for x0, y0, z0, xmax, ymax, zmax (G.pmlthickness) */
    float dx, dy, dz;            /* cell sizes as fp32 (the PML kernels' `float d`) */
    int32_t nsrc;                /* sources (voltage sources, then Hertzian, then magnetic) */
    int32_t nrx;                 /* receivers */
    int32_t nsnap;               /* snapshots */
    int32_t options;             /* bit 0: read coefficient tables from global memory instead
                                    of staging them in shared memory (tuning); bit 1: form the
                                    PML differences dF/d by division even where the reciprocal
                                    product is exact (gbf_check_cell_division); bit 2: keep the
                                    dispersive state complex even when every pole is Debye
                                    (otherwise only its real parts are stored then, the
                                    imaginary parts being +0 throughout; needed to batch such a
                                    model with others whose state is complex); bit 3: advance
                                    every iteration with the two half-step kernels even where
                                    the fused step applies (see gbf_run); bit 4: take the plain
                                    half-step kernels even where the staged ones apply (3D
                                    grids with at most 1024 materials, for E no poles or at most
                                    two Debye-like poles: their inputs are copied chunk by chunk
                                    into shared memory ahead of the threads that update them;
                                    the same results bit for bit); bit 5: allocate the fused
                                    step's second field buffer for a model with PML slabs too
                                    (otherwise such models, for which the fused step is slower,
                                    do without it and gbf_set_fused_tiles refuses them); other
                                    bits 0 */
    int32_t ntl;                 /* transmission lines among the nsrc sources */
    int32_t reserved[2];         /* must be zero */
} gbf_grid_desc;

typedef struct gbf_ctx gbf_ctx;

/* Create a context on the current CUDA device and allocate all device state.
 * Replaces: the array set-up of solve_gpu (model_build_run.py:505-583; grid.py:251-272;
 * pml.py:298-364). */
int gbf_create(const gbf_grid_desc* desc, gbf_ctx** out);

/* Destroy a context and free its device memory. Safe on NULL. */
void gbf_destroy(gbf_ctx* ctx);

/* Copy the material IDs and coefficient tables.
 *   ID       uint32 [6][nx+1][ny+1][nz+1]   component order Ex, Ey, Ez, Hx, Hy, Hz (grid.py:168)
 *   coeffE   fp32   [nmat][5]  CA, CBx, CBy, CBz, srce   (materials.py:200-201)
 *   coeffH   fp32   [nmat][5]  DA, DBx, DBy, DBz, srcm
 *   coeffD   complex64 as fp32 pairs [nmat][3*maxpoles] (e0*eqt2, eqt, zt) per pole, or NULL
 *            when maxpoles == 0 (materials.py:204-208)
 * Replaces: the __constant__ coefficient upload of solve_gpu (model_build_run.py:512-529). */
int gbf_upload_materials(gbf_ctx* ctx, const uint32_t* ID, const float* coeffE,
                         const float* coeffH, const float* coeffD);

/* The material IDs as two packed words per node (models with at most 1024 materials), made
 * by gbf_pack_ids: PE uint32 [nx+1][ny+1][nz+1] = IDx | IDy << 10 | IDz << 20 of the E
 * components, PH the same for H; coefficient tables as for gbf_upload_materials. Copies a third
 * of the bytes of the ID array (from page-locked memory, see gbf_host_alloc, at the full copy
 * rate). PH may be NULL when every material has the same H row (no magnetic materials: no
 * kernel then reads H IDs), which halves the copy. GBF_EINVAL when an ID does not index the
 * tables, PH is NULL for a model whose H rows differ, or the model has more than 1024
 * materials. No counterpart in the reference: the same upload as gbf_upload_materials
 * (model_build_run.py:512-529) from a compact form of the ID array. */
int gbf_upload_materials_packed(gbf_ctx* ctx, const uint32_t* PE, const uint32_t* PH,
                                const float* coeffE, const float* coeffH, const float* coeffD);

/* Pack an ID array [6][n] (n nodes per component, the layout of gbf_upload_materials) into
 * PE and PH [n] on the host's cores (PH NULL: the E words only, and only the E IDs read);
 * *maxid gets the largest ID packed (GBF_EINVAL above 1023). Host arithmetic only. No
 * counterpart in the reference. */
int gbf_pack_ids(const uint32_t* ID, int64_t n, uint32_t* PE, uint32_t* PH, uint32_t* maxid);

/* Page-locked host memory (cudaHostAlloc) for the inputs of gbf_upload_materials_packed, and
 * its release. No counterpart in the reference. */
int gbf_host_alloc(size_t bytes, void** out);
void gbf_host_free(void* p);

/* Use another context's material IDs and coefficient tables instead of uploading them: the
 * traces of a B-scan over one fixed geometry then share one copy of the IDs and tables on the
 * device (the reference's --geometry-fixed model runs build the grid once and reuse it,
 * model_build_run.py:104-106 and :400-403). The contexts must have the same grid, material
 * and pole counts, dispersive-state layout (options bit 2) and device; the shared arrays live
 * until the last context holding them is destroyed. Replaces: nothing in the reference, whose
 * GPU solver uploads every model run's arrays. */
int gbf_share_materials(gbf_ctx* ctx, gbf_ctx* owner);

/* Copy one PML slab's coefficient rows, each fp32 [pml_order][thickness], E then H:
 * ERA, ERB, ERE, ERF, HRA, HRB, HRE, HRF (pml.py:221-274). `slab` indexes x0, y0, z0, xmax,
 * ymax, zmax; slabs with zero thickness take no call. Replaces: PML.gpu_initialise_arrays
 * (pml.py:306-319). */
int gbf_upload_pml(gbf_ctx* ctx, int slab, const float* const rows[8]);

/* Copy the source list. Per source: info int32[8] = kind (GBF_SRC_*), component (0-2 for E,
 * 3-5 for H), i, j, k, first and last active iteration (inclusive), 0; scale fp32[2]; waves
 * fp32 [nsrc][iterations] (whole-step table for Hertzian and resistive sources, half-step for
 * hard voltage sources and magnetic dipoles). Order matters: within one iteration E sources
 * apply in list order after the PML (model_build_run.py:459-461).
 * Replaces: gpu_initialise_src_arrays (sources.py:235-283). */
int gbf_upload_sources(gbf_ctx* ctx, const int32_t* info, const float* scale,
                       const float* waves);

/* Receiver positions int32 [nrx][3]. Outputs per receiver are Ex, Ey, Ez, Hx, Hy, Hz, Ix,
 * Iy, Iz. Replaces: gpu_initialise_rx_arrays (receivers.py:45-68). */
int gbf_set_receivers(gbf_ctx* ctx, const int32_t* coords);

/* Snapshot definitions int32 [nsnap][10] = xs, ys, zs, dx, dy, dz (cells), nx, ny, nz, time.
 * Snapshot s is taken at the start of iteration time-1 (model_build_run.py:429-431). */
int gbf_set_snapshots(gbf_ctx* ctx, const int32_t* defs);

/* Zero the fields, PML and dispersive state and restart at iteration 0. */
int gbf_reset(gbf_ctx* ctx);

/* Advance `nsteps` iterations from the current one (flags: GBF_RUN_*). Each iteration runs
 * the H half-step (update, PML, magnetic sources), the E half-step (update or dispersive
 * update, PML, E sources, dispersive second part) and stores receiver samples, in the order of
 * solve_cpu (model_build_run.py:424-470). Asynchronous on the context stream unless
 * GBF_RUN_CHECK is set.
 * 3D models with at most 1024 materials, at most 2 poles and no transmission lines can also
 * advance with one fused kernel per iteration (both half-steps in one pass over the grid; the
 * same results bit for bit), unless options bit 3 is set. For models without PML slabs, which
 * form runs, and the fused kernel's tiles, are chosen by timing: the first steps of the first
 * run of each model shape in the process each use one candidate (twice round; the model
 * advances as usual, the choice changing no result) and the fastest is kept from then on.
 * Models with PML slabs take the half-step kernels (measured faster there) unless
 * gbf_set_fused_tiles selects the fused step. Where a staged sweep applies to a half-step
 * (options bit 4), staged or plain is chosen the same way (the first steps of the first run of
 * each model shape run all staged sweeps and all plain kernels in turn, each half-step timed
 * apart and keeping its faster form; gbf_set_step_forms fixes it); the staged sweeps'
 * waits for shared-memory stages are bounded, and one that ran out makes GBF_RUN_CHECK,
 * gbf_download_rx and gbf_download_fields return GBF_ECUDA. */
int gbf_run(gbf_ctx* ctx, int nsteps, uint32_t flags);

/* Iteration the next gbf_run call starts at. */
int gbf_current_iteration(gbf_ctx* ctx, int32_t* it);

/* Block until all work on the context stream is complete. */
int gbf_synchronize(gbf_ctx* ctx);

/* Receiver samples fp32 [9][iterations][nrx] (Ex, Ey, Ez, Hx, Hy, Hz, Ix, Iy, Iz).
 * Replaces: gpu_get_rx_array (receivers.py:71-88). */
int gbf_download_rx(gbf_ctx* ctx, float* rxs);

/* Fields fp32 [6][nx+1][ny+1][nz+1] (Ex, Ey, Ez, Hx, Hy, Hz): download / upload. */
int gbf_download_fields(gbf_ctx* ctx, float* fields);
int gbf_upload_fields(gbf_ctx* ctx, const float* fields);

/* Dispersive state complex64 as fp32 pairs [3][maxpoles][nx+1][ny+1][nz+1] (Tx, Ty, Tz);
 * when only real parts are stored (Debye poles, options bit 2 clear) they come back with
 * imaginary parts +0, which is what the complex update holds there. */
int gbf_download_dispersive(gbf_ctx* ctx, float* T);

/* Snapshot s: fp32 [6][snx][sny][snz] cell-averaged Ex, Ey, Ez, Hx, Hy, Hz
 * (snapshots_ext.pyx:24-71). */
int gbf_download_snapshot(gbf_ctx* ctx, int s, float* out);

/* Time `nsteps` iterations on the context stream with CUDA events around every launch; adds
 * the summed device milliseconds of the H and E half-step kernels and of the whole sequence.
 * With the fused step the whole update is one kernel: its time goes to *ms_e, *ms_h gets 0. */
int gbf_profile(gbf_ctx* ctx, int nsteps, float* ms_h, float* ms_e, float* ms_total);

/* Fix the fused step's tiles instead of letting the first run time candidates: tile height tj
 * (7 or 15 rows) and nch chunks along x (<= 0: one wave of resident blocks). Results do not depend
 * on the tiling. GBF_ESTATE when the model does not take the fused step. No counterpart in the
 * reference. */
int gbf_set_fused_tiles(gbf_ctx* ctx, int32_t tj, int32_t nch);

/* A fractal field on the device (#fractal_box, #add_surface_roughness): the fp32 real part of
 * the inverse FFT of FFT(noise) / r^D, r the distance of each frequency from the spectrum's
 * centre with per-axis weights, r^D = 0.9 where it is 0, the DC term zeroed
 * (gprMax/fractals.py:141-194 and :29-111, filter fractals_generate_ext.pyx:24-86). rank 2 or 3,
 * dims [rank], weights [rank], noise float64 [dims] (host, the seeded Gaussian noise), field
 * float32 [dims] (host). Double-precision transforms (cuFFT): equal to the reference's field to
 * rounding, not bit for bit; the reference's binning of it is left to the caller. */
int gbf_fractal_field(int32_t rank, const int32_t* dims, const double* weights, float dimension,
                      const double* noise, float* field);

/* The fused step's launch decomposition for a grid of nx x ny x nz cells, tile height tj rows
 * and nch chunks along x (host arithmetic only, no device call): out[0] k segments, [1] j
 * tiles, [2] chunks, [3] planes per chunk, [4] blocks, [5] k nodes owned per tile. Block b works
 * on segment b % out[0], tile (b / out[0]) % out[1], chunk b / (out[0] * out[1]) with tj + 1
 * warps, warp w on row tile * tj - 1 + w. No counterpart in the reference; exported so the tiling
 * can be checked without a GPU. */
int gbf_fused_tiles(int32_t nx, int32_t ny, int32_t nz, int32_t tj, int32_t nch, int32_t* out);

/* How the context steps: info[0] 1 for the fused step (0: two half-step kernels), [1] its tile
 * height in j, [2] chunks along x, [3] planes per chunk, [4] blocks per launch, [5] 1 once the
 * step form and tiles are chosen, [6] the field buffer holding the current iteration, [7] bit 0
 * the second buffer exists, bit 1 a fused kernel exists for the model, bits 2 and 3 the E and
 * the H half-step are staged sweeps (their inputs copied into shared memory by bulk copies;
 * options bit 4), bit 4 set once staged or plain is chosen for each, bits 5 and 6 a staged
 * sweep applies to E, to H. No counterpart in the reference (its GPU solver has one fixed launch
 * shape, grid.py:103). */
int gbf_step_info(gbf_ctx* ctx, int32_t info[8]);

/* Fix the form of the half-steps: bit 0 the staged E sweep, bit 1 the staged H sweep (clear:
 * the plain kernel), instead of choosing by timing at the first run. GBF_EINVAL when a staged
 * sweep asked for does not apply to the model. The results are the same bit for bit. No
 * counterpart in the reference. */
int gbf_set_step_forms(gbf_ctx* ctx, int32_t forms);

/* Run `nsteps` iterations like gbf_run, bracketed by CUDA events recorded on the context
 * stream; blocks until done and returns the elapsed device milliseconds in *ms. */
int gbf_run_timed(gbf_ctx* ctx, int nsteps, uint32_t flags, float* ms);

/* Bytes of device memory the context holds. */
int gbf_device_bytes(gbf_ctx* ctx, size_t* bytes);

/* Make CUDA device `device` current for the calling host thread, so that the contexts it creates
 * next live there. Replaces the device choice of the reference's -gpu option (gprMax/gprMax.py:
 * 132-144: the first of the given device IDs for a standard run; the reference then opens its
 * context on that device in solve_gpu, model_build_run.py:477-500). GBF_EINVAL for an index
 * outside [0, device count); the failure message is read with gbf_last_error(NULL, ...). */
int gbf_set_device(int32_t device);

/* Copy the message of the last failure on `ctx` (or of the last gbf_create failure when ctx
 * is NULL) into buf. */
int gbf_last_error(gbf_ctx* ctx, char* buf, size_t n);

/* Library version string. */
const char* gbf_version(void);

/* Transmission lines (sources.py:286-451), after gbf_upload_sources (whose kind-4 entries are
 * the lines, in order). info [ntl][9]: component, i, j, k, first and last active iteration,
 * cells of the connected line, injector cell, antenna cell; coef [ntl][4] (float64): (1/R) c dt/dl,
 * R c dt/dl, c dt/dl and the absorbing end's (c dt - dl)/(c dt + dl); state [ntl][34]: voltage
 * [16], current [16], abcv0, abcv1 of the line after the incident-wave run
 * (calculate_incident_V_I); cell [ntl]: the edge's cell size (fp32); waves [ntl][2][iterations]:
 * the waveform at whole and half steps. Replaces: TransmissionLine.update_magnetic/_electric. */
int gbf_upload_tls(gbf_ctx* ctx, const int32_t* info, const double* coef, const float* state,
                   const float* cell, const float* waves);
/* [ntl][2][iterations]: Vtotal, Itotal (fields_outputs.py:65-67, tl.Vtotal / tl.Itotal) */
int gbf_download_tls(gbf_ctx* ctx, float* out);

/* ---- batches: many models advanced together ----------------------------------------
 * A batch borrows contexts that are fully set up (materials, PML rows, sources, receivers
 * uploaded; no snapshots; all at the same iteration, with the same PML kind, pole count and
 * material-ID layout) and advances all of them with one persistent launch per half-step plus
 * one end-of-step launch, replaying the requested time loop from one CUDA graph; a model of
 * 2^21 nodes or more, which fills the GPU alone, takes its own half-step kernels (staged where
 * they apply) within the same graph instead of a share of the batched ones. Results are
 * read from each context as usual (gbf_download_rx ...). While a batch exists, its contexts
 * must not be run or re-uploaded on their own; destroy the batch before the contexts.
 * Replaces: the task farm of independent model runs for B-scans and parameter sweeps
 * (gprMax/gprMax.py:run_std_sim, run_mpi_sim and model_build_run.py:84-405 per model). */
typedef struct gbf_batch gbf_batch;
int gbf_batch_create(gbf_ctx* const* models, int32_t nmodels, gbf_batch** out);
void gbf_batch_destroy(gbf_batch* batch);
/* Advance every model nsteps iterations (flags: GBF_RUN_GRAPH). The first run of a batch
 * chooses the grid size of its persistent launches by timing: its first steps each use one
 * candidate (1 to 4 blocks per SM, twice round; real steps, the grid size changing no result),
 * and the fastest is kept for the batch and, per set of model shapes, for the process. */
int gbf_batch_run(gbf_batch* batch, int32_t nsteps, uint32_t flags);
/* The same, timed with CUDA events on the batch's stream (graph capture outside the timing
 * once the grid size is chosen). */
int gbf_batch_run_timed(gbf_batch* batch, int32_t nsteps, uint32_t flags, float* ms);
/* info[0] 1 once the grid size is chosen, [1] blocks of the H launch, [2] of the E launch,
 * [3] models stepped with their own kernels. No counterpart in the reference. */
int gbf_batch_info(gbf_batch* batch, int32_t info[4]);
int gbf_batch_synchronize(gbf_batch* batch);
int gbf_batch_last_error(gbf_batch* batch, char* buf, size_t n);

/* ---- differentiable time loop (adjoint) ---------------------------------------------
 * Receiver traces of a non-dispersive 3D model with one (CA, CB) pair per E edge, and the
 * gradient of a misfit with respect to every CA and CB through the discrete adjoint
 * (transposed updates in reverse time, recomputed from checkpoints every checkpoint_interval
 * steps). The update, ranges, HORIPML order-1 slab corrections, Hertzian dipoles and receivers
 * are the reference's (fields_updates_ext.pyx, pml_updates_*_HORIPML_ext.pyx order1_*,
 * sources.py:163-193, fields_outputs.py:40-67); H uses free-space coefficients. CA, CB,
 * traces and gradients are DEVICE pointers of the caller (e.g. torch tensors), laid out
 * [3][nx+1][ny+1][nz+1] (CA, CB, gradients) and [nrx][iterations] (traces). No counterpart in
 * the reference, which has no gradient path. */
typedef struct gbf_adj_desc {
    int32_t nx, ny, nz, iterations;
    float d;                     /* cubic cell size */
    float dt;
    float dbd;                   /* H curl coefficient DB/d (fp32) */
    float srcm;                  /* H PML coefficient DB (fp32) */
    int32_t pml_thickness[6];    /* x0, y0, z0, xmax, ymax, zmax; HORIPML order 1 */
    int32_t nsrc;                /* Hertzian dipoles, at most 16 */
    int32_t nrx;                 /* receivers, at least 1 */
    int32_t checkpoint_interval; /* steps between checkpoints; 0: ceil(sqrt(iterations));
                                    -1: the last segment as long as its recompute slots fit in
                                    60 % of the free device memory (all steps if they fit, when
                                    nothing is recomputed) and the steps before it in segments
                                    of ceil(sqrt(their count)). The forward leaves the last
                                    segment in the slots, so the first backward after it
                                    recomputes every segment but that one */
    int32_t reserved[3];         /* must be zero */
} gbf_adj_desc;
typedef struct gbf_adj gbf_adj;
int gbf_adj_create(const gbf_adj_desc* desc, gbf_adj** out);
void gbf_adj_destroy(gbf_adj* adj);
int gbf_adj_last_error(gbf_adj* adj, char* buf, size_t n);
/* rows: ERA ERB ERE ERF HRA HRB HRE HRF of the slab's CFS term, thickness values each */
int gbf_adj_upload_pml(gbf_adj* adj, int32_t slab, const float* const rows[8]);
/* info [nsrc][4]: component (0..2), i, j, k; scale [nsrc]: dl/(dx dy dz);
 * waves [nsrc][iterations]: the waveform at whole steps, zero where inactive */
int gbf_adj_upload_sources(gbf_adj* adj, const int32_t* info, const float* scale, const float* waves);
/* info [nrx][4]: component (0..2), i, j, k */
int gbf_adj_set_receivers(gbf_adj* adj, const int32_t* info);
/* run every iteration; writes traces and keeps the checkpoints for gbf_adj_backward */
int gbf_adj_forward(gbf_adj* adj, const float* CA, const float* CB, float* traces);
/* gCA, gCB (fp64, overwritten) = d(misfit)/d(CA, CB) given gtraces = d(misfit)/d(traces) */
int gbf_adj_backward(gbf_adj* adj, const float* CA, const float* CB, const float* gtraces,
                     double* gCA, double* gCB);
/* gbf_adj_backward with its fp32 per-segment partial sums in a fixed 16 MiB device array of
 * the library instead of the context's two buffers (which gbf_adj_create still allocates);
 * the call itself allocates no memory, for callers that must not allocate while they run (a
 * caller whose own allocator owns all device memory, or a time-critical loop). Same arguments
 * and results. Grids of more than 699,050 nodes per component ((nx+1)(ny+1)(nz+1)) are rejected
 * with GBF_EINVAL. The array exists on every device that loads the library, used or not. The
 * first call on a device looks up the array's address (setup; again after a device reset);
 * make it before any stream capture. All contexts on a device share the array: overlapping
 * calls, from two threads or two contexts, race on it and must be serialised by the caller; a
 * call returns only when it no longer uses the array, on failure too. No counterpart in the
 * reference. */
int gbf_adj_backward_static(gbf_adj* adj, const float* CA, const float* CB, const float* gtraces,
                            double* gCA, double* gCB);

/* 1 if, for this cell size, the PML kernels may form dF/d as the product with the rounded
 * reciprocal corrected once by the exact residual, because that equals the IEEE quotient for
 * every dF; 0 otherwise (the kernels then divide). Host only, no device needed; gbf_create
 * asks the same of each axis's cell size on the device (gbf_check_cell_division_device). No
 * counterpart in the reference, whose PML kernels
 * divide (pml_updates_electric_HORIPML_ext.pyx:80 `dHz = (...) / dx`). */
int gbf_check_cell_division(float d);

/* The same check on the current CUDA device, with the kernels' own operations (*exact = 1 or
 * 0); what gbf_create runs for each axis's cell size, in microseconds where the host loop of
 * gbf_check_cell_division takes about a millisecond. GBF_ECUDA without a device. */
int gbf_check_cell_division_device(float d, int32_t* exact);

/* The sweep boxes a half-step kernel walks for a grid (electric != 0: E half-step, domain
 * [0,nx) x [0,ny) x [0,nz); else H, domain [0,nx] x [0,ny] x [0,nz]): six rows of ten int32
 * (i0, j0, k0, bi, bj, bk, ksplit, kgap, start, count), box 0 the PML-free core. Host only, no
 * device needed; for checking the decomposition. No counterpart in the reference, whose kernels
 * loop over the whole domain and then over each slab (fields_updates_ext.pyx:30-110, pml.py). */
int gbf_sweep_boxes(int32_t nx, int32_t ny, int32_t nz, const int32_t thickness[6],
                    int32_t electric, int32_t* boxes);

/* ---- model geometry in device memory ------------------------------------------------
 * The solid, rigid and ID arrays of a grid (grid.py:157-169: solid and ID start as
 * free_space = 1, nothing rigid) built on the device by the geometry primitives, then the
 * per-edge IDs of the non-rigid edges from their neighbouring cells
 * (yee_cell_build_ext.pyx:110-257). A box is six int32: first cell (xs, ys, zs) and extent
 * (sx, sy, sz), inside the grid. Host arrays are C order with k fastest. Every call finishes its
 * device work before it returns. */
typedef struct gbf_geom gbf_geom;
int gbf_geom_create(int32_t nx, int32_t ny, int32_t nz, gbf_geom** out);
void gbf_geom_destroy(gbf_geom* geom);
int gbf_geom_last_error(gbf_geom* geom, char* buf, size_t n);
/* build_voxel (geometry_primitives_ext.pyx:314-377) on the cells of `box` where mask (uint8
 * [sx][sy][sz], NULL: every cell) is non-zero, with material numbers num = (numID, numIDx,
 * numIDy, numIDz); averaging != 0 only sets solid and clears the rigid flags. Replaces the cell
 * loops of build_sphere (:873-928) and build_cylinder (:692-871) once the host has selected
 * their cells. */
int gbf_geom_cells(gbf_geom* geom, const int32_t box[6], const uint8_t* mask, const uint32_t num[4],
                   int32_t averaging);
/* build_box (geometry_primitives_ext.pyx:618-691): the cells as gbf_geom_cells, the IDs over
 * the box's per-component node ranges (which differ from its cells' build_voxel edges). */
int gbf_geom_box(gbf_geom* geom, const int32_t box[6], const uint32_t num[4], int32_t averaging);
/* build_voxels_from_array (geometry_primitives_ext.pyx:934-980) for a block already clipped to
 * the grid: data int16 [sx][sy][sz], negative = leave the cell; cell material numexist + value.
 * Edges shared by cells of different materials keep the value of the last cell in (i, j, k)
 * order, as the reference's loop leaves them. */
int gbf_geom_voxels(gbf_geom* geom, const int32_t box[6], const int16_t* data, int32_t numexist,
                    int32_t averaging);
/* Rigid E edges with their material: recs int32 [n][5] = (component 0..2, i, j, k, numID), the
 * edge's cell inside the grid. Replaces the build_edge_x/y/z and build_face_* writes of #edge
 * and #plate (geometry_primitives_ext.pyx:30-312; set_rigid_Ex/Ey/Ez,
 * yee_cell_setget_rigid_ext.pyx:72-97). */
int gbf_geom_edges(gbf_geom* geom, int32_t n, const int32_t* recs);
/* build_electric_components (electric != 0) or build_magnetic_components: every non-rigid edge
 * whose neighbouring cells share one material takes it; the others are collected, in the
 * reference's loop order (components in order, i, j, k), with a key of their neighbours'
 * material numbers (E: four 16-bit numbers, first in the top bits; H: two), counts[3] per
 * component. Fetch the keys with gbf_geom_averaged_keys, resolve them to material numbers on the
 * host (create_electric_average / create_magnetic_average, yee_cell_build_ext.pyx:31-108) and
 * hand them back with gbf_geom_resolve. Material numbers must fit in 16 bits. */
int gbf_geom_components(gbf_geom* geom, int32_t electric, int64_t counts[3]);
int gbf_geom_averaged_keys(gbf_geom* geom, uint64_t* keys);
/* table: the distinct keys, strictly increasing; numbers: their material numbers */
int gbf_geom_resolve(gbf_geom* geom, int64_t m, const uint64_t* table, const uint32_t* numbers);
/* Fill or read a box of one array: 0 solid, 1 rigid flags (bits 0-11 rigidE[0..11], 12-17
 * rigidH[0..5]), 2 + c the IDs of component c (Ex..Hz; node boxes within [nx+1][ny+1][nz+1]).
 * out: uint32 [sx][sy][sz]. */
int gbf_geom_fill(gbf_geom* geom, int32_t array, const int32_t box[6], uint32_t value);
int gbf_geom_read(gbf_geom* geom, int32_t array, const int32_t box[6], uint32_t* out);
/* the largest material number in the ID array */
int gbf_geom_max_id(gbf_geom* geom, uint32_t* out);
/* gbf_upload_materials with the ID array of a geometry built on the same device (copied on the
 * device; the geometry can be destroyed afterwards). Every ID must be below nmat. */
int gbf_upload_materials_geom(gbf_ctx* ctx, gbf_geom* geom, const float* coeffE,
                              const float* coeffH, const float* coeffD);

#ifdef __cplusplus
}
#endif

#endif /* GBFDTD_H */
