/*
 * seis_gb300.h -- C ABI of the GB300 (sm_103a) 2-D acoustic finite-difference engine.
 *
 * The engine replaces the body of jcottaar/seismic's
 *     seis_forward2.vel_to_seis(vec, vec_diff=None, vec_adjoint=None,
 *                               adjoint_on_residual=False)
 * (core/seis_forward2.py:146-331) and the module state it keeps
 * (buffers and CUDA graphs, core/seis_forward2.py:13-17,102-144,163-176).
 *
 * Conventions
 *  - Every function returns 0 on success or a negative SEIS_E* status; the
 *    message of the last failure of an engine is in seis_last_error(engine)
 *    (seis_last_error(NULL) for failures of seis_create).
 *  - All array arguments of the compute calls are DEVICE pointers owned by the
 *    caller; the engine owns its workspace.  Calls are asynchronous on the
 *    given stream (cudaStream_t passed as void*; NULL = legacy default stream).
 *  - Vectors use the reference's layout: a model vector is nz*nx velocities
 *    (row-major, row = depth) followed by min_vel (core/kaggle_support.py:243-245);
 *    a record vector is [shot][t][receiver] (core/seis_forward2.py:249,320).
 *    Several models of the same geometry are laid end to end.
 *  - Inputs and outputs are FP64 like the reference; the sweeps compute in FP32;
 *    gradient and misfit reductions are FP64.
 *  - An engine serialises its own calls (internal mutex); use one engine per
 *    concurrent stream of work.
 */
#ifndef SEIS_GB300_H
#define SEIS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SEIS_OK 0
#define SEIS_E_INVALID -1     /* bad argument (null pointer, size, geometry) */
#define SEIS_E_CUDA -2        /* a CUDA call failed; the message names it */
#define SEIS_E_NOMEM -3       /* workspace does not fit in device memory */
#define SEIS_E_STATE -4       /* call order / engine state error */
#define SEIS_E_TIMEOUT -5     /* a bounded device-side wait gave up (see seis_device_status) */

/* Acquisition geometry.  Replaces the hard-coded module constants of
 * core/seis_forward2.py:69-101 (70x70 grid, dx=10, nbc=120, nt=999, dt=1 ms,
 * 15 Hz Ricker, 5 shots, 70 receivers).  Source and receiver positions are
 * PADDED-grid indices, as adjust_sr() produces them (core/seis_forward2.py:60-68). */
typedef struct SeisGeometry {
    int32_t nz, nx;          /* model grid: rows (depth) x columns */
    int32_t nbc;             /* absorbing-layer cells on every side (>= 2) */
    int32_t nt;              /* time steps = record rows */
    double dx;               /* grid spacing [m] */
    double dt;               /* time step [s] */
    double freq;             /* Ricker peak frequency [Hz] */
    int32_t nshots;
    const int32_t* src_z;    /* host arrays [nshots]: padded row / column of each source */
    const int32_t* src_x;
    int32_t nrec;
    const int32_t* rec_z;    /* host arrays [nrec]: padded row / column of each receiver */
    const int32_t* rec_x;
} SeisGeometry;

typedef struct SeisEngine SeisEngine;

/* Create an engine for one geometry and up to max_models models per call.
 * max_shots_per_chunk bounds how many shots sweep concurrently (and so the
 * workspace: about 4*(nt+12)*(nz+2nbc)*(nx+2nbc) bytes per shot when a
 * gradient is requested); 0 picks as many as 60% of the free device memory
 * holds (at most max_models * nshots).
 * Replaces the module-level set-up of core/seis_forward2.py:13-144. */
int seis_create(const SeisGeometry* geometry, int32_t max_models, int32_t max_shots_per_chunk,
                SeisEngine** engine_out);

/* Release the engine and all its device memory. */
int seis_destroy(SeisEngine* engine);

/* Message of the engine's last failure ("" if none); engine = NULL gives the
 * calling thread's last failure of a call without an engine (seis_create,
 * seis_forward_noalloc). */
const char* seis_last_error(const SeisEngine* engine);

/* result = F(vec); result_diff = J vec_diff (if vec_diff != NULL);
 * result_adjoint = J^T w (if vec_adjoint != NULL) with w = vec_adjoint, or
 * w = F(vec) - vec_adjoint when adjoint_on_residual != 0.
 * Shapes per model: vec, vec_diff, result_adjoint: nz*nx+1; vec_adjoint,
 * result, result_diff: nshots*nt*nrec.  result_diff must be non-NULL exactly
 * when vec_diff is, result_adjoint exactly when vec_adjoint is.
 * misfit (optional, double[nmodels]) receives sum((F(vec)-vec_adjoint)^2)
 * when vec_adjoint is given.
 * Each array may be device memory or host memory (pinned for the copies to
 * overlap the sweeps; pageable works, with blocking copies).  Host inputs are
 * staged on the device: vec_adjoint is uploaded on the engine's own copy stream
 * while the forward sweep runs; host records are downloaded chunk by chunk
 * while the adjoint sweep runs.  Every copy is ordered before the work that
 * follows the call on `stream`: synchronise the stream before reading host
 * outputs.
 * Replaces seis_forward2.vel_to_seis (core/seis_forward2.py:146-331). */
int seis_vel_to_seis(SeisEngine* engine, int32_t nmodels,
                     const double* vec, const double* vec_diff, const double* vec_adjoint,
                     int32_t adjoint_on_residual,
                     double* result, double* result_diff, double* result_adjoint,
                     double* misfit, void* stream);

/* Gauss-Newton matrix-vector product in one call: the records F(vec), the
 * tangent records J vec_diff (result_diff) and the gradient-shaped
 * J^T (J vec_diff) (result_adjoint), the adjoint sweep seeded with this call's
 * own tangent records.  The same as seis_vel_to_seis with vec_diff, followed by
 * a call with vec_adjoint = result_diff and adjoint_on_residual = 0, but one
 * forward sweep instead of two.  Shapes as for seis_vel_to_seis.  (No counterpart
 * in core/seis_forward2.py; it replaces the two vel_to_seis calls of each
 * Gauss-Newton matvec, core/seis_invert.py:84-87.)  Host arrays as for
 * seis_vel_to_seis. */
int seis_gn_matvec(SeisEngine* engine, int32_t nmodels, const double* vec, const double* vec_diff,
                   double* result, double* result_diff, double* result_adjoint, void* stream);

/* Cost and gradient (or records only) of several engines' batches -- models on
 * different geometries, the uneven batch -- with the tiled kernels as ONE
 * persistent wavefront launch for all their forward sweeps and one for all their
 * reverse sweeps (per round of chunks: round r sweeps chunk r of every engine that
 * has one, so one round when every engine's models fit its slots).  For engine i:
 * nmodels[i] models, device arrays vec[i] [nmodels][nv], result[i]
 * [nmodels][nshots][nt][nrec], and with vec_adjoint (the arrays of targets, or of
 * weights, per engine; NULL for records only) result_adjoint[i] [nmodels][nv] and
 * optionally misfit[i] [nmodels].  Each engine's own options hold (its
 * "checkpoint_every", "wave_group_slots"); results are bitwise those of
 * seis_vel_to_seis on each engine alone.  Engines must be distinct; all work on
 * `stream`; a bounded wait that gives up sets bit 8 of every engine's error word
 * (seis_device_status).  No counterpart in core/seis_forward2.py, which sweeps
 * one geometry per call (:146-331).  Errors: seis_last_error(NULL). */
int seis_vel_to_seis_multi(int32_t n, SeisEngine* const* engines, const int32_t* nmodels,
                           const double* const* vec, const double* const* vec_adjoint,
                           int32_t adjoint_on_residual, double* const* result,
                           double* const* result_adjoint, double* const* misfit, void* stream);

/* Kernel launches issued by this engine since creation (graph nodes counted
 * one by one), and the device time of the last call's sweeps in ms
 * (forward/tangent sweep, adjoint sweep), measured with CUDA events on the
 * call's stream; valid once that stream has been synchronised. */
int seis_stats(const SeisEngine* engine, int64_t* launches, double* fwd_ms, double* adj_ms,
               int64_t* fwd_step_launches, int64_t* adj_step_launches);

/* Number of shot slots the engine sweeps concurrently (its chunk size). */
int seis_chunk_slots(const SeisEngine* engine);

/* Engine options.  "sweep_path": 0 = automatic (cluster-resident sweeps where the
 * geometry fits on chip, tiled per-step sweeps otherwise), 1 = tiled per-step
 * sweeps only, 2 = cluster sweeps (SEIS_E_INVALID when they do not apply),
 * 3 = the tiled kernels as one persistent wavefront launch per sweep (work items
 * of (stage, shot slot, tile) that wait, bounded, for their neighbour tiles'
 * previous stage; results bitwise those of 1).  "wave_group_slots": shot slots
 * whose stages advance together in the wavefront sweeps, 0 (default) = as many
 * as give each stage twice the resident blocks' worth of tiles.
 * "checkpoint_every": k > 0 keeps the forward wavefield only every k steps
 * (p and u, 2*ceil(nt/k) levels instead of nt+1) and recomputes each segment
 * before its adjoint steps (one extra forward sweep; tiled sweeps); 0 = keep
 * the whole increment history.  Results do not depend on k.
 * "fwd_cluster": CTAs per cluster of the cluster forward sweep, 8 (39- or
 * 40-row bands, 15 resident clusters on GB300), 10 (32-row bands, 13 resident)
 * or 16 (20-row bands, 7 resident): larger clusters finish one shot sooner,
 * smaller ones sweep more shots at once.  0 (default) picks the size whose
 * clusters cover the most SMs with the engine's chunk of shots (16 for up to
 * 11 shots, 10 above).  Results are bitwise the same.
 * "columns": grid columns per thread of the cluster sweeps, 2 (default; used
 * where the padded width is even) or 1.  Results are bitwise the same.
 * "adj_cluster": CTAs per cluster of the cluster adjoint sweep: 10 (32-row bands;
 * alpha, the gradient sums and the carried history level in tensor memory; 13
 * resident clusters on GB300) or 16 (20-row bands, all in registers and shared
 * memory; 7 resident); 0 (default) picks the shape whose resident clusters cover
 * the most SMs with the engine's chunk of shots.  "adj_rows": rows per thread of
 * the 10-CTA adjoint, 8 (640 threads, default) or 11 (480 threads).  Results are
 * bitwise the same.
 * "fwd_tmem": 1 (default) keeps the band's alpha of the 10-CTA column-pair
 * forward sweep in tensor memory, 0 in shared memory.  Results are bitwise the same.
 * "neighbour_shuffle": 1 makes the 10-CTA column-pair forward sweep take the
 * horizontal neighbours from the adjacent lanes by warp shuffles instead of
 * shared-memory loads (0, default).  Results are bitwise the same.
 * "adj_side" / "fwd_side": slots of each chunk whose adjoint / forward (or
 * tangent) sweep runs on the tiled kernels beside the cluster sweep, on the
 * SMs its clusters leave free (the cluster part then takes whole rounds of its
 * resident clusters); -1 (default) = automatic (sized per chunk on its own
 * shot count from the free SMs and the kernels' measured throughputs; none
 * for small chunks), 0 = none, n > 0 = the last n slots of every chunk.
 * Results are bitwise the same.
 * "fwd_side_cluster": where the forward's side slots run: -1 (default)
 * automatic -- two concurrent 8-CTA cluster sweeps on the SMs that 10-CTA main
 * clusters leave free (at least 16), else the tiled kernels; 0 the tiled
 * kernels; 8, 10 or 16 clusters of that size ("fwd_side_clusters" of them,
 * default 2).  The tangent's side slots always run tiled.  Results are bitwise
 * the same.
 * "fwd_fuse" / "adj_fuse": 1 (default) lets the tiled forward (without
 * tangent) / adjoint sweep take two time steps per launch where the padded
 * grid is even-wide and at least 72 x 40; 0 = one step per launch.  Results
 * are bitwise the same.
 * "adj_hoist": 1, 2 or 4 (default) rows of a thread whose history and
 * gradient-sum loads the two-step tiled adjoint issues together, before the
 * rows' stores.  Results are bitwise the same.
 * "test_skip_history_copy": test hook for the device-side failure path -- the
 * cluster adjoint never copies this history level, so its bounded wait gives
 * up after about 2 s and seis_device_status returns SEIS_E_TIMEOUT (the call's
 * results are then invalid; the engine stays usable); -1 = off (default). */
int seis_set_option(SeisEngine* engine, const char* key, int64_t value);

/* Read-only facts: "cluster_fwd" / "cluster_adj" (concurrently resident
 * clusters of the cluster sweeps, 0 when they do not apply), "sweep_path",
 * "slots", "tiles" (64 x 32 tiles of one shot of the tiled sweeps), "fwd_cluster",
 * "cluster_fwd10" / "cluster_fwd16" (resident 10- and 16-CTA forward clusters),
 * "fwd_columns" / "adj_columns" (columns per thread of the cluster sweeps in use),
 * "fwd_shuffle" (1 when the forward in use takes its neighbours by shuffles),
 * "fwd_tmem" (1 when it keeps alpha in tensor memory),
 * "adj_cluster" / "adj_tmem" (CTAs per cluster of the adjoint in use, and 1 when it
 * keeps its per-point state in tensor memory),
 * and of the last call: "last_fwd_launches" / "last_adj_launches"
 * (sweep kernel launches), "last_fwd_path" / "last_adj_path" (1 tiled
 * per-step sweeps, 2 cluster sweeps, 3 wavefront sweeps, 0 not run), "last_adj_side" /
 * "last_fwd_side" (active slots that ran the side adjoint / forward),
 * "fwd_side_cluster" (CTAs per side cluster of the forward in use, 0 tiled),
 * "last_adj_cluster_ns" (device time of
 * the last call's cluster adjoint launches; synchronise the call's stream
 * first), "adj_side" / "fwd_side" (the options), "err_word" (host mirror of
 * the sticky device error word, see seis_device_status; read without a sync). */
int seis_get_info(const SeisEngine* engine, const char* key, int64_t* value);

/* Wait for the engine's last call and report device-side failures of its
 * sweeps: SEIS_E_TIMEOUT when a bounded wait gave up in any call since the
 * previous report (the device error word is sticky across calls, so a later
 * call does not hide an earlier failure; reporting clears it), else 0.
 * Without a sync, seis_get_info(engine, "err_word", &w) reads the word's host
 * mirror, which every call updates in stream order at its end: once the
 * caller has synchronised the call's stream for its own reasons, w != 0 means
 * a failure is pending and seis_device_status will report it. */
int seis_device_status(SeisEngine* engine);

/* L-BFGS search directions d = -H g of nprob independent problems by the
 * two-loop recursion over the first num_old[p] stored pairs (s_i, y_i), FP64.
 * Replaces the reference's lbfgs_backward / lbfgs_forward kernels and their
 * torch wrappers (core/seis_numerics.py:450-639), batched over problems.
 * Device arrays: num_old [nprob] (int32), old_stps / old_dirs
 * [nprob][m_cap][n], ro / al [nprob][m_cap] (al written), grad / d
 * [nprob][n], h_diag [nprob].  Errors: seis_last_error(NULL). */
int seis_lbfgs_direction(int32_t nprob, int32_t n, int32_t m_cap, const int32_t* num_old,
                         const double* old_stps, const double* old_dirs, const double* ro, double* al,
                         const double* grad, const double* h_diag, double* d, void* stream);

/* Fixed-order FP64 block reductions of nprob vectors of n (one block each):
 * op 0 out[p] = <a_p, b_p>, 1 out[p] = sum |a_p|, 2 out[p] = max |a_p|.  The
 * device-resident optimiser uses the same reductions, so a host-driven L-BFGS
 * that calls this gets the same bits.  Device arrays.  Errors: seis_last_error(NULL). */
int seis_reduce(int32_t nprob, int32_t n, int32_t op, const double* a, const double* b, double* out, void* stream);

/* Device-resident L-BFGS with a strong-Wolfe line search (the reference's bfgs and
 * _strong_wolfe, core/seis_numerics.py:138-277 and 307-448, lr 1, c1 1e-4, c2 0.9,
 * line-search tolerance 1e-9, 25 line-search evaluations) for nprob independent
 * problems of n unknowns, as a state machine: no host read per evaluation (the
 * reference reads f, g.d and norms back at :155,162,169,324).  `state` holds
 * nprob * seis_lbfgs_state_bytes(n, max_iter) bytes of device memory (256-byte
 * aligned).  With x0 [nprob][n] (f, g ignored) a call initialises every problem:
 * x_eval = x0, done = 0.  Otherwise f [nprob] and g [nprob][n] are the objective
 * and gradient at the current x_eval, and each problem's optimiser runs to its
 * next point to evaluate (written to x_eval) or to its end (x_eval = the final
 * point, done[p] = 1; later calls leave it).  Device arrays; one launch on
 * `stream`.  Errors: seis_last_error(NULL). */
int64_t seis_lbfgs_state_bytes(int32_t n, int32_t max_iter);
int seis_lbfgs_step(int32_t nprob, int32_t n, int32_t max_iter, double tolerance_grad, double tolerance_change,
                    const double* x0, const double* f, const double* g, void* state, double* x_eval,
                    int32_t* done, void* stream);

/* Smoothed total-variation prior of m models (nz x nx grid), fused cost and
 * gradient: cost[i] = lam * mean(sqrt(d^2 + epsilon^2)) over the vertical and
 * horizontal neighbour differences d of model i, grad[i] its gradient (0 for
 * the min_vel entry).  Replaces TotalVariation._compute_cost_and_gradient
 * (core/seis_prior.py:135-177) for any grid; one block per model, so each
 * model's result is independent of m.  Device arrays: x, grad [m][nz*nx+1],
 * cost [m].  Errors: seis_last_error(NULL). */
int seis_tv_prior(int32_t m, int32_t nz, int32_t nx, double epsilon, double lam, const double* x, double* cost,
                  double* grad, void* stream);

/* Size of the fixed device workspace of seis_forward_noalloc: 8 MiB.  A
 * geometry needs 24 bytes per padded point at the row pitch (NZ x pitch, pitch
 * = NX rounded up to 32 columns: alpha, three p levels, two u levels), 4*nt*nrec
 * bytes of FP32 records and a few KB of constants -- about 330k padded points at
 * nt = 1000 with 70 receivers; 200x300 models with nbc = 120 (440 x 544) fit up
 * to nt = 2000 with 300 receivers. */
#define SEIS_NOALLOC_SCRATCH_BYTES ((size_t)8 << 20)
/* Limits of the geometry constants seis_forward_noalloc passes by value. */
#define SEIS_NOALLOC_MAX_SHOTS 64
#define SEIS_NOALLOC_MAX_RECEIVERS 1024
#define SEIS_NOALLOC_MAX_NBC 512
#define SEIS_NOALLOC_MAX_WAVELET 1536   /* Ricker samples 2*(int(2.2/freq/dt)/2)+1 */

/* Records of ONE model without allocating device memory.  No counterpart in
 * the reference: it is for callers that cannot call cudaMalloc after start-up
 * (hosts whose allocator has already reserved the device's memory, latency-
 * critical loops that may not take cudaMalloc's implicit synchronisation,
 * plugin hosts that forbid allocation in their callbacks).
 * vec: double[nz*nx+1], result: double[nshots*nt*nrec], both device memory of
 * the current device (other pointers are rejected with SEIS_E_INVALID); the
 * records equal those of seis_vel_to_seis for the same inputs.  The workspace
 * is a static device array of SEIS_NOALLOC_SCRATCH_BYTES that every GPU
 * loading the library holds until exit; geometries that need more, or exceed
 * the SEIS_NOALLOC_MAX_* limits, are rejected with SEIS_E_INVALID.  The first
 * call on a device looks up the array's device address, so make it before any
 * stream capture.  All calls share the array: calls whose work overlaps on the
 * GPU race and must be ordered by the caller.  Errors: seis_last_error(NULL). */
int seis_forward_noalloc(const SeisGeometry* geometry, const double* vec, double* result, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SEIS_GB300_H */
