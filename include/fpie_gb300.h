/*
 * fpie_gb300 -- C ABI of the GB300 Jacobi Poisson solver backend for fpie.
 *
 * The reference binds its native solvers to Python with pybind11 classes
 * (fpie/core/cuda/solver.cc:3-15): EquSolver(block_size) with
 * partition/reset/sync/step and GridSolver(grid_x, grid_y) with
 * reset/sync/step, on top of the base classes in fpie/core/base_solver.h.
 * This header is the same surface as plain C: an opaque solver handle, host
 * pointers and sizes, an int status (0 = success) and a thread-local error
 * message.  Arrays are C-contiguous in the layouts the reference uses:
 *   grid mask  int32[n][m],  grid tgt/grad float32[n][m][3],
 *   equ A      int32[N][4],  equ X/B       float32[N][3],
 *   images     uint8, same shape as the state they come from.
 * Every CUDA error is checked and reported through the status; nothing falls
 * back to the CPU.
 */
#ifndef FPIE_GB300_H_
#define FPIE_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fpie_solver fpie_solver;

enum fpie_status {
  FPIE_OK = 0,
  FPIE_ERR_ARG = 1,      /* invalid argument (shape, index, null pointer) */
  FPIE_ERR_CUDA = 2,     /* a CUDA runtime call failed */
  FPIE_ERR_STATE = 3,    /* call not valid in the solver's current state */
  FPIE_ERR_TIMEOUT = 4,  /* a bounded device-side wait gave up */
};

/* Precision of the sweep state (the mixed forms keep an FP32 solution and
 * solve for an FP16 / BF16 correction by iterative refinement). */
enum fpie_precision { FPIE_FP32 = 0, FPIE_MIXED_FP16 = 1, FPIE_MIXED_BF16 = 2 };

/* Iteration order of an EquSolver (fpie_equ_set_order).
 * FPIE_ORDER_JACOBI: every sweep reads the previous sweep's values -- the
 *   numpy EquSolver (fpie/np_solver.py:33-41); partition numbers unknowns
 *   row-major.
 * FPIE_ORDER_RED_BLACK: the reference's OpenMP EquSolver -- partition
 *   numbers the cells with odd row + col first, then the even ones
 *   (fpie/core/openmp/equ.cc:22-56); a sweep updates unknowns 1..n_mid-1 in
 *   place, then n_mid..N-1 reading the new values (openmp/equ.cc:107-118). */
enum fpie_order { FPIE_ORDER_JACOBI = 0, FPIE_ORDER_RED_BLACK = 1 };

/* Library version as 10000*major + 100*minor + patch. */
int fpie_version(void);

/* Message of the last failed call on this thread ("" if none). */
const char* fpie_last_error(void);

/* Number of visible CUDA devices (0 is not an error). */
int fpie_device_count(int* count);

/* ---- EquSolver: fpie/core/base_solver.h:12-75, fpie/core/cuda/equ.cu ---- */

/* Replaces CudaEquSolver(block_size) (fpie/core/cuda/equ.cu:7-17).
 * block_size is the sweep kernel's block size when it is a multiple of 32
 * in [32,1024]; otherwise the backend's default is used. */
int fpie_equ_create(int block_size, fpie_solver** out);

/* Replaces EquSolver.partition (fpie/core/cuda/equ.cu:36-54,
 * fpie/np_solver.py:14-16): ids[i][j] = row-major running count of
 * mask > 0 at set pixels, 0 elsewhere.  In FPIE_ORDER_RED_BLACK it replaces
 * OpenMPEquSolver::partition (fpie/core/openmp/equ.cc:22-56): the count runs
 * over cells with odd i + j first, then even ones, and the solver keeps
 * n_mid = the first even id for its sweeps. */
int fpie_equ_partition(fpie_solver* s, const int32_t* mask, int n, int m,
                       int32_t* ids_out);

/* Selects the iteration order (enum fpie_order; default Jacobi).  A change
 * discards the loaded system: call partition and reset again.  In red-black
 * order reset checks that every unknown's neighbours have the other colour
 * for the last partition's n_mid (FPIE_ERR_ARG if not, FPIE_ERR_STATE if no
 * partition was made), and fpie_equ_reset_images numbers the unknowns as
 * the red-black partition does (n_mid from its own count). */
int fpie_equ_set_order(fpie_solver* s, int order);

/* The current order and, if n_mid is not NULL, the last red-black
 * partition's n_mid (0 if none). */
int fpie_equ_order(fpie_solver* s, int* order, int* n_mid);

/* Replaces EquSolver.reset (fpie/core/base_solver.h:27-59 and
 * CudaEquSolver::post_reset, fpie/core/cuda/equ.cu:56-74).  Copies the
 * inputs; every A entry must lie in [0, N). */
int fpie_equ_reset(fpie_solver* s, int N, const int32_t* A, const float* X,
                   const float* B);

/* fpie_equ_reset with the caller's placement of the unknowns on a grid:
 * pos int32[N] (pos[0] ignored) = row * m + col of unknown i in an n x m
 * crop, every unknown off the crop's 1-pixel frame -- what EquProcessor
 * knows from its mask (fpie/process.py:180-190, 219-225).  The placement is checked
 * on the device (each unknown alone on its pixel, its four grid neighbours
 * exactly its A entries, row 0 the zero constant, in red-black order the
 * colour parity) instead of being searched for on the host; FPIE_ERR_ARG if
 * it does not fit.  Results are those of fpie_equ_reset. */
int fpie_equ_reset_placed(fpie_solver* s, int N, const int32_t* A, const float* X,
                          const float* B, const int32_t* pos, int n, int m);

/* Replaces EquSolver.step (fpie/core/cuda/equ.cu:189-211,
 * fpie/core/openmp/equ.cc:107-125): runs `iteration` sweeps (Jacobi, or
 * red-black in that order) continuing from the current state, then writes
 * the clipped uint8 state x_out[N][3] and the per-channel sum of |residual|
 * err_out[3]. */
int fpie_equ_step(fpie_solver* s, int iteration, uint8_t* x_out,
                  float* err_out);

/* ---- GridSolver: fpie/core/base_solver.h:77-152, fpie/core/cuda/grid.cu -- */

/* Replaces CudaGridSolver(grid_x, grid_y) (fpie/core/cuda/grid.cu:7-17).
 * grid_x/grid_y are accepted for interface compatibility; tile shapes are
 * chosen by the backend. */
int fpie_grid_create(int grid_x, int grid_y, fpie_solver** out);

/* Replaces GridSolver.reset (fpie/core/base_solver.h:101-140 and
 * CudaGridSolver::post_reset, fpie/core/cuda/grid.cu:33-52).  N is the
 * caller's unknown count (bookkeeping only, as in the reference); the grid
 * is n x m. */
int fpie_grid_reset(fpie_solver* s, int N, int n, int m, const int32_t* mask,
                    const float* tgt, const float* grad);

/* Replaces GridSolver.step (fpie/core/cuda/grid.cu:133-153): img_out is
 * uint8[n][m][3]. */
int fpie_grid_step(fpie_solver* s, int iteration, uint8_t* img_out,
                   float* err_out);

/* ---- shared ------------------------------------------------------------ */

/* Replaces EquSolver.sync / GridSolver.sync (fpie/core/base_solver.h:61,142),
 * a no-op there; here it waits for the solver's stream. */
int fpie_sync(fpie_solver* s);

/* Frees the solver and its device memory (the pybind object's destructor). */
int fpie_destroy(fpie_solver* s);

/* Runs later calls of this solver on `stream`, a cudaStream_t used as given:
 * NULL is the CUDA legacy default stream (torch's default stream).  Until
 * this is called a solver uses a private non-blocking stream.  Lets a caller
 * order the solver's work with its own (e.g. torch CUDA events). */
int fpie_set_stream(fpie_solver* s, void* stream);

/* Selects the sweep precision (default FPIE_FP32).  Takes effect at the
 * next step; the FP32 solution is kept across changes.  The mixed forms
 * (grid solvers only) run each step as cycles of 64 inner Jacobi sweeps on
 * a correction stored in FP16 / BF16 (FP32 arithmetic), each cycle
 * followed by x += e and a fresh FP32 residual; results equal FP32 Jacobi
 * up to the correction's rounding, not bit for bit. */
int fpie_set_precision(fpie_solver* s, int precision);

/* ---- device-resident forms (torch tensor handoff; no host copies) --------
 * Same meaning as the calls above, with all array pointers in device memory
 * of the solver's device.  The *_device step calls only enqueue work on the
 * solver's stream; img/err may be NULL to skip those outputs. */
int fpie_grid_reset_device(fpie_solver* s, int n, int m, const int32_t* mask,
                           const float* tgt, const float* grad);
int fpie_grid_step_device(fpie_solver* s, int iteration, uint8_t* img,
                          float* err);
int fpie_equ_reset_device(fpie_solver* s, int N, const int32_t* A,
                          const float* X, const float* B);
int fpie_equ_step_device(fpie_solver* s, int iteration, uint8_t* x,
                         float* err);

/* GPU-side counterpart of GridProcessor.reset (fpie/process.py:321-386):
 * builds the grid inputs from the uint8 images -- src [src_h][src_w][3],
 * mask [mask_h][mask_w][mask_channels] (1 or 3), tgt [tgt_h][tgt_w][3] --
 * the mask's placement (src_row, src_col) on the source and (tgt_row,
 * tgt_col) on the target, and gradient 0 = 'src', 1 = 'avg', 2 = 'max'.
 * Bit-identical to the host construction.  on_device != 0: the pointers are
 * device memory (nothing is copied from the host).  box receives the crop on
 * the target: row0, row1, col0, col1 (end-exclusive).  Errors: a mask with no
 * set pixel, or a crop leaving either image (FPIE_ERR_ARG). */
int fpie_grid_reset_images(fpie_solver* s, const uint8_t* src, int src_h, int src_w,
                           const uint8_t* mask, int mask_h, int mask_w, int mask_channels,
                           const uint8_t* tgt, int tgt_h, int tgt_w, int src_row, int src_col,
                           int tgt_row, int tgt_col, int gradient, int on_device, int* box);

/* GPU-side counterpart of EquProcessor.reset (fpie/process.py:192-271):
 * partition (row-major ids of the set pixels, by a prefix scan), A, X, B,
 * with the same images, offsets and gradient codes as
 * fpie_grid_reset_images; bit-identical to the host construction.  N_out
 * receives the unknown count (set pixels + 1); box the crop on the target. */
int fpie_equ_reset_images(fpie_solver* s, const uint8_t* src, int src_h, int src_w,
                          const uint8_t* mask, int mask_h, int mask_w, int mask_channels,
                          const uint8_t* tgt, int tgt_h, int tgt_w, int src_row, int src_col,
                          int tgt_row, int tgt_col, int gradient, int on_device, int* box,
                          int* N_out);

/* Target-image coordinates of unknowns 1..N-1 after fpie_equ_reset_images
 * (the processor's tgt_index, fpie/process.py:269): rows, cols int32[N-1]. */
int fpie_equ_get_index(fpie_solver* s, int32_t* rows, int32_t* cols);

/* Copies the equation inputs the solver holds: A int32[N][4], B
 * float32[N][3]. */
int fpie_equ_get_inputs(fpie_solver* s, int32_t* A, float* B);

/* How the EquSolver sweeps (reference: the equation sweep of
 * fpie/core/cuda/equ.cu:76-96 and fpie/np_solver.py:33-41).  "auto"
 * (default): a system that is a 4-neighbour raster stencil -- the ones
 * EquProcessor builds from a mask (fpie/process.py:252-266), row 0 constant
 * and zero -- is placed on a grid and swept by the grid kernels (temporally
 * blocked, autotuned; same operations in the same order, so bit-identical
 * results), any other system by the gather kernel.  "gather": always the
 * gather kernel.  A grid kernel name (see fpie_grid_set_kernel): grid
 * placement with that kernel, FPIE_ERR_ARG at reset if the system is not a
 * raster stencil.  Applies from the next reset. */
int fpie_equ_set_kernel(fpie_solver* s, const char* name);

/* Writes "gather", "grid:<grid kernel>" or, in red-black order on the
 * equation kernels, "red_black" (NUL-terminated) into buf.  The red-black
 * grid kernels are "rb16w8k8" (8 red-black sweeps per launch) and
 * "rb16w8k8d" (the whole step in one dependency-flow launch); in red-black
 * order fpie_equ_set_kernel accepts "auto", "gather" and these two. */
int fpie_equ_kernel(fpie_solver* s, char* buf, int len);

/* Spin limit of the grid kernels' bounded waits in grid placement (see
 * fpie_grid_set_spin_limit). */
int fpie_equ_set_spin_limit(fpie_solver* s, long long spins);

/* Host-only: whether A (int32[N][4]: up, down, left, right; 0 = the
 * constant row 0) is a 4-neighbour raster stencil, and if so a placement:
 * pos int32[N] (pos[0] = -1; pos[i] = row * m + col of unknown i in an n x m
 * crop with a 1-pixel frame, connected components one below the other, a
 * row apart).  FPIE_OK if it is, FPIE_ERR_ARG if not.  No GPU needed. */
int fpie_equ_raster_layout(int N, const int32_t* A, int32_t* pos, int* n, int* m);

/* Copies the grid inputs the solver holds (mask int32[n][m], grad
 * float32[n][m][3]) to host memory. */
int fpie_grid_get_inputs(fpie_solver* s, int32_t* mask_out, float* grad_out);

/* Only the sweeps of a step (no residual, no image); for timing the sweep
 * kernels on their own. */
int fpie_sweeps(fpie_solver* s, int iteration);

/* Copies the current FP32 state, in the reference layout ([n][m][3] or
 * [N][3]), to host memory: the unclipped values the numpy backend keeps. */
int fpie_get_state(fpie_solver* s, float* out);

/* Per-channel norms of the current state's residual r = grad + sum of
 * neighbours - 4x over masked pixels (grid solvers): out[0..2] = max |r|,
 * out[3..5] = sum |r|, reduced in FP64 on the GPU.  Synchronizes. */
int fpie_residual_norms(fpie_solver* s, double* out);

/* Grid solvers: sweeps in blocks of check_every until every channel's
 * max |r| <= tol, or max_sweeps are done; *sweeps_done (may be NULL)
 * receives the count.  Works in every precision; for the mixed forms
 * check_every is best a multiple of 64 (one refinement cycle).  No
 * counterpart in the reference, whose step() always runs a fixed count. */
int fpie_grid_solve(fpie_solver* s, double tol, int max_sweeps, int check_every,
                    int* sweeps_done);

/* Selects the grid sweep kernel by name: "auto" (default: the autotuner
 * times the candidates on the first long step and keeps the fastest for this
 * grid shape), "sweep1" (one sweep per launch), a packed temporally
 * blocked variant "p16w8k16", "p8w16k16" or "p16w8k8" (R rows per thread, W
 * warps, K sweeps per launch), "p16w8k16d" (the whole step in one
 * cooperative launch, items started by neighbourhood dependencies, levels
 * of 16 sweeps on 96x96 tiles), "p16w8k12d" (the same with levels of 12
 * sweeps on 104x104 tiles; FP32 Jacobi only), "p16w8k16dp" / "p16w8k12dp"
 * (the same two with selects only at the unmasked pixels next to masked
 * ones where a region's mask edge is straight; FP32 Jacobi only) or
 * "p16w8k16t" (persistent CTAs prefetching each region by TMA).  Every
 * choice gives bit-identical results. */
int fpie_grid_set_kernel(fpie_solver* s, const char* name);

/* The dependency-flow kernels ("p16w8k16d", "p16w8k12d" and their "dp"
 * forms) wait for neighbour tiles to finish the previous level, the TMA
 * kernel ("p16w8k16t") for its region copies; each wait gives up after
 * `spins` polls (~64 ns apart), and the step (or fpie_sync) then returns
 * FPIE_ERR_TIMEOUT, leaving the state undefined.  Default 2^26. */
int fpie_grid_set_spin_limit(fpie_solver* s, long long spins);

/* Writes the current grid sweep kernel's name (NUL-terminated) into buf. */
int fpie_grid_kernel(fpie_solver* s, char* buf, int len);

/* ---- allocation-free grid step ---------------------------------------------
 * No counterpart in the reference: an addition for callers that cannot
 * allocate device memory where they need a step -- hosts whose device
 * memory is owned by their own pool allocator (a cudaMalloc behind its back
 * breaks its accounting), and loops where cudaMalloc/cudaFree's possible
 * device synchronization is not acceptable.
 *
 * Runs `iteration` Jacobi sweeps of a grid given in the reference layout,
 * all pointers in device memory of the calling thread's current device:
 * mask int32[n][m]; x float32[n][m][3], the state, updated in place; grad
 * float32[n][m][3].  Then, if non-NULL, writes the clipped image
 * img uint8[n][m][3] and the per-channel sum of |residual| err float32[3].
 * Work is enqueued on `stream` (NULL = legacy default stream).  The state
 * and the image are bit-identical to GridSolver's after the same sweeps;
 * err is the same per-pixel |residual| summed in double in another fixed
 * order, so it agrees to float rounding (rtol 1e-5 in the tests).
 *
 * Limit: n*m <= 262,144 pixels (e.g. 512 x 512); larger grids are rejected
 * with FPIE_ERR_ARG.  The second state buffer and the residual partials
 * live in a fixed 3 MiB array in the library's device image, held on every
 * GPU that loads the library until the process exits.  The first call on
 * a device resolves that array's address and loads the kernels; make it
 * before any stream capture.  Calls share the array, so calls whose GPU work
 * may overlap (other streams or threads) must be serialized by the caller.
 * The resolved address is kept per device for the life of the process: do
 * not call this across a cudaDeviceReset of that device.
 * Nothing here calls cudaMalloc, cudaFree or an allocating library routine. */
int fpie_grid_step_noalloc(int n, int m, const int32_t* mask, float* x,
                           const float* grad, int iteration, uint8_t* img,
                           float* err, void* stream);

/* ---- batched form: many uneven grid jobs in one persistent launch --------
 * No counterpart in the reference (which solves one paste per process).
 * A batch owns device memory for its jobs up to `budget_bytes`; each job is
 * a grid problem in the GridSolver layouts plus its own sweep count.
 * fpie_batch_run advances every job by min(max_sweeps, its remaining
 * sweeps) (max_sweeps < 0: to completion) in one persistent kernel whose
 * CTAs pull (job, tile, channel, level) items from a queue; the first run
 * with enough work autotunes the tile shape and temporal depth on real
 * sweeps.  A job's result is bit-identical to a GridSolver run of the same
 * sweeps.  Dependency waits inside the kernel are bounded: past the spin
 * limit the call returns FPIE_ERR_TIMEOUT and the jobs' states are
 * undefined (remove and re-add them). */
typedef struct fpie_batch fpie_batch;
int fpie_batch_create(double budget_bytes, fpie_batch** out);
int fpie_batch_destroy(fpie_batch* b);
/* Device bytes a job of an n x m grid holds (for admission decisions). */
int fpie_batch_job_bytes(int n, int m, double* bytes);
/* Same for this batch's precision (the mixed forms also hold the correction
 * and residual planes). */
int fpie_batch_job_bytes_for(fpie_batch* b, int n, int m, double* bytes);
/* FPIE_FP32 (default) or a mixed form; only before the first job is added.
 * In the mixed forms every 64 sweeps of a job are 64 correction sweeps
 * followed by a fold and an FP32 residual, as in fpie_set_precision. */
int fpie_batch_set_precision(fpie_batch* b, int precision);
/* Copies the job's inputs (host arrays, layouts as fpie_grid_reset); fails
 * with FPIE_ERR_STATE when the budget has no room.  *job_id receives the
 * slot, reused after fpie_batch_remove. */
int fpie_batch_add(fpie_batch* b, int n, int m, const int32_t* mask,
                   const float* tgt, const float* grad, int iterations,
                   int* job_id);
/* A job from the three uint8 images and the offsets, as
 * fpie_grid_reset_images builds a grid solver's inputs (GridProcessor.reset,
 * fpie/process.py:321-386): the mask is thresholded and its frame cleared
 * on the host, the crop's gradient mixing and layout are built on the
 * device.  The copies run on a second stream, so adding a job does not wait
 * for a run in flight (only for its own copies: the caller's arrays may be
 * reused on return); the job joins the next run.  box (may be NULL)
 * receives the crop on the target: row0, row1, col0, col1. */
int fpie_batch_add_images(fpie_batch* b, const uint8_t* src, int src_h, int src_w,
                          const uint8_t* mask, int mask_h, int mask_w, int mask_channels,
                          const uint8_t* tgt, int tgt_h, int tgt_w, int src_row, int src_col,
                          int tgt_row, int tgt_col, int gradient, int iterations, int* job_id,
                          int* box);
int fpie_batch_run(fpie_batch* b, int max_sweeps);
/* fpie_batch_run without waiting for the launch (the first run with enough
 * work still tunes synchronously); fpie_batch_wait waits for all queued work
 * and reports a dependency wait that exceeded its limit (FPIE_ERR_TIMEOUT).
 * Jobs added or removed meanwhile take effect in stream order. */
int fpie_batch_run_async(fpie_batch* b, int max_sweeps);
int fpie_batch_wait(fpie_batch* b);
/* fpie_batch_norms split in two: queue the norms of `count` jobs (after the
 * work already queued) and one copy of them to pinned host memory; then wait
 * for that copy only and receive them (6 doubles per job, as
 * fpie_batch_norms). */
int fpie_batch_norms_async(fpie_batch* b, const int* jobs, int count);
int fpie_batch_norms_wait(fpie_batch* b, double* out);
int fpie_batch_progress(fpie_batch* b, int job, int* done, int* total);
/* Clipped uint8 image [n][m][3] and per-channel sum |residual| of a job. */
int fpie_batch_result(fpie_batch* b, int job, uint8_t* img, float* err);
int fpie_batch_state(fpie_batch* b, int job, float* out);
/* FP64 residual norms of `count` jobs: out[6k..6k+2] = max |r| per channel,
 * out[6k+3..6k+5] = sum |r|, for jobs[k]'s current state. */
int fpie_batch_norms(fpie_batch* b, const int* jobs, int count, double* out);
int fpie_batch_remove(fpie_batch* b, int job);
int fpie_batch_memory(fpie_batch* b, double* used, double* budget);
/* "auto" or a variant name ("p16w8k16", "p8w16k16", "p16w8k8"). */
int fpie_batch_set_kernel(fpie_batch* b, const char* name);
int fpie_batch_kernel(fpie_batch* b, char* buf, int len);
/* Iterations (about 128 ns each) a CTA may wait for a dependency. */
int fpie_batch_set_spin_limit(fpie_batch* b, long long spins);
int fpie_batch_launch_count(fpie_batch* b, long long* count);

/* Kernel launches this solver has issued since creation (sweeps, residual,
 * image, conversions), counted on the host. */
int fpie_launch_count(fpie_solver* s, long long* count);

/* ---- measurement ------------------------------------------------------------
 * No counterpart in the reference: the denominator of the sweep kernels'
 * compute roofline.  Times one launch of `iters` rounds of independent
 * packed FP32 chains on every SM of the current device (CUDA events on
 * `stream`) and writes the rate in operations per second, one operation
 * per value: kind 0 packed add (__fadd2_rn), 1 packed multiply, 2 packed
 * fused multiply-add (one operation per value), 3 scalar add. */
int fpie_probe_fp32_rate(void* stream, int kind, int iters, double* ops_per_s);

#ifdef __cplusplus
}
#endif

#endif /* FPIE_GB300_H_ */
