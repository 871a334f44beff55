/*
 * tcs.h — C-ABI of tcstencil_gb300, a GB300 (sm_103a) engine for the 2-D
 * Jacobi sweeps star2d1r, star2d2r, box2d1r and box2d2r of TCStencil.
 *
 * Plain C: pointers, sizes and ints only.  Every int-returning entry point
 * returns a TCS_* status; tcs_last_error() gives the message of the last
 * failure on the calling thread.  Device pointers are CUDA device pointers of
 * the current device; `stream` is a cudaStream_t (NULL = legacy default).
 *
 * Stencil semantics (common/gold_*.cpp): out[i][j] = sum over taps of
 * B[dy+r][dx+r] * in[i+dy][j+dx] on an update rectangle; star stencils read
 * only the centre row and column of the n x n coefficient matrix B (n = 2r+1).
 * Cells outside the rectangle keep their value (a fixed border): a multi-step
 * sweep is a ping-pong whose border never changes, as gold's is.
 *
 * Device plane format of the sweep engine ("panel planes"): 16-row
 * half-bricks of 16 bytes per row (8 FP16 or 4 FP32 cells) in column-major
 * brick order, i.e. column panels of 16 bytes per row with the rows of a
 * panel contiguous.  With cpp = 8 (FP16) or 4 (FP32) cells per panel row,
 * nyp = ceil(ny/128)*128 + 8 rows per panel and npan = ceil(nx/128)*128/cpp
 * + 2 panels, cell (y, x) is at element
 *     ((x/cpp + 1) * nyp + (y + 4)) * cpp + x % cpp,
 * and tcs_plane_elems() gives the element count.  Padding rows and panels
 * must hold finite values (tcs_pack_* writes every element; zero-fill planes
 * that are only written by sweeps).  FP16 planes hold IEEE binary16 bits
 * (uint16_t); a split grid is two FP16 planes (hi, lo, see tcs_pack_split).
 * The reference's own 16 x 16 brick layout (layout16, brick_layout_2D of
 * layout16/host_*.cu:77-88) is produced by tcs_brick_layout_2d.
 */
#ifndef TCS_H_
#define TCS_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define TCS_OK 0
#define TCS_ERR_INVALID 1     /* an argument is out of range                  */
#define TCS_ERR_CUDA 2        /* a CUDA runtime or driver call failed         */
#define TCS_ERR_UNSUPPORTED 3 /* valid request this build/device cannot run   */
#define TCS_ERR_NOMEM 4       /* device allocation failed or budget exceeded  */
#define TCS_ERR_TIMEOUT 5     /* a bounded device wait gave up                */
#define TCS_ERR_CANCELLED 6   /* a server request was cancelled (tcs_server_cancel) */

enum tcs_stencil { TCS_STAR2D1R = 0, TCS_STAR2D2R = 1, TCS_BOX2D1R = 2, TCS_BOX2D2R = 3 };
/* TENSOR: tcgen05 banded-matrix kernel; CUDACORE: FP32 FMA warp-strip kernel */
enum tcs_engine { TCS_ENGINE_TENSOR = 0, TCS_ENGINE_CUDACORE = 1 };
/* F16: FP16 storage, FP32 accumulate.  SPLIT: hi+lo FP16 pair storage, four
 * tensor-core products, FP32-level accuracy (tensor engine only; needs a
 * non-expanding stencil, sum of |c| <= 1).  F32: FP32 storage with gold's
 * exact arithmetic (CUDA-core engine only). */
enum tcs_precision { TCS_PREC_F16 = 0, TCS_PREC_SPLIT = 1, TCS_PREC_F32 = 2 };

const char *tcs_status_string(int status);
const char *tcs_last_error(void);
/* Radius of a stencil (1 or 2), or -1. */
int tcs_stencil_radius(int stencil);
/* Elements of the reference's layout16 bricks of an ny x nx grid:
 * ceil(ny/16)*ceil(nx/16)*256. */
size_t tcs_brick_elems(int ny, int nx);
/* Elements of one engine plane of an ny x nx grid for a precision (uint16_t
 * elements for F16 and SPLIT, floats for F32). */
size_t tcs_plane_elems(int ny, int nx, int precision);
/* Reads and clears the device error word that bounded in-kernel waits set on
 * timeout (0 = none).  Synchronises the device. */
int tcs_device_error(int *code);

/* ------------------------------------------------ drop-in host entry points
 * Same signature, arguments and behaviour as the reference's
 *   extern "C" void host_code(float *h_A, float *h_B, float *h_C, int N, int n)
 * (tensor form: layout16/host_<stencil>.cu, e.g. layout16/host_star2d1r.cu:129;
 *  CUDA-core form: baseline/host_<stencil>.cu, e.g. baseline/host_star2d1r.cu:78):
 * h_A is N x N FP32 (N a multiple of 16), h_B is n x n, the grid is padded by
 * 16 cells of value 1.0, stored as an FP16 plane, swept once per launch for
 * RUN_TIMES launches (timed from launch SKIP_TIMES on, printed as
 * "[Time] Time used: %f ms"), and all N x N cells of the result are written to
 * h_C as FP32.  Device memory is allocated and freed inside the call.  On a
 * CUDA error the message is printed and the process exits, as the reference's
 * check_error does (common/common.hpp:10-16). */
void host_star2d1r(float *h_A, float *h_B, float *h_C, int N, int n);
void host_star2d2r(float *h_A, float *h_B, float *h_C, int N, int n);
void host_box2d1r(float *h_A, float *h_B, float *h_C, int N, int n);
void host_box2d2r(float *h_A, float *h_B, float *h_C, int N, int n);
void host_cc_star2d1r(float *h_A, float *h_B, float *h_C, int N, int n);
void host_cc_star2d2r(float *h_A, float *h_B, float *h_C, int N, int n);
void host_cc_box2d1r(float *h_A, float *h_B, float *h_C, int N, int n);
void host_cc_box2d2r(float *h_A, float *h_B, float *h_C, int N, int n);

/* The parametrised form behind the eight entry points above and behind the
 * per-variant `host_code` shims, with the common/param.hpp macros as
 * arguments (RUN_TIMES, SKIP_TIMES, STEP_TIMES, TILE_SIZE; tile_size is
 * accepted and ignored: tiles are chosen by the engine).  Returns a status
 * instead of exiting. */
int tcs_host_code(float *h_A, float *h_B, float *h_C, int N, int n, int stencil, int engine,
                  int run_times, int skip_times, int step_times, int tile_size);

/* ------------------------------------------- layout transforms (device)
 * Bit-exact device forms of the reference's host helpers
 * (layout16/host_star2d1r.cu:63-101, common/common.hpp:146-160). */

/* padding_2D (layout16/host_star2d1r.cu:63-75): d_in size x size FP16 ->
 * d_out (size+2*halo)^2 FP16, border cells = value16 (FP16 bits). */
int tcs_padding_2d(const uint16_t *d_in, uint16_t *d_out, int size, int halo, uint16_t value16,
                   void *stream);
/* brick_layout_2D (layout16/host_star2d1r.cu:77-88), generalised to ny x nx;
 * cells of partial bricks past the grid are 0. */
int tcs_brick_layout_2d(const uint16_t *d_in, uint16_t *d_out, int ny, int nx, void *stream);
/* reverse_layout_2D (layout16/host_star2d1r.cu:90-101), generalised likewise. */
int tcs_reverse_layout_2d(const uint16_t *d_in, uint16_t *d_out, int ny, int nx, void *stream);
/* array_float2half + padding_2D + the layout change in one pass: d_in is an
 * ny x nx FP32 row-major grid, the result is the FP16 engine plane of the
 * (ny+2*pad) x (nx+2*pad) grid whose border cells are pad_value. */
int tcs_pack_f16(const float *d_in, int ny, int nx, int pad, float pad_value, uint16_t *d_plane,
                 void *stream);
/* The inverse (reverse layout + interior copy + array_half2float): the ny x nx
 * cells at offset (pad, pad) of the (ny+2*pad) x (nx+2*pad) plane, as FP32. */
int tcs_unpack_f16(const uint16_t *d_plane, int ny, int nx, int pad, float *d_out, void *stream);
/* FP32 counterparts of the two above. */
int tcs_pack_f32(const float *d_in, int ny, int nx, int pad, float pad_value, float *d_plane,
                 void *stream);
int tcs_unpack_f32(const float *d_plane, int ny, int nx, int pad, float *d_out, void *stream);
/* Split counterparts.  A split grid stores x' = x 2^-scale_exp as
 * hi = rint(x' 2^11) 2^-11 (FP16, fixed point) and lo = fp16((x' - hi) 2^11);
 * scale_exp should make max|x'| <= 1 (tcs_split_scale_exp). */
int tcs_pack_split(const float *d_in, int ny, int nx, int pad, float pad_value, int scale_exp,
                   uint16_t *d_hi, uint16_t *d_lo, void *stream);
int tcs_unpack_split(const uint16_t *d_hi, const uint16_t *d_lo, int ny, int nx, int pad,
                     int scale_exp, float *d_out, void *stream);
/* max |x| of n device floats, returned in host memory (synchronous). */
int tcs_max_abs_f32(const float *d_in, size_t n, float *h_max, void *stream);
/* Smallest E with max_abs 2^-E <= 1 (0 when max_abs is 0). */
int tcs_split_scale_exp(float max_abs);

/* Band builders (host): the reference's init_coe, bit-exact.  B16 is n x n
 * FP16 bits.  Star (layout16/host_star2d1r.cu:33-61, host_star2d2r.cu:33-67):
 * a, b are 16x16.  Box (layout16/host_box2d1r.cu:29-46, host_box2d2r.cu:29-50):
 * coe is n bands of 16x16. */
int tcs_init_coe_star(const uint16_t *B16, int n, uint16_t *a, uint16_t *b);
int tcs_init_coe_box(const uint16_t *B16, int n, uint16_t *coe);

/* ------------------------------------------------------ one sweep step
 * One Jacobi step on caller-owned device planes (the device kernel the
 * reference launches as mma_run / kernel_run, layout16/kernel_*.cu,
 * baseline/kernel_*.cu).  `coeffs` is the n x n FP32 matrix in host memory;
 * the update rectangle is [y0,y1) x [x0,x1), or gold's interior
 * [r, ny-r) x [r, nx-r) when all four are 0; it must lie inside
 * [r, ny-r) x [r, nx-r).  d_out cells outside the rectangle receive d_in's.
 * For TCS_PREC_SPLIT, *_lo are the lo planes; otherwise pass NULL.
 * For TCS_PREC_F32 the planes are float planes. */
typedef struct tcs_step_args {
    int ny, nx;
    int stencil;   /* enum tcs_stencil   */
    int engine;    /* enum tcs_engine    */
    int precision; /* enum tcs_precision */
    int y0, y1, x0, x1;
    const float *coeffs; /* host, n*n */
} tcs_step_args;

int tcs_sweep_step(const tcs_step_args *args, const void *d_in, const void *d_in_lo, void *d_out,
                   void *d_out_lo, void *stream);

/* ------------------------------------------------ sweeps without allocation
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * where they sweep: real-time loops that forbid allocator calls and the device
 * synchronisation they may bring, and hosts whose device memory is all handed
 * out by a pool or budget they do not own.  d_out receives `steps` FP16 Jacobi
 * steps of d_in (planes as in tcs_sweep_step; d_in is only read, and its
 * padding must be finite; precision must be TCS_PREC_F16).  The ping-pong
 * partner plane is a library-owned static device array of
 * tcs_noalloc_scratch_bytes() = 32 MiB, held by every GPU that loads the
 * library until exit: grids whose plane (tcs_plane_elems) has up to
 * 16,777,216 cells (square grids up to 3968 x 3968); larger ones are rejected
 * with TCS_ERR_INVALID.  No device memory is allocated.  The first call on a
 * device looks up the array's device address (and configures the tensor
 * kernel): make that first call before any stream capture.  The address is
 * kept for the process, so after cudaDeviceReset the entry point must not be
 * used on that device again.  All calls on a device share the array and keep
 * the last call's contents; each call first copies d_in (padding included)
 * over the part of the array it uses and over d_out, so nothing left by an
 * earlier call is read.  Calls that overlap on the GPU (other streams or
 * threads) race on the array. */
size_t tcs_noalloc_scratch_bytes(void);
int tcs_sweep_steps_noalloc(const tcs_step_args *args, const void *d_in, void *d_out, int steps,
                            void *stream);

/* ------------------------------------------------------------------ plans
 * A plan owns the device state of one grid (ping-pong planes) and runs
 * multi-step sweeps; steps > 1 run as one captured CUDA graph per step count. */
typedef struct tcs_plan_s *tcs_plan;

typedef struct tcs_problem {
    int ny, nx;
    int stencil, engine, precision;
    int y0, y1, x0, x1; /* all 0 = [r, ny-r) x [r, nx-r) */
    const float *coeffs; /* host, n*n; copied into the plan */
} tcs_problem;

int tcs_plan_create(const tcs_problem *problem, tcs_plan *out);
int tcs_plan_destroy(tcs_plan plan);
/* Loads an ny x nx FP32 row-major grid (host or device memory). */
int tcs_plan_upload(tcs_plan plan, const float *grid, int grid_on_host, void *stream);
/* Writes the current state as an ny x nx FP32 row-major grid. */
int tcs_plan_download(tcs_plan plan, float *grid, int grid_on_host, void *stream);
/* Runs `steps` sweep steps.  use_graph != 0 replays a CUDA graph of the steps. */
int tcs_plan_run(tcs_plan plan, int steps, int use_graph, void *stream);
/* Device pointers of the current state planes (lo = NULL unless split), and
 * the bytes of one plane. */
int tcs_plan_state(tcs_plan plan, void **hi, void **lo, size_t *plane_bytes);
/* Scale exponent of a split plan's planes (0 for other precisions). */
int tcs_plan_scale_exp(tcs_plan plan, int *scale_exp);
/* Replaces the coefficients (host n*n). */
int tcs_plan_set_coeffs(tcs_plan plan, const float *coeffs);
/* Temporal blocking depth: 1 (one launch per step, the default) or 2 (two
 * steps per launch, intermediate kept on chip; split precision on the tensor
 * engine).  Results are bit-identical either way; the autotuner picks. */
int tcs_plan_set_temporal_depth(tcs_plan plan, int depth);
/* Tensor engine (FP16 or split, temporal depth 1): run(steps >= 2) as ONE
 * launch whose tiles of step j wait only for the neighbouring tile rows of
 * step j-1 (per-row completion counts), instead of one launch per step.
 * mode -1 (default): FP16 when a step has more than two tiles per SM, split
 * when it has more than one and at most eight (where each measured
 * faster); 0: never; 1: always.  Results are bit-identical either way.
 * TCS_MULTI=0 in the environment turns it off for the process. */
int tcs_plan_set_multistep(tcs_plan plan, int mode);
/* Tile shape of the plain FP16 tensor sweeps: 128 rows by tile_w = 128
 * (default), 96 or 64 columns.  Narrower tiles give a grid more tiles: on
 * grids with few tiles per SM more SMs share a step, and each tile's MMAs and
 * epilogue shrink with its width.  Results are bit-identical at every width;
 * the autotuner picks the width per size class (it replaces the reference's
 * TILE_SIZE sweep, script/param.py:5).  TCS_ERR_UNSUPPORTED for widths below
 * 128 on other engines and precisions. */
int tcs_plan_set_tile_width(tcs_plan plan, int tile_w);
int tcs_plan_tile_width(tcs_plan plan, int *tile_w);
/* Kernel launches tcs_plan_run(plan, steps, ...) makes (the device work of
 * one call: 1 for a multi-step launch, else one per step or step pair). */
int tcs_plan_launches(tcs_plan plan, int steps, int *launches);

/* One-call form: host FP32 grid in, `steps` steps, host FP32 grid out.  Device
 * state is kept in a per-thread cache keyed by shape and mode, so repeated
 * calls of one shape do not reallocate. */
int tcs_sweep_host(const float *h_in, float *h_out, const tcs_problem *problem, int steps);
/* Frees the calling thread's cached plans. */
void tcs_release_cache(void);

/* ------------------------------------------------------------------ pipes
 * Many grids of one shape streamed through the device: each submission
 * copies a host FP32 grid in, runs `steps` steps and copies the result out,
 * double-buffered over two plans and two streams, so one grid's transfers
 * and packing overlap the other's sweeps.  Host buffers should be pinned
 * (cudaHostAlloc / torch pin_memory) for the copies to overlap.  Submission
 * k's h_in and h_out belong to the pipe until submission k + 2 has been
 * submitted or tcs_pipe_wait has returned; every result is the same bits as
 * tcs_sweep_host's for that grid. */
typedef struct tcs_pipe_s *tcs_pipe;
int tcs_pipe_create(const tcs_problem *problem, tcs_pipe *out);
int tcs_pipe_destroy(tcs_pipe pipe);
int tcs_pipe_submit(tcs_pipe pipe, const float *h_in, float *h_out, int steps);
/* Waits for every submission; reports a device wait timeout as tcs_device_error. */
int tcs_pipe_wait(tcs_pipe pipe);

/* ---------------------------------------------------------------- batches
 * A batch advances many independent grids (any mix of sizes, stencils,
 * coefficients, FP16 or split precision, and step counts) with ONE persistent
 * tensor-core launch per run: every (grid, step, tile) is a work item, and a
 * tile of step t starts once its grid's step t-1 is stored.  Each grid gets
 * the same bits as a tcs_plan of the same problem run alone.  No reference
 * counterpart: the reference runs one grid per process (main_1r.cu /
 * main_2r.cu); batches serve many small problems at once.
 *
 * Use: tcs_batch_add every grid, then upload each, then tcs_batch_run (any
 * number of times; each run advances every grid by its own step count), then
 * download.  Grids are added only before the first upload or run. */
typedef struct tcs_batch_s *tcs_batch;

int tcs_batch_create(tcs_batch *out);
int tcs_batch_destroy(tcs_batch batch);
/* Adds a grid (engine must be TCS_ENGINE_TENSOR, precision F16 or SPLIT) that
 * advances `steps` steps per run; *index receives its position. */
int tcs_batch_add(tcs_batch batch, const tcs_problem *problem, int steps, int *index);
/* Loads grid `index` from an ny x nx FP32 row-major array (host or device). */
int tcs_batch_upload(tcs_batch batch, int index, const float *grid, int grid_on_host, void *stream);
/* Writes grid `index`'s current state as an ny x nx FP32 row-major array. */
int tcs_batch_download(tcs_batch batch, int index, float *grid, int grid_on_host, void *stream);
/* One run: every grid advances by its step count.  use_graph != 0 replays a
 * captured CUDA graph of the run. */
int tcs_batch_run(tcs_batch batch, int use_graph, void *stream);
/* Point updates per run, work items per run and the number of grids. */
int tcs_batch_info(tcs_batch batch, long long *point_updates, int *items, int *grids);
/* External gate: grid `index` starts its first step only once the device
 * word *d_flag is >= value (written by another stream, kernel or copy), so a
 * batch can consume what a producer elsewhere writes without a host round
 * trip.  Set before the first upload or run. */
int tcs_batch_set_gate(tcs_batch batch, int index, const unsigned *d_flag, unsigned value);
/* Limit of the in-kernel dependency and gate waits (default 1 s).  A wait
 * that runs out stops the launch cleanly and tcs_device_error reports
 * TCS_ERR_TIMEOUT (code 6). */
int tcs_batch_set_wait_limit(tcs_batch batch, double seconds);

/* ------------------------------------------------------- FP64 drift check
 * An FP64 shadow of a problem on the device, stepped with gold's tap order
 * and separately rounded multiply and add (the oracle's FP64 restatement of
 * common/gold_*.cpp, bit for bit), and a comparison of any FP32 grid with it.
 * FP64 appears only here, never in the sweep kernels.  Step it beside a plan
 * and compare every k steps to watch the error of the FP16 or split form. */
typedef struct tcs_drift_s *tcs_drift;

int tcs_drift_create(const tcs_problem *problem, tcs_drift *out);
int tcs_drift_destroy(tcs_drift drift);
/* Loads the ny x nx FP32 starting grid (host or device), widened to FP64. */
int tcs_drift_upload(tcs_drift drift, const float *grid, int grid_on_host, void *stream);
int tcs_drift_run(tcs_drift drift, int steps, void *stream);
/* Relative L2 (||a - ref|| / ||ref||) and max |a - ref| of the device FP32
 * grid a (ny x nx row-major) against the shadow's state.  Synchronises. */
int tcs_drift_compare(tcs_drift drift, const float *d_grid, double *rel_l2, double *max_abs,
                      void *stream);
/* Copies the shadow's FP64 state to host memory (ny x nx).  Synchronises. */
int tcs_drift_download(tcs_drift drift, double *h_grid, void *stream);
/* Device pointer of the shadow's current FP64 state (ny x nx row-major). */
int tcs_drift_state(tcs_drift drift, const double **d_grid);

/* ---------------------------------------------------------------- serving
 * A request server does continuous batching of stencil solves on one GPU.
 * No reference counterpart.  A native scheduler thread does the work:
 *   - admits queued requests while the HBM budget has room for their state
 *     (ping-pong planes plus an FP32 staging grid);
 *   - uploads and packs each one on a copy stream;
 *   - folds every resident request into the next round, which is ONE batched
 *     persistent launch advancing each request by up to round_steps steps
 *     (all of its remaining steps when round_steps is 0);
 *   - unpacks and downloads finished requests while later rounds run, then
 *     frees their memory.
 * A request's state stays on the device between rounds.  A request that
 * arrives while a round runs joins a following round.  Results are
 * bit-identical to the same problem run alone (tcs_plan, tensor engine). */
typedef struct tcs_server_s *tcs_server;

typedef struct tcs_server_config {
    size_t hbm_budget_bytes; /* device memory for request state (allocated once) */
    int max_active;          /* resident requests at most (0 = 1024)            */
    int round_steps;         /* steps per request per round (0 = all remaining)  */
} tcs_server_config;

typedef struct tcs_server_stats {
    long long submitted, completed, failed;
    long long rounds;
    long long point_updates;   /* completed requests' interior point-updates */
    long long algorithmic_bytes; /* 4 B (FP16) / 8 B (split) per point-update  */
    double gpu_busy_s;         /* sum of round durations (CUDA events)       */
    size_t budget_bytes, peak_bytes_in_use;
    int active, queued;
    /* scheduler passes: time in reap, admit, round polling and round launch
     * (total and the worst single pass), seconds */
    double sched_total_s[4], sched_max_s[4];
    /* round launch: host build of the round, compute-stream enqueue, and the
     * enqueue of finished requests' downloads (total and worst), seconds */
    double launch_total_s[3], launch_max_s[3];
    long long cancelled;       /* requests ended by tcs_server_cancel */
} tcs_server_stats;

int tcs_server_create(const tcs_server_config *config, tcs_server *out);
/* Waits for every submitted request, stops the scheduler, frees everything. */
int tcs_server_destroy(tcs_server server);
/* Queues a solve: `steps` steps of `problem` (tensor engine, F16 or SPLIT)
 * from the ny x nx FP32 grid h_in into h_out.  Both are host buffers, ideally
 * pinned.  They belong to the server until the ticket completes.  Fails with
 * TCS_ERR_NOMEM when the request alone exceeds the budget. */
int tcs_server_submit(tcs_server server, const tcs_problem *problem, int steps, const float *h_in,
                      float *h_out, long long *ticket);
/* Ticket state: 0 queued, 1 resident, 2 done, 3 failed; *status = its status. */
int tcs_server_poll(tcs_server server, long long ticket, int *state, int *status);
/* Blocks until the ticket is done or failed, or until timeout_s (< 0: no limit). */
int tcs_server_wait(tcs_server server, long long ticket, double timeout_s);
/* Cancels a request.  A queued one is dropped at once; a resident one takes
 * part in no further round and is retired (its memory freed) once its
 * rounds and upload are done.  Either way the ticket ends failed with
 * TCS_ERR_CANCELLED and h_out is left as it was.  TCS_ERR_INVALID when the
 * ticket is unknown, done, failed, already cancelled, or finishing (its
 * result being downloaded: it completes normally).  With tcs_server_wait's
 * timeout this gives a deadline: wait, and cancel on TCS_ERR_TIMEOUT. */
int tcs_server_cancel(tcs_server server, long long ticket);
/* Seconds, on the server's clock, of the ticket's submission, admission and
 * completion (its result in h_out). */
int tcs_server_times(tcs_server server, long long ticket, double *submitted, double *admitted,
                     double *completed);
/* The server's clock (seconds since creation). */
double tcs_server_clock(tcs_server server);
int tcs_server_get_stats(tcs_server server, tcs_server_stats *stats);

/* ------------------------------------- allocation hook and guard regions ---
 * Test and debug aids; neither is needed in production.  No reference
 * counterpart (the reference's allocations exit on failure,
 * common/common.hpp:10-16).
 *
 * Every device and pinned-host allocation the library makes (plans, batches,
 * the server, the drift check, tcs_sweep_host, host_code) first asks the
 * hook, if one is installed: hook(bytes, what, user) != 0 makes that
 * allocation fail as out of memory, so the call that needed it returns
 * TCS_ERR_NOMEM with `what` in tcs_last_error(), after freeing what it had
 * allocated.  NULL removes the hook.  The hook runs on the allocating
 * thread (the server's scheduler thread for round buffers).
 *
 * tcs_set_guard_bytes(n): allocations made from now on carry n bytes
 * (rounded up to a multiple of 256; 0 turns it off) of a canary pattern
 * before and after them; batches and the server also put n canary bytes
 * between the planes of their pools and around each request, and
 * tcs_sweep_steps_noalloc after the part of its scratch a call uses.
 * tcs_guard_check waits for the device, compares every live guard region
 * with the canary and sets *damaged to the number found changed, counting
 * those found changed when their memory was freed since the last check; a
 * non-zero count names the regions in tcs_last_error().  A changed guard
 * means a kernel or copy wrote out of bounds.
 *
 * tcs_alloc_stats: the library's live allocations, count and bytes (a test
 * of error paths can compare them before and after a failed call). */
typedef int (*tcs_alloc_hook)(size_t bytes, const char *what, void *user);
int tcs_set_alloc_hook(tcs_alloc_hook hook, void *user);
int tcs_set_guard_bytes(size_t bytes);
int tcs_guard_check(long long *damaged);
int tcs_alloc_stats(long long *live_count, size_t *live_bytes);

#ifdef __cplusplus
}
#endif

#endif /* TCS_H_ */
