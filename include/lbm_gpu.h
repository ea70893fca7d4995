/* lbm_gpu.h -- extended C API of the GB300 engine (no counterpart in lbc).
 *
 * lbc's main_lbm moves every array between host and device on each call. This
 * API keeps a case resident on the GPU instead: create a solver from the same
 * inputs main_lbm takes, upload a state once, advance it n steps on the device
 * (graph-captured step loop), and read fields, forces or the full state back
 * when needed. lbm_gpu_run(s, n) leaves exactly what n main_lbm calls plus the
 * caller-side f/f_new swap would leave (FP64 storage: bit for bit).
 *
 * Every function returns LBM_GPU_OK (0) or a negative code; the message is in
 * lbm_gpu_last_error() (thread-local). Nothing falls back to the CPU.
 */
#ifndef LBM_GPU_H
#define LBM_GPU_H

#include <stddef.h>

#include "lbm_types.h"

#ifdef __cplusplus
extern "C" {
#endif

#define LBM_GPU_OK 0
#define LBM_GPU_ERR_ARG (-1)
#define LBM_GPU_ERR_CUDA (-2)
#define LBM_GPU_ERR_NOMEM (-3)
#define LBM_GPU_ERR_IO (-4)

/* Population storage. F64: lbc's arithmetic, bit for bit. F32/F16_SHIFTED:
 * populations stored as f_k - w_k in FP32 / FP16, collision in FP32.
 * F64_FMA: FP64 storage, the step's moments and collision with fused
 * multiply-adds and the D2Q9 pair symmetry (74 FP64 instructions per node
 * against 125, so 1.6-1.9x faster on a part whose FP64 rate bounds the step);
 * lbc's results to rounding (1e-12 relative), not bit for bit. It needs lbc's
 * weight symmetry (w1 = w2 = w3 = w4, w5 = w6 = w7 = w8). */
enum { LBM_GPU_F64 = 0, LBM_GPU_F32_SHIFTED = 1, LBM_GPU_F16_SHIFTED = 2, LBM_GPU_F64_FMA = 3 };

typedef struct lbm_gpu_solver lbm_gpu_solver;

/* The inputs of main_lbm that describe a case (lbc include/lbm_core.h:6-31),
 * plus optional moving walls and the storage mode. Arrays are read during
 * lbm_gpu_create only (new Boundary values go through lbm_gpu_set_bc_values). */
typedef struct {
    int Nx, Ny;
    const int *cx, *cy, *opp;      /* must be lbc's D2Q9 ordering */
    const double *w;
    const double *omega_eff;       /* [Ny][Nx] */
    const int *solid_mask;         /* [Ny][Nx] */
    const double *phi;             /* [Ny][Nx] level set, used when use_IBB */
    int use_IBB;
    const Boundary *boundaries;    /* apply = this library's BC functions (a function of
                                      the caller's own runs only through main_lbm) */
    int num_boundaries;
    int isperiodic_x, isperiodic_y;
    double Fx, Fy;
    const double *wall_u, *wall_v; /* [Ny][Nx] wall velocity of solid nodes, or NULL */
    int storage;                   /* LBM_GPU_F64 / _F32_SHIFTED / _F16_SHIFTED / _F64_FMA */
} lbm_gpu_case;

typedef struct {
    int Nx, Ny, pitch, storage;
    int has_geometry;              /* 0: fully periodic, no solids, no edge BCs */
    int edge_stages;               /* Boundary entries run as edge kernels */
    int launches_per_step;         /* kernel launches per time step in the loop: the bulk
                                      step; the special-node step (F32/F16 storage with
                                      a flag word); edge_launches, which also finish the
                                      BC-written nodes and reduce the wall force, or,
                                      with wall links but no edge stages, one force
                                      reduction when a force history is enabled (the
                                      loop's steps reduce the force only then; a run's
                                      last step always does, for lbm_gpu_forces) */
    size_t device_bytes;
    long long steps_done;
    int edge_launches;             /* launches the edge stages take per step: consecutive
                                      entries on disjoint nodes share one */
} lbm_gpu_info;

const char *lbm_gpu_last_error(void);
int lbm_gpu_device_count(void);
/* The current device's FP64 fused multiply-add issue rate, measured (thread
 * FMA instructions per second, the fastest of five timed launches of a kernel
 * of independent DFMA chains): the ceiling of the FP64 step kernels, which are
 * bound by FP64 issue on parts with a low FP64 rate such as GB300. */
int lbm_gpu_fp64_rate(double *lane_ops_per_s);
/* How kernels can reach host memory at p: 1 page-locked and mapped at the
 * same address, 2 any pageable memory (the device walks the host page tables,
 * e.g. over NVLink-C2C), 0 neither (copies only), -1 no device. */
int lbm_gpu_host_access(const void *p);

int lbm_gpu_create(const lbm_gpu_case *c, lbm_gpu_solver **out);
int lbm_gpu_destroy(lbm_gpu_solver *s);

/* f, f_new: [Ny][Nx][9] as main_lbm receives them; rho/u/v: the stored fields
 * the next collision uses (lbc collides its first step with these arrays). */
int lbm_gpu_set_state(lbm_gpu_solver *s, const double *f, const double *f_new, const double *rho,
                      const double *u, const double *v);
/* After n steps: f = newest populations (what the caller's f holds after the
 * swap), f_new = the other buffer. Any pointer may be NULL. */
int lbm_gpu_get_state(lbm_gpu_solver *s, double *f, double *f_new, double *rho, double *u,
                      double *v);
int lbm_gpu_get_fields(lbm_gpu_solver *s, double *rho, double *u, double *v);
/* Copy new val1/val2 (length Ny or Nx; NULL keeps the current values) of
 * Boundary entry `entry` to the device; later steps use them. The arrays are
 * not kept. LBM_GPU_ERR_ARG for an entry outside the Boundary list. */
int lbm_gpu_set_bc_values(lbm_gpu_solver *s, int entry, const double *val1, const double *val2);

int lbm_gpu_run(lbm_gpu_solver *s, int nsteps);
/* Same as lbm_gpu_run, timed with CUDA events on the solver's stream. */
int lbm_gpu_run_timed(lbm_gpu_solver *s, int nsteps, double *ms);
/* Waits for the solver's device work and for a pending lbm_gpu_write_vtk. */
int lbm_gpu_sync(lbm_gpu_solver *s);

/* ---- Checkpoint / restart (no counterpart in lbc). Save writes everything a
 * continued run reads: both population buffers as stored, rho/u/v, the edge
 * band's moments, each Boundary entry's values and impedance-wall state, the
 * last force and the force history. Load needs a solver created from the same
 * case, with the same impedance walls set up and the same force-history
 * capacity; save after lbm_gpu_run(a), load, lbm_gpu_run(b) then equals
 * lbm_gpu_run(a + b) bit for bit. The file is raw host-order binary for this
 * library (a header, then length-prefixed blocks). LBM_GPU_ERR_IO on a file or
 * mismatch error (lbm_gpu_last_error says which). */
int lbm_gpu_checkpoint_save(lbm_gpu_solver *s, const char *path);
int lbm_gpu_checkpoint_load(lbm_gpu_solver *s, const char *path);

/* ---- VTK output packed on the device: the bytes lbc's write_vtk_binary_2D
 * writes for the stored fields (rho, u, v after the last run), the FP32
 * big-endian payload packed by a kernel, copied to pinned memory and written
 * by a host thread while the solver keeps stepping. The file is complete after
 * lbm_gpu_sync, the next lbm_gpu_write_vtk or lbm_gpu_destroy. */
int lbm_gpu_write_vtk(lbm_gpu_solver *s, const char *filename, double dx, double cu, double crho);

/* Momentum-exchange force of the last step: *D = x, *L = y (as main_lbm). */
int lbm_gpu_forces(lbm_gpu_solver *s, double *L, double *D);
/* Record the force of every step in a device ring of `capacity` steps. */
int lbm_gpu_enable_force_history(lbm_gpu_solver *s, int capacity);
/* Copies up to max_steps records (x, y), oldest first; returns the count. */
int lbm_gpu_force_history(lbm_gpu_solver *s, double *xy, int max_steps);
/* lbc's force record file (cases/cylinder/cylinder.c:162-185): for each step n
 * (counted from lbm_gpu_enable_force_history) not written yet, the doubles
 * n * dt, L * cf, D * cf. append = 1 adds to the file, 0 starts it. Called at
 * least every `capacity` steps, it streams the whole run. Returns the number
 * of records written; LBM_GPU_ERR_ARG when steps left the ring unwritten (the
 * ones still held are written), LBM_GPU_ERR_IO when the file fails. */
long long lbm_gpu_write_force_records(lbm_gpu_solver *s, const char *path, double dt, double cf, int append);

/* ---- Probes (no counterpart in lbc): density and velocity at n chosen nodes
 * (i[q], j[q]) after every step, from the populations the step leaves, in a
 * device ring of `capacity` steps; one small launch per step while set (in a
 * batch, one launch for all of its cases; set probes before the batch is
 * made). n = 0 removes them. At most 4096 probes. Probes are not saved in
 * checkpoints. */
int lbm_gpu_set_probes(lbm_gpu_solver *s, int n, const int *i, const int *j, int capacity);
/* Copies up to max_steps records, oldest first: out[(t * n + q) * 3 + {0, 1, 2}]
 * = rho, ux, uy of probe q at the t-th step held. Returns the count. */
int lbm_gpu_probe_history(lbm_gpu_solver *s, double *out, int max_steps);

/* ---- Time-domain impedance wall (no counterpart in lbc's library; it
 * replaces the host-side ADE coupling of lbc's cases/nit/nit.c:276-303).
 * Boundary entry `entry` must be velocity_bottom_regularized. Each of its
 * nodes with m[i] > 0 carries a mass-spring-damper m v' + R v + K x = p'
 * (FP64 state, exact zero-order-hold update per step) driven by the pressure
 * fluctuation p' = (rho - rhobar) / 3 of the interior neighbour at the
 * previous step, where rhobar starts at rho_ref and follows rho as an
 * exponential average, rhobar += alpha (rho - rhobar) (alpha = 0: fixed
 * reference; alpha > 0 keeps the mean-flow static pressure from loading the
 * spring); the BC then imposes u_y = -v (v > 0: flow into the liner) and
 * u_x = val1[i].
 * Nodes with m[i] <= 0 keep the entry's own val2. Running DFTs of p' and v at
 * nf <= 8 angular frequencies (rad / step) are kept per node, weighted by a
 * Hann window over window_steps steps (0: unweighted). Arrays have Nx
 * entries. */
int lbm_gpu_set_impedance_wall(lbm_gpu_solver *s, int entry, const double *R, const double *m,
                               const double *K, int nf, const double *omegas, double rho_ref,
                               double alpha, int window_steps);
/* spectra[(i * nf + f) * 4 + q]: q = 0,1 sum p' e^{-i w n} (re, im); q = 2,3 the
 * same for v. state[2 i + {0,1}] = (x, v). Either pointer may be NULL. */
int lbm_gpu_impedance_readback(lbm_gpu_solver *s, int entry, double *spectra, double *state);
/* The wall's per-step trace, streamed from a device ring of `capacity` steps:
 * the mean over its active nodes of the pressure fluctuation p' it was driven
 * with and of the velocity v it imposed (lbc's nit case traces the same pair
 * for its one global impedance model, cases/nit/nit.c:262-273). */
int lbm_gpu_enable_impedance_trace(lbm_gpu_solver *s, int entry, int capacity);
/* Writes the trace as lbc's text file does: one "%lf %lf %lf" line per step,
 * time, pressure, velocity, where the line of step n holds the values of step
 * n - 1 (a first line of zeros starts the file): lines n dt, p' cp, v cu. Lines
 * not written yet are appended (append = 1) or start the file (append = 0);
 * called at least every `capacity` steps it streams the whole run. Returns the
 * lines written; LBM_GPU_ERR_ARG when steps left the ring unwritten (the ones
 * still held are written), LBM_GPU_ERR_IO when the file fails. */
long long lbm_gpu_write_impedance_trace(lbm_gpu_solver *s, int entry, const char *path, double dt, double cp,
                                        double cu, int append);
/* The per-step update the wall uses: (x, v) <- A (x, v) + b p' is the exact
 * solution of m v' + R v + K x = p' over one step with p' held constant.
 * A row-major 2x2, b 2. Returns 0, or LBM_GPU_ERR_ARG unless m, K > 0, R >= 0. */
int lbm_gpu_msd_zoh(double R, double m, double K, double *A, double *b);

int lbm_gpu_get_info(lbm_gpu_solver *s, lbm_gpu_info *info);
/* Thread-block shape of the fused step (bx * by <= 256, bx multiple of 32).
 * No result depends on it: populations, fields and the momentum-exchange force
 * (summed in a fixed order per 32-node row segment in FP64 storage, per
 * 32-entry chunk of the case's special-node list in shifted storage) are
 * bit-identical for every shape. */
int lbm_gpu_set_block(lbm_gpu_solver *s, int bx, int by);
int lbm_gpu_get_block(lbm_gpu_solver *s, int *bx, int *by);

/* ---- Launch-shape autotuner (no counterpart in lbc).
 * mode 1: use the shape cached for this solver's key (device, storage, grid,
 * geometry class); without one, the next lbm_gpu_run with at least 17 steps
 * times the candidate blocks (64x4, 32x8, 128x2, 256x1, 32x4, 64x2, 128x1)
 * over interleaved windows of its own first steps, keeps the fastest for the
 * rest of the run and caches it. The trial steps are steps of the run, so
 * tuning costs no memory and changes no result. mode 0: off (the default,
 * unless the environment variable LBM_GPU_AUTOTUNE is a nonzero integer when
 * the solver is created). The cache lives in the process; when
 * LBM_GPU_TUNE_CACHE names a file it is also read from and appended to that
 * file. tuned: 1 once a shape was chosen; us_per_step: the chosen shape's time
 * per step in its trial windows (0 when it came from the cache). */
int lbm_gpu_set_autotune(lbm_gpu_solver *s, int mode);
int lbm_gpu_autotune_status(lbm_gpu_solver *s, int *tuned, int *bx, int *by, double *us_per_step);
void lbm_gpu_tune_cache_clear(void);

/* ---- Batches: many independent cases of one storage type advanced together.
 * Per step: one persistent kernel over the flattened tile list of every case
 * (uneven grids and different geometries share the launch), the i-th Boundary
 * entry of every case in one launch, one launch for all BC-written nodes, one
 * per-case force reduction; the loop runs from a captured CUDA graph. Every
 * case ends exactly as lbm_gpu_run(s, n) alone would leave it (FP64: bit for
 * bit, forces included). The solvers stay owned by the caller and must
 * outlive the batch. */
typedef struct lbm_gpu_batch lbm_gpu_batch;
int lbm_gpu_batch_create(lbm_gpu_solver *const *solvers, int n, lbm_gpu_batch **out);
int lbm_gpu_batch_run(lbm_gpu_batch *b, int nsteps);
int lbm_gpu_batch_run_timed(lbm_gpu_batch *b, int nsteps, double *ms);
/* Total nodes of all cases and kernel launches per batched step. */
int lbm_gpu_batch_info(lbm_gpu_batch *b, long long *nodes, int *launches_per_step);
/* Tile shape of the batched bulk kernel: tw x th = 256 nodes, tw in
 * {32, 64, 128, 256} (default 64 x 4). No result depends on it. */
int lbm_gpu_batch_set_tile(lbm_gpu_batch *b, int tw, int th);
/* Tile-shape tuning, as lbm_gpu_set_autotune: candidates 64x4, 32x8, 128x2,
 * 256x1 timed over step pairs of the next lbm_gpu_batch_run with at least 19
 * steps; the cache key is the batch's composition (every case's grid and
 * geometry class, in order). */
int lbm_gpu_batch_set_autotune(lbm_gpu_batch *b, int mode);
int lbm_gpu_batch_autotune_status(lbm_gpu_batch *b, int *tuned, int *tw, int *th, double *us_per_step);
int lbm_gpu_batch_destroy(lbm_gpu_batch *b);

/* ---- Serving: a continuous-batching request loop.
 * Any thread prepares a request (case, initial state, step count; all inputs
 * are copied), optionally attaches an impedance wall, and enqueues it. Each
 * storage type has a lane; a lane's round (lbm_gpu_server_poll runs one round
 * of every lane in the caller's thread; lbm_gpu_server_start gives each lane
 * its own thread) takes queued requests of its type in arrival order while the
 * device-memory budget and the slot limit (over all lanes) allow, launches one
 * chunk for its active requests (one graph-captured persistent batch, reused
 * while the set of requests is unchanged), admits the taken requests while the
 * chunk runs, then retires finished ones: their fields (and populations when
 * asked for) are copied to host memory and their device memory is returned to
 * the pool. Lanes run concurrently. Results are identical to running each
 * request alone (lbm_gpu_run). Admission is by the device memory free at the
 * time of the round (cudaMemGetInfo, plus what the pool holds unused from
 * retired requests), less a reserve (5 % of the device by default,
 * lbm_gpu_server_set_reserve) and less the requests taken but not set up yet:
 * memory that anything else takes after the server starts holds admissions
 * back. budget_bytes > 0 also caps the estimated bytes of the active requests
 * (0: no cap). When nothing is active one request is let in regardless, so a
 * request larger than the memory left runs alone or fails cleanly. */
typedef struct lbm_gpu_server lbm_gpu_server;
int lbm_gpu_server_create(size_t budget_bytes, int max_active, int chunk_steps, lbm_gpu_server **out);
/* Returns the request id (> 0) or a negative code. f = f_new = NULL: the
 * request starts from f = f_new = f_eq(rho, u, v) (lbc's equilibrium, formed
 * when the request is admitted), so a queued request holds only rho, u, v. */
int lbm_gpu_server_prepare(lbm_gpu_server *srv, const lbm_gpu_case *c, const double *f,
                           const double *f_new, const double *rho, const double *u, const double *v,
                           int nsteps, int keep_populations);
int lbm_gpu_server_set_impedance(lbm_gpu_server *srv, int id, int entry, const double *R,
                                 const double *m, const double *K, int nf, const double *omegas,
                                 double rho_ref, double alpha, int window_steps);
int lbm_gpu_server_enqueue(lbm_gpu_server *srv, int id);
/* One scheduling round; returns the number of requests still queued or active. */
int lbm_gpu_server_poll(lbm_gpu_server *srv);
int lbm_gpu_server_start(lbm_gpu_server *srv);
int lbm_gpu_server_stop(lbm_gpu_server *srv);
/* Returns 0 prepared, 1 queued, 2 running, 3 done, 4 failed (message in
 * lbm_gpu_last_error); times in seconds on a monotonic clock. */
int lbm_gpu_server_status(lbm_gpu_server *srv, int id, double *t_submit, double *t_admit,
                          double *t_done);
/* Copies a finished request's results; spectra as lbm_gpu_impedance_readback. */
int lbm_gpu_server_fetch(lbm_gpu_server *srv, int id, double *f, double *f_new, double *rho,
                         double *u, double *v, double *spectra);
int lbm_gpu_server_release(lbm_gpu_server *srv, int id);
int lbm_gpu_server_stats(lbm_gpu_server *srv, long long *lups_done, double *busy_s, int *queued,
                         int *active, size_t *bytes_in_use);
/* Device memory admissions leave free (default: 5 % of the device). */
int lbm_gpu_server_set_reserve(lbm_gpu_server *srv, size_t reserve_bytes);
/* The device memory a request could be admitted into now (free memory plus the
 * pool's unused part, less the reserve and the requests being set up). */
int lbm_gpu_server_available(lbm_gpu_server *srv, size_t *bytes);
/* Host time per phase of the scheduling rounds so far: out[0] rounds, [1]
 * admission (solver setup and state upload), [2] batch construction, [3]
 * launching and waiting for the chunks, [4] retiring (results to host, device
 * memory freed), [5..7] wall time of the FP64, FP32 and FP16 lanes' rounds
 * that ran a chunk; seconds (phases summed over lanes); [8] the same for the
 * FP64-FMA lane. Writes min(n, 9) values. */
int lbm_gpu_server_profile(lbm_gpu_server *srv, double *out, int n);
int lbm_gpu_server_destroy(lbm_gpu_server *srv);

/* ---- Force on caller-owned device memory, allocating nothing (no counterpart
 * in lbc; it is compute_force_mem of lbm_core.h on device arrays).
 * For callers that cannot let a library allocate device memory: processes
 * whose device memory is already held by their own pool (a framework's caching
 * allocator, a server that reserves memory up front) and loops that must not
 * stall the device, which cudaMalloc / cudaFree would do. f, f_new
 * ([Ny][Nx][9], lbc's layout) and solid_mask ([Ny][Nx]) are device arrays;
 * cx, cy, opp are host arrays (NULL: lbc's ordering); out is a device array of
 * two doubles that receives (x, y), asynchronously on `stream` (a
 * cudaStream_t, NULL for the default stream). Limit: at most 65536 blocks of
 * 64 x 4 nodes (4096 x 4096); larger grids are rejected with LBM_GPU_ERR_ARG.
 * Its scratch is a fixed 1 MiB device array inside the library, held on every
 * GPU that loads it until exit. The first call on a device looks up that
 * array's address (make it before any stream capture); calls share the array,
 * so calls that overlap on the GPU race: order them. */
int lbm_gpu_compute_force_mem_noalloc(int Nx, int Ny, int Q, const double *f, const double *f_new,
                                      const int *solid_mask, int isperiodic_x, int isperiodic_y,
                                      const int *cx, const int *cy, const int *opp, double *out,
                                      void *stream);

/* Page-locked host memory for fast transfers. */
void *lbm_gpu_host_alloc(size_t bytes);
void lbm_gpu_host_free(void *p);

/* The drop-in main_lbm keeps device buffers and geometry tables keyed by the
 * caller's array pointers. Call this after changing solid_mask, omega_eff or
 * phi in place; it also frees those buffers. */
void lbm_gpu_dropin_release(void);
/* main_lbm streams the caller's arrays through its kernels when the device can
 * reach them (lbm_gpu_host_access > 0) and stages them through copies
 * otherwise; staged = 1 forces the copies (both give identical results). */
void lbm_gpu_dropin_set_staged(int staged);
/* Lazy drop-in (off by default). lazy = 1: main_lbm leaves its results on the
 * device and returns only *L and *D. The next main_lbm call continues there when
 * the caller has swapped f and f_new and passes the same rho, u, v and case (lbc's
 * case mains do, cases/nit/nit.c:309-311); any other call writes the results
 * back first. So do every other lbc function of this library, lbm_gpu_dropin_sync,
 * lbm_gpu_dropin_release and set_lazy itself. Until then the caller's arrays
 * are stale and must be neither read nor written. Results are the same bits as
 * with lazy = 0. */
void lbm_gpu_dropin_set_lazy(int lazy);
/* Writes a pending lazy main_lbm result to the caller's arrays. */
int lbm_gpu_dropin_sync(void);

#ifdef __cplusplus
}
#endif
#endif
