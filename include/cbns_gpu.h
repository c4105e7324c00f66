/*
 * cbns_gpu.h — C ABI of the GB300 (sm_103a) right-hand-side library for the
 * cbns3d compressible Navier-Stokes solver.
 *
 * One handle is one Block3d-equivalent solve living in device memory.  The
 * library owns every device allocation behind the opaque handle; the caller
 * keeps its host arrays (the reference allocates them in Block3d::allocate_mem,
 * src/Block3d.cpp:41-135) and passes plain host pointers.  Nothing throws across
 * this boundary: every entry point returns a cbns_status.
 *
 * Host array layouts are the reference's (include/Block3d.h:169-199):
 *   Q          Q[n + 5*((NG+i) + IM_G*((NG+j) + JM_G*(NG+k)))], ghosts included,
 *              IM_G = IM + 2*NG, NG = 4   (get_idx_Q)
 *   primitives f[(NG+i) + IM_G*((NG+j) + JM_G*(NG+k))]            (get_idx)
 *
 * Threading: one handle per host thread at a time; each handle runs on its own
 * CUDA stream.  Batch entry points take a set of handles and launch their
 * stages together.
 */
#ifndef CBNS_GPU_H
#define CBNS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CBNS_NEQ 5 /* equations, include/constants.h:13 */
#define CBNS_NG 4  /* ghost layers of Q and primitives, include/constants.h:15-17 */
#define CBNS_NGV 2 /* ghost layers of gradients, include/constants.h:16 */

typedef enum cbns_status {
  CBNS_OK = 0,
  CBNS_FINISHED = 1,              /* t_cur + 1e-5 > t_end: no step taken (Block3d::is_finished) */
  CBNS_ERR_INVALID_ARG = -1,      /* null pointer, unknown stage/precision, bad parameter */
  CBNS_ERR_BAD_DIMS = -2,         /* a block dimension below CBNS_NG or above the limit */
  CBNS_ERR_CUDA = -3,             /* a CUDA runtime call failed; see cbns_last_error() */
  CBNS_ERR_OUT_OF_MEMORY = -4,    /* device allocation failed */
  CBNS_ERR_NONPHYSICAL = -5,      /* a stage produced rho <= 0, p <= 0 or a NaN */
  CBNS_ERR_TIMEOUT = -6,          /* a bounded device-side wait gave up */
  CBNS_ERR_NO_DEVICE = -7,        /* no CUDA device, or not an sm_103 device */
  CBNS_ERR_IO = -8,               /* host file could not be read or written */
  CBNS_ERR_FORMAT = -9,           /* host file is truncated or its dimensions do not match */
  CBNS_ERR_CANCELLED = -10,       /* a serving request was cancelled or its server stopped */
  CBNS_ERR_BOUNDS = -11           /* bounds-checked build only: a kernel index left its array */
} cbns_status;

typedef enum cbns_precision {
  CBNS_FP64 = 0,       /* every operation in IEEE binary64 */
  CBNS_FP32_MIXED = 1, /* WENO, projections and fluxes in binary32; state, RK3 and sums in binary64 */
  CBNS_FP64_FF = 2     /* the state, its RK3 combination and the KE/enstrophy sums in binary64;
                          the face fluxes, viscous terms, flux differences, primitives and the
                          time step's per-cell speed in float-float arithmetic (pairs of binary32
                          numbers, about 47 significant bits) on the binary32 pipes.  Within
                          the binary64 path's 1e-11 parity bar of the reference. */
} cbns_precision;

/*
 * Simulation parameters: the fields of SimulationParams
 * (include/simulation_params.h:15-53), in the order read_input() reads them
 * from input.txt (src/read_input.cpp:24-72), then the derived constants of
 * src/read_input.cpp:78-90 (filled by cbns_params_derive).
 */
typedef struct cbns_params {
  char checkpoint_fname[256];
  double CFL;
  double t_cur;
  double t_end;
  double Pr;
  double gamma;
  double Mach;
  double Re;
  double T_inf;
  double L; /* read but unused, as in the reference */
  uint32_t IM, JM, KM;
  uint32_t nstep_max;
  uint32_t checkpoint_freq;
  uint32_t num_output;
  int32_t is_restart; /* 1 = start from the initial condition, 0 = read the checkpoint */
  /* derived */
  double Mach2, Re_inv, Pr_inv, gam1, gM2, gam1_inv, p_inf, C_T_inf, C_dt_v;
} cbns_params;

typedef struct cbns_handle cbns_handle;

/* Derived constants of src/read_input.cpp:78-90. */
cbns_status cbns_params_derive(cbns_params* p);

/* Block3d::Block3d + allocate_mem (src/Block3d.cpp:11-135) and gen_mesh's spacing
 * (src/Block3d.cpp:208-219): dx = 2*pi/p->IM etc.  IM, JM, KM are this block's
 * extents (the whole grid on one GPU).  Uses the calling thread's current CUDA device unless the environment variable
 * CBNS_DEVICE names one. */
cbns_status cbns_create(const cbns_params* p, uint32_t IM, uint32_t JM, uint32_t KM,
                        int precision, cbns_handle** out);
cbns_status cbns_destroy(cbns_handle* h);

/* Upload the conserved state (get_idx_Q layout, ghosts ignored and refilled) and
 * run the start-up sequence of src/cbns3d.cpp:149-153: boundary_condition(Q),
 * calc_primitive(Q), init_Q_p().  mu is reset to 1 in the interior, the value
 * Block3d::initial_condition gives it (src/Block3d.cpp:265).  Sets t_cur = t. */
cbns_status cbns_upload_Q(cbns_handle* h, const double* Q, double t);

/* Device-side initial condition (no host state): the Taylor-Green state of
 * Block3d::initial_condition + calc_conservative (src/Block3d.cpp:237-300),
 * plus, when nmodes > 0 (at most 64), the project-defined solenoidal velocity
 * perturbation that cbns_host_initial_condition_perturbed draws from the same
 * seed; then the start-up sequence of cbns_upload_Q.  Equal to uploading the
 * host-built state up to the last-place differences of device sin/cos. */
cbns_status cbns_init_tgv(cbns_handle* h, uint64_t seed, double amp, int nmodes, int kmax, double t);

/* Block3d::get_Q / get_Q_p (src/Block3d.cpp:302-316): copy Q or Q_p, ghosts
 * included, into a host array of NEQ*IM_G*JM_G*KM_G doubles. */
cbns_status cbns_download_Q(cbns_handle* h, double* Q);
cbns_status cbns_download_Q_p(cbns_handle* h, double* Q_p);

/* The primitive arrays of the current state (Block3d::calc_primitive,
 * src/Block3d.cpp:359-385) in the padded get_idx layout; any pointer may be NULL. */
cbns_status cbns_download_prims(cbns_handle* h, double* rho, double* u, double* v,
                                double* w, double* p, double* T);

/* Checkpoints streamed between a file and the device, in the format of
 * Block3d::output_bin / read_bin (src/Block3d.cpp:964-987, :318-357): t_cur
 * (binary64), IM_G, JM_G, KM_G (uint32), then Q in the get_idx_Q layout.
 * cbns_load_checkpoint replaces Block3d::read_bin + cbns_upload_Q on restart
 * (src/cbns3d.cpp:145-153): it checks the padded extents (CBNS_ERR_FORMAT on a
 * mismatch or a short file, CBNS_ERR_IO if the file cannot be opened), streams
 * the state to the device through two pinned chunk buffers, then does what
 * cbns_upload_Q does, with t_cur from the file (*t_out, may be NULL).  A failed
 * load leaves the solve's state unchanged.  cbns_save_checkpoint writes the
 * current Q and t_cur the same way (Block3d::output_bin); the file is byte for
 * byte what cbns_host_output_bin writes for cbns_download_Q's array. */
cbns_status cbns_load_checkpoint(cbns_handle* h, const char* path, double* t_out);
cbns_status cbns_save_checkpoint(cbns_handle* h, const char* path);

/* Block3d::calc_dt (src/Block3d.cpp:515-553): CFL / max over interior cells. */
cbns_status cbns_calc_dt(cbns_handle* h, double* dt);

/* One RK3 stage with a given dt (src/cbns3d.cpp:203-240): rec_riemann_x/y/z,
 * calc_viscous_flux_contribution, update_rk3(dt, stage), boundary_condition and
 * calc_primitive of the stage's output.  stage is 1, 2 or 3. */
cbns_status cbns_stage(cbns_handle* h, double dt, int stage);

/* One iteration of the time loop of src/cbns3d.cpp:176-241: returns
 * CBNS_FINISHED without stepping if t_cur + 1e-5 > t_end (Block3d::is_finished),
 * else dt = calc_dt() clipped to t_end - t_cur, t_cur += dt, three stages.
 * dt_out / t_out may be NULL.  The call waits for the step (cbns_step_async
 * does not). */
cbns_status cbns_step(cbns_handle* h, double t_end, double* dt_out, double* t_out);

/* nsteps iterations of cbns_step as a replayed CUDA graph with the
 * is_finished test, dt and t_cur kept on the device; steps taken go to
 * *steps_done (may be NULL). */
cbns_status cbns_run(cbns_handle* h, uint32_t nsteps, double t_end, uint32_t* steps_done);

/* Asynchronous forms of cbns_upload_Q, cbns_step and cbns_download_Q, for a
 * Block3d-style driver that keeps one handle and wants the host copies of one
 * state to overlap the kernels of the next step (the loop of
 * src/cbns3d.cpp:176-241 with get_Q/checkpoint output between steps).  Each
 * call only enqueues work and returns:
 *   cbns_upload_Q_async    the host copy of Q, then the start-up sequence of
 *                          cbns_upload_Q; t_cur = t;
 *   cbns_step_async        one step of cbns_step (the is_finished test, dt,
 *                          three stages), as a replayed CUDA graph;
 *   cbns_download_Q_async  the current Q into a host array.
 * Work runs in call order.  Host copies go to two more streams of the handle
 * (one per direction), through staging buffers of their own (the first
 * asynchronous call allocates one more state-sized device buffer,
 * NEQ*IM_G*JM_G*KM_G doubles), so a download overlaps the steps enqueued after
 * it and an upload overlaps the steps enqueued before it.  Q must stay valid and unchanged (upload) or
 * untouched (download) until cbns_wait returns; pass page-locked host memory
 * (cudaMallocHost / cudaHostRegister) for the copies to overlap: with pageable
 * memory the call still works but returns only once its copy is done.
 * cbns_wait waits for everything enqueued on the handle and returns the status
 * cbns_step would (CBNS_FINISHED once t_end is reached, CBNS_ERR_NONPHYSICAL
 * after a bad state), with the last dt and t_cur (either may be NULL).
 * cbns_poll sets *done to 1 when nothing enqueued is still running, without
 * waiting. */
cbns_status cbns_upload_Q_async(cbns_handle* h, const double* Q, double t);
cbns_status cbns_step_async(cbns_handle* h, double t_end);
cbns_status cbns_download_Q_async(cbns_handle* h, double* Q);
cbns_status cbns_wait(cbns_handle* h, double* dt_last, double* t_cur);
cbns_status cbns_poll(cbns_handle* h, int* done);

/* Current simulated time and last dt, read from the device. */
cbns_status cbns_get_time(cbns_handle* h, double* t_cur, double* dt_last);

/* Kinetic energy and enstrophy of the current state (project-defined
 * diagnostics, absent from the reference): KE = sum(0.5*rho*|u|^2)/N,
 * Omega = sum(0.5*rho*|curl u|^2)/N over interior cells, N = IM*JM*KM, with the
 * 4th-order central difference of src/calc_gradient.cpp:29-64 for the curl and
 * compensated binary64 sums. */
cbns_status cbns_diagnostics(cbns_handle* h, double* ke, double* enstrophy);

/* Device status word: CBNS_OK, or CBNS_ERR_NONPHYSICAL once any stage met
 * rho <= 0, p <= 0 or a NaN.  Clears the word. */
cbns_status cbns_check_state(cbns_handle* h);

/* The handle's cudaStream_t (as void*), for callers that time or order work. */
void* cbns_stream(cbns_handle* h);

/* Device bytes cbns_create would allocate for a block of these extents (the
 * admission test of the serving loop). */
cbns_status cbns_footprint(uint32_t IM, uint32_t JM, uint32_t KM, int precision, uint64_t* bytes);

/* Block extents and device bytes the handle holds. */
cbns_status cbns_get_info(cbns_handle* h, uint32_t dims[3], uint64_t* device_bytes,
                          int* precision);

/* ---- Batched ensembles ---------------------------------------------------
 * A batch steps many independent solves (uneven grid sizes and parameters)
 * together: each kernel of a step is one launch over a flattened table of the
 * tiles of every solve, optionally persistent (a fixed number of CTAs per SM
 * walking the table), and a step of the whole batch is one replayed CUDA graph.
 * Every solve keeps its own t_cur, t_end, dt and is_finished test on the
 * device, so solves that finish early stop while the others go on.  The handles
 * keep their state; the batch owns only descriptor and tile tables.  All handles
 * must be on one device and share one precision.  Results are bitwise those of
 * stepping each handle alone. */
typedef struct cbns_batch cbns_batch;

typedef struct cbns_launch_config {
  int tile_rows;     /* rows of 32 cells per tile (CTA of 32*tile_rows threads): 2, 4 or 8 */
  int ctas_per_sm;   /* persistent CTAs per SM; 0 = one CTA per tile (not persistent) */
} cbns_launch_config;

cbns_status cbns_batch_create(cbns_handle* const* handles, int n, cbns_batch** out);
cbns_status cbns_batch_destroy(cbns_batch* b);
/* nsteps batch steps (each solve stops at its own t_end); per-solve steps taken
 * since the batch was created go to steps_out[n] (may be NULL). */
cbns_status cbns_batch_run(cbns_batch* b, uint32_t nsteps, uint32_t* steps_out);
cbns_status cbns_batch_set_config(cbns_batch* b, const cbns_launch_config* cfg);
cbns_status cbns_batch_get_config(cbns_batch* b, cbns_launch_config* cfg);
/* Project autotuner: times `reps` steps of the batch for each candidate launch
 * configuration, keeps the fastest, and restores every solve's device state
 * (the timing steps leave no trace).  ms_out[i] receives the time per step of
 * candidate i (up to cap entries), *ncand their count; both may be NULL. */
cbns_status cbns_batch_autotune(cbns_batch* b, int reps, double* ms_out, int cap, int* ncand);
void* cbns_batch_stream(cbns_batch* b);

/* ---- Serving ---------------------------------------------------------------
 * A continuous-batching request loop.  A worker thread admits queued requests
 * (first come, first served among those that fit) while their device footprint
 * (cbns_footprint) fits the memory budget and fewer than max_active run; each
 * admitted request's state is created on, and stays resident on, the device;
 * all running requests step together as one batch for steps_per_round steps;
 * requests that reach their t_end (or fail, or are cancelled) are retired and
 * their memory goes to the next ones, so requests arriving while others run
 * join at the next round.  Each request's result is bitwise the one stepping it
 * alone gives.  Times in cbns_request_info are seconds on the server's clock. */
typedef struct cbns_server cbns_server;

typedef struct cbns_server_opts {
  int precision;                /* a cbns_precision */
  uint64_t memory_budget_bytes; /* device bytes for request state; 0 = 80% of free memory */
  uint32_t max_active;          /* most requests stepped together; 0 = no limit */
  uint32_t steps_per_round;     /* batch steps between scheduling rounds; 0 = 10 */
  int tile_rows;                /* batch launch shape (cbns_launch_config); 0 = default */
  int ctas_per_sm;
} cbns_server_opts;

typedef struct cbns_request_info {
  int status;        /* CBNS_OK, or the error that retired the request */
  uint32_t steps;    /* RK3 steps taken */
  double t_final;    /* simulated time reached */
  double ke, enstrophy;  /* diagnostics of the final state (status CBNS_OK) */
  double submit_s, admit_s, done_s;
  uint64_t device_bytes;
} cbns_request_info;

typedef struct cbns_server_stats {
  uint64_t submitted, completed, failed;
  uint64_t rounds, batch_builds, cell_steps;
  uint32_t peak_active, queued;
  uint64_t budget_bytes, used_bytes;
  double clock_s;
} cbns_server_stats;

/* Starts a server on the calling thread's current CUDA device (or the one
 * CBNS_DEVICE names); its worker thread owns every solve it admits. */
cbns_status cbns_server_create(const cbns_server_opts* opts, cbns_server** out);
/* Cancels queued and running requests and joins the worker. */
cbns_status cbns_server_destroy(cbns_server* s);
/* A request with a host initial state (get_idx_Q layout, copied at submit).
 * p->t_cur and p->t_end give its start and end time.  keep_state != 0 keeps the
 * final state for cbns_server_result. */
cbns_status cbns_server_submit(cbns_server* s, const cbns_params* p, uint32_t IM, uint32_t JM, uint32_t KM,
                               const double* Q0, int keep_state, uint64_t* id);
/* A request whose initial state is built on the device (cbns_init_tgv). */
cbns_status cbns_server_submit_tgv(cbns_server* s, const cbns_params* p, uint32_t IM, uint32_t JM, uint32_t KM,
                                   uint64_t seed, double amp, int nmodes, int kmax, int keep_state,
                                   uint64_t* id);
/* A request whose initial state is a checkpoint file in the format of
 * cbns_save_checkpoint, read by the worker at admission (cbns_load_checkpoint),
 * so the caller holds no state.  It starts at the file's t_cur (p->t_cur is
 * not used); a file that cannot be read retires the request with CBNS_ERR_IO
 * or CBNS_ERR_FORMAT. */
cbns_status cbns_server_submit_checkpoint(cbns_server* s, const cbns_params* p, uint32_t IM, uint32_t JM,
                                          uint32_t KM, const char* path, int keep_state, uint64_t* id);
cbns_status cbns_server_cancel(cbns_server* s, uint64_t id);
/* Waits for a request (timeout_s < 0: no limit; CBNS_ERR_TIMEOUT if it runs out)
 * and returns its final status. */
cbns_status cbns_server_wait(cbns_server* s, uint64_t id, double timeout_s, cbns_request_info* info);
cbns_status cbns_server_result(cbns_server* s, uint64_t id, double* Q_out);
/* Forgets a finished request (frees its stored result). */
cbns_status cbns_server_release(cbns_server* s, uint64_t id);
cbns_status cbns_server_get_stats(cbns_server* s, cbns_server_stats* out);

/* Per-kernel timing.  Between cbns_profile_begin and cbns_profile_end every kernel
 * the handle launches is bracketed by CUDA events on its stream and launched
 * directly rather than through the step graph.  cbns_profile_end waits for the
 * device and fills up to cap records, one per kernel name, *n set to the count. */
typedef struct cbns_kernel_time {
  char name[32];
  uint32_t launches;
  double total_ms;
} cbns_kernel_time;
cbns_status cbns_profile_begin(cbns_handle* h);
cbns_status cbns_profile_end(cbns_handle* h, cbns_kernel_time* out, int cap, int* n);

/* No counterpart in the reference.  Kinetic energy and enstrophy, as
 * cbns_diagnostics computes them, of a conserved state the caller already holds
 * in its own device memory, computed without allocating anything.  For callers
 * that may not call cudaMalloc while they run: an in-situ monitor called from
 * inside another solver's time loop that must not change the device's memory
 * footprint, a host framework whose caching allocator owns the device budget, a
 * real-time loop that cannot take an allocation's latency or implicit syncs.
 *   Q_dev    device pointer, the reference's Q layout (get_idx_Q, ghosts filled)
 *   out_dev  device pointer to 2 doubles: KE, enstrophy
 *   stream   cudaStream_t (as void*) the two kernels are launched on; NULL = default
 * Asynchronous on `stream`.  Scratch is a static device array of 4096 partial
 * sums (128 KiB, held on every GPU that loads the library until exit), each
 * covering 16384 cells, so IM*JM*KM may be at most 67,108,864 (e.g. 406^3);
 * larger blocks are rejected with CBNS_ERR_BAD_DIMS.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) with that device
 * current; make that first call before any stream capture.  Later calls outside
 * a capture look it up again, so the address stays valid after a
 * cudaDeviceReset; a call inside a capture uses the address found before the
 * capture began.  All calls share the
 * one scratch array: calls whose kernels may overlap on the GPU (unordered
 * streams) race and must be serialised by the caller. */
cbns_status cbns_diagnostics_noalloc(const double* Q_dev, uint32_t IM, uint32_t JM, uint32_t KM, double dx,
                                     double dy, double dz, double* out_dev, void* stream);

/* Text of the last error on this host thread ("" if none). */
const char* cbns_last_error(void);

/* Library version string. */
const char* cbns_version(void);

#ifdef __cplusplus
}
#endif

#endif /* CBNS_GPU_H */
