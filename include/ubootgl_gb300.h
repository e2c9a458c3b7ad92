/*
 * ubootgl_gb300 -- C ABI of the GB300 (sm_103a) fluid step.
 *
 * This is the drop-in boundary for ubootgl's hot path: the 2-D staggered-MAC
 * fluid time step `Simulation::step` (simulation.cpp:356-374) and its
 * multigrid pressure solver `class MG` (pressure_solver.hpp:13-76) of
 * te42kyfo/ubootgl.  Each entry point below names the reference interface it
 * replaces.  The C++ classes in ubootgl_gb300/simulation.hpp wrap these calls
 * with the reference's own class and method names.
 *
 * Conventions
 *  - Grids are row-major, element (x, y) at y*width + x, exactly as
 *    Single2DGrid / DoubleBuffered2DGrid (db2dgrid.hpp:12-108).  For a
 *    simulation of width W and height H: p, f, flag are W x H; vx is
 *    (W-1) x H; vy is W x (H-1).
 *  - Host pointers ("const float *" arguments of the non-_device calls) are
 *    plain host memory; the call copies through the handle's own stream and
 *    returns after the copy is complete.
 *  - Every function returns UBG_OK (0) or a negative UBG_E* code; the message
 *    of the last error on the calling thread is ubg_last_error().  No C++
 *    exception crosses this boundary.  The reference has no error path (void
 *    functions, asserts compiled out by -DNDEBUG).
 *  - Flags must be exactly 0.0 (solid) or 1.0 (fluid), which is what the
 *    reference's terrain produces (terrain.cpp:3-11); they are stored on the
 *    device as one byte per cell.  Other values are rejected (UBG_EINVAL).
 *  - One CUDA stream per handle; distinct handles may be used from different
 *    threads.  A handle must not be used by two threads at once.
 *  - No CPU fallback: without a usable CUDA device every call that needs the
 *    GPU returns UBG_ECUDA.
 */
#ifndef UBOOTGL_GB300_H
#define UBOOTGL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define UBG_OK 0
#define UBG_EINVAL -1  /* bad argument (size, flag value, field id, ...) */
#define UBG_ECUDA -2   /* CUDA runtime error (message in ubg_last_error) */
#define UBG_ENOMEM -3  /* device or host allocation failed / over budget */
#define UBG_ESTATE -4  /* call not valid in the current state */
#define UBG_ETIMEOUT -5 /* a bounded device-side wait ran out */
#define UBG_EBUSY -6   /* admission refused (server at capacity) */

/* Boundary types, Simulation::BC (simulation.hpp:69). */
enum ubg_bc { UBG_BC_INFLOW = 0, UBG_BC_OUTFLOW = 1, UBG_BC_OUTFLOW_ZERO_PRESSURE = 2, UBG_BC_NOSLIP = 3 };

/* Fields of Simulation (simulation.hpp:128-134).  VX/VY are the front
 * buffers (vx.f(), vy.f()); VX_BACK/VY_BACK the back buffers (vx.b()).
 * VX_CURRENT/VY_CURRENT are the display copies that step() leaves
 * (saveCurrentVelocityFields, simulation.cpp:16-19); they read the front
 * buffer as of the end of the last step.  FLAG is read/written as float. */
enum ubg_field {
  UBG_VX = 0,
  UBG_VY = 1,
  UBG_VX_BACK = 2,
  UBG_VY_BACK = 3,
  UBG_P = 4,
  UBG_F = 5,
  UBG_FLAG = 6,
  UBG_VX_ACCUM = 7,
  UBG_VY_ACCUM = 8,
  UBG_VX_CURRENT = 9,
  UBG_VY_CURRENT = 10
};

/* Pressure-solver policy (extension; the reference always runs exactly two
 * V-cycles, simulation.cpp:189-190, and never looks at the residual). */
enum ubg_solver_mode {
  UBG_SOLVE_FIXED = 0,     /* `vcycles` V-cycles (2 = the reference) */
  UBG_SOLVE_TOLERANCE = 1  /* flexible CG preconditioned by one V-cycle per
                              iteration until ||r|| <= tol * ||f_c|| (FP64 norms
                              over the interior fluid cells) or max_vcycles.  The
                              system has zero-gradient edges everywhere and is
                              singular; f_c is f with its sum over the fluid cells
                              moved onto the fluid cells of the outflow column
                              x = W-2.  The pressure iterate is double-float; a
                              solve that ends above the residual it started from
                              keeps its starting pressure.  The solve waits on the
                              host for its residuals, so a tolerance step is not
                              captured into a graph. */
};

/* Precision of the multigrid corrections (extension).  FP32 is the
 * reference's arithmetic.  TOLERANCE mode: the preconditioner's level 0 is
 * always FP32; MIXED_* store the coarse levels in FP16 / BF16 (scaled by a
 * power of two found on the device, FP32 arithmetic).  FIXED mode: MIXED_*
 * run an FP32 defect-correction loop (residual and p += e in FP32) whose
 * inner V-cycle stores the error equation in FP16 / BF16 on every level and
 * solves the coarse levels (<= 2048 cells) in FP64; k corrections equal (in
 * exact arithmetic) k V-cycles of the reference started from p with
 * zero-gradient edges. */
enum ubg_precision { UBG_FP32 = 0, UBG_MIXED_FP16 = 1, UBG_MIXED_BF16 = 2 };

typedef struct ubg_options {
  int solver_mode;    /* ubg_solver_mode, default UBG_SOLVE_FIXED */
  int vcycles;        /* FIXED mode: V-cycles per projection, default 2 */
  float tol;          /* TOLERANCE mode: relative residual target, default 1e-6 */
  int max_vcycles;    /* TOLERANCE mode: cap, default 100 */
  int precision;      /* ubg_precision, default UBG_FP32 */
  int use_graph;      /* capture the step into a CUDA graph, default 1 */
  int advect_bilinear; /* 1: advection samples with bilinearSample (interpolators.hpp:11-27)
                          instead of bicubicSample (extension); default 0, the reference */
} ubg_options;

typedef struct ubg_sim ubg_sim;
typedef struct ubg_mg ubg_mg;

/* Last error message of the calling thread ("" if none). */
const char *ubg_last_error(void);

/* Library / device information: writes a short JSON object. */
int ubg_device_info(char *buf, size_t len);

/* Page-locked host memory for fast ubg_upload / ubg_download (extension; the
 * reference keeps its fields in std::vector). */
int ubg_host_alloc(size_t bytes, void **ptr);
int ubg_host_free(void *ptr);

/* ---------------------------------------------------------- Simulation */

/* Simulation(const Single2DGrid &flag, float pwidth, float mu),
 * simulation.hpp:32-67: allocates all fields on the device, sets the
 * reference's boundary types (W inflow, E outflow with zero pressure, N/S
 * no-slip), vy(x,0) = 0 and vx(0,y) = 1 in both buffers, h = pwidth/(W-1),
 * and builds the multigrid hierarchy from `flag` (MG(flag)).  W, H >= 8. */
int ubg_create(const float *flag, int width, int height, float pwidth, float mu, ubg_sim **out);
int ubg_destroy(ubg_sim *sim);

/* Solver options (see ubg_options); applies from the next step. */
int ubg_default_options(ubg_options *opt);
int ubg_set_options(ubg_sim *sim, const ubg_options *opt);

/* bcWest/bcEast/bcNorth/bcSouth members (simulation.hpp:124). */
int ubg_set_bcs(ubg_sim *sim, int west, int east, int north, int south);

/* Simulation::step(float timestep), simulation.cpp:356-374:
 * applyAccumulatedVelocity, diffuse, advect, setVBCs, project, setVBCs,
 * saveCurrentVelocityFields.  Enqueued on the handle's stream; returns when
 * enqueued (ubg_sync waits). */
int ubg_step(ubg_sim *sim, float dt);

/* The same step with dt = cfl * h / max|u| computed on the device from the
 * current fields (extension: the reference takes dt from its caller,
 * sim_loop.cpp:28).  The dt used is readable with ubg_last_dt after a sync. */
int ubg_step_cfl(ubg_sim *sim, float cfl);
int ubg_last_dt(ubg_sim *sim, float *dt);

/* Pressure-solve statistics of the last step or projection (extension):
 * V-cycles (mixed modes: corrections) run, and in TOLERANCE mode the final
 * ||r|| / ||f * flag|| (else -1).  Host values; no synchronisation. */
int ubg_solver_stats(ubg_sim *sim, int *vcycles, double *rel_residual);

/* Asynchronous host I/O (extension), for callers that feed and read every
 * step without stalling the GPU:
 *  - ubg_io_upload_async copies vx ((W-1) x H) and vy (W x (H-1)) from
 *    pinned host memory into device staging buffers on the handle's I/O
 *    stream; the next step (ubg_step / ubg_step_cfl / a batch step) makes
 *    them the front velocity before its first kernel.
 *  - ubg_io_download_async snapshots the current vx / vy on the device
 *    (ordered after the steps enqueued so far) and copies the snapshot to
 *    pinned host memory on a second I/O stream, overlapping the following
 *    steps and uploads.
 *  - ubg_io_wait waits for every copy of both I/O streams.
 * The host buffers must stay valid, and unmodified (uploads) or unread
 * (downloads), until ubg_io_wait; alternate two sets to overlap steps. */
int ubg_io_upload_async(ubg_sim *sim, const float *vx, const float *vy);
int ubg_io_download_async(ubg_sim *sim, float *vx, float *vy);
int ubg_io_wait(ubg_sim *sim);

/* Individual stages of the step, for callers that drive them one by one and
 * for stage-wise parity tests.  `dt` sets the member Simulation::dt first. */
int ubg_apply_accumulated_velocity(ubg_sim *sim); /* simulation.cpp:376-396 */
int ubg_diffuse(ubg_sim *sim, float dt);          /* simulation.cpp:104-162 */
int ubg_advect(ubg_sim *sim, float dt);           /* simulation.cpp:241-354 */
int ubg_set_vbcs(ubg_sim *sim);                   /* simulation.cpp:80-102 */
int ubg_set_pbc(ubg_sim *sim);                    /* simulation.cpp:36-45 */
int ubg_project(ubg_sim *sim, float dt);          /* simulation.cpp:164-208 */

/* sinks.push_back(glm::vec3(x, y, strength)) (explosion.cpp:33); consumed
 * by project() (simulation.cpp:173-187). */
int ubg_add_sink(ubg_sim *sim, float x, float y, float strength);

/* Host <-> device copies of one field (see ubg_field).  Uploading UBG_FLAG
 * is memcpy(sim.flag.data(), ...) followed by mg.updateFields(sim.flag)
 * (ubootgl_app.cpp:111-112): the coarse flags are rebuilt on the device. */
int ubg_upload(ubg_sim *sim, int field, const float *src);
int ubg_download(ubg_sim *sim, int field, float *dst);

/* ------------------------------------------------ game-side field access */

/* bilinearScatter into the accumulation fields (interpolators.hpp:29-40) as
 * the floating items apply their force to the fluid
 * (advect_floating_items.cpp:116-120, 239-244): for each of n items,
 * xy[2i..2i+1] = pos / h (grid units) and v[2i..2i+1] the values to add;
 * v.x is scattered into vx_accum at xy - (0.5, 0) and v.y into vy_accum at
 * xy - (0, 0.5) (callers pass -deltaVec).  Coordinates are clamped as in the
 * reference.  On the device with atomic adds: items whose stencils overlap
 * sum in an unspecified order.  The next step applies the accumulation. */
int ubg_scatter_accum(ubg_sim *sim, int n, const float *xy, const float *v);

/* Simulation::bilinearVel (advect_floating_items.cpp:11-14) for n points
 * xy (grid units, pos / h) on the device's current vx / vy: out[2i..2i+1]. */
int ubg_sample_velocity(ubg_sim *sim, int n, const float *xy, float *out);

/* Simulation::setGrids(c, val) (simulation.hpp:82-98) for n cells
 * xy[2i..2i+1] with values vals[i] (0.0 or 1.0), in call order: the flag
 * takes the last value, a cell set to 0.0 has its four faces (front
 * buffers) and p zeroed; cells outside the grid are ignored.  The coarse
 * flags and stencil codes are rebuilt (mg.updateFields), as the reference's
 * callers do after editing the flag. */
int ubg_set_grids(ubg_sim *sim, int n, const int *xy, const float *vals);

/* UbootGlApp::shiftMap (ubootgl_app.cpp:245-298) on the device: vx, vy
 * (both buffers from the front) and p move one column west, new_flag (the
 * shifted terrain, width x height, 0.0 / 1.0) is applied cell by cell with
 * setGrids, the inflow column is reset to 0.07 * height / inletArea *
 * flag(0, y), and mg.updateFields runs. */
int ubg_shift_map(ubg_sim *sim, const float *new_flag);

/* Session snapshot / restore (extension, for eviction and checkpoints): a
 * header (magic "UBGSNAP1", version 1, width, height, pwidth, mu, h, last dt,
 * boundary types, sinks), then vx, vx back, vy, vy back, p, f, vx_accum,
 * vy_accum as unpitched float arrays and the flag as bytes.  Restore needs a
 * simulation of the same width and height; solver options are not part of
 * a snapshot. */
int ubg_snapshot_bytes(ubg_sim *sim, size_t *bytes);
int ubg_snapshot(ubg_sim *sim, void *dst);
int ubg_restore(ubg_sim *sim, const void *src);

/* ------------------------------------------- autotuner and batches */

/* Autotuner (extension): times the candidate smoother tiles of every
 * multigrid level (pre- and post-smoothing launches separately) and the
 * sizes of the one-CTA coarse tail on this simulation's own arrays, and
 * keeps the fastest.  The simulation's state is unchanged and results are
 * bit-identical for every choice.  report (may be NULL) receives a JSON
 * object with the per-level choices and times (truncated to len). */
int ubg_autotune(ubg_sim *sim, char *report, size_t len);

/* Batch (extension): n independent simulations of any sizes advanced
 * together, one CUDA graph launch per batch step.  With dt from the device,
 * the FP32 fixed-mode members of at most 2^20 cells (at least two of them)
 * are fused: each kernel of the step is one launch over all of them (blocks
 * mapped to members through prefix sums, per-member arguments in a device
 * table), ~40 launches whatever their count.  The other members' own step
 * bodies run as parallel branches of the same graph.  dts: n host time
 * steps (every member then a branch), or NULL for dt = cfl * h / max|u| per
 * member on the device.  Members keep their own fields, options and
 * streams (ordered after the batch step); each member's result is
 * bit-identical to stepping it alone.  Members need UBG_SOLVE_FIXED and no
 * pending sinks.  The batch does not own the members. */
typedef struct ubg_batch ubg_batch;
int ubg_batch_create(int n, ubg_sim *const *sims, ubg_batch **out);
int ubg_batch_destroy(ubg_batch *batch);
int ubg_batch_step(ubg_batch *batch, const float *dts, float cfl);
int ubg_batch_stream(ubg_batch *batch, void **stream);
int ubg_batch_sync(ubg_batch *batch);

/* Device bytes a simulation of width x height holds (fields + multigrid,
 * FP32 solver), and the bytes a live handle holds now. */
int ubg_device_bytes(int width, int height, size_t *bytes);
int ubg_sim_device_bytes(ubg_sim *sim, size_t *bytes);

/* Diagnostic (no counterpart in the reference): the kernels replace a
 * division x / d by a constant d > 0 with Markstein's correction of
 * x * RN(1/d) (exact for |x| in [2^-100, 2^100], the division otherwise).
 * This compares the two bit for bit on the device for the n host values x
 * and writes the number of differences (0 expected). */
int ubg_selftest_div(const float *x, int n, float d, unsigned *mismatches);

/* ------------------------------------------------------------ step server */

/* Step server (extension): continuous batching of step requests over
 * sessions whose fields stay resident on the device.  Sessions are admitted
 * against a device-memory budget when opened (UBG_EBUSY and a rejection
 * count when the budget is exhausted).  A request asks for `steps` device-CFL
 * steps of one session.  A worker thread admits queued requests in arrival
 * order, one in flight per session, while fewer than max_active stream
 * requests (or 4 * max_active fused requests) are in flight.  In
 * the fused mode (the default) the worker enqueues one step of every
 * in-flight request of an FP32 fixed-mode session of at most 2^20 cells
 * (ubg_server_set_fuse_cells) per iteration, as one launch per kernel over
 * all of them, on a high-priority stream: a request joins at the next step
 * boundary and leaves after its last step.  Other sessions, and every
 * session in the stream mode, run on a pool of max_active host threads,
 * each stepping one request on its session's own stream (a tolerance-mode
 * solve waits on the device once per V-cycle there), and the device
 * overlaps the streams.  Either way a session's results are
 * bit-identical to stepping it alone.  Latency = completion - submission. */
typedef struct ubg_server ubg_server;
typedef struct ubg_serve_stats {
  int sessions, queued, active;
  long long completed, rejected_sessions, cell_steps;
  size_t device_bytes_used;
  double busy_ms;              /* first admission to last completion */
  double p50_ms, p99_ms, max_ms; /* request latencies so far */
  long long fused_steps;         /* fused launch sequences enqueued */
  long long fused_member_steps;  /* session steps they covered */
  double worker_fused_ms;        /* worker time spent enqueueing fused steps */
  double worker_streams_ms;      /* pool-thread time spent enqueueing stream requests */
  int pending_sessions;          /* sessions waiting for device memory (UBG_ADMIT_QUEUE) */
  long long admitted_from_queue; /* sessions admitted after waiting for memory */
} ubg_serve_stats;
int ubg_server_create(size_t budget_bytes, int max_active, ubg_server **out);
int ubg_server_destroy(ubg_server *srv);
#define UBG_SERVE_STREAMS 0 /* every request on its session's stream */
#define UBG_SERVE_FUSED 1   /* fused steps over the in-flight requests (default) */
/* Selects how later-admitted requests are stepped. */
int ubg_server_set_mode(ubg_server *srv, int mode);
/* The largest session (in cells) the fused mode steps fused (default 2^20);
 * larger sessions take their own stream. */
int ubg_server_set_fuse_cells(ubg_server *srv, long long max_cells);
#define UBG_ADMIT_REJECT 0 /* an open over budget fails with UBG_EBUSY (default) */
#define UBG_ADMIT_QUEUE 1  /* it waits, in open order, until closes free the budget */
/* Admission policy of later opens.  With UBG_ADMIT_QUEUE an open that does
 * not fit returns UBG_OK and a session id at once; the inputs are kept in
 * host memory and the session is built (in the thread of the ubg_server_close
 * that frees the memory) when it reaches the front of the line and fits.
 * Requests may be submitted to it meanwhile; they start once it is built.
 * A session larger than the whole budget is still refused. */
int ubg_server_set_admission(ubg_server *srv, int admission);
/* Opens a session (Simulation(flag, pwidth, mu); vx / vy may be NULL, else
 * they initialise both buffers; opt may be NULL). */
int ubg_server_open(ubg_server *srv, const float *flag, int width, int height, float pwidth,
                    float mu, const float *vx, const float *vy, const ubg_options *opt,
                    int *session);
int ubg_server_close(ubg_server *srv, int session);
int ubg_server_submit(ubg_server *srv, int session, int steps, float cfl, uint64_t *request);
int ubg_server_wait(ubg_server *srv, uint64_t request, double *latency_ms);
int ubg_server_drain(ubg_server *srv);
/* The session's simulation handle, for reading its fields while it has no
 * request in flight. */
int ubg_server_session_sim(ubg_server *srv, int session, ubg_sim **sim);
int ubg_server_stats(ubg_server *srv, ubg_serve_stats *out);

/* Multigrid of the simulation: number of levels, size and (float) flag of
 * one level (MG::flagcs, pressure_solver.hpp:72). */
int ubg_mg_levels(ubg_sim *sim, int *levels);
int ubg_mg_level_flag(ubg_sim *sim, int level, int *w, int *h, float *dst);

/* Runs the simulation's mg.solve(p, f, flag, h, zeroGradientBC) once
 * (pressure_solver.hpp:59-62) on the device-resident p and f. */
int ubg_mg_solve_sim(ubg_sim *sim, int zero_gradient_bc);

/* Device views for zero-copy composition with other CUDA code: pointer,
 * row pitch in elements, width, height.  Valid until the next step (the
 * velocity buffers rotate). FLAG is uint8 (one byte per cell). */
int ubg_field_device(ubg_sim *sim, int field, void **ptr, int *pitch, int *w, int *h);
/* The handle's cudaStream_t. */
int ubg_stream(ubg_sim *sim, void **stream);
int ubg_sync(ubg_sim *sim);

/* Per-kernel timing (extension, for the benchmark).  While enabled, steps
 * run as direct launches (no graph) with a CUDA event pair around every
 * kernel; ubg_profile_read gives the mean level-0 smoother launch time, the
 * mean profiled step time and the launch count of the last step;
 * ubg_profile_class gives the accumulated time and launch count of one
 * kernel class (0 <= kc < 19, name returned). */
int ubg_profile_enable(ubg_sim *sim, int on);
int ubg_profile_read(ubg_sim *sim, double *smoother_ms, int *smoother_launches,
                     double *step_ms, int *kernel_launches);
int ubg_profile_class(ubg_sim *sim, int kc, const char **name, double *total_ms, int *count);
int ubg_profile_reset(ubg_sim *sim);

/* ------------------------------------------------------- display tracers */

/* Display velocity texture of the simulation's current fields
 * (VelocityTextures::updateFromStaggered + interp_shader.cs:14-34,
 * velocity_textures.cpp:63-93), computed on the device into a headless
 * buffer: vxy holds (2W-1) x (2H-1) pairs (vx, vy), mag (may be NULL) their
 * lengths.  Host arrays; the call returns when they are filled. */
int ubg_velocity_texture(ubg_sim *sim, float *vxy, float *mag);

/* Fluid tracers (DrawTracersCS's GLTracers, draw_tracers_cs.cpp:131-169 and
 * advect_tracer_points.cs:42-82) as device state bound to a simulation:
 * ntracers rings of npoints positions, ring start / end pointers and ages.
 * All start at zero; upload initial state with ubg_tracers_upload. */
typedef struct ubg_tracers ubg_tracers;
int ubg_tracers_create(ubg_sim *sim, int ntracers, int npoints, ubg_tracers **out);
int ubg_tracers_destroy(ubg_tracers *tr);
/* points: ntracers * npoints * 2 floats; start, end: ntracers each; ages:
 * ntracers.  Any pointer may be NULL to skip that array. */
int ubg_tracers_upload(ubg_tracers *tr, const float *points, const uint32_t *start,
                       const uint32_t *end, const float *ages);
int ubg_tracers_download(ubg_tracers *tr, float *points, uint32_t *start, uint32_t *end,
                         float *ages);
/* updateTracers (draw_tracers_cs.cpp:131-156): rebuilds the velocity texture
 * from the simulation's current fields and advances every tracer by dt;
 * rand_seed is the shader's rand_seed uniform.  Enqueued on the
 * simulation's stream. */
int ubg_tracers_step(ubg_tracers *tr, float dt, uint32_t rand_seed);

/* --------------------------------------------------------------- class MG */

/* MG(int width, int height) (pressure_solver.hpp:16-31), with every coarse
 * flag 1.0; flag != NULL gives MG(Single2DGrid &flag) (pressure_solver.hpp:32),
 * which also runs updateFields(flag). */
int ubg_mg_create(int width, int height, const float *flag, ubg_mg **out);
int ubg_mg_destroy(ubg_mg *mg);
/* MG::updateFields(flag), pressure_solver.hpp:34-57. */
int ubg_mg_update_fields(ubg_mg *mg, const float *flag);
/* MG::solve(p, f, flag, h, zeroGradientBC), pressure_solver.hpp:59-62, on
 * host arrays of width x height; p is updated in place. */
int ubg_mg_solve(ubg_mg *mg, float *p, const float *f, const float *flag, float h,
                 int zero_gradient_bc);
/* Same, on device arrays (row pitch in elements; flag as uint8), enqueued on
 * `stream` (a cudaStream_t, NULL = the handle's stream). */
int ubg_mg_solve_device(ubg_mg *mg, float *p, int p_pitch, const float *f, int f_pitch,
                        const uint8_t *flag, int flag_pitch, float h, int zero_gradient_bc,
                        void *stream);

/* Allocation-free solve.  No counterpart in the reference: it is the
 * ubg_mg_create(flag) + ubg_mg_solve_device pair for callers that must not
 * allocate GPU memory while they run (a fixed device-memory budget owned by
 * a host framework, real-time loops that must not reach the allocator,
 * plug-ins whose host owns every device allocation).  The caller passes device
 * arrays p (in/out), f and flag (bytes 0 / 1), each with its row pitch in
 * elements; the solver's scratch (the level hierarchy) lives in one static
 * 24 MiB device array per GPU, held until the process exits.  Grids whose
 * hierarchy needs more (about 14 bytes x width rounded up to 32 x height x
 * 4/3; 1024 x 1024 fits, 2048 x 1024 does not) return UBG_EINVAL.  The first
 * call on a device looks up the array's address (cudaGetSymbolAddress): make
 * it before any stream capture (on a capturing stream it returns UBG_ESTATE).
 * h must be finite and > 0.  Calls share the array: calls that overlap
 * on the GPU race.  Enqueued on `stream` (a cudaStream_t, NULL = the legacy
 * default stream); returns once enqueued. */
int ubg_mg_solve_noalloc(float *p, int p_pitch, const float *f, int f_pitch, const uint8_t *flag,
                         int flag_pitch, int width, int height, float h, int zero_gradient_bc,
                         void *stream);

/* Free functions of pressure_solver.hpp:3-11 on host arrays:
 * rbgs(p, f, flag, h, alpha) (one red-black sweep, pressure_solver.cpp:35-89)
 * and calculateResidualField(p, f, flag, r, h) (pressure_solver.cpp:91-116;
 * the L2 norm is accumulated in double). */
int ubg_rbgs(float *p, const float *f, const float *flag, int width, int height, float h,
             float alpha);
int ubg_residual(const float *p, const float *f, const float *flag, float *r, int width,
                 int height, float h, double *l2norm);

#ifdef __cplusplus
}
#endif
#endif /* UBOOTGL_GB300_H */
