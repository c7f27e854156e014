/* gbint.h -- C ABI of the GB300 momentum-loop integration engine (libgbint.so).
 *
 * DiFfRG evaluates every loop integral of a flow equation through C++ class templates
 * (Integrator*GPU / Integrator*FiniteT*GPU + QuadratureProvider) that launch one CUDA
 * grid per integral, write one FP64 value per quadrature point to global memory and
 * reduce it with thrust/CUB.  This library replaces the runtime beneath those templates:
 * quadrature storage, device-resident dressing tables, batched fused FP32-compensated
 * (or FP64) evaluation with an in-kernel FP64 cross-block reduction, CUDA-graph replay,
 * and a continuously batching request loop.  The C++ compatibility layer
 * (include/gbint/integrators.hh) keeps the reference class names and calls only this ABI.
 *
 * Plain C types only: pointers, sizes, ints, doubles.  cudaStream_t is passed as void*.
 * Every call returns a status code (GB_OK == 0).  The reference throws std::runtime_error
 * on CUDA errors, bad sizes or a missing device (DiFfRG/src/DiFfRG/common/cuda_prefix.cu:9-14,
 * DiFfRG/include/DiFfRG/physics/integration/integrator_4D_gpu.hh:81,92-93); the C++ layer
 * maps non-zero codes back onto such exceptions.
 */
#ifndef GBINT_H
#define GBINT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBINT_ABI_VERSION 1

/* ------------------------------------------------------------------ status codes */
enum {
  GB_OK = 0,
  GB_EINVAL = 1,     /* malformed argument or descriptor                           */
  GB_ENOMEM = 2,     /* device or pinned allocation failed                          */
  GB_EBUDGET = 3,    /* request refused: it can never fit the context's HBM budget  */
  GB_ETIMEDOUT = 4,  /* gb_wait gave up, or a device-side bounded wait expired       */
  GB_ECUDA = 5,      /* a CUDA runtime call failed (see gb_last_error)               */
  GB_ENODEV = 6,     /* no CUDA device / device index out of range                   */
  GB_EAGAIN = 7,     /* gb_poll: result not ready yet                                */
  GB_EDEVICE = 8,    /* a kernel reported an error flag (bounded wait, bad index)    */
  GB_ECANCELED = 9   /* request was cancelled before it ran                          */
};

/* ------------------------------------------------------------------ enumerations */
/* integrator families -- one per reference class template */
enum {
  GB_FAM_1D = 1,          /* IntegratorGPU<d,NT,K>          integration/integrator_gpu.hh:21-128          */
  GB_FAM_ANGLE = 2,       /* IntegratorAngleGPU<d,NT,K>     integration/integrator_angle_gpu.hh:21-219    */
  GB_FAM_3D = 3,          /* Integrator3DGPU<NT,K>          integration/integrator_3D_gpu.hh:21-197       */
  GB_FAM_4D2ANG = 4,      /* Integrator4D2AngGPU<NT,K>      integration/integrator_4D_2ang_gpu.hh:21-260  */
  GB_FAM_4D = 5,          /* Integrator4DGPU<NT,K>          integration/integrator_4D_gpu.hh:21-263       */
  GB_FAM_CART1 = 6,       /* Integrator1DCartesianGPU       integration/integrator_1D_cartesian_gpu.hh    */
  GB_FAM_CART2 = 7,       /* Integrator2DCartesianGPU       integration/integrator_2D_cartesian_gpu.hh    */
  GB_FAM_CART3 = 8,       /* Integrator3DCartesianGPU       integration/integrator_3D_cartesian_gpu.hh    */
  GB_FAM_2DPQ0 = 9,       /* Integrator2Dpq0GPU             integration/integrator_2Dpq0_gpu.hh:21-243    */
  GB_FAM_2DPX0 = 10,      /* Integrator2Dpx0GPU             integration/integrator_2Dpx0_gpu.hh           */
  GB_FAM_3DPQ0 = 11,      /* Integrator3Dpq0GPU             integration/integrator_3Dpq0_gpu.hh           */
  GB_FAM_3DPX0 = 12,      /* Integrator3Dpx0GPU             integration/integrator_3Dpx0_gpu.hh           */
  GB_FAM_FTQ0 = 13,       /* IntegratorFiniteTq0GPU<d>      integration_finiteT/integrator_finiteTq0_gpu.hh:21-238 */
  GB_FAM_ANGLE_FTQ0 = 14, /* IntegratorAngleFiniteTq0GPU<d> integration_finiteT/integrator_angle_finiteTq0_gpu.hh */
  GB_FAM_4D_FTQ0 = 15,    /* Integrator4DFiniteTq0GPU       integration_finiteT/integrator_4D_finiteTq0_gpu.hh    */
  GB_FAM_FTX0 = 16,       /* IntegratorFiniteTx0GPU<d>      integration_finiteT/integrator_finiteTx0_gpu.hh:21-225 */
  GB_FAM_ANGLE_FTX0 = 17, /* IntegratorAngleFiniteTx0GPU<d> integration_finiteT/integrator_angle_finiteTx0_gpu.hh */
  GB_FAM_4D_FTX0 = 18,    /* Integrator4DFiniteTx0GPU       integration_finiteT/integrator_4D_finiteTx0_gpu.hh:21-249 */
  GB_FAM_CONST = 19,      /* IntegratorConstant<d>          integration/integrator_constant.hh:11-73      */
  GB_FAM_QLOOP = 20,      /* d=4 loop, GL in q on [0,qmax] x cos (benchmark workload C1)            */
  GB_FAM_QLOOP_T = 21     /* finite-T loop, explicit modes n=-M..M, GL in q x cos (workload C2)      */
};

/* catalogue integrands (device code compiled into the library) */
enum {
  GB_IG_POLY = 0,  /* product of polynomials per coordinate (reference test KERNEL)      */
  GB_IG_PROP1 = 1, /* sqrt(1-c^2) G(q^2) G(q^2+p^2+2pqc) Rdot(q^2) * kfac                */
  GB_IG_PROP3 = 3, /* Rdot G_A(q^2) G_B(|q-p|^2) V_C(s) V_D(|q-p/2|^2), 4 x 1D tables     */
  GB_IG_VERT4 = 5, /* 4D vertex loop, two 2D (log x, t) tables                           */
  GB_IG_FTLOOP = 6 /* q^2 G(w,q^2) G(w,|q+p|^2) Rdot(q^2), one 2D (mode, |q|) table       */
};

/* arithmetic of a batch */
enum {
  GB_PREC_FP32C = 0, /* FP32-compensated, the accurate form (double-float per-point factors
                        and sums on the FP32 pipe, FP64 cross-unit reduction): within 1e-9 of
                        FP64 (measured 3e-12 .. 9e-11 on the benchmark workloads)            */
  GB_PREC_FP64 = 1,  /* FP64 evaluation (generic fused kernel)                            */
  GB_PREC_FP32F = 2, /* FP32 per-point factors with Kahan sums: faster, ~1e-8 of FP64       */
  GB_PREC_FP32A = 3  /* the accurate form, as GB_PREC_FP32C                                 */
};

enum { GB_DTYPE_F64 = 0, GB_DTYPE_F32 = 1 };

/* ------------------------------------------------------------------ opaque handles */
typedef struct gb_ctx gb_ctx;
typedef struct gb_table gb_table;
typedef struct gb_batch gb_batch;
typedef uint64_t gb_ticket;

/* ------------------------------------------------------------------ descriptors */
/* Table axes: log-spaced (index linear in ln x) or linear; 2D tables are row-major [n0][n1].
 * Replaces LinearCoordinates1D / LogarithmicCoordinates1D + TexLinearInterpolator{1D,2D}
 * (discretization/grid/coordinates.hh:97-195, physics/interpolation/tex_linear_interpolation_1D.hh:86-106). */
typedef struct {
  int n0, log0;
  double lo0, hi0;
  int n1, log1; /* n1 == 0 for a 1D table */
  double lo1, hi1;
} gb_table_spec;

#define GB_MAX_ARGS 24

/* One integral.  Field meaning follows the reference constructors
 * (QuadratureProvider&, grid_sizes, x_extent[, x0_extent|q0_extent, x0_summands, T]) and get(k, args...). */
typedef struct {
  int family;      /* GB_FAM_*                                                             */
  int integrand;   /* GB_IG_*                                                              */
  int d;           /* template dimension of IntegratorGPU<d>, IntegratorAngleGPU<d>, ...     */
  int n[4];        /* grid_sizes (finite-T x0: spatial orders then the tail order)           */
  int table_base;  /* the integral reads tables[table_base ...] of its batch/request (0: first) */
  double x_extent; /* x = q^2/k^2 in [0, x_extent]; qmax for GB_FAM_QLOOP*                   */
  double x0_extent;/* q0_extent (pq0), x0_extent (px0, finite-T x0)                          */
  int x0_summands; /* explicit Matsubara terms (finite-T x0); M for GB_FAM_QLOOP_T            */
  double T;        /* temperature                                                          */
  double E;        /* typical energy of the Matsubara rule (finite-T q0); 0: reference rule  */
  double k;        /* RG scale                                                             */
  double qmin[3], qmax[3]; /* Cartesian boxes                                              */
  double args[GB_MAX_ARGS]; /* args[0] = constant(); integrand parameters follow             */
} gb_integral;

typedef struct {
  uint64_t submitted, completed, rejected, batches_launched;
  uint64_t points_evaluated;
  double busy_seconds;
  double p50_latency_s, p99_latency_s, max_latency_s;
  uint64_t bytes_in_use, bytes_budget;
} gb_stats;

/* ------------------------------------------------------------------ context */
int gb_version(void);
const char *gb_status_string(int status);
/* hbm_budget_bytes: admission cap for batch work memory (0 = 8 GiB default) */
int gb_ctx_create(int device, size_t hbm_budget_bytes, gb_ctx **out);
int gb_ctx_destroy(gb_ctx *ctx);
int gb_last_error(gb_ctx *ctx, char *buf, size_t len);

/* ------------------------------------------------------------------ QuadratureProvider
 * get_points/get_weights (Gauss-Legendre on [0,1]) and get_matsubara_points/weights:
 * common/quadrature/quadrature_provider.hh:138-248.  Host arrays are FP64; device arrays are
 * of dtype.  Pointers stay valid until gb_ctx_destroy (the provider owns them for the
 * process lifetime, as in the reference). */
int gb_quad_gl(gb_ctx *ctx, int order, int dtype, const double **h_nodes, const double **h_weights,
               const void **d_nodes, const void **d_weights);
/* The rule of a QuadratureType (common/quadrature/quadrature.hh:47, same order): Quadrature<NT>::reinit
 * (quadrature.cu:12-60) takes GSL's fixed types with a = 0, b = 1, alpha = beta = 0:
 *   GB_QUAD_LEGENDRE   [0,1], weight 1 (the rule of gb_quad_gl)
 *   GB_QUAD_CHEBYSHEV  [0,1], weight 1/sqrt(x (1-x))
 *   GB_QUAD_LAGUERRE   [0,inf), weight exp(-x)
 *   GB_QUAD_HERMITE    (-inf,inf), weight exp(-x^2)
 *   GB_QUAD_JACOBI     [0,1], weight (1-x)^0 x^0 (the Legendre rule)
 * Nodes ascending.  Cached per (type, order) like gb_quad_gl; an unknown type is GB_EINVAL
 * ("Unknown quadrature type", as the reference throws). */
enum { GB_QUAD_LEGENDRE = 0, GB_QUAD_CHEBYSHEV = 1, GB_QUAD_LAGUERRE = 2, GB_QUAD_HERMITE = 3, GB_QUAD_JACOBI = 4 };
int gb_quad_rule(gb_ctx *ctx, int type, int order, int dtype, const double **h_nodes, const double **h_weights,
                 const void **d_nodes, const void **d_weights);
/* The same rule into caller arrays of `order` doubles; host only, needs no context or GPU. */
int gb_quad_rule_host(int type, int order, double *nodes, double *weights);
/* Monien rule for (T, E): MatsubaraStorage::get_matsubara_quadrature (quadrature_provider.cu:12-58).
 * *size receives the rule size, *T_rule the rule's own T (0 for the vacuum form). */
int gb_quad_matsubara(gb_ctx *ctx, double T, double E, int dtype, int *size, const double **h_nodes,
                      const double **h_weights, const void **d_nodes, const void **d_weights, double *T_rule);
/* /integration/{min_matsubara_size, vacuum_quad_size, add_matsubara_size} (quadrature_provider.cu:220-227) */
int gb_quad_config(gb_ctx *ctx, int min_matsubara_size, int vacuum_quad_size, int add_matsubara_size);

/* ------------------------------------------------------------------ dressing tables
 * Device-resident FP32 tables, double-buffered with an epoch: an update writes the back
 * buffer on `stream` and becomes visible to work enqueued after it on that stream.
 * Replaces TexLinearInterpolator*::update() (tex_linear_interpolation_1D.cu:169-186), which
 * copies and then calls cudaDeviceSynchronize. */
int gb_table_create(gb_ctx *ctx, const gb_table_spec *spec, gb_table **out);
int gb_table_update(gb_ctx *ctx, gb_table *t, const float *host_data, void *stream);
int gb_table_update_device(gb_ctx *ctx, gb_table *t, const float *device_data, void *stream);
/* Several tables updated as one step (a right-hand side's dressing functions): between
 * gb_table_group_begin and gb_table_group_end the serving loop launches no new batch, so every
 * served request sees all updates of the group or none of them.  Blocks nest. */
int gb_table_group_begin(gb_ctx *ctx);
int gb_table_group_end(gb_ctx *ctx);
/* n tables from host data in one call, as one group: one serving fence, the n copies on
 * `stream`, one directory write for all of them (instead of one per table).  Each table at most
 * once in the list. */
int gb_table_update_many(gb_ctx *ctx, int n, gb_table *const *tables, const float *const *host_data, void *stream);
int gb_table_epoch(gb_ctx *ctx, gb_table *t, uint64_t *epoch);
int gb_table_destroy(gb_ctx *ctx, gb_table *t);

/* ------------------------------------------------------------------ batches
 * A batch is a fixed list of integrals planned once (work units, node arrays, scratch) and
 * run many times: the request_data/update_data fan-out of physics/utils.hh:115-147 as one
 * submission.  tables[] are referenced by position (integrand-specific: PROP1 t0 = Z;
 * PROP3 t0..t3 = A,B,C,D; VERT4 t0 = A, t1 = B; FTLOOP t0 = Z(mode,|q|)). */
int gb_batch_create(gb_ctx *ctx, const gb_integral *items, int n, gb_table *const *tables, int n_tables,
                    int precision, gb_batch **out);
/* Enqueue one evaluation on `stream` (NULL: the context stream).  d_out: device array of n
 * doubles, or NULL to keep results in the batch's own device buffer. */
int gb_batch_run(gb_ctx *ctx, gb_batch *b, double *d_out, void *stream);
/* Same, replayed from a CUDA graph captured at the first call (fixed sweeps). */
int gb_batch_run_graph(gb_ctx *ctx, gb_batch *b, void *stream);
/* Copy the results of the last run to host (synchronises `stream`). */
int gb_batch_results(gb_ctx *ctx, gb_batch *b, double *host_out, void *stream);
/* End-to-end synchronous evaluation: run + D2H into host_out. */
int gb_batch_get(gb_ctx *ctx, gb_batch *b, double *host_out, void *stream);
/* Reference execution pattern in FP64: one launch per integral writing one value per point
 * to global memory, CUB DeviceReduce, D2H and a sync per integral, integrals spread over
 * n_streams pooled streams (integrator_4D_gpu.hh:141-197).  The 20x denominator. */
int gb_batch_run_plain(gb_ctx *ctx, gb_batch *b, double *host_out, int n_streams);
/* points of the tensor-product grids (as the reference counts them) */
int gb_batch_info(gb_ctx *ctx, gb_batch *b, uint64_t *points, int *n_units, int *n_items);
int gb_batch_destroy(gb_ctx *ctx, gb_batch *b);

/* one-shot synchronous get(): constant(k,args) + integral, in `precision` */
int gb_get(gb_ctx *ctx, const gb_integral *item, gb_table *const *tables, int n_tables, int precision,
           double *out);

/* Allocation-free get() in FP64 -- no counterpart in the reference.  For callers that cannot let
 * the library allocate device memory while they integrate: a host program whose HBM belongs to
 * another allocator (a caching or pool allocator that reserved it at start-up, or a fixed budget
 * granted once), and callers on a latency-critical path, where cudaFree (and possibly cudaMalloc)
 * would wait for the whole device.  It calls no cudaMalloc/cudaFree nor any allocating library
 * routine; its scratch is one fixed file-scope device array of GB_NOALLOC_SCRATCH_BYTES per
 * device, held by every GPU that loads the library until process exit.  Limit:
 * GB_NOALLOC_MAX_POINTS grid points per integral (larger ones return GB_EINVAL, nothing runs).
 * The first call on a device looks up the array's device address (cudaGetSymbolAddress with
 * that device current) -- make it before any CUDA stream capture begins.  All calls on a device
 * share the array, which keeps the last call's contents (the counters are cleared before each
 * launch): calls through one context serialise, calls from two contexts whose work overlaps on
 * the GPU race.  The call runs at once on the context's stream and waits for it, returning with
 * the result in *out; a CUDA graph being captured on another stream does not record it (a replay
 * does not evaluate the integral again).  Waiting on a stream is a potentially unsafe call in
 * CUDA's stream-capture rules: made while this thread captures in global or thread-local mode,
 * or while any thread captures in global mode, it invalidates that capture (CUDA's error
 * cudaErrorStreamCaptureInvalidated at the capture's end).  Call it outside such captures, or
 * capture in relaxed mode.  A quadrature axis seen for the first time is uploaded into the node
 * pool on the context's stream (from pageable host memory: use each axis once before a capture
 * begins).  Results equal gb_get(..., GB_PREC_FP64, ...). */
#define GB_NOALLOC_MAX_POINTS 4194304
#define GB_NOALLOC_SCRATCH_BYTES 36864
int gb_get_noalloc(gb_ctx *ctx, const gb_integral *item, gb_table *const *tables, int n_tables, double *out);

/* ------------------------------------------------------------------ user-kernel launches
 * Runtime side of the C++ class templates (include/gbint/integrators.hh), which compile the
 * user's KERNEL into a fused kernel in the user's translation unit.  A slot is the per-request
 * state the reference takes from its RMM pool and rmm::cuda_stream_pool
 * (integrator_4D_gpu.hh:141-197): a pooled stream, FP64 partials for up to `units` work units,
 * two counters (cleared on the slot's stream by acquire), a device result and a pinned host copy.
 * request() launches on slot.stream right away; gb_slot_wait is the future's get(). */
typedef struct {
  double *partials; /* device, capacity_units entries                 */
  int *counters;    /* device: [0] work-unit counter, [1] arrivals     */
  double *result;   /* device: the reduced integral                    */
  void *stream;     /* cudaStream_t the request runs on                */
  int capacity_units;
  int id;
} gb_slot;
/* Device buffers owned by the context (counted against its HBM budget): the data of the
 * interpolator objects of the C++ layer (TexLinearInterpolator*::update copies host data and
 * synchronises, tex_linear_interpolation_1D.cu:169-186; gb_buffer_upload copies synchronously). */
int gb_buffer_create(gb_ctx *ctx, size_t bytes, void **d_ptr);
int gb_buffer_upload(gb_ctx *ctx, void *d_ptr, const void *host, size_t bytes);
int gb_buffer_destroy(gb_ctx *ctx, void *d_ptr);
int gb_slot_acquire(gb_ctx *ctx, int units, gb_slot *out);
int gb_slot_wait(gb_ctx *ctx, const gb_slot *slot, double *out);
int gb_slot_release(gb_ctx *ctx, const gb_slot *slot);
/* A pinned host buffer of at least `bytes` owned by the slot (kept and grown across uses) for
 * the uploads and read-backs of a batched launch; valid while the slot is held. */
int gb_slot_host(gb_ctx *ctx, const gb_slot *slot, size_t bytes, void **host);
int gb_device_info(gb_ctx *ctx, int *device, int *num_sms);

/* ------------------------------------------------------------------ autotuner
 * Work-unit schedule of the FP32-compensated kernels (no reference counterpart; the reference
 * takes a max_block_size from its JSON settings and launches one grid per integral).  The
 * kernels evaluate quadrature rows (a row = the outer nodes of a point, its inner loop runs in
 * one thread) in work units that persistent CTAs claim from an atomic counter.  A schedule is:
 *   threads          CTA width, 128, 256 or 512;
 *   rows_per_thread  rows of a work unit per thread, 1, 2 or 4 (unit = threads x this);
 *   inner_split      GB_KIND_S3 / S3R / S5Z only: parts each row's inner (S3: phi) or middle
 *                    (S5Z: c2) loop is split into, each on its own thread, 1, 2 or 4;
 *   unit_order       GB_ORDER_ITEM: units go out in item order; GB_ORDER_COST: largest cost
 *                    (rows x inner points) first, so the long units of uneven integrals do not
 *                    end the launch.  Results do not depend on the order (every unit writes its
 *                    partial to its item-order slot and the finish sums slots in order).
 * gb_autotune times, for every kind present in the integrals, the schedule parameters one at a
 * time on a batch of them (widths; then rows per thread; then the split; then the order, each
 * at the best of the previous ones; a cold L2 before every timed run) and keeps the fastest in
 * the context; batches created afterwards use it.  With cache_path (NULL: none) choices are
 * read from / written to a text file keyed by GPU model and SM count, and a cached kind is not
 * timed again unless flags has GB_TUNE_REFRESH.  chosen (may be NULL) receives the 16 per-slot
 * widths (0 = default), indexed by kind slot = GB_KIND_* (+ 8 for the double-float form used by
 * GB_PREC_FP32C/FP32A).  gb_tune_report copies the last gb_autotune's measurements as JSON
 * (every candidate's median milliseconds per parameter, the default's and the chosen
 * schedule's) into buf (cap bytes, NUL-terminated; *len = full length).
 * GB_KIND_S5Z is the 4D vertex kernel that reads its 2D tables through slices along their cos
 * axis (double-float form only; used when the slices fit shared memory, else GB_KIND_S5).
 * GB_KIND_S3R is the 3D loop kernel that reads its three point-dependent 1D tables through
 * per-cell records (double-float form only; used when the tables are log tables with cells at
 * most 12 % wide, else GB_KIND_S3).
 * A zero field means the kind's default (S1: 128 threads; S2, S3: 256; S5: 512; S5Z: 256 with
 * the c2 loop split in two; one row per thread, item order).  gb_tune_set pins one slot's width
 * by hand (0 = default width); gb_tune_set_schedule pins a whole schedule; gb_tune_get_schedule
 * reads the schedule a batch would use now, defaults filled in. */
enum { GB_KIND_S1 = 1, GB_KIND_S2 = 2, GB_KIND_S3 = 3, GB_KIND_S5 = 5, GB_KIND_S5Z = 6, GB_KIND_S3R = 7, GB_KIND_ACC = 8 };
enum { GB_ORDER_ITEM = 0, GB_ORDER_COST = 1 };
#define GB_TUNE_REFRESH 1
typedef struct gb_schedule {
  int threads;
  int rows_per_thread;
  int inner_split;
  int unit_order;
} gb_schedule;
int gb_autotune(gb_ctx *ctx, const gb_integral *items, int n, gb_table *const *tables, int n_tables, int precision,
                const char *cache_path, int flags, int *chosen);
int gb_tune_set(gb_ctx *ctx, int kind_slot, int threads);
int gb_tune_set_schedule(gb_ctx *ctx, int kind_slot, const gb_schedule *schedule);
int gb_tune_get_schedule(gb_ctx *ctx, int kind_slot, gb_schedule *out);
int gb_tune_report(gb_ctx *ctx, char *buf, size_t cap, size_t *len);

/* ------------------------------------------------------------------ CUDA-graph sweeps
 * A fixed sweep -- several gb_batch_run calls in order on one caller stream, e.g. every
 * right-hand side of a timestep -- captured once and replayed with one graph launch
 * (no reference counterpart: the reference launches every integral separately).  Between
 * gb_graph_capture_begin and gb_graph_capture_end, gb_batch_run on that stream (NULL: the
 * context's stream) is recorded, not executed.  Table updates and result reads are refused on a capturing stream: tables are
 * updated before gb_graph_launch and read when the replay runs; results are read after it. */
typedef struct gb_graph gb_graph;
int gb_graph_capture_begin(gb_ctx *ctx, void *stream);
int gb_graph_capture_end(gb_ctx *ctx, void *stream, gb_graph **out);
int gb_graph_launch(gb_ctx *ctx, gb_graph *g, void *stream);
int gb_graph_info(gb_ctx *ctx, gb_graph *g, int *kernel_launches);
int gb_graph_destroy(gb_ctx *ctx, gb_graph *g);

/* ------------------------------------------------------------------ serving (request loop)
 * Replaces the request()/get() fan-out of a flow's right-hand side (physics/utils.hh:31-147;
 * integrator request() launches, e.g. integration/integrator_angle_gpu.hh:166-219) with one
 * continuously batching loop per context.
 * gb_serve_start: up to max_inflight_batches device batches in flight (1..64); a batch merges
 *   consecutive queued requests of one precision up to max_batch_items integrals.
 * gb_submit: queue one request of n integrals (tables: that request's tables, as in
 *   gb_batch_create); returns a ticket at once.  Work that arrives while other batches are
 *   on the GPU is launched on another stream as soon as a slot frees and its buffers fit the
 *   HBM budget (GB_EBUDGET: a request that can never fit).  A batch starts after the latest
 *   gb_table_update issued before it and reads one epoch of every table; a table update
 *   waits for batches in flight.
 * gb_poll: GB_OK and n results in out, GB_EAGAIN while pending; the ticket is consumed on any
 *   other return.  gb_wait blocks (timeout_s <= 0: no limit; GB_ETIMEDOUT keeps the ticket).
 * gb_cancel: GB_OK if still queued (its gb_poll then returns GB_ECANCELED), GB_EAGAIN if it
 *   already runs.
 * gb_get_stats: counts, busy time, p50/p99/max latency (submit -> result ready, nearest rank)
 *   since gb_serve_start / gb_reset_stats, and the budget in use. */
int gb_serve_start(gb_ctx *ctx, int max_inflight_batches, int max_batch_items);
/* The device-resident request loop, the other serving mode (a loop on the GPU that takes
 * request() calls as they arrive; replaces the same fan-out as gb_serve_start).
 * gb_submit then writes each request straight into a ring the GPU reads (descriptors and a
 * snapshot of its tables' directory entries in the request's ring slot, then the published
 * work-unit count in mapped host memory); a persistent kernel claims published units of 1024
 * grid points as CTAs free up, so requests arriving while others run are batched continuously;
 * results and a done flag land in mapped host memory.  Requests are evaluated in FP64, equal to
 * gb_get(..., GB_PREC_FP64) to rounding and bit-identical alone or in any mix.  ring_slots (1..64) requests in
 * flight, each up to max_items integrals and max_units work units (device memory reserved at
 * start against the HBM budget; larger requests: GB_EBUDGET); a request waits for its slot.  The
 * loop leaves after idle_seconds without work (a bounded clock64 spin, counted as an idle exit)
 * and is relaunched by the next gb_submit / gb_wait; table updates wait for published requests.
 * gb_poll / gb_wait / gb_get_stats / gb_reset_stats / gb_serve_stop act on it as on the host
 * loop; gb_cancel returns GB_EAGAIN (published at submit). */
int gb_serve_start_device(gb_ctx *ctx, int ring_slots, int max_items, long long max_units, double idle_seconds);
/* launches of the loop kernel so far, CTAs that left after the idle budget, whether it runs now */
int gb_serve_device_info(gb_ctx *ctx, long long *launches, int *idle_exits, int *running);
int gb_serve_stop(gb_ctx *ctx);
int gb_submit(gb_ctx *ctx, const gb_integral *items, int n, gb_table *const *tables, int n_tables, int precision,
              gb_ticket *out);
int gb_poll(gb_ctx *ctx, gb_ticket t, double *out);
int gb_wait(gb_ctx *ctx, gb_ticket t, double *out, double timeout_s);
int gb_cancel(gb_ctx *ctx, gb_ticket t);
int gb_get_stats(gb_ctx *ctx, gb_stats *out);
int gb_reset_stats(gb_ctx *ctx);

/* ------------------------------------------------------------------ diagnostics
 * Throughput probes of this GPU (no reference counterpart): FP32 FMA (TFLOP/s, FMA = 2 flops),
 * MUFU lg2 (G ops/s) and FP64 FMA (TFLOP/s), each timed with CUDA events over the whole
 * device.  They are the denominators of the engine's roofline. */
int gb_measure_peaks(gb_ctx *ctx, double *fp32_tflops, double *mufu_gops, double *fp64_tflops);
/* Failure-detection self-test: one kernel waits on an mbarrier that nothing completes, with the
 * same bounded wait the TMA staging uses but a limit of max_cycles (1..2^31) SM cycles.  Returns
 * GB_ETIMEDOUT when the wait gave up and recorded its error flag (the expected outcome); the
 * context stays usable and its error word is left as it was. */
int gb_selftest_wait(gb_ctx *ctx, long long max_cycles);

#ifdef __cplusplus
}
#endif
#endif /* GBINT_H */
