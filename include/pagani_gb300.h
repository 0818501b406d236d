/*
 * pagani_gb300.h -- C ABI of the GB300-native PAGANI / m-Cubes library.
 *
 * Plain C types only: pointers, sizes, PODs.  One pg_context owns its device
 * memory (region pool, scratch, pinned host mirrors) and its CUDA stream; calls
 * on one context are serialised, different contexts are independent.  No call
 * aborts the process: every entry point returns a pg_status code, and
 * pg_last_error() gives the message of the last failure on a context.
 *
 * Reference interfaces each entry point replaces are cited by file:line of the
 * reference project (marcpaterno/gpuintegration).
 */
#ifndef PAGANI_GB300_H
#define PAGANI_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PG_MAX_DIM 16
#define PG_MIN_NDIM 2
#define PG_MAX_NDIM 12

/* Return codes.  PG_NOT_CONVERGED mirrors the reference's status 1
 * (common/integration_result.hh:17); the negative codes replace the
 * reference's abort() on CUDA errors (common/cuda/cudaDebugUtil.h:119-151) and
 * std::bad_alloc (common/cuda/cudaMemoryUtil.h:198-208). */
typedef enum pg_status {
  PG_OK = 0,
  PG_NOT_CONVERGED = 1,
  PG_BAD_ARG = -1,
  PG_OOM = -2,
  PG_CUDA_ERROR = -3,
  PG_TIMEOUT = -4,
  PG_UNSUPPORTED = -5,
  PG_CANCELLED = -6
} pg_status;

/* Integrand families.  Device functors cannot cross a C ABI, so an integrand
 * is named by family + parameters (the reference passes a functor:
 * cuda/pagani/quad/GPUquad/Workspace.cuh:52-61).  The six Genz families follow
 * common/cuda/integrands.cuh:1303-1934 with per-axis a_i (sharpness) and u_i
 * (offset):
 *   OSCILLATORY     cos(2*pi*u_0 + sum a_i x_i)
 *   PRODUCT_PEAK    prod 1 / (a_i^-2 + (x_i - u_i)^2)
 *   CORNER_PEAK     (1 + sum a_i x_i)^-(d+1)
 *   GAUSSIAN        exp(-sum a_i^2 (x_i - u_i)^2), times c^d when c != 0 (normalised Gaussians)
 *   C0              exp(-sum a_i |x_i - u_i|)
 *   DISCONTINUOUS   0 if any x_i > u_i, else exp(sum a_i x_i)
 * and the test integrands of the reference's own tests:
 *   CONSTANT        c                                  (test/cuda/pagani/RegionSampling.cu:19-44)
 *   PRODUCT         prod x_i                           (test/cuda/pagani/do_integration_from_c.cu:7-14)
 *   NAN_VALUE       NaN                                (test/cuda/pagani/NanIntegral.cu:9-16)
 *   BOX             (sum x_i^2)^(c/2)                  (cuda/pagani/demos/function.cuh:113-172)
 *   FUN6            6-D test function of test/cuda/pagani/accuracy_improves_with_epsrel.cu:17-27
 *   GAUSSIAN_SUM    exp(-sum a_i^2 (x_i - u_i)^2) as one exponential of the sum
 *                   (squares summed in axis order), times c^d when c != 0: the
 *                   form of the reference's m-Cubes Gaussian functors
 *                   (cuda/mcubes/demos/Gauss9D.cu:8-24); one exp per point
 *                   instead of d, not product-form
 * The product-form families (PRODUCT_PEAK, GAUSSIAN, C0, DISCONTINUOUS,
 * PRODUCT) are evaluated as a product of per-axis factors h_i taken in two
 * halves, (h_0 * ... * h_{m-1}) * (h_m * ... * h_{d-1}) with m = ndim / 2, each
 * half in axis order; a caller who needs another order passes a functor
 * through the C++ layer (pagani_gb300.cuh). */
typedef enum pg_family {
  PG_FAMILY_CONSTANT = 0,
  PG_FAMILY_OSCILLATORY = 1,
  PG_FAMILY_PRODUCT_PEAK = 2,
  PG_FAMILY_CORNER_PEAK = 3,
  PG_FAMILY_GAUSSIAN = 4,
  PG_FAMILY_C0 = 5,
  PG_FAMILY_DISCONTINUOUS = 6,
  PG_FAMILY_PRODUCT = 7,
  PG_FAMILY_NAN_VALUE = 8,
  PG_FAMILY_BOX = 9,
  PG_FAMILY_FUN6 = 10,
  PG_FAMILY_GAUSSIAN_SUM = 11,
  PG_FAMILY_COUNT = 12
} pg_family;

typedef struct pg_integrand {
  int32_t family; /* pg_family */
  int32_t ndim;   /* 2..PG_MAX_NDIM */
  double a[PG_MAX_DIM];
  double u[PG_MAX_DIM];
  double c;
} pg_integrand;

/* numint::integration_result (common/integration_result.hh:11-21).  neval is
 * filled here (regions evaluated x points per region); the reference leaves it 0. */
typedef struct pg_result {
  double estimate;
  double errorest;
  double chi_sq;
  uint64_t neval;
  uint64_t nregions;
  uint64_t nfinished;
  uint64_t iters;
  int32_t status;     /* 0 converged, 1 not converged (reference semantics) */
  int32_t last_phase; /* -1 as in the reference */
} pg_result;

/* Region-evaluation modes (pg_options.eval_mode, pg_evaluate_regions' eval_mode).
 * PG_EVAL_POINTS evaluates every point of the degree-9 rule and accumulates
 * the five rule sums point by point in the reference's order
 * (cuda/pagani/quad/GPUquad/Sample.cuh:103-290): estimates, errors and split
 * axes are bit-identical to the reference's own kernel.
 * PG_EVAL_SET_SUMS applies to the product-form families (PRODUCT_PEAK,
 * GAUSSIAN, C0, DISCONTINUOUS, PRODUCT) and falls back to PG_EVAL_POINTS for
 * the others: the nine generator-set sums of f are formed by a recurrence over
 * the axes from the 11 per-axis factor values, so a region costs O(ndim)
 * instead of FEVAL(ndim) point values.  Estimates and errors agree with
 * PG_EVAL_POINTS to about 1e-15 of the region's estimate (the rounding of the
 * sums differs); the split axes are the reference's, because the values the
 * fourth differences read are formed exactly as PG_EVAL_POINTS forms them. */
#define PG_EVAL_POINTS 0
#define PG_EVAL_SET_SUMS 1

/* Options of the PAGANI iteration.  pg_options_default() gives the reference's
 * behaviour: relative-error classification on (Workspace.cuh:360-368), 700
 * iterations (Workspace.cuh:399), and the heuristic classifier's device-memory
 * model fixed at 16e9 bytes (heuristic_classifier.cuh:89-94). */
typedef struct pg_options {
  int32_t relerr_classification;
  int32_t max_iters;
  double device_mem_model;  /* bytes seen by the memory-pressure classifier */
  uint64_t max_regions;     /* hard cap of the region pool (0 = derived from the model) */
  int32_t eval_mode;        /* PG_EVAL_POINTS (default) or PG_EVAL_SET_SUMS */
  int32_t predict_split;    /* 1: the reference's predict_split variant (Workspace.cuh:415-441): no rel-err
                               classification in the first 15 iterations while the list has <= 15e6 regions and
                               nothing has finished; the list of iteration 15 is kept (pg_last_snapshot) */
} pg_options;

typedef struct pg_context pg_context;

/* Kernel-level counters of a context (CUDA-event timed when profiling is on). */
typedef struct pg_stats {
  uint64_t launches;         /* kernels launched by this context */
  uint64_t eval_launches;    /* region-evaluation launches */
  uint64_t regions_evaluated;
  uint64_t points_evaluated;
  double eval_ms;            /* summed CUDA-event time of evaluation launches */
  double stage_ms;           /* summed time of the two-level/classify/compact/split launches */
  uint64_t stage_bytes;      /* algorithmic bytes moved by those stages */
  uint64_t h2d_bytes;
  uint64_t d2h_bytes;
  int32_t tune_warps[2];        /* autotuned regions per block: [0] ndim <= 8, [1] ndim > 8 */
  int32_t tune_ctas_per_sm[2];  /* autotuned grid cap (blocks per SM) of the evaluation kernel */
  uint64_t eval_bytes;          /* algorithmic HBM bytes of the evaluation launches */
  double host_ms;               /* host time from an iteration's readback to the next evaluation launch */
  double sync_ms;               /* host time blocked waiting for an iteration's device work */
  double spill_ms;              /* device time of moving region lists out of the pool (compaction + copies) */
  double admit_ms;              /* device time of admissions: first splits and region lists moved back in */
  uint64_t setsum_regions;      /* regions evaluated by generator-set sums (PG_EVAL_SET_SUMS) */
  double classify_ms;           /* host time in the memory-pressure classifier (its passes included) */
  uint64_t classify_passes;     /* threshold passes of the classifier (each a launch and a readback) */
  uint64_t setsum_pairs;        /* sibling pairs evaluated together by the set-sum kernel */
  uint64_t setsum_cached_pairs; /* of those, pairs that took their parent's kept per-axis terms */
} pg_stats;

/* One iteration of a run (recorded while profiling is on): regions in the
 * list, integrals resident, evaluation launches and their CUDA-event time, and
 * the time of the two-level/classification launches.  No counterpart in the
 * reference, whose debug mode writes per-iteration CSV files instead
 * (cuda/pagani/quad/GPUquad/PaganiUtils.cuh:203-241). */
typedef struct pg_iteration_record {
  uint64_t regions;
  uint32_t integrals;
  uint32_t eval_launches;
  double eval_ms;
  double stage_ms;
} pg_iteration_record;

void pg_options_default(pg_options* opt);
int pg_feval(int ndim); /* points per region: cuda/pagani/quad/quad.h:67-76 */

/* Context lifetime.  Replaces the reference's per-call allocations
 * (Region_estimates.cuh:11-16, Sub_regions.cuh:199-207) with one pool. */
int pg_context_create(int device, pg_context** out);
int pg_context_destroy(pg_context* ctx);
const char* pg_last_error(const pg_context* ctx);
int pg_context_set_profiling(pg_context* ctx, int on);
int pg_context_stats(const pg_context* ctx, pg_stats* out);
int pg_context_reset_stats(pg_context* ctx);
/* The iterations recorded since the last pg_context_reset_stats: *count
 * receives their number, out[0 .. min(count, capacity)) the records. */
int pg_context_iterations(const pg_context* ctx, pg_iteration_record* out, uint64_t capacity, uint64_t* count);
/* Testing hook, no counterpart in the reference: of the device and pinned
 * host buffers this context allocates from now on, the one after `after` more
 * fails as cudaMalloc fails when memory runs out, and the call that needed it
 * returns PG_OOM; later allocations succeed again and the context stays
 * usable.  after < 0 turns the hook off.  Nothing reaches the GPU: the
 * failure is made on the host before cudaMalloc is called. */
int pg_context_fail_allocation(pg_context* ctx, int64_t after);
void* pg_context_stream(pg_context* ctx); /* the cudaStream_t the context launches on */
int pg_synchronize(pg_context* ctx);

/* Full PAGANI integration of one integrand over [lows, highs].
 * Replaces Workspace<T,ndim>::integrate(f, epsrel, epsabs, vol, relerr)
 * (cuda/pagani/quad/GPUquad/Workspace.cuh:361-494).  Returns the result status
 * (PG_OK / PG_NOT_CONVERGED) or a negative error code.  lows/highs may be NULL
 * for the unit cube. */
int pg_integrate(pg_context* ctx, const pg_integrand* f, double epsrel, double epsabs, const double* lows,
                 const double* highs, const pg_options* opt, pg_result* out);

/* PAGANI from a caller-given first region list: the reference's
 * Workspace::integrate(f, subregions, epsrel, epsabs, vol, relerr, optional)
 * overload (cuda/pagani/quad/GPUquad/Workspace.cuh:148-158).  n regions in the
 * unit coordinates of [lows, highs], host SoA [dim * n + i] (the layout of
 * Sub_regions, Sub_regions.cuh:38-258). */
int pg_integrate_regions(pg_context* ctx, const pg_integrand* f, const double* left, const double* length,
                         uint64_t n, double epsrel, double epsabs, const double* lows, const double* highs,
                         const pg_options* opt, pg_result* out);

/* The region list the last pg_integrate / pg_integrate_regions (or their
 * launcher forms) with opt->predict_split kept at iteration 15
 * (Sub_regions::take_snapshot, Sub_regions.cuh:220-229).  *n receives its
 * region count (0: none kept) and *ndim its dimension; left/length (SoA
 * [dim * n + i], may be NULL) receive it when capacity >= *n. */
int pg_last_snapshot(pg_context* ctx, int32_t* ndim, uint64_t* n, double* left, double* length, uint64_t capacity);

/* Region evaluation on a caller-given region list (host buffers, SoA
 * [dim * n + i]).  Replaces Cubature_rules::apply_cubature_integration_rules
 * (cuda/pagani/quad/GPUquad/PaganiUtils.cuh:243-289), which the reference's
 * stage tests call directly (test/cuda/pagani/RegionSampling.cu:48-88). */
int pg_evaluate_regions(pg_context* ctx, const pg_integrand* f, const double* lows, const double* highs,
                        uint64_t n, const double* left, const double* length, double* est, double* err,
                        int32_t* bisect, int32_t eval_mode /* PG_EVAL_POINTS or PG_EVAL_SET_SUMS */);

/* Same on device buffers, asynchronous on the context stream. */
int pg_evaluate_regions_device(pg_context* ctx, const pg_integrand* f, const double* lows, const double* highs,
                               uint64_t n, const double* d_left, const double* d_length, double* d_est,
                               double* d_err, int32_t* d_bisect, int32_t eval_mode);

/* ---------------- user integrands (C++ layer) ----------------
 * A device functor cannot cross a C ABI, but a caller compiled with nvcc can
 * instantiate the region-evaluation kernel for its own functor and give the
 * library a launcher for it.  include/pagani_gb300.cuh does this for
 * Workspace<T,ndim>::integrate(f, epsrel, epsabs, vol, relerr_classification)
 * (cuda/pagani/quad/GPUquad/Workspace.cuh:52-70), whose integrands are any
 * copyable type with a __device__ operator() of ndim doubles
 * (common/cuda/cudaApply.cuh:7-26).  The library runs the whole iteration and
 * calls launch(args, user) once per evaluation launch; args point at the
 * library's device buffers, `descs` and `rule` are opaque to C, and launch
 * returns 0 or a cudaError_t value. */
typedef struct pg_eval_args {
  const double* left;    /* SoA region list, coordinate k of region i at [k * stride + i] */
  const double* length;
  uint64_t n;            /* regions */
  uint64_t stride;
  const uint32_t* owner; /* integral of each region, NULL when the list holds one integral */
  const void* descs;     /* device array of the library's per-integral descriptors */
  const void* rule;      /* host pointer to the library's rule-table block (device pointers inside) */
  double* est;
  double* err;
  int32_t* bisect;
  int32_t maxd;          /* largest ndim in the list */
  int32_t num_sms;
  void* stream;          /* cudaStream_t to launch on */
  int32_t warps;         /* autotuned regions per block: 4 or 8 */
  int32_t ctas_per_sm;   /* autotuned grid cap */
} pg_eval_args;

typedef int (*pg_eval_launcher)(const pg_eval_args* args, void* user);

/* pg_integrate for a user integrand of ndim dimensions evaluated by `launch`. */
int pg_integrate_launcher(pg_context* ctx, int32_t ndim, pg_eval_launcher launch, void* user, double epsrel,
                          double epsabs, const double* lows, const double* highs, const pg_options* opt,
                          pg_result* out);

/* pg_integrate_regions for a user integrand. */
int pg_integrate_regions_launcher(pg_context* ctx, int32_t ndim, pg_eval_launcher launch, void* user,
                                  const double* left, const double* length, uint64_t n, double epsrel,
                                  double epsabs, const double* lows, const double* highs, const pg_options* opt,
                                  pg_result* out);

/* pg_evaluate_regions for a user integrand (host buffers, SoA [dim * n + i]):
 * the region-evaluation stage test (test/cuda/pagani/RegionSampling.cu:48-88)
 * for functors. */
int pg_evaluate_regions_launcher(pg_context* ctx, int32_t ndim, pg_eval_launcher launch, void* user,
                                 const double* lows, const double* highs, uint64_t n, const double* left,
                                 const double* length, double* est, double* err, int32_t* bisect);

/* Two-level error estimate and relative-error classification on host buffers.
 * Replaces two_level_errorest_and_relerr_classify / RefineError
 * (cuda/pagani/quad/GPUquad/hybrid.cuh:11-45, Phases.cuh:219-268). */
int pg_two_level(pg_context* ctx, uint64_t n, const double* est, const double* err, const double* parent_est,
                 double* new_err, uint8_t* active, double epsrel, int32_t relerr_classification);

/* Filter + split on host buffers: keeps the active regions in order and bisects
 * each along its split axis; child 0 of the k-th kept region lands at k, child
 * 1 at A + k, SoA stride 2A.  Replaces Sub_regions_filter::filter and
 * Sub_region_splitter::split (Sub_region_filter.cuh:84-139,
 * Sub_region_splitter.cuh:55-87).  *n_active receives A; out_left/out_length
 * must hold 2*A*ndim doubles (A <= n). */
int pg_filter_split(pg_context* ctx, int ndim, uint64_t n, const double* left, const double* length,
                    const uint8_t* active, const int32_t* bisect, const double* est, const double* err,
                    double* out_left, double* out_length, double* parent_est, double* parent_err,
                    uint64_t* n_active);

/* Deterministic compensated sum of n doubles on the GPU (blocked Neumaier
 * order; see the library's reduction kernels).  Replaces reduction()
 * (common/cuda/thrust_utils.cuh:37-47). */
int pg_reduce_sum(pg_context* ctx, const double* x, uint64_t n, double* out);

/* Exclusive scan of 0/1 flags, as used for compaction offsets.  Replaces
 * exclusive_scan (common/cuda/thrust_utils.cuh:49-60). */
int pg_exclusive_scan_flags(pg_context* ctx, const uint8_t* flags, uint64_t n, uint64_t* out, uint64_t* total);

/* Degree-9 rule tables as generated by the library (host-side).  w, scale,
 * norm: 45 doubles each ([set*5 + rule]); set_of: feval ints; gen: feval*ndim
 * doubles, point-major.  Returns feval.  Mirrors quad::Rule<T>::Init
 * (cuda/pagani/quad/GPUquad/Rule.cuh:370-510). */
int pg_rule_tables(int ndim, double* w, double* scale, double* norm, int32_t* set_of, double* gen);

/* The reference's C-language precedent, with the same contract:
 * integrates x*y over the unit square at epsrel 1e-6, returns the status and
 * writes the estimate only when it is 0.  test/cuda/pagani/do_integration_from_c.cu:21-37 */
int do_integration_from_c(double* res);

/* ---------------- m-Cubes (stratified VEGAS) ----------------
 * Replaces cuda_mcubes::integrate<F,ndim>(f, epsrel, epsabs, ncall, &vol,
 * totalIters, adjustIters, skipIters) (cuda/mcubes/vegasT.cuh:999-1030).
 * The reference seeds from the wall clock (vegasT.cuh:801-803); here the
 * Philox4x32-10 stream is keyed by `seed`, so runs are reproducible. */
typedef struct pg_mcubes_options {
  double ncall;      /* requested calls per iteration */
  int32_t titer;     /* total iterations */
  int32_t itmax;     /* adapting iterations */
  int32_t skip;      /* iterations excluded from the weighted mean */
  int32_t nbins;     /* bins per axis, 500 in the reference (vegasT.cuh:650) */
  uint64_t seed;
  double alpha;      /* grid damping exponent, 1.5 in the reference's GPU code */
} pg_mcubes_options;

void pg_mcubes_options_default(pg_mcubes_options* opt);
int pg_mcubes_integrate(pg_context* ctx, const pg_integrand* f, double epsrel, double epsabs, const double* lows,
                        const double* highs, const pg_mcubes_options* opt, pg_result* out);

/* m-Cubes for a user integrand (C++ layer: cuda_mcubes::integrate<F, NDIM> in
 * include/pagani_gb300.cuh): launch(args, user) runs one sampling iteration
 * of the library's m-Cubes kernel instantiated for the caller's functor;
 * `args` is the kernel's argument block (opaque to C), launch returns 0 or a
 * cudaError_t value. */
typedef struct pg_mcubes_args {
  const void* args; /* kernel argument block */
  uint64_t smem;    /* dynamic shared memory bytes */
  void* stream;     /* cudaStream_t */
  int32_t maxd;     /* ndim */
  int32_t pad;
} pg_mcubes_args;

typedef int (*pg_mcubes_launcher)(const pg_mcubes_args* args, void* user);

int pg_mcubes_integrate_launcher(pg_context* ctx, int32_t ndim, pg_mcubes_launcher launch, void* user,
                                 double epsrel, double epsabs, const double* lows, const double* highs,
                                 const pg_mcubes_options* opt, pg_result* out);

/* ---------------- batched PAGANI ----------------
 * Integrates `count` independent integrands (any mix of ndim, family and
 * tolerance) together: one device-side region pool shared by all of them, one
 * evaluation launch per iteration over every live region of every integrand.
 * No counterpart in the reference beyond running Workspace::integrate once per
 * integrand (Workspace.cuh:361-494).  out[i] has the same semantics as
 * pg_integrate's result for integrand i. */
int pg_batch_integrate(pg_context* ctx, uint64_t count, const pg_integrand* fs, const double* epsrel,
                       const double* epsabs, const pg_options* opt, pg_result* out);

/* Same as pg_batch_integrate; completion_ms[i] (may be NULL) receives the
 * host time in milliseconds from the start of the call to the end of the
 * iteration in which integral i finished (its latency within the batch). */
int pg_batch_integrate_timed(pg_context* ctx, uint64_t count, const pg_integrand* fs, const double* epsrel,
                             const double* epsabs, const pg_options* opt, pg_result* out, double* completion_ms);

/* ---------------- served PAGANI ----------------
 * Continuous batching over an arrival schedule: request i (integrand fs[i],
 * tolerances epsrel[i]/epsabs[i]) arrives arrival_ms[i] milliseconds after the
 * call starts (ascending).  At every iteration boundary the requests that have
 * arrived join the device region pool, in arrival order, while the pool's
 * footprint stays under budget_bytes of device memory (0: 60% of free memory);
 * their regions are evaluated in the same launches as the requests already
 * running, each request's region list stays on the device across iterations
 * (or moves to host memory while the pool is full), and each request retires
 * in the iteration it converges.  completion_ms[i] receives the time the
 * result was ready (latency = completion_ms[i] - arrival_ms[i]).  With
 * deadline_ms > 0 the call returns at the first iteration boundary after that
 * time; requests not finished by then get status -1 and completion_ms -1.
 * Every finished result is bit-identical to pg_integrate's for the same
 * request.  No counterpart in the reference (a loop of Workspace::integrate
 * calls, Workspace.cuh:361-494). */
int pg_serve(pg_context* ctx, uint64_t count, const pg_integrand* fs, const double* epsrel, const double* epsabs,
             const double* arrival_ms, uint64_t budget_bytes, double deadline_ms, const pg_options* opt,
             pg_result* out, double* completion_ms);

/* Measurement utility, no counterpart in the reference: runs a fixed FP64
 * fused-multiply-add loop on the context's GPU and returns the achieved
 * FP64 rate in TFLOP/s (an FMA counts as 2 flops), the denominator of the
 * region-evaluation roofline. */
int pg_probe_fp64_peak(pg_context* ctx, double* tflops);

/* Largest element count pg_reduce_sum_noalloc accepts (2^28 doubles). */
#define PG_REDUCE_NOALLOC_MAX_N (1ull << 28)

/* Compensated FP64 sum of the n doubles at d_x (device memory), written to
 * *d_out (device memory), asynchronously on `stream` (a cudaStream_t of the
 * current device; NULL for the default stream).  No counterpart in the
 * reference: it is the allocation-free form of pg_reduce_sum, for callers that
 * cannot allocate device memory -- a program whose device memory is owned by
 * another allocator, or a loop that cannot take cudaMalloc's implicit
 * synchronisation.  It calls no allocator; its only scratch is a fixed 2 MB
 * array in the library's device image, which every GPU that loads the
 * library holds until the process exits.  n above PG_REDUCE_NOALLOC_MAX_N is
 * rejected with PG_BAD_ARG before anything runs.  The first call on a device
 * looks up that array's device address, so make it before any stream capture.
 * Every call uses the same array: calls whose kernels can overlap on the GPU
 * (other streams, other host threads) race, and the caller must serialise
 * them.  The result is bit-identical to pg_reduce_sum on the same data.
 * The call ends with cudaGetLastError, which also returns (and clears) an
 * error left pending by the caller's own earlier launches, so PG_CUDA_ERROR
 * may report an error this call did not cause.  The scratch array's device
 * address is looked up once per device and belongs to that device's primary
 * context: after cudaDeviceReset it is stale, and the entry point must not be
 * called again in that process. */
int pg_reduce_sum_noalloc(const double* d_x, uint64_t n, double* d_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PAGANI_GB300_H */
