// C ABI of the GB300 PAGANI library (declarations: include/pagani_gb300.h).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/pagani_gb300.h"
#include "pg_engine.h"
#include "pg_mcubes.h"

struct pg_context {
  pg::Engine* eng = nullptr;
  std::mutex mu;
  std::string err;
  // scratch of the stage-level entry points
  pg::DevBuf s_left, s_len, s_est, s_err, s_err2, s_bis, s_act, s_par, s_out_left, s_out_len, s_owner, s_seg,
      s_chunks, s_trans, s_off, s_part, s_desc, s_x, s_res;
  pg::McubesState* mc = nullptr;
  // region list kept by the last predict_split run
  std::vector<double> snap_left, snap_length;
  uint64_t snap_n = 0;
  int32_t snap_d = 0;
};

namespace {

int set_err(pg_context* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

__host__ __device__ inline uint64_t div_up(uint64_t a, uint64_t b) { return (a + b - 1) / b; }

#define CAPI_TRY(ctx, call, what)                                                               \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      return set_err(ctx, e_ == cudaErrorMemoryAllocation ? PG_OOM : PG_CUDA_ERROR,              \
                     std::string(what) + ": " + cudaGetErrorString(e_));                       \
  } while (0)

#define CAPI_ENSURE(ctx, buf, bytes)                             \
  do {                                                           \
    int rc_ = (ctx)->eng->ensure((buf), (bytes));                \
    if (rc_ != PG_OK) return set_err(ctx, rc_, (ctx)->eng->last_error); \
  } while (0)

// Per-chunk flag counts and in-chunk exclusive offsets (chunk = 2048 flags,
// 8 consecutive flags per thread).
__global__ void flag_count_kernel(const uint8_t* __restrict__ f, uint64_t n, uint64_t* __restrict__ counts) {
  __shared__ unsigned long long s;
  if (threadIdx.x == 0) s = 0;
  __syncthreads();
  uint64_t c = 0;
  const uint64_t first = (uint64_t)blockIdx.x * pg::kChunk + (uint64_t)threadIdx.x * pg::kRedItems;
  for (int q = 0; q < pg::kRedItems; ++q)
    if (first + q < n) c += f[first + q] ? 1 : 0;
  atomicAdd(&s, (unsigned long long)c);
  __syncthreads();
  if (threadIdx.x == 0) counts[blockIdx.x] = s;
}

__global__ void chunk_scan_kernel(const uint64_t* __restrict__ counts, uint64_t nchunks, uint64_t* __restrict__ off,
                                  uint64_t* __restrict__ total) {
  __shared__ uint64_t sc[33];
  const uint64_t per = div_up(nchunks, pg::kRedThreads);
  const uint64_t b0 = threadIdx.x * per, b1 = b0 + per < nchunks ? b0 + per : nchunks;
  uint64_t local = 0;
  for (uint64_t b = b0; b < b1; ++b) local += counts[b];
  uint64_t tot;
  uint64_t run = pg::block_exclusive_scan(local, sc, &tot);
  for (uint64_t b = b0; b < b1; ++b) {
    off[b] = run;
    run += counts[b];
  }
  if (threadIdx.x == 0) *total = tot;
}

__global__ void flag_offsets_kernel(const uint8_t* __restrict__ f, uint64_t n, const uint64_t* __restrict__ off,
                                    uint64_t* __restrict__ out) {
  __shared__ uint64_t sc[33];
  const uint64_t first = (uint64_t)blockIdx.x * pg::kChunk + (uint64_t)threadIdx.x * pg::kRedItems;
  uint64_t c = 0;
  for (int q = 0; q < pg::kRedItems; ++q)
    if (first + q < n) c += f[first + q] ? 1 : 0;
  uint64_t tot;
  uint64_t run = pg::block_exclusive_scan(c, sc, &tot) + off[blockIdx.x];
  for (int q = 0; q < pg::kRedItems; ++q)
    if (first + q < n) {
      out[first + q] = run;
      run += f[first + q] ? 1 : 0;
    }
}

// Eight independent FMA chains per thread (FP64 issue-rate probe).
__global__ void fp64_fma_probe_kernel(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = __fma_rn(x0, a, b);
    x1 = __fma_rn(x1, a, b);
    x2 = __fma_rn(x2, a, b);
    x3 = __fma_rn(x3, a, b);
    x4 = __fma_rn(x4, a, b);
    x5 = __fma_rn(x5, a, b);
    x6 = __fma_rn(x6, a, b);
    x7 = __fma_rn(x7, a, b);
  }
  const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 12345.678) out[0] = s;  // keeps the chains alive
}

struct Guard {
  explicit Guard(pg_context* c) : lk(c->mu) { cudaSetDevice(c->eng->device); }
  std::lock_guard<std::mutex> lk;
};

}  // namespace

extern "C" {

void pg_options_default(pg_options* opt) {
  if (!opt) return;
  std::memset(opt, 0, sizeof *opt);
  opt->relerr_classification = 1;
  opt->max_iters = 700;
  opt->device_mem_model = 16e9;
  opt->max_regions = 0;
  opt->eval_mode = 0;
  opt->predict_split = 0;
}

int pg_feval(int ndim) {
  if (ndim < PG_MIN_NDIM || ndim > pg::kMaxNdim) return -1;
  return pg::feval_count(ndim);
}

int pg_context_create(int device, pg_context** out) {
  if (!out) return PG_BAD_ARG;
  *out = nullptr;
  pg_context* ctx = new (std::nothrow) pg_context;
  if (!ctx) return PG_OOM;
  ctx->eng = new (std::nothrow) pg::Engine(device);
  if (!ctx->eng) {
    delete ctx;
    return PG_OOM;
  }
  std::string why;
  const int rc = ctx->eng->init(&why);
  if (rc != PG_OK) {
    delete ctx->eng;
    delete ctx;
    return rc;
  }
  *out = ctx;
  return PG_OK;
}

int pg_context_destroy(pg_context* ctx) {
  if (!ctx) return PG_BAD_ARG;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->eng->device);
    pg::DevBuf* bufs[] = {&ctx->s_left, &ctx->s_len, &ctx->s_est, &ctx->s_err, &ctx->s_err2, &ctx->s_bis,
                          &ctx->s_act, &ctx->s_par, &ctx->s_out_left, &ctx->s_out_len, &ctx->s_owner, &ctx->s_seg,
                          &ctx->s_chunks, &ctx->s_trans, &ctx->s_off, &ctx->s_part, &ctx->s_desc, &ctx->s_x,
                          &ctx->s_res};
    for (pg::DevBuf* b : bufs)
      if (b->p) cudaFree(b->p);
    pg::mcubes_destroy(ctx->mc);
    ctx->mc = nullptr;
    delete ctx->eng;
  }
  delete ctx;
  return PG_OK;
}

const char* pg_last_error(const pg_context* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int pg_context_set_profiling(pg_context* ctx, int on) {
  if (!ctx) return PG_BAD_ARG;
  ctx->eng->profiling = on != 0;
  return PG_OK;
}

int pg_context_stats(const pg_context* ctx, pg_stats* out) {
  if (!ctx || !out) return PG_BAD_ARG;
  *out = ctx->eng->stats;
  for (int c = 0; c < 2; ++c) {
    out->tune_warps[c] = ctx->eng->tune[c].warps;
    out->tune_ctas_per_sm[c] = ctx->eng->tune[c].ctas_per_sm;
  }
  return PG_OK;
}

int pg_context_reset_stats(pg_context* ctx) {
  if (!ctx) return PG_BAD_ARG;
  ctx->eng->stats = pg_stats{};
  ctx->eng->iterations.clear();
  return PG_OK;
}

int pg_context_fail_allocation(pg_context* ctx, int64_t after) {
  if (!ctx) return PG_BAD_ARG;
  ctx->eng->fail_alloc_after = after < 0 ? -1 : after;
  return PG_OK;
}

int pg_context_iterations(const pg_context* ctx, pg_iteration_record* out, uint64_t capacity, uint64_t* count) {
  if (!ctx || !count || (capacity && !out)) return PG_BAD_ARG;
  const auto& it = ctx->eng->iterations;
  *count = it.size();
  for (uint64_t i = 0; i < capacity && i < it.size(); ++i) out[i] = it[i];
  return PG_OK;
}

void* pg_context_stream(pg_context* ctx) { return ctx ? (void*)ctx->eng->stream() : nullptr; }

int pg_synchronize(pg_context* ctx) {
  if (!ctx) return PG_BAD_ARG;
  Guard g(ctx);
  CAPI_TRY(ctx, cudaStreamSynchronize(ctx->eng->stream()), "synchronize");
  return PG_OK;
}

static int validate_eps(pg_context* ctx, double epsrel, double epsabs) {
  if (!(epsrel > 0.0) || !(epsabs >= 0.0) || !std::isfinite(epsrel))
    return set_err(ctx, PG_BAD_ARG, "epsrel must be > 0 and epsabs >= 0");
  return PG_OK;
}

// One integral through the engine: descriptor prepared by the caller,
// optional first region list, predict_split snapshot kept in the context.
static int run_single(pg_context* ctx, const pg::IntegralDesc& D, double epsrel, double epsabs, const pg_options* opt,
                      const double* left, const double* length, uint64_t n, const pg::EvalLauncher& launch,
                      pg_result* out) {
  std::vector<pg::Job> jobs(1);
  jobs[0].desc = D;
  jobs[0].epsrel = epsrel;
  jobs[0].epsabs = epsabs;
  if (opt) jobs[0].opt = *opt; else pg_options_default(&jobs[0].opt);
  if (jobs[0].opt.eval_mode != PG_EVAL_POINTS && jobs[0].opt.eval_mode != PG_EVAL_SET_SUMS)
    return set_err(ctx, PG_BAD_ARG, "eval_mode must be PG_EVAL_POINTS or PG_EVAL_SET_SUMS");
  if (jobs[0].opt.max_iters <= 0) jobs[0].opt.max_iters = 700;
  if (n) {
    if (!left || !length) return set_err(ctx, PG_BAD_ARG, "null region list");
    for (uint64_t q = 0; q < n * (uint64_t)D.d; ++q)
      if (!(length[q] > 0.0) || !std::isfinite(left[q]) || !std::isfinite(length[q]))
        return set_err(ctx, PG_BAD_ARG, "region lists need finite coordinates and positive lengths");
    jobs[0].init_left = left;
    jobs[0].init_length = length;
    jobs[0].init_n = n;
  }
  if (jobs[0].opt.predict_split) {
    ctx->snap_n = 0;
    ctx->snap_d = D.d;
    jobs[0].snap_left = &ctx->snap_left;
    jobs[0].snap_length = &ctx->snap_length;
    jobs[0].snap_n = &ctx->snap_n;
  }
  int rc = ctx->eng->run(jobs, launch);
  if (rc != PG_OK) return set_err(ctx, rc, ctx->eng->last_error);
  *out = jobs[0].res;
  return out->status == 0 ? PG_OK : PG_NOT_CONVERGED;
}

int pg_integrate(pg_context* ctx, const pg_integrand* f, double epsrel, double epsabs, const double* lows,
                 const double* highs, const pg_options* opt, pg_result* out) {
  return pg_integrate_regions(ctx, f, nullptr, nullptr, 0, epsrel, epsabs, lows, highs, opt, out);
}

int pg_integrate_regions(pg_context* ctx, const pg_integrand* f, const double* left, const double* length,
                         uint64_t n, double epsrel, double epsabs, const double* lows, const double* highs,
                         const pg_options* opt, pg_result* out) {
  if (!ctx || !f || !out) return set_err(ctx, PG_BAD_ARG, "null argument");
  int rc = validate_eps(ctx, epsrel, epsabs);
  if (rc != PG_OK) return rc;
  Guard g(ctx);
  pg::IntegralDesc D;
  std::string why;
  rc = pg::prepare_desc(*f, lows, highs, &D, &why);
  if (rc != PG_OK) return set_err(ctx, rc, why);
  return run_single(ctx, D, epsrel, epsabs, opt, left, length, n, pg::launch_family_eval, out);
}

int pg_last_snapshot(pg_context* ctx, int32_t* ndim, uint64_t* n, double* left, double* length, uint64_t capacity) {
  if (!ctx || !n) return set_err(ctx, PG_BAD_ARG, "null argument");
  Guard g(ctx);
  *n = ctx->snap_n;
  if (ndim) *ndim = ctx->snap_d;
  if (ctx->snap_n && left && length) {
    if (capacity < ctx->snap_n) return set_err(ctx, PG_BAD_ARG, "snapshot buffers too small");
    const size_t m = ctx->snap_n * (size_t)ctx->snap_d;
    std::memcpy(left, ctx->snap_left.data(), m * 8);
    std::memcpy(length, ctx->snap_length.data(), m * 8);
  }
  return PG_OK;
}

int pg_batch_integrate(pg_context* ctx, uint64_t count, const pg_integrand* fs, const double* epsrel,
                       const double* epsabs, const pg_options* opt, pg_result* out) {
  return pg_batch_integrate_timed(ctx, count, fs, epsrel, epsabs, opt, out, nullptr);
}

int pg_batch_integrate_timed(pg_context* ctx, uint64_t count, const pg_integrand* fs, const double* epsrel,
                             const double* epsabs, const pg_options* opt, pg_result* out, double* completion_ms) {
  if (!ctx || (!fs && count) || !epsrel || !epsabs || (!out && count)) return set_err(ctx, PG_BAD_ARG, "null argument");
  if (count > 0xffffffffull) return set_err(ctx, PG_BAD_ARG, "too many integrands");
  Guard g(ctx);
  std::vector<pg::Job> jobs(count);
  for (uint64_t i = 0; i < count; ++i) {
    std::string why;
    int rc = validate_eps(ctx, epsrel[i], epsabs[i]);
    if (rc != PG_OK) return rc;
    rc = pg::prepare_desc(fs[i], nullptr, nullptr, &jobs[i].desc, &why);
    if (rc != PG_OK) return set_err(ctx, rc, "integrand " + std::to_string(i) + ": " + why);
    jobs[i].epsrel = epsrel[i];
    jobs[i].epsabs = epsabs[i];
    if (opt) jobs[i].opt = *opt; else pg_options_default(&jobs[i].opt);
    if (jobs[i].opt.eval_mode != PG_EVAL_POINTS && jobs[i].opt.eval_mode != PG_EVAL_SET_SUMS)
      return set_err(ctx, PG_BAD_ARG, "eval_mode must be PG_EVAL_POINTS or PG_EVAL_SET_SUMS");
    if (jobs[i].opt.max_iters <= 0) jobs[i].opt.max_iters = 700;
  }
  pg::RunPolicy pol;
  if (opt) pol.max_regions = opt->max_regions;
  int rc = ctx->eng->run(jobs, pg::launch_family_eval, pol);
  if (rc != PG_OK) return set_err(ctx, rc, ctx->eng->last_error);
  for (uint64_t i = 0; i < count; ++i) {
    out[i] = jobs[i].res;
    if (completion_ms) completion_ms[i] = jobs[i].done_ms;
  }
  return PG_OK;
}

int pg_serve(pg_context* ctx, uint64_t count, const pg_integrand* fs, const double* epsrel, const double* epsabs,
             const double* arrival_ms, uint64_t budget_bytes, double deadline_ms, const pg_options* opt,
             pg_result* out, double* completion_ms) {
  if (!ctx || (count && (!fs || !epsrel || !epsabs || !arrival_ms || !out)))
    return set_err(ctx, PG_BAD_ARG, "null argument");
  if (count > 0xffffffffull) return set_err(ctx, PG_BAD_ARG, "too many requests");
  for (uint64_t i = 1; i < count; ++i)
    if (arrival_ms[i] < arrival_ms[i - 1]) return set_err(ctx, PG_BAD_ARG, "arrivals must be ascending");
  Guard g(ctx);
  std::vector<pg::Job> jobs(count);
  for (uint64_t i = 0; i < count; ++i) {
    std::string why;
    int rc = validate_eps(ctx, epsrel[i], epsabs[i]);
    if (rc != PG_OK) return rc;
    rc = pg::prepare_desc(fs[i], nullptr, nullptr, &jobs[i].desc, &why);
    if (rc != PG_OK) return set_err(ctx, rc, "request " + std::to_string(i) + ": " + why);
    jobs[i].epsrel = epsrel[i];
    jobs[i].epsabs = epsabs[i];
    if (opt) jobs[i].opt = *opt; else pg_options_default(&jobs[i].opt);
    if (jobs[i].opt.eval_mode != PG_EVAL_POINTS && jobs[i].opt.eval_mode != PG_EVAL_SET_SUMS)
      return set_err(ctx, PG_BAD_ARG, "eval_mode must be PG_EVAL_POINTS or PG_EVAL_SET_SUMS");
    if (jobs[i].opt.max_iters <= 0) jobs[i].opt.max_iters = 700;
  }
  pg::RunPolicy pol;
  pol.arrival_ms = arrival_ms;
  pol.budget_bytes = budget_bytes;
  pol.deadline_ms = deadline_ms;
  if (opt) pol.max_regions = opt->max_regions;
  int rc = ctx->eng->run(jobs, pg::launch_family_eval, pol);
  if (rc != PG_OK) return set_err(ctx, rc, ctx->eng->last_error);
  for (uint64_t i = 0; i < count; ++i) {
    out[i] = jobs[i].res;
    if (completion_ms) completion_ms[i] = jobs[i].done_ms;
  }
  return PG_OK;
}

int pg_evaluate_regions_device(pg_context* ctx, const pg_integrand* f, const double* lows, const double* highs,
                               uint64_t n, const double* d_left, const double* d_length, double* d_est, double* d_err,
                               int32_t* d_bisect, int32_t eval_mode) {
  if (!ctx || !f) return set_err(ctx, PG_BAD_ARG, "null argument");
  if (eval_mode != PG_EVAL_POINTS && eval_mode != PG_EVAL_SET_SUMS)
    return set_err(ctx, PG_BAD_ARG, "eval_mode must be PG_EVAL_POINTS or PG_EVAL_SET_SUMS");
  Guard g(ctx);
  pg::IntegralDesc D;
  std::string why;
  int rc = pg::prepare_desc(*f, lows, highs, &D, &why);
  if (rc != PG_OK) return set_err(ctx, rc, why);
  rc = ctx->eng->evaluate(D, n, d_left, d_length, n, d_est, d_err, d_bisect, pg::launch_family_eval, eval_mode);
  if (rc != PG_OK) return set_err(ctx, rc, ctx->eng->last_error);
  return PG_OK;
}

// Host-buffer region evaluation shared by the family and user-integrand entry points.
static int evaluate_host(pg_context* ctx, const pg::IntegralDesc& D, uint64_t n, const double* left,
                         const double* length, double* est, double* err, int32_t* bisect,
                         const pg::EvalLauncher& launch, int mode = PG_EVAL_POINTS) {
  int rc;
  if (n == 0) return PG_OK;
  const size_t nd = n * (size_t)D.d;
  CAPI_ENSURE(ctx, ctx->s_left, nd * 8);
  CAPI_ENSURE(ctx, ctx->s_len, nd * 8);
  CAPI_ENSURE(ctx, ctx->s_est, n * 8);
  CAPI_ENSURE(ctx, ctx->s_err, n * 8);
  CAPI_ENSURE(ctx, ctx->s_bis, n * 4);
  cudaStream_t s = ctx->eng->stream();
  CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_left.p, left, nd * 8, cudaMemcpyHostToDevice, s), "upload");
  CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_len.p, length, nd * 8, cudaMemcpyHostToDevice, s), "upload");
  rc = ctx->eng->evaluate(D, n, (const double*)ctx->s_left.p, (const double*)ctx->s_len.p, n, (double*)ctx->s_est.p,
                          (double*)ctx->s_err.p, (int32_t*)ctx->s_bis.p, launch, mode);
  if (rc != PG_OK) return set_err(ctx, rc, ctx->eng->last_error);
  CAPI_TRY(ctx, cudaMemcpyAsync(est, ctx->s_est.p, n * 8, cudaMemcpyDeviceToHost, s), "download");
  CAPI_TRY(ctx, cudaMemcpyAsync(err, ctx->s_err.p, n * 8, cudaMemcpyDeviceToHost, s), "download");
  CAPI_TRY(ctx, cudaMemcpyAsync(bisect, ctx->s_bis.p, n * 4, cudaMemcpyDeviceToHost, s), "download");
  CAPI_TRY(ctx, cudaStreamSynchronize(s), "evaluate");
  ctx->eng->stats.h2d_bytes += 2 * nd * 8;
  ctx->eng->stats.d2h_bytes += n * 20;
  return PG_OK;
}

int pg_evaluate_regions(pg_context* ctx, const pg_integrand* f, const double* lows, const double* highs, uint64_t n,
                        const double* left, const double* length, double* est, double* err, int32_t* bisect,
                        int32_t eval_mode) {
  if (!ctx || !f || (n && (!left || !length || !est || !err || !bisect)))
    return set_err(ctx, PG_BAD_ARG, "null argument");
  if (eval_mode != PG_EVAL_POINTS && eval_mode != PG_EVAL_SET_SUMS)
    return set_err(ctx, PG_BAD_ARG, "eval_mode must be PG_EVAL_POINTS or PG_EVAL_SET_SUMS");
  Guard g(ctx);
  pg::IntegralDesc D;
  std::string why;
  int rc = pg::prepare_desc(*f, lows, highs, &D, &why);
  if (rc != PG_OK) return set_err(ctx, rc, why);
  return evaluate_host(ctx, D, n, left, length, est, err, bisect, pg::launch_family_eval, eval_mode);
}

// ---------------------------------------------------------------------------
// User integrands: the caller's launcher instantiates the evaluation kernel
// for its functor; everything else is the library's iteration.
// ---------------------------------------------------------------------------
static pg::EvalLauncher user_launcher(pg_eval_launcher fn, void* user) {
  return [fn, user](const pg::EvalLaunch& L) -> cudaError_t {
    const pg_eval_args a = pg::eval_args_of(L);
    return (cudaError_t)fn(&a, user);
  };
}

int pg_integrate_launcher(pg_context* ctx, int32_t ndim, pg_eval_launcher launch, void* user, double epsrel,
                          double epsabs, const double* lows, const double* highs, const pg_options* opt,
                          pg_result* out) {
  return pg_integrate_regions_launcher(ctx, ndim, launch, user, nullptr, nullptr, 0, epsrel, epsabs, lows, highs,
                                       opt, out);
}

int pg_integrate_regions_launcher(pg_context* ctx, int32_t ndim, pg_eval_launcher launch, void* user,
                                  const double* left, const double* length, uint64_t n, double epsrel,
                                  double epsabs, const double* lows, const double* highs, const pg_options* opt,
                                  pg_result* out) {
  if (!ctx || !launch || !out) return set_err(ctx, PG_BAD_ARG, "null argument");
  int rc = validate_eps(ctx, epsrel, epsabs);
  if (rc != PG_OK) return rc;
  Guard g(ctx);
  pg::IntegralDesc D;
  std::string why;
  rc = pg::prepare_user_desc(ndim, lows, highs, &D, &why);
  if (rc != PG_OK) return set_err(ctx, rc, why);
  return run_single(ctx, D, epsrel, epsabs, opt, left, length, n, user_launcher(launch, user), out);
}

int pg_evaluate_regions_launcher(pg_context* ctx, int32_t ndim, pg_eval_launcher launch, void* user,
                                 const double* lows, const double* highs, uint64_t n, const double* left,
                                 const double* length, double* est, double* err, int32_t* bisect) {
  if (!ctx || !launch || (n && (!left || !length || !est || !err || !bisect)))
    return set_err(ctx, PG_BAD_ARG, "null argument");
  Guard g(ctx);
  pg::IntegralDesc D;
  std::string why;
  int rc = pg::prepare_user_desc(ndim, lows, highs, &D, &why);
  if (rc != PG_OK) return set_err(ctx, rc, why);
  return evaluate_host(ctx, D, n, left, length, est, err, bisect, user_launcher(launch, user));
}

int pg_two_level(pg_context* ctx, uint64_t n, const double* est, const double* err, const double* parent_est,
                 double* new_err, uint8_t* active, double epsrel, int32_t relerr_classification) {
  if (!ctx || (n && (!est || !err || !new_err || !active))) return set_err(ctx, PG_BAD_ARG, "null argument");
  if (parent_est && (n % 2)) return set_err(ctx, PG_BAD_ARG, "two-level needs an even region count");
  Guard g(ctx);
  if (n == 0) return PG_OK;
  const uint64_t nch = div_up(n, pg::kChunk);
  CAPI_ENSURE(ctx, ctx->s_est, n * 8);
  CAPI_ENSURE(ctx, ctx->s_err, n * 8);
  CAPI_ENSURE(ctx, ctx->s_err2, n * 8);
  CAPI_ENSURE(ctx, ctx->s_act, n);
  CAPI_ENSURE(ctx, ctx->s_par, (n / 2 + 1) * 8);
  CAPI_ENSURE(ctx, ctx->s_seg, sizeof(pg::SegDesc));
  CAPI_ENSURE(ctx, ctx->s_chunks, nch * sizeof(pg::ChunkRef));
  CAPI_ENSURE(ctx, ctx->s_part, nch * sizeof(pg::Partial));
  cudaStream_t s = ctx->eng->stream();
  pg::SegDesc S;
  std::memset(&S, 0, sizeof S);
  S.start = 0;
  S.n = n;
  S.par_start = 0;
  S.chunk_start = 0;
  S.nchunks = (uint32_t)nch;
  S.has_parent = parent_est ? 1 : 0;
  S.relerr = relerr_classification;
  S.epsrel = epsrel;
  std::vector<pg::ChunkRef> ch(nch);
  for (uint64_t b = 0; b < nch; ++b) ch[b] = pg::ChunkRef{0, (uint32_t)b};
  CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_seg.p, &S, sizeof S, cudaMemcpyHostToDevice, s), "upload");
  CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_chunks.p, ch.data(), nch * sizeof(pg::ChunkRef), cudaMemcpyHostToDevice, s),
           "upload");
  CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_est.p, est, n * 8, cudaMemcpyHostToDevice, s), "upload");
  CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_err.p, err, n * 8, cudaMemcpyHostToDevice, s), "upload");
  if (parent_est)
    CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_par.p, parent_est, (n / 2) * 8, cudaMemcpyHostToDevice, s), "upload");
  pg::two_level_kernel<<<(unsigned)nch, pg::kRedThreads, 0, s>>>(
      (const pg::ChunkRef*)ctx->s_chunks.p, (const pg::SegDesc*)ctx->s_seg.p, (const double*)ctx->s_est.p,
      (const double*)ctx->s_err.p, (const double*)ctx->s_par.p, (double*)ctx->s_err2.p, (uint8_t*)ctx->s_act.p,
      (pg::Partial*)ctx->s_part.p);
  ctx->eng->stats.launches++;
  CAPI_TRY(ctx, cudaGetLastError(), "two-level launch");
  CAPI_TRY(ctx, cudaMemcpyAsync(new_err, ctx->s_err2.p, n * 8, cudaMemcpyDeviceToHost, s), "download");
  CAPI_TRY(ctx, cudaMemcpyAsync(active, ctx->s_act.p, n, cudaMemcpyDeviceToHost, s), "download");
  CAPI_TRY(ctx, cudaStreamSynchronize(s), "two-level");
  return PG_OK;
}

int pg_filter_split(pg_context* ctx, int ndim, uint64_t n, const double* left, const double* length,
                    const uint8_t* active, const int32_t* bisect, const double* est, const double* err,
                    double* out_left, double* out_length, double* parent_est, double* parent_err,
                    uint64_t* n_active) {
  if (!ctx || !n_active || (n && (!left || !length || !active || !bisect || !est)))
    return set_err(ctx, PG_BAD_ARG, "null argument");
  if (ndim < PG_MIN_NDIM || ndim > pg::kMaxNdim) return set_err(ctx, PG_BAD_ARG, "ndim out of range");
  if (parent_err && !err) return set_err(ctx, PG_BAD_ARG, "parent_err needs err");
  Guard g(ctx);
  *n_active = 0;
  if (n == 0) return PG_OK;
  uint64_t A = 0;
  for (uint64_t i = 0; i < n; ++i) A += active[i] ? 1 : 0;
  *n_active = A;
  if (A == 0) return PG_OK;
  if (!out_left || !out_length) return set_err(ctx, PG_BAD_ARG, "null output");
  const uint64_t nch = div_up(n, pg::kChunk);
  const size_t nd = n * (size_t)ndim, od = 2 * A * (size_t)ndim;
  CAPI_ENSURE(ctx, ctx->s_left, nd * 8);
  CAPI_ENSURE(ctx, ctx->s_len, nd * 8);
  CAPI_ENSURE(ctx, ctx->s_act, n);
  CAPI_ENSURE(ctx, ctx->s_bis, n * 4);
  CAPI_ENSURE(ctx, ctx->s_est, n * 8);
  CAPI_ENSURE(ctx, ctx->s_err, n * 8);
  CAPI_ENSURE(ctx, ctx->s_out_left, od * 8);
  CAPI_ENSURE(ctx, ctx->s_out_len, od * 8);
  CAPI_ENSURE(ctx, ctx->s_owner, 2 * A * 4);
  CAPI_ENSURE(ctx, ctx->s_par, A * 8);
  CAPI_ENSURE(ctx, ctx->s_err2, A * 8);
  CAPI_ENSURE(ctx, ctx->s_seg, sizeof(pg::SegDesc));
  CAPI_ENSURE(ctx, ctx->s_trans, sizeof(pg::Transition));
  CAPI_ENSURE(ctx, ctx->s_desc, sizeof(pg::IntegralDesc));
  CAPI_ENSURE(ctx, ctx->s_chunks, nch * sizeof(pg::ChunkRef));
  CAPI_ENSURE(ctx, ctx->s_off, nch * 8 + 8);
  CAPI_ENSURE(ctx, ctx->s_part, nch * 8);
  cudaStream_t s = ctx->eng->stream();
  pg::SegDesc S;
  std::memset(&S, 0, sizeof S);
  S.n = n;
  S.nchunks = (uint32_t)nch;
  pg::Transition T;
  std::memset(&T, 0, sizeof T);
  T.mode = 1;
  T.A = A;
  pg::IntegralDesc D;
  std::memset(&D, 0, sizeof D);
  D.d = ndim;
  std::vector<pg::ChunkRef> ch(nch);
  for (uint64_t b = 0; b < nch; ++b) ch[b] = pg::ChunkRef{0, (uint32_t)b};
  CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_seg.p, &S, sizeof S, cudaMemcpyHostToDevice, s), "upload");
  CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_trans.p, &T, sizeof T, cudaMemcpyHostToDevice, s), "upload");
  CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_desc.p, &D, sizeof D, cudaMemcpyHostToDevice, s), "upload");
  CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_chunks.p, ch.data(), nch * sizeof(pg::ChunkRef), cudaMemcpyHostToDevice, s),
           "upload");
  CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_left.p, left, nd * 8, cudaMemcpyHostToDevice, s), "upload");
  CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_len.p, length, nd * 8, cudaMemcpyHostToDevice, s), "upload");
  CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_act.p, active, n, cudaMemcpyHostToDevice, s), "upload");
  CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_bis.p, bisect, n * 4, cudaMemcpyHostToDevice, s), "upload");
  CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_est.p, est, n * 8, cudaMemcpyHostToDevice, s), "upload");
  if (err) CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_err.p, err, n * 8, cudaMemcpyHostToDevice, s), "upload");
  uint64_t* counts = (uint64_t*)ctx->s_part.p;
  uint64_t* off = (uint64_t*)ctx->s_off.p;
  flag_count_kernel<<<(unsigned)nch, pg::kRedThreads, 0, s>>>((const uint8_t*)ctx->s_act.p, n, counts);
  chunk_scan_kernel<<<1, pg::kRedThreads, 0, s>>>(counts, nch, off, off + nch);
  ctx->eng->stats.launches += 2;
  auto launch = [&](const double* val, double* par_out) {
    if (ndim <= 8)
      pg::compact_split_kernel<8><<<(unsigned)nch, pg::kRedThreads, 0, s>>>(
          (const pg::ChunkRef*)ctx->s_chunks.p, (const pg::SegDesc*)ctx->s_seg.p, (const pg::Transition*)ctx->s_trans.p,
          off, (const pg::IntegralDesc*)ctx->s_desc.p, (const uint8_t*)ctx->s_act.p, (const double*)ctx->s_left.p,
          (const double*)ctx->s_len.p, n, (const int32_t*)ctx->s_bis.p, val, (double*)ctx->s_out_left.p,
          (double*)ctx->s_out_len.p, 2 * A, (uint32_t*)ctx->s_owner.p, par_out, 0u, nullptr, 0, nullptr);
    else
      pg::compact_split_kernel<16><<<(unsigned)nch, pg::kRedThreads, 0, s>>>(
          (const pg::ChunkRef*)ctx->s_chunks.p, (const pg::SegDesc*)ctx->s_seg.p, (const pg::Transition*)ctx->s_trans.p,
          off, (const pg::IntegralDesc*)ctx->s_desc.p, (const uint8_t*)ctx->s_act.p, (const double*)ctx->s_left.p,
          (const double*)ctx->s_len.p, n, (const int32_t*)ctx->s_bis.p, val, (double*)ctx->s_out_left.p,
          (double*)ctx->s_out_len.p, 2 * A, (uint32_t*)ctx->s_owner.p, par_out, 0u, nullptr, 0, nullptr);
    ctx->eng->stats.launches++;
  };
  launch((const double*)ctx->s_est.p, (double*)ctx->s_par.p);
  if (parent_err) launch((const double*)ctx->s_err.p, (double*)ctx->s_err2.p);
  CAPI_TRY(ctx, cudaGetLastError(), "compact/split launch");
  CAPI_TRY(ctx, cudaMemcpyAsync(out_left, ctx->s_out_left.p, od * 8, cudaMemcpyDeviceToHost, s), "download");
  CAPI_TRY(ctx, cudaMemcpyAsync(out_length, ctx->s_out_len.p, od * 8, cudaMemcpyDeviceToHost, s), "download");
  if (parent_est) CAPI_TRY(ctx, cudaMemcpyAsync(parent_est, ctx->s_par.p, A * 8, cudaMemcpyDeviceToHost, s), "download");
  if (parent_err) CAPI_TRY(ctx, cudaMemcpyAsync(parent_err, ctx->s_err2.p, A * 8, cudaMemcpyDeviceToHost, s), "download");
  CAPI_TRY(ctx, cudaStreamSynchronize(s), "filter/split");
  return PG_OK;
}

int pg_reduce_sum(pg_context* ctx, const double* x, uint64_t n, double* out) {
  if (!ctx || !out || (n && !x)) return set_err(ctx, PG_BAD_ARG, "null argument");
  Guard g(ctx);
  const uint64_t nch = div_up(n, pg::kChunk);
  CAPI_ENSURE(ctx, ctx->s_x, n * 8 + 8);
  CAPI_ENSURE(ctx, ctx->s_part, (nch + 1) * sizeof(pg::NS));
  CAPI_ENSURE(ctx, ctx->s_res, 8);
  cudaStream_t s = ctx->eng->stream();
  if (n) CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_x.p, x, n * 8, cudaMemcpyHostToDevice, s), "upload");
  if (nch) pg::sum_chunks_kernel<<<(unsigned)nch, pg::kRedThreads, 0, s>>>((const double*)ctx->s_x.p, n, (pg::NS*)ctx->s_part.p);
  pg::sum_final_kernel<<<1, pg::kRedThreads, 0, s>>>((const pg::NS*)ctx->s_part.p, nch, (double*)ctx->s_res.p);
  ctx->eng->stats.launches += nch ? 2 : 1;
  CAPI_TRY(ctx, cudaGetLastError(), "reduce launch");
  CAPI_TRY(ctx, cudaMemcpyAsync(out, ctx->s_res.p, 8, cudaMemcpyDeviceToHost, s), "download");
  CAPI_TRY(ctx, cudaStreamSynchronize(s), "reduce");
  return PG_OK;
}

int pg_exclusive_scan_flags(pg_context* ctx, const uint8_t* flags, uint64_t n, uint64_t* out, uint64_t* total) {
  if (!ctx || (n && (!flags || !out))) return set_err(ctx, PG_BAD_ARG, "null argument");
  Guard g(ctx);
  if (n == 0) {
    if (total) *total = 0;
    return PG_OK;
  }
  const uint64_t nch = div_up(n, pg::kChunk);
  CAPI_ENSURE(ctx, ctx->s_act, n);
  CAPI_ENSURE(ctx, ctx->s_x, n * 8);
  CAPI_ENSURE(ctx, ctx->s_part, nch * 8);
  CAPI_ENSURE(ctx, ctx->s_off, nch * 8 + 8);
  cudaStream_t s = ctx->eng->stream();
  CAPI_TRY(ctx, cudaMemcpyAsync(ctx->s_act.p, flags, n, cudaMemcpyHostToDevice, s), "upload");
  uint64_t* counts = (uint64_t*)ctx->s_part.p;
  uint64_t* off = (uint64_t*)ctx->s_off.p;
  flag_count_kernel<<<(unsigned)nch, pg::kRedThreads, 0, s>>>((const uint8_t*)ctx->s_act.p, n, counts);
  chunk_scan_kernel<<<1, pg::kRedThreads, 0, s>>>(counts, nch, off, off + nch);
  flag_offsets_kernel<<<(unsigned)nch, pg::kRedThreads, 0, s>>>((const uint8_t*)ctx->s_act.p, n, off,
                                                                (uint64_t*)ctx->s_x.p);
  ctx->eng->stats.launches += 3;
  CAPI_TRY(ctx, cudaGetLastError(), "scan launch");
  CAPI_TRY(ctx, cudaMemcpyAsync(out, ctx->s_x.p, n * 8, cudaMemcpyDeviceToHost, s), "download");
  uint64_t tot = 0;
  CAPI_TRY(ctx, cudaMemcpyAsync(&tot, off + nch, 8, cudaMemcpyDeviceToHost, s), "download");
  CAPI_TRY(ctx, cudaStreamSynchronize(s), "scan");
  if (total) *total = tot;
  return PG_OK;
}

int pg_rule_tables(int ndim, double* w, double* scale, double* norm, int32_t* set_of, double* gen) {
  if (ndim < PG_MIN_NDIM || ndim > pg::kMaxNdim) return PG_BAD_ARG;
  const pg::RuleTable r = pg::make_rule(ndim);
  if (w) std::memcpy(w, r.w, sizeof r.w);
  if (scale) std::memcpy(scale, r.scale, sizeof r.scale);
  if (norm) std::memcpy(norm, r.norm, sizeof r.norm);
  if (set_of)
    for (int p = 0; p < r.feval; ++p) set_of[p] = r.set_of[p];
  if (gen) std::memcpy(gen, r.gen.data(), r.gen.size() * sizeof(double));
  return r.feval;
}

int do_integration_from_c(double* res) {
  if (!res) return 1;
  pg_context* ctx = nullptr;
  if (pg_context_create(0, &ctx) != PG_OK) return PG_CUDA_ERROR;
  pg_integrand f;
  std::memset(&f, 0, sizeof f);
  f.family = PG_FAMILY_PRODUCT;
  f.ndim = 2;
  pg_result r;
  const int rc = pg_integrate(ctx, &f, 1.0e-6, 1.0e-12, nullptr, nullptr, nullptr, &r);
  pg_context_destroy(ctx);
  if (rc < 0) return rc;
  if (r.status == 0) *res = r.estimate;
  return r.status;
}

int pg_probe_fp64_peak(pg_context* ctx, double* tflops) {
  if (!ctx || !tflops) return set_err(ctx, PG_BAD_ARG, "null argument");
  Guard g(ctx);
  CAPI_ENSURE(ctx, ctx->s_res, 8);
  cudaStream_t s = ctx->eng->stream();
  cudaEvent_t a, b;
  CAPI_TRY(ctx, cudaEventCreate(&a), "event");
  CAPI_TRY(ctx, cudaEventCreate(&b), "event");
  const int blocks = ctx->eng->num_sms * 8, threads = 256, iters = 4096;
  double best = 0;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(a, s);
    fp64_fma_probe_kernel<<<blocks, threads, 0, s>>>((double*)ctx->s_res.p, iters, 0.999999, 1e-7);
    cudaEventRecord(b, s);
    CAPI_TRY(ctx, cudaEventSynchronize(b), "probe");
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    const double tf = 2.0 * 8 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
    if (rep > 0 && tf > best) best = tf;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  ctx->eng->stats.launches += 3;
  *tflops = best;
  return PG_OK;
}

// ---------------- m-Cubes ----------------
void pg_mcubes_options_default(pg_mcubes_options* opt) {
  if (!opt) return;
  std::memset(opt, 0, sizeof *opt);
  opt->ncall = 1e6;
  opt->titer = 15;
  opt->itmax = 15;
  opt->skip = 5;
  opt->nbins = 500;
  opt->seed = 0x5eed;
  opt->alpha = 1.5;
}

int pg_mcubes_integrate(pg_context* ctx, const pg_integrand* f, double epsrel, double epsabs, const double* lows,
                        const double* highs, const pg_mcubes_options* opt, pg_result* out) {
  if (!ctx || !f || !out) return set_err(ctx, PG_BAD_ARG, "null argument");
  int rc = validate_eps(ctx, epsrel, epsabs);
  if (rc != PG_OK) return rc;
  Guard g(ctx);
  pg_mcubes_options o;
  if (opt) o = *opt; else pg_mcubes_options_default(&o);
  pg::IntegralDesc D;
  std::string why;
  rc = pg::prepare_desc(*f, lows, highs, &D, &why);
  if (rc != PG_OK) return set_err(ctx, rc, why);
  if (!ctx->mc) {
    ctx->mc = pg::mcubes_create(ctx->eng);
    if (!ctx->mc) return set_err(ctx, PG_OOM, "m-Cubes state");
  }
  rc = pg::mcubes_run(ctx->mc, D, epsrel, epsabs, o, out, &why);
  if (rc < 0) return set_err(ctx, rc, why);
  return out->status == 0 ? PG_OK : PG_NOT_CONVERGED;
}

int pg_mcubes_integrate_launcher(pg_context* ctx, int32_t ndim, pg_mcubes_launcher launch, void* user,
                                 double epsrel, double epsabs, const double* lows, const double* highs,
                                 const pg_mcubes_options* opt, pg_result* out) {
  if (!ctx || !launch || !out) return set_err(ctx, PG_BAD_ARG, "null argument");
  int rc = validate_eps(ctx, epsrel, epsabs);
  if (rc != PG_OK) return rc;
  Guard g(ctx);
  pg_mcubes_options o;
  if (opt) o = *opt; else pg_mcubes_options_default(&o);
  pg::IntegralDesc D;
  std::string why;
  rc = pg::prepare_user_desc(ndim, lows, highs, &D, &why);
  if (rc != PG_OK) return set_err(ctx, rc, why);
  if (!ctx->mc) {
    ctx->mc = pg::mcubes_create(ctx->eng);
    if (!ctx->mc) return set_err(ctx, PG_OOM, "m-Cubes state");
  }
  const pg::McubesLauncher L = [launch, user](const pg_mcubes_args& a) -> cudaError_t {
    return (cudaError_t)launch(&a, user);
  };
  rc = pg::mcubes_run(ctx->mc, D, epsrel, epsabs, o, out, &why, L);
  if (rc < 0) return set_err(ctx, rc, why);
  return out->status == 0 ? PG_OK : PG_NOT_CONVERGED;
}

}  // extern "C"
