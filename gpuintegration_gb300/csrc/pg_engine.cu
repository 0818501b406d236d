// Host engine of the GB300 PAGANI iteration (see pg_engine.h).
#include "pg_engine.h"
#include "pg_setsum.cuh"

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cmath>
#include <thread>
#include <cstdio>
#include <cstring>
#include <sstream>

namespace pg {

namespace {

inline uint64_t div_up(uint64_t a, uint64_t b) { return (a + b - 1) / b; }

inline int parts_for(int d) { return d < 5 ? 4 : (d <= 10 ? 2 : 1); }

inline uint64_t ipow_u(uint64_t b, int e) {
  uint64_t r = 1;
  for (int i = 0; i < e; ++i) r *= b;
  return r;
}

std::string fixed15(double v) {
  std::ostringstream out;
  out.precision(15);
  out << std::fixed << v;
  return out.str();
}

}  // namespace

// ---------------------------------------------------------------------------
// Classifier state (heuristic_classifier.cuh:89-280).
// ---------------------------------------------------------------------------
uint64_t ClassifierState::mem_required(uint64_t n) const {
  // Bytes a full split of n regions needs in the reference's accounting
  // (heuristic_classifier.cuh:227-264).
  const uint64_t d = (uint64_t)ndim;
  const uint64_t doubles = n + n + 2 * n + 2 * n + 2 * n * d + 2 * n * d + n * d * 2 + n * d * 2 + n + n + n * d + n * d;
  const uint64_t ints = n + 2 * n + n;
  return 8 * doubles + 4 * ints;
}

uint64_t ClassifierState::free_mem(uint64_t n) const {
  const uint64_t total = (uint64_t)total_mem;
  const uint64_t occ = mem_required(n);
  return total > occ ? total - occ : 1;
}

bool ClassifierState::sig_digits_same() const {
  double third = std::fabs(last[0]), second = std::fabs(last[1]), first = std::fabs(last[2]);
  while (first != 0. && first < 1.) first *= 10;
  while (second != 0. && second < 1.) second *= 10;
  while (third != 0. && third < 1.) third *= 10;
  const std::string a = fixed15(third), b = fixed15(second), c = fixed15(first);
  bool verdict = true;
  int sig = 0;
  for (int i = 0; i < required_digits + 1 && sig < required_digits && verdict; ++i) {
    const char ci = i < (int)c.size() ? c[i] : '\0';
    const char bi = i < (int)b.size() ? b[i] : '\0';
    const char ai = i < (int)a.size() ? a[i] : '\0';
    verdict = (ci == bi && bi == ai);
    sig += (verdict && ci != '.') ? 1 : 0;
  }
  return verdict;
}

bool ClassifierState::estimate_converged() const { return !(iters_collected - 1 < 1 || !sig_digits_same()); }

void ClassifierState::store(double e) {
  last[0] = last[1];
  last[1] = last[2];
  last[2] = e;
  iters_collected++;
}

bool ClassifierState::criteria_met(uint64_t n) const {
  const double ratio = (double)mem_required(n) / (double)free_mem(n);
  if (ratio > 1.) return true;
  if (ratio > .1 && estimate_converged()) return true;
  return false;
}

// ---------------------------------------------------------------------------
// c^d (1 when c is 0), the constant factor of GAUSSIAN_SUM: d - 1 multiplies
// in axis order.
static double gaussian_sum_scale(double c, int d) {
  if (c == 0.0) return 1.0;
  double r = c;
  for (int k = 1; k < d; ++k) r = r * c;
  return r;
}

int prepare_desc(const pg_integrand& f, const double* lows, const double* highs, IntegralDesc* out,
                 std::string* why) {
  if (f.ndim < PG_MIN_NDIM || f.ndim > kMaxNdim) {
    if (why) *why = "ndim out of range";
    return PG_BAD_ARG;
  }
  if (f.family < 0 || f.family >= FAM_COUNT) {
    if (why) *why = "unknown integrand family";
    return PG_BAD_ARG;
  }
  if (f.family == FAM_FUN6 && f.ndim != 6) {
    if (why) *why = "FUN6 is a 6-dimensional integrand";
    return PG_BAD_ARG;
  }
  IntegralDesc D;
  std::memset(&D, 0, sizeof D);
  D.family = f.family;
  D.d = f.ndim;
  D.c = f.c;
  D.s0 = 2.0 * 3.14159265358979323846 * f.u[0];
  if (f.family == FAM_FUN6) D.c = 12.0 / (7.0 - 6.0 * std::log(2.0) * std::log(2.0) + std::log(64.0));
  if (f.family == FAM_GAUSSIAN_SUM) D.s0 = gaussian_sum_scale(f.c, f.ndim);
  D.jac = 1.0;
  int unit = 1;
  for (int k = 0; k < kMaxDim; ++k) {
    D.a[k] = f.a[k];
    D.u[k] = f.u[k];
    D.ia2[k] = 1.0 / (f.a[k] * f.a[k]);
  }
  for (int k = 0; k < f.ndim; ++k) {
    const double lo = lows ? lows[k] : 0.0, hi = highs ? highs[k] : 1.0;
    if (!(hi > lo) || !std::isfinite(lo) || !std::isfinite(hi)) {
      if (why) *why = "each axis needs finite bounds with low < high";
      return PG_BAD_ARG;
    }
    D.glo[k] = lo;
    D.range[k] = hi - lo;
    D.jac = D.jac * D.range[k];
    if (lo != 0.0 || D.range[k] != 1.0) unit = 0;
  }
  D.unit = unit;
  *out = D;
  return PG_OK;
}

int prepare_user_desc(int ndim, const double* lows, const double* highs, IntegralDesc* out, std::string* why) {
  pg_integrand f;
  std::memset(&f, 0, sizeof f);
  f.family = FAM_CONSTANT;
  f.ndim = ndim;
  const int rc = prepare_desc(f, lows, highs, out, why);
  if (rc == PG_OK) out->family = FAM_USER;
  return rc;
}

// ---------------------------------------------------------------------------
Engine::Engine(int dev) : device(dev) {}

Engine::~Engine() {
  cudaSetDevice(device);
  DevBuf* dev_bufs[] = {&rule_trie_, &rule_leafset_, &rule_code_, &rule_w_, &rule_scale_, &rule_norm_, &left_[0], &left_[1], &len_[0], &len_[1],
                        &owner_[0], &owner_[1], &parent_[0], &parent_[1], &est_, &err_a_, &err_b_, &bisect_,
                        &terms_[0], &terms_[1], &ppos_[0], &ppos_[1], &chk_,
                        &active_, &partials_, &chunk_off_, &chunks_, &segs_, &trans_, &descs_, &scal_, &live_,
                        &thr_out_, &thr_counts_, &adm_starts_, &adm_ids_, &rst_items_, &chain_, &chain_ts_};
  for (DevBuf* b : dev_bufs)
    if (b->p) cudaFree(b->p);
  DevBuf* host_bufs[] = {&h_segs_, &h_chunks_, &h_trans_, &h_trans_spill_, &h_scal_, &h_live_, &h_thr_,
                         &h_adm_starts_, &h_adm_ids_, &h_rst_items_, &h_thr_counts_, &h_chain_, &h_chk_};
  for (DevBuf* b : host_bufs)
    if (b->p) cudaFreeHost(b->p);
  for (auto& e : ev_)
    if (e) cudaEventDestroy(e);
  if (stream_) cudaStreamDestroy(stream_);
}

int Engine::fail(cudaError_t e, const char* what) {
  last_error = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return PG_OOM;
  return PG_CUDA_ERROR;
}

#define PG_TRY(call, what)                  \
  do {                                      \
    cudaError_t e_ = (call);                \
    if (e_ != cudaSuccess) return fail(e_, what); \
  } while (0)

SpillArena::~SpillArena() {
  for (Block& b : blocks_) cudaFreeHost(b.base);
}

void* SpillArena::alloc(size_t bytes) {
  bytes = (bytes + 255) & ~(size_t)255;
  if (bytes == 0) bytes = 256;
  for (int attempt = 0; attempt < 2; ++attempt) {
    for (Block& b : blocks_)
      for (auto it = b.free.begin(); it != b.free.end(); ++it)
        if (it->second >= bytes) {
          const size_t off = it->first, len = it->second;
          b.free.erase(it);
          if (len > bytes) b.free[off + bytes] = len - bytes;
          return b.base + off;
        }
    // No room: a new block of at least 1 GiB.
    const size_t want = std::max(bytes, (size_t)1 << 30);
    void* p = nullptr;
    if (cudaMallocHost(&p, want) != cudaSuccess) return nullptr;
    Block nb;
    nb.base = (char*)p;
    nb.bytes = want;
    nb.free[0] = want;
    blocks_.push_back(std::move(nb));
    total_ += want;
  }
  return nullptr;
}

void SpillArena::release(void* ptr, size_t bytes) {
  if (!ptr) return;
  bytes = (bytes + 255) & ~(size_t)255;
  if (bytes == 0) bytes = 256;
  char* p = (char*)ptr;
  for (Block& b : blocks_) {
    if (p < b.base || p >= b.base + b.bytes) continue;
    size_t off = (size_t)(p - b.base), len = bytes;
    auto next = b.free.lower_bound(off);
    if (next != b.free.end() && off + len == next->first) {  // merge with the following range
      len += next->second;
      next = b.free.erase(next);
    }
    if (next != b.free.begin()) {  // merge with the preceding range
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        prev->second += len;
        return;
      }
    }
    b.free[off] = len;
    return;
  }
}

void SpillArena::reset() {
  for (Block& b : blocks_) {
    b.free.clear();
    b.free[0] = b.bytes;
  }
}

int Engine::ensure(DevBuf& b, size_t bytes) {
  if (b.bytes >= bytes) return PG_OK;
  // Kernels queued on the stream may still read the old buffer.
  if (stream_) PG_TRY(cudaStreamSynchronize(stream_), "stream sync before reallocation");
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
  size_t want = std::max(bytes, (size_t)4096);
  if (fail_alloc_after >= 0 && fail_alloc_after-- == 0) return fail(cudaErrorMemoryAllocation, "cudaMalloc (injected)");
  PG_TRY(cudaMalloc(&b.p, want), "cudaMalloc");
  b.bytes = want;
  return PG_OK;
}

int Engine::ensure_pinned(DevBuf& b, size_t bytes) {
  if (b.bytes >= bytes) return PG_OK;
  if (stream_) PG_TRY(cudaStreamSynchronize(stream_), "stream sync before reallocation");
  if (b.p) cudaFreeHost(b.p);
  b.p = nullptr;
  b.bytes = 0;
  size_t want = std::max(bytes, (size_t)4096);
  if (fail_alloc_after >= 0 && fail_alloc_after-- == 0)
    return fail(cudaErrorMemoryAllocation, "cudaMallocHost (injected)");
  PG_TRY(cudaMallocHost(&b.p, want), "cudaMallocHost");
  b.bytes = want;
  return PG_OK;
}

int Engine::init(std::string* why) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    if (why) *why = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
    return PG_CUDA_ERROR;
  }
  int rc;
#define PG_INIT_TRY(call, what)                                                     \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      if (why) *why = std::string(what) + ": " + cudaGetErrorString(e_);            \
      return e_ == cudaErrorMemoryAllocation ? PG_OOM : PG_CUDA_ERROR;              \
    }                                                                               \
  } while (0)
  PG_INIT_TRY(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
  PG_INIT_TRY(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device), "cudaDeviceGetAttribute");
  for (auto& ev : ev_) PG_INIT_TRY(cudaEventCreate(&ev), "cudaEventCreate");
  // Rule tables for every supported ndim.
  std::vector<uint64_t> codes;
  std::vector<double> w((kMaxNdim + 1) * 45, 0.0), sc((kMaxNdim + 1) * 45, 0.0), nm((kMaxNdim + 1) * 45, 0.0);
  RuleDev R;
  std::memset(&R, 0, sizeof R);
  RuleTable r2;
  for (int d = PG_MIN_NDIM; d <= kMaxNdim; ++d) {
    RuleTable t = make_rule(d);
    R.code_off[d] = (int32_t)codes.size();
    R.feval[d] = t.feval;
    codes.insert(codes.end(), t.code.begin(), t.code.end());
    std::memcpy(&w[d * 45], t.w, sizeof t.w);
    std::memcpy(&sc[d * 45], t.scale, sizeof t.scale);
    std::memcpy(&nm[d * 45], t.norm, sizeof t.norm);
    if (d == PG_MIN_NDIM) r2 = t;
  }
  code_coefficients(r2, R.A, R.B);
  std::vector<uint16_t> tries;
  std::vector<uint32_t> leafset;
  for (int d = PG_MIN_NDIM; d <= kMaxNdim; ++d) {
    RuleTable t = make_rule(d);
    std::vector<uint16_t> inner;
    std::vector<uint32_t> leaf;
    split_trie(t, &inner, &leaf);
    R.trie_off[d] = (int32_t)tries.size();
    tries.insert(tries.end(), inner.begin(), inner.end());
    R.leafset_off[d] = (int32_t)leafset.size();
    leafset.insert(leafset.end(), leaf.begin(), leaf.end());
  }
  const double q = r2.G[1] / r2.G[0];
  R.ratio = q * q;
  R.omr = 1.0 - R.ratio;
  if ((rc = ensure(rule_code_, codes.size() * 8)) != PG_OK) {
    if (why) *why = last_error;
    return rc;
  }
  if ((rc = ensure(rule_w_, w.size() * 8)) != PG_OK || (rc = ensure(rule_scale_, sc.size() * 8)) != PG_OK ||
      (rc = ensure(rule_norm_, nm.size() * 8)) != PG_OK) {
    if (why) *why = last_error;
    return rc;
  }
  PG_INIT_TRY(cudaMemcpy(rule_code_.p, codes.data(), codes.size() * 8, cudaMemcpyHostToDevice), "rule upload");
  PG_INIT_TRY(cudaMemcpy(rule_w_.p, w.data(), w.size() * 8, cudaMemcpyHostToDevice), "rule upload");
  PG_INIT_TRY(cudaMemcpy(rule_scale_.p, sc.data(), sc.size() * 8, cudaMemcpyHostToDevice), "rule upload");
  PG_INIT_TRY(cudaMemcpy(rule_norm_.p, nm.data(), nm.size() * 8, cudaMemcpyHostToDevice), "rule upload");
  if ((rc = ensure(rule_trie_, tries.size() * 2)) != PG_OK) {
    if (why) *why = last_error;
    return rc;
  }
  PG_INIT_TRY(cudaMemcpy(rule_trie_.p, tries.data(), tries.size() * 2, cudaMemcpyHostToDevice), "rule upload");
  if ((rc = ensure(rule_leafset_, leafset.size() * 4)) != PG_OK) {
    if (why) *why = last_error;
    return rc;
  }
  PG_INIT_TRY(cudaMemcpy(rule_leafset_.p, leafset.data(), leafset.size() * 4, cudaMemcpyHostToDevice), "rule upload");
  R.leafset = (const uint32_t*)rule_leafset_.p;
  R.trie = (const uint16_t*)rule_trie_.p;
  R.code = (const uint64_t*)rule_code_.p;
  R.w = (const double*)rule_w_.p;
  R.scale = (const double*)rule_scale_.p;
  R.norm = (const double*)rule_norm_.p;
  rule_ = R;
  if ((rc = ensure(thr_out_, 64)) != PG_OK || (rc = ensure_pinned(h_thr_, 64)) != PG_OK ||
      (rc = ensure(thr_counts_, kMaxThresholds * 8)) != PG_OK ||
      (rc = ensure_pinned(h_thr_counts_, kMaxThresholds * 8)) != PG_OK || (rc = ensure(chain_, 64 * 8)) != PG_OK ||
      (rc = ensure_pinned(h_chain_, 64 * 8)) != PG_OK || (rc = ensure(chain_ts_, sizeof(ThresholdSet))) != PG_OK ||
      (rc = ensure(chk_, 64)) != PG_OK || (rc = ensure_pinned(h_chk_, 64)) != PG_OK) {
    if (why) *why = last_error;
    return rc;
  }
#undef PG_INIT_TRY
  return PG_OK;
}

void Engine::record(cudaEvent_t a, cudaEvent_t b, double* acc) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) == cudaSuccess) *acc += ms;
}

int Engine::evaluate(const IntegralDesc& desc, uint64_t n, const double* d_left, const double* d_length,
                     uint64_t stride, double* d_est, double* d_err, int32_t* d_bisect, const EvalLauncher& launch,
                     int mode) {
  int rc;
  if ((rc = autotune()) != PG_OK) return rc;
  if ((rc = ensure(descs_, sizeof(IntegralDesc))) != PG_OK) return rc;
  PG_TRY(cudaMemcpyAsync(descs_.p, &desc, sizeof desc, cudaMemcpyHostToDevice, stream_), "desc upload");
  if (n == 0) return PG_OK;
  const EvalTune& tn = tune[desc.d <= 8 ? 0 : 1];
  EvalLaunch L{d_left, d_length, n, stride, nullptr, (const IntegralDesc*)descs_.p, &rule_, d_est, d_err, d_bisect,
               desc.d, num_sms, stream_, tn.warps, tn.ctas_per_sm};
  L.mode = (mode == PG_EVAL_SET_SUMS && family_separable(desc.family)) ? PG_EVAL_SET_SUMS : PG_EVAL_POINTS;
  L.scale = desc.jac != 1.0;
  if (profiling) cudaEventRecord(ev_[0], stream_);
  PG_TRY(launch(L), "evaluation launch");
  stats.launches++;
  stats.eval_launches++;
  stats.regions_evaluated += n;
  if (L.mode == PG_EVAL_SET_SUMS) stats.setsum_regions += n;
  stats.points_evaluated += n * (uint64_t)rule_.feval[desc.d];
  stats.eval_bytes += n * (16ull * desc.d + 20ull);  // bounds in; estimate, error, split axis out
  if (profiling) {
    cudaEventRecord(ev_[1], stream_);
    PG_TRY(cudaEventSynchronize(ev_[1]), "evaluation");
    record(ev_[0], ev_[1], &stats.eval_ms);
  }
  return PG_OK;
}

// One pass of the threshold kernels over integral jidx's chunks; out = {sum
// err*flag, sum est*flag, count, min err, max err}.
// Without readback the pass is only enqueued (its flags and chunk offsets feed
// the compaction later on the stream).
int Engine::threshold_pass(uint32_t jidx, double thr, int write_flags, int minmax, int scan, double out[5],
                           bool readback) {
  const SegDesc& S = ((const SegDesc*)h_segs_.p)[jidx];
  if (S.nchunks) {
    // the sums are read only from a pass that neither writes flags nor takes extremes
    auto kern = (!write_flags && !minmax) ? threshold_kernel<true> : threshold_kernel<false>;
    kern<<<S.nchunks, kRedThreads, 0, stream_>>>((const ChunkRef*)chunks_.p, (const SegDesc*)segs_.p, S.chunk_start,
                                                 (const double*)est_.p, (const double*)err_b_.p, thr, nullptr,
                                                 write_flags, minmax, (uint8_t*)active_.p, (Partial*)partials_.p);
    stats.launches++;
  }
  threshold_finalize_kernel<<<1, kRedThreads, 0, stream_>>>((const SegDesc*)segs_.p, jidx,
                                                            (const Partial*)partials_.p, (uint64_t*)chunk_off_.p,
                                                            scan, (double*)thr_out_.p);
  stats.launches++;
  PG_TRY(cudaGetLastError(), "threshold launch");
  if (!readback) return PG_OK;
  PG_TRY(cudaMemcpyAsync(h_thr_.p, thr_out_.p, 5 * sizeof(double), cudaMemcpyDeviceToHost, stream_),
         "threshold readback");
  PG_TRY(cudaStreamSynchronize(stream_), "threshold pass");
  stats.classify_passes++;
  std::memcpy(out, h_thr_.p, 5 * sizeof(double));
  stats.d2h_bytes += 5 * sizeof(double);
  return PG_OK;
}

int Engine::threshold_counts(uint32_t jidx, const double* thr, int k, uint64_t* counts) {
  const SegDesc& S = ((const SegDesc*)h_segs_.p)[jidx];
  ThresholdSet ts;
  std::memset(&ts, 0, sizeof ts);
  ts.k = k;
  for (int q = 0; q < k; ++q) {
    if (!(thr[q] >= 0.0)) {  // the kernel compares bit patterns of non-negative values
      last_error = "negative threshold";
      return PG_BAD_ARG;
    }
    const double t = thr[q] + 0.0;  // +0 for a -0 threshold
    std::memcpy(&ts.bits[q], &t, 8);
  }
  PG_TRY(cudaMemsetAsync(thr_counts_.p, 0, kMaxThresholds * 8, stream_), "threshold counts");
  if (S.nchunks) {
    threshold_count_kernel<<<S.nchunks, kRedThreads, 0, stream_>>>(
        (const ChunkRef*)chunks_.p, (const SegDesc*)segs_.p, S.chunk_start, (const double*)err_b_.p, ts, nullptr,
        (unsigned long long*)thr_counts_.p);
    stats.launches++;
  }
  PG_TRY(cudaGetLastError(), "threshold count launch");
  PG_TRY(cudaMemcpyAsync(h_thr_counts_.p, thr_counts_.p, k * 8, cudaMemcpyDeviceToHost, stream_), "count readback");
  PG_TRY(cudaStreamSynchronize(stream_), "threshold counts");
  stats.classify_passes++;
  std::memcpy(counts, h_thr_counts_.p, k * 8);
  stats.d2h_bytes += k * 8;
  return PG_OK;
}

// The classifier's first three passes with one host round trip: the min/max
// pass, the counts above the 20 thresholds of the raise sequence (built on
// the device from the maximum), and the pass at the threshold where the raise
// loop stops (chosen on the device from the counts).  The host repeats the
// sequence and the choice with the same operations and takes the results from
// h_chain_.
int Engine::classify_chain(uint32_t jidx, double thr0, double pct, uint64_t n) {
  const SegDesc& S = ((const SegDesc*)h_segs_.p)[jidx];
  double* cb = (double*)chain_.p;
  unsigned long long* cnt = (unsigned long long*)(cb + 16);
  ThresholdSet* ts = (ThresholdSet*)chain_ts_.p;
  const ChunkRef* ch = (const ChunkRef*)chunks_.p;
  const SegDesc* sg = (const SegDesc*)segs_.p;
  ThresholdSet none;
  std::memset(&none, 0, sizeof none);
  if (S.nchunks) {
    threshold_kernel<false><<<S.nchunks, kRedThreads, 0, stream_>>>(ch, sg, S.chunk_start, (const double*)est_.p,
                                                                    (const double*)err_b_.p, INFINITY, nullptr, 0,
                                                                    1, (uint8_t*)active_.p, (Partial*)partials_.p);
    stats.launches++;
  }
  threshold_finalize_kernel<<<1, kRedThreads, 0, stream_>>>(sg, jidx, (const Partial*)partials_.p,
                                                            (uint64_t*)chunk_off_.p, 0, cb);
  threshold_seq_kernel<<<1, 32, 0, stream_>>>(cb, thr0, ts, cb + 40);
  PG_TRY(cudaMemsetAsync(cnt, 0, kMaxThresholds * 8, stream_), "threshold counts");
  if (S.nchunks) {
    threshold_count_kernel<<<S.nchunks, kRedThreads, 0, stream_>>>(ch, sg, S.chunk_start, (const double*)err_b_.p,
                                                                   none, ts, cnt);
    stats.launches++;
  }
  threshold_select_kernel<<<1, 32, 0, stream_>>>(cnt, cb + 40, n, pct, cb + 60);
  if (S.nchunks) {
    threshold_kernel<true><<<S.nchunks, kRedThreads, 0, stream_>>>(ch, sg, S.chunk_start, (const double*)est_.p,
                                                                   (const double*)err_b_.p, 0.0, cb + 60, 0, 0,
                                                                   (uint8_t*)active_.p, (Partial*)partials_.p);
    stats.launches++;
  }
  threshold_finalize_kernel<<<1, kRedThreads, 0, stream_>>>(sg, jidx, (const Partial*)partials_.p,
                                                            (uint64_t*)chunk_off_.p, 0, cb + 8);
  stats.launches += 4;
  PG_TRY(cudaGetLastError(), "threshold chain launch");
  PG_TRY(cudaMemcpyAsync(h_chain_.p, cb, 64 * 8, cudaMemcpyDeviceToHost, stream_), "threshold chain readback");
  PG_TRY(cudaStreamSynchronize(stream_), "threshold chain");
  stats.classify_passes++;
  stats.d2h_bytes += 64 * 8;
  return PG_OK;
}

// Memory-pressure classification of one integral (heuristic_classifier.cuh:362-451,
// Workspace.cuh:74-118).  On success the integral's active flags and chunk
// offsets are rewritten for the threshold found.
int Engine::classify_job(Job& J, uint32_t jidx, double iter_err, double fin_err, bool* ok_out, double* fin_est_out,
                         double* fin_err_out, uint64_t* num_active_out, double iter_est) {
  ClassifierState& C = J.cls;
  const uint64_t n = J.n;
  double o[5];
  int rc;
  const auto t_cls = std::chrono::steady_clock::now();
  const double thr0 = iter_err / (double)n;
  // A first raise step is certain (nothing passes before it); with a
  // non-negative start its three passes run chained, with one round trip.
  bool first = thr0 >= 0.0;
  const double* hc = (const double*)h_chain_.p;
  if (first) {
    if ((rc = classify_chain(jidx, thr0, C.max_active_regions_percentage, n)) != PG_OK) return rc;
    std::memcpy(o, hc, sizeof o);
  } else if ((rc = threshold_pass(jidx, INFINITY, 0, 1, 0, o)) != PG_OK) {
    return rc;
  }
  const double mn = o[3], mx = o[4];
  double low = mn, high = mx, thr = thr0, flags_thr = thr;
  bool pass_mem = false, pass_budget = false;
  uint64_t num_active = 0;
  double dot_err = 0, dot_est = 0, finished_errorest = 0;
  const double target = std::fabs(C.last[2]) * C.epsrel;
  uint64_t inc = 0, dec = 0;
  auto take = [&](const double* q, double t) {
    flags_thr = t;
    dot_err = q[0];
    dot_est = q[1];
    num_active = (uint64_t)q[2];
    const double pct = (double)(int)num_active / (double)(int)n;
    pass_mem = pct <= C.max_active_regions_percentage;
  };
  auto apply = [&](double t) -> int {
    double q[5];
    int r2 = threshold_pass(jidx, t, 0, 0, 0, q);
    if (r2 != PG_OK) return r2;
    take(q, t);
    return PG_OK;
  };
  do {
    if (!pass_mem && inc <= 20 && !(thr >= 0.0)) {  // (never: thresholds are error values) one pass each
      pass_mem = false;
      for (uint64_t cnt = 0; !pass_mem && cnt < 20; ++cnt) {
        if ((rc = apply(thr)) != PG_OK) return rc;
        if (!pass_mem) {
          low = thr;
          thr += std::fabs(high - thr) * .5;
        }
      }
      inc++;
    } else if (!pass_mem && inc <= 20) {
      // The reference raises the threshold up to 20 times until few enough
      // regions stay active (heuristic_classifier.cuh:380-395).  The
      // thresholds it tries do not depend on the outcomes, and the test needs
      // only the count above each, so all 20 counts come from one pass; the
      // full pass then runs at the threshold where the search stops.
      double seq[kMaxThresholds];
      double t = thr;
      for (int q = 0; q < kMaxThresholds; ++q) {
        seq[q] = t;
        t += std::fabs(high - t) * .5;
      }
      uint64_t cnt[kMaxThresholds];
      // the chain's sequence is this one, bit for bit (same operations)
      const bool chained = first && std::memcmp(seq, hc + 40, sizeof seq) == 0;
      first = false;
      if (chained)
        std::memcpy(cnt, hc + 16, sizeof cnt);
      else if ((rc = threshold_counts(jidx, seq, kMaxThresholds, cnt)) != PG_OK)
        return rc;
      int stop = -1;
      for (int q = 0; q < kMaxThresholds && stop < 0; ++q)
        if ((double)(int)cnt[q] / (double)(int)n <= C.max_active_regions_percentage) stop = q;
      const int last = stop >= 0 ? stop : kMaxThresholds - 1;
      if (chained && std::memcmp(&seq[last], hc + 60, 8) == 0)
        take(hc + 8, seq[last]);
      else if ((rc = apply(seq[last])) != PG_OK)
        return rc;
      if (stop >= 0) {
        if (stop > 0) low = seq[stop - 1];
        thr = seq[stop];
      } else {
        low = seq[last];
        thr = t;  // the threshold after the 20th
      }
      inc++;
    }
    if (pass_mem) {
      const double extra = iter_err - dot_err - fin_err;
      const double budget = target - J.res.errorest;
      pass_budget = extra <= C.max_percent_error_budget * budget;
      finished_errorest = extra;
      if (!pass_budget && dec <= 20) {
        high = thr;
        thr -= std::fabs(low - thr) * .5;
        pass_mem = false;
        dec++;
      }
    }
    const bool exhausted = dec >= 20 || inc >= 20;
    if (exhausted && C.max_percent_error_budget < .7) {
      C.max_percent_error_budget += 0.1;
      dec = inc = 0;
      low = mn;
      high = mx;
      thr = iter_err / (double)n;
    } else if (exhausted && C.max_percent_error_budget >= .7 && C.max_active_regions_percentage <= .7) {
      C.max_active_regions_percentage += .1;
    } else if (exhausted) {
      break;
    }
  } while (!pass_mem || !pass_budget);
  C.max_active_regions_percentage = .5;
  C.max_percent_error_budget = .25;
  const bool ok = pass_mem && pass_budget;
  stats.classify_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_cls).count();
  *ok_out = ok;
  *num_active_out = num_active;
  if (ok) {
    if ((rc = threshold_pass(jidx, flags_thr, 1, 0, 1, o, false)) != PG_OK) return rc;  // flags for the compaction
    *fin_est_out = iter_est - dot_est;
    *fin_err_out = finished_errorest;
  }
  return PG_OK;
}

// Grows region list `which` to hold `need` regions with `rows` rows, keeping
// its first `live` regions (and `live_par` parent estimates).
int Engine::grow_list(int which, uint64_t need, int rows, uint64_t live, uint64_t live_par) {
  int rc;
  if (reg_cap_[which] < need || reg_rows_[which] < rows) {
    const uint64_t cap = std::max<uint64_t>(std::max<uint64_t>(need, reg_cap_[which] + reg_cap_[which] / 2), 4096);
    const int r = std::max(rows, reg_rows_[which]);
    PG_TRY(cudaStreamSynchronize(stream_), "stream sync before reallocation");
    DevBuf nl, nn, no;
    PG_TRY(cudaMalloc(&nl.p, cap * r * 8), "cudaMalloc region list");
    nl.bytes = cap * r * 8;
    if (cudaMalloc(&nn.p, cap * r * 8) != cudaSuccess) {
      cudaFree(nl.p);
      return fail(cudaErrorMemoryAllocation, "cudaMalloc region list");
    }
    nn.bytes = cap * r * 8;
    if (cudaMalloc(&no.p, cap * 4) != cudaSuccess) {
      cudaFree(nl.p);
      cudaFree(nn.p);
      return fail(cudaErrorMemoryAllocation, "cudaMalloc region owners");
    }
    no.bytes = cap * 4;
    if (live) {
      const int old_rows = reg_rows_[which];
      PG_TRY(cudaMemcpy2DAsync(nl.p, cap * 8, left_[which].p, reg_cap_[which] * 8, live * 8, old_rows,
                               cudaMemcpyDeviceToDevice, stream_), "grow copy");
      PG_TRY(cudaMemcpy2DAsync(nn.p, cap * 8, len_[which].p, reg_cap_[which] * 8, live * 8, old_rows,
                               cudaMemcpyDeviceToDevice, stream_), "grow copy");
      PG_TRY(cudaMemcpyAsync(no.p, owner_[which].p, live * 4, cudaMemcpyDeviceToDevice, stream_), "grow copy");
      PG_TRY(cudaStreamSynchronize(stream_), "grow copy");
    }
    if (left_[which].p) cudaFree(left_[which].p);
    if (len_[which].p) cudaFree(len_[which].p);
    if (owner_[which].p) cudaFree(owner_[which].p);
    left_[which] = nl;
    len_[which] = nn;
    owner_[which] = no;
    reg_cap_[which] = cap;
    reg_rows_[which] = r;
  }
  // Parent estimates: at most one per region.
  if (parent_[which].bytes < need * 8) {
    DevBuf np;
    const size_t bytes = std::max<size_t>(need * 8, parent_[which].bytes + parent_[which].bytes / 2);
    PG_TRY(cudaStreamSynchronize(stream_), "stream sync before reallocation");
    PG_TRY(cudaMalloc(&np.p, bytes), "cudaMalloc parents");
    np.bytes = bytes;
    if (live_par) PG_TRY(cudaMemcpyAsync(np.p, parent_[which].p, live_par * 8, cudaMemcpyDeviceToDevice, stream_),
                         "grow copy");
    PG_TRY(cudaStreamSynchronize(stream_), "grow copy");
    if (parent_[which].p) cudaFree(parent_[which].p);
    parent_[which] = np;
  }
  (void)rc;
  return PG_OK;
}

// The bounds record of the term lookups, read after a synchronisation: a
// recorded check means a lookup was skipped and the run's results are void.
int Engine::check_bounds() {
  const unsigned long long* r = (const unsigned long long*)h_chk_.p;
  if (r[0] == 0) return PG_OK;
  static const char* what[] = {"", "parent index", "parent position", "term position", "parent record"};
  last_error = std::string("set-sum term lookup out of bounds: ") + what[r[0] < 5 ? r[0] : 0] + " " +
               std::to_string(r[1]) + " >= " + std::to_string(r[2]) + " (integral " + std::to_string(r[3]) +
               ", segment start " + std::to_string(r[4]) + ", regions " + std::to_string(r[5]) + ", position " +
               std::to_string(r[6]) + ")";
  return PG_CUDA_ERROR;
}

int Engine::compact(int cur, int nxt, uint32_t chunk0, uint32_t nchunks, int maxd, double* out_left, double* out_len,
                    uint64_t out_stride, uint32_t* out_owner, double* parent_out, uint32_t* ppos_out,
                    uint64_t ppos_n) {
  (void)nxt;
  if (nchunks == 0) return PG_OK;
  if (maxd <= 8) {
    compact_split_kernel<8><<<nchunks, kRedThreads, 0, stream_>>>(
        (const ChunkRef*)chunks_.p, (const SegDesc*)segs_.p, (const Transition*)trans_.p,
        (const uint64_t*)chunk_off_.p, (const IntegralDesc*)descs_.p, (const uint8_t*)active_.p,
        (const double*)left_[cur].p, (const double*)len_[cur].p, reg_cap_[cur], (const int32_t*)bisect_.p,
        (const double*)est_.p, out_left, out_len, out_stride, out_owner, parent_out, chunk0, ppos_out, ppos_n,
        (unsigned long long*)chk_.p);
  } else {
    compact_split_kernel<16><<<nchunks, kRedThreads, 0, stream_>>>(
        (const ChunkRef*)chunks_.p, (const SegDesc*)segs_.p, (const Transition*)trans_.p,
        (const uint64_t*)chunk_off_.p, (const IntegralDesc*)descs_.p, (const uint8_t*)active_.p,
        (const double*)left_[cur].p, (const double*)len_[cur].p, reg_cap_[cur], (const int32_t*)bisect_.p,
        (const double*)est_.p, out_left, out_len, out_stride, out_owner, parent_out, chunk0, ppos_out, ppos_n,
        (unsigned long long*)chk_.p);
  }
  stats.launches++;
  PG_TRY(cudaGetLastError(), "compact/split launch");
  return PG_OK;
}

int Engine::evaluate_list(std::vector<Job>& jobs, const std::vector<uint32_t>& live, int cur, uint64_t N,
                          const EvalLauncher& launch) {
  // Runs: maximal ranges of consecutive segments whose integrals share an
  // evaluation kernel (placement keeps the kernels' integrals together, so an
  // iteration has a handful of runs).
  struct Run {
    uint64_t start, n;
    int mode, maxd;
    bool scale;
  };
  std::vector<uint32_t> order(live);
  std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return jobs[a].start < jobs[b].start; });
  std::vector<Run> runs;
  for (uint32_t j : order) {
    const Job& J = jobs[j];
    if (J.n == 0) continue;
    const int md = job_eval_mode(J);
    const bool sc = J.desc.jac != 1.0;
    if (!runs.empty() && runs.back().mode == md && runs.back().start + runs.back().n == J.start) {
      runs.back().n += J.n;
      runs.back().maxd = std::max(runs.back().maxd, J.desc.d);
      runs.back().scale |= sc;
    } else {
      runs.push_back(Run{J.start, J.n, md, J.desc.d, sc});
    }
  }
  const double* left = (const double*)left_[cur].p;
  const double* len = (const double*)len_[cur].p;
  const uint32_t* own = (const uint32_t*)owner_[cur].p;
  for (const Run& R : runs) {
    if (R.start + R.n > N) {
      last_error = "evaluation run outside the region list";
      return PG_CUDA_ERROR;
    }
    const EvalTune& tn = tune[R.maxd <= 8 ? 0 : 1];
    EvalLaunch L{left + R.start, len + R.start, R.n, reg_cap_[cur], own + R.start, (const IntegralDesc*)descs_.p,
                 &rule_, (double*)est_.p + R.start, (double*)err_a_.p + R.start, (int32_t*)bisect_.p + R.start,
                 R.maxd, num_sms, stream_, tn.warps, tn.ctas_per_sm};
    L.mode = R.mode;
    L.segs = (const SegDesc*)segs_.p;
    L.base = R.start;
    L.scale = R.scale;
    if (R.mode == PG_EVAL_SET_SUMS && terms_rows_ > 0) {
      L.pterms = (const double*)terms_[cur ^ 1].p;
      L.ppos = (const uint32_t*)ppos_[cur].p;
      L.terms = (double*)terms_[cur].p;
      L.terms_rows = terms_rows_;
      L.terms_n = terms_n_[cur];
      L.pterms_n = terms_n_[cur ^ 1];
      L.ppos_n = ppos_n_[cur];
      L.chk = (unsigned long long*)chk_.p;
    }
    PG_TRY(launch(L), "evaluation launch");
    stats.launches++;
    stats.eval_launches++;
    if (R.mode == PG_EVAL_SET_SUMS) stats.setsum_regions += R.n;
  }
  return PG_OK;
}

int Engine::run(std::vector<Job>& jobs, const EvalLauncher& launch, const RunPolicy& policy) {
  int rc;
  PG_TRY(cudaSetDevice(device), "cudaSetDevice");
  if ((rc = autotune()) != PG_OK) return rc;
  const uint32_t njobs = (uint32_t)jobs.size();
  if (njobs == 0) return PG_OK;
  int maxd = 2;
  bool use_cache = false;  // keep the bisected regions' per-axis terms for the set-sum kernel
  for (auto& J : jobs) {
    maxd = std::max(maxd, J.desc.d);
    use_cache |= job_eval_mode(J) == PG_EVAL_SET_SUMS;
  }
  {
    const char* env = std::getenv("PG_SETSUM_CACHE");
    if (env && env[0] == '0') use_cache = false;
  }
  const int term_rows = kTermValues * maxd + 1;  // the per-axis terms and the split axis
  // Pool capacity in regions: both region lists, owners, parents and the
  // per-region scratch of one iteration (with the kept terms: both lists'
  // terms and parent positions).
  const uint64_t bytes_per_region = 32ull * maxd + 53 + (use_cache ? 16ull * term_rows + 4 : 0);
  uint64_t cap = policy.max_regions;
  if (cap == 0) {
    size_t fr = 0, tot = 0;
    PG_TRY(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
    cap = (uint64_t)(0.6 * (double)fr) / bytes_per_region;
  }
  if (policy.budget_bytes) cap = std::min<uint64_t>(cap, policy.budget_bytes / bytes_per_region);
  cap = std::max<uint64_t>(cap, 4096);
  if (cap >= (1ull << 32)) use_cache = false;  // parent positions are 32-bit
  const uint64_t admit_limit = (uint64_t)(policy.admit_fraction * (double)cap);
  // Per-integral arrays.
  if ((rc = ensure(descs_, njobs * sizeof(IntegralDesc))) != PG_OK) return rc;
  if ((rc = ensure(segs_, njobs * sizeof(SegDesc))) != PG_OK) return rc;
  if ((rc = ensure(trans_, njobs * sizeof(Transition))) != PG_OK) return rc;
  if ((rc = ensure(scal_, njobs * sizeof(IterScalars))) != PG_OK) return rc;
  if ((rc = ensure(live_, (njobs + 1) * sizeof(uint64_t))) != PG_OK) return rc;
  if ((rc = ensure(adm_starts_, (njobs + 1) * sizeof(uint64_t))) != PG_OK) return rc;
  if ((rc = ensure(adm_ids_, (njobs + 1) * sizeof(uint32_t))) != PG_OK) return rc;
  if ((rc = ensure_pinned(h_segs_, njobs * sizeof(SegDesc))) != PG_OK) return rc;
  if ((rc = ensure_pinned(h_trans_, njobs * sizeof(Transition))) != PG_OK) return rc;
  if ((rc = ensure_pinned(h_trans_spill_, njobs * sizeof(Transition))) != PG_OK) return rc;
  if ((rc = ensure_pinned(h_scal_, njobs * sizeof(IterScalars))) != PG_OK) return rc;
  if ((rc = ensure_pinned(h_live_, (njobs + 1) * sizeof(uint64_t))) != PG_OK) return rc;
  if ((rc = ensure_pinned(h_adm_starts_, (njobs + 1) * sizeof(uint64_t))) != PG_OK) return rc;
  if ((rc = ensure_pinned(h_adm_ids_, (njobs + 1) * sizeof(uint32_t))) != PG_OK) return rc;
  {
    std::vector<IntegralDesc> descs(njobs);
    for (uint32_t j = 0; j < njobs; ++j) descs[j] = jobs[j].desc;
    PG_TRY(cudaMemcpyAsync(descs_.p, descs.data(), njobs * sizeof(IntegralDesc), cudaMemcpyHostToDevice, stream_),
           "desc upload");
    PG_TRY(cudaStreamSynchronize(stream_), "desc upload");
    stats.h2d_bytes += njobs * sizeof(IntegralDesc);
  }
  for (uint32_t j = 0; j < njobs; ++j) {
    Job& J = jobs[j];
    J.res = pg_result{};
    J.res.status = 1;
    J.res.last_phase = -1;
    J.cls = ClassifierState{};
    J.cls.epsrel = J.epsrel;
    J.cls.epsabs = J.epsabs;
    J.cls.required_digits = (int)std::ceil(std::log10(1 / J.epsrel));
    J.cls.ndim = J.desc.d;
    J.cls.total_mem = J.opt.device_mem_model > 0 ? J.opt.device_mem_model : 16e9;
    J.n = J.init_n ? J.init_n : ipow_u((uint64_t)parts_for(J.desc.d), J.desc.d);
    J.start = J.par_start = 0;
    J.has_parent = 0;
    J.has_cache = 0;
    J.iters = 0;
    J.done = false;
    J.state = JOB_PENDING;
    J.sp_batch = -1;
    J.sp_off = J.sp_poff = 0;
  }
  spill_.reset();
  PG_TRY(cudaMemsetAsync(chk_.p, 0, 64, stream_), "bounds record");
  terms_n_[0] = terms_n_[1] = ppos_n_[0] = ppos_n_[1] = 0;
  spill_batches_.clear();
  const auto t_start = std::chrono::steady_clock::now();
  // Host decision time: from the end of an iteration's readback to the next
  // evaluation launch (the device idles in between unless work is queued).
  bool decision_open = false;
  auto t_decision = t_start;
  int cur = 0;
  uint64_t T = 0, P = 0;  // regions and parent estimates in the current list
  uint32_t first_waiting = 0;
  std::vector<uint32_t> live;
  std::vector<ChunkRef> chunk_list;
  std::vector<int> mode(njobs);
  std::vector<uint64_t> keepA(njobs);
  std::vector<uint32_t> adm_pending;
  auto elapsed_ms = [&]() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
  };
  while (true) {
    if (policy.deadline_ms > 0 && elapsed_ms() > policy.deadline_ms) {
      for (uint32_t j = 0; j < njobs; ++j)
        if (jobs[j].state != JOB_DONE) {
          jobs[j].res.status = -1;  // not finished before the deadline
          jobs[j].done_ms = -1.0;
          jobs[j].state = JOB_DONE;
        }
      break;
    }
    // ---- admission: waiting integrals join at the end of the list, in order
    adm_pending.clear();
    const double now_admit = elapsed_ms();
    {
      uint64_t t = T, pp = P;
      uint64_t* hs = (uint64_t*)h_adm_starts_.p;
      uint32_t* hi = (uint32_t*)h_adm_ids_.p;
      std::vector<uint32_t> restore, custom;
      while (first_waiting < njobs && jobs[first_waiting].state == JOB_DONE) ++first_waiting;
      std::vector<uint32_t> admitted;
      for (uint32_t j = first_waiting; j < njobs; ++j) {
        Job& J = jobs[j];
        if (J.state != JOB_PENDING && J.state != JOB_SPILLED) continue;
        if (J.state == JOB_PENDING && policy.arrival_ms && policy.arrival_ms[j] > now_admit) break;  // not yet arrived
        if (t + J.n > admit_limit && t > 0) break;
        t += J.n;
        admitted.push_back(j);
      }
      // Placement of the admitted integrals: those evaluated by generator-set
      // sums first, then the others, so each evaluation kernel sees few runs.
      t = T;
      for (int pass = 0; pass < 2; ++pass)
        for (uint32_t j : admitted) {
          Job& J = jobs[j];
          if ((job_eval_mode(J) == PG_EVAL_SET_SUMS) != (pass == 0)) continue;
          J.start = t;
          J.par_start = pp;
          t += J.n;
          if (J.state == JOB_SPILLED) {
            pp += J.n / 2;
            restore.push_back(j);
          } else if (J.init_n) {
            custom.push_back(j);
          } else {
            hs[adm_pending.size()] = J.start;
            hi[adm_pending.size()] = j;
            adm_pending.push_back(j);
          }
          J.state = JOB_RESIDENT;
          J.has_cache = 0;
        }
      if (t > T) {
        if ((rc = grow_list(cur, t, maxd, T, P)) != PG_OK) return rc;
        if (profiling) {
          cudaEventRecord(ev_[8], stream_);
          admit_timing_pending_ = true;
        }
        if (!adm_pending.empty()) {
          const uint32_t m = (uint32_t)adm_pending.size();
          hs[m] = jobs[adm_pending.back()].start + jobs[adm_pending.back()].n;
          PG_TRY(cudaMemcpyAsync(adm_starts_.p, hs, (m + 1) * 8, cudaMemcpyHostToDevice, stream_), "admit upload");
          PG_TRY(cudaMemcpyAsync(adm_ids_.p, hi, m * 4, cudaMemcpyHostToDevice, stream_), "admit upload");
          const uint64_t span = hs[m] - hs[0];
          uniform_split_batch_kernel<<<(unsigned)div_up(span, 256), 256, 0, stream_>>>(
              (double*)left_[cur].p, (double*)len_[cur].p, reg_cap_[cur], (uint32_t*)owner_[cur].p,
              (const uint64_t*)adm_starts_.p, (const uint32_t*)adm_ids_.p, (const IntegralDesc*)descs_.p, m);
          stats.launches++;
          PG_TRY(cudaGetLastError(), "uniform split launch");
        }
        for (uint32_t j : custom) {  // caller-given first lists (pageable host memory: synchronous copies)
          Job& J = jobs[j];
          const int d = J.desc.d;
          PG_TRY(cudaMemcpy2DAsync((double*)left_[cur].p + J.start, reg_cap_[cur] * 8, J.init_left, J.n * 8, J.n * 8,
                                   d, cudaMemcpyHostToDevice, stream_), "initial regions");
          PG_TRY(cudaMemcpy2DAsync((double*)len_[cur].p + J.start, reg_cap_[cur] * 8, J.init_length, J.n * 8,
                                   J.n * 8, d, cudaMemcpyHostToDevice, stream_), "initial regions");
          fill_owner_kernel<<<(unsigned)div_up(J.n, 256), 256, 0, stream_>>>((uint32_t*)owner_[cur].p, J.start, J.n,
                                                                            j);
          stats.launches++;
          PG_TRY(cudaGetLastError(), "initial regions launch");
          stats.h2d_bytes += J.n * 16 * d;
        }
        // Restores: one kernel reads every restored integral's list straight
        // from its pinned slice (the table's host mirror is rewritten only
        // after the iteration's synchronisation, so its last upload is done).
        if (!restore.empty()) {
          if ((rc = ensure(rst_items_, restore.size() * sizeof(RestoreItem))) != PG_OK) return rc;
          if ((rc = ensure_pinned(h_rst_items_, restore.size() * sizeof(RestoreItem))) != PG_OK) return rc;
          RestoreItem* items = (RestoreItem*)h_rst_items_.p;
          uint64_t blocks = 0;
          for (size_t q = 0; q < restore.size(); ++q) {
            Job& J = jobs[restore[q]];
            SpillBatch& B = spill_batches_[J.sp_batch];
            RestoreItem& I = items[q];
            I.src_left = B.dp + J.sp_off;
            I.src_len = B.dp + (uint64_t)B.rows * B.stride + J.sp_off;
            I.src_par = B.dp + 2ull * B.rows * B.stride + J.sp_poff;
            I.src_stride = B.stride;
            I.start = J.start;
            I.par_start = J.par_start;
            I.n = J.n;
            I.block0 = blocks;
            I.owner = restore[q];
            I.d = J.desc.d;
            blocks += div_up(J.n, kRestoreRegions);
            stats.h2d_bytes += J.n * 16 * (uint64_t)J.desc.d + (J.n / 2) * 8;
          }
          PG_TRY(cudaMemcpyAsync(rst_items_.p, items, restore.size() * sizeof(RestoreItem), cudaMemcpyHostToDevice,
                                 stream_), "restore table");
          if (blocks > 0x7fffffffull) {
            last_error = "restore grid too large";
            return PG_BAD_ARG;
          }
          restore_kernel<<<(unsigned)blocks, 256, 0, stream_>>>((const RestoreItem*)rst_items_.p,
                                                                (uint32_t)restore.size(), (double*)left_[cur].p,
                                                                (double*)len_[cur].p, reg_cap_[cur],
                                                                (uint32_t*)owner_[cur].p, (double*)parent_[cur].p);
          stats.launches++;
          PG_TRY(cudaGetLastError(), "restore launch");
          // When a batch's last integral is back, its slice may be handed out
          // again at once: the next writer is a kernel queued behind this one
          // on the same stream.
          for (uint32_t j : restore) {
            Job& J = jobs[j];
            SpillBatch& B = spill_batches_[J.sp_batch];
            if (--B.live == 0) spill_.release(B.p, B.bytes);
            J.sp_batch = -1;
          }
        }
        if (profiling) cudaEventRecord(ev_[9], stream_);
        T = t;
        P = pp;
      }
    }
    live.clear();
    for (uint32_t j = 0; j < njobs; ++j)
      if (jobs[j].state == JOB_RESIDENT) live.push_back(j);
    if (live.empty()) {
      // Idle: wait for the next arrival, or stop when every job is done.
      uint32_t next = njobs;
      for (uint32_t j = first_waiting; j < njobs; ++j)
        if (jobs[j].state == JOB_PENDING || jobs[j].state == JOB_SPILLED) {
          next = j;
          break;
        }
      if (next == njobs) break;
      if (policy.arrival_ms && jobs[next].state == JOB_PENDING) {
        double wait = policy.arrival_ms[next] - elapsed_ms();
        if (policy.deadline_ms > 0) wait = std::min(wait, policy.deadline_ms - elapsed_ms() + 0.001);
        if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double, std::milli>(wait));
      }
      continue;
    }
    // Segments and chunk list of the resident integrals.
    chunk_list.clear();
    SegDesc* hs = (SegDesc*)h_segs_.p;
    for (uint32_t j = 0; j < njobs; ++j) {
      Job& J = jobs[j];
      SegDesc S;
      std::memset(&S, 0, sizeof S);
      const bool res = J.state == JOB_RESIDENT;
      S.start = J.start;
      S.n = res ? J.n : 0;
      S.par_start = J.par_start;
      S.chunk_start = (uint32_t)chunk_list.size();
      S.nchunks = (uint32_t)div_up(S.n, kChunk);
      S.has_parent = J.has_parent;
      S.has_cache = J.has_cache;
      // predict_split (Workspace.cuh:415-420): no rel-err classification while
      // the list is small, in the first 15 iterations, and nothing finished yet.
      S.relerr = J.opt.predict_split ? !(J.n <= 15000000ull && J.iters < 15 && J.res.nregions == 0)
                                     : J.opt.relerr_classification;
      S.epsrel = J.epsrel;
      if (res && S.has_parent && S.n > 0 && (S.n & 1ull) == 0 && job_eval_mode(J) == PG_EVAL_SET_SUMS) {
        stats.setsum_pairs += S.n / 2;  // the set-sum kernel's sibling pairing
        if (S.has_cache) stats.setsum_cached_pairs += S.n / 2;
      }
      for (uint32_t b = 0; b < S.nchunks; ++b) chunk_list.push_back(ChunkRef{j, b});
      hs[j] = S;
    }
    const uint64_t N = T;
    const uint64_t nchunks = chunk_list.size();
    if ((rc = ensure(est_, N * 8)) != PG_OK) return rc;
    if ((rc = ensure(err_a_, N * 8)) != PG_OK) return rc;
    if ((rc = ensure(err_b_, N * 8)) != PG_OK) return rc;
    if ((rc = ensure(bisect_, N * 4)) != PG_OK) return rc;
    if ((rc = ensure(active_, N)) != PG_OK) return rc;
    terms_rows_ = use_cache ? term_rows : 0;
    if (use_cache && (rc = ensure(terms_[cur], div_up(N, 32) * 256 * (uint64_t)term_rows)) != PG_OK) return rc;
    terms_n_[cur] = use_cache ? N : 0;
    if ((rc = ensure(partials_, nchunks * sizeof(Partial))) != PG_OK) return rc;
    if ((rc = ensure(chunk_off_, nchunks * 8)) != PG_OK) return rc;
    if ((rc = ensure(chunks_, nchunks * sizeof(ChunkRef))) != PG_OK) return rc;
    if ((rc = ensure_pinned(h_chunks_, nchunks * sizeof(ChunkRef))) != PG_OK) return rc;
    std::memcpy(h_chunks_.p, chunk_list.data(), nchunks * sizeof(ChunkRef));
    uint32_t* hl = (uint32_t*)h_live_.p;
    for (size_t q = 0; q < live.size(); ++q) hl[q] = live[q];
    PG_TRY(cudaMemcpyAsync(segs_.p, hs, njobs * sizeof(SegDesc), cudaMemcpyHostToDevice, stream_), "seg upload");
    PG_TRY(cudaMemcpyAsync(chunks_.p, h_chunks_.p, nchunks * sizeof(ChunkRef), cudaMemcpyHostToDevice, stream_),
           "chunk upload");
    PG_TRY(cudaMemcpyAsync(live_.p, hl, live.size() * 4, cudaMemcpyHostToDevice, stream_), "live upload");
    stats.h2d_bytes += njobs * sizeof(SegDesc) + nchunks * sizeof(ChunkRef) + live.size() * 4;
    // 1. evaluation
    if (decision_open) {
      stats.host_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_decision).count();
      decision_open = false;
    }
    if (profiling) cudaEventRecord(ev_[0], stream_);
    const uint64_t eval_launches0 = stats.eval_launches;
    if ((rc = evaluate_list(jobs, live, cur, N, launch)) != PG_OK) return rc;
    stats.regions_evaluated += N;
    for (uint32_t j : live) {
      const Job& J = jobs[j];
      const uint64_t d = (uint64_t)J.desc.d;
      stats.points_evaluated += J.n * (uint64_t)rule_.feval[J.desc.d];
      stats.eval_bytes += J.n * (16ull * d + 24ull);  // + the 4-byte owner of a shared list
      if (use_cache && job_eval_mode(J) == PG_EVAL_SET_SUMS) {
        stats.eval_bytes += J.n * (8ull * kTermValues * d + 8);  // the terms and split axes written
        if (J.has_cache) stats.eval_bytes += (J.n / 2) * (8ull * kTermValues * (d - 1) + 12ull);  // parents' read
      }
    }
    if (profiling) cudaEventRecord(ev_[1], stream_);
    // 2. two-level error + classification + partial sums; 3. per-integral totals
    two_level_kernel<<<(unsigned)nchunks, kRedThreads, 0, stream_>>>(
        (const ChunkRef*)chunks_.p, (const SegDesc*)segs_.p, (const double*)est_.p, (const double*)err_a_.p,
        (const double*)parent_[cur].p, (double*)err_b_.p, (uint8_t*)active_.p, (Partial*)partials_.p);
    finalize_kernel<<<(unsigned)live.size(), kRedThreads, 0, stream_>>>(
        (const uint32_t*)live_.p, (const SegDesc*)segs_.p, (const Partial*)partials_.p, (uint64_t*)chunk_off_.p,
        (IterScalars*)scal_.p);
    stats.launches += 2;
    PG_TRY(cudaGetLastError(), "two-level launch");
    if (profiling) cudaEventRecord(ev_[2], stream_);
    PG_TRY(cudaMemcpyAsync(h_scal_.p, scal_.p, njobs * sizeof(IterScalars), cudaMemcpyDeviceToHost, stream_),
           "scalar readback");
    {
      const auto w0 = std::chrono::steady_clock::now();
      PG_TRY(cudaMemcpyAsync(h_chk_.p, chk_.p, 64, cudaMemcpyDeviceToHost, stream_), "bounds record");
      PG_TRY(cudaStreamSynchronize(stream_), "iteration");
      if ((rc = check_bounds()) != PG_OK) return rc;
      t_decision = std::chrono::steady_clock::now();
      decision_open = true;
      stats.sync_ms += std::chrono::duration<double, std::milli>(t_decision - w0).count();
    }
    stats.d2h_bytes += njobs * sizeof(IterScalars);
    stats.stage_bytes += N * 29;
    if (profiling) {
      pg_iteration_record rec{N, (uint32_t)live.size(), (uint32_t)(stats.eval_launches - eval_launches0), 0.0, 0.0};
      record(ev_[0], ev_[1], &rec.eval_ms);
      record(ev_[1], ev_[2], &rec.stage_ms);
      stats.eval_ms += rec.eval_ms;
      stats.stage_ms += rec.stage_ms;
      iterations.push_back(rec);
      if (compact_timing_pending_) record(ev_[2 + 2], ev_[3 + 2], &stats.stage_ms);
      if (spill_timing_pending_) record(ev_[6], ev_[7], &stats.spill_ms);
      if (admit_timing_pending_) record(ev_[8], ev_[9], &stats.admit_ms);
      compact_timing_pending_ = spill_timing_pending_ = admit_timing_pending_ = false;
    }
    const IterScalars* sc = (const IterScalars*)h_scal_.p;
    // Host decisions, per integral, exactly as Workspace::integrate.
    for (uint32_t j : live) {
      Job& J = jobs[j];
      pg_result& cum = J.res;
      const IterScalars S = sc[j];
      const uint64_t n = J.n;
      cum.neval += n * (uint64_t)rule_.feval[J.desc.d];
      mode[j] = 0;
      keepA[j] = 0;
      const double iter_est = S.iter_est, iter_err = S.iter_err;
      const double cest = std::fabs(cum.estimate + iter_est), cerr = cum.errorest + iter_err;
      if (J.opt.predict_split && J.snap_n && J.iters == 15 && cum.nregions == 0) {
        // take_snapshot of the list evaluated in iteration 15 (Workspace.cuh:437-441)
        const int d = J.desc.d;
        J.snap_left->resize(n * d);
        J.snap_length->resize(n * d);
        PG_TRY(cudaMemcpy2DAsync(J.snap_left->data(), n * 8, (const double*)left_[cur].p + J.start, reg_cap_[cur] * 8,
                                 n * 8, d, cudaMemcpyDeviceToHost, stream_), "snapshot");
        PG_TRY(cudaMemcpy2DAsync(J.snap_length->data(), n * 8, (const double*)len_[cur].p + J.start,
                                 reg_cap_[cur] * 8, n * 8, d, cudaMemcpyDeviceToHost, stream_), "snapshot");
        PG_TRY(cudaStreamSynchronize(stream_), "snapshot");
        *J.snap_n = n;
        stats.d2h_bytes += n * 16 * d;
      }
      J.iters++;
      if (cerr / cest <= J.epsrel || cerr <= J.epsabs) {  // accuracy_reached (PaganiUtils.cuh:387-394)
        cum.estimate += iter_est;
        cum.errorest += iter_err;
        cum.status = 0;
        cum.nregions += n;
        J.done = true;
        continue;
      }
      J.cls.store(cum.estimate + iter_est);
      double fin_est = iter_est - S.act_est;
      double fin_err = iter_err - S.act_err;
      int m = 1;
      uint64_t A = S.active;
      // fix_error_budget_overflow (Workspace.cuh:121-146)
      if (cum.errorest + fin_err > std::fabs(cum.estimate + iter_est) * J.epsrel) {
        m = 2;
        A = n;
        fin_err = 0.;
        fin_est = 0.;
      }
      // heuristic_classify (Workspace.cuh:74-118)
      bool must_terminate;
      {
        const double ratio = (double)J.cls.mem_required(n) / (double)J.cls.free_mem(n);
        const bool necessary = ratio > 1.;
        if (!J.cls.criteria_met(n)) {
          must_terminate = necessary;
        } else {
          bool ok = false;
          uint64_t na = 0;
          double fe = fin_est, fr = fin_err;
          if ((rc = classify_job(J, j, iter_err, fin_err, &ok, &fe, &fr, &na, iter_est)) != PG_OK) return rc;
          if (ok) {
            m = 1;
            A = na;
            fin_est = fe;
            fin_err = fr;
          }
          must_terminate = (!ok && necessary) || na == 0;
        }
      }
      if (must_terminate) {
        cum.estimate += iter_est;
        cum.errorest += iter_err;
        cum.nregions += n;
        J.done = true;
        continue;
      }
      cum.estimate += fin_est;
      cum.errorest += fin_err;
      cum.nregions += n - A;
      cum.nfinished += n - A;
      cum.iters++;
      if (A == 0) {
        J.done = true;
        continue;
      }
      if (J.iters >= J.opt.max_iters) {  // loop cap: the split list is counted, never evaluated
        cum.nregions += 2 * A;
        J.done = true;
        continue;
      }
      mode[j] = m;
      keepA[j] = A;
    }
    const double now_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    for (uint32_t j : live)
      if (jobs[j].done) {
        jobs[j].state = JOB_DONE;
        jobs[j].done_ms = now_ms;
      }
    // ---- placement of the next list: in order, while the pool has room;
    // the rest leave the pool with their next list in host memory.
    // Integrals evaluated by generator-set sums are placed first, then the
    // others, so each evaluation kernel sees few runs of the list.
    Transition* ht = (Transition*)h_trans_.p;
    uint64_t out_total = 0, par_total = 0;
    std::vector<uint32_t> spill;
    std::memset(ht, 0, njobs * sizeof(Transition));
    for (int pass = 0; pass < 2; ++pass)
      for (uint32_t j = 0; j < njobs; ++j) {
        Job& J = jobs[j];
        if (J.state != JOB_RESIDENT || mode[j] == 0) continue;
        if ((job_eval_mode(J) == PG_EVAL_SET_SUMS) != (pass == 0)) continue;
        Transition& Tr = ht[j];
        Tr.mode = mode[j];
        Tr.A = keepA[j];
        Tr.cache = use_cache && job_eval_mode(J) == PG_EVAL_SET_SUMS;
        if (out_total + 2 * keepA[j] <= cap || out_total == 0) {
          Tr.out_start = out_total;
          Tr.par_out = par_total;
          out_total += 2 * keepA[j];
          par_total += keepA[j];
        } else {
          spill.push_back(j);
        }
      }
    // Spill groups are formed in integral order (their chunks are contiguous).
    std::sort(spill.begin(), spill.end());
    // Spilled integrals, in groups of at most one pool's worth of regions:
    // the children of a group go to a transient device buffer in one
    // compaction (integral j at its own offset, rows `stride` apart) and from
    // there in three copies to one pinned slice (a spill batch); every spilled
    // integral is then excluded (mode 0) from the compaction of the resident
    // list.  The two transition tables are separate pinned arrays that the
    // host does not touch again before the end-of-iteration synchronisation,
    // so no copy here needs a host wait.
    Transition* hsp = (Transition*)h_trans_spill_.p;
    if (!spill.empty()) {
      if (profiling) {
        cudaEventRecord(ev_[6], stream_);
        spill_timing_pending_ = true;
      }
      // groups [gbeg[g], gbeg[g+1]) of the spill list, with their region and parent totals
      std::vector<size_t> gbeg{0};
      std::vector<uint64_t> gsst, gspt;
      uint64_t sst = 0, spt = 0;
      std::memcpy(hsp, ht, njobs * sizeof(Transition));
      for (uint32_t j = 0; j < njobs; ++j) hsp[j].mode = 0;
      for (size_t q = 0; q < spill.size(); ++q) {
        const uint32_t j = spill[q];
        const uint64_t n2 = 2 * keepA[j];
        if (sst > 0 && sst + n2 > cap) {  // close the group
          gsst.push_back(sst);
          gspt.push_back(spt);
          gbeg.push_back(q);
          sst = spt = 0;
        }
        hsp[j] = ht[j];
        hsp[j].out_start = sst;
        hsp[j].par_out = spt;
        jobs[j].sp_off = sst;
        jobs[j].sp_poff = spt;
        sst += n2;
        spt += keepA[j];
        ht[j].mode = 0;
      }
      gsst.push_back(sst);
      gspt.push_back(spt);
      gbeg.push_back(spill.size());
      PG_TRY(cudaMemcpyAsync(trans_.p, hsp, njobs * sizeof(Transition), cudaMemcpyHostToDevice, stream_),
             "transition upload");
      stats.h2d_bytes += njobs * sizeof(Transition);
      for (size_t g = 0; g + 1 < gbeg.size(); ++g) {
        const uint32_t jf = spill[gbeg[g]], jl = spill[gbeg[g + 1] - 1];
        const uint32_t c0 = hs[jf].chunk_start, c1 = hs[jl].chunk_start + hs[jl].nchunks;
        const uint64_t st = gsst[g], pt = gspt[g];
        // The group's children and parents go straight into a pinned slice:
        // the compaction writes host memory over NVLink-C2C.
        SpillBatch B;
        B.bytes = (2 * st * (uint64_t)maxd + pt) * 8;
        B.p = (double*)spill_.alloc(B.bytes);
        B.rows = maxd;
        B.stride = st;
        B.live = (int)(gbeg[g + 1] - gbeg[g]);
        if (!B.p) {
          last_error = "pinned host memory for spilled region lists";
          return PG_OOM;
        }
        void* dp = nullptr;
        PG_TRY(cudaHostGetDevicePointer(&dp, B.p, 0), "device address of a pinned slice");
        B.dp = (double*)dp;
        if ((rc = compact(cur, cur ^ 1, c0, c1 - c0, maxd, B.dp, B.dp + st * maxd, st, nullptr,
                          B.dp + 2 * st * maxd)) != PG_OK)
          return rc;
        stats.d2h_bytes += st * maxd * 16 + pt * 8;
        const int bidx = (int)spill_batches_.size();
        spill_batches_.push_back(B);
        for (size_t q = gbeg[g]; q < gbeg[g + 1]; ++q) {
          Job& J = jobs[spill[q]];
          J.sp_batch = bidx;
          J.state = JOB_SPILLED;
          J.n = 2 * keepA[spill[q]];
          J.has_parent = 1;
          J.has_cache = 0;
        }
      }
      PG_TRY(cudaMemcpyAsync(trans_.p, ht, njobs * sizeof(Transition), cudaMemcpyHostToDevice, stream_),
             "transition upload");
      stats.h2d_bytes += njobs * sizeof(Transition);
      if (profiling) cudaEventRecord(ev_[7], stream_);
    } else {
      PG_TRY(cudaMemcpyAsync(trans_.p, ht, njobs * sizeof(Transition), cudaMemcpyHostToDevice, stream_),
             "transition upload");
      stats.h2d_bytes += njobs * sizeof(Transition);
    }
    const int nxt = cur ^ 1;
    if (out_total > 0) {
      if ((rc = grow_list(nxt, out_total, maxd, 0, 0)) != PG_OK) return rc;
      // This iteration's evaluation has read the parents' terms; the cache now
      // takes the terms of the regions being bisected.
      if (use_cache && (rc = ensure(ppos_[nxt], par_total * 4)) != PG_OK) return rc;
      ppos_n_[nxt] = use_cache ? par_total : 0;
      if (profiling) cudaEventRecord(ev_[4], stream_);
      if ((rc = compact(cur, nxt, 0, (uint32_t)nchunks, maxd, (double*)left_[nxt].p, (double*)len_[nxt].p,
                        reg_cap_[nxt], (uint32_t*)owner_[nxt].p, (double*)parent_[nxt].p,
                        use_cache ? (uint32_t*)ppos_[nxt].p : nullptr, ppos_n_[nxt])) != PG_OK)
        return rc;
      if (profiling) {
        cudaEventRecord(ev_[5], stream_);
        compact_timing_pending_ = true;  // read after the next synchronisation
      }
    }
    for (uint32_t j = 0; j < njobs; ++j) {
      const Transition& Tr = ht[j];
      Job& J = jobs[j];
      if (J.state != JOB_RESIDENT || Tr.mode == 0) continue;
      stats.stage_bytes += J.n + Tr.A * (uint64_t)(16 * J.desc.d + 12) + 2 * Tr.A * (uint64_t)(16 * J.desc.d + 4) +
                           Tr.A * 8;
      if (Tr.cache) stats.stage_bytes += Tr.A * 4;  // the parents' positions
      J.start = Tr.out_start;
      J.n = 2 * Tr.A;
      J.par_start = Tr.par_out;
      J.has_parent = 1;
      J.has_cache = Tr.cache;
    }
    T = out_total;
    P = par_total;
    cur = nxt;
  }
  PG_TRY(cudaMemcpyAsync(h_chk_.p, chk_.p, 64, cudaMemcpyDeviceToHost, stream_), "bounds record");
  PG_TRY(cudaStreamSynchronize(stream_), "run");
  if ((rc = check_bounds()) != PG_OK) return rc;
  if (profiling && compact_timing_pending_) record(ev_[4], ev_[5], &stats.stage_ms);
  if (profiling && spill_timing_pending_) record(ev_[6], ev_[7], &stats.spill_ms);
  if (profiling && admit_timing_pending_) record(ev_[8], ev_[9], &stats.admit_ms);
  compact_timing_pending_ = spill_timing_pending_ = admit_timing_pending_ = false;
  return PG_OK;
}

int Engine::autotune() {
  const EvalLauncher launch = launch_family_eval;
  if (tuned) return PG_OK;
  const char* env = std::getenv("PG_AUTOTUNE");
  tuned = true;
  if (env && env[0] == '0') return PG_OK;
  // One synthetic list per kernel class: 8-D and 10-D Gaussians on 24576
  // regions of mixed sizes (the work of one region does not depend on its
  // size, so the list only has to fill the GPU several times over).
  const int dims[2] = {8, 10};
  const int warps_c[2] = {4, 8};
  const int ctas_c[3] = {8, 16, 32};
  const uint64_t n = 24576;
  int rc;
  for (int cls = 0; cls < 2; ++cls) {
    const int d = dims[cls];
    std::vector<double> left((size_t)d * n), len((size_t)d * n);
    uint64_t state = 0x9E3779B97F4A7C15ull * (cls + 1);
    for (size_t i = 0; i < left.size(); ++i) {
      state = state * 6364136223846793005ull + 1442695040888963407ull;
      const int depth = (int)((state >> 33) % 6);
      const double h = std::ldexp(1.0, -depth);
      const uint64_t cells = 1ull << depth;
      len[i] = h;
      left[i] = (double)((state >> 20) % cells) * h;
    }
    DevBuf dl, dn, de, dr, db;
    if ((rc = ensure(dl, left.size() * 8)) != PG_OK || (rc = ensure(dn, len.size() * 8)) != PG_OK ||
        (rc = ensure(de, n * 8)) != PG_OK || (rc = ensure(dr, n * 8)) != PG_OK || (rc = ensure(db, n * 4)) != PG_OK)
      return rc;
    pg_integrand f;
    std::memset(&f, 0, sizeof f);
    f.family = FAM_GAUSSIAN;
    f.ndim = d;
    for (int k = 0; k < d; ++k) {
      f.a[k] = 3.0 + 0.25 * k;
      f.u[k] = 0.5;
    }
    IntegralDesc D;
    prepare_desc(f, nullptr, nullptr, &D, nullptr);
    PG_TRY(cudaMemcpyAsync(dl.p, left.data(), left.size() * 8, cudaMemcpyHostToDevice, stream_), "tune upload");
    PG_TRY(cudaMemcpyAsync(dn.p, len.data(), len.size() * 8, cudaMemcpyHostToDevice, stream_), "tune upload");
    if ((rc = ensure(descs_, sizeof(IntegralDesc))) != PG_OK) return rc;
    PG_TRY(cudaMemcpyAsync(descs_.p, &D, sizeof D, cudaMemcpyHostToDevice, stream_), "tune upload");
    EvalTune best;
    best.ms = 1e30;
    for (int w : warps_c)
      for (int c : ctas_c) {
        EvalLaunch L{(const double*)dl.p, (const double*)dn.p, n, n, nullptr, (const IntegralDesc*)descs_.p, &rule_,
                     (double*)de.p, (double*)dr.p, (int32_t*)db.p, d, num_sms, stream_, w, c};
        PG_TRY(launch(L), "tune launch");  // warm-up
        PG_TRY(cudaEventRecord(ev_[0], stream_), "tune event");
        for (int rep = 0; rep < 2; ++rep) PG_TRY(launch(L), "tune launch");
        PG_TRY(cudaEventRecord(ev_[1], stream_), "tune event");
        PG_TRY(cudaEventSynchronize(ev_[1]), "tune");
        float ms = 0;
        cudaEventElapsedTime(&ms, ev_[0], ev_[1]);
        stats.launches += 3;
        if (ms < best.ms) {
          best.ms = ms;
          best.warps = w;
          best.ctas_per_sm = c;
        }
      }
    tune[cls] = best;
    DevBuf* bufs[] = {&dl, &dn, &de, &dr, &db};
    for (DevBuf* b : bufs) cudaFree(b->p);
  }
  return PG_OK;
}

// ---------------------------------------------------------------------------
// Evaluation launcher for the C ABI families.
// ---------------------------------------------------------------------------
cudaError_t launch_family_eval(const EvalLaunch& L) {
  const pg_eval_args a = eval_args_of(L);
  if (L.mode == PG_EVAL_SET_SUMS) {
    SetSumCache c;
    c.pterms = L.pterms;
    c.ppos = L.ppos;
    c.terms = L.terms;
    c.terms_rows = L.terms_rows;
    c.terms_n = L.terms_n;
    c.pterms_n = L.pterms_n;
    c.ppos_n = L.ppos_n;
    c.chk = L.chk;
    c.scale = L.scale;
    return launch_setsum(a, L.segs, L.base, c);
  }
  return L.maxd <= 8 ? launch_eval<8>(a, FamilyFn{}) : launch_eval<16>(a, FamilyFn{});
}

}  // namespace pg
