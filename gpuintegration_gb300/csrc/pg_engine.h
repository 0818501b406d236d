// Host engine of the GB300 PAGANI iteration.
//
// One engine runs any number of integrals together (a batch of one is the
// plain per-call path).  Each integral follows exactly the reference's
// Workspace::integrate loop (cuda/pagani/quad/GPUquad/Workspace.cuh:361-494);
// the integrals only share the device region list and the kernel launches, so
// an integral's result is bit-identical whether it runs alone or in a batch.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <map>
#include <string>
#include <vector>

#include "../../include/pagani_gb300.h"
#include "pg_kernels.cuh"
#include "pg_rule.h"

namespace pg {

// Arguments of one evaluation launch.
struct EvalLaunch {
  const double* left;
  const double* length;
  uint64_t n;
  uint64_t stride;
  const uint32_t* owner;
  const IntegralDesc* descs;
  const RuleDev* rule;
  double* est;
  double* err;
  int32_t* bisect;
  int maxd;
  int num_sms;
  cudaStream_t stream;
  int warps;        // regions per block (warps per CTA)
  int ctas_per_sm;  // grid cap of the grid-stride evaluation loop
  int mode = 0;     // 0: point-by-point rule sums (eval_kernel); 1: generator-set sums (setsum_kernel)
  // Set-sum kernel only: the integrals' segments of the list (siblings are
  // evaluated together; null: every region alone) and the list position of
  // left[0].
  const SegDesc* segs = nullptr;
  uint64_t base = 0;
  // Set-sum kernel only: the parents' kept terms and this list's terms
  // (null: none kept / none written).
  const double* pterms = nullptr;
  const uint32_t* ppos = nullptr;
  double* terms = nullptr;
  int terms_rows = 0;
  uint64_t terms_n = 0, pterms_n = 0, ppos_n = 0;
  unsigned long long* chk = nullptr;
  bool scale = true;  // some integral of the launch has a Jacobian other than 1
};

// Launch shape of the evaluation kernel for one kernel class (d <= 8, d > 8),
// chosen by Engine::autotune.
struct EvalTune {
  int warps = 8;
  int ctas_per_sm = 32;
  double ms = 0;  // time of the tuning launch with this shape
};

// Launches the evaluation kernel for some integrand functor type.
using EvalLauncher = std::function<cudaError_t(const EvalLaunch&)>;

// The same launch as the C ABI's plain argument block.
inline pg_eval_args eval_args_of(const EvalLaunch& L) {
  pg_eval_args a;
  a.left = L.left;
  a.length = L.length;
  a.n = L.n;
  a.stride = L.stride;
  a.owner = L.owner;
  a.descs = L.descs;
  a.rule = L.rule;
  a.est = L.est;
  a.err = L.err;
  a.bisect = L.bisect;
  a.maxd = L.maxd;
  a.num_sms = L.num_sms;
  a.stream = (void*)L.stream;
  a.warps = L.warps;
  a.ctas_per_sm = L.ctas_per_sm;
  return a;
}

// The launcher of the C ABI families.
cudaError_t launch_family_eval(const EvalLaunch& L);

// Host mirror of the memory-pressure classifier's state
// (heuristic_classifier.cuh:147-225).
struct ClassifierState {
  double epsrel = 0, epsabs = 0;
  int required_digits = 0;
  double last[3] = {0, 0, 0};
  uint64_t iters_collected = 0;
  double max_percent_error_budget = .25;
  double max_active_regions_percentage = .5;
  double total_mem = 16e9;
  int ndim = 0;

  uint64_t mem_required(uint64_t n) const;
  uint64_t free_mem(uint64_t n) const;
  bool sig_digits_same() const;
  bool estimate_converged() const;
  void store(double e);
  bool criteria_met(uint64_t n) const;
};

enum JobState { JOB_PENDING = 0, JOB_RESIDENT = 1, JOB_SPILLED = 2, JOB_DONE = 3 };

struct Job {
  IntegralDesc desc{};
  double epsrel = 1e-3, epsabs = 1e-12;
  pg_options opt{};
  ClassifierState cls;
  pg_result res{};
  uint64_t n = 0;      // regions in the current list
  uint64_t start = 0;  // first region in the current list
  uint64_t par_start = 0;
  int has_parent = 0;
  int has_cache = 0;  // its parents' per-axis terms are in the previous list's term buffer
  int iters = 0;
  bool done = false;
  int error = 0;
  int state = JOB_PENDING;
  double done_ms = 0.0;  // host time from the start of the run to the iteration that finished it
  // Next region list of a job moved out of the device pool: its place in a
  // spill batch (pinned slice holding the lists of every integral spilled in
  // one iteration: left rows [row][stride], length rows, parent estimates).
  int sp_batch = -1;
  uint64_t sp_off = 0;   // first region of the job within each row
  uint64_t sp_poff = 0;  // first parent estimate of the job
  // Caller-given initial region list (host, SoA [dim * init_n + i]); 0
  // regions: the uniform split (Workspace.cuh:379-387).
  const double* init_left = nullptr;
  const double* init_length = nullptr;
  uint64_t init_n = 0;
  // With opt.predict_split: receives the region list of iteration 15
  // (Workspace.cuh:437-441), SoA [dim * n + i].
  std::vector<double>* snap_left = nullptr;
  std::vector<double>* snap_length = nullptr;
  uint64_t* snap_n = nullptr;
};

// Pinned host storage for region lists moved out of the device pool.  Blocks
// of page-locked memory are allocated as needed and kept for the engine's
// lifetime; slices are handed out first-fit.  Every access to a slice is a
// copy on the engine's stream, so reusing a slice needs no host
// synchronisation.
class SpillArena {
 public:
  ~SpillArena();
  // A slice of at least `bytes` (256-byte aligned), or nullptr when pinned
  // memory cannot be had.
  void* alloc(size_t bytes);
  void release(void* p, size_t bytes);
  // Marks every block free (no job of a finished run still holds a slice).
  void reset();
  size_t pinned_bytes() const { return total_; }

 private:
  struct Block {
    char* base;
    size_t bytes;
    std::map<size_t, size_t> free;  // offset -> length
  };
  std::vector<Block> blocks_;
  size_t total_ = 0;
};

// Scheduling limits of one run.
struct RunPolicy {
  uint64_t max_regions = 0;   // pool capacity in regions (0: from free device memory)
  double admit_fraction = 0.5;  // new work is admitted while the list is below this share of the pool
  uint64_t budget_bytes = 0;  // device bytes the pool may use (0: no byte budget); caps max_regions
  // Serving: job j may not be admitted before arrival_ms[j] (ascending), in
  // milliseconds from the start of the run; nullptr admits every job at once.
  const double* arrival_ms = nullptr;
  // Serving: stop at the first iteration boundary after this many milliseconds
  // (0: run to completion); unfinished jobs keep status -1 and done_ms -1.
  double deadline_ms = 0;
};

// Evaluation kernel of a job: the generator-set sums when the options ask for
// them and the integrand is a product of per-axis factors, else point by point.
inline int job_eval_mode(const Job& J) {
  return (J.opt.eval_mode == PG_EVAL_SET_SUMS && family_separable(J.desc.family)) ? PG_EVAL_SET_SUMS
                                                                                   : PG_EVAL_POINTS;
}

// Prepares an IntegralDesc from the C ABI description (host, no contraction).
int prepare_desc(const pg_integrand& f, const double* lows, const double* highs, IntegralDesc* out, std::string* why);

// Descriptor of a caller's functor integrand: the integration box only.
int prepare_user_desc(int ndim, const double* lows, const double* highs, IntegralDesc* out, std::string* why);

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

class Engine {
 public:
  explicit Engine(int device);
  ~Engine();
  int init(std::string* why);

  // Runs every job to completion.  Returns PG_OK or a negative pg_status.
  int run(std::vector<Job>& jobs, const EvalLauncher& launch, const RunPolicy& policy = RunPolicy());

  // Evaluates caller-given regions (device pointers, SoA stride n).
  int evaluate(const IntegralDesc& desc, uint64_t n, const double* d_left, const double* d_length, uint64_t stride,
               double* d_est, double* d_err, int32_t* d_bisect, const EvalLauncher& launch, int mode = 0);

  // Times the candidate launch shapes of the evaluation kernel on a synthetic
  // region list per kernel class and keeps the fastest (once per context).
  // Always with the library's own families: a caller's functor is never run
  // outside its integration box.
  int autotune();
  EvalTune tune[2];
  bool tuned = false;

  cudaStream_t stream() const { return stream_; }
  const RuleDev& rule() const { return rule_; }
  pg_stats stats{};
  std::vector<pg_iteration_record> iterations;  // while profiling
  bool profiling = false;
  std::string last_error;
  // Allocation-failure hook (pg_context_fail_allocation): the allocation after
  // this many more fails as an out-of-memory cudaMalloc would; -1: off.
  int64_t fail_alloc_after = -1;
  int device = 0;
  int num_sms = 152;

  // Device scratch helpers (grow-only).
  int ensure(DevBuf& b, size_t bytes);
  int ensure_pinned(DevBuf& b, size_t bytes);

 private:
  int fail(cudaError_t e, const char* what);
  int classify_job(Job& J, uint32_t jidx, double iter_err, double fin_err, bool* ok, double* fin_est_out,
                   double* fin_err_out, uint64_t* num_active, double iter_est);
  int threshold_pass(uint32_t jidx, double thr, int write_flags, int minmax, int scan, double out[5],
                     bool readback = true);
  int classify_chain(uint32_t jidx, double thr0, double pct, uint64_t n);
  // Counts of integral jidx's errors above each of the k thresholds (one pass).
  int threshold_counts(uint32_t jidx, const double* thr, int k, uint64_t* counts);
  int grow_list(int which, uint64_t need, int rows, uint64_t live, uint64_t live_par);
  int compact(int cur, int nxt, uint32_t chunk0, uint32_t nchunks, int maxd, double* out_left, double* out_len,
              uint64_t out_stride, uint32_t* out_owner, double* parent_out, uint32_t* ppos_out = nullptr,
              uint64_t ppos_n = 0);
  int check_bounds();
  // Launches the evaluation of list `cur`'s regions [0, N): one launch per
  // maximal range of resident integrals that share an evaluation kernel.
  int evaluate_list(std::vector<Job>& jobs, const std::vector<uint32_t>& live, int cur, uint64_t N,
                    const EvalLauncher& launch);
  void record(cudaEvent_t a, cudaEvent_t b, double* acc);

  cudaStream_t stream_ = nullptr;
  RuleDev rule_{};
  DevBuf rule_code_, rule_w_, rule_scale_, rule_norm_, rule_trie_, rule_leafset_;
  // region lists (ping-pong) and owners
  DevBuf left_[2], len_[2], owner_[2], parent_[2];
  uint64_t reg_cap_[2] = {0, 0};
  int reg_rows_[2] = {0, 0};
  // per-region scratch
  DevBuf est_, err_a_, err_b_, bisect_, active_;
  // set-sum evaluation: each list's per-axis terms and split axes (tiles of
  // terms_rows_ rows by list position), and per list the positions of its
  // parents in the other list (by parent index)
  DevBuf terms_[2], ppos_[2];
  int terms_rows_ = 0;
  uint64_t terms_n_[2] = {0, 0}, ppos_n_[2] = {0, 0};  // positions with terms, parents with positions
  DevBuf chk_, h_chk_;                                // bounds record of the term lookups
  // per-chunk
  DevBuf partials_, chunk_off_, chunks_;
  // per-integral
  DevBuf segs_, trans_, descs_, scal_, live_, thr_out_, thr_counts_, adm_starts_, adm_ids_;
  // The classifier's chained first passes: [0..4] min/max pass, [8..12] pass
  // at the chosen threshold, [16..35] counts (u64), [40..59] the threshold
  // sequence, [60] the chosen threshold; and the device-built threshold set.
  DevBuf chain_, h_chain_, chain_ts_;
  // restore table of one admission (device, and its pinned host mirror)
  DevBuf rst_items_, h_rst_items_;
  SpillArena spill_;
  // Spill batches of the current run: slice, its size, rows and row stride
  // (regions) of its region block, and the number of integrals still in it.
  struct SpillBatch {
    double* p;
    double* dp;  // the same slice as the device addresses it
    size_t bytes;
    int rows;
    uint64_t stride;
    int live;
  };
  std::vector<SpillBatch> spill_batches_;
  bool compact_timing_pending_ = false;
  // pinned host mirrors
  DevBuf h_segs_, h_chunks_, h_trans_, h_trans_spill_, h_scal_, h_live_, h_thr_, h_thr_counts_, h_adm_starts_,
      h_adm_ids_;
  // 0-1 evaluation, 1-2 stages, 4-5 compaction, 6-7 spills, 8-9 admission and restores
  cudaEvent_t ev_[10] = {};
  bool spill_timing_pending_ = false, admit_timing_pending_ = false;
};

}  // namespace pg
