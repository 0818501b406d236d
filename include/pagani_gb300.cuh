/*
 * pagani_gb300.cuh -- C++ layer of the GB300 PAGANI library for callers
 * compiled with nvcc: the reference's class templates, with user functors,
 * over the C ABI of pagani_gb300.h.
 *
 *   Workspace<T, ndim>::integrate(f, epsrel, epsabs, vol, relerr_classification)
 *                                   cuda/pagani/quad/GPUquad/Workspace.cuh:23-70
 *   quad::Volume<T, NDIM>           common/cuda/Volume.cuh:9-52
 *   numint::integration_result      common/integration_result.hh:11-21
 *   cuda_mcubes::integrate<F, NDIM>(f, epsrel, epsabs, ncall, &vol, totalIters, adjustIters, skipIters)
 *   cuda_mcubes::simple_integrate, cuda_mcubes::mcubes
 *                                   cuda/mcubes/vegasT.cuh:999-1111
 *   quad::mcubes                    cuda/mcubes/mcubes.cuh:9-41
 *
 * An integrand is any copyable type with a __device__ operator() taking ndim
 * doubles and returning a double (the reference calls it through gpu::apply,
 * common/cuda/cudaApply.cuh:7-26).  The region-evaluation kernel is
 * instantiated for it in the caller's translation unit and handed to the
 * library as a launcher (pg_integrate_launcher); the library runs the rest of
 * the iteration.  The functor reaches the kernel as a copy: by value when it is
 * trivially copyable and small, otherwise copy-constructed into managed memory
 * for the duration of the call, as the reference does
 * (common/cuda/cudaMemoryUtil.h:181-196).
 *
 * Build: nvcc -std=c++17 -gencode arch=compute_103a,code=sm_103a -cudart shared
 *        -I<repo>/include app.cu -L<repo>/gpuintegration_gb300 -lpagani_gb300
 *
 * ::Workspace, cuda_mcubes:: and quad::mcubes are declared as aliases of the
 * pagani:: implementations unless PAGANI_GB300_NO_REFERENCE_NAMES is defined
 * before inclusion (do not include the reference's Workspace.cuh or
 * vegasT.cuh with this header: they are what it replaces).
 */
#ifndef PAGANI_GB300_CUH
#define PAGANI_GB300_CUH

#include <cuda_runtime.h>

#include <array>
#include <cstddef>
#include <cstring>
#include <new>
#include <ostream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "pagani_gb300.h"
#include "../gpuintegration_gb300/csrc/pg_eval.cuh"
#include "../gpuintegration_gb300/csrc/pg_mcubes_kernel.cuh"

// numint::integration_result (common/integration_result.hh:11-21) and
// quad::Volume (common/cuda/Volume.cuh:9-52) are declared under the
// reference headers' own include guards, with the same members, so that the
// reference's integrand-side headers (Interp1D/2D/3D, cudaArray, ...), which
// include them, can be used inside functors together with this header, in
// either include order.
#ifndef GPUINTEGRATION_COMMON_INTEGRATION_RESULT_H
#define GPUINTEGRATION_COMMON_INTEGRATION_RESULT_H
namespace numint {
// neval is filled here (regions evaluated x points per region).
struct integration_result {
  double estimate = 0.;
  double errorest = 0.;
  size_t neval = 0;
  size_t nregions = 0;
  size_t nFinishedRegions = 0;
  int status = -1;
  int lastPhase = -1;
  double chi_sq = 0.;
  size_t iters = 0;
};

inline std::ostream& operator<<(std::ostream& os, integration_result const& res) {
  os << res.estimate << "," << res.errorest << "," << res.nregions << "," << res.chi_sq << "," << res.status;
  return os;
}
}  // namespace numint
#endif

#ifndef CUDACUHRE_QUAD_GPUQUAD_VOLUME_CUH
#define CUDACUHRE_QUAD_GPUQUAD_VOLUME_CUH
namespace quad {
// The integration box.
template <typename T, int NDIM>
struct Volume {
  T lows[NDIM] = {0.0};
  T highs[NDIM];

  __host__ Volume() {
    for (T& x : highs) x = 1.0;
  }
  __host__ Volume(std::array<T, NDIM> l, std::array<T, NDIM> h) {
    std::memcpy(lows, l.data(), NDIM * sizeof(T));
    std::memcpy(highs, h.data(), NDIM * sizeof(T));
  }
  __host__ __device__ Volume(T const* l, T const* h) {
    for (int i = 0; i < NDIM; ++i) {
      lows[i] = l[i];
      highs[i] = h[i];
    }
  }
  __host__ Volume(T l, T h) {
    for (int i = 0; i < NDIM; ++i) {
      lows[i] = l;
      highs[i] = h;
    }
  }
};
}  // namespace quad
#endif

namespace pagani {

using integration_result = numint::integration_result;
template <typename T, int NDIM>
using Volume = quad::Volume<T, NDIM>;

namespace detail {

// Largest functor passed to the kernel by value (the rest go through managed memory).
constexpr size_t kByValueMax = 2048;

template <class F>
constexpr bool by_value() {
  return std::is_trivially_copyable<F>::value && sizeof(F) <= kByValueMax;
}

// The evaluation kernel's integrand interface for a caller's functor: not a
// product of per-axis factors, evaluated point by point on the ND coordinates.
template <class F, size_t ND, bool BYVAL = by_value<F>()>
struct UserFn;

template <class F, size_t ND>
struct UserFn<F, ND, true> {
  mutable F f;
  template <size_t... I>
  __device__ __forceinline__ double call(const double* x, std::index_sequence<I...>) const {
    return static_cast<double>(f(x[I]...));
  }
  template <int MAXD>
  __device__ __forceinline__ double eval(const pg::IntegralDesc&, const double* x) const {
    return call(x, std::make_index_sequence<ND>{});
  }
  __device__ __forceinline__ bool separable(const pg::IntegralDesc&) const { return false; }
  __device__ __forceinline__ double factor(const pg::IntegralDesc&, int, double) const { return 1.0; }
};

template <class F, size_t ND>
struct UserFn<F, ND, false> {
  F* f;  // copy in managed memory
  template <size_t... I>
  __device__ __forceinline__ double call(const double* x, std::index_sequence<I...>) const {
    return static_cast<double>((*f)(x[I]...));
  }
  template <int MAXD>
  __device__ __forceinline__ double eval(const pg::IntegralDesc&, const double* x) const {
    return call(x, std::make_index_sequence<ND>{});
  }
  __device__ __forceinline__ bool separable(const pg::IntegralDesc&) const { return false; }
  __device__ __forceinline__ double factor(const pg::IntegralDesc&, int, double) const { return 1.0; }
};

// C-ABI launcher: instantiates the evaluation kernel for the functor (kernel
// class d <= 8 or d <= 16, the same classes as the library's families).
template <class Fn, size_t ND>
int launch_user(const pg_eval_args* a, void* user) {
  constexpr int MAXD = ND <= 8 ? 8 : 16;
  return (int)pg::launch_eval<MAXD>(*a, *static_cast<const Fn*>(user));
}

// C-ABI launcher of one m-Cubes sampling iteration for the functor.
template <class Fn, size_t ND>
int launch_user_mcubes(const pg_mcubes_args* a, void* user) {
  constexpr int MAXD = ND <= 8 ? 8 : 16;
  return (int)pg::launch_mcubes<MAXD>(*a, *static_cast<const Fn*>(user));
}

// Number of parameters of a functor's (non-template) operator(), as
// cubacpp::arity gives it to quad::mcubes (cuda/mcubes/mcubes.cuh:32).
template <class T>
struct arity_of;
template <class C, class R, class... A>
struct arity_of<R (C::*)(A...)> {
  static constexpr size_t value = sizeof...(A);
};
template <class C, class R, class... A>
struct arity_of<R (C::*)(A...) const> {
  static constexpr size_t value = sizeof...(A);
};

// Owns the kernel's copy of a functor for the duration of one call.
template <class F, size_t ND, bool BYVAL = by_value<F>()>
struct FunctorCopy;

template <class F, size_t ND>
struct FunctorCopy<F, ND, true> {
  UserFn<F, ND, true> fn;
  explicit FunctorCopy(const F& f) : fn{f} {}
};

template <class F, size_t ND>
struct FunctorCopy<F, ND, false> {
  UserFn<F, ND, false> fn{nullptr};
  explicit FunctorCopy(const F& f) {
    void* p = nullptr;
    if (cudaMallocManaged(&p, sizeof(F)) != cudaSuccess) throw std::bad_alloc();
    fn.f = new (p) F(f);
  }
  ~FunctorCopy() {
    if (fn.f) {
      cudaDeviceSynchronize();
      fn.f->~F();
      cudaFree(fn.f);
    }
  }
  FunctorCopy(const FunctorCopy&) = delete;
  FunctorCopy& operator=(const FunctorCopy&) = delete;
};

inline integration_result to_result(const pg_result& r) {
  integration_result o;
  o.estimate = r.estimate;
  o.errorest = r.errorest;
  o.neval = (size_t)r.neval;
  o.nregions = (size_t)r.nregions;
  o.nFinishedRegions = (size_t)r.nfinished;
  o.status = r.status;
  o.lastPhase = r.last_phase;
  o.chi_sq = r.chi_sq;
  o.iters = (size_t)r.iters;
  return o;
}

}  // namespace detail

// Sub_regions (cuda/pagani/quad/GPUquad/Sub_regions.cuh:38-258): a region
// list in unit coordinates, SoA [dim * size + i], on the device (dLeftCoord,
// dLength) with a host mirror (LeftCoord, Length), and the snapshot that a
// predict_split run keeps at iteration 15.
template <typename T, size_t ndim>
struct Sub_regions {
  static_assert(std::is_same<T, double>::value, "region lists are double precision");

  Sub_regions() {}
  explicit Sub_regions(const size_t partitions_per_axis) { uniform_split(partitions_per_axis); }
  Sub_regions(const Sub_regions& other) {
    device_init(other.size);
    cudaMemcpy(dLeftCoord, other.dLeftCoord, sizeof(T) * size * ndim, cudaMemcpyDeviceToDevice);
    cudaMemcpy(dLength, other.dLength, sizeof(T) * size * ndim, cudaMemcpyDeviceToDevice);
  }
  Sub_regions& operator=(const Sub_regions&) = delete;
  ~Sub_regions() {
    delete[] LeftCoord;
    delete[] Length;
    cudaFree(dLeftCoord);
    cudaFree(dLength);
    cudaFree(snapshot_dLeftCoord);
    cudaFree(snapshot_dLength);
  }

  void host_init() {
    delete[] LeftCoord;
    delete[] Length;
    host_data_size = size;
    LeftCoord = new T[size * ndim];
    Length = new T[size * ndim];
  }
  void device_init(const size_t numRegions) {
    cudaFree(dLeftCoord);
    cudaFree(dLength);
    size = numRegions;
    dLeftCoord = nullptr;
    dLength = nullptr;
    cudaMalloc((void**)&dLeftCoord, sizeof(T) * numRegions * ndim);
    cudaMalloc((void**)&dLength, sizeof(T) * numRegions * ndim);
  }
  void host_device_init(const size_t numRegions) {
    device_init(numRegions);
    host_init();
  }
  void refresh_host_device() {
    if (host_data_size != size || !LeftCoord) host_init();
    cudaMemcpy(LeftCoord, dLeftCoord, sizeof(T) * size * ndim, cudaMemcpyDeviceToHost);
    cudaMemcpy(Length, dLength, sizeof(T) * size * ndim, cudaMemcpyDeviceToHost);
  }
  void refresh_device_from_host() {
    cudaMemcpy(dLeftCoord, LeftCoord, sizeof(T) * size * ndim, cudaMemcpyHostToDevice);
    cudaMemcpy(dLength, Length, sizeof(T) * size * ndim, cudaMemcpyHostToDevice);
  }

  // p^ndim equal cells: cell i has index (i / p^k) % p on axis k
  // (Sub_regions.cuh:164-185).
  void uniform_split(const size_t p) {
    size_t count = 1;
    for (size_t k = 0; k < ndim; ++k) count *= p;
    const T len = 1.0 / (T)p;
    device_init(count);
    host_init();
    for (size_t i = 0; i < count; ++i) {
      size_t q = i;
      for (size_t k = 0; k < ndim; ++k) {
        const size_t id = q % p;
        q /= p;
        LeftCoord[k * count + i] = (T)id * len;
        Length[k * count + i] = len;
      }
    }
    refresh_device_from_host();
  }

  T compute_region_volume(const size_t regionID) {
    T reg_vol = 1.;
    for (size_t dim = 0; dim < ndim; dim++) reg_vol *= Length[size * dim + regionID];
    return reg_vol;
  }
  T compute_total_volume() {
    refresh_host_device();
    T total_vol = 0.;
    for (size_t i = 0; i < size; i++) total_vol += compute_region_volume(i);
    return total_vol;
  }
  quad::Volume<T, (int)ndim> extract_region(const size_t regionID) {
    refresh_host_device();
    quad::Volume<T, (int)ndim> b;
    for (size_t dim = 0; dim < ndim; dim++) {
      b.lows[dim] = LeftCoord[size * dim + regionID];
      b.highs[dim] = LeftCoord[size * dim + regionID] + Length[size * dim + regionID];
    }
    return b;
  }

  void take_snapshot() {
    cudaFree(snapshot_dLeftCoord);
    cudaFree(snapshot_dLength);
    snapshot_size = size;
    cudaMalloc((void**)&snapshot_dLeftCoord, sizeof(T) * size * ndim);
    cudaMalloc((void**)&snapshot_dLength, sizeof(T) * size * ndim);
    cudaMemcpy(snapshot_dLeftCoord, dLeftCoord, sizeof(T) * size * ndim, cudaMemcpyDeviceToDevice);
    cudaMemcpy(snapshot_dLength, dLength, sizeof(T) * size * ndim, cudaMemcpyDeviceToDevice);
  }
  // The snapshot becomes the region list (Sub_regions.cuh:231-239).
  void load_snapshot() {
    cudaFree(dLeftCoord);
    cudaFree(dLength);
    dLeftCoord = snapshot_dLeftCoord;
    dLength = snapshot_dLength;
    size = snapshot_size;
    snapshot_dLeftCoord = nullptr;
    snapshot_dLength = nullptr;
    snapshot_size = 0;
  }

  T* LeftCoord = nullptr;
  T* Length = nullptr;
  T* dLeftCoord = nullptr;
  T* dLength = nullptr;
  T* snapshot_dLeftCoord = nullptr;
  T* snapshot_dLength = nullptr;
  size_t size = 0;
  size_t host_data_size = 0;
  size_t snapshot_size = 0;
};

// Workspace (cuda/pagani/quad/GPUquad/Workspace.cuh:23-70): one PAGANI
// integrator on the current CUDA device.  It owns a library context (region
// pool, stream, rule tables), created at the first integrate call and kept for
// the object's lifetime, so repeated calls reuse the device memory.  Failures
// of the library (bad arguments, out of memory, CUDA errors) throw
// std::runtime_error where the reference aborts; a run that does not converge
// returns status 1 as in the reference.
template <typename T, size_t ndim, int debug = 0, bool use_custom = false, bool collect_mult_runs = false>
class Workspace {
  static_assert(std::is_same<T, double>::value, "the GB300 PAGANI library integrates in double precision");
  static_assert(ndim >= PG_MIN_NDIM && ndim <= PG_MAX_NDIM, "ndim outside the library's 2..PG_MAX_NDIM");

 public:
  Workspace() = default;
  ~Workspace() {
    if (ctx_) pg_context_destroy(ctx_);
  }
  Workspace(const Workspace&) = delete;
  Workspace& operator=(const Workspace&) = delete;

  // From the uniform split (Workspace.cuh:361-368).  predict_split: no
  // rel-err classification in the first 15 iterations while the list is small
  // and nothing has finished (Workspace.cuh:415-420).  collect_iters (debug
  // output of the reference) is accepted and ignored.
  template <typename IntegT, bool predict_split = false, bool collect_iters = false>
  integration_result integrate(const IntegT& integrand, T epsrel, T epsabs, Volume<T, (int)ndim> const& vol,
                               bool relerr_classification = true) {
    return run<IntegT, predict_split>(integrand, nullptr, epsrel, epsabs, vol, relerr_classification);
  }

  // From the caller's region list (Workspace.cuh:148-158); with predict_split
  // the list of iteration 15 is kept in subregions' snapshot
  // (Workspace.cuh:437-441).  `optional` names the run in the reference's
  // debug output and is ignored.
  template <typename IntegT, bool predict_split = false, bool collect_iters = false>
  integration_result integrate(const IntegT& integrand, Sub_regions<T, ndim>& subregions, T epsrel, T epsabs,
                               Volume<T, (int)ndim> const& vol, bool relerr_classification = true,
                               const std::string& optional = "default") {
    (void)optional;
    return run<IntegT, predict_split>(integrand, &subregions, epsrel, epsabs, vol, relerr_classification);
  }

  // Region evaluation of the functor on caller-given regions (SoA
  // [dim * n + i] on the host): the stage unit the reference's tests call
  // through Cubature_rules::apply_cubature_integration_rules
  // (cuda/pagani/quad/GPUquad/PaganiUtils.cuh:243-289).
  template <typename IntegT>
  void evaluate_regions(const IntegT& integrand, Volume<T, (int)ndim> const& vol, size_t n, const double* left,
                        const double* length, double* est, double* err, int* bisect) {
    using Fn = detail::UserFn<IntegT, ndim>;
    detail::FunctorCopy<IntegT, ndim> copy(integrand);
    const int rc = pg_evaluate_regions_launcher(context(), (int32_t)ndim, &detail::launch_user<Fn, ndim>,
                                                (void*)&copy.fn, vol.lows, vol.highs, (uint64_t)n, left, length,
                                                est, err, reinterpret_cast<int32_t*>(bisect));
    if (rc < 0)
      throw std::runtime_error(std::string("pagani::Workspace::evaluate_regions: ") + pg_last_error(ctx_));
  }

 private:
  template <typename IntegT, bool predict_split>
  integration_result run(const IntegT& integrand, Sub_regions<T, ndim>* sub, T epsrel, T epsabs,
                         Volume<T, (int)ndim> const& vol, bool relerr_classification) {
    using Fn = detail::UserFn<IntegT, ndim>;
    detail::FunctorCopy<IntegT, ndim> copy(integrand);
    pg_options opt;
    pg_options_default(&opt);
    opt.relerr_classification = relerr_classification ? 1 : 0;
    opt.predict_split = predict_split ? 1 : 0;
    pg_result r;
    std::memset(&r, 0, sizeof r);
    const T* left = nullptr;
    const T* length = nullptr;
    uint64_t n = 0;
    if (sub) {
      sub->refresh_host_device();
      left = sub->LeftCoord;
      length = sub->Length;
      n = sub->size;
    }
    const int rc = pg_integrate_regions_launcher(context(), (int32_t)ndim, &detail::launch_user<Fn, ndim>,
                                                 (void*)&copy.fn, left, length, n, epsrel, epsabs, vol.lows,
                                                 vol.highs, &opt, &r);
    if (rc < 0) throw std::runtime_error(std::string("pagani::Workspace::integrate: ") + pg_last_error(ctx_));
    if (sub && predict_split) {
      int32_t d = 0;
      uint64_t sn = 0;
      pg_last_snapshot(ctx_, &d, &sn, nullptr, nullptr, 0);
      if (sn) {
        std::vector<T> sl(sn * ndim), sd(sn * ndim);
        pg_last_snapshot(ctx_, &d, &sn, sl.data(), sd.data(), sn);
        cudaFree(sub->snapshot_dLeftCoord);
        cudaFree(sub->snapshot_dLength);
        cudaMalloc((void**)&sub->snapshot_dLeftCoord, sizeof(T) * sn * ndim);
        cudaMalloc((void**)&sub->snapshot_dLength, sizeof(T) * sn * ndim);
        cudaMemcpy(sub->snapshot_dLeftCoord, sl.data(), sizeof(T) * sn * ndim, cudaMemcpyHostToDevice);
        cudaMemcpy(sub->snapshot_dLength, sd.data(), sizeof(T) * sn * ndim, cudaMemcpyHostToDevice);
        sub->snapshot_size = (size_t)sn;
      }
    }
    return detail::to_result(r);
  }

 public:
  // The library context (created on the current device at first use).
  pg_context* context() {
    if (!ctx_) {
      int dev = 0;
      cudaGetDevice(&dev);
      if (pg_context_create(dev, &ctx_) != PG_OK) {
        ctx_ = nullptr;
        throw std::runtime_error("pagani::Workspace: no library context on this device");
      }
    }
    return ctx_;
  }

 private:
  pg_context* ctx_ = nullptr;
};

template <class F>
constexpr size_t arity() {
  return detail::arity_of<decltype(&F::operator())>::value;
}

// m-Cubes (stratified VEGAS) of a user functor, cuda_mcubes::integrate
// (cuda/mcubes/vegasT.cuh:999-1030), on the current device.  The random
// stream is Philox4x32-10 keyed by `seed` (the reference seeds from the
// clock), so a run is reproducible.
template <typename IntegT, int NDIM>
integration_result mcubes_integrate(IntegT const& integrand, double epsrel, double epsabs, double ncall,
                                    Volume<double, NDIM> const* volume, int totalIters = 15, int adjustIters = 15,
                                    int skipIters = 5, uint64_t seed = 0) {
  static_assert(NDIM >= PG_MIN_NDIM && NDIM <= PG_MAX_NDIM, "ndim outside the library's 2..PG_MAX_NDIM");
  using Fn = detail::UserFn<IntegT, (size_t)NDIM>;
  detail::FunctorCopy<IntegT, (size_t)NDIM> copy(integrand);
  int dev = 0;
  cudaGetDevice(&dev);
  pg_context* ctx = nullptr;
  if (pg_context_create(dev, &ctx) != PG_OK) throw std::runtime_error("pagani::mcubes_integrate: no library context");
  pg_mcubes_options opt;
  pg_mcubes_options_default(&opt);
  opt.ncall = ncall;
  opt.titer = totalIters;
  opt.itmax = adjustIters;
  opt.skip = skipIters;
  if (seed) opt.seed = seed;
  pg_result r;
  std::memset(&r, 0, sizeof r);
  Volume<double, NDIM> unit;
  const Volume<double, NDIM>& v = volume ? *volume : unit;
  const int rc = pg_mcubes_integrate_launcher(ctx, NDIM, &detail::launch_user_mcubes<Fn, (size_t)NDIM>,
                                              (void*)&copy.fn, epsrel, epsabs, v.lows, v.highs, &opt, &r);
  std::string msg = rc < 0 ? pg_last_error(ctx) : "";
  pg_context_destroy(ctx);
  if (rc < 0) throw std::runtime_error("pagani::mcubes_integrate: " + msg);
  return detail::to_result(r);
}

}  // namespace pagani

#ifndef PAGANI_GB300_NO_REFERENCE_NAMES
template <typename T, size_t ndim, int debug = 0, bool use_custom = false, bool collect_mult_runs = false>
using Workspace = pagani::Workspace<T, ndim, debug, use_custom, collect_mult_runs>;
template <typename T, size_t ndim>
using Sub_regions = pagani::Sub_regions<T, ndim>;

namespace cuda_mcubes {
// cuda/mcubes/vegasT.cuh:999-1030 (GeneratorType is accepted and ignored: the
// library samples with Philox4x32-10).
template <typename IntegT, int NDIM, bool DEBUG_MCUBES = false, typename GeneratorType = void>
numint::integration_result integrate(IntegT const& ig, double epsrel, double epsabs, double ncall,
                                     quad::Volume<double, NDIM> const* volume, int totalIters = 15,
                                     int adjustIters = 15, int skipIters = 5) {
  return pagani::mcubes_integrate<IntegT, NDIM>(ig, epsrel, epsabs, ncall, volume, totalIters, adjustIters,
                                                skipIters);
}

// Retry policy of simple_integrate (cuda/mcubes/util/vegas_utils.cuh:282-296).
inline bool AdjustParams(double& ncall, int& totalIters) {
  if (ncall >= 8.e9 && totalIters >= 100) return false;
  if (ncall >= 8.e9) {
    totalIters += 10;
    return true;
  }
  if (ncall >= 1.e9) {
    ncall += 1.e9;
    return true;
  }
  ncall *= 10.;
  return true;
}

// cuda/mcubes/vegasT.cuh:1076-1111: integrate, and while the result has not
// converged, again with more calls or iterations.
template <typename IntegT, int NDIM, bool DEBUG_MCUBES = false, typename GeneratorType = void>
numint::integration_result simple_integrate(IntegT const& integrand, double epsrel, double epsabs, double ncall,
                                            quad::Volume<double, NDIM> const* volume, int totalIters = 15,
                                            int adjustIters = 15, int skipIters = 5) {
  numint::integration_result result;
  result.status = 1;
  do {
    result = pagani::mcubes_integrate<IntegT, NDIM>(integrand, epsrel, epsabs, ncall, volume, totalIters,
                                                    adjustIters, skipIters);
  } while (result.status == 1 && AdjustParams(ncall, totalIters));
  return result;
}

// cuda/mcubes/vegasT.cuh:1035-1073.
class mcubes {
 public:
  mcubes(double epsrel, double epsabs, double ncall, int totalIters = 15, int adjustIters = 15, int skipIters = 5)
      : epsrel_(epsrel), epsabs_(epsabs), ncall_(ncall), totalIters_(totalIters), adjustIters_(adjustIters),
        skipIters_(skipIters) {}
  template <typename F, int NDIM>
  numint::integration_result integrate(F const& integrand, quad::Volume<double, NDIM> const* volume) {
    return cuda_mcubes::integrate<F, NDIM>(integrand, epsrel_, epsabs_, ncall_, volume, totalIters_, adjustIters_,
                                           skipIters_);
  }

 private:
  double epsrel_, epsabs_, ncall_;
  int totalIters_, adjustIters_, skipIters_;
};
}  // namespace cuda_mcubes

namespace quad {
// cuda/mcubes/mcubes.cuh:9-41 (note the epsabs, epsrel argument order).
struct mcubes {
  long long int maxcalls = 1000 * 1000ULL;
  int total_iters = 70;
  int adjust_iters = 20;
  int skip_iters = 0;

  template <typename F>
  numint::integration_result integrate(F const& f, double epsabs, double epsrel,
                                       quad::Volume<double, (int)pagani::arity<F>()> const* pvol) {
    constexpr int ndim = (int)pagani::arity<F>();
    return cuda_mcubes::simple_integrate<F, ndim>(f, epsrel, epsabs, static_cast<double>(maxcalls), pvol,
                                                  total_iters, adjust_iters, skip_iters);
  }
};
}  // namespace quad
#endif

#endif  // PAGANI_GB300_CUH
