/* Integrand-side helpers for C++ callers of pagani_gb300.cuh.
 *
 * Physics integrands handed to Workspace<T, ndim>::integrate often carry
 * state: coefficient arrays, run-time-sized parameter lists and tabulated
 * functions.  The reference ships helpers for that state, and this header
 * provides them under the same names and interfaces so such functors compile
 * unchanged:
 *
 *   gpu::cudaArray<T, N>      fixed-size array usable in device code
 *                             (common/cuda/cudaArray.cuh:10-60)
 *   gpu::cudaDynamicArray<T>  run-time-sized array in managed memory whose
 *                             copies are deep (cudaArray.cuh:62-150)
 *   quad::polynomial<Order>   Horner evaluation, highest power first
 *                             (cuda/pagani/quad/GPUquad/Polynomial.cuh:8-27)
 *   quad::Interp1D            piecewise-linear table (common/cuda/Interp1D.cuh)
 *   quad::Interp2D            bilinear table, z(x_i, y_j) at zs[j * nx + i]
 *                             (common/cuda/Interp2D.cuh)
 *   quad::Interp3D            trilinear table, v(x_i, y_j, z_k) at
 *                             vs[i + nx * j + nx * ny * k] (common/cuda/Interp3D.cuh)
 *
 * Interpolation tables.  A table never changes after it is built, so its
 * copies share one store instead of each owning a device copy: the axes and
 * values sit in one device allocation in HBM, uploaded once at construction,
 * beside a host copy of the same numbers; a copy made on the host takes a
 * reference to the store (a host-side count), and the last one frees it.
 * Handing a functor that holds tables to the integrator (which copies the
 * functor into managed memory for the evaluation kernel) therefore allocates
 * and copies nothing on the device.  Device code reads the device arrays
 * through the read-only data path; host code reads the host copy, so a table
 * can be evaluated on either side with the same result bit for bit.
 *
 * Lookup: the interval [a_i, a_{i+1}] holding v is found by bisection over the
 * axis; a value below the first knot uses the first interval and one above
 * the last uses the last (the line of the end interval is extended; clamp()
 * clamps to the table first, as in the reference).  Inside an interval the
 * weight t = (v - a_i) / (a_{i+1} - a_i) interpolates as (1 - t) y_i + t y_{i+1},
 * axis by axis (x, then y, then z), which returns the tabulated value exactly
 * at every knot.  Every floating-point operation is an explicit IEEE operation
 * (a multiply, then a fused multiply-add), so the caller's contraction
 * settings do not change the bits.  Axes must hold at least two strictly
 * increasing knots; a table that breaks this throws std::invalid_argument,
 * and a failed allocation throws std::bad_alloc (the reference aborts or
 * throws std::bad_alloc).  A default-constructed table evaluates to NaN.
 *
 * Each type sits under the include guard of the reference header it stands
 * for, so a translation unit that also includes the reference's helpers
 * compiles with whichever header comes first.
 */
#ifndef PAGANI_GB300_HELPERS_CUH
#define PAGANI_GB300_HELPERS_CUH

#include <cuda_runtime.h>

#include <array>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <initializer_list>
#include <istream>
#include <new>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

// ---------------------------------------------------------------------------
#ifndef CUDACUHRE_QUAD_UTIL_CUDAARRAY_CUH
#define CUDACUHRE_QUAD_UTIL_CUDAARRAY_CUH
namespace gpu {

// Fixed-size array that is trivially copyable, so a functor holding one is
// passed to the evaluation kernel by value.
template <typename T, std::size_t s>
class cudaArray {
 public:
  void Initialize(T const* initData) { std::memcpy(data, initData, sizeof(T) * s); }
  __host__ __device__ const T* begin() const { return &data[0]; }
  __host__ __device__ const T* end() const { return &data[0] + s; }
  __host__ __device__ constexpr std::size_t size() const { return s; }
  __host__ __device__ T& operator[](std::size_t i) { return data[i]; }
  __host__ __device__ T const& operator[](std::size_t i) const { return data[i]; }
  T data[s];
};

// Run-time-sized array in managed memory, readable and writable on the host
// and in kernels.  A copy is deep: a copy made on the host gets its own
// managed allocation, a copy made in device code its own device-heap buffer,
// so a copy passed by value to a kernel can be changed there without
// touching the original (the reference's semantics).  Unlike the reference,
// which never frees under nvcc, each object frees what it allocated: on the
// host with cudaFree (which waits for the device), in device code with
// delete[].
template <typename T>
class cudaDynamicArray {
 public:
  __host__ __device__ cudaDynamicArray() : _data(nullptr), N(0), _heap(false) {}

  cudaDynamicArray(T const* initData, size_t s) : _data(nullptr), N(0), _heap(false) {
    allocate(s);
    if (s) std::memcpy(_data, initData, sizeof(T) * s);
  }

  explicit cudaDynamicArray(size_t s) : _data(nullptr), N(0), _heap(false) { allocate(s); }

  __host__ __device__ cudaDynamicArray(const cudaDynamicArray& a) : _data(nullptr), N(0), _heap(false) {
#ifdef __CUDA_ARCH__
    N = a.N;
    _heap = true;
    _data = N ? new T[N] : nullptr;
    for (size_t i = 0; _data && i < N; ++i) _data[i] = a._data[i];
#else
    allocate(a.N);
    if (N) std::memcpy(_data, a._data, sizeof(T) * N);
#endif
  }

  cudaDynamicArray(cudaDynamicArray&& a) noexcept : _data(a._data), N(a.N), _heap(a._heap) {
    a._data = nullptr;
    a.N = 0;
  }

  cudaDynamicArray& operator=(const cudaDynamicArray& a) {
    cudaDynamicArray tmp(a);
    swap(tmp);
    return *this;
  }

  cudaDynamicArray& operator=(cudaDynamicArray&& a) noexcept {
    swap(a);
    return *this;
  }

  __host__ __device__ ~cudaDynamicArray() { release(); }

  // Replaces the contents by s default values (the old buffer is freed).
  void Reserve(size_t s) {
    release();
    allocate(s);
  }

  void swap(cudaDynamicArray& o) noexcept {
    std::swap(_data, o._data);
    std::swap(N, o.N);
    std::swap(_heap, o._heap);
  }

  __host__ __device__ const T* begin() const { return &_data[0]; }
  __host__ __device__ const T* end() const { return &_data[0] + N; }
  __host__ __device__ constexpr std::size_t size() const { return N; }
  __host__ __device__ T* data() { return _data; }
  __host__ __device__ T& operator[](std::size_t i) { return _data[i]; }
  __host__ __device__ T operator[](std::size_t i) const { return _data[i]; }

 private:
  void allocate(size_t s) {
    N = s;
    _heap = false;
    _data = nullptr;
    if (!s) return;
    void* p = nullptr;
    if (cudaMallocManaged(&p, sizeof(T) * s) != cudaSuccess) {
      cudaGetLastError();
      N = 0;
      throw std::bad_alloc();
    }
    _data = static_cast<T*>(p);
  }

  __host__ __device__ void release() {
#ifdef __CUDA_ARCH__
    if (_heap) delete[] _data;
#else
    if (_data && !_heap) cudaFree(_data);
#endif
    _data = nullptr;
    N = 0;
  }

  T* _data;
  size_t N;
  bool _heap;  // _data is a device-heap buffer made by a copy in device code
};

}  // namespace gpu
#endif  // CUDACUHRE_QUAD_UTIL_CUDAARRAY_CUH

// ---------------------------------------------------------------------------
#ifndef POLYNOMIAL_H
#define POLYNOMIAL_H
namespace quad {

// sum_i coeffs[i] x^(Order-1-i), by Horner's rule with one fused multiply-add
// per coefficient.
template <size_t Order>
class polynomial {
 private:
  const gpu::cudaArray<double, Order> coeffs;

 public:
  __host__ __device__ polynomial(gpu::cudaArray<double, Order> c) : coeffs(c) {}

  __host__ __device__ double operator()(const double x) const {
    double out = 0.0;
    for (size_t i = 0; i < Order; ++i) {
#ifdef __CUDA_ARCH__
      out = __fma_rn(x, out, coeffs[i]);
#else
      out = std::fma(x, out, coeffs[i]);
#endif
    }
    return out;
  }
};

}  // namespace quad
#endif  // POLYNOMIAL_H

// ---------------------------------------------------------------------------
// Shared machinery of the interpolation tables.
#ifndef PAGANI_GB300_TABLE_STORE
#define PAGANI_GB300_TABLE_STORE
namespace pagani {
namespace table {

// The numbers of one table, on the host and in one device allocation, with
// the count of the table objects that use them.
struct Store {
  std::atomic<long> refs{1};
  std::vector<double> host;
  double* dev = nullptr;
};

// Builds a store from `parts` (axes, then values), each copied in order.
inline Store* make_store(std::initializer_list<std::pair<const double*, size_t>> parts) {
  size_t n = 0;
  for (const auto& p : parts) n += p.second;
  Store* s = new Store;
  s->host.resize(n);
  size_t at = 0;
  for (const auto& p : parts) {
    if (p.second) std::memcpy(s->host.data() + at, p.first, sizeof(double) * p.second);
    at += p.second;
  }
  void* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * n) != cudaSuccess ||
      cudaMemcpy(d, s->host.data(), sizeof(double) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    if (d) cudaFree(d);
    delete s;
    throw std::bad_alloc();
  }
  s->dev = static_cast<double*>(d);
  return s;
}

inline Store* retain(Store* s) {
  if (s) s->refs.fetch_add(1, std::memory_order_relaxed);
  return s;
}

inline void release(Store* s) {
  if (s && s->refs.fetch_sub(1, std::memory_order_acq_rel) == 1) {
    cudaFree(s->dev);  // waits for kernels that may still read it
    delete s;
  }
}

inline void check_axis(const double* a, size_t n, const char* what) {
  if (n < 2) throw std::invalid_argument(std::string(what) + ": an axis needs at least two knots");
  for (size_t i = 0; i + 1 < n; ++i)
    if (!(a[i] < a[i + 1])) throw std::invalid_argument(std::string(what) + ": axis knots must increase strictly");
}

// Element i of a table array: the device copy in device code (read-only
// path), the host copy on the host.
__host__ __device__ __forceinline__ double at(const double* dev, const double* host, size_t i) {
#ifdef __CUDA_ARCH__
  (void)host;
  return __ldg(dev + i);
#else
  (void)dev;
  return host[i];
#endif
}

// Interval [a_i, a_{i+1}] of the n-knot axis holding v, by bisection; values
// outside the axis take the end intervals.
__host__ __device__ __forceinline__ size_t interval(const double* dev, const double* host, size_t n, double v) {
  size_t lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    const size_t mid = lo + (hi - lo) / 2;
    if (v < at(dev, host, mid))
      hi = mid;
    else
      lo = mid;
  }
  return lo;
}

// Weight of v in [a0, a1] and the interpolation (1 - t) y0 + t y1.
__host__ __device__ __forceinline__ double weight(double v, double a0, double a1) {
#ifdef __CUDA_ARCH__
  return __ddiv_rn(__dsub_rn(v, a0), __dsub_rn(a1, a0));
#else
  return (v - a0) / (a1 - a0);
#endif
}

__host__ __device__ __forceinline__ double lerp(double y0, double y1, double t) {
#ifdef __CUDA_ARCH__
  return __fma_rn(t, y1, __dmul_rn(__dsub_rn(1.0, t), y0));
#else
  const double u = 1.0 - t;
  const double p = u * y0;
  return std::fma(t, y1, p);
#endif
}

// Value of a table that holds nothing (default-constructed): NaN.
__host__ __device__ __forceinline__ double empty_value() {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(0x7ff8000000000000ll);
#else
  return std::nan("");
#endif
}

__host__ __device__ __forceinline__ double clamp_to(double v, double lo, double hi) {
  return (v < lo) ? lo : (hi < v) ? hi : v;
}

// Whitespace-separated numbers of one line (decimal or hexadecimal floats).
inline std::vector<double> line_of_doubles(std::istream& is) {
  std::string buffer;
  std::getline(is, buffer);
  std::istringstream in(buffer);
  std::vector<double> vals;
  std::string tok;
  while (in >> tok) vals.push_back(std::stod(tok));
  return vals;
}

}  // namespace table
}  // namespace pagani
#endif  // PAGANI_GB300_TABLE_STORE

// ---------------------------------------------------------------------------
#ifndef GPUQUADINTERP1D_H
#define GPUQUADINTERP1D_H
namespace quad {

class Interp1D {
 public:
  Interp1D() = default;

  template <size_t M>
  Interp1D(std::array<double, M> const& xs, std::array<double, M> const& zs) : Interp1D(xs.data(), zs.data(), M) {}

  Interp1D(double const* xs, double const* zs, size_t cols) { build(xs, zs, cols); }

  Interp1D(std::vector<double> const& xs, std::vector<double> const& zs) {
    if (xs.size() != zs.size()) throw std::invalid_argument("Interp1D: xs and zs differ in length");
    build(xs.data(), zs.data(), xs.size());
  }

  __host__ __device__ Interp1D(const Interp1D& o) : _cols(o._cols), _dev(o._dev), _host(o._host), _store(o._store) {
#ifndef __CUDA_ARCH__
    pagani::table::retain(_store);
#endif
  }

  Interp1D& operator=(Interp1D const& rhs) {
    Interp1D tmp(rhs);
    swap(tmp);
    return *this;
  }

  __host__ __device__ ~Interp1D() {
#ifndef __CUDA_ARCH__
    pagani::table::release(_store);
#endif
  }

  void swap(Interp1D& o) noexcept {
    std::swap(_cols, o._cols);
    std::swap(_dev, o._dev);
    std::swap(_host, o._host);
    std::swap(_store, o._store);
  }

  // Device bytes the table holds (shared by all copies).
  size_t get_device_mem_footprint() const { return 8 * 2 * _cols; }

  __host__ __device__ double operator()(double x) const {
    using namespace pagani::table;
    if (_cols < 2) return empty_value();
    const size_t i = interval(_dev, _host, _cols, x);
    const double t = weight(x, at(_dev, _host, i), at(_dev, _host, i + 1));
    return lerp(at(_dev, _host, _cols + i), at(_dev, _host, _cols + i + 1), t);
  }

  __host__ __device__ double min_x() const { return pagani::table::at(_dev, _host, 0); }
  __host__ __device__ double max_x() const { return pagani::table::at(_dev, _host, _cols - 1); }
  __host__ __device__ double do_clamp(double v, double lo, double hi) const {
    return pagani::table::clamp_to(v, lo, hi);
  }
  __host__ __device__ double eval(double x) const { return (*this)(x); }
  __host__ __device__ double clamp(double x) const { return eval(do_clamp(x, min_x(), max_x())); }

  // Two lines: the knots, then the values.
  friend std::istream& operator>>(std::istream& is, Interp1D& interp) {
    const std::vector<double> xs = pagani::table::line_of_doubles(is);
    const std::vector<double> zs = pagani::table::line_of_doubles(is);
    Interp1D tmp(xs, zs);
    interp.swap(tmp);
    return is;
  }

 private:
  void build(double const* xs, double const* zs, size_t cols) {
    pagani::table::check_axis(xs, cols, "Interp1D");
    _store = pagani::table::make_store({{xs, cols}, {zs, cols}});
    _cols = cols;
    _dev = _store->dev;
    _host = _store->host.data();
  }

  size_t _cols = 0;
  const double* _dev = nullptr;   // [xs | zs] in device memory
  const double* _host = nullptr;  // the same on the host
  pagani::table::Store* _store = nullptr;
};

}  // namespace quad
#endif  // GPUQUADINTERP1D_H

// ---------------------------------------------------------------------------
#ifndef GPUQUADINTERP2D_H
#define GPUQUADINTERP2D_H
namespace quad {

class Interp2D {
 public:
  __host__ __device__ Interp2D() {}

  // zs[j * M + i] = z(xs[i], ys[j])
  template <size_t M, size_t N>
  Interp2D(std::array<double, M> const& xs, std::array<double, N> const& ys, std::array<double, N * M> const& zs) {
    build(xs.data(), ys.data(), zs.data(), M, N);
  }

  Interp2D(double const* xs, double const* ys, double const* zs, size_t cols, size_t rows) {
    build(xs, ys, zs, cols, rows);
  }

  Interp2D(std::vector<double> const& xs, std::vector<double> const& ys, std::vector<double> const& zs) {
    if (zs.size() != xs.size() * ys.size()) throw std::invalid_argument("Interp2D: zs must hold xs.size() * ys.size()");
    build(xs.data(), ys.data(), zs.data(), xs.size(), ys.size());
  }

  // zs[i][j] = z(xs[i], ys[j])
  template <size_t M, size_t N>
  Interp2D(std::array<double, M> xs, std::array<double, N> ys, std::array<std::array<double, N>, M> zs) {
    std::vector<double> buffer(N * M);
    for (size_t i = 0; i < M; ++i)
      for (size_t j = 0; j < N; ++j) buffer[i + j * M] = zs[i][j];
    build(xs.data(), ys.data(), buffer.data(), M, N);
  }

  __host__ __device__ Interp2D(const Interp2D& o)
      : _rows(o._rows), _cols(o._cols), _dev(o._dev), _host(o._host), _store(o._store) {
#ifndef __CUDA_ARCH__
    pagani::table::retain(_store);
#endif
  }

  Interp2D& operator=(Interp2D const& rhs) {
    Interp2D tmp(rhs);
    swap(tmp);
    return *this;
  }

  __host__ __device__ ~Interp2D() {
#ifndef __CUDA_ARCH__
    pagani::table::release(_store);
#endif
  }

  void swap(Interp2D& o) noexcept {
    std::swap(_rows, o._rows);
    std::swap(_cols, o._cols);
    std::swap(_dev, o._dev);
    std::swap(_host, o._host);
    std::swap(_store, o._store);
  }

  size_t get_device_mem_footprint() const { return 8 * (_cols * _rows + _cols + _rows); }

  __host__ __device__ double operator()(double x, double y) const {
    using namespace pagani::table;
    if (_cols < 2 || _rows < 2) return empty_value();
    const double* xs_d = _dev;
    const double* xs_h = _host;
    const double* ys_d = _dev ? _dev + _cols : nullptr;
    const double* ys_h = _host ? _host + _cols : nullptr;
    const size_t vo = _cols + _rows;
    const size_t i = interval(xs_d, xs_h, _cols, x);
    const size_t j = interval(ys_d, ys_h, _rows, y);
    const double tx = weight(x, at(xs_d, xs_h, i), at(xs_d, xs_h, i + 1));
    const double ty = weight(y, at(ys_d, ys_h, j), at(ys_d, ys_h, j + 1));
    const size_t r0 = vo + j * _cols + i, r1 = r0 + _cols;
    const double z0 = lerp(at(_dev, _host, r0), at(_dev, _host, r0 + 1), tx);
    const double z1 = lerp(at(_dev, _host, r1), at(_dev, _host, r1 + 1), tx);
    return lerp(z0, z1, ty);
  }

  __host__ __device__ double min_x() const { return pagani::table::at(_dev, _host, 0); }
  __host__ __device__ double max_x() const { return pagani::table::at(_dev, _host, _cols - 1); }
  __host__ __device__ double min_y() const { return pagani::table::at(_dev, _host, _cols); }
  __host__ __device__ double max_y() const { return pagani::table::at(_dev, _host, _cols + _rows - 1); }
  __host__ __device__ double do_clamp(double v, double lo, double hi) const {
    return pagani::table::clamp_to(v, lo, hi);
  }
  __host__ __device__ double eval(double x, double y) const { return (*this)(x, y); }
  __host__ __device__ double clamp(double x, double y) const {
    return eval(do_clamp(x, min_x(), max_x()), do_clamp(y, min_y(), max_y()));
  }

  // Three lines: the x knots, the y knots, the values (z(x_i, y_j) at j * nx + i).
  friend std::istream& operator>>(std::istream& is, Interp2D& interp) {
    const std::vector<double> xs = pagani::table::line_of_doubles(is);
    const std::vector<double> ys = pagani::table::line_of_doubles(is);
    const std::vector<double> zs = pagani::table::line_of_doubles(is);
    Interp2D tmp(xs, ys, zs);
    interp.swap(tmp);
    return is;
  }

 private:
  void build(double const* xs, double const* ys, double const* zs, size_t cols, size_t rows) {
    pagani::table::check_axis(xs, cols, "Interp2D");
    pagani::table::check_axis(ys, rows, "Interp2D");
    _store = pagani::table::make_store({{xs, cols}, {ys, rows}, {zs, cols * rows}});
    _cols = cols;
    _rows = rows;
    _dev = _store->dev;
    _host = _store->host.data();
  }

  size_t _rows = 0;  // y knots
  size_t _cols = 0;  // x knots
  const double* _dev = nullptr;   // [xs | ys | zs] in device memory
  const double* _host = nullptr;  // the same on the host
  pagani::table::Store* _store = nullptr;
};

}  // namespace quad
#endif  // GPUQUADINTERP2D_H

// ---------------------------------------------------------------------------
#ifndef CUDA_INTERP_3D_CUH
#define CUDA_INTERP_3D_CUH
namespace quad {

class Interp3D {
 public:
  __host__ __device__ Interp3D() {}

  // vals[i + M * j + M * N * k] = v(xs[i], ys[j], zs[k])
  template <size_t M, size_t N, size_t S>
  Interp3D(std::array<double, M> const& xs, std::array<double, N> const& ys, std::array<double, S> const& zs,
           std::array<double, N * M * S> const& vals) {
    build(xs.data(), ys.data(), zs.data(), vals.data(), M, N, S);
  }

  Interp3D(double const* xs, double const* ys, double const* zs, double const* vs, size_t x_size, size_t y_size,
           size_t z_size) {
    build(xs, ys, zs, vs, x_size, y_size, z_size);
  }

  Interp3D(std::vector<double> const& xs, std::vector<double> const& ys, std::vector<double> const& zs,
           std::vector<double> const& vs) {
    if (vs.size() != xs.size() * ys.size() * zs.size())
      throw std::invalid_argument("Interp3D: vs must hold xs.size() * ys.size() * zs.size()");
    build(xs.data(), ys.data(), zs.data(), vs.data(), xs.size(), ys.size(), zs.size());
  }

  __host__ __device__ Interp3D(const Interp3D& o)
      : size_x(o.size_x), size_y(o.size_y), size_z(o.size_z), _dev(o._dev), _host(o._host), _store(o._store) {
#ifndef __CUDA_ARCH__
    pagani::table::retain(_store);
#endif
  }

  Interp3D& operator=(Interp3D const& rhs) {
    Interp3D tmp(rhs);
    swap(tmp);
    return *this;
  }

  __host__ __device__ ~Interp3D() {
#ifndef __CUDA_ARCH__
    pagani::table::release(_store);
#endif
  }

  void swap(Interp3D& o) noexcept {
    std::swap(size_x, o.size_x);
    std::swap(size_y, o.size_y);
    std::swap(size_z, o.size_z);
    std::swap(_dev, o._dev);
    std::swap(_host, o._host);
    std::swap(_store, o._store);
  }

  size_t get_device_mem_footprint() const { return 8 * (size_x * size_y * size_z + size_x + size_y + size_z); }

  __host__ __device__ size_t index(size_t x, size_t y, size_t z) const {
    return x + size_x * y + size_x * size_y * z;
  }

  __host__ __device__ double operator()(double x, double y, double z) const {
    using namespace pagani::table;
    if (size_x < 2 || size_y < 2 || size_z < 2) return empty_value();
    const double* xd = _dev;
    const double* xh = _host;
    const double* yd = _dev ? _dev + size_x : nullptr;
    const double* yh = _host ? _host + size_x : nullptr;
    const double* zd = _dev ? _dev + size_x + size_y : nullptr;
    const double* zh = _host ? _host + size_x + size_y : nullptr;
    const double* vd = _dev ? _dev + size_x + size_y + size_z : nullptr;
    const double* vh = _host ? _host + size_x + size_y + size_z : nullptr;
    const size_t i = interval(xd, xh, size_x, x);
    const size_t j = interval(yd, yh, size_y, y);
    const size_t k = interval(zd, zh, size_z, z);
    const double tx = weight(x, at(xd, xh, i), at(xd, xh, i + 1));
    const double ty = weight(y, at(yd, yh, j), at(yd, yh, j + 1));
    const double tz = weight(z, at(zd, zh, k), at(zd, zh, k + 1));
    const double c00 = lerp(at(vd, vh, index(i, j, k)), at(vd, vh, index(i + 1, j, k)), tx);
    const double c01 = lerp(at(vd, vh, index(i, j, k + 1)), at(vd, vh, index(i + 1, j, k + 1)), tx);
    const double c10 = lerp(at(vd, vh, index(i, j + 1, k)), at(vd, vh, index(i + 1, j + 1, k)), tx);
    const double c11 = lerp(at(vd, vh, index(i, j + 1, k + 1)), at(vd, vh, index(i + 1, j + 1, k + 1)), tx);
    const double c0 = lerp(c00, c10, ty);
    const double c1 = lerp(c01, c11, ty);
    return lerp(c0, c1, tz);
  }

  __host__ __device__ double min_x() const { return pagani::table::at(_dev, _host, 0); }
  __host__ __device__ double max_x() const { return pagani::table::at(_dev, _host, size_x - 1); }
  __host__ __device__ double min_y() const { return pagani::table::at(_dev, _host, size_x); }
  __host__ __device__ double max_y() const { return pagani::table::at(_dev, _host, size_x + size_y - 1); }
  __host__ __device__ double min_z() const { return pagani::table::at(_dev, _host, size_x + size_y); }
  __host__ __device__ double max_z() const { return pagani::table::at(_dev, _host, size_x + size_y + size_z - 1); }
  __host__ __device__ double do_clamp(double v, double lo, double hi) const {
    return pagani::table::clamp_to(v, lo, hi);
  }
  __host__ __device__ double eval(double x, double y, double z) const { return (*this)(x, y, z); }
  __host__ __device__ double clamp(double x, double y, double z) const {
    return eval(do_clamp(x, min_x(), max_x()), do_clamp(y, min_y(), max_y()), do_clamp(z, min_z(), max_z()));
  }

 private:
  void build(double const* xs, double const* ys, double const* zs, double const* vs, size_t nx, size_t ny,
             size_t nz) {
    pagani::table::check_axis(xs, nx, "Interp3D");
    pagani::table::check_axis(ys, ny, "Interp3D");
    pagani::table::check_axis(zs, nz, "Interp3D");
    _store = pagani::table::make_store({{xs, nx}, {ys, ny}, {zs, nz}, {vs, nx * ny * nz}});
    size_x = nx;
    size_y = ny;
    size_z = nz;
    _dev = _store->dev;
    _host = _store->host.data();
  }

  size_t size_x = 0, size_y = 0, size_z = 0;
  const double* _dev = nullptr;   // [xs | ys | zs | values] in device memory
  const double* _host = nullptr;  // the same on the host
  pagani::table::Store* _store = nullptr;
};

}  // namespace quad
#endif  // CUDA_INTERP_3D_CUH

#endif  // PAGANI_GB300_HELPERS_CUH
