// Stateful functors of the shapes the reference's integrand-side helpers give
// (common/cuda/cudaArray.cuh's cudaDynamicArray, common/cuda/Interp1D.cuh,
// Interp2D.cuh; test/cuda/common/StatefulIntegrand.cu:34-97), run through the
// C++ layer's Workspace::integrate.  The helper types here are this test's
// own: an array in managed memory whose copy constructor makes a deep copy
// (managed memory on the host, the heap on the device), so the functor is not
// trivially copyable and reaches the kernel as a managed copy; and 1-D / 2-D
// piecewise-linear tables with an interval search.  Each integral has an
// exact value: a polynomial the rule integrates exactly, or the trapezoid sum
// of the tabulated values, which is the integral of the interpolant.
// Prints one line per case and exits non-zero on any failure.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "pagani_gb300.cuh"

template <class T>
class ManagedArray {
 public:
  ManagedArray() = default;
  ManagedArray(const T* v, size_t n) : n_(n) {
    p_ = alloc(n);
    std::memcpy(p_, v, n * sizeof(T));
  }
  __host__ __device__ ManagedArray(const ManagedArray& o) : n_(o.n_) {
#ifdef __CUDA_ARCH__
    p_ = new T[o.n_];
#else
    p_ = alloc(o.n_);
    ++copies;
#endif
    for (size_t i = 0; i < n_; ++i) p_[i] = o.p_[i];
  }
  ManagedArray& operator=(const ManagedArray&) = delete;
  __host__ __device__ ~ManagedArray() {
#ifndef __CUDA_ARCH__
    if (p_) cudaFree(p_);
#else
    delete[] p_;
#endif
  }
  __host__ __device__ T operator[](size_t i) const { return p_[i]; }
  __host__ __device__ size_t size() const { return n_; }
  static int copies;  // host-side copies made (the functor's managed copy among them)

 private:
  static T* alloc(size_t n) {
    void* q = nullptr;
    if (cudaMallocManaged(&q, n * sizeof(T)) != cudaSuccess) throw std::bad_alloc();
    return static_cast<T*>(q);
  }
  T* p_ = nullptr;
  size_t n_ = 0;
};
template <class T>
int ManagedArray<T>::copies = 0;

// Index i of the interval [xs[i], xs[i+1]] holding x (clamped to the table).
__host__ __device__ inline size_t interval(const ManagedArray<double>& xs, double x) {
  size_t lo = 0, hi = xs.size() - 1;
  while (hi - lo > 1) {
    const size_t mid = (lo + hi) / 2;
    if (x < xs[mid])
      hi = mid;
    else
      lo = mid;
  }
  return lo;
}

struct LinearTable {
  ManagedArray<double> xs, zs;
  __host__ __device__ double operator()(double x) const {
    const size_t i = interval(xs, x);
    const double t = (x - xs[i]) / (xs[i + 1] - xs[i]);
    return zs[i] + t * (zs[i + 1] - zs[i]);
  }
};

struct BilinearTable {
  ManagedArray<double> xs, ys, zs;  // zs[j * nx + i] = g(xs[i], ys[j])
  __host__ __device__ double operator()(double x, double y) const {
    const size_t nx = xs.size();
    const size_t i = interval(xs, x), j = interval(ys, y);
    const double tx = (x - xs[i]) / (xs[i + 1] - xs[i]);
    const double ty = (y - ys[j]) / (ys[j + 1] - ys[j]);
    const double z0 = zs[j * nx + i] + tx * (zs[j * nx + i + 1] - zs[j * nx + i]);
    const double z1 = zs[(j + 1) * nx + i] + tx * (zs[(j + 1) * nx + i + 1] - zs[(j + 1) * nx + i]);
    return z0 + ty * (z1 - z0);
  }
};

// a0 + a1 x + a2 y + a3 x y with the coefficients on the heap: the reference's
// ToyIntegrandWithHeapModel (StatefulIntegrand.cu:34-62).
struct HeapModel {
  ManagedArray<int> c;
  __device__ double operator()(double x, double y) const { return c[0] + x * c[1] + y * c[2] + x * y * c[3]; }
};

struct Interp1Times {
  LinearTable t;
  __device__ double operator()(double x, double y, double z) const { return t(x) * exp(-y) * z; }
};

struct Interp2Times {
  BilinearTable t;
  __device__ double operator()(double x, double y, double z, double w) const { return t(x, y) * (z + w); }
};

static double trapezoid(const std::vector<double>& x, const std::vector<double>& z) {
  double s = 0.0;
  for (size_t i = 0; i + 1 < x.size(); ++i) s += 0.5 * (z[i] + z[i + 1]) * (x[i + 1] - x[i]);
  return s;
}

static int failures = 0;

static void check(const char* name, const pagani::integration_result& r, double exact, double tol) {
  const double rel = std::fabs(r.estimate - exact) / std::fabs(exact);
  const bool ok = r.status == 0 && rel <= tol;
  std::printf("%s %s %.17g exact %.17g rel %.3g status %d nregions %zu\n", ok ? "PASS" : "FAIL", name, r.estimate,
              exact, rel, r.status, r.nregions);
  if (!ok) ++failures;
}

int main() {
  {
    const int c[5] = {5, 4, 3, 2, 1};
    HeapModel f{ManagedArray<int>(c, 5)};
    const int before = ManagedArray<int>::copies;
    pagani::Workspace<double, 2> ws;
    const auto r = ws.integrate(f, 1e-10, 0.0, quad::Volume<double, 2>());
    // 5 + 4/2 + 3/2 + 2/4: the degree-7 rule integrates the bilinear form exactly
    check("heap_model2", r, 9.0, 1e-14);
    const bool copied = ManagedArray<int>::copies > before;
    std::printf("%s heap_model2_managed_copy %d\n", copied ? "PASS" : "FAIL", ManagedArray<int>::copies - before);
    if (!copied) ++failures;
  }
  {
    std::vector<double> xs(11), zs(11);
    for (int i = 0; i <= 10; ++i) {
      xs[i] = 0.1 * i;
      zs[i] = xs[i] * xs[i];
    }
    Interp1Times f{LinearTable{ManagedArray<double>(xs.data(), xs.size()), ManagedArray<double>(zs.data(), zs.size())}};
    pagani::Workspace<double, 3> ws;
    const auto r = ws.integrate(f, 1e-6, 0.0, quad::Volume<double, 3>());
    check("interp1d_3", r, trapezoid(xs, zs) * (1.0 - std::exp(-1.0)) * 0.5, 1e-6);
  }
  {
    std::vector<double> xs(5), ys(7), zs(5 * 7), zy(7);
    for (int i = 0; i < 5; ++i) xs[i] = 0.25 * i;
    for (int j = 0; j < 7; ++j) {
      ys[j] = j / 6.0;
      zy[j] = ys[j] * ys[j];
    }
    for (int j = 0; j < 7; ++j)
      for (int i = 0; i < 5; ++i) zs[j * 5 + i] = (1.0 + xs[i]) * zy[j];
    Interp2Times f{BilinearTable{ManagedArray<double>(xs.data(), 5), ManagedArray<double>(ys.data(), 7),
                                 ManagedArray<double>(zs.data(), zs.size())}};
    pagani::Workspace<double, 4> ws;
    const auto r = ws.integrate(f, 1e-6, 0.0, quad::Volume<double, 4>());
    // (1 + x) is linear, so its trapezoid sum is exact (1.5); (z + w) integrates to 1
    check("interp2d_4", r, 1.5 * trapezoid(ys, zy), 1e-6);
  }
  std::printf("%s %d failures\n", failures ? "FAIL" : "DONE", failures);
  return failures ? 1 : 0;
}
