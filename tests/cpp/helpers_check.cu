// The integrand-side helpers of include/pagani_gb300_helpers.cuh on the GPU.
//
// 1. The reference's own known answers for its helpers
//    (test/cuda/common/Interpolation1D.cu, Interpolation2D.cu,
//    Interpolation3D.cu, cudaDynamicArray.cu, StatefulIntegrand.cu), evaluated
//    in kernels as those tests do.
// 2. Each table evaluated on the device and on the host at seeded points
//    (knots, interior, outside): bit-identical, and within 1e-14 (relative,
//    or absolute below 1) of a plain restatement of the reference's formulas.
// 3. Functors holding the helpers through Workspace::integrate, against exact
//    integrals: a polynomial the rule integrates exactly, or the trapezoid sum
//    of the tabulated values (the integral of the interpolant, which the rule
//    reaches once the regions follow the knots).
// 4. Copies of a table share its device store: copying a 32 MB table leaves
//    the device's free memory unchanged.
// Prints one line per case and exits non-zero on any failure.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <sstream>
#include <vector>

#include "pagani_gb300.cuh"
#include "pagani_gb300_helpers.cuh"

static int failures = 0;

static void report(const char* name, bool ok, const char* fmt = "", double a = 0, double b = 0) {
  std::printf("%s %s ", ok ? "PASS" : "FAIL", name);
  std::printf(fmt, a, b);
  std::printf("\n");
  if (!ok) ++failures;
}

static double* managed(size_t n) {
  void* p = nullptr;
  if (cudaMallocManaged(&p, n * sizeof(double)) != cudaSuccess) {
    std::printf("FAIL cudaMallocManaged\n");
    std::exit(1);
  }
  return static_cast<double*>(p);
}

// ---------------------------------------------------------------------------
// Kernels of the reference's helper tests: the table passed by value.
__global__ void eval1(quad::Interp1D f, size_t n, const double* x, double* out) {
  for (size_t i = 0; i < n; ++i) out[i] = f(x[i]);
}
__global__ void eval2(quad::Interp2D f, size_t n, const double* x, const double* y, double* out, int clamp) {
  for (size_t i = 0; i < n; ++i) out[i] = clamp ? f.clamp(x[i], y[i]) : f(x[i], y[i]);
}
__global__ void eval3(quad::Interp3D f, size_t n, const double* x, const double* y, const double* z, double* out,
                      int clamp) {
  for (size_t i = 0; i < n; ++i) out[i] = clamp ? f.clamp(x[i], y[i], z[i]) : f(x[i], y[i], z[i]);
}
template <class A>
__global__ void set_vals_at_indices(A array, A indices, A vals) {
  for (size_t i = 0; i < indices.size(); ++i) array[indices[i]] = vals[i];
}
template <class A>
__global__ void set_vals_through_pointer(int* array, A indices, A vals) {
  for (size_t i = 0; i < indices.size(); ++i) array[indices[i]] = vals[i];
}
template <class T>
__global__ void call_at_2_3(const T* t, double* out) {
  *out = (*t)(2., 3.);
}
template <size_t O>
__global__ void eval_poly(quad::polynomial<O> p, size_t n, const double* x, double* out) {
  for (size_t i = 0; i < n; ++i) out[i] = p(x[i]);
}
// A copy made in device code owns a device-heap buffer; it is changed and freed there.
__global__ void device_copy(gpu::cudaDynamicArray<int> a, int* out) {
  gpu::cudaDynamicArray<int> b(a);
  b[0] = 100;
  out[0] = b[0];
  out[1] = a[0];
  out[2] = (int)b.size();
}

// The reference's stateful integrands (StatefulIntegrand.cu:34-97).
struct ToyModelWithHeapArray {
  ToyModelWithHeapArray(int const* d, size_t s) : data(d, s) {}
  ToyModelWithHeapArray() = default;
  __host__ __device__ double operator()(double x, double y) const {
    return data[0] + x * data[1] + y * data[2] + x * y * data[3];
  }
  gpu::cudaDynamicArray<int> data;
};
struct ToyIntegrandWithHeapModel {
  explicit ToyIntegrandWithHeapModel(int* const modeldata, size_t s) : model(modeldata, s) {}
  __host__ __device__ double operator()(double x, double y) const { return model(x, y); }
  double true_value = 34.0;
  ToyModelWithHeapArray model;
};
struct ToyModel {
  explicit ToyModel(int const* d) { data.Initialize(d); }
  ToyModel() = default;
  __host__ __device__ double operator()(double x, double y) const {
    return data[0] + x * data[1] + y * data[2] + x * y * data[3];
  }
  gpu::cudaArray<int, 5> data;
};
struct ToyIntegrand {
  explicit ToyIntegrand(std::array<int, 5> const& modeldata) : model(modeldata.data()) {}
  __host__ __device__ double operator()(double x, double y) const { return model(x, y); }
  double true_value = 34.0;
  ToyModel model;
};

// Runs f(2, 3) in a kernel from a copy in managed memory, the reference's
// toy_integration_algorithm (StatefulIntegrand.cu:99-120).
template <class T>
static double toy_integration(const T& on_host) {
  void* p = nullptr;
  cudaMallocManaged(&p, sizeof(T));
  T* t = new (p) T(on_host);
  double* r = managed(1);
  call_at_2_3<<<1, 1>>>(t, r);
  cudaDeviceSynchronize();
  const double v = *r;
  t->~T();
  cudaFree(p);
  cudaFree(r);
  return v;
}

// ---------------------------------------------------------------------------
// The reference's formulas, restated plainly: interval by bisection, then
// (y0 (x1 - x) + y1 (x - x0)) / (x1 - x0) per axis.
static size_t find_interval(const std::vector<double>& a, double v) {
  size_t lo = 0, hi = a.size() - 1;
  while (hi - lo > 1) {
    const size_t mid = (lo + hi) / 2;
    (v < a[mid] ? hi : lo) = mid;
  }
  return lo;
}
static double lin(double y0, double y1, double x0, double x1, double x) {
  return (y0 * (x1 - x) + y1 * (x - x0)) / (x1 - x0);
}

static double trapezoid(const std::vector<double>& x, const std::vector<double>& z) {
  double s = 0.0;
  for (size_t i = 0; i + 1 < x.size(); ++i) s += 0.5 * (z[i] + z[i + 1]) * (x[i + 1] - x[i]);
  return s;
}

static void check_integral(const char* name, const numint::integration_result& r, double exact, double tol) {
  const double rel = std::fabs(r.estimate - exact) / std::fabs(exact);
  std::printf("%s %s %.17g exact %.17g rel %.3g status %d nregions %zu\n",
              (r.status == 0 && rel <= tol) ? "PASS" : "FAIL", name, r.estimate, exact, rel, r.status,
              (size_t)r.nregions);
  if (!(r.status == 0 && rel <= tol)) ++failures;
}

// Functors for the integrals.
struct Interp1Times {
  quad::Interp1D t;
  __device__ double operator()(double x, double y, double z) const { return t(x) * exp(-y) * z; }
};
struct Interp2Times {
  quad::Interp2D t;
  __device__ double operator()(double x, double y, double z, double w) const { return t(x, y) * (z + w); }
};
struct Interp3Plain {
  quad::Interp3D t;
  __device__ double operator()(double x, double y, double z) const { return t(x, y, z); }
};
struct PolyTimesArray {
  quad::polynomial<4> p;
  gpu::cudaDynamicArray<double> c;
  __device__ double operator()(double x, double y) const { return p(x) * (c[0] + c[1] * y); }
};

// ---------------------------------------------------------------------------
static void reference_known_answers() {
  // Interpolation1D.cu: exact at knots; x^2 tabulated on 1..5 at four points (1e-4).
  {
    std::array<double, 9> xs = {1., 2., 3., 4., 5., 6, 7., 8., 9.};
    std::array<double, 9> ys;
    for (size_t i = 0; i < 9; ++i) ys[i] = 2 * xs[i] * (3 - xs[i]) * std::cos(xs[i]);
    quad::Interp1D f(xs, ys);
    double* in = managed(9);
    double* out = managed(9);
    for (size_t i = 0; i < 9; ++i) in[i] = xs[i];
    eval1<<<1, 1>>>(f, 9, in, out);
    cudaDeviceSynchronize();
    bool ok = true;
    for (size_t i = 0; i < 9; ++i) ok = ok && out[i] == ys[i];
    report("ref_interp1d_exact_at_knots", ok);
    std::array<double, 5> qx = {1., 2., 3., 4., 5.}, qy = {1., 4., 9., 16., 25.};
    quad::Interp1D g(qx, qy);
    const double pts[4] = {1.41421, 2.41421, 3.41421, 4.41421};
    const double want[4] = {2.24263, 6.07105, 11.89947, 19.72789};
    for (int i = 0; i < 4; ++i) in[i] = pts[i];
    eval1<<<1, 1>>>(g, 4, in, out);
    cudaDeviceSynchronize();
    ok = true;
    for (int i = 0; i < 4; ++i) ok = ok && std::fabs(out[i] - want[i]) <= 1e-4 * want[i];
    report("ref_interp1d_quadratic", ok);
    cudaFree(in);
    cudaFree(out);
  }
  // Interpolation2D.cu: 3xy + 2x + 4y on {1,2,3} x {4,5}; clamping; 2x + 3y - 5.
  {
    std::array<double, 3> xs = {1., 2., 3.};
    std::array<double, 2> ys = {4., 5.};
    std::array<double, 6> zs;
    auto fxy = [](double x, double y) { return 3 * x * y + 2 * x + 4 * y; };
    for (size_t i = 0; i < 3; ++i)
      for (size_t j = 0; j < 2; ++j) zs[j * 3 + i] = fxy(xs[i], ys[j]);
    quad::Interp2D f(xs, ys, zs);
    double* x = managed(32);
    double* y = managed(32);
    double* out = managed(32);
    x[0] = 2.5, y[0] = 4.5;
    eval2<<<1, 1>>>(f, 1, x, y, out, 0);
    cudaDeviceSynchronize();
    report("ref_interp2d_value", out[0] == 56.75, "%.17g", out[0]);
    const double cl[16][2] = {{0., 4.5}, {1., 4.5}, {4., 4.5}, {3., 4.5}, {2., 3.}, {2., 4.}, {2., 5.5}, {2., 5.},
                              {0., 0.},  {1., 4.},  {4., 3.},  {3., 4.},  {0., 6.}, {1., 5.}, {4., 6.},  {3., 5.}};
    for (int i = 0; i < 16; ++i) x[i] = cl[i][0], y[i] = cl[i][1];
    eval2<<<1, 1>>>(f, 16, x, y, out, 1);
    cudaDeviceSynchronize();
    bool ok = true;
    for (int i = 0; i < 16; i += 2) ok = ok && out[i] == out[i + 1];
    report("ref_interp2d_clamp", ok);
    int k = 0;
    for (size_t i = 0; i < 3; ++i)
      for (size_t j = 0; j < 2; ++j, ++k) x[k] = xs[i], y[k] = ys[j];
    eval2<<<1, 1>>>(f, 6, x, y, out, 0);
    cudaDeviceSynchronize();
    ok = true;
    k = 0;
    for (size_t i = 0; i < 3; ++i)
      for (size_t j = 0; j < 2; ++j, ++k) ok = ok && out[k] == zs[j * 3 + i];
    report("ref_interp2d_exact_at_knots", ok);
    std::array<double, 3> bx = {1., 2., 3.};
    std::array<double, 4> by = {1., 2., 3., 4.};
    std::array<double, 12> bz;
    for (size_t i = 0; i < 3; ++i)
      for (size_t j = 0; j < 4; ++j) bz[j * 3 + i] = 2 * bx[i] + 3 * by[j] - 5;
    quad::Interp2D g(bx, by, bz);
    x[0] = 2.5, y[0] = 1.5;
    eval2<<<1, 1>>>(g, 1, x, y, out, 0);
    cudaDeviceSynchronize();
    report("ref_interp2d_bilinear", out[0] == 4.5, "%.17g", out[0]);
    cudaFree(x);
    cudaFree(y);
    cudaFree(out);
  }
  // Interpolation3D.cu: linear (1e-15) and quadratic (1e-2) on {1,2,3} x {4,5} x {4..7}; clamping.
  {
    std::array<double, 3> xs = {1., 2., 3.};
    std::array<double, 2> ys = {4., 5.};
    std::array<double, 4> zs = {4., 5., 6., 7.};
    std::array<double, 24> lv, qv;
    auto flin = [](double x, double y, double z) { return 2 * x + 3 * y + 4 * z; };
    auto fq = [](double x, double y, double z) {
      return 2 * x * x + 3 * y * y + 4 * z * z + 5 * x + 6 * y + 7 * z + x * y - x * z + z * y;
    };
    for (size_t k = 0; k < 4; ++k)
      for (size_t i = 0; i < 3; ++i)
        for (size_t j = 0; j < 2; ++j) {
          lv[i + 3 * j + 6 * k] = flin(xs[i], ys[j], zs[k]);
          qv[i + 3 * j + 6 * k] = fq(xs[i], ys[j], zs[k]);
        }
    quad::Interp3D fl(xs, ys, zs, lv), fqi(xs, ys, zs, qv);
    double* x = managed(16);
    double* y = managed(16);
    double* z = managed(16);
    double* out = managed(16);
    x[0] = 2.3, y[0] = 4.3, z[0] = 6.3;
    eval3<<<1, 1>>>(fl, 1, x, y, z, out, 0);
    cudaDeviceSynchronize();
    const double tl = flin(2.3, 4.3, 6.3);
    report("ref_interp3d_linear", std::fabs(out[0] - tl) <= 1e-15 * tl, "%.17g vs %.17g", out[0], tl);
    x[0] = 2.1, y[0] = 4.9, z[0] = 6.1;
    eval3<<<1, 1>>>(fqi, 1, x, y, z, out, 0);
    cudaDeviceSynchronize();
    const double tq = fq(2.1, 4.9, 6.1);
    report("ref_interp3d_quadratic", std::fabs(out[0] - tq) <= 1e-2 * tq, "%.17g vs %.17g", out[0], tq);
    const double cl[16][3] = {{0., 4.5, 6.3}, {1., 4.5, 6.3}, {4., 4.5, 6.3},   {3., 4.5, 6.3},
                              {2., 3., 6.3},  {2., 4., 6.3},  {2., 5.5, 6.3},   {2., 5., 6.3},
                              {1.1, 4.2, 3.1}, {1.1, 4.2, 4.}, {1.1, 4.2, 7.4}, {1.1, 4.2, 7.},
                              {0., 3.1, 3.1}, {1., 4., 4.},   {3.5, 5.6, 7.3},  {3., 5., 7.}};
    for (int i = 0; i < 16; ++i) x[i] = cl[i][0], y[i] = cl[i][1], z[i] = cl[i][2];
    eval3<<<1, 1>>>(fl, 16, x, y, z, out, 1);
    cudaDeviceSynchronize();
    bool ok = true;
    for (int i = 0; i < 16; i += 2) ok = ok && out[i] == out[i + 1];
    report("ref_interp3d_clamp", ok);
    cudaFree(x);
    cudaFree(y);
    cudaFree(z);
    cudaFree(out);
  }
  // cudaDynamicArray.cu: host access, the pointer constructor, deep copies to a
  // kernel, edits through data() seen on the host, the copy constructor.
  {
    using int_array = gpu::cudaDynamicArray<int>;
    int_array array;
    array.Reserve(5);
    for (int i = 0; i < (int)array.size(); ++i) array[i] = i;
    bool ok = array[0] == 0 && array[4] == 4;
    std::array<int, 3> indices = {1, 3, 4}, vals = {11, 33, 44};
    int_array d_indices(indices.data(), indices.size()), d_vals(vals.data(), vals.size());
    ok = ok && d_indices[0] == 1 && d_indices[1] == 3 && d_indices[2] == 4 && d_vals[0] == 11 && d_vals[2] == 44;
    set_vals_at_indices<int_array><<<1, 1>>>(array, d_indices, d_vals);
    cudaDeviceSynchronize();
    const bool deep = array[1] != 11 && array[3] != 33 && array[4] != 44;
    set_vals_through_pointer<int_array><<<1, 1>>>(array.data(), d_indices, d_vals);
    cudaDeviceSynchronize();
    const bool shared = array[1] == 11 && array[3] == 33 && array[4] == 44;
    int_array copy(array);
    bool same = true;
    for (int i = 0; i < (int)array.size(); ++i) same = same && copy[i] == array[i];
    copy[0] = -1;
    report("ref_dynamic_array", ok && deep && shared && same && array[0] == 0);
    int* dout = nullptr;
    cudaMallocManaged(&dout, 3 * sizeof(int));
    device_copy<<<1, 1>>>(array, dout);
    const cudaError_t e = cudaDeviceSynchronize();
    report("dynamic_array_device_copy", e == cudaSuccess && dout[0] == 100 && dout[1] == 0 && dout[2] == 5);
    cudaFree(dout);
  }
  // StatefulIntegrand.cu: state in a cudaArray and in a cudaDynamicArray, f(2, 3) = 34.
  {
    std::array<int, 5> attributes{5, 4, 3, 2, 1};
    ToyIntegrand a(attributes);
    const double ra = toy_integration(a);
    report("ref_stateful_array", ra == 34.0 && ra == a.true_value, "%.17g", ra);
    ToyIntegrandWithHeapModel b(attributes.data(), attributes.size());
    const double rb = toy_integration(b);
    report("ref_stateful_dynamic_array", rb == 34.0 && rb == b.true_value, "%.17g", rb);
  }
}

// ---------------------------------------------------------------------------
static void device_host_and_restatement() {
  std::mt19937_64 gen(20261204);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  // knots: uneven spacing
  auto axis = [&](size_t n, double lo, double hi) {
    std::vector<double> a(n);
    double s = 0.0;
    for (size_t i = 0; i < n; ++i) a[i] = (s += 0.2 + U(gen));
    for (size_t i = 0; i < n; ++i) a[i] = lo + (hi - lo) * (a[i] - a[0]) / (a[n - 1] - a[0]);
    return a;
  };
  const size_t npts = 4096;
  double* px = managed(npts);
  double* py = managed(npts);
  double* pz = managed(npts);
  double* out = managed(npts);
  auto points = [&](const std::vector<double>& a, double* p) {
    for (size_t i = 0; i < npts; ++i) {
      const int kind = i % 4;
      if (kind == 0)
        p[i] = a[gen() % a.size()];  // a knot
      else if (kind == 3)
        p[i] = a.front() + (a.back() - a.front()) * (1.4 * U(gen) - 0.2);  // may lie outside
      else
        p[i] = a.front() + (a.back() - a.front()) * U(gen);
    }
  };
  // 1-D
  {
    const std::vector<double> xs = axis(37, -2.0, 3.0);
    std::vector<double> zs(xs.size());
    for (size_t i = 0; i < xs.size(); ++i) zs[i] = std::sin(3 * xs[i]) + 0.1 * xs[i] * xs[i];
    quad::Interp1D f(xs, zs);
    points(xs, px);
    eval1<<<1, 1>>>(f, npts, px, out);
    cudaDeviceSynchronize();
    bool same = true;
    double worst = 0.0;
    for (size_t i = 0; i < npts; ++i) {
      const double h = f(px[i]);
      same = same && std::memcmp(&out[i], &h, 8) == 0;
      const size_t k = find_interval(xs, px[i]);
      const double r = lin(zs[k], zs[k + 1], xs[k], xs[k + 1], px[i]);
      worst = std::fmax(worst, std::fabs(out[i] - r) / std::fmax(1.0, std::fabs(r)));
    }
    report("interp1d_device_equals_host", same);
    report("interp1d_vs_reference_formula", worst <= 1e-14, "max diff %.3g", worst);
  }
  // 2-D
  {
    const std::vector<double> xs = axis(23, 0.0, 1.0), ys = axis(17, -1.0, 4.0);
    std::vector<double> zs(xs.size() * ys.size());
    for (size_t j = 0; j < ys.size(); ++j)
      for (size_t i = 0; i < xs.size(); ++i) zs[j * xs.size() + i] = std::cos(xs[i] * ys[j]) + xs[i];
    quad::Interp2D f(xs, ys, zs);
    points(xs, px);
    points(ys, py);
    eval2<<<1, 1>>>(f, npts, px, py, out, 0);
    cudaDeviceSynchronize();
    bool same = true;
    double worst = 0.0;
    const size_t nx = xs.size();
    for (size_t q = 0; q < npts; ++q) {
      const double h = f(px[q], py[q]);
      same = same && std::memcmp(&out[q], &h, 8) == 0;
      const size_t i = find_interval(xs, px[q]), j = find_interval(ys, py[q]);
      const double a = lin(zs[j * nx + i], zs[j * nx + i + 1], xs[i], xs[i + 1], px[q]);
      const double b = lin(zs[(j + 1) * nx + i], zs[(j + 1) * nx + i + 1], xs[i], xs[i + 1], px[q]);
      const double r = lin(a, b, ys[j], ys[j + 1], py[q]);
      worst = std::fmax(worst, std::fabs(out[q] - r) / std::fmax(1.0, std::fabs(r)));
    }
    report("interp2d_device_equals_host", same);
    report("interp2d_vs_reference_formula", worst <= 1e-14, "max diff %.3g", worst);
  }
  // 3-D
  {
    const std::vector<double> xs = axis(9, 0.0, 2.0), ys = axis(11, 1.0, 2.0), zs = axis(7, -3.0, 0.0);
    const size_t nx = xs.size(), ny = ys.size(), nz = zs.size();
    std::vector<double> vs(nx * ny * nz);
    for (size_t k = 0; k < nz; ++k)
      for (size_t j = 0; j < ny; ++j)
        for (size_t i = 0; i < nx; ++i) vs[i + nx * j + nx * ny * k] = std::exp(0.3 * zs[k]) * (xs[i] - ys[j]);
    quad::Interp3D f(xs, ys, zs, vs);
    points(xs, px);
    points(ys, py);
    points(zs, pz);
    eval3<<<1, 1>>>(f, npts, px, py, pz, out, 0);
    cudaDeviceSynchronize();
    bool same = true;
    double worst = 0.0;
    for (size_t q = 0; q < npts; ++q) {
      const double h = f(px[q], py[q], pz[q]);
      same = same && std::memcmp(&out[q], &h, 8) == 0;
      const size_t i = find_interval(xs, px[q]), j = find_interval(ys, py[q]), k = find_interval(zs, pz[q]);
      auto v = [&](size_t a, size_t b, size_t c) { return vs[a + nx * b + nx * ny * c]; };
      const double c00 = lin(v(i, j, k), v(i + 1, j, k), xs[i], xs[i + 1], px[q]);
      const double c01 = lin(v(i, j, k + 1), v(i + 1, j, k + 1), xs[i], xs[i + 1], px[q]);
      const double c10 = lin(v(i, j + 1, k), v(i + 1, j + 1, k), xs[i], xs[i + 1], px[q]);
      const double c11 = lin(v(i, j + 1, k + 1), v(i + 1, j + 1, k + 1), xs[i], xs[i + 1], px[q]);
      const double c0 = lin(c00, c10, ys[j], ys[j + 1], py[q]);
      const double c1 = lin(c01, c11, ys[j], ys[j + 1], py[q]);
      const double r = lin(c0, c1, zs[k], zs[k + 1], pz[q]);
      worst = std::fmax(worst, std::fabs(out[q] - r) / std::fmax(1.0, std::fabs(r)));
    }
    report("interp3d_device_equals_host", same);
    report("interp3d_vs_reference_formula", worst <= 1e-14, "max diff %.3g", worst);
  }
  // polynomial: device equals host; against the plain Horner sum.
  {
    gpu::cudaArray<double, 6> c;
    const double cs[6] = {0.5, -1.25, 2.0, 0.75, -3.0, 1.5};
    c.Initialize(cs);
    quad::polynomial<6> p(c);
    for (size_t i = 0; i < 256; ++i) px[i] = -2.0 + 4.0 * U(gen);
    eval_poly<<<1, 1>>>(p, 256, px, out);
    cudaDeviceSynchronize();
    bool same = true;
    double worst = 0.0;
    for (size_t i = 0; i < 256; ++i) {
      const double h = p(px[i]);
      same = same && std::memcmp(&out[i], &h, 8) == 0;
      double r = 0.0;
      for (int k = 0; k < 6; ++k) r = cs[k] + px[i] * r;
      worst = std::fmax(worst, std::fabs(out[i] - r) / std::fmax(1.0, std::fabs(r)));
    }
    report("polynomial_device_equals_host", same);
    report("polynomial_vs_horner", worst <= 1e-14, "max diff %.3g", worst);
  }
  // Text input: the operator>> forms.
  {
    std::istringstream in1("0 0.5 1\n1 3 2\n");
    quad::Interp1D f1;
    in1 >> f1;
    std::istringstream in2("0 1\n0 2\n1 2 3 4\n");
    quad::Interp2D f2;
    in2 >> f2;
    report("interp_stream_input", f1(0.25) == 2.0 && f2(0.5, 1.0) == 2.5, "%.17g %.17g", f1(0.25), f2(0.5, 1.0));
  }
  // Bad tables are rejected; an empty table gives NaN.
  {
    bool threw = false;
    try {
      const double x[3] = {0.0, 1.0, 1.0}, z[3] = {0, 0, 0};
      quad::Interp1D bad(x, z, 3);
    } catch (const std::invalid_argument&) {
      threw = true;
    }
    quad::Interp1D empty;
    report("interp_rejects_unordered_axis", threw && std::isnan(empty(0.5)));
  }
  cudaFree(px);
  cudaFree(py);
  cudaFree(pz);
  cudaFree(out);
}

// ---------------------------------------------------------------------------
static void integrals() {
  {
    std::vector<double> xs(11), zs(11);
    for (int i = 0; i <= 10; ++i) {
      xs[i] = 0.1 * i;
      zs[i] = xs[i] * xs[i];
    }
    Interp1Times f{quad::Interp1D(xs, zs)};
    pagani::Workspace<double, 3> ws;
    const auto r = ws.integrate(f, 1e-6, 0.0, quad::Volume<double, 3>());
    check_integral("interp1d_3", r, trapezoid(xs, zs) * (1.0 - std::exp(-1.0)) * 0.5, 1e-6);
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
    Interp2Times f{quad::Interp2D(xs, ys, zs)};
    pagani::Workspace<double, 4> ws;
    const auto r = ws.integrate(f, 1e-6, 0.0, quad::Volume<double, 4>());
    // (1 + x) is linear, so its trapezoid sum is exact (1.5); (z + w) integrates to 1
    check_integral("interp2d_4", r, 1.5 * trapezoid(ys, zy), 1e-6);
  }
  {
    // v = (1 + x)(2 - y) z^2 on a 3 x 3 x 9 grid of [0,1]^3: trilinear in x and y
    // (exact), the z^2 factor's trapezoid sum.
    std::vector<double> xs = {0.0, 0.5, 1.0}, ys = {0.0, 0.5, 1.0}, zs(9), vz(9), vs(3 * 3 * 9);
    for (int k = 0; k < 9; ++k) {
      zs[k] = k / 8.0;
      vz[k] = zs[k] * zs[k];
    }
    for (int k = 0; k < 9; ++k)
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) vs[i + 3 * j + 9 * k] = (1.0 + xs[i]) * (2.0 - ys[j]) * vz[k];
    Interp3Plain f{quad::Interp3D(xs, ys, zs, vs)};
    pagani::Workspace<double, 3> ws;
    const auto r = ws.integrate(f, 1e-7, 0.0, quad::Volume<double, 3>());
    check_integral("interp3d_3", r, 1.5 * 1.5 * trapezoid(zs, vz), 1e-7);
  }
  {
    // p(x) = x^3 - 2x^2 + 0.5x + 1, times (c0 + c1 y) with c in a dynamic array:
    // the degree-9 rule integrates it exactly.
    gpu::cudaArray<double, 4> c;
    const double cs[4] = {1.0, -2.0, 0.5, 1.0};
    c.Initialize(cs);
    const double cy[2] = {2.0, 3.0};
    PolyTimesArray f{quad::polynomial<4>(c), gpu::cudaDynamicArray<double>(cy, 2)};
    pagani::Workspace<double, 2> ws;
    const auto r = ws.integrate(f, 1e-10, 0.0, quad::Volume<double, 2>());
    const double ip = 0.25 - 2.0 / 3.0 + 0.25 + 1.0;  // integral of p over [0,1]
    check_integral("polynomial_dynamic_array_2", r, ip * (2.0 + 1.5), 1e-13);
  }
}

// A 32 MB table copied four times and handed to a functor copy: the device's
// free memory does not change (the copies share the store).
static void shared_store() {
  const size_t n = 2u << 20;
  std::vector<double> xs(n), zs(n);
  for (size_t i = 0; i < n; ++i) xs[i] = (double)i, zs[i] = 0.5 * (double)i;
  quad::Interp1D t(xs, zs);
  cudaDeviceSynchronize();
  size_t free0 = 0, total = 0, free1 = 0;
  cudaMemGetInfo(&free0, &total);
  {
    quad::Interp1D a(t), b(t), c = a, d;
    d = b;
    Interp1Times f{d};
    Interp1Times g(f);
    cudaMemGetInfo(&free1, &total);
  }
  report("interp_copies_share_device_store", free1 == free0, "free before %.0f after %.0f", (double)free0,
         (double)free1);
}

int main() {
  reference_known_answers();
  device_host_and_restatement();
  integrals();
  shared_store();
  std::printf("%s %d failures\n", failures ? "FAIL" : "DONE", failures);
  return failures ? 1 : 0;
}
