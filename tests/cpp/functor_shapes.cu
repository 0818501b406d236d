// Compile-only check: the functor shapes the reference's callers write are
// accepted by the C++ layer (include/pagani_gb300.cuh): __device__ __host__
// operators, non-const operators, float parameters, integral or float
// returns, functors holding device pointers, and template operators.
#include "pagani_gb300.cuh"

struct HostDevice {
  __device__ __host__ double operator()(double x, double y, double z) const { return x * y + z; }
};
struct NonConst {
  double scale = 2.0;
  __device__ double operator()(double x, double y) { return scale * x * y; }
};
struct FloatArgs {
  __device__ float operator()(float x, float y) const { return x + y; }
};
struct IntReturn {
  __device__ int operator()(double x, double y) const { return x < y ? 1 : 0; }
};
struct Pointer {
  const double* table;
  __device__ double operator()(double x, double y) const { return table[0] * x + y; }
};
struct Variadic {
  template <class... X>
  __device__ double operator()(X... xs) const {
    double s = 0.0;
    for (double v : {static_cast<double>(xs)...}) s += v;
    return s;
  }
};

int shapes() {
  Workspace<double, 3> w3;
  Workspace<double, 2> w2;
  Workspace<double, 6> w6;
  quad::Volume<double, 3> v3;
  quad::Volume<double, 2> v2;
  quad::Volume<double, 6> v6;
  int s = 0;
  s += w3.integrate(HostDevice{}, 1e-3, 0.0, v3).status;
  s += w2.integrate(NonConst{}, 1e-3, 0.0, v2).status;
  s += w2.integrate(FloatArgs{}, 1e-3, 0.0, v2).status;
  s += w2.integrate(IntReturn{}, 1e-3, 0.0, v2).status;
  s += w2.integrate(Pointer{nullptr}, 1e-3, 0.0, v2).status;
  s += w6.integrate(Variadic{}, 1e-3, 0.0, v6).status;
  s += cuda_mcubes::integrate<HostDevice, 3>(HostDevice{}, 1e-3, 0.0, 1e5, &v3).status;
  quad::mcubes m;
  s += m.integrate(HostDevice{}, 0.0, 1e-3, &v3).status;
  return s;
}
