// Compile-only check: functors built on the reference's integrand-side
// helpers (common/cuda/Interp1D.cuh, Interp2D.cuh, Interp3D.cuh and
// common/cuda/cudaArray.cuh's cudaDynamicArray, as test/cuda/common/
// StatefulIntegrand.cu:34-97 uses it) passed to this library's
// pagani::Workspace::integrate.  Built against the reference tree when it is
// present.  This library's own helpers (pagani_gb300_helpers.cuh) sit under
// the same include guards, so the translation unit also includes them, before
// the reference's headers (HELPERS_FIRST=1) or after them (0): whichever comes
// first provides the types and the other adds nothing.
#if HELPERS_FIRST
#include "pagani_gb300_helpers.cuh"
#endif
#include "common/cuda/Interp1D.cuh"
#include "common/cuda/Interp2D.cuh"
#include "common/cuda/Interp3D.cuh"
#include "common/cuda/cudaArray.cuh"
#include "cuda/pagani/quad/GPUquad/Polynomial.cuh"
#if !HELPERS_FIRST
#include "pagani_gb300_helpers.cuh"
#endif
#include "pagani_gb300.cuh"

struct Table1Times {
  quad::Interp1D t;
  __device__ double operator()(double x, double y) const { return t(x) * y; }
};

struct Table2Times {
  quad::Interp2D t;
  __device__ double operator()(double x, double y, double z) const { return t(x, y) * z; }
};

struct Table3 {
  quad::Interp3D t;
  __device__ double operator()(double x, double y, double z) const { return t(x, y, z); }
};

struct Cubic {
  quad::polynomial<4> p;
  __device__ double operator()(double x, double y) const { return p(x) * y; }
};

struct HeapModel {
  gpu::cudaDynamicArray<int> c;
  __device__ double operator()(double x, double y) const { return c[0] + x * c[1] + y * c[2] + x * y * c[3]; }
};

int run_all(const Table1Times& a, const Table2Times& b, const Table3& c, const HeapModel& h, const Cubic& q) {
  pagani::Workspace<double, 2> w2;
  pagani::Workspace<double, 3> w3;
  int s = w2.integrate(a, 1e-3, 0.0, quad::Volume<double, 2>()).status;
  s += w3.integrate(b, 1e-3, 0.0, quad::Volume<double, 3>()).status;
  s += w3.integrate(c, 1e-3, 0.0, quad::Volume<double, 3>()).status;
  s += w2.integrate(h, 1e-3, 0.0, quad::Volume<double, 2>()).status;
  s += w2.integrate(q, 1e-3, 0.0, quad::Volume<double, 2>()).status;
  return s;
}
