// Error behaviour of include/pagani_gb300_helpers.cuh that needs no GPU:
// tables with fewer than two knots, unordered axes or mismatched sizes throw
// std::invalid_argument before any allocation; without a CUDA device, a table
// or a dynamic array throws std::bad_alloc (the device or managed allocation
// fails) instead of crashing; default-constructed tables evaluate to NaN on
// the host.  Prints one line per case and exits non-zero on any failure.
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "pagani_gb300_helpers.cuh"

static int failures = 0;

template <class F>
static void expect_throw(const char* name, F&& f, bool want_invalid) {
  int got = 0;  // 1 invalid_argument, 2 bad_alloc, 3 other, 0 none
  try {
    f();
  } catch (const std::invalid_argument&) {
    got = 1;
  } catch (const std::bad_alloc&) {
    got = 2;
  } catch (...) {
    got = 3;
  }
  const bool ok = got == (want_invalid ? 1 : 2);
  std::printf("%s %s (caught %d)\n", ok ? "PASS" : "FAIL", name, got);
  if (!ok) ++failures;
}

int main() {
  const std::vector<double> one = {0.0}, two = {0.0, 1.0}, flat = {0.0, 0.0}, down = {1.0, 0.0};
  expect_throw("interp1d_one_knot", [&] { quad::Interp1D t(one, one); }, true);
  expect_throw("interp1d_repeated_knot", [&] { quad::Interp1D t(flat, two); }, true);
  expect_throw("interp1d_decreasing", [&] { quad::Interp1D t(down, two); }, true);
  expect_throw("interp1d_size_mismatch", [&] { quad::Interp1D t(two, std::vector<double>{1.0, 2.0, 3.0}); }, true);
  expect_throw("interp2d_size_mismatch", [&] { quad::Interp2D t(two, two, std::vector<double>{1.0, 2.0, 3.0}); }, true);
  expect_throw("interp3d_bad_axis", [&] { quad::Interp3D t(two, down, two, std::vector<double>(8, 1.0)); }, true);
  quad::Interp1D e1;
  quad::Interp2D e2;
  quad::Interp3D e3;
  const bool nan_ok = std::isnan(e1(0.5)) && std::isnan(e2(0.5, 0.5)) && std::isnan(e3(0.5, 0.5, 0.5));
  std::printf("%s empty_tables_are_nan\n", nan_ok ? "PASS" : "FAIL");
  if (!nan_ok) ++failures;
  int devices = 0;
  if (cudaGetDeviceCount(&devices) != cudaSuccess) devices = 0;
  cudaGetLastError();
  if (devices == 0) {
    expect_throw("interp1d_no_device", [&] { quad::Interp1D t(two, two); }, false);
    expect_throw("interp2d_no_device", [&] { quad::Interp2D t(two, two, std::vector<double>(4, 1.0)); }, false);
    expect_throw("dynamic_array_no_device", [&] { gpu::cudaDynamicArray<double> a(4); }, false);
  } else {
    std::printf("SKIP no_device_cases (a device is present)\n");
  }
  gpu::cudaDynamicArray<int> empty;  // no allocation, nothing to free
  std::printf("%s %d failures\n", failures ? "FAIL" : "DONE", failures);
  return failures ? 1 : 0;
}
