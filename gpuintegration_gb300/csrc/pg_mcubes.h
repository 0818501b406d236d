// m-Cubes (stratified VEGAS) on the GB300: host side.
#pragma once

#include <functional>
#include <string>

#include "../../include/pagani_gb300.h"
#include "pg_engine.h"

namespace pg {

struct McubesState;

McubesState* mcubes_create(Engine* eng);
void mcubes_destroy(McubesState* st);
// Launches one sampling iteration for some integrand functor type.
using McubesLauncher = std::function<cudaError_t(const pg_mcubes_args&)>;

// The launcher of the C ABI families.
cudaError_t launch_family_mcubes(const pg_mcubes_args& a);

int mcubes_run(McubesState* st, const IntegralDesc& D, double epsrel, double epsabs, const pg_mcubes_options& opt,
               pg_result* out, std::string* why, const McubesLauncher& launcher = launch_family_mcubes);

}  // namespace pg
