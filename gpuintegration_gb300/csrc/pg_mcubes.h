// m-Cubes (stratified VEGAS) on the GB300: host side.
#pragma once

#include <string>

#include "../../include/pagani_gb300.h"
#include "pg_engine.h"

namespace pg {

struct McubesState;

McubesState* mcubes_create(Engine* eng);
void mcubes_destroy(McubesState* st);
int mcubes_run(McubesState* st, const IntegralDesc& D, double epsrel, double epsabs, const pg_mcubes_options& opt,
               pg_result* out, std::string* why);

}  // namespace pg
