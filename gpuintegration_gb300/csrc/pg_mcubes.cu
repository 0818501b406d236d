// m-Cubes (stratified VEGAS) on the GB300.
#include "pg_mcubes.h"

namespace pg {

struct McubesState {
  Engine* eng = nullptr;
};

McubesState* mcubes_create(Engine* eng) {
  McubesState* st = new McubesState;
  st->eng = eng;
  return st;
}

void mcubes_destroy(McubesState* st) { delete st; }

int mcubes_run(McubesState* st, const IntegralDesc& D, double epsrel, double epsabs, const pg_mcubes_options& opt,
               pg_result* out, std::string* why) {
  (void)st; (void)D; (void)epsrel; (void)epsabs; (void)opt; (void)out;
  if (why) *why = "m-Cubes not built yet";
  return PG_UNSUPPORTED;
}

}  // namespace pg
