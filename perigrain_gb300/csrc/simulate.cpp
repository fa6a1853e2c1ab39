// bin/simulate2d and bin/simulate3d: drop-in replacements of the reference executables
// (run/simulate2d.cpp:31-94; the reference's run/simulate3d.cpp does not compile, this one is
// built from the same driver with dim = 3). Run from the directory that holds config/, data/
// and output/. PERIGRAIN_PRECISION=mixed selects the FP32-force / FP64-state path.
#include <cstdlib>
#include <cstring>
#include <iostream>

#include "../../include/perigrain.h"
#include "../../include/perigrain_io.h"

#ifndef PG_SIM_DIM
#define PG_SIM_DIM 2
#endif

int main() {
  const char* p = std::getenv("PERIGRAIN_PRECISION");
  int precision = (p && std::strcmp(p, "mixed") == 0) ? PG_MIXED : PG_FP64;
  int rc = pg_run_simulation(".", PG_SIM_DIM, precision);
  if (rc != PG_OK) {
    std::cout << "\033[31mError: " << pg_status_string(rc) << "\033[0m" << std::endl;
    return 1;
  }
  return 0;
}
