// TEST INFRASTRUCTURE -- oracle driver. No driver of the reference calls run_timeloop_worm
// (src/particle/timeloop.h:1018-1369); this project-written 2D driver does what
// run/simulate2d.cpp does (read config/main.conf, load data/hdf5/all.h5 with the reference
// loaders, apply the config, mark every grain break_bonds = 1) and calls the reference's own
// run_timeloop_worm<2>.
#include <chrono>
#include <iostream>

#include "Eigen/Dense"
#include "read/load_hdf5.h"
#include "read/read_config.h"
#include "particle/timeloop.h"

int main() {
  const unsigned dim = 2;
  omp_set_nested(1);
  ConfigVal cfg;
  cfg.read_file("config/main.conf");
  auto grains = load_particles<dim>(cfg);
  Contact contact = load_contact(cfg);
  RectWall<dim> wall = load_wall<dim>(cfg);
  Timeloop tl(100);
  tl.apply_config(cfg);
  contact.apply_config(cfg);
  wall.apply_config(cfg);
  for (auto& g : grains) g.break_bonds = 1;
  auto t0 = std::chrono::system_clock::now();
  run_timeloop_worm<dim>(grains, tl, contact, wall);
  auto t1 = std::chrono::system_clock::now();
  std::cout << "Runtime: " << std::chrono::duration_cast<std::chrono::seconds>(t1 - t0).count() << "s" << std::endl;
  return 0;
}
