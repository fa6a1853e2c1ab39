// TEST INFRASTRUCTURE -- oracle driver. The reference's own run/simulate3d.cpp does not compile
// (it calls load_particles<dim>() with no argument; src/read/load_hdf5.h:42 takes a ConfigVal),
// so this project-written driver runs the reference's 3D path: it reads config/main.conf,
// loads data/hdf5/all.h5 with the reference loaders, applies the config, marks every grain
// break_bonds = 1 (as run/simulate2d.cpp does for 2D) and calls the reference run_timeloop<3>.
#include <chrono>
#include <iostream>

#include "Eigen/Dense"
#include "read/load_hdf5.h"
#include "read/read_config.h"
#include "particle/timeloop.h"

int main() {
  const unsigned dim = 3;
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
  run_timeloop<dim>(grains, tl, contact, wall);
  auto t1 = std::chrono::system_clock::now();
  std::cout << "Runtime: " << std::chrono::duration_cast<std::chrono::seconds>(t1 - t0).count() << "s" << std::endl;
  return 0;
}
