// TEST INFRASTRUCTURE -- oracle driver. Runs the reference's own config parser
// (src/read/read_config.h, ConfigVal::read_file, compiled unmodified) on the file named by argv[1]
// and writes every field it holds, in ConfigVal's declaration order, as one JSON object to
// argv[2]. Booleans are written as 0/1, doubles with 17 significant digits.
#include <cstdio>
#include <iostream>

#include "read/read_config.h"

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s <main.conf> <out.json>\n", argv[0]);
    return 2;
  }
  ConfigVal c;
  c.read_file(argv[1]);
  FILE* f = std::fopen(argv[2], "w");
  if (!f) return 1;
  auto I = [&](const char* k, long long v, bool last = false) { std::fprintf(f, "\"%s\": %lld%s", k, v, last ? "" : ", "); };
  auto D = [&](const char* k, double v) { std::fprintf(f, "\"%s\": %.17g, ", k, v); };
  std::fprintf(f, "{");
  I("timesteps", c.timesteps);
  I("modulo", c.modulo);
  D("dt", c.dt);
  I("is_parallel", c.is_parallel);
  I("do_resume", c.do_resume);
  I("wall_resume", c.wall_resume);
  I("resume_ind", c.resume_ind);
  I("save_file", c.save_file);
  I("enable_fracture", c.enable_fracture);
  I("nl_bdry_only", c.nl_bdry_only);
  I("allow_damping", c.allow_damping);
  I("allow_friction", c.allow_friction);
  D("normal_stiffness", c.normal_stiffness);
  D("damping_ratio", c.damping_ratio);
  D("friction_coefficient", c.friction_coefficient);
  I("self_contact", c.self_contact);
  D("self_contact_rad", c.self_contact_rad);
  I("enable_torque", c.enable_torque);
  I("set_movable_index", c.set_movable_index);
  I("set_movable_timestep", c.set_movable_timestep);
  I("set_stoppable_index", c.set_stoppable_index);
  I("set_stoppable_timestep", c.set_stoppable_timestep);
  I("reset_partzero_y", c.reset_partzero_y);
  I("reset_partzero_y_timestep", c.reset_partzero_y_timestep);
  D("wheel_rad", c.wheel_rad);
  D("wall_left", c.wall_left);
  D("wall_right", c.wall_right);
  D("wall_top", c.wall_top);
  D("wall_bottom", c.wall_bottom);
  D("wall_x_min", c.wall_x_min);
  D("wall_y_min", c.wall_y_min);
  D("wall_z_min", c.wall_z_min);
  D("wall_x_max", c.wall_x_max);
  D("wall_y_max", c.wall_y_max);
  D("wall_z_max", c.wall_z_max);
  D("speed_wall_left", c.speed_wall_left);
  D("speed_wall_right", c.speed_wall_right);
  D("speed_wall_top", c.speed_wall_top);
  D("speed_wall_bottom", c.speed_wall_bottom);
  D("speed_wall_x_min", c.speed_wall_x_min);
  D("speed_wall_y_min", c.speed_wall_y_min);
  D("speed_wall_z_min", c.speed_wall_z_min);
  D("speed_wall_x_max", c.speed_wall_x_max);
  D("speed_wall_y_max", c.speed_wall_y_max);
  D("speed_wall_z_max", c.speed_wall_z_max);
  I("gradient_extforce", c.gradient_extforce);
  I("extforce_maxstep", c.extforce_maxstep, true);
  std::fprintf(f, "}\n");
  std::fclose(f);
  return 0;
}
