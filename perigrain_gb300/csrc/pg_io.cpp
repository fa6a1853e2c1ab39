// Process/file contract of the reference simulator on top of the GPU engine:
// config parser (read_config.h), all.h5 loader (load_hdf5.h), output writers and the
// run_timeloop driver (timeloop.h:501-1015, run/simulate2d.cpp). See include/perigrain_io.h.
#include <sys/stat.h>

#include <algorithm>
#include <cctype>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/perigrain.h"
#include "../../include/perigrain_io.h"
#include "h5lite.h"

static thread_local std::string io_err;

static int iofail(int code, const std::string& m) {
  io_err = m;
  std::cerr << "Error: " << m << std::endl;
  return code;
}

// =============================================================================================
// config
// =============================================================================================
extern "C" void pg_conf_default(pg_conf* c) {
  std::memset(c, 0, sizeof(*c));
  c->timesteps = 8000;
  c->modulo = 100;
  c->dt = 0.02 / 1e5;
  c->is_parallel = 1;
  c->do_resume = 0;
  c->wall_resume = 0;
  c->resume_ind = 50;
  c->save_file = 1;
  c->enable_fracture = 0;
  c->nl_bdry_only = 0;
  c->allow_damping = 1;
  c->allow_friction = 1;
  c->self_contact = 1;
  c->self_contact_rad = -1;
  c->enable_torque = 0;
  c->normal_stiffness = -1;
  c->damping_ratio = -1;
  c->friction_coefficient = -1;
  c->set_movable_index = -1;
  c->set_movable_timestep = -1;
  c->set_stoppable_index = -1;
  c->set_stoppable_timestep = -1;
  c->reset_partzero_y = 0;
  c->reset_partzero_y_timestep = 0;
  c->wheel_rad = 0;
  c->wall_left = c->wall_right = c->wall_top = c->wall_bottom = -999;
  c->wall_x_min = c->wall_y_min = c->wall_z_min = -999;
  c->wall_x_max = c->wall_y_max = c->wall_z_max = -999;
  c->gradient_extforce = 0;
  c->extforce_maxstep = 0;
}

static int conf_parse(pg_conf* c, std::istream& in, bool quiet) {
  std::string line;
  while (std::getline(in, line)) {
    line.erase(std::remove_if(line.begin(), line.end(), [](unsigned char ch) { return std::isspace(ch); }),
               line.end());
    if (line.empty() || line[0] == '#') continue;
    auto pos = line.find('=');
    std::string name = line.substr(0, pos);
    std::string value = pos == std::string::npos ? line : line.substr(pos + 1);
    try {
      auto I = [&](int32_t* p) { *p = std::stoi(value); };
      auto U = [&](uint32_t* p) { *p = (uint32_t)std::stoi(value); };
      auto B = [&](int32_t* p) { *p = std::stoi(value) != 0; };
      auto F = [&](double* p) { *p = std::stod(value); };
      if (name == "timesteps") U(&c->timesteps);
      else if (name == "modulo") U(&c->modulo);
      else if (name == "dt") F(&c->dt);
      else if (name == "is_parallel") B(&c->is_parallel);
      else if (name == "do_resume") B(&c->do_resume);
      else if (name == "wall_resume") B(&c->wall_resume);
      else if (name == "resume_ind") U(&c->resume_ind);
      else if (name == "save_file") B(&c->save_file);
      else if (name == "enable_fracture") B(&c->enable_fracture);
      else if (name == "nl_bdry_only") B(&c->nl_bdry_only);
      else if (name == "allow_damping") B(&c->allow_damping);
      else if (name == "allow_friction") B(&c->allow_friction);
      else if (name == "damping_ratio") F(&c->damping_ratio);
      else if (name == "friction_coefficient") F(&c->friction_coefficient);
      else if (name == "normal_stiffness") F(&c->normal_stiffness);
      else if (name == "self_contact") B(&c->self_contact);
      else if (name == "self_contact_rad") F(&c->self_contact_rad);
      else if (name == "enable_torque") B(&c->enable_torque);
      else if (name == "set_movable_index") I(&c->set_movable_index);
      else if (name == "set_movable_timestep") I(&c->set_movable_timestep);
      else if (name == "set_stoppable_index") I(&c->set_stoppable_index);
      else if (name == "set_stoppable_timestep") I(&c->set_stoppable_timestep);
      else if (name == "reset_partzero_y") B(&c->reset_partzero_y);
      else if (name == "reset_partzero_y_timestep") U(&c->reset_partzero_y_timestep);
      else if (name == "wheel_rad") F(&c->wheel_rad);
      else if (name == "wall_left") F(&c->wall_left);
      else if (name == "wall_right") F(&c->wall_right);
      else if (name == "wall_top") F(&c->wall_top);
      else if (name == "wall_bottom") F(&c->wall_bottom);
      else if (name == "speed_wall_left") F(&c->speed_wall_left);
      else if (name == "speed_wall_right") F(&c->speed_wall_right);
      else if (name == "speed_wall_top") F(&c->speed_wall_top);
      else if (name == "speed_wall_bottom") F(&c->speed_wall_bottom);
      else if (name == "wall_x_min") F(&c->wall_x_min);
      else if (name == "wall_y_min") F(&c->wall_y_min);
      else if (name == "wall_z_min") F(&c->wall_z_min);
      else if (name == "wall_x_max") F(&c->wall_x_max);
      else if (name == "wall_y_max") F(&c->wall_y_max);
      else if (name == "wall_z_max") F(&c->wall_z_max);
      else if (name == "speed_wall_x_min") F(&c->speed_wall_x_min);
      else if (name == "speed_wall_y_min") F(&c->speed_wall_y_min);
      else if (name == "speed_wall_z_min") F(&c->speed_wall_z_min);
      else if (name == "speed_wall_x_max") F(&c->speed_wall_x_max);
      else if (name == "speed_wall_y_max") F(&c->speed_wall_y_max);
      else if (name == "speed_wall_z_max") F(&c->speed_wall_z_max);
      else if (name == "gradient_extforce") B(&c->gradient_extforce);
      else if (name == "extforce_maxstep") U(&c->extforce_maxstep);
      else if (!quiet) std::cerr << "Error: Wrong config name: " << name << " !!\n";
    } catch (const std::exception&) {
      io_err = "config value of '" + name + "' does not parse: '" + value + "'";
      if (!quiet) std::cerr << "Error: " << io_err << "\n";
      return PG_EINVAL;
    }
  }
  return PG_OK;
}

extern "C" int pg_conf_read_file(pg_conf* c, const char* path) {
  std::ifstream f(path);
  if (!f.is_open()) {
    std::cerr << "Couldn't open config file for reading.\n";
    return PG_OK;
  }
  std::cout << "Reading config file: " << path << std::endl;
  return conf_parse(c, f, false);
}

extern "C" int pg_conf_read_string(pg_conf* c, const char* text, int quiet) {
  std::istringstream s(text ? text : "");
  return conf_parse(c, s, quiet != 0);
}

// =============================================================================================
// setup
// =============================================================================================
struct pg_setup {
  uint32_t dim = 2;
  uint32_t G = 0, N = 0;
  std::vector<uint32_t> grain_instance, node_off;
  std::vector<double> pos, vol, disp, vel, acc, extforce;
  std::vector<uint64_t> bond_offset;
  std::vector<uint32_t> bond_local;
  std::vector<uint32_t> bdry_offset, bdry_nodes, clamped_offset, clamped_nodes;
  std::vector<double> delta, rho, cnot, snot, torque_val;
  std::vector<int32_t> movable, breakable, stoppable;
  std::vector<uint8_t> break_bonds;
  std::vector<uint32_t> torque_axis;
  double contact_radius = 0, normal_stiffness = 0, friction_coefficient = 0, damping_ratio = 0;
  int32_t allow_wall = 0;
  bool wall_geom_given = false;
  double wall_geom[6] = {0, 0, 0, 0, 0, 0};
  double wall_speed[6] = {0, 0, 0, 0, 0, 0};
};

namespace {
struct H5In {
  h5l::Reader r;
  std::string file;
  int ok(const std::string& path) { return r.exists(path); }
  bool f64(const std::string& p, std::vector<uint64_t>* dims, std::vector<double>* v) {
    return r.read_vec(p, h5l::DType::F64, dims, v);
  }
  bool u32(const std::string& p, std::vector<uint64_t>* dims, std::vector<uint32_t>* v) {
    return r.read_vec(p, h5l::DType::U32, dims, v);
  }
  bool i32(const std::string& p, std::vector<uint64_t>* dims, std::vector<int32_t>* v) {
    return r.read_vec(p, h5l::DType::I32, dims, v);
  }
};

uint64_t ncols(const std::vector<uint64_t>& dims) { return dims.size() >= 2 ? dims[1] : 1; }
uint64_t nrows(const std::vector<uint64_t>& dims) { return dims.empty() ? 1 : dims[0]; }
}  // namespace

// conn2NArr (load_hdf5.h:28-38): row (i, j) appends j to NArr[i] and i to NArr[j]
// conn2NArr (load_hdf5.h:28-38) as CSR: row i lists the partners of i in the order the pairs
// name them (for pair (i, j): j appended to row i, i to row j). off has n + 1 entries.
static void conn_to_csr(const uint32_t* conn, uint64_t m, uint32_t n, std::vector<uint64_t>* off,
                        std::vector<uint32_t>* col) {
  off->assign((size_t)n + 1, 0);
  for (uint64_t l = 0; l < 2 * m; ++l) ++(*off)[conn[l] + 1];
  for (uint32_t i = 0; i < n; ++i) (*off)[i + 1] += (*off)[i];
  col->resize(2 * m);
  std::vector<uint64_t> fill(off->begin(), off->end() - 1);
  for (uint64_t l = 0; l < m; ++l) {
    const uint32_t i = conn[2 * l], j = conn[2 * l + 1];
    (*col)[fill[i]++] = j;
    (*col)[fill[j]++] = i;
  }
}

extern "C" int pg_setup_load(const char* path, uint32_t dim, int32_t load_torque, pg_setup** out) {
  if (!out || (dim != 2 && dim != 3)) return iofail(PG_EINVAL, "bad arguments to pg_setup_load");
  *out = nullptr;
  H5In in;
  if (!in.r.open(path)) return iofail(PG_EIO, std::string(path) + ": " + in.r.error());
  std::unique_ptr<pg_setup> s(new pg_setup);
  s->dim = dim;
  std::vector<uint64_t> dims;
  std::vector<uint32_t> u;
  std::vector<int32_t> iv;
  std::vector<double> f;
  if (!in.u32("total_particles_univ", &dims, &u) || u.empty())
    return iofail(PG_EIO, std::string(path) + ": total_particles_univ: " + in.r.error());
  const uint32_t P = u[0];
  std::cout << "Reading total particles: " << P << std::endl;
  s->G = P;
  s->node_off.push_back(0);
  s->bond_offset.push_back(0);
  s->bdry_offset.push_back(0);
  s->clamped_offset.push_back(0);
  for (uint32_t g = 0; g < P; ++g) {
    char buf[32];
    std::snprintf(buf, sizeof buf, "P_%05u/", g + 1);
    const std::string pre(buf);
    auto need = [&](bool ok, const char* what) {
      if (!ok) iofail(PG_EIO, std::string(path) + ": " + pre + what + ": " + in.r.error());
      return ok;
    };
    if (!need(in.f64(pre + "Pos", &dims, &f), "Pos")) return PG_EIO;
    const uint64_t n = nrows(dims), nc = ncols(dims);
    if (nc < dim || dims.size() != 2) return iofail(PG_EIO, pre + "Pos must be n x dim");
    if (n == 0) return iofail(PG_EIO, pre + "Pos is empty");
    const uint32_t n0 = s->N;
    for (uint64_t i = 0; i < n; ++i)
      for (uint32_t c = 0; c < dim; ++c) s->pos.push_back(f[i * nc + c]);
    auto rowvecs = [&](const char* name, std::vector<double>* dst) {
      if (!need(in.f64(pre + name, &dims, &f), name)) return false;
      const uint64_t k = ncols(dims);
      if (nrows(dims) != n || k < dim) {
        iofail(PG_EIO, pre + name + " must be n x dim");
        return false;
      }
      for (uint64_t i = 0; i < n; ++i)
        for (uint32_t c = 0; c < dim; ++c) dst->push_back(f[i * k + c]);
      return true;
    };
    if (!need(in.f64(pre + "Vol", &dims, &f), "Vol")) return PG_EIO;
    if (nrows(dims) != n) return iofail(PG_EIO, pre + "Vol must have n rows");
    for (uint64_t i = 0; i < n; ++i) s->vol.push_back(f[i * ncols(dims)]);
    if (!need(in.u32(pre + "bdry_nodes", &dims, &u), "bdry_nodes")) return PG_EIO;
    for (uint64_t i = 0; i < nrows(dims) && !u.empty(); ++i) s->bdry_nodes.push_back(u[i * ncols(dims)]);
    s->bdry_offset.push_back((uint32_t)s->bdry_nodes.size());
    if (!need(in.u32(pre + "clamped_nodes", &dims, &u), "clamped_nodes")) return PG_EIO;
    for (auto x : u) s->clamped_nodes.push_back(x);
    s->clamped_offset.push_back((uint32_t)s->clamped_nodes.size());
    if (!rowvecs("disp", &s->disp) || !rowvecs("vel", &s->vel) || !rowvecs("acc", &s->acc) ||
        !rowvecs("extforce", &s->extforce))
      return PG_EIO;
    if (!need(in.u32(pre + "Connectivity", &dims, &u), "Connectivity")) return PG_EIO;
    uint64_t m = u.empty() ? 0 : nrows(dims);
    if (m && ncols(dims) != 2) return iofail(PG_EIO, pre + "Connectivity must be m x 2");
    for (auto x : u)
      if (x >= n) return iofail(PG_EIO, pre + "Connectivity index out of range");
    std::vector<uint64_t> roff;
    std::vector<uint32_t> rcol;
    conn_to_csr(u.data(), m, (uint32_t)n, &roff, &rcol);
    const uint64_t b0 = s->bond_local.size();
    s->bond_local.insert(s->bond_local.end(), rcol.begin(), rcol.end());
    for (uint64_t i = 0; i < n; ++i) s->bond_offset.push_back(b0 + roff[i + 1]);
    auto scalar = [&](const char* name, double* dst) {
      if (!need(in.f64(pre + name, &dims, &f), name) || f.empty()) return false;
      *dst = f[0];
      return true;
    };
    auto iscalar = [&](const char* name, int32_t* dst) {
      if (!need(in.i32(pre + name, &dims, &iv), name) || iv.empty()) return false;
      *dst = iv[0];
      return true;
    };
    double de, rh, cn, sn, tv = 0;
    int32_t mv, br, st;
    uint32_t ta = 2;
    if (!scalar("delta", &de) || !scalar("rho", &rh) || !scalar("cnot", &cn) || !scalar("snot", &sn) ||
        !iscalar("movable", &mv) || !iscalar("breakable", &br) || !iscalar("stoppable", &st))
      return PG_EIO;
    if (load_torque) {
      if (!need(in.u32(pre + "torque_axis", &dims, &u), "torque_axis") || u.empty()) return PG_EIO;
      ta = u[0];
      if (!scalar("torque_val", &tv)) return PG_EIO;
    }
    s->delta.push_back(de);
    s->rho.push_back(rh);
    s->cnot.push_back(cn);
    s->snot.push_back(sn);
    s->movable.push_back(mv);
    s->breakable.push_back(br);
    s->stoppable.push_back(st);
    s->break_bonds.push_back(1);  // run/simulate2d.cpp:76-78
    s->torque_axis.push_back(ta);
    s->torque_val.push_back(tv);
    s->grain_instance.push_back(0);
    s->N = n0 + (uint32_t)n;
    s->node_off.push_back(s->N);
  }
  std::cout << "Done reading particles." << std::endl;
  auto pw = [&](const char* name, double* dst) {
    std::vector<double> v;
    if (!in.f64(std::string("pairwise/") + name, &dims, &v) || v.empty()) {
      iofail(PG_EIO, std::string(path) + ": pairwise/" + name + ": " + in.r.error());
      return false;
    }
    *dst = v[0];
    return true;
  };
  if (!pw("contact_radius", &s->contact_radius) || !pw("normal_stiffness", &s->normal_stiffness) ||
      !pw("friction_coefficient", &s->friction_coefficient) || !pw("damping_ratio", &s->damping_ratio))
    return PG_EIO;
  std::cout << "Done reading contact." << std::endl;
  if (!in.u32("wall/allow_wall", &dims, &u) || u.empty())
    return iofail(PG_EIO, std::string(path) + ": wall/allow_wall: " + in.r.error());
  s->allow_wall = u[0] != 0;
  if (!in.f64("wall/geom_wall_info", &dims, &f))
    return iofail(PG_EIO, std::string(path) + ": wall/geom_wall_info: " + in.r.error());
  std::vector<double> ci;
  for (uint64_t i = 0; i < nrows(dims) && !f.empty(); ++i) ci.push_back(f[i * ncols(dims)]);
  if (ci.size() != 1) {
    if (ci.size() >= 2 * dim) {
      for (uint32_t k = 0; k < 2 * dim; ++k) s->wall_geom[k] = ci[k];
      s->wall_geom_given = true;
    } else {
      std::cout << "hdf data geom_wall_info length is not 4 or 6. " << std::endl;
    }
  }
  std::cout << "Done reading wall size." << std::endl;
  *out = s.release();
  return PG_OK;
}

extern "C" int pg_setup_from_desc(const pg_setup_desc* d, pg_setup** out) {
  if (!d || !out || d->n_instances != 1) return iofail(PG_EINVAL, "pg_setup_from_desc needs one instance");
  std::unique_ptr<pg_setup> s(new pg_setup);
  const uint32_t D = d->dim, G = d->n_grains, N = d->n_nodes;
  s->dim = D;
  s->G = G;
  s->N = N;
  s->grain_instance.assign(G, 0);
  s->node_off.assign(d->grain_node_offset, d->grain_node_offset + G + 1);
  auto cp = [&](const double* p, size_t n, std::vector<double>* v) { v->assign(p, p + n); };
  cp(d->pos, (size_t)N * D, &s->pos);
  cp(d->vol, N, &s->vol);
  cp(d->disp, (size_t)N * D, &s->disp);
  cp(d->vel, (size_t)N * D, &s->vel);
  cp(d->acc, (size_t)N * D, &s->acc);
  cp(d->extforce, (size_t)N * D, &s->extforce);
  s->bond_offset.assign(d->bond_offset, d->bond_offset + N + 1);
  s->bond_local.assign(d->bond_local, d->bond_local + d->bond_offset[N]);
  s->bdry_offset.assign(d->bdry_offset, d->bdry_offset + G + 1);
  s->bdry_nodes.assign(d->bdry_nodes, d->bdry_nodes + d->bdry_offset[G]);
  s->clamped_offset.assign(d->clamped_offset, d->clamped_offset + G + 1);
  s->clamped_nodes.assign(d->clamped_nodes, d->clamped_nodes + d->clamped_offset[G]);
  cp(d->delta, G, &s->delta);
  cp(d->rho, G, &s->rho);
  cp(d->cnot, G, &s->cnot);
  cp(d->snot, G, &s->snot);
  s->movable.assign(d->movable, d->movable + G);
  s->breakable.assign(d->breakable, d->breakable + G);
  s->stoppable.assign(d->stoppable, d->stoppable + G);
  s->break_bonds.assign(d->break_bonds, d->break_bonds + G);
  s->torque_axis.assign(G, 2);
  s->torque_val.assign(G, 0.0);
  if (d->torque_axis) s->torque_axis.assign(d->torque_axis, d->torque_axis + G);
  if (d->torque_val) s->torque_val.assign(d->torque_val, d->torque_val + G);
  s->contact_radius = d->contact_radius[0];
  s->normal_stiffness = d->normal_stiffness[0];
  s->friction_coefficient = d->friction_coefficient[0];
  s->damping_ratio = d->damping_ratio[0];
  s->allow_wall = d->allow_wall[0];
  s->wall_geom_given = true;
  for (uint32_t k = 0; k < 2 * D; ++k) {
    s->wall_geom[k] = d->wall_geom[k];
    s->wall_speed[k] = d->wall_speed[k];
  }
  *out = s.release();
  return PG_OK;
}

extern "C" int pg_setup_free(pg_setup* s) {
  delete s;
  return PG_OK;
}

extern "C" int pg_setup_desc_get(pg_setup* s, pg_setup_desc* d) {
  if (!s || !d) return iofail(PG_EINVAL, "null argument");
  std::memset(d, 0, sizeof(*d));
  d->dim = s->dim;
  d->n_instances = 1;
  d->n_grains = s->G;
  d->n_nodes = s->N;
  d->grain_instance = s->grain_instance.data();
  d->grain_node_offset = s->node_off.data();
  d->pos = s->pos.data();
  d->vol = s->vol.data();
  d->disp = s->disp.data();
  d->vel = s->vel.data();
  d->acc = s->acc.data();
  d->extforce = s->extforce.data();
  d->bond_offset = s->bond_offset.data();
  d->bond_local = s->bond_local.data();
  d->bdry_offset = s->bdry_offset.data();
  d->bdry_nodes = s->bdry_nodes.data();
  d->clamped_offset = s->clamped_offset.data();
  d->clamped_nodes = s->clamped_nodes.data();
  d->delta = s->delta.data();
  d->rho = s->rho.data();
  d->cnot = s->cnot.data();
  d->snot = s->snot.data();
  d->movable = s->movable.data();
  d->breakable = s->breakable.data();
  d->stoppable = s->stoppable.data();
  d->break_bonds = s->break_bonds.data();
  d->torque_axis = s->torque_axis.data();
  d->torque_val = s->torque_val.data();
  d->contact_radius = &s->contact_radius;
  d->normal_stiffness = &s->normal_stiffness;
  d->friction_coefficient = &s->friction_coefficient;
  d->damping_ratio = &s->damping_ratio;
  d->allow_wall = &s->allow_wall;
  d->wall_geom = s->wall_geom;
  d->wall_speed = s->wall_speed;
  return PG_OK;
}

extern "C" int pg_setup_apply_conf(pg_setup* s, const pg_conf* c) {
  if (!s || !c) return iofail(PG_EINVAL, "null argument");
  // Contact::apply_config (contact.h:85-108)
  if (c->damping_ratio != (-1)) s->damping_ratio = c->damping_ratio;
  if (c->friction_coefficient != (-1)) s->friction_coefficient = c->friction_coefficient;
  if (c->normal_stiffness != (-1)) s->normal_stiffness = c->normal_stiffness;
  // RectWall::apply_config (contact.h:254-301); lrtb: 2D [l, r, t, b], 3D [x0, y0, z0, x1, y1, z1]
  double* w = s->wall_geom;
  if (s->dim == 2) {
    if (c->wall_top != (-999)) w[2] = c->wall_top;
    if (c->wall_right != (-999)) w[1] = c->wall_right;
    if (c->wall_left != (-999)) w[0] = c->wall_left;
    if (c->wall_right != (-999)) w[1] = c->wall_right;
    if (c->wall_top != (-999)) w[2] = c->wall_top;
    if (c->wall_bottom != (-999)) w[3] = c->wall_bottom;
    s->wall_speed[0] = c->speed_wall_left;
    s->wall_speed[1] = c->speed_wall_right;
    s->wall_speed[2] = c->speed_wall_top;
    s->wall_speed[3] = c->speed_wall_bottom;
  } else {
    if (c->wall_top != (-999)) w[5] = c->wall_top;
    if (c->wall_right != (-999)) w[4] = c->wall_right;
    if (c->wall_x_min != (-999)) w[0] = c->wall_x_min;
    if (c->wall_y_min != (-999)) w[1] = c->wall_y_min;
    if (c->wall_z_min != (-999)) w[2] = c->wall_z_min;
    if (c->wall_x_max != (-999)) w[3] = c->wall_x_max;
    if (c->wall_y_max != (-999)) w[4] = c->wall_y_max;
    if (c->wall_z_max != (-999)) w[5] = c->wall_z_max;
    s->wall_speed[0] = c->speed_wall_x_min;
    s->wall_speed[1] = c->speed_wall_y_min;
    s->wall_speed[2] = c->speed_wall_z_min;
    s->wall_speed[3] = c->speed_wall_x_max;
    s->wall_speed[4] = c->speed_wall_y_max;
    s->wall_speed[5] = c->speed_wall_z_max;
  }
  return PG_OK;
}

extern "C" int pg_setup_set_connectivity(pg_setup* s, uint32_t g, const uint32_t* conn, uint64_t m) {
  if (!s || g >= s->G || (m && !conn)) return iofail(PG_EINVAL, "bad arguments");
  const uint32_t n0 = s->node_off[g], n = s->node_off[g + 1] - n0;
  for (uint64_t k = 0; k < 2 * m; ++k)
    if (conn[k] >= n) return iofail(PG_EINVAL, "connectivity index out of range");
  std::vector<uint64_t> roff;
  std::vector<uint32_t> rcol;
  conn_to_csr(conn, m, n, &roff, &rcol);
  std::vector<uint64_t> off;
  std::vector<uint32_t> loc;
  off.push_back(0);
  for (uint32_t i = 0; i < s->N; ++i) {
    if (i >= n0 && i < n0 + n) {
      loc.insert(loc.end(), rcol.begin() + roff[i - n0], rcol.begin() + roff[i - n0 + 1]);
    } else {
      for (uint64_t b = s->bond_offset[i]; b < s->bond_offset[i + 1]; ++b) loc.push_back(s->bond_local[b]);
    }
    off.push_back(loc.size());
  }
  s->bond_offset.swap(off);
  s->bond_local.swap(loc);
  return PG_OK;
}

// NbdArr2conn (timeloop.h:25-49): rows (i, q) for i < q in row order
static void rows_to_conn(const pg_setup* s, uint32_t g, const uint8_t* alive, std::vector<uint32_t>* conn) {
  const uint32_t n0 = s->node_off[g], n1 = s->node_off[g + 1];
  conn->resize(2 * (s->bond_offset[n1] - s->bond_offset[n0]));  // at most one pair per row entry
  uint32_t* o = conn->data();
  size_t k = 0;
  for (uint32_t i = n0; i < n1; ++i)
    for (uint64_t b = s->bond_offset[i]; b < s->bond_offset[i + 1]; ++b) {
      if (alive && !alive[b]) continue;
      const uint32_t q = s->bond_local[b];
      if (i - n0 < q) {
        o[k++] = i - n0;
        o[k++] = q;
      }
    }
  conn->resize(k);
}

extern "C" int pg_setup_save(pg_setup* s, const char* path) {
  if (!s || !path) return iofail(PG_EINVAL, "null argument");
  h5l::Writer w;
  const uint32_t D = s->dim;
  auto i64 = [](std::vector<int64_t> v) { return v; };
  (void)i64;
  for (uint32_t g = 0; g < s->G; ++g) {
    char buf[32];
    std::snprintf(buf, sizeof buf, "P_%05u/", g + 1);
    std::string pre(buf);
    const uint32_t n0 = s->node_off[g], n = s->node_off[g + 1] - n0;
    w.add_dataset(pre + "Pos", h5l::DType::F64, {n, D}, s->pos.data() + (size_t)n0 * D);
    w.add_dataset(pre + "Vol", h5l::DType::F64, {n, 1}, s->vol.data() + n0);
    std::vector<uint32_t> conn;
    rows_to_conn(s, g, nullptr, &conn);
    std::vector<int64_t> c64(conn.begin(), conn.end());
    w.add_dataset(pre + "Connectivity", h5l::DType::I64, {conn.size() / 2, 2}, c64.data());
    std::vector<int64_t> bd(s->bdry_nodes.begin() + s->bdry_offset[g], s->bdry_nodes.begin() + s->bdry_offset[g + 1]);
    w.add_dataset(pre + "bdry_nodes", h5l::DType::I64, {bd.size(), 1}, bd.data());
    w.add_dataset(pre + "bdry_edges", h5l::DType::I64, {0, 2}, nullptr);
    std::vector<int64_t> cl(s->clamped_nodes.begin() + s->clamped_offset[g],
                            s->clamped_nodes.begin() + s->clamped_offset[g + 1]);
    if (cl.empty()) {
      w.add_dataset(pre + "clamped_nodes", h5l::DType::F64, {0}, nullptr);
    } else {
      w.add_dataset(pre + "clamped_nodes", h5l::DType::I64, {cl.size()}, cl.data());
    }
    w.add_dataset(pre + "disp", h5l::DType::F64, {n, D}, s->disp.data() + (size_t)n0 * D);
    w.add_dataset(pre + "vel", h5l::DType::F64, {n, D}, s->vel.data() + (size_t)n0 * D);
    w.add_dataset(pre + "acc", h5l::DType::F64, {n, D}, s->acc.data() + (size_t)n0 * D);
    w.add_dataset(pre + "extforce", h5l::DType::F64, {n, D}, s->extforce.data() + (size_t)n0 * D);
    w.add_dataset(pre + "delta", h5l::DType::F64, {1, 1}, &s->delta[g]);
    w.add_dataset(pre + "rho", h5l::DType::F64, {1, 1}, &s->rho[g]);
    w.add_dataset(pre + "cnot", h5l::DType::F64, {1, 1}, &s->cnot[g]);
    w.add_dataset(pre + "snot", h5l::DType::F64, {1, 1}, &s->snot[g]);
    int64_t ta = s->torque_axis[g];
    w.add_dataset(pre + "torque_axis", h5l::DType::I64, {1, 1}, &ta);
    w.add_dataset(pre + "torque_val", h5l::DType::F64, {1, 1}, &s->torque_val[g]);
    int64_t mv = s->movable[g], br = s->breakable[g], st = s->stoppable[g];
    w.add_dataset(pre + "movable", h5l::DType::I64, {1, 1}, &mv);
    w.add_dataset(pre + "breakable", h5l::DType::I64, {1, 1}, &br);
    w.add_dataset(pre + "stoppable", h5l::DType::I64, {1, 1}, &st);
  }
  int64_t tp = s->G;
  w.add_dataset("total_particles_univ", h5l::DType::I64, {1, 1}, &tp);
  w.add_dataset("pairwise/contact_radius", h5l::DType::F64, {1, 1}, &s->contact_radius);
  w.add_dataset("pairwise/normal_stiffness", h5l::DType::F64, {1, 1}, &s->normal_stiffness);
  w.add_dataset("pairwise/damping_ratio", h5l::DType::F64, {1, 1}, &s->damping_ratio);
  w.add_dataset("pairwise/friction_coefficient", h5l::DType::F64, {1, 1}, &s->friction_coefficient);
  int64_t aw = s->allow_wall;
  w.add_dataset("wall/allow_wall", h5l::DType::I64, {1, 1}, &aw);
  if (s->wall_geom_given) {
    w.add_dataset("wall/geom_wall_info", h5l::DType::F64, {2ull * D, 1}, s->wall_geom);
  } else {
    double z = 0;
    w.add_dataset("wall/geom_wall_info", h5l::DType::F64, {1, 1}, &z);
  }
  if (!w.write(path)) return iofail(PG_EIO, std::string("cannot write ") + path);
  return PG_OK;
}

// =============================================================================================
// output
// =============================================================================================
static int write_tc(pg_setup* s, const std::string& dir, uint32_t counter, const double* cur, const double* vel,
                    const double* acc, const double* force, const uint8_t* alive, const double* wall,
                    const double* reaction, bool connectivity = true) {
  const uint32_t D = s->dim;
  char buf[64];
  std::snprintf(buf, sizeof buf, "%05u", counter);
  h5l::Writer w;
  std::vector<std::vector<uint32_t>> conns(connectivity ? s->G : 0);  // borrowed by w until written
  for (uint32_t g = 0; g < s->G; ++g) {
    char gb[32];
    std::snprintf(gb, sizeof gb, "P_%05u/", g);
    std::string pre(gb);
    const uint32_t n0 = s->node_off[g], n = s->node_off[g + 1] - n0;
    w.create_group(pre);
    w.add_dataset_ref(pre + "CurrPos", h5l::DType::F64, {n, D}, cur + (size_t)n0 * D);
    w.add_dataset_ref(pre + "vel", h5l::DType::F64, {n, D}, vel + (size_t)n0 * D);
    w.add_dataset_ref(pre + "acc", h5l::DType::F64, {n, D}, acc + (size_t)n0 * D);
    w.add_dataset_ref(pre + "force", h5l::DType::F64, {n, D}, force + (size_t)n0 * D);
    if (connectivity) {  // run_timeloop_worm writes none (timeloop.h:1283-1292)
      rows_to_conn(s, g, alive, &conns[g]);
      w.add_dataset_ref(pre + "Connectivity", h5l::DType::U32, {conns[g].size() / 2, 2}, conns[g].data());
    }
  }
  if (!w.write(dir + "/tc_" + buf + ".h5")) return iofail(PG_EIO, "cannot write " + dir + "/tc_" + buf + ".h5");
  h5l::Writer ww;
  ww.add_dataset("wall_info", h5l::DType::F64, {2ull * D, 1}, wall);
  ww.add_dataset("reaction", h5l::DType::F64, {2ull * D, D}, reaction);
  if (!ww.write(dir + "/wall_" + buf + ".h5")) return iofail(PG_EIO, "cannot write wall file");
  return PG_OK;
}

static int snapshot(pg_handle* h, pg_setup* s, const char* out_dir, uint32_t counter, bool connectivity) {
  const uint32_t D = s->dim;
  std::vector<double> cur((size_t)s->N * D), vel(cur.size()), acc(cur.size()), force(cur.size());
  std::vector<uint8_t> alive(s->bond_local.size() + 1);
  std::vector<double> wall(2 * D), reaction(2 * D * D);
  int rc;
  if ((rc = pg_get_field(h, PG_FIELD_CURRPOS, cur.data())) || (rc = pg_get_field(h, PG_FIELD_VEL, vel.data())) ||
      (rc = pg_get_field(h, PG_FIELD_ACC, acc.data())) || (rc = pg_get_field(h, PG_FIELD_FORCE, force.data())) ||
      (rc = pg_get_bond_alive(h, alive.data())) || (rc = pg_get_wall(h, wall.data())) ||
      (rc = pg_get_reaction(h, reaction.data())))
    return iofail(rc, pg_last_error());
  return write_tc(s, out_dir, counter, cur.data(), vel.data(), acc.data(), force.data(), alive.data(), wall.data(),
                  reaction.data(), connectivity);
}

// One output's buffers (page-locked: the snapshot copies land there directly) and its job.
struct OutSet {
  void* fields_mem = nullptr;
  void* alive_mem = nullptr;
  double *cur = nullptr, *vel = nullptr, *acc = nullptr, *force = nullptr;
  uint8_t* alive = nullptr;
  std::vector<double> wall, react;
  uint64_t too_close = 0;
  uint32_t counter = 0, e = 0;
  int rc = PG_OK;
  std::string err;
  bool done = false;
  std::vector<double> v, a, x, f, dmg, fs, phi;  // post-processing at the output step
  ~OutSet() {
    pg_host_free(fields_mem);
    pg_host_free(alive_mem);
  }
};

// Writer threads over a ring of OutSets: acquire() a free set, fill it, submit() it; outputs are
// written concurrently and handed back in submission order by pop_done().
class OutputPool {
 public:
  OutputPool(pg_handle* h, pg_setup* s, const std::string& dir, bool connectivity, uint32_t n_writers)
      : h_(h), s_(s), dir_(dir), conn_(connectivity) {
    for (uint32_t k = 0; k < n_writers; ++k) th_.emplace_back([this] { work(); });
    if (n_writers) sets_.resize(n_writers + 1);
  }
  ~OutputPool() {
    pg_wait(h_);  // a snapshot still copying into a set (an error return) completes first
    {
      std::lock_guard<std::mutex> lk(m_);
      stop_ = true;
    }
    cv_job_.notify_all();
    for (auto& t : th_) t.join();
  }
  int alloc(size_t nd, size_t n_bonds, uint32_t dim) {
    for (auto& o : sets_) {
      int rc = pg_host_alloc(4 * nd * sizeof(double), &o.fields_mem);
      if (!rc) rc = pg_host_alloc(n_bonds + 1, &o.alive_mem);
      if (rc) return rc;
      o.cur = static_cast<double*>(o.fields_mem);
      o.vel = o.cur + nd;
      o.acc = o.vel + nd;
      o.force = o.acc + nd;
      o.alive = static_cast<uint8_t*>(o.alive_mem);
      o.wall.assign(2 * dim, 0.0);
      o.react.assign((size_t)2 * dim * dim, 0.0);
      free_.push_back(&o);
    }
    return PG_OK;
  }
  // A free set, or null when every set holds an output not yet finalised.
  OutSet* acquire() {
    if (free_.empty()) return nullptr;
    OutSet* o = free_.front();
    free_.pop_front();
    return o;
  }
  void submit(OutSet* o) {
    {
      std::lock_guard<std::mutex> lk(m_);
      o->done = false;
      o->rc = PG_OK;
      o->err.clear();
      q_.push_back(o);
      order_.push_back(o);
    }
    cv_job_.notify_one();
  }
  // Whether the oldest submitted output is written (waiting for it when `wait`); false if none.
  bool front_done(bool wait) {
    std::unique_lock<std::mutex> lk(m_);
    if (order_.empty()) return false;
    if (wait) cv_done_.wait(lk, [this] { return order_.front()->done; });
    return order_.front()->done;
  }
  // The oldest submitted output, after its files are written.
  OutSet* pop_done() {
    std::unique_lock<std::mutex> lk(m_);
    cv_done_.wait(lk, [this] { return order_.front()->done; });
    OutSet* o = order_.front();
    order_.pop_front();
    return o;
  }
  void release(OutSet* o) { free_.push_back(o); }

 private:
  void work() {
    for (;;) {
      OutSet* o;
      {
        std::unique_lock<std::mutex> lk(m_);
        cv_job_.wait(lk, [this] { return stop_ || !q_.empty(); });
        if (q_.empty()) return;
        o = q_.front();
        q_.pop_front();
      }
      int rc = write_tc(s_, dir_, o->counter, o->cur, o->vel, o->acc, o->force, conn_ ? o->alive : nullptr,
                        o->wall.data(), o->react.data(), conn_);
      {
        std::lock_guard<std::mutex> lk(m_);
        o->rc = rc;
        if (rc) o->err = io_err;
        o->done = true;
      }
      cv_done_.notify_all();
    }
  }
  pg_handle* h_;
  pg_setup* s_;
  std::string dir_;
  bool conn_;
  std::vector<std::thread> th_;
  std::deque<OutSet> sets_;
  std::deque<OutSet*> free_, q_, order_;
  std::mutex m_;
  std::condition_variable cv_job_, cv_done_;
  bool stop_ = false;
};

extern "C" int pg_write_tc(pg_setup* s, const char* out_dir, uint32_t counter, const double* currpos,
                           const double* vel, const double* acc, const double* force, const uint8_t* bond_alive,
                           const double* wall, const double* reaction, int32_t connectivity) {
  if (!s || !out_dir || !currpos || !vel || !acc || !force || !wall || !reaction)
    return iofail(PG_EINVAL, "null argument");
  return write_tc(s, out_dir, counter, currpos, vel, acc, force, bond_alive, wall, reaction, connectivity != 0);
}

extern "C" int pg_write_snapshot(pg_handle* h, pg_setup* s, const char* out_dir, uint32_t counter) {
  if (!h || !s || !out_dir) return iofail(PG_EINVAL, "null argument");
  return snapshot(h, s, out_dir, counter, true);
}

// =============================================================================================
// driver: run_timeloop (timeloop.h:501-1015) + main of run/simulate2d.cpp
// =============================================================================================
static bool is_dir(const std::string& p) {
  struct stat st;
  return stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

extern "C" int pg_run_simulation(const char* root_c, uint32_t dim, int32_t precision) {
  const std::string root = root_c && *root_c ? root_c : ".";
  auto start_all = std::chrono::system_clock::now();
  pg_conf C;
  pg_conf_default(&C);
  int rc = pg_conf_read_file(&C, (root + "/config/main.conf").c_str());
  if (rc) return rc;
  pg_setup* S = nullptr;
  rc = pg_setup_load((root + "/data/hdf5/all.h5").c_str(), dim, C.enable_torque, &S);
  if (rc) return rc;
  std::unique_ptr<pg_setup, int (*)(pg_setup*)> guard(S, pg_setup_free);
  pg_setup_apply_conf(S, &C);
  std::cout << "extforce_gradient" << C.gradient_extforce << std::endl;
  const std::string out = root + "/output/hdf5";
  if (!is_dir(out)) return iofail(PG_EIO, "output directory " + out + " does not exist");

  uint32_t counter, first_counter, last_counter;
  std::vector<double> resume_cur, resume_vel, resume_acc;
  if (C.do_resume) {
    counter = C.resume_ind + 1;
    first_counter = counter;
    last_counter = C.resume_ind + C.timesteps / C.modulo;
    char buf[32];
    std::snprintf(buf, sizeof buf, "tc_%05u.h5", C.resume_ind);
    const std::string fn = out + "/" + buf;
    std::cout << "Loading from file: " << fn << std::endl;
    h5l::Reader r;
    if (!r.open(fn)) return iofail(PG_EIO, fn + ": " + r.error());
    const uint32_t D = dim;
    resume_cur.resize((size_t)S->N * D);
    resume_vel.resize(resume_cur.size());
    resume_acc.resize(resume_cur.size());
    for (uint32_t g = 0; g < S->G; ++g) {
      char gb[32];
      std::snprintf(gb, sizeof gb, "P_%05u/", g);
      const std::string pre(gb);
      const uint32_t n0 = S->node_off[g], n = S->node_off[g + 1] - n0;
      std::vector<uint64_t> dims;
      std::vector<double> v;
      auto rd = [&](const char* name, std::vector<double>* dst) {
        if (!r.read_vec(pre + name, h5l::DType::F64, &dims, &v) || dims.size() != 2 || dims[0] != n || dims[1] < D)
          return false;
        for (uint32_t i = 0; i < n; ++i)
          for (uint32_t c = 0; c < D; ++c) (*dst)[(size_t)(n0 + i) * D + c] = v[(size_t)i * dims[1] + c];
        return true;
      };
      if (!rd("CurrPos", &resume_cur) || !rd("vel", &resume_vel) || !rd("acc", &resume_acc))
        return iofail(PG_EIO, fn + ": " + pre + " state missing or wrong shape");
      if (C.enable_fracture) {
        std::vector<uint32_t> conn;
        if (!r.read_vec(pre + "Connectivity", h5l::DType::U32, &dims, &conn))
          return iofail(PG_EIO, fn + ": " + pre + "Connectivity: " + r.error());
        rc = pg_setup_set_connectivity(S, g, conn.data(), conn.size() / 2);
        if (rc) return rc;
      }
    }
    for (size_t k = 0; k < resume_cur.size(); ++k) S->disp[k] = resume_cur[k] - S->pos[k];
    S->vel = resume_vel;
    S->acc = resume_acc;
    if (C.wall_resume) {
      std::snprintf(buf, sizeof buf, "wall_%05u.h5", C.resume_ind);
      const std::string fw = out + "/" + buf;
      std::cout << "Loading wall from file: " << fw << std::endl;
      h5l::Reader rw;
      std::vector<uint64_t> dims;
      std::vector<double> v;
      if (!rw.open(fw) || !rw.read_vec("wall_info", h5l::DType::F64, &dims, &v) || v.size() < 2 * dim)
        return iofail(PG_EIO, fw + ": wall_info missing");
      for (uint32_t k = 0; k < 2 * dim; ++k) S->wall_geom[k] = v[k];
    }
    std::cout << "Resuming from counter " << counter << std::endl;
  } else {
    counter = 1;
    first_counter = counter;
    last_counter = C.timesteps / C.modulo;
  }

  // plotinfo.h5 (timeloop.h:560-582)
  {
    h5l::Writer w;
    uint32_t flc[2] = {first_counter, last_counter}, dd = dim, mo = C.modulo;
    int32_t aw = S->allow_wall;
    w.add_dataset("f_l_counter", h5l::DType::U32, {2, 1}, flc);
    w.add_dataset("dimension", h5l::DType::U32, {1, 1}, &dd);
    w.add_dataset("dt", h5l::DType::F64, {1, 1}, &C.dt);
    w.add_dataset("modulo", h5l::DType::U32, {1, 1}, &mo);
    w.create_group("/wall");
    w.add_dataset("/wall/allow_wall", h5l::DType::I32, {1, 1}, &aw);
    w.add_dataset("/wall/geom_wall_info", h5l::DType::F64, {2ull * dim, 1}, S->wall_geom);
    if (!w.write(out + "/plotinfo.h5")) return iofail(PG_EIO, "cannot write plotinfo.h5");
  }

  pg_setup_desc desc;
  pg_setup_desc_get(S, &desc);
  pg_config cfg;
  pg_config_default(&cfg);
  cfg.dt = C.dt;
  cfg.enable_fracture = C.enable_fracture;
  cfg.nl_bdry_only = C.nl_bdry_only;
  cfg.allow_damping = C.allow_damping;
  cfg.allow_friction = C.allow_friction;
  cfg.self_contact = C.self_contact;
  cfg.enable_torque = C.enable_torque;
  cfg.gradient_extforce = C.gradient_extforce;
  cfg.extforce_maxstep = C.extforce_maxstep;
  cfg.precision = precision;
  cfg.first_step = 1;
  // PERIGRAIN_TIMELOOP=worm: the reference's run_timeloop_worm (timeloop.h:1018-1369) instead of
  // run_timeloop -- no hooks, no Connectivity in tc_ files, its progress line
  const char* tl_env = std::getenv("PERIGRAIN_TIMELOOP");
  const bool worm = tl_env && std::string(tl_env) == "worm";
  cfg.timeloop = worm ? 1 : 0;
  pg_handle* H = nullptr;
  rc = pg_create(&desc, &cfg, &H);
  if (rc) return iofail(rc, std::string("pg_create: ") + pg_last_error());
  std::unique_ptr<pg_handle, int (*)(pg_handle*)> hguard(H, pg_destroy);

  time_t my_time = time(NULL);
  std::cout << "----------------------------------------------------------------------" << std::endl;
  std::cout << "Starting time loop (Parallel=" << C.is_parallel << "): " << ctime(&my_time);
  const int column_w = 12;
  char str_count[64];
  std::snprintf(str_count, sizeof str_count, "count[%d:%d]", first_counter, last_counter);
  std::cout << std::left << std::setw(column_w) << "t " << std::left << std::setw(column_w) << str_count
            << std::left << std::setw(column_w) << "duration(s)" << std::left << std::setw(column_w + 5)
            << "rem(h:m:s.ms)" << std::left << std::setw(column_w) << "date" << std::endl;

  auto start_time = std::chrono::system_clock::now();
  std::vector<double> run_time, t_ind;
  // PERIGRAIN_TIMESTEP_DATA=1: the time series gen_timestep_data.py / gen_damage_data.py /
  // gen_wall_reaction.py build from the output files, computed on the device at each output
  const char* tsd_env = std::getenv("PERIGRAIN_TIMESTEP_DATA");
  const bool tsd = tsd_env && *tsd_env && std::string(tsd_env) != "0";
  const uint32_t NSd = 2 * dim;
  std::vector<double> ts_time, ts_wall, ts_react, ts_phi, ts_dmg, ts_force, ts_vel, ts_acc, ts_pos, ts_fsum;
  const uint32_t T = C.timesteps;
  uint64_t too_close_seen = 0;

  // Output is pipelined: the snapshot of output step e is taken on the device (pg_snapshot) into
  // one of a ring of page-locked buffer sets while the GPU runs the next segment, and its files
  // are written by a pool of writer threads, several outputs at once (each output is its own pair
  // of files). Progress lines are printed in output order, before a hook's message at the step
  // after them, as the reference prints them.
  const size_t nd = (size_t)S->N * dim;
  const size_t set_bytes = 4 * nd * sizeof(double) + S->bond_local.size() + 1;
  uint32_t n_writers = 0;
  if (C.save_file && C.modulo) {
    const char* w_env = std::getenv("PERIGRAIN_WRITERS");
    long w = w_env && *w_env ? std::strtol(w_env, nullptr, 10) : 8;
    w = std::max(1L, std::min(16L, w));
    // at most ~4 GB of page-locked buffers
    while (w > 1 && (size_t)(w + 1) * set_bytes > ((size_t)4 << 30)) --w;
    n_writers = (uint32_t)w;
  }
  OutputPool pool(H, S, out, !worm, n_writers);
  if (n_writers && (rc = pool.alloc(nd, S->bond_local.size(), dim))) return iofail(rc, pg_last_error());
  // finalise the oldest output (its files written): messages, time series, progress line
  auto finalize_one = [&]() -> int {
    OutSet* o = pool.pop_done();
    if (o->rc) return iofail(o->rc, o->err);
    for (; too_close_seen < o->too_close; ++too_close_seen) std::cout << "Error: nodes too close" << std::endl;
    if (tsd) {
      ts_time.push_back((double)o->counter * C.dt * (double)C.modulo);  // extract_bulk: t * dt * modulo
      ts_wall.insert(ts_wall.end(), o->wall.begin(), o->wall.end());
      ts_react.insert(ts_react.end(), o->react.begin(), o->react.end());
      ts_phi.push_back(o->phi[0]);
      ts_dmg.insert(ts_dmg.end(), o->dmg.begin(), o->dmg.end());
      ts_force.insert(ts_force.end(), o->f.begin(), o->f.end());
      ts_vel.insert(ts_vel.end(), o->v.begin(), o->v.end());
      ts_acc.insert(ts_acc.end(), o->a.begin(), o->a.end());
      ts_pos.insert(ts_pos.end(), o->x.begin(), o->x.end());
      ts_fsum.insert(ts_fsum.end(), o->fs.begin(), o->fs.end());
    }
    auto stop_time = std::chrono::system_clock::now();
    auto duration = std::chrono::duration_cast<std::chrono::milliseconds>(stop_time - start_time);
    start_time = stop_time;
    int avgsteps = 10;
    double avg_duration = 0;
    if (run_time.size() >= 10) {
      for (size_t cc = run_time.size() - avgsteps; cc < run_time.size(); ++cc) avg_duration += run_time[cc];
      avg_duration /= avgsteps;
    }
    int rem_counts = (int)last_counter - (int)o->counter;
    if (worm) {
      // the worm loop's line (timeloop.h:1331-1350): t, counter, duration/100, remaining m s, ctime
      avg_duration = 0;
      if (run_time.size() >= 10)
        for (size_t cc = run_time.size() - avgsteps; cc < run_time.size(); ++cc) avg_duration += run_time[cc];
      avg_duration /= avgsteps;
      const double rem_min = (rem_counts * avg_duration) / 1e3 / 60;
      time_t now = time(NULL);
      std::cout << o->e << "\t" << o->counter << "\t" << duration.count() / 100 << "\t" << (int)rem_min << "m"
                << (rem_min - (int)rem_min) * 60 << "s" << "\t" << ctime(&now);
    } else {
      int rem_s = (int)((rem_counts * avg_duration) / 1e3);
      char rem[32];
      std::snprintf(rem, sizeof rem, "%02d:%02d:%02d", (rem_s / 60) / 60, (rem_s / 60) % 60, rem_s % 60);
      time_t now = time(NULL);
      char ts[80];
      strftime(ts, sizeof ts, "%F-%T", localtime(&now));
      std::cout << std::left << std::setw(column_w) << o->e << std::left << std::setw(column_w) << o->counter
                << std::left << std::setw(column_w) << (double)duration.count() / 1000 << std::left
                << std::setw(column_w + 5) << rem << std::left << std::setw(column_w + 10) << ts << std::endl;
    }
    run_time.push_back((double)duration.count());
    t_ind.push_back(o->e);
    pool.release(o);
    return PG_OK;
  };
  OutSet* filling = nullptr;  // snapshot in flight
  // hand the snapshot in flight to the writers (its copies done); with `all`, also wait for
  // every output written and finalise it
  auto flush_outputs = [&](bool all) -> int {
    if (filling) {
      int r = pg_wait(H);
      if (r) return iofail(r, pg_last_error());
      pool.submit(filling);
      filling = nullptr;
    }
    while (pool.front_done(all)) {
      int r = finalize_one();
      if (r) return r;
    }
    return PG_OK;
  };

  uint32_t t = 1;
  while (t <= T) {
    const bool hook_movable = !worm && C.set_movable_index != -1 && (uint32_t)C.set_movable_timestep == t;
    const bool hook_stoppable = !worm && C.set_stoppable_index != -1 && (uint32_t)C.set_stoppable_timestep == t;
    const bool hook_reset = !worm && C.reset_partzero_y && C.reset_partzero_y_timestep == t && S->G > 1;
    if (hook_movable || hook_stoppable || hook_reset)
      if ((rc = flush_outputs(true))) return rc;
    // hooks at the start of step t (timeloop.h:612-650); the worm loop has none
    if (hook_movable) {
      std::cout << "Setting particle " << C.set_movable_index << " to movable on timestep " << t << std::endl;
      if ((rc = pg_set_grain_flags(H, (uint32_t)C.set_movable_index, 1, -1))) return iofail(rc, pg_last_error());
    }
    if (hook_stoppable) {
      std::cout << "Setting particle " << C.set_stoppable_index << " to stoppable on timestep " << t << std::endl;
      if ((rc = pg_set_grain_flags(H, (uint32_t)C.set_stoppable_index, -1, 1))) return iofail(rc, pg_last_error());
    }
    if (hook_reset) {
      std::vector<double> pos((size_t)S->N * dim), disp(pos.size());
      if ((rc = pg_get_field(H, PG_FIELD_POS, pos.data())) || (rc = pg_get_field(H, PG_FIELD_DISP, disp.data())))
        return iofail(rc, pg_last_error());
      const uint32_t b1 = S->node_off[1];
      double max_bulk_y = pos[(size_t)b1 * dim + 1] + disp[(size_t)(b1 + 1) * dim + 1];
      for (uint32_t i = b1; i < S->N; ++i) {
        double now_y = pos[(size_t)i * dim + 1] + disp[(size_t)i * dim + 1];
        if (now_y > max_bulk_y) max_bulk_y = now_y;
      }
      double dest = max_bulk_y + C.wheel_rad + S->contact_radius;
      double mean_y = 0;
      const uint32_t n0 = S->node_off[1] - S->node_off[0];
      for (uint32_t j = 0; j < n0; ++j) mean_y += (pos[(size_t)j * dim + 1] + disp[(size_t)j * dim + 1]);
      mean_y /= n0;
      double to_move_by = dest - mean_y;
      std::cout << "Setting particle zero mean y val to  " << dest << std::endl;
      for (uint32_t j = 0; j < n0; ++j) pos[(size_t)j * dim + 1] += to_move_by;
      if ((rc = pg_set_field(H, PG_FIELD_POS, pos.data()))) return iofail(rc, pg_last_error());
    }
    // run up to the next output step or hook
    uint32_t e = T;
    if (C.save_file && C.modulo) e = std::min<uint32_t>(e, ((t + C.modulo - 1) / C.modulo) * C.modulo);
    auto hook = [&](int64_t ts) {
      if (ts > (int64_t)t && ts - 1 < (int64_t)e) e = (uint32_t)(ts - 1);
    };
    if (!worm && C.set_movable_index != -1) hook((uint32_t)C.set_movable_timestep);
    if (!worm && C.set_stoppable_index != -1) hook((uint32_t)C.set_stoppable_timestep);
    if (!worm && C.reset_partzero_y) hook(C.reset_partzero_y_timestep);
    if (e < t) e = t;
    if ((rc = pg_step(H, e - t + 1))) return iofail(rc, pg_last_error());
    // the previous output goes to the writers while these steps run
    if ((rc = flush_outputs(false))) return rc;
    t = e + 1;
    if (C.save_file && C.modulo && (e % C.modulo) == 0) {
      OutSet* o = pool.acquire();  // a free buffer set: may wait for the oldest output's files
      if (!o) {
        if ((rc = finalize_one())) return rc;
        o = pool.acquire();
      }
      pg_snapshot_desc sd{};
      sd.currpos = o->cur;
      sd.vel = o->vel;
      sd.acc = o->acc;
      sd.force = o->force;
      sd.bond_alive = worm ? nullptr : o->alive;
      sd.wall = o->wall.data();
      sd.reaction = o->react.data();
      sd.too_close_events = &o->too_close;
      if ((rc = pg_snapshot(H, &sd))) return iofail(rc, pg_last_error());
      o->counter = counter;
      o->e = e;
      filling = o;
      if (tsd) {
        const uint32_t G = S->G;
        o->v.assign((size_t)G * dim, 0.0);
        o->a = o->x = o->f = o->v;
        o->dmg.assign(G, 0.0);
        o->fs.assign(dim, 0.0);
        o->phi.assign(1, 0.0);
        pg_post po{};
        po.grain_mean_vel = o->v.data();
        po.grain_mean_acc = o->a.data();
        po.grain_mean_currpos = o->x.data();
        po.grain_force = o->f.data();
        po.grain_damage = o->dmg.data();
        po.inertial_force = o->fs.data();
        po.volume_fraction = o->phi.data();
        if ((rc = pg_postprocess(H, &po))) return iofail(rc, pg_last_error());
      }
      ++counter;
    }
  }
  if ((rc = flush_outputs(true))) return rc;
  if ((rc = pg_synchronize(H))) return iofail(rc, pg_last_error());
  {
    h5l::Writer w;
    w.add_dataset("run_time", h5l::DType::F64, {run_time.size(), 1}, run_time.data());
    w.add_dataset("t_ind", h5l::DType::F64, {t_ind.size(), 1}, t_ind.data());
    if (!w.write(out + "/run_time.h5")) return iofail(PG_EIO, "cannot write run_time.h5");
  }
  if (tsd) {
    // one row per output step, field names of gen_timestep_data.py (plus the damage and f_sum of
    // gen_damage_data.py / read_force_val)
    h5l::Writer w;
    const uint64_t T = ts_time.size(), G = S->G;
    w.add_dataset("time", h5l::DType::F64, {T}, ts_time.data());
    w.add_dataset("wall_loc", h5l::DType::F64, {T, NSd}, ts_wall.data());
    w.add_dataset("wall_force", h5l::DType::F64, {T, NSd, dim}, ts_react.data());
    w.add_dataset("volume_fraction", h5l::DType::F64, {T}, ts_phi.data());
    w.add_dataset("particle_damage", h5l::DType::F64, {T, G}, ts_dmg.data());
    w.add_dataset("particle_force", h5l::DType::F64, {T, G, dim}, ts_force.data());
    w.add_dataset("particle_mean_vel", h5l::DType::F64, {T, G, dim}, ts_vel.data());
    w.add_dataset("particle_mean_acc", h5l::DType::F64, {T, G, dim}, ts_acc.data());
    w.add_dataset("particle_mean_CurrPos", h5l::DType::F64, {T, G, dim}, ts_pos.data());
    w.add_dataset("f_sum", h5l::DType::F64, {T, dim}, ts_fsum.data());
    if (!w.write(out + "/timestep_data.h5")) return iofail(PG_EIO, "cannot write timestep_data.h5");
  }
  auto stop_all = std::chrono::system_clock::now();
  std::cout << "Runtime: " << std::chrono::duration_cast<std::chrono::seconds>(stop_all - start_all).count()
            << "s" << std::endl;
  return PG_OK;
}

// =============================================================================================
// HDF5 subset C API
// =============================================================================================
struct pg_h5w {
  h5l::Writer w;
};

extern "C" pg_h5w* pg_h5w_new(void) { return new pg_h5w; }
extern "C" void pg_h5w_free(pg_h5w* w) { delete w; }

extern "C" int pg_h5w_add(pg_h5w* w, const char* path, int32_t dtype, uint32_t rank, const uint64_t* dims,
                          const void* data) {
  if (!w || !path || dtype < 0 || dtype > 6 || rank > 8) return PG_EINVAL;
  std::vector<uint64_t> d(dims, dims + rank);
  return w->w.add_dataset(path, (h5l::DType)dtype, d, data) ? PG_OK : PG_EINVAL;
}

extern "C" int pg_h5w_group(pg_h5w* w, const char* path) {
  if (!w || !path) return PG_EINVAL;
  w->w.create_group(path);
  return PG_OK;
}

extern "C" int pg_h5w_write(pg_h5w* w, const char* filename) {
  if (!w || !filename) return PG_EINVAL;
  return w->w.write(filename) ? PG_OK : PG_EIO;
}

extern "C" int pg_h5_info(const char* filename, const char* path, uint32_t* rank, uint64_t* dims,
                          int32_t* type_class, uint32_t* type_size, int32_t* is_signed) {
  h5l::Reader r;
  if (!r.open(filename)) return iofail(PG_EIO, r.error());
  h5l::DatasetInfo di;
  if (!r.info(path, &di)) {
    io_err = r.error();
    return PG_EIO;
  }
  if (di.dims.size() > 8) return PG_EINVAL;
  if (rank) *rank = (uint32_t)di.dims.size();
  if (dims)
    for (size_t i = 0; i < di.dims.size(); ++i) dims[i] = di.dims[i];
  if (type_class) *type_class = di.type_class;
  if (type_size) *type_size = di.type_size;
  if (is_signed) *is_signed = di.is_signed;
  return PG_OK;
}

extern "C" int pg_h5_read(const char* filename, const char* path, int32_t dtype, void* out, uint64_t capacity) {
  if (dtype < 0 || dtype > 6) return PG_EINVAL;
  h5l::Reader r;
  if (!r.open(filename)) {
    io_err = r.error();
    return PG_EIO;
  }
  std::vector<uint64_t> dims;
  std::vector<uint8_t> raw;
  if (!r.read(path, (h5l::DType)dtype, &dims, &raw)) {
    io_err = r.error();
    return PG_EIO;
  }
  const size_t es = h5l::dtype_size((h5l::DType)dtype);
  if (raw.size() / es > capacity) return PG_EINVAL;
  if (!raw.empty()) std::memcpy(out, raw.data(), raw.size());
  return PG_OK;
}

extern "C" int pg_h5_list(const char* filename, const char* path, char* buf, uint64_t bufsize) {
  h5l::Reader r;
  if (!r.open(filename)) {
    io_err = r.error();
    return PG_EIO;
  }
  std::vector<std::string> names;
  if (!r.list(path ? path : "", &names)) {
    io_err = r.error();
    return PG_EIO;
  }
  std::string s;
  for (auto& n : names) s += n + "\n";
  if (s.size() + 1 > bufsize) return PG_EINVAL;
  std::memcpy(buf, s.c_str(), s.size() + 1);
  return PG_OK;
}
