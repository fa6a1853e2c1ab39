// TEST INFRASTRUCTURE -- the oracle. Not part of the product; only tests/, smoke() and the
// CPU-baseline leg of bench.py load it, as the checker.
//
// A plain C++ restatement of the reference's time step (debdeepbh/perigrain), FP64, serial,
// with the reference's data structures (per-grain neighbour lists with order-preserving erase)
// and its operation order. Compiled with -ffp-contract=off. It follows, line by line:
//   position update        src/particle/timeloop.h:661-669
//   bond force             src/particle/particle2.h:102-150
//   bond removal           src/particle/particle2.h:191-232
//   gen_xi                 src/particle/particle2.h:236-252
//   contact (self, other)  src/particle/contact.h:668-812, called from timeloop.h:709-747
//   bounding boxes         src/particle/contact.h:984-1062, :1066-1080
//   wall                   src/particle/contact.h:900-964 -> :314-431 -> :16-41
//   external force/torque  src/particle/timeloop.h:774-824, mean_CurrPos particle2.h:89-98
//   velocity update        src/particle/timeloop.h:834-863
//   wall move              src/particle/timeloop.h:866-878
// The one liberty: node pairs are enumerated from a uniform cell grid instead of all n_i x n_j
// pairs, then visited in the reference's loop order (self-contact first, then grains j
// ascending, nodes in loop order); pairs farther apart than the contact radius contribute
// nothing in the reference, so the result is identical. This is checked bit-for-bit against the
// reference compiled unmodified (oracle/Makefile, tests/test_oracle_vs_reference.py).
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "../include/perigrain.h"

namespace {

struct Grain {
  uint32_t n = 0, gid0 = 0;
  std::vector<double> pos, disp, cur, vel, acc, force, extf, vol;  // flattened, D per node
  std::vector<std::vector<uint32_t>> nbd;                          // NbdArr
  std::vector<std::vector<uint64_t>> bid;                          // original bond index
  std::vector<std::vector<double>> xi;                             // D per entry
  std::vector<std::vector<double>> xi_norm, stretch;
  std::vector<uint32_t> bdry, clamped;
  std::vector<uint32_t> loop_pos;  // position in the contact loop list (bdry order or identity)
  double delta, rho, cnot, snot;
  int movable, breakable, stoppable;
  bool break_bonds;
  uint32_t torque_axis;
  double torque_val;
  uint32_t inst;
};

struct Inst {
  double Rc, Kn, mu, zeta;
  int allow_wall;
  double wall[6], speed[6];
  double reaction[6][3];
  uint32_t g0, g1;  // grain range
};

uint64_t splitmix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

}  // namespace

struct orc_sim {
  uint32_t D = 2;
  std::vector<Grain> G;
  std::vector<Inst> I;
  pg_config cfg;
  uint64_t t = 1;
  uint64_t nbonds = 0;
  std::vector<uint32_t> break_step;
  std::vector<uint64_t> log_count, log_hash;
  uint64_t too_close = 0;
  // reference_structured: enumerate node pairs the way the reference does (all n_i x n_j pairs
  // of bbox-touching grains, std::find before the distance test, bounding boxes recomputed per
  // grain pair, the two grains copied per contact call) -- same arithmetic, the reference's cost.
  int reference_structured = 0;
  int threads = 1;

  double& v(std::vector<double>& a, uint32_t i, uint32_t c) { return a[(size_t)i * D + c]; }

  // get_minmax (contact.h:1024-1062): 2D [xmin, xmax, ymax, ymin], 3D [x0, y0, z0, x1, y1, z1]
  std::vector<double> minmax(const Grain& g) const {
    std::vector<double> out;
    const double* P = g.cur.data();
    if (D == 2) {
      out = {P[0], P[0], P[1], P[1]};
      for (uint32_t i = 0; i < g.n; ++i) {
        out[0] = std::min(out[0], P[i * 2 + 0]);
        out[1] = std::max(out[1], P[i * 2 + 0]);
        out[2] = std::max(out[2], P[i * 2 + 1]);
        out[3] = std::min(out[3], P[i * 2 + 1]);
      }
    } else {
      out = {P[0], P[1], P[2], P[0], P[1], P[2]};
      for (uint32_t i = 0; i < g.n; ++i) {
        out[0] = std::min(out[0], P[i * 3 + 0]);
        out[1] = std::min(out[1], P[i * 3 + 1]);
        out[2] = std::min(out[2], P[i * 3 + 2]);
        out[3] = std::max(out[3], P[i * 3 + 0]);
        out[4] = std::max(out[4], P[i * 3 + 1]);
        out[5] = std::max(out[5], P[i * 3 + 2]);
      }
    }
    return out;
  }
  bool intersects(const std::vector<double>& A, const std::vector<double>& B, double c) const {
    if (D == 2) {
      double AL = A[0] - c, AR = A[1] + c, AT = A[2] + c, AB = A[3] - c;
      return (AL <= B[1]) && (AR >= B[0]) && (AT >= B[3]) && (AB <= B[2]);
    }
    double ax0 = A[0] - c, ay0 = A[1] - c, az0 = A[2] - c, ax1 = A[3] + c, ay1 = A[4] + c, az1 = A[5] + c;
    return (ax0 <= B[3]) && (ax1 >= B[0]) && (ay1 >= B[1]) && (ay0 <= B[4]) && (az0 <= B[5]) && (az1 >= B[2]);
  }
  static bool within_interior(const std::vector<double>& A, const double* B, double c) {
    double AL = A[0] - c, AR = A[1] + c, AT = A[2] + c, AB = A[3] - c;
    return (B[0] < AL) && (AR < B[1]) && (B[2] > AT) && (B[3] < AB);
  }

  double norm(const double* x) const {
    double s = x[0] * x[0];
    for (uint32_t c = 1; c < D; ++c) s = s + x[c] * x[c];
    return std::sqrt(s);
  }

  // ---- get_peridynamic_force (particle2.h:102-150) ----
  void bond_force(Grain& g, std::vector<double>& ft) {
    for (uint32_t i = 0; i < g.n; ++i) {
      double acc[3] = {0, 0, 0};
      for (size_t j = 0; j < g.nbd[i].size(); ++j) {
        uint32_t q = g.nbd[i][j];
        double e[3];
        for (uint32_t c = 0; c < D; ++c) e[c] = (g.disp[q * D + c] - g.disp[i * D + c]) + g.xi[i][j * D + c];
        double en = norm(e);
        double xn = g.xi_norm[i][j];
        double diff = (en - xn);
        double str = diff / xn;
        double sc = (g.cnot * str) * g.vol[q];
        for (uint32_t c = 0; c < D; ++c) acc[c] += sc * (e[c] / en);
        g.stretch[i][j] = str;
      }
      for (uint32_t c = 0; c < D; ++c) ft[i * D + c] = acc[c];
    }
  }

  // ---- remove_bonds (particle2.h:191-232) ----
  void remove_bonds(Grain& g) {
    if (!g.break_bonds) return;
    for (uint32_t i = 0; i < g.n; ++i) {
      size_t w = 0;
      for (size_t j = 0; j < g.nbd[i].size(); ++j) {
        if (g.stretch[i][j] > g.snot) {
          break_step[g.bid[i][j]] = (uint32_t)t;
          continue;
        }
        g.nbd[i][w] = g.nbd[i][j];
        g.bid[i][w] = g.bid[i][j];
        for (uint32_t c = 0; c < D; ++c) g.xi[i][w * D + c] = g.xi[i][j * D + c];
        g.xi_norm[i][w] = g.xi_norm[i][j];
        g.stretch[i][w] = g.stretch[i][j];
        ++w;
      }
      g.nbd[i].resize(w);
      g.bid[i].resize(w);
      g.xi[i].resize(w * D);
      g.xi_norm[i].resize(w);
      g.stretch[i].resize(w);
    }
  }

  // ---- one node pair of update_contact_force_by_boundary (contact.h:683-809) ----
  void pair(Grain& C, uint32_t i, Grain& Nn, uint32_t j, bool self, const Inst& in, double* fi,
            uint64_t* pc, uint64_t* ph) {
    double dir[3];
    for (uint32_t c = 0; c < D; ++c) dir[c] = Nn.cur[j * D + c] - C.cur[i * D + c];
    double dn = norm(dir);
    bool do_compute = true;
    double Rc = in.Rc, Kn = in.Kn;
    if (self) {
      if (i == j) {
        do_compute = false;
      } else if (std::find(C.nbd[i].begin(), C.nbd[i].end(), j) != C.nbd[i].end()) {
        do_compute = false;
      } else {
        double r[3];
        for (uint32_t c = 0; c < D; ++c) r[c] = C.pos[i * D + c] - C.pos[j * D + c];
        double ref = norm(r);
        if (ref < in.Rc) {
          Rc = ref;
          Kn = C.cnot / ref;
        } else {
          Rc = in.Rc;
          Kn = C.cnot / in.Rc;
        }
      }
    }
    if (!(do_compute && (dn <= Rc))) return;
    *pc += 1;
    *ph += splitmix64(((uint64_t)(C.gid0 + i) << 32) | (uint64_t)(Nn.gid0 + j));
    if (dn == 0) {
#pragma omp atomic
      ++too_close;
    }
    double u[3], fc[3];
    for (uint32_t c = 0; c < D; ++c) u[c] = dir[c] / dn;
    double crc = (Rc - dn);
    double nvol = Nn.vol[j];
    double s1 = -Kn * crc * nvol;
    for (uint32_t c = 0; c < D; ++c) fc[c] = s1 * u[c];
    double cfn = norm(fc);
    for (uint32_t c = 0; c < D; ++c) fi[c] += fc[c];
    if (cfg.allow_damping) {
      double rv[3];
      for (uint32_t c = 0; c < D; ++c) rv[c] = C.vel[i * D + c] - Nn.vel[j * D + c];
      double proj = rv[0] * u[0];
      for (uint32_t c = 1; c < D; ++c) proj = proj + rv[c] * u[c];
      double dc = 2 * in.zeta * std::sqrt(Kn * C.rho) * std::sqrt(nvol);
      for (uint32_t c = 0; c < D; ++c) fi[c] += (-dc) * (proj * u[c]);
    }
    if (cfg.allow_friction) {
      double rv[3], tg[3];
      for (uint32_t c = 0; c < D; ++c) rv[c] = C.vel[i * D + c] - Nn.vel[j * D + c];
      double proj = rv[0] * u[0];
      for (uint32_t c = 1; c < D; ++c) proj = proj + rv[c] * u[c];
      for (uint32_t c = 0; c < D; ++c) tg[c] = rv[c] - proj * u[c];
      double tn = norm(tg);
      if (tn > 0) {
        double ut[3], ff[3];
        for (uint32_t c = 0; c < D; ++c) ut[c] = tg[c] / tn;
        for (uint32_t c = 0; c < D; ++c) ff[c] = -in.mu * cfn * ut[c];
        if (tn < in.mu * cfn * cfg.dt / C.rho) {
          for (uint32_t c = 0; c < D; ++c) ff[c] = -tn / C.rho / cfg.dt * ut[c];
        }
        for (uint32_t c = 0; c < D; ++c) fi[c] += ff[c];
      }
    }
  }

  // ---- wall_side_force_update (contact.h:314-431) with segment_mass (contact.h:16-41) ----
  void wall_side(double dist, uint32_t dir, const double* vel_i, double vol_i, double rho, double* f,
                 double wspeed, double* react, const Inst& in) {
    const double R = in.Rc;
    if (!(std::fabs(dist) <= R)) return;
    double d = std::fabs(dist);
    double Area, Ic;
    if (D == 2) {
      Area = M_PI * std::pow(R, 2) / 2 - std::pow(R, 2) * std::asin(d / R) - std::sqrt(R * R - d * d) * d;
      Ic = 2 / 3 * std::pow((R * R - d * d), 1.5);
    } else {
      Area = M_PI / 3 * std::pow((R - d), 2) * (2 * R - d);
      Ic = M_PI / 4 * std::pow(std::pow(R, 2) - std::pow(d, 2), 2);
    }
    double centroid = Ic / Area;
    double crc = (R - centroid);
    double pcrc = (crc > 0 ? crc : 0);
    double F = (in.Kn * pcrc * Area);
    double c_sign = (dist > 0 ? 1 : -1);
    f[dir] += (c_sign * F);
    react[dir] -= (vol_i * c_sign * F);
    double rv[3];
    for (uint32_t c = 0; c < D; ++c) rv[c] = vel_i[c];
    rv[dir] -= wspeed;
    if (cfg.allow_friction) {
      if (D == 2) {
        uint32_t tg = (dir + 1) % 2;
        if (std::fabs(rv[tg]) > 0) {
          double vts = (rv[tg] > 0 ? 1 : -1);
          double ff = (-in.mu) * std::fabs(F) * vts;
          if (std::fabs(rv[tg]) < in.mu * std::fabs(F) * cfg.dt / rho) ff = -rv[tg] * rho / cfg.dt;
          f[tg] += ff;
          react[tg] -= (vol_i * ff);
        }
      } else {
        uint32_t t1 = (dir + 1) % 3, t2 = (dir + 2) % 3;
        double v1 = rv[t1], v2 = rv[t2];
        double vn = std::sqrt(std::pow(v1, 2) + std::pow(v2, 2));
        if (vn > 0) {
          double u1 = v1 / vn, u2 = v2 / vn;
          double f1 = (-in.mu) * std::fabs(F) * u1;
          double f2 = (-in.mu) * std::fabs(F) * u2;
          if (vn < in.mu * std::fabs(F) * cfg.dt / rho) {
            f1 = -vn / rho / cfg.dt * u1;
            f2 = -vn / rho / cfg.dt * u2;
          }
          f[t1] += f1;
          f[t2] += f2;
          react[t1] -= (vol_i * f1);
          react[t2] -= (vol_i * f2);
        }
      }
    }
    if (cfg.allow_damping) {
      double dc = 2 * in.zeta * std::sqrt(in.Kn * rho) * std::sqrt(std::fabs(Area));
      double df = (-dc) * rv[dir];
      f[dir] += df;
      react[dir] -= (vol_i * df);
    }
  }

  struct CellKey {
    int64_t x, y, z;
    bool operator==(const CellKey& o) const { return x == o.x && y == o.y && z == o.z; }
  };
  struct CellHash {
    size_t operator()(const CellKey& k) const {
      return (size_t)splitmix64((uint64_t)k.x * 73856093ull ^ (uint64_t)k.y * 19349663ull ^ (uint64_t)k.z * 83492791ull);
    }
  };

  // The reference's loop structure (timeloop.h:709-747 -> contact.h:668-812): self-contact over
  // all node pairs of grain i, then every other grain j whose extended bounding box (recomputed
  // for each pair, timeloop.h:723-730) touches, over all node pairs; each call works on copies
  // of both grains (contact.h:669 passes ParticleN by value).
  void contact_reference_structured(Inst& in, uint32_t gi, bool self, std::vector<double>& ft, uint64_t* pc,
                                    uint64_t* ph) {
    Grain& g = G[gi];
    auto loop_list = [&](const Grain& h) {
      std::vector<uint32_t> l;
      if (cfg.nl_bdry_only) return h.bdry;
      for (uint32_t i = 0; i < h.n; ++i) l.push_back(i);
      return l;
    };
    auto visit = [&](Grain& C, Grain& Nn, bool is_self) {
      std::vector<uint32_t> li = loop_list(C), lj = loop_list(Nn);
      for (uint32_t i : li)
        for (uint32_t j : lj) pair(C, i, Nn, j, is_self, in, &ft[i * D], pc, ph);
    };
    if (self && cfg.self_contact) {
      Grain c1 = g, c2 = g;
      visit(c1, c2, true);
    }
    if (g.stoppable || cfg.timeloop == 1) {
      std::vector<double> C = minmax(g);
      for (uint32_t gj = in.g0; gj < in.g1; ++gj) {
        if (gj == gi) continue;
        std::vector<double> Nb = minmax(G[gj]);
        if (intersects(C, Nb, in.Rc)) {
          Grain c1 = g, c2 = G[gj];
          visit(c1, c2, false);
        }
      }
    }
  }

  void force_instance(Inst& in, const std::vector<std::vector<double>>& boxes, uint64_t* pcp, uint64_t* php) {
    uint64_t pc = 0, ph = 0;
    const bool worm = cfg.timeloop == 1;
    {
      // cell grid of this instance
      const double cell = in.Rc > 0 ? in.Rc * 1.01 : 1.0;
      std::unordered_map<CellKey, std::vector<std::pair<uint32_t, uint32_t>>, CellHash> grid;
      auto key_of = [&](const double* x) {
        CellKey k{0, 0, 0};
        k.x = (int64_t)std::floor(x[0] / cell);
        k.y = (int64_t)std::floor(x[1] / cell);
        if (D == 3) k.z = (int64_t)std::floor(x[2] / cell);
        return k;
      };
      for (uint32_t gi = in.g0; gi < in.g1; ++gi)
        for (uint32_t i = 0; i < G[gi].n; ++i) grid[key_of(&G[gi].cur[i * D])].push_back({gi, i});
      for (uint32_t gi = in.g0; gi < in.g1; ++gi) {
        Grain& g = G[gi];
        std::vector<double> ft((size_t)g.n * D, 0.0);
        if (g.movable) {
          bond_force(g, ft);
          const bool self = cfg.enable_fracture && g.breakable;
          if (self) remove_bonds(g);
          if (reference_structured) {
            contact_reference_structured(in, gi, self, ft, &pc, &ph);
          } else
          // candidate lists per node: (order key, grain, node)
          for (uint32_t i = 0; i < g.n; ++i) {
            if (cfg.nl_bdry_only && g.loop_pos[i] == UINT32_MAX) continue;
            std::vector<std::tuple<uint64_t, uint32_t, uint32_t>> cand;
            CellKey k0 = key_of(&g.cur[i * D]);
            for (int dz = (D == 3 ? -1 : 0); dz <= (D == 3 ? 1 : 0); ++dz)
              for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                  auto it = grid.find(CellKey{k0.x + dx, k0.y + dy, k0.z + dz});
                  if (it == grid.end()) continue;
                  for (auto& e : it->second) {
                    const Grain& h = G[e.first];
                    if (cfg.nl_bdry_only && h.loop_pos[e.second] == UINT32_MAX) continue;
                    double dd[3];
                    for (uint32_t c = 0; c < D; ++c) dd[c] = h.cur[e.second * D + c] - g.cur[i * D + c];
                    if (!(norm(dd) <= in.Rc)) continue;
                    uint64_t ord = ((uint64_t)(e.first == gi ? 0 : 1) << 63) | ((uint64_t)e.first << 32) |
                                   h.loop_pos[e.second];
                    cand.emplace_back(ord, e.first, e.second);
                  }
                }
            std::sort(cand.begin(), cand.end());
            double fi[3] = {0, 0, 0};
            for (uint32_t c = 0; c < D; ++c) fi[c] = ft[i * D + c];
            for (auto& cd : cand) {
              uint32_t gj = std::get<1>(cd), j = std::get<2>(cd);
              if (gj == gi) {
                if (self && cfg.self_contact) pair(g, i, g, j, true, in, fi, &pc, &ph);
              } else if ((g.stoppable || worm) && intersects(boxes[gi], boxes[gj], in.Rc)) {
                pair(g, i, G[gj], j, false, in, fi, &pc, &ph);
              }
            }
            for (uint32_t c = 0; c < D; ++c) ft[i * D + c] = fi[c];
          }
          // walls
          if ((g.stoppable || worm) && in.allow_wall && !within_interior(boxes[gi], in.wall, in.Rc)) {
            std::vector<uint32_t> order;
            if (cfg.nl_bdry_only) {
              order = g.bdry;
            } else {
              for (uint32_t i = 0; i < g.n; ++i) order.push_back(i);
            }
            for (uint32_t i : order) {
              double* f = &ft[i * D];
              const double* x = &g.cur[i * D];
              const double* vv = &g.vel[i * D];
              if (D == 2) {
                wall_side(x[1] - in.wall[3], 1, vv, g.vol[i], g.rho, f, in.speed[3], in.reaction[3], in);
                wall_side(x[0] - in.wall[0], 0, vv, g.vol[i], g.rho, f, in.speed[0], in.reaction[0], in);
                wall_side(x[0] - in.wall[1], 0, vv, g.vol[i], g.rho, f, in.speed[1], in.reaction[1], in);
                wall_side(x[1] - in.wall[2], 1, vv, g.vol[i], g.rho, f, in.speed[2], in.reaction[2], in);
              } else {
                wall_side(x[0] - in.wall[0], 0, vv, g.vol[i], g.rho, f, in.speed[0], in.reaction[0], in);
                wall_side(x[0] - in.wall[3], 0, vv, g.vol[i], g.rho, f, in.speed[3], in.reaction[3], in);
                wall_side(x[1] - in.wall[1], 1, vv, g.vol[i], g.rho, f, in.speed[1], in.reaction[1], in);
                wall_side(x[1] - in.wall[4], 1, vv, g.vol[i], g.rho, f, in.speed[4], in.reaction[4], in);
                wall_side(x[2] - in.wall[2], 2, vv, g.vol[i], g.rho, f, in.speed[2], in.reaction[2], in);
                wall_side(x[2] - in.wall[5], 2, vv, g.vol[i], g.rho, f, in.speed[5], in.reaction[5], in);
              }
            }
          }
          // external force; run_timeloop_worm: ft_i += ((t_num + 1) % 2) * extforce, no ramp and
          // no torque (timeloop.h:1171)
          if (worm) {
            const double gate = (double)((worm_phase(t) + 1) % 2);
            for (size_t k = 0; k < ft.size(); ++k) ft[k] += gate * g.extf[k];
          } else if (cfg.gradient_extforce) {
            double sc = (double)t / (double)cfg.extforce_maxstep;
            if (sc > 1) sc = 1;
            for (size_t k = 0; k < ft.size(); ++k) ft[k] += sc * g.extf[k];
          } else {
            for (size_t k = 0; k < ft.size(); ++k) ft[k] += g.extf[k];
          }
          // torque about mean_CurrPos
          if (cfg.enable_torque && !worm) {
            double m[3] = {0, 0, 0};
            for (uint32_t i = 0; i < g.n; ++i)
              for (uint32_t c = 0; c < D; ++c) m[c] += (g.pos[i * D + c] + g.disp[i * D + c]);
            for (uint32_t c = 0; c < D; ++c) m[c] /= g.n;
            uint32_t ta = g.torque_axis;
            for (uint32_t i = 0; i < g.n; ++i) {
              double r[3] = {0, 0, 0}, rp[3] = {0, 0, 0};
              for (uint32_t c = 0; c < D; ++c) r[c] = g.cur[i * D + c] - m[c];
              if (D == 3) r[ta] = 0;
              rp[(ta + 1) % 3] = -r[(ta + 2) % 3];
              rp[(ta + 2) % 3] = r[(ta + 1) % 3];
              double pn = norm(rp);
              if (pn > 0) {
                for (uint32_t c = 0; c < D; ++c) rp[c] /= pn;
              } else {
                rp[(ta + 1) % 3] = 0;
                rp[(ta + 2) % 3] = 0;
              }
              for (uint32_t c = 0; c < D; ++c) ft[i * D + c] += (g.torque_val * rp[c]);
            }
          }
        }
        g.force = ft;
      }
    }
    *pcp += pc;
    *php += ph;
  }

  static uint32_t worm_phase(uint64_t t) { return ((t / 1000) % 3 == 0) ? 0u : 1u; }

  void step() {
    const double dt = cfg.dt;
    for (auto& in : I)
      for (auto& r : in.reaction)
        for (double& x : r) x = 0.0;
    // loop 1: position update
    for (auto& g : G) {
      for (uint32_t i = 0; i < g.n; ++i)
        for (uint32_t c = 0; c < D; ++c) {
          if (g.movable) g.disp[i * D + c] += dt * g.vel[i * D + c] + (dt * dt * 0.5) * g.acc[i * D + c];
          g.cur[i * D + c] = g.pos[i * D + c] + g.disp[i * D + c];
        }
    }
    std::vector<std::vector<double>> boxes(G.size());
    for (size_t k = 0; k < G.size(); ++k) boxes[k] = minmax(G[k]);
    uint64_t pc = 0, ph = 0;
    // loop 2, one instance at a time (instances never interact)
    if (threads > 1) {
#pragma omp parallel for schedule(dynamic) num_threads(threads) reduction(+ : pc, ph)
      for (size_t k = 0; k < I.size(); ++k) force_instance(I[k], boxes, &pc, &ph);
    } else {
      for (auto& in : I) force_instance(in, boxes, &pc, &ph);
    }
    log_count.push_back(pc);
    log_hash.push_back(ph);
    // loop 3: velocity update
    const bool worm = cfg.timeloop == 1;
    for (auto& g : G) {
      if (!g.movable) continue;
      double orho = 1 / g.rho;
      for (uint32_t i = 0; i < g.n; ++i)
        for (uint32_t c = 0; c < D; ++c) {
          double tmp = g.acc[i * D + c];
          g.acc[i * D + c] = orho * g.force[i * D + c];
          tmp += g.acc[i * D + c];
          tmp *= (0.5 * dt);
          g.vel[i * D + c] += tmp;
        }
      for (uint32_t cid : g.clamped)
        for (uint32_t c = 0; c < D; ++c) {
          g.disp[cid * D + c] = 0;
          g.vel[cid * D + c] = 0;
          g.acc[cid * D + c] = 0;
        }
      if (worm) {
        // gait clamps (timeloop.h:1213-1244): nodes 0, 3 or 1, 2 held, then no y motion for 0-3
        const uint32_t ph = worm_phase(t);
        const uint32_t held[2][2] = {{0, 3}, {1, 2}};
        for (uint32_t cid : held[ph])
          for (uint32_t c = 0; c < D; ++c) {
            g.vel[cid * D + c] = 0;
            g.acc[cid * D + c] = 0;
          }
        for (uint32_t cid = 0; cid < 4; ++cid) {
          g.vel[cid * D + 1] = 0;
          g.acc[cid * D + 1] = 0;
        }
      }
    }
    // wall move
    for (auto& in : I)
      for (uint32_t s = 0; s < 2 * D; ++s) in.wall[s] += in.speed[s] * dt;
    ++t;
  }
};

extern "C" {

int orc_create(const pg_setup_desc* s, const pg_config* cfg, orc_sim** out) {
  if (!s || !cfg || !out || (s->dim != 2 && s->dim != 3)) return PG_EINVAL;
  std::unique_ptr<orc_sim> o(new orc_sim);
  const uint32_t D = s->dim;
  o->D = D;
  o->cfg = *cfg;
  o->t = cfg->first_step ? cfg->first_step : 1;
  o->nbonds = s->bond_offset[s->n_nodes];
  o->break_step.assign(o->nbonds, 0);
  o->I.resize(s->n_instances);
  for (uint32_t k = 0; k < s->n_instances; ++k) {
    Inst& in = o->I[k];
    in.Rc = s->contact_radius[k];
    in.Kn = s->normal_stiffness[k];
    in.mu = s->friction_coefficient[k];
    in.zeta = s->damping_ratio[k];
    in.allow_wall = s->allow_wall[k];
    for (uint32_t a = 0; a < 2 * D; ++a) {
      in.wall[a] = s->wall_geom[(size_t)k * 2 * D + a];
      in.speed[a] = s->wall_speed[(size_t)k * 2 * D + a];
    }
    in.g0 = UINT32_MAX;
    in.g1 = 0;
  }
  o->G.resize(s->n_grains);
  for (uint32_t gi = 0; gi < s->n_grains; ++gi) {
    Grain& g = o->G[gi];
    const uint32_t n0 = s->grain_node_offset[gi], n = s->grain_node_offset[gi + 1] - n0;
    g.n = n;
    g.gid0 = n0;
    g.inst = s->grain_instance[gi];
    Inst& in = o->I[g.inst];
    in.g0 = std::min(in.g0, gi);
    in.g1 = std::max(in.g1, gi + 1);
    auto cp = [&](const double* a, std::vector<double>* dst) { dst->assign(a + (size_t)n0 * D, a + (size_t)(n0 + n) * D); };
    cp(s->pos, &g.pos);
    cp(s->disp, &g.disp);
    cp(s->vel, &g.vel);
    cp(s->acc, &g.acc);
    cp(s->extforce, &g.extf);
    g.cur.assign((size_t)n * D, 0.0);
    g.force.assign((size_t)n * D, 0.0);
    g.vol.assign(s->vol + n0, s->vol + n0 + n);
    g.nbd.resize(n);
    g.bid.resize(n);
    g.xi.resize(n);
    g.xi_norm.resize(n);
    g.stretch.resize(n);
    for (uint32_t i = 0; i < n; ++i) {
      for (uint64_t b = s->bond_offset[n0 + i]; b < s->bond_offset[n0 + i + 1]; ++b) {
        uint32_t q = s->bond_local[b];
        g.nbd[i].push_back(q);
        g.bid[i].push_back(b);
      }
      // gen_xi (particle2.h:236-252)
      size_t ss = g.nbd[i].size();
      g.xi[i].resize(ss * D);
      g.xi_norm[i].resize(ss);
      g.stretch[i].resize(ss);
      for (size_t j = 0; j < ss; ++j) {
        uint32_t q = g.nbd[i][j];
        for (uint32_t c = 0; c < D; ++c) g.xi[i][j * D + c] = g.pos[q * D + c] - g.pos[i * D + c];
        g.xi_norm[i][j] = o->norm(&g.xi[i][j * D]);
      }
    }
    g.bdry.assign(s->bdry_nodes + s->bdry_offset[gi], s->bdry_nodes + s->bdry_offset[gi + 1]);
    g.clamped.assign(s->clamped_nodes + s->clamped_offset[gi], s->clamped_nodes + s->clamped_offset[gi + 1]);
    g.loop_pos.assign(n, UINT32_MAX);
    if (cfg->nl_bdry_only) {
      for (uint32_t k = 0; k < g.bdry.size(); ++k) g.loop_pos[g.bdry[k]] = k;
    } else {
      for (uint32_t i = 0; i < n; ++i) g.loop_pos[i] = i;
    }
    g.delta = s->delta[gi];
    g.rho = s->rho[gi];
    g.cnot = s->cnot[gi];
    g.snot = s->snot[gi];
    g.movable = s->movable[gi];
    g.breakable = s->breakable[gi];
    g.stoppable = s->stoppable[gi];
    g.break_bonds = s->break_bonds[gi];
    g.torque_axis = s->torque_axis ? s->torque_axis[gi] : 2;
    g.torque_val = s->torque_val ? s->torque_val[gi] : 0.0;
  }
  *out = o.release();
  return PG_OK;
}

int orc_destroy(orc_sim* o) {
  delete o;
  return PG_OK;
}

int orc_step(orc_sim* o, uint32_t n) {
  for (uint32_t k = 0; k < n; ++k) o->step();
  return PG_OK;
}

int orc_get_field(orc_sim* o, int field, double* out) {
  size_t off = 0;
  for (auto& g : o->G) {
    const std::vector<double>* src = nullptr;
    std::vector<double> tmp;
    switch (field) {
      case PG_FIELD_CURRPOS: src = &g.cur; break;
      case PG_FIELD_VEL: src = &g.vel; break;
      case PG_FIELD_ACC: src = &g.acc; break;
      case PG_FIELD_FORCE: src = &g.force; break;
      case PG_FIELD_DISP: src = &g.disp; break;
      case PG_FIELD_POS: src = &g.pos; break;
      default: return PG_EINVAL;
    }
    std::memcpy(out + off, src->data(), src->size() * 8);
    off += src->size();
  }
  return PG_OK;
}

int orc_set_field(orc_sim* o, int field, const double* in) {
  size_t off = 0;
  for (auto& g : o->G) {
    std::vector<double>* dst = nullptr;
    switch (field) {
      case PG_FIELD_VEL: dst = &g.vel; break;
      case PG_FIELD_ACC: dst = &g.acc; break;
      case PG_FIELD_DISP: dst = &g.disp; break;
      case PG_FIELD_POS: dst = &g.pos; break;  // xi is kept, as the reference keeps it
      default: return PG_EINVAL;
    }
    std::memcpy(dst->data(), in + off, dst->size() * 8);
    off += dst->size();
  }
  return PG_OK;
}

int orc_get_bond_alive(orc_sim* o, uint8_t* out) {
  std::memset(out, 0, o->nbonds);
  for (auto& g : o->G)
    for (auto& row : g.bid)
      for (uint64_t b : row) out[b] = 1;
  return PG_OK;
}

int orc_get_bond_break_step(orc_sim* o, uint32_t* out) {
  std::memcpy(out, o->break_step.data(), o->nbonds * 4);
  return PG_OK;
}

int orc_get_reaction(orc_sim* o, double* out) {
  const uint32_t D = o->D;
  for (size_t k = 0; k < o->I.size(); ++k)
    for (uint32_t s = 0; s < 2 * D; ++s)
      for (uint32_t c = 0; c < D; ++c) out[(k * 2 * D + s) * D + c] = o->I[k].reaction[s][c];
  return PG_OK;
}

int orc_get_wall(orc_sim* o, double* out) {
  const uint32_t D = o->D;
  for (size_t k = 0; k < o->I.size(); ++k)
    for (uint32_t s = 0; s < 2 * D; ++s) out[k * 2 * D + s] = o->I[k].wall[s];
  return PG_OK;
}

int orc_set_grain_flags(orc_sim* o, uint32_t g, int32_t movable, int32_t stoppable) {
  if (g >= o->G.size()) return PG_EINVAL;
  if (movable >= 0) o->G[g].movable = movable;
  if (stoppable >= 0) o->G[g].stoppable = stoppable;
  return PG_OK;
}

// Pair log of all steps taken: count[k], hash[k] for step first_step + k.
uint64_t orc_pair_log_size(orc_sim* o) { return o->log_count.size(); }
int orc_get_pair_log(orc_sim* o, uint64_t* count, uint64_t* hash) {
  std::memcpy(count, o->log_count.data(), o->log_count.size() * 8);
  std::memcpy(hash, o->log_hash.data(), o->log_hash.size() * 8);
  return PG_OK;
}

uint64_t orc_too_close(orc_sim* o) { return o->too_close; }

// reference_structured: 1 = enumerate pairs with the reference's loops (its cost model);
// threads > 1 = run independent instances concurrently (OpenMP).
int orc_set_mode(orc_sim* o, int reference_structured, int threads) {
  o->reference_structured = reference_structured;
  o->threads = threads < 1 ? 1 : threads;
  return PG_OK;
}

}  // extern "C"
