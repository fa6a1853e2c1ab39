// GB300 (sm_103a) kernels of the gradient path, forward side: one FP64 time step under frozen
// masks (the map the reverse step in pg_adjoint_rev.cu differentiates).
//
// Forward map of step t (reference src/particle/timeloop.h:661-669, :686-863), per node p of a
// movable grain:
//   disp' = disp + dt*vel + (dt*dt*0.5)*acc ;  X = pos + disp'
//   F     = sum_bonds cnot*s*vol_j*e  (particle2.h:102-150)
//         + sum_contacts [elastic + damping + friction]  (contact.h:668-812)
//         + sum_wall_sides [normal + friction + damping]  (contact.h:314-431)  + extforce
//   acc'  = F / rho ;  vel' = vel + (acc + acc')*(0.5*dt)
// Bond use, contact pairs, friction branches (sliding with its 2D direction, sticking) and wall
// contacts are the recorded masks of step t, so the map is smooth.
//
// Compiled with --fmad=false: the replay performs the FP64 path's operations in its order, so
// under the masks the FP64 engine recorded it reproduces that engine bit for bit.
#include <cuda_runtime.h>

#include <cmath>

#include "pg_adjoint.cuh"
#include "pg_adjoint.h"
#include "pg_common.cuh"
#include "pg_device.cuh"

namespace pg {

// ---------------------------------------------------------------------------------------------
// replay forward (frozen masks), FP64
// ---------------------------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(256) k_rp_predict(const Dev P) {
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= P.N) return;
  const GrainDev& gr = P.grain[P.node_grain[d]];
  double dp[D], ps[D], cu[D];
  ldv<D>(P.disp, d, dp);
  bool wrote = false;
  if (P.clamp_pending[d]) {
    for (int c = 0; c < D; ++c) dp[c] = 0.0;
    P.clamp_pending[d] = 0;
    wrote = true;
  }
  if (gr.flags & GF_MOVABLE) {
    double v[D], a[D];
    ldv<D>(P.vel_in, d, v);
    ldv<D>(P.acc, d, a);
    for (int c = 0; c < D; ++c) dp[c] = dp[c] + ((P.dt * v[c]) + (P.hdt2 * a[c]));
    wrote = true;
  }
  if (wrote) stv<D>(P.disp, d, dp);
  ldv<D>(P.pos, d, ps);
  for (int c = 0; c < D; ++c) cu[c] = ps[c] + dp[c];
  stv<D>(P.cur, d, cu);
}

template <int D>
__global__ void __launch_bounds__(128) k_rp_force(const Dev P, const ReplayStep R) {
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31;
  if (d >= P.N) return;
  const uint32_t chunk = d >> 5;
  const uint32_t t = *P.step;
  const uint32_t g = P.node_grain[d];
  const GrainDev gr = P.grain[g];
  const bool mov = gr.flags & GF_MOVABLE;
  const InstDev& in = P.inst[gr.inst];
  constexpr int NS = 2 * D;
  double f[D];
  for (int c = 0; c < D; ++c) f[c] = 0.0;
  double vp[D];
  ldv<D>(P.vel_in, d, vp);
  if (R.wall_out) {
    for (int k = 0; k < NS * 4; ++k) R.wall_out[(size_t)d * NS * 4 + k] = 0.0;
  }
  if (mov) {
    // bonds (particle2.h:102-150) in the SELL slot order of the FP64 path
    const uint32_t cdeg = P.chunk_deg[chunk];
    const uint32_t slot0 = P.chunk_slot[chunk] + lane;
    const uint32_t w0 = P.chunk_word[chunk];
    double dp[D], xp[D];
    ldv<D>(P.disp, d, dp);
    ldv<D>(P.xpos, d, xp);
    for (uint32_t k = 0; k < cdeg; ++k) {
      const uint32_t s = slot0 + 32u * k;
      if (!bond_used(R.end_alive, R.break_step, w0 + k, lane, s, t)) continue;
      const uint32_t j = P.bcol[s];
      const double xin = P.bxin[s];
      double dj[D], xj[D];
      ldv<D>(P.disp, j, dj);
      ldv<D>(P.xpos, j, xj);
      double e[D];
      for (int c = 0; c < D; ++c) e[c] = (dj[c] - dp[c]) + (xj[c] - xp[c]);
      double n2 = e[0] * e[0];
      for (int c = 1; c < D; ++c) n2 = n2 + e[c] * e[c];
      const double en = sqrt(n2);
      const double str = (en - xin) / xin;
      const double sc = (gr.cnot * str) * P.vol[j];
      for (int c = 0; c < D; ++c) f[c] = f[c] + sc * (e[c] / en);
    }

    // recorded contacts, in the recorded order (contact.h:668-812)
    double xpc[D];
    ldv<D>(P.cur, d, xpc);
    const uint32_t o = R.off[d], n = R.cnt[d];
    for (uint32_t i = 0; i < n; ++i) {
      const uint32_t e = R.ent[o + i];
      const uint32_t q = e & ENT_NODE, fr = e >> 30;
      const uint32_t gqi = P.node_grain[q];
      const bool same = gqi == g;
      double Kn, Rc, zeta, mu;
      pair_params<D>(P, in, gr, P.grain[gqi], same, d, q, &Kn, &Rc, &zeta, &mu);
      double xq[D], dir[D];
      ldv<D>(P.cur, q, xq);
      for (int c = 0; c < D; ++c) dir[c] = xq[c] - xpc[c];
      double n2 = dir[0] * dir[0];
      for (int c = 1; c < D; ++c) n2 = n2 + dir[c] * dir[c];
      const double dn = sqrt(n2);
      double u[D];
      for (int c = 0; c < D; ++c) u[c] = dir[c] / dn;
      const double crc = Rc - dn;
      const double nvol = P.vol[q];
      const double s1 = ((-Kn) * crc) * nvol;
      double fc[D];
      for (int c = 0; c < D; ++c) fc[c] = s1 * u[c];
      double cf2 = fc[0] * fc[0];
      for (int c = 1; c < D; ++c) cf2 = cf2 + fc[c] * fc[c];
      const double cfn = sqrt(cf2);
      for (int c = 0; c < D; ++c) f[c] = f[c] + fc[c];
      if (P.allow_damping || P.allow_friction) {
        double vq[D], rv[D];
        ldv<D>(P.vel_in, q, vq);
        for (int c = 0; c < D; ++c) rv[c] = vp[c] - vq[c];
        double rvp = rv[0] * u[0];
        for (int c = 1; c < D; ++c) rvp = rvp + rv[c] * u[c];
        if (P.allow_damping) {
          const double dc = ((2.0 * zeta) * sqrt(Kn * gr.rho)) * sqrt(nvol);
          for (int c = 0; c < D; ++c) f[c] = f[c] + ((-dc) * (rvp * u[c]));
        }
        if (P.allow_friction && fr) {
          double tg[D];
          for (int c = 0; c < D; ++c) tg[c] = rv[c] - (rvp * u[c]);
          double t2 = tg[0] * tg[0];
          for (int c = 1; c < D; ++c) t2 = t2 + tg[c] * tg[c];
          const double tn = sqrt(t2);
          if (fr == FR_STICK) {
            if (tn > 0) {
              const double sfr = ((-tn) / gr.rho) / P.dt;
              for (int c = 0; c < D; ++c) f[c] = f[c] + sfr * (tg[c] / tn);
            }
          } else {
            // |s1| continued as -s1 past R_c (equal while the contact is active), so the frozen
            // map stays smooth when a perturbed run moves the pair apart
            const double sfr = (-mu) * (s1 <= 0 ? cfn : -cfn);
            bool as_recorded = tn > 0;
            if constexpr (D == 2) as_recorded = as_recorded && (((tg[1] * u[0] - tg[0] * u[1]) < 0) == (fr == FR_SLIDE_NEG));
            if (as_recorded) {
              for (int c = 0; c < D; ++c) f[c] = f[c] + sfr * (tg[c] / tn);
            } else if constexpr (D == 2) {
              // the recorded sliding direction +-perp(u), perp(u) = (-u_y, u_x)
              const double sg = (fr == FR_SLIDE_NEG) ? -1.0 : 1.0;
              f[0] = f[0] + sfr * (sg * -u[1]);
              f[1] = f[1] + sfr * (sg * u[0]);
            }
          }
        }
      }
    }

    // recorded wall contacts (contact.h:900-964, :314-431)
    const uint32_t wb = R.wall[d];
    if (wb) {
      const double vol_i = P.vol[d];
      for (int k = 0; k < NS; ++k) {
        if (!wb_contact(wb, k)) continue;
        int side, dir;
        wall_side<D>(k, &side, &dir);
        const double dist = xpc[dir] - in.wall[side];
        const double Rr = in.contact_rad;
        // a frozen wall contact can drift past R in a perturbed run: the force is extended by
        // its value at R (zero, and C1 there); recorded runs have |dist| <= R, so this is exact
        const double dd = fmin(fabs(dist), Rr);
        double Area, I;
        if constexpr (D == 2) {
          Area = M_PI * pow(Rr, 2.0) / 2 - pow(Rr, 2.0) * asin(dd / Rr) - sqrt(Rr * Rr - dd * dd) * dd;
          I = 0.0 * pow((Rr * Rr - dd * dd), 1.5);
        } else {
          Area = M_PI / 3 * pow((Rr - dd), 2.0) * (2 * Rr - dd);
          I = M_PI / 4 * pow(pow(Rr, 2.0) - pow(dd, 2.0), 2.0);
        }
        const double centroid = I / Area;
        const double crc = Rr - centroid;
        const double pcrc = crc > 0 ? crc : 0;
        const double F = (gr.kn * pcrc) * Area;
        const double c_sign = dist > 0 ? 1 : -1;
        f[dir] = f[dir] + (c_sign * F);
        double a_t1 = 0, a_t2 = 0, a_damp = 0;
        double rv[D];
        for (int c = 0; c < D; ++c) rv[c] = vp[c];
        rv[dir] = rv[dir] - in.wall_speed[side];
        if (P.allow_friction && wb_fric(wb, k)) {
          const bool stick = wb_stick(wb, k);
          const double mu = gr.mu;
          if constexpr (D == 2) {
            const int tg = (dir + 1) % 2;
            const double vts = wb_neg(wb, k) ? -1 : 1;  // recorded sliding direction
            const double ff = stick ? ((-rv[tg]) * gr.rho) / P.dt : ((-mu) * fabs(F)) * vts;
            f[tg] = f[tg] + ff;
            a_t1 = vol_i * ff;
          } else {
            const int t1 = (dir + 1) % 3, t2 = (dir + 2) % 3;
            const double v1 = rv[t1], v2 = rv[t2];
            const double vn = sqrt(pow(v1, 2.0) + pow(v2, 2.0));
            if (vn > 0) {
              const double u1 = v1 / vn, u2 = v2 / vn;
              double ff1 = ((-mu) * fabs(F)) * u1;
              double ff2 = ((-mu) * fabs(F)) * u2;
              if (stick) {
                ff1 = (((-vn) / gr.rho) / P.dt) * u1;
                ff2 = (((-vn) / gr.rho) / P.dt) * u2;
              }
              f[t1] = f[t1] + ff1;
              f[t2] = f[t2] + ff2;
              a_t1 = vol_i * ff1;
              a_t2 = vol_i * ff2;
            }
          }
        }
        if (P.allow_damping) {
          const double dc = ((2.0 * gr.zeta) * sqrt(gr.kn * gr.rho)) * sqrt(fabs(Area));
          const double df = (-dc) * rv[dir];
          f[dir] = f[dir] + df;
          a_damp = vol_i * df;
        }
        if (R.wall_out) {
          double* wo = R.wall_out + ((size_t)d * NS + side) * 4;
          wo[0] = (vol_i * c_sign) * F;
          wo[1] = a_t1;
          wo[2] = a_t2;
          wo[3] = a_damp;
        }
      }
    }

    // external force (timeloop.h:774-790)
    double ef[D];
    ldv<D>(P.extf, d, ef);
    if (P.gradient_extforce) {
      double sc = (double)t / (double)P.extforce_maxstep;
      if (sc > 1) sc = 1;
      for (int c = 0; c < D; ++c) f[c] = f[c] + sc * ef[c];
    } else {
      for (int c = 0; c < D; ++c) f[c] = f[c] + ef[c];
    }
  }

  // velocity update (timeloop.h:834-863)
  if (mov) {
    double ao[D], a[D], v[D];
    ldv<D>(P.acc, d, ao);
    for (int c = 0; c < D; ++c) {
      a[c] = gr.one_over_rho * f[c];
      double tmp = ao[c] + a[c];
      tmp = tmp * P.half_dt;
      v[c] = vp[c] + tmp;
    }
    if (P.clamped[d]) {
      for (int c = 0; c < D; ++c) {
        a[c] = 0.0;
        v[c] = 0.0;
      }
      P.clamp_pending[d] = 1;
    }
    stv<D>(P.acc, d, a);
    stv<D>(P.vel_out, d, v);
  } else {
    stv<D>(P.vel_out, d, vp);
  }
  stv<D>(P.force, d, f);
}

// Wall reactions of the step from the per-node terms, in node order (contact.h:339, :374, :428):
// one thread per (instance, side).
template <int D>
__global__ void k_rp_reaction(const Dev P, const ReplayStep R) {
  constexpr int NS = 2 * D;
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.I * NS) return;
  const uint32_t inst = p / NS, side = p % NS;
  const InstDev& in = P.inst[inst];
  const int dir = (D == 2) ? ((side == 0 || side == 1) ? 0 : 1) : (int)(side % 3);
  double r[3] = {0.0, 0.0, 0.0};
  for (uint32_t o = in.node_begin; o < in.node_end; ++o) {  // the input's node order
    const uint32_t d = at_of(P, o);
    const double* wo = R.wall_out + ((size_t)d * NS + side) * 4;
    if (wo[0] == 0.0 && wo[1] == 0.0 && wo[2] == 0.0 && wo[3] == 0.0) continue;
    r[dir] = r[dir] - wo[0];
    if constexpr (D == 2) {
      r[(dir + 1) % 2] = r[(dir + 1) % 2] - wo[1];
    } else {
      r[(dir + 1) % 3] = r[(dir + 1) % 3] - wo[1];
      r[(dir + 2) % 3] = r[(dir + 2) % 3] - wo[2];
    }
    r[dir] = r[dir] - wo[3];
  }
  for (int c = 0; c < D; ++c) P.reaction[((size_t)inst * NS + side) * D + c] = r[c];
}

// End of a replay step: wall move (timeloop.h:866-878) and step counter.
template <int D>
__global__ void k_rp_advance(const Dev P) {
  constexpr int NS = 2 * D;
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < P.I * NS) {
    InstDev* in = &P.inst[p / NS];
    const int s = p % NS;
    in->wall[s] = in->wall[s] + in->wall_speed[s] * P.dt;
  }
  if (p == 0) *P.step = *P.step + 1;
}

// ---------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------
template <int D>
static void replay_t(const Dev& P, const ReplayStep& R, cudaStream_t s, uint64_t* launches) {
  k_rp_predict<D><<<cdiv(P.N, 256), 256, 0, s>>>(P);
  k_rp_force<D><<<cdiv(P.N, 128), 128, 0, s>>>(P, R);
  *launches += 2;
  if (R.wall_out) {
    k_rp_reaction<D><<<cdiv(P.I * 2 * D, 64), 64, 0, s>>>(P, R);
    *launches += 1;
  }
  k_rp_advance<D><<<cdiv(P.I * 2 * D, 64), 64, 0, s>>>(P);
  *launches += 1;
}

void launch_replay_step(const Dev& P, const ReplayStep& R, cudaStream_t s, uint64_t* launches) {
  if (P.dim == 2) {
    replay_t<2>(P, R, s, launches);
  } else {
    replay_t<3>(P, R, s, launches);
  }
}

}  // namespace pg
