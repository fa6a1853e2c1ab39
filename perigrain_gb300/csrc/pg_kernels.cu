// GB300 (sm_103a) kernels of the PeriDEM time step, FP64 parity path.
//
// One step (reference src/particle/timeloop.h:608-879) is six launches on one stream:
//   k_predict      position update (timeloop.h:661-669) + grid key + per-grain bounding box
//   k_scan_reduce  \ exclusive scan of the per-bucket counts = cell-start table
//   k_scan_final   /
//   k_scatter      nodes -> bucket order (counting sort, one digit spanning all buckets)
//   k_force        bond force + break (particle2.h:102-232), self/inter-grain contact
//                  (contact.h:668-812), wall (contact.h:900-964, :314-431, :16-41),
//                  external force and torque (timeloop.h:774-824), velocity update
//                  (timeloop.h:834-863) -- fused, one node per thread
//   k_finalize     ordered wall-reaction sums, pair log, wall move (timeloop.h:866-878)
//
// This file is compiled with --fmad=false: every FP64 operation is the IEEE operation the
// reference performs, in the reference's order, so the non-wall path is bit-exact.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "pg_common.cuh"
#include "pg_device.cuh"
#include "pg_ieee64.cuh"
#include "pg_kernels.h"

namespace pg {

// ---------------------------------------------------------------------------------------------
// k_predict: disp += dt*vel + (dt*dt*0.5)*acc for movable grains; CurrPos = pos + disp.
// ---------------------------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(256) k_predict(const Dev P) {
  pdl_enter();
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31;
  const bool act = d < P.N;
  uint32_t g = 0;
  unsigned long long kmin[D], kmax[D];
  if (act) {
    g = P.node_grain[d];
    const GrainDev& gr = P.grain[g];
    double dp[D], ps[D], cu[D];
    ldv<D>(P.disp, d, dp);
    bool wrote = false;
    if (P.clamp_pending[d]) {
      // a clamped node zeroed at the end of the previous step (timeloop.h:854-860)
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

    // grid cell from the FP32 offset to this step's grid origin
    const InstDev& in = P.inst[gr.inst];
    float rf[4] = {0.f, 0.f, 0.f, 0.f};
    int32_t ci[3] = {0, 0, 0};
    bool ok = true;
    for (int c = 0; c < D; ++c) {
      if (!isfinite(cu[c])) ok = false;
      rf[c] = (float)(cu[c] - in.origin[c]);
      ci[c] = cell_coord(rf[c] + in.frame_off_f[c], in.inv_cell_f, in.dims[c]);
    }
    if (!ok) set_status(P.status, PG_ENAN);
    if constexpr (D == 2) {
      reinterpret_cast<float2*>(P.curf)[d] = make_float2(rf[0], rf[1]);
    } else {
      reinterpret_cast<float4*>(P.curf)[d] = make_float4(rf[0], rf[1], rf[2], 0.f);
    }
    const uint32_t key = in.table_off + ((uint32_t)ci[2] * in.dims[1] + (uint32_t)ci[1]) * in.dims[0] + (uint32_t)ci[0];
    if (P.cand_q) {
      // candidate lists: keys only on rebuild steps (k_keys); rebuild once any node has moved
      // 0.45 skin since the last build
      constexpr uint32_t SF = (D == 2) ? 2 : 4;
      float m2 = 0.f;
      for (int c = 0; c < D; ++c) {
        const float dd = (float)dp[c] - P.disp_b[(size_t)d * SF + c];
        m2 += dd * dd;
      }
      if (m2 > in.skin_lim2) *P.rebuild = 1;
    } else {
      P.cell_key[d] = key;
      P.cell_rank[d] = atomicAdd(&P.cell_count[key], 1u);
    }
    for (int c = 0; c < D; ++c) {
      kmin[c] = dbl_to_ordered(cu[c]);
      kmax[c] = kmin[c];
    }
  } else {
    for (int c = 0; c < D; ++c) {
      kmin[c] = ~0ull;
      kmax[c] = 0ull;
    }
  }
  // per-grain bounding box (contact.h:1024-1062), min/max are exact so atomics are deterministic
  const uint32_t full = 0xffffffffu;
  uint32_t g0 = __shfl_sync(full, g, 0);
  bool lane0_act = __shfl_sync(full, act ? 1 : 0, 0);
  if (!lane0_act) return;
  uint32_t same = __ballot_sync(full, !act || g == g0);
  if (same == full) {
    for (int c = 0; c < D; ++c) {
      kmin[c] = warp_min_u64(kmin[c]);
      kmax[c] = warp_max_u64(kmax[c]);
    }
    if (lane == 0) {
      for (int c = 0; c < D; ++c) {
        atomicMin(&P.bbox[(size_t)g0 * 2 * D + c], kmin[c]);
        atomicMax(&P.bbox[(size_t)g0 * 2 * D + D + c], kmax[c]);
      }
    }
  } else if (act) {
    for (int c = 0; c < D; ++c) {
      atomicMin(&P.bbox[(size_t)g * 2 * D + c], kmin[c]);
      atomicMax(&P.bbox[(size_t)g * 2 * D + D + c], kmax[c]);
    }
  }
}

template <int D, bool REC, bool GC>
__global__ void __launch_bounds__(128) k_force(const Dev P) {
  pdl_enter();
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t chunk = d >> 5;
  if (chunk >= P.n_chunks) return;  // uniform per warp
  const bool act = d < P.N;
  const uint32_t t = *P.step;
  const uint32_t g = act ? P.node_grain[d] : 0;
  const GrainDev gr = P.grain[g];
  const bool mov = act && (gr.flags & GF_MOVABLE);
  const bool brk = P.enable_fracture && (gr.flags & GF_BREAKABLE) && (gr.flags & GF_BREAK_BONDS);

  double f[D];
  for (int c = 0; c < D; ++c) f[c] = 0.0;
  double vp[D];
  if (act) ldv<D>(P.vel_in, d, vp);

  // ---- bond force and bond breaking (particle2.h:102-150, :191-232) ----
  const uint32_t cdeg = P.chunk_deg[chunk];
  const uint32_t slot0 = P.chunk_slot[chunk] + lane;
  const uint32_t w0 = P.chunk_word[chunk];
  {
    // the break test str > snot on the integer pipe when snot is +0 or more and not NaN
    const uint64_t snot_bits = ieee64::bits(gr.snot);
    const bool snot_int = ieee64::gt_nonneg_ok(snot_bits);
    double dp[D], xp[D];
    if (mov) {
      ldv<D>(P.disp, d, dp);
      ldv<D>(P.xpos, d, xp);
    }
    for (uint32_t k = 0; k < cdeg; ++k) {
      const uint32_t word = P.alive[w0 + k];
      bool bit = (word >> lane) & 1u;
      if (mov && bit) {
        const uint32_t s = slot0 + 32u * k;
        const uint32_t j = P.bcol[s];
        const double xin = P.bxin[s];
        double dj[D], xj[D];
        ldv<D>(P.disp, j, dj);
        ldv<D>(P.xpos, j, xj);
        double e[D];
        for (int c = 0; c < D; ++c) e[c] = (dj[c] - dp[c]) + (xj[c] - xp[c]);
        // the squares on the integer pipe too (the sums stay FP64 instructions: the integer sum
        // measured slower, and so did moving the scale and force products as well)
        double n2 = ieee64::mul_rn(e[0], e[0]);
        for (int c = 1; c < D; ++c) n2 = n2 + ieee64::mul_rn(e[c], e[c]);
        // sqrt and the divisions on the integer pipe, bit-identical to the IEEE operations
        const double en = ieee64::sqrt_rn(n2);
        const double str = ieee64::div_rn(en - xin, xin);
        const double sc = (gr.cnot * str) * P.vol[j];
        // an unstretched bond (sc = +-0 with 0 < en < inf, so |e[c] / en| <= 1) adds +-0, which
        // leaves f's bits unchanged (f starts at +0 and never becomes -0 under round-to-nearest)
        const uint64_t enb = ieee64::bits(en);
        if ((ieee64::bits(sc) << 1) != 0 || enb - 1 >= 0x7fefffffffffffffull) {
          const ieee64::Divisor den = ieee64::make_divisor(en);
          for (int c = 0; c < D; ++c) f[c] = f[c] + sc * ieee64::div_rn(e[c], den);
        }
        if (brk && (snot_int ? ieee64::gt_nonneg(str, snot_bits) : str > gr.snot)) {
          bit = false;
          P.break_step[s] = t;
        }
      }
      const uint32_t nw = __ballot_sync(0xffffffffu, bit);
      if (lane == 0 && nw != word) P.alive[w0 + k] = nw;
    }
  }
  __syncwarp();

  unsigned long long my_pairs = 0, my_hash = 0, my_close = 0;
  uint32_t rent[REC ? MAX_CAND : 1];  // recorded contact entries of this node (REC only)
  uint32_t nrec = 0, wbits = 0;
  const InstDev& in = P.inst[gr.inst];
  const bool p_bdry = !P.nl_bdry_only || (act && P.bdry_rank[d] != NONE);
  const bool selfc = mov && P.enable_fracture && (gr.flags & GF_BREAKABLE) && P.self_contact;
  // contact with other grains and walls only for stoppable grains (timeloop.h:719), for every
  // movable grain in the worm loop (timeloop.h:1146-1168)
  const bool other = mov && (P.worm || (gr.flags & GF_STOPPABLE));
  double xpc[D];
  if (act) ldv<D>(P.cur, d, xpc);

  // ---- node-node contact: self-contact first, then grains j ascending (timeloop.h:709-747) ----
  // with candidate lists a node whose list is empty has no contact this step
  const uint32_t ncl = (P.cand_q && act) ? (uint32_t)P.cand_n[d] : 0u;
  if ((selfc || other) && p_bdry && (!P.cand_q || ncl > 0)) {
    double bmn[D], bmx[D];
    grain_box<D>(P, g, bmn, bmx);
    float pf[D];
    ldf<D>(P.curf, d, pf);
    int32_t cc[3] = {0, 0, 0};
    for (int c = 0; c < D; ++c) cc[c] = cell_coord(pf[c] + in.frame_off_f[c], in.inv_cell_f, in.dims[c]);
    const float thr2 = in.pre_f * in.pre_f;
    unsigned long long keys[MAX_CAND];
    uint32_t idx[MAX_CAND];
    int nc = 0;
    // one candidate q of node d: the FP32 prefilter, the contact rules and the grain-box test,
    // then insertion in the reference's visit order
    auto consider = [&](uint32_t q) {
      float qf[D];
      ldf<D>(P.curf, q, qf);
      float d2 = 0.f;
      for (int c = 0; c < D; ++c) {
        float dd = qf[c] - pf[c];
        d2 += dd * dd;
      }
      if (d2 > thr2) return;
      const uint32_t gq = P.node_grain[q];
      const bool same = (gq == g);
      if (same ? !selfc : !other) return;
      if (P.nl_bdry_only && P.bdry_rank[q] == NONE) return;
      if (!same) {
        double qmn[D], qmx[D];
        grain_box<D>(P, gq, qmn, qmx);
        if (!boxes_touch<D>(bmn, bmx, qmn, qmx, in.contact_rad)) return;
      }
      const uint32_t sub = P.node_sub[q];
      const unsigned long long key =
          ((unsigned long long)(same ? 0u : 1u) << 63) | ((unsigned long long)gq << 32) | sub;
      insert_cand<D>(keys, idx, nc, key, q, P);
    };
    if (P.cand_q) {
      // candidate list of the last rebuild (a superset of the grid search's candidates)
      const size_t cbase = (size_t)chunk * P.cand_cap * 32 + lane;
      for (uint32_t k = 0; k < ncl; ++k) consider(P.cand_q[cbase + (size_t)k * 32]);
    } else {
    const int z0 = (D == 3) ? max(cc[2] - 1, 0) : 0, z1 = (D == 3) ? min(cc[2] + 1, (int)in.dims[2] - 1) : 0;
    const int y0 = max(cc[1] - 1, 0), y1 = min(cc[1] + 1, (int)in.dims[1] - 1);
    const int x0 = max(cc[0] - 1, 0), x1 = min(cc[0] + 1, (int)in.dims[0] - 1);
    for (int z = z0; z <= z1; ++z)
      for (int y = y0; y <= y1; ++y) {
        const uint32_t row = in.table_off + ((uint32_t)z * in.dims[1] + (uint32_t)y) * in.dims[0];
        const uint32_t b0 = P.cell_start[row + x0], b1 = P.cell_start[row + x1 + 1];
        for (uint32_t b = b0; b < b1; ++b) {
          const uint32_t q = P.sorted[b];
          if (q != d) consider(q);
        }
      }
    }
    const uint32_t mydeg = P.node_deg[d];
    for (int ci = 0; ci < nc; ++ci) {
      const uint32_t q = idx[ci];
      const bool same = (keys[ci] >> 63) == 0;
      double xq[D], dir[D];
      ldv<D>(P.cur, q, xq);
      for (int c = 0; c < D; ++c) dir[c] = xq[c] - xpc[c];
      double n2 = dir[0] * dir[0];
      for (int c = 1; c < D; ++c) n2 = n2 + dir[c] * dir[c];
      // dn <= R_c <= contact_rad needs n2 <= contact_s_max (the same outcome as the sqrt test):
      // candidates beyond it skip the square root and the bonded-neighbour scan
      if (!(n2 <= in.contact_s_max)) continue;
      const double dn = ieee64::sqrt_rn(n2);
      double Rc = in.contact_rad, Kn = in.normal_stiffness;
      double zeta = in.damping_ratio, mu = in.friction_coefficient;
      if constexpr (GC) {
        const GrainDev& gq = P.grain[(uint32_t)(keys[ci] >> 32) & 0x7fffffffu];
        Kn = (gr.kn + gq.kn) * 0.5;
        zeta = (gr.zeta + gq.zeta) * 0.5;
        mu = (gr.mu + gq.mu) * 0.5;
      }
      if (same) {
        bool bonded = false;
        for (uint32_t k = 0; k < mydeg && !bonded; ++k) {
          if (((P.alive[w0 + k] >> lane) & 1u) && P.bcol[slot0 + 32u * k] == q) bonded = true;
        }
        if (bonded) continue;
        double pp[D], pq[D], r[D];
        ldv<D>(P.pos, d, pp);
        ldv<D>(P.pos, q, pq);
        for (int c = 0; c < D; ++c) r[c] = pp[c] - pq[c];
        double r2 = r[0] * r[0];
        for (int c = 1; c < D; ++c) r2 = r2 + r[c] * r[c];
        const double ref = ieee64::sqrt_rn(r2);
        Rc = ref < in.contact_rad ? ref : in.contact_rad;
        Kn = ieee64::div_rn(gr.cnot, Rc);
      }
      if (!(dn <= Rc)) continue;
      if (P.record_pairs) {
        my_pairs += 1;
        my_hash += splitmix64(((unsigned long long)orig_of(P, d) << 32) | orig_of(P, q));
      }
      if (dn == 0.0) my_close += 1;
      double u[D];
      {
        const ieee64::Divisor ddn = ieee64::make_divisor(dn);
        for (int c = 0; c < D; ++c) u[c] = ieee64::div_rn(dir[c], ddn);
      }
      const double crc = Rc - dn;
      const double nvol = P.vol[q];
      const double s1 = ((-Kn) * crc) * nvol;
      double fc[D];
      for (int c = 0; c < D; ++c) fc[c] = s1 * u[c];
      double cf2 = fc[0] * fc[0];
      for (int c = 1; c < D; ++c) cf2 = cf2 + fc[c] * fc[c];
      const double cfn = ieee64::sqrt_rn(cf2);
      for (int c = 0; c < D; ++c) f[c] = f[c] + fc[c];
      uint32_t fr = 0;
      if (P.allow_damping || P.allow_friction) {
        double vq[D], rv[D];
        ldv<D>(P.vel_in, q, vq);
        for (int c = 0; c < D; ++c) rv[c] = vp[c] - vq[c];
        double rvp = rv[0] * u[0];
        for (int c = 1; c < D; ++c) rvp = rvp + rv[c] * u[c];
        if (P.allow_damping) {
          const double dc = ((2.0 * zeta) * ieee64::sqrt_rn(Kn * gr.rho)) * ieee64::sqrt_rn(nvol);
          for (int c = 0; c < D; ++c) f[c] = f[c] + ((-dc) * (rvp * u[c]));
        }
        if (P.allow_friction) {
          double tg[D];
          for (int c = 0; c < D; ++c) tg[c] = rv[c] - (rvp * u[c]);
          double t2 = tg[0] * tg[0];
          for (int c = 1; c < D; ++c) t2 = t2 + tg[c] * tg[c];
          const double tn = ieee64::sqrt_rn(t2);
          if (tn > 0) {
            double sfr = (-mu) * cfn;
            fr = (D == 2 && (tg[1] * u[0] - tg[0] * u[1]) < 0) ? FR_SLIDE_NEG : FR_SLIDE;
            if (tn < ieee64::div_rn((mu * cfn) * P.dt, gr.rho)) {
              sfr = ieee64::div_rn(ieee64::div_rn(-tn, gr.rho), P.dt);
              fr = FR_STICK;
            }
            const ieee64::Divisor dtn = ieee64::make_divisor(tn);
            for (int c = 0; c < D; ++c) f[c] = f[c] + sfr * ieee64::div_rn(tg[c], dtn);
          }
        }
      }
      if constexpr (REC) rent[nrec++] = q | (fr << 30);
    }
  }

  // ---- analytic wall (timeloop.h:753-769 -> contact.h:900-964) ----
  if (mov && other && p_bdry && in.allow_wall) {
    double bmn[D], bmx[D];
    grain_box<D>(P, g, bmn, bmx);
    if (!within_interior<D>(bmn, bmx, in.wall, in.contact_rad)) {
      const double vol_i = P.vol[d];
      const double Knw = GC ? gr.kn : in.normal_stiffness;
      const double zetaw = GC ? gr.zeta : in.damping_ratio;
      const double muw = GC ? gr.mu : in.friction_coefficient;
      constexpr int NS = 2 * D;
      // (side, dir) in the reference's call order
      const int order2[4][2] = {{3, 1}, {0, 0}, {1, 0}, {2, 1}};
      const int order3[6][2] = {{0, 0}, {3, 0}, {1, 1}, {4, 1}, {2, 2}, {5, 2}};
      for (int k = 0; k < NS; ++k) {
        const int side = (D == 2) ? order2[k][0] : order3[k][0];
        const int dir = (D == 2) ? order2[k][1] : order3[k][1];
        const double dist = xpc[dir] - in.wall[side];
        const double R = in.contact_rad;
        if (!(fabs(dist) <= R)) continue;
        wbits |= 1u << (4 * k);
        const double dd = fabs(dist);
        // segment_mass<dim>(R, d) (contact.h:16-41)
        double Area, I;
        if constexpr (D == 2) {
          Area = M_PI * pow(R, 2.0) / 2 - pow(R, 2.0) * asin(dd / R) - sqrt(R * R - dd * dd) * dd;
          I = 0.0 * pow((R * R - dd * dd), 1.5);  // 2 / 3 is integer division in the reference
        } else {
          Area = M_PI / 3 * pow((R - dd), 2.0) * (2 * R - dd);
          I = M_PI / 4 * pow(pow(R, 2.0) - pow(dd, 2.0), 2.0);
        }
        const double centroid = I / Area;
        const double crc = R - centroid;
        const double pcrc = crc > 0 ? crc : 0;
        const double F = (Knw * pcrc) * Area;
        const double c_sign = dist > 0 ? 1 : -1;
        f[dir] = f[dir] + (c_sign * F);
        WallRec rec;
        rec.a_normal = (vol_i * c_sign) * F;
        rec.a_t1 = 0;
        rec.a_t2 = 0;
        rec.a_damp = 0;
        // replay key: the reference sums reactions grain by grain in its node-loop order
        rec.gid = P.nl_bdry_only ? (gr.node_begin + P.bdry_rank[d]) : orig_of(P, d);
        rec.side = (uint16_t)side;
        rec.has_fric = 0;
        rec.has_damp = 0;
        double rv[D];
        for (int c = 0; c < D; ++c) rv[c] = vp[c];
        rv[dir] = rv[dir] - in.wall_speed[side];
        if (P.allow_friction) {
          const double mu = muw;
          if constexpr (D == 2) {
            const int tg = (dir + 1) % 2;
            if (fabs(rv[tg]) > 0) {
              const double vts = rv[tg] > 0 ? 1 : -1;
              double ff = ((-mu) * fabs(F)) * vts;
              wbits |= (rv[tg] > 0 ? 2u : 10u) << (4 * k);
              if (fabs(rv[tg]) < (((mu * fabs(F)) * P.dt) / gr.rho)) {
                ff = ((-rv[tg]) * gr.rho) / P.dt;
                wbits |= 4u << (4 * k);
              }
              f[tg] = f[tg] + ff;
              rec.a_t1 = vol_i * ff;
              rec.has_fric = 1;
            }
          } else {
            const int t1 = (dir + 1) % 3, t2 = (dir + 2) % 3;
            const double v1 = rv[t1], v2 = rv[t2];
            const double vn = sqrt(pow(v1, 2.0) + pow(v2, 2.0));
            if (vn > 0) {
              const double u1 = v1 / vn, u2 = v2 / vn;
              double ff1 = ((-mu) * fabs(F)) * u1;
              double ff2 = ((-mu) * fabs(F)) * u2;
              wbits |= 2u << (4 * k);
              if (vn < (((mu * fabs(F)) * P.dt) / gr.rho)) {
                ff1 = (((-vn) / gr.rho) / P.dt) * u1;
                ff2 = (((-vn) / gr.rho) / P.dt) * u2;
                wbits |= 4u << (4 * k);
              }
              f[t1] = f[t1] + ff1;
              f[t2] = f[t2] + ff2;
              rec.a_t1 = vol_i * ff1;
              rec.a_t2 = vol_i * ff2;
              rec.has_fric = 1;
            }
          }
        }
        if (P.allow_damping) {
          const double dc = ((2.0 * zetaw) * sqrt(Knw * gr.rho)) * sqrt(fabs(Area));
          const double df = (-dc) * rv[dir];
          f[dir] = f[dir] + df;
          rec.a_damp = vol_i * df;
          rec.has_damp = 1;
        }
        const uint32_t slot = atomicAdd(P.wrec_count, 1u);
        if (slot < P.wrec_cap) {
          P.wrec[slot] = rec;
        } else {
          set_status(P.status, PG_ECAPACITY);
        }
      }
    }
  }

  // ---- external force and torque (timeloop.h:774-824) ----
  if (mov && P.worm) {
    // ft_i += ((t_num + 1) % 2) * extforce (timeloop.h:1171)
    double ef[D];
    ldv<D>(P.extf, d, ef);
    const double gate = (double)((worm_phase(t) + 1u) % 2u);
    for (int c = 0; c < D; ++c) f[c] = f[c] + gate * ef[c];
  } else if (mov) {
    double ef[D];
    ldv<D>(P.extf, d, ef);
    if (P.gradient_extforce) {
      double sc = (double)t / (double)P.extforce_maxstep;
      if (sc > 1) sc = 1;
      for (int c = 0; c < D; ++c) f[c] = f[c] + sc * ef[c];
    } else {
      for (int c = 0; c < D; ++c) f[c] = f[c] + ef[c];
    }
    if (P.enable_torque) {
      const uint32_t ta = gr.torque_axis;
      double r[3] = {0, 0, 0}, rp[3] = {0, 0, 0};
      for (int c = 0; c < D; ++c) r[c] = xpc[c] - P.torque_c[(size_t)g * 3 + c];
      if (D == 3) r[ta] = 0;
      if (D == 3) rp[ta] = 0;
      rp[(ta + 1) % 3] = -r[(ta + 2) % 3];
      rp[(ta + 2) % 3] = r[(ta + 1) % 3];
      double pn2 = rp[0] * rp[0];
      for (int c = 1; c < D; ++c) pn2 = pn2 + rp[c] * rp[c];
      const double pn = sqrt(pn2);
      if (pn > 0) {
        for (int c = 0; c < D; ++c) rp[c] = rp[c] / pn;
      } else {
        rp[(ta + 1) % 3] = 0;
        rp[(ta + 2) % 3] = 0;
      }
      for (int c = 0; c < D; ++c) f[c] = f[c] + (gr.torque_val * rp[c]);
    }
  }

  // ---- velocity update (timeloop.h:834-863) ----
  if (act) {
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
      if (P.worm) worm_clamp<D>(orig_of(P, d) - gr.node_begin, worm_phase(t), a, v);
      stv<D>(P.acc, d, a);
      stv<D>(P.vel_out, d, v);
    } else {
      stv<D>(P.vel_out, d, vp);
    }
    stv<D>(P.force, d, f);  // zero for grains that are not movable
  }

  if constexpr (REC) {
    record_masks(P, d, act, lane, rent, nrec, wbits);
    if (P.rec_x) record_tape<D>(P, d, act, t, xpc, vp);
  }

  // ---- diagnostics: warp-aggregated counters ----
  if (P.record_pairs) {
    for (int off = 16; off > 0; off >>= 1) {
      my_pairs += __shfl_down_sync(0xffffffffu, my_pairs, off);
      my_hash += __shfl_down_sync(0xffffffffu, my_hash, off);
    }
    if (lane == 0 && my_pairs) {
      atomicAdd(&P.pair_acc[0], my_pairs);
      atomicAdd(&P.pair_acc[1], my_hash);
    }
  }
  if (my_close) atomicAdd(P.too_close, my_close);
}

// ---------------------------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------------------------
template <int D>
static void launch_step_t(const Dev& P, const LaunchCfg& L, cudaStream_t s, uint64_t* launches,
                          cudaEvent_t e0 = nullptr, cudaEvent_t e1 = nullptr, bool rec = false) {
  const uint32_t nthr_nodes = P.n_chunks * 32;
  // programmatic dependent launch between the kernels of a step, except where events are
  // recorded between them (timed mode)
  const bool pdl = !e0 && !e1;
  launch_k(k_predict<D>, cdiv(P.N, 256), 256, 0, s, pdl, P);
  *launches += 1;
  launch_grid_build<D>(P, s, launches, pdl);
  if (P.enable_torque) {
    launch_k(k_torque_center<D>, cdiv(P.G, 128), 128, 0, s, pdl, P);
    *launches += 1;
  }
  if (e0) cudaEventRecord(e0, s);
  const dim3 grid(cdiv(nthr_nodes, L.force_block)), block(L.force_block);
  if (P.grain_contact) {
    if (rec) launch_k(k_force<D, true, true>, grid, block, 0, s, pdl, P);
    else launch_k(k_force<D, false, true>, grid, block, 0, s, pdl, P);
  } else {
    if (rec) launch_k(k_force<D, true, false>, grid, block, 0, s, pdl, P);
    else launch_k(k_force<D, false, false>, grid, block, 0, s, pdl, P);
  }
  if (e1) cudaEventRecord(e1, s);
  launch_k(k_finalize<D>, finalize_blocks(P.I), FINAL_THREADS, P.wrec_smem ? FINAL_SMEM : 0, s, pdl, P);
  *launches += 2;
}

cudaError_t kernels_init() {
  cudaError_t e = cudaFuncSetAttribute(k_finalize<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, FINAL_SMEM);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_finalize<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, FINAL_SMEM);
  if (e != cudaSuccess) return e;
  // the recording variants of the force kernel have local frames of about 1.1 KB
  const void* fs[] = {(const void*)k_force<2, false, false>, (const void*)k_force<2, false, true>,
                      (const void*)k_force<2, true, false>,  (const void*)k_force<2, true, true>,
                      (const void*)k_force<3, false, false>, (const void*)k_force<3, false, true>,
                      (const void*)k_force<3, true, false>,  (const void*)k_force<3, true, true>};
  size_t need = 0;
  e = max_local_bytes(fs, 8, &need);
  return e == cudaSuccess ? ensure_local_bytes(need) : e;
}

void launch_step(const Dev& P, const LaunchCfg& L, cudaStream_t s, uint64_t* launches, bool rec) {
  if (P.dim == 2) {
    launch_step_t<2>(P, L, s, launches, nullptr, nullptr, rec);
  } else {
    launch_step_t<3>(P, L, s, launches, nullptr, nullptr, rec);
  }
}

void launch_step_timed(const Dev& P, const LaunchCfg& L, cudaStream_t s, uint64_t* launches,
                       cudaEvent_t e0, cudaEvent_t e1) {
  if (P.dim == 2) {
    launch_step_t<2>(P, L, s, launches, e0, e1);
  } else {
    launch_step_t<3>(P, L, s, launches, e0, e1);
  }
}

uint32_t grid_coop_blocks(const Dev& P, int device) {
  int per_sm = 0, sms = 0, coop = 0;
  const void* k = P.dim == 2 ? (const void*)k_grid_coop<2> : (const void*)k_grid_coop<3>;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) != cudaSuccess || !coop) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, SCAN_THREADS, 0) != cudaSuccess || per_sm < 1) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms < 1) return 0;
  const uint32_t want = std::max(cdiv(P.N, SCAN_THREADS), cdiv(P.table_total, SCAN_TILE));
  // three blocks per SM: threads enough for the candidate-list phase, few blocks to schedule on
  // the (common) steps without a rebuild and to meet at the grid barriers (same box, collision
  // ensemble: 2 -> 3 blocks 0.0793 -> 0.0780 ms/step at skin 0.25; 4 and 5 blocks were slower
  // than 3, other workloads unchanged)
  return std::max(1u, std::min((uint32_t)(std::min(per_sm, 3) * sms), want));
}

const void* force_kernel_ptr(uint32_t dim) {
  return dim == 2 ? (const void*)k_force<2, false, false> : (const void*)k_force<3, false, false>;
}

// ---------------------------------------------------------------------------------------------
// Check kernel of the integer FP64 arithmetic (pg_ieee64.cuh): out[i] = op(a[i], b[i]), the
// division through a prepared divisor.
// ---------------------------------------------------------------------------------------------
__global__ void k_ieee64_check(int32_t op, const double* a, const double* b, int64_t n, double* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = a[i], y = b[i];
  double r;
  switch (op) {
    case PG_IEEE_DIV: r = ieee64::div_rn(x, ieee64::make_divisor(y)); break;
    case PG_IEEE_SQRT: r = ieee64::sqrt_rn(fabs(x)); break;
    case PG_IEEE_ADD: r = ieee64::add_rn(x, y); break;
    case PG_IEEE_SUB: r = ieee64::sub_rn(x, y); break;
    case PG_IEEE_MUL: r = ieee64::mul_rn(x, y); break;
    default: r = ieee64::widen_f32((float)x); break;
  }
  out[i] = r;
}

cudaError_t launch_ieee64_check(int32_t op, const double* a, const double* b, int64_t n, double* out,
                                cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t blocks = (n + 255) / 256;
  k_ieee64_check<<<(unsigned)blocks, 256, 0, s>>>(op, a, b, n, out);
  return cudaGetLastError();
}

}  // namespace pg
