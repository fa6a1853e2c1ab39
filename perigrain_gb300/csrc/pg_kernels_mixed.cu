// GB300 (sm_103a) kernels of the PeriDEM time step, mixed precision (PG_MIXED).
//
// State that accumulates over time stays FP64: disp, vel, pos and CurrPos. Everything per bond and
// per contact pair is FP32:
//   * the bond reference vector xi = x_j - x_i and the deformation eta = u_j - u_i are formed from
//     FP32 hi/lo pairs of the FP64 values, (hi_j - hi_i) + (lo_j - lo_i), which keeps ~48 bits of
//     the FP64 difference without an FP64 instruction;
//   * the stretch is evaluated without cancellation,
//       s = (|xi + eta| - |xi|) / |xi| = (2 xi.eta + eta.eta) / (|xi| (|xi + eta| + |xi|)),
//     so its relative error stays ~1e-7 even for stretches of 1e-6, where the reference form
//     would lose every digit in FP32;
//   * forces accumulate per node in FP32; the velocity update adds them to the FP64 state.
// The bond stream is the neighbour index plus one alive bit (4.125 B per directed bond; the FP64
// path also streams xi_norm). Compiled with FMA contraction on.
#include <cuda_runtime.h>

#include <cmath>

#include "pg_common.cuh"
#include "pg_device.cuh"
#include "pg_kernels_mixed.h"

namespace pg {

template <int D>
__device__ __forceinline__ void ld_hl(const float* a, uint32_t i, float (&h)[D], float (&l)[D]) {
  if constexpr (D == 2) {
    float4 t = reinterpret_cast<const float4*>(a)[i];
    h[0] = t.x;
    h[1] = t.y;
    l[0] = t.z;
    l[1] = t.w;
  } else {
    const float4* p = reinterpret_cast<const float4*>(a) + 2ull * i;
    float4 t0 = p[0], t1 = p[1];
    h[0] = t0.x;
    h[1] = t0.y;
    h[2] = t0.z;
    l[0] = t1.x;
    l[1] = t1.y;
    l[2] = t1.z;
  }
}
template <int D>
__device__ __forceinline__ void st_hl(float* a, uint32_t i, const double (&x)[D]) {
  float h[D], l[D];
  for (int c = 0; c < D; ++c) {
    h[c] = (float)x[c];
    l[c] = (float)(x[c] - (double)h[c]);
  }
  if constexpr (D == 2) {
    reinterpret_cast<float4*>(a)[i] = make_float4(h[0], h[1], l[0], l[1]);
  } else {
    float4* p = reinterpret_cast<float4*>(a) + 2ull * i;
    p[0] = make_float4(h[0], h[1], h[2], 0.f);
    p[1] = make_float4(l[0], l[1], l[2], 0.f);
  }
}
template <int D>
__device__ __forceinline__ void ldvf(const float* a, uint32_t i, float (&v)[D]) {
  if constexpr (D == 2) {
    float2 t = reinterpret_cast<const float2*>(a)[i];
    v[0] = t.x;
    v[1] = t.y;
  } else {
    float4 t = reinterpret_cast<const float4*>(a)[i];
    v[0] = t.x;
    v[1] = t.y;
    v[2] = t.z;
  }
}
template <int D>
__device__ __forceinline__ void stvf(float* a, uint32_t i, const float (&v)[D]) {
  if constexpr (D == 2) {
    reinterpret_cast<float2*>(a)[i] = make_float2(v[0], v[1]);
  } else {
    reinterpret_cast<float4*>(a)[i] = make_float4(v[0], v[1], v[2], 0.f);
  }
}
template <int D>
__device__ __forceinline__ float dotf(const float (&a)[D], const float (&b)[D]) {
  float s = a[0] * b[0];
  for (int c = 1; c < D; ++c) s = fmaf(a[c], b[c], s);
  return s;
}

// ---------------------------------------------------------------------------------------------
// position update: FP64 disp and CurrPos, plus their FP32 hi/lo images and the grid key
// ---------------------------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(256) k_predict_mx(const Dev P) {
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
      for (int c = 0; c < D; ++c) dp[c] = 0.0;
      P.clamp_pending[d] = 0;
      wrote = true;
    }
    if (gr.flags & GF_MOVABLE) {
      double v[D];
      float a[D];
      ldv<D>(P.vel_in, d, v);
      ldvf<D>(P.acc_f, d, a);
      for (int c = 0; c < D; ++c) dp[c] = dp[c] + fma(P.dt, v[c], P.hdt2 * (double)a[c]);
      wrote = true;
    }
    if (wrote) {
      stv<D>(P.disp, d, dp);
      st_hl<D>(P.disp_hl, d, dp);
    }
    ldv<D>(P.pos, d, ps);
    for (int c = 0; c < D; ++c) cu[c] = ps[c] + dp[c];
    stv<D>(P.cur, d, cu);
    const InstDev& in = P.inst[gr.inst];
    double rel[D];
    float rf[4] = {0.f, 0.f, 0.f, 0.f};
    int32_t ci[3] = {0, 0, 0};
    bool ok = true;
    for (int c = 0; c < D; ++c) {
      if (!isfinite(cu[c])) ok = false;
      rel[c] = cu[c] - in.origin[c];
      rf[c] = (float)rel[c];
      if (!(fabsf(rf[c]) <= in.range_f)) ok = false;
      ci[c] = (int32_t)floorf(rf[c] * in.inv_cell_f);
    }
    if (!ok) {
      set_status(P.status, isfinite(cu[0] + cu[1] + (D == 3 ? cu[D - 1] : 0.0)) ? PG_ERANGE : PG_ENAN);
      for (int c = 0; c < D; ++c) ci[c] = 0;
    }
    st_hl<D>(P.cur_hl, d, rel);
    if constexpr (D == 2) {
      reinterpret_cast<float2*>(P.curf)[d] = make_float2(rf[0], rf[1]);
    } else {
      reinterpret_cast<float4*>(P.curf)[d] = make_float4(rf[0], rf[1], rf[2], 0.f);
    }
    uint32_t m = (D == 2) ? morton2((uint32_t)ci[0], (uint32_t)ci[1])
                          : morton3((uint32_t)ci[0], (uint32_t)ci[1], (uint32_t)ci[2]);
    uint32_t key = in.table_off + (m & in.table_mask);
    P.cell_key[d] = key;
    P.cell_rank[d] = atomicAdd(&P.cell_count[key], 1u);
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
  const uint32_t full = 0xffffffffu;
  uint32_t g0 = __shfl_sync(full, g, 0);
  bool lane0_act = __shfl_sync(full, act ? 1 : 0, 0);
  if (!lane0_act) return;
  uint32_t same = __ballot_sync(full, !act || g == g0);
  if (same == full) {
    for (int c = 0; c < D; ++c) {
      for (int off = 16; off > 0; off >>= 1) {
        unsigned long long o1 = __shfl_down_sync(full, kmin[c], off);
        unsigned long long o2 = __shfl_down_sync(full, kmax[c], off);
        kmin[c] = o1 < kmin[c] ? o1 : kmin[c];
        kmax[c] = o2 > kmax[c] ? o2 : kmax[c];
      }
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

// ---------------------------------------------------------------------------------------------
// fused force + integrate, FP32 forces
// ---------------------------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(128) k_force_mx(const Dev P) {
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t chunk = d >> 5;
  if (chunk >= P.n_chunks) return;
  const bool act = d < P.N;
  const uint32_t t = *P.step;
  const uint32_t g = act ? P.node_grain[d] : 0;
  const GrainDev gr = P.grain[g];
  const bool mov = act && (gr.flags & GF_MOVABLE);
  const bool brk = P.enable_fracture && (gr.flags & GF_BREAKABLE) && (gr.flags & GF_BREAK_BONDS);
  const float cnot = (float)gr.cnot, snot = (float)gr.snot;

  float f[D];
  for (int c = 0; c < D; ++c) f[c] = 0.f;
  double vpd[D];
  if (act) ldv<D>(P.vel_in, d, vpd);

  const uint32_t cdeg = P.chunk_deg[chunk];
  const uint32_t slot0 = P.chunk_slot[chunk] + lane;
  const uint32_t w0 = P.chunk_word[chunk];
  {
    float dh[D], dl[D], xh[D], xl[D];
    if (mov) {
      ld_hl<D>(P.disp_hl, d, dh, dl);
      ld_hl<D>(P.xpos_hl, d, xh, xl);
    }
    for (uint32_t k = 0; k < cdeg; ++k) {
      const uint32_t word = P.alive[w0 + k];
      bool bit = (word >> lane) & 1u;
      if (mov && bit) {
        const uint32_t s = slot0 + 32u * k;
        const uint32_t j = P.bcol[s];
        float jdh[D], jdl[D], jxh[D], jxl[D];
        ld_hl<D>(P.disp_hl, j, jdh, jdl);
        ld_hl<D>(P.xpos_hl, j, jxh, jxl);
        const float vj = P.vol_f[j];
        float xi[D], et[D], y[D];
        for (int c = 0; c < D; ++c) {
          xi[c] = (jxh[c] - xh[c]) + (jxl[c] - xl[c]);
          et[c] = (jdh[c] - dh[c]) + (jdl[c] - dl[c]);
          y[c] = xi[c] + et[c];
        }
        const float xn = sqrtf(dotf<D>(xi, xi));
        const float yn = sqrtf(dotf<D>(y, y));
        const float num = fmaf(2.f, dotf<D>(xi, et), dotf<D>(et, et));
        const float str = num / (xn * (yn + xn));
        const float sc = (cnot * str * vj) / yn;
        for (int c = 0; c < D; ++c) f[c] = fmaf(sc, y[c], f[c]);
        if (brk && str > snot) {
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
  const InstDev& in = P.inst[gr.inst];
  const bool p_bdry = !P.nl_bdry_only || (act && P.bdry_rank[d] != NONE);
  const bool selfc = mov && P.enable_fracture && (gr.flags & GF_BREAKABLE) && P.self_contact;
  const bool other = mov && (gr.flags & GF_STOPPABLE);
  float vp[D];
  for (int c = 0; c < D; ++c) vp[c] = act ? (float)vpd[c] : 0.f;

  if ((selfc || other) && p_bdry) {
    double bmn[D], bmx[D];
    grain_box<D>(P, g, bmn, bmx);
    float ph[D], pl[D];
    ld_hl<D>(P.cur_hl, d, ph, pl);
    int32_t cc[3] = {0, 0, 0};
    for (int c = 0; c < D; ++c) cc[c] = (int32_t)floorf(ph[c] * in.inv_cell_f);
    const float thr2 = in.cell_f * in.cell_f;
    unsigned long long keys[MAX_CAND];
    uint32_t idx[MAX_CAND];
    int nc = 0;
    uint32_t seen[27];
    int nseen = 0;
    const int nnb = (D == 2) ? 9 : 27;
    for (int nb = 0; nb < nnb; ++nb) {
      int ox = nb % 3 - 1, oy = (nb / 3) % 3 - 1, oz = (D == 3) ? (nb / 9 - 1) : 0;
      uint32_t m = (D == 2) ? morton2((uint32_t)(cc[0] + ox), (uint32_t)(cc[1] + oy))
                            : morton3((uint32_t)(cc[0] + ox), (uint32_t)(cc[1] + oy), (uint32_t)(cc[2] + oz));
      uint32_t bucket = in.table_off + (m & in.table_mask);
      bool dup = false;
      for (int s = 0; s < nseen; ++s) dup = dup || (seen[s] == bucket);
      if (dup) continue;
      seen[nseen++] = bucket;
      const uint32_t b0 = P.cell_start[bucket], b1 = P.cell_start[bucket + 1];
      for (uint32_t b = b0; b < b1; ++b) {
        const uint32_t q = P.sorted[b];
        if (q == d) continue;
        float qf[D];
        ldf<D>(P.curf, q, qf);
        float d2 = 0.f;
        for (int c = 0; c < D; ++c) {
          float dd = qf[c] - ph[c];
          d2 = fmaf(dd, dd, d2);
        }
        if (d2 > thr2) continue;
        const uint32_t gq = P.node_grain[q];
        const bool same = (gq == g);
        if (same ? !selfc : !other) continue;
        if (P.nl_bdry_only && P.bdry_rank[q] == NONE) continue;
        if (!same) {
          double qmn[D], qmx[D];
          grain_box<D>(P, gq, qmn, qmx);
          if (!boxes_touch<D>(bmn, bmx, qmn, qmx, in.contact_rad)) continue;
        }
        const uint32_t sub = P.nl_bdry_only ? P.bdry_rank[q] : (q - P.grain[gq].node_begin);
        const unsigned long long key =
            ((unsigned long long)(same ? 0u : 1u) << 63) | ((unsigned long long)gq << 32) | sub;
        insert_cand<D>(keys, idx, nc, key, q, P);
      }
    }
    const uint32_t mydeg = P.node_deg[d];
    const float Rc0 = (float)in.contact_rad, Kn0 = (float)in.normal_stiffness;
    const float mu = (float)in.friction_coefficient, zeta = (float)in.damping_ratio;
    const float rho = (float)gr.rho, dtf = (float)P.dt;
    for (int ci = 0; ci < nc; ++ci) {
      const uint32_t q = idx[ci];
      const bool same = (keys[ci] >> 63) == 0;
      float qh[D], ql[D], dir[D];
      ld_hl<D>(P.cur_hl, q, qh, ql);
      for (int c = 0; c < D; ++c) dir[c] = (qh[c] - ph[c]) + (ql[c] - pl[c]);
      const float dn = sqrtf(dotf<D>(dir, dir));
      float Rc = Rc0, Kn = Kn0;
      if (same) {
        bool bonded = false;
        for (uint32_t k = 0; k < mydeg && !bonded; ++k) {
          if (((P.alive[w0 + k] >> lane) & 1u) && P.bcol[slot0 + 32u * k] == q) bonded = true;
        }
        if (bonded) continue;
        double pp[D], pq[D];
        ldv<D>(P.pos, d, pp);
        ldv<D>(P.pos, q, pq);
        float r[D];
        for (int c = 0; c < D; ++c) r[c] = (float)(pp[c] - pq[c]);
        const float ref = sqrtf(dotf<D>(r, r));
        Rc = ref < Rc0 ? ref : Rc0;
        Kn = (float)gr.cnot / Rc;
      }
      if (!(dn <= Rc)) continue;
      if (P.record_pairs) {
        my_pairs += 1;
        my_hash += splitmix64(((unsigned long long)d << 32) | q);
      }
      if (dn == 0.f) my_close += 1;
      const float inv = 1.f / dn;
      float u[D];
      for (int c = 0; c < D; ++c) u[c] = dir[c] * inv;
      const float nvol = P.vol_f[q];
      const float s1 = -Kn * (Rc - dn) * nvol;
      for (int c = 0; c < D; ++c) f[c] = fmaf(s1, u[c], f[c]);
      const float cfn = fabsf(s1);
      if (P.allow_damping || P.allow_friction) {
        double vqd[D];
        ldv<D>(P.vel_in, q, vqd);
        float rv[D];
        for (int c = 0; c < D; ++c) rv[c] = (float)(vpd[c] - vqd[c]);
        const float rvp = dotf<D>(rv, u);
        if (P.allow_damping) {
          const float dc = 2.f * zeta * sqrtf(Kn * rho) * sqrtf(nvol);
          for (int c = 0; c < D; ++c) f[c] = fmaf(-dc * rvp, u[c], f[c]);
        }
        if (P.allow_friction) {
          float tg[D];
          for (int c = 0; c < D; ++c) tg[c] = fmaf(-rvp, u[c], rv[c]);
          const float tn = sqrtf(dotf<D>(tg, tg));
          if (tn > 0.f) {
            float sfr = -mu * cfn;
            if (tn < mu * cfn * dtf / rho) sfr = -tn / rho / dtf;
            const float it = sfr / tn;
            for (int c = 0; c < D; ++c) f[c] = fmaf(it, tg[c], f[c]);
          }
        }
      }
    }
  }

  if (mov && other && p_bdry && in.allow_wall) {
    double bmn[D], bmx[D];
    grain_box<D>(P, g, bmn, bmx);
    if (!within_interior<D>(bmn, bmx, in.wall, in.contact_rad)) {
      double xc[D];
      ldv<D>(P.cur, d, xc);
      const double vol_i = (double)P.vol_f[d];
      const float R = (float)in.contact_rad, Kn = (float)in.normal_stiffness;
      const float mu = (float)in.friction_coefficient, zeta = (float)in.damping_ratio;
      const float rho = (float)gr.rho, dtf = (float)P.dt;
      constexpr int NS = 2 * D;
      const int order2[4][2] = {{3, 1}, {0, 0}, {1, 0}, {2, 1}};
      const int order3[6][2] = {{0, 0}, {3, 0}, {1, 1}, {4, 1}, {2, 2}, {5, 2}};
      for (int k = 0; k < NS; ++k) {
        const int side = (D == 2) ? order2[k][0] : order3[k][0];
        const int dir = (D == 2) ? order2[k][1] : order3[k][1];
        const float dist = (float)(xc[dir] - in.wall[side]);
        if (!(fabsf(dist) <= R)) continue;
        const float dd = fabsf(dist);
        float Area, I;
        if constexpr (D == 2) {
          Area = 0.5f * (float)M_PI * R * R - R * R * asinf(dd / R) - sqrtf(fmaxf(R * R - dd * dd, 0.f)) * dd;
          I = 0.f;
        } else {
          const float a = R - dd, b = R * R - dd * dd;
          Area = ((float)M_PI / 3.f) * a * a * (2.f * R - dd);
          I = ((float)M_PI / 4.f) * b * b;
        }
        const float centroid = I / Area;
        const float crc = R - centroid;
        const float F = Kn * (crc > 0.f ? crc : 0.f) * Area;
        const float c_sign = dist > 0.f ? 1.f : -1.f;
        f[dir] += c_sign * F;
        WallRec rec;
        rec.a_normal = vol_i * (double)(c_sign * F);
        rec.a_t1 = 0;
        rec.a_t2 = 0;
        rec.a_damp = 0;
        rec.gid = P.nl_bdry_only ? (gr.node_begin + P.bdry_rank[d]) : d;
        rec.side = (uint16_t)side;
        rec.has_fric = 0;
        rec.has_damp = 0;
        float rv[D];
        for (int c = 0; c < D; ++c) rv[c] = vp[c];
        rv[dir] -= (float)in.wall_speed[side];
        if (P.allow_friction) {
          if constexpr (D == 2) {
            const int tg = (dir + 1) % 2;
            if (fabsf(rv[tg]) > 0.f) {
              float ff = -mu * fabsf(F) * (rv[tg] > 0.f ? 1.f : -1.f);
              if (fabsf(rv[tg]) < mu * fabsf(F) * dtf / rho) ff = -rv[tg] * rho / dtf;
              f[tg] += ff;
              rec.a_t1 = vol_i * (double)ff;
              rec.has_fric = 1;
            }
          } else {
            const int t1 = (dir + 1) % 3, t2 = (dir + 2) % 3;
            const float vn = sqrtf(rv[t1] * rv[t1] + rv[t2] * rv[t2]);
            if (vn > 0.f) {
              const float u1 = rv[t1] / vn, u2 = rv[t2] / vn;
              float sfr = -mu * fabsf(F);
              if (vn < mu * fabsf(F) * dtf / rho) sfr = -vn / rho / dtf;
              f[t1] += sfr * u1;
              f[t2] += sfr * u2;
              rec.a_t1 = vol_i * (double)(sfr * u1);
              rec.a_t2 = vol_i * (double)(sfr * u2);
              rec.has_fric = 1;
            }
          }
        }
        if (P.allow_damping) {
          const float df = -(2.f * zeta * sqrtf(Kn * rho) * sqrtf(fabsf(Area))) * rv[dir];
          f[dir] += df;
          rec.a_damp = vol_i * (double)df;
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

  if (mov) {
    float ef[D];
    ldvf<D>(P.extf_f, d, ef);
    float sc = 1.f;
    if (P.gradient_extforce) {
      double scd = (double)t / (double)P.extforce_maxstep;
      sc = (float)(scd > 1 ? 1.0 : scd);
    }
    for (int c = 0; c < D; ++c) f[c] = fmaf(sc, ef[c], f[c]);
    if (P.enable_torque) {
      double xc[D];
      ldv<D>(P.cur, d, xc);
      const uint32_t ta = gr.torque_axis;
      float r[3] = {0, 0, 0}, rp[3] = {0, 0, 0};
      for (int c = 0; c < D; ++c) r[c] = (float)(xc[c] - P.torque_c[(size_t)g * 3 + c]);
      if (D == 3) r[ta] = 0;
      rp[(ta + 1) % 3] = -r[(ta + 2) % 3];
      rp[(ta + 2) % 3] = r[(ta + 1) % 3];
      float pn = 0.f;
      for (int c = 0; c < D; ++c) pn = fmaf(rp[c], rp[c], pn);
      pn = sqrtf(pn);
      const float tv = (float)gr.torque_val;
      if (pn > 0.f) {
        for (int c = 0; c < D; ++c) f[c] = fmaf(tv, rp[c] / pn, f[c]);
      }
    }
  }

  if (act) {
    if (mov) {
      float ao[D], a[D];
      double v[D];
      ldvf<D>(P.acc_f, d, ao);
      const float orho = (float)gr.one_over_rho;
      for (int c = 0; c < D; ++c) {
        a[c] = orho * f[c];
        v[c] = vpd[c] + ((double)ao[c] + (double)a[c]) * P.half_dt;
      }
      if (P.clamped[d]) {
        for (int c = 0; c < D; ++c) {
          a[c] = 0.f;
          v[c] = 0.0;
        }
        P.clamp_pending[d] = 1;
      }
      stvf<D>(P.acc_f, d, a);
      stv<D>(P.vel_out, d, v);
    } else {
      stv<D>(P.vel_out, d, vpd);
    }
    stvf<D>(P.force_f, d, f);
  }

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

template <int D>
static void launch_mx(const Dev& P, const LaunchCfg& L, cudaStream_t s, uint64_t* launches, cudaEvent_t e0,
                      cudaEvent_t e1) {
  k_predict_mx<D><<<cdiv(P.N, 256), 256, 0, s>>>(P);
  *launches += 1;
  launch_grid_build(P, s, launches);
  if (P.enable_torque) {
    k_torque_center<D><<<cdiv(P.G, 128), 128, 0, s>>>(P);
    *launches += 1;
  }
  if (e0) cudaEventRecord(e0, s);
  k_force_mx<D><<<cdiv(P.n_chunks * 32, L.force_block), L.force_block, 0, s>>>(P);
  if (e1) cudaEventRecord(e1, s);
  k_finalize<D><<<1, FINAL_THREADS, WREC_SMEM_CAP * sizeof(unsigned long long), s>>>(P);
  *launches += 2;
}

cudaError_t kernels_mixed_init() {
  cudaError_t e = cudaFuncSetAttribute(k_finalize<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       WREC_SMEM_CAP * (int)sizeof(unsigned long long));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_finalize<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              WREC_SMEM_CAP * (int)sizeof(unsigned long long));
}

void launch_step_mixed(const Dev& P, const LaunchCfg& L, cudaStream_t s, uint64_t* launches, cudaEvent_t e0,
                       cudaEvent_t e1) {
  if (P.dim == 2) {
    launch_mx<2>(P, L, s, launches, e0, e1);
  } else {
    launch_mx<3>(P, L, s, launches, e0, e1);
  }
}

}  // namespace pg
