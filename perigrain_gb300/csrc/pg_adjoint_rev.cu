// GB300 (sm_103a) kernels of the gradient path, reverse side: the hand-written adjoint of one
// frozen-mask time step (the forward map is spelled out in pg_adjoint.cu) and the per-grain
// parameter reduction.
//
// With cotangents (db, vb, ab) of the state (disp', vel', acc') after step t:
//   Fb   = (ab + 0.5*dt*vb) / rho                         cotangent of the force density
//   Xb   = (dF/dX)^T Fb  (+ wall-reaction cotangent at the objective's step)
//   Vf   = (dF/dvel)^T Fb
//   db_o = db + Xb ;  vb_o = vb + dt*(db + Xb) + Vf ;  ab_o = 0.5*dt*vb + (dt*dt*0.5)*(db + Xb)
// and the step's parameter cotangents are added per node. Every pair term is gathered at both of
// its nodes (a node reads its own contact list and finds itself in each partner's list), so the
// step is atomic-free and deterministic.
//
// Two kernels per reverse step. k_adj_bonds: one block per 32-node SELL chunk, SUB warps per
// block, warp w taking the node's bond slots k = w, w+SUB, ... (one coalesced access per warp and
// slot, as in the force kernels), partial sums added in shared memory in a fixed order; its bond
// products run in FP32 for mixed-precision handles (GB300 runs FP64 at a small fraction of its
// FP32 rate) and in FP64 for FP64 handles and frozen replays (the FP64 reference gradient).
// k_adj_rest: same chunk x SUB-warp split for contacts (entries round-robin over the warps),
// walls and the integrator, FP64; the cotangent state is FP64 throughout.
#include <cuda_runtime.h>

#include <cmath>

#include "pg_adjoint.cuh"
#include "pg_adjoint.h"
#include "pg_common.cuh"
#include "pg_device.cuh"

namespace pg {

constexpr int SUB = 4;

// Adjoint of one node-node contact force phi(y, r) received by a node of density rho from a
// partner of volume vq; y = x_partner - x_node, r = v_node - v_partner, g = cotangent of phi.
// Adds the cotangents of y and r to yb, rb and of (K_n, zeta, mu) to pb.
template <int D>
__device__ void pair_vjp(const double* y, const double* r, const double* g, double Kn, double Rc, double zeta,
                         double mu, double vq, double rho, uint32_t fr, bool damp, bool fric, double dt, double* yb,
                         double* rb, double* pb) {
  double n2 = 0.0;
  for (int c = 0; c < D; ++c) n2 += y[c] * y[c];
  const double dn = sqrt(n2);
  if (!(dn > 0.0)) return;
  const double idn = 1.0 / dn;
  double u[D];
  for (int c = 0; c < D; ++c) u[c] = y[c] * idn;
  double gu = 0.0;
  for (int c = 0; c < D; ++c) gu += g[c] * u[c];
  // elastic: phi1 = s1*u, s1 = -K_n (R_c - |y|) vol_q
  const double s1 = -Kn * (Rc - dn) * vq;
  for (int c = 0; c < D; ++c) yb[c] += Kn * vq * gu * u[c] + (s1 * idn) * (g[c] - gu * u[c]);
  pb[0] += -(Rc - dn) * vq * gu;
  if (!(damp || (fric && fr))) return;
  double ru = 0.0;
  for (int c = 0; c < D; ++c) ru += r[c] * u[c];
  if (damp) {
    // phi2 = -dc (r.u) u, dc = 2 zeta sqrt(K_n rho) sqrt(vol_q)
    const double sq = sqrt(Kn * rho) * sqrt(vq);
    const double dc = 2.0 * zeta * sq;
    for (int c = 0; c < D; ++c) {
      rb[c] += -dc * gu * u[c];
      yb[c] += -dc * (gu * (r[c] - ru * u[c]) + ru * (g[c] - gu * u[c])) * idn;
    }
    const double dcb = -ru * gu;
    pb[1] += dcb * 2.0 * sq;
    if (Kn != 0.0) pb[0] += dcb * dc / (2.0 * Kn);
  }
  if (!(fric && fr)) return;
  double z[D];
  if (fr == FR_STICK) {
    // phi3 = -tg / (rho dt), tg = r - (r.u) u
    for (int c = 0; c < D; ++c) z[c] = -g[c] / (rho * dt);
  } else {
    // phi3 = -mu cfn th, th = tg/|tg| (2D: the recorded direction +-perp(u)); cfn = |s1| = -s1
    // on the recorded run, continued as -s1 (the replay's smooth extension)
    const double cfn = -s1;
    const double sgn = -1.0;
    if constexpr (D == 2) {
      const double sg = (fr == FR_SLIDE_NEG) ? -1.0 : 1.0;
      const double th[2] = {-sg * u[1], sg * u[0]};
      const double a = g[0] * th[0] + g[1] * th[1];
      for (int c = 0; c < D; ++c) yb[c] += -mu * a * sgn * Kn * vq * u[c] + mu * cfn * gu * th[c] * idn;
      pb[2] += -cfn * a;
      pb[0] += -mu * a * vq * (Rc - dn);
      return;
    } else {
      double tg[D], t2 = 0.0;
      for (int c = 0; c < D; ++c) {
        tg[c] = r[c] - ru * u[c];
        t2 += tg[c] * tg[c];
      }
      const double tn = sqrt(t2);
      if (!(tn > 0.0)) return;
      double a = 0.0;
      for (int c = 0; c < D; ++c) a += g[c] * tg[c] / tn;
      for (int c = 0; c < D; ++c) {
        z[c] = -mu * cfn * (g[c] - a * tg[c] / tn) / tn;
        yb[c] += -mu * a * sgn * Kn * vq * u[c];
      }
      pb[2] += -cfn * a;
      pb[0] += -mu * a * vq * (Rc - dn);
    }
  }
  // through tg = r - (r.u) u
  double zu = 0.0;
  for (int c = 0; c < D; ++c) zu += z[c] * u[c];
  for (int c = 0; c < D; ++c) {
    rb[c] += z[c] - zu * u[c];
    yb[c] += -(zu * (r[c] - ru * u[c]) + ru * (z[c] - zu * u[c])) * idn;
  }
}

// Wall geometry of one side at distance dd <= R (segment_mass, contact.h:16-41): F = K_n*FK with
// FK = max(R - centroid, 0) * Area, and the derivatives d(Area)/d(dd), d(FK)/d(dd).
template <int D>
__device__ __forceinline__ void wall_geom(double R, double dd, double* A, double* Ap, double* FK, double* FKp) {
  if constexpr (D == 2) {
    const double s = sqrt(fmax(R * R - dd * dd, 0.0));
    *A = M_PI * R * R / 2 - R * R * asin(dd / R) - s * dd;
    *Ap = -2.0 * s;
    // the centroid is 0 (integer 2/3 in the reference), so FK = R * Area
    *FK = R * *A;
    *FKp = R * *Ap;
  } else {
    const double a = R - dd, b = R * R - dd * dd;
    *A = M_PI / 3 * a * a * (2 * R - dd);
    *Ap = -M_PI / 3 * a * (5 * R - 3 * dd);
    const double I = M_PI / 4 * b * b;
    const double Ip = -M_PI * dd * b;
    const double crc = R - I / *A;
    if (crc > 0) {
      *FK = R * *A - I;
      *FKp = R * *Ap - Ip;
    } else {
      *FK = 0.0;
      *FKp = 0.0;
    }
  }
}

// cotangent of the force on node j: Fb = (ab + 0.5 dt vb) / rho; zero where the force does not
// reach the state (grains that are not movable, clamped nodes)
template <int D>
__device__ __forceinline__ bool force_bar(const Dev& P, const AdjStep& A, uint32_t j, double* Fb) {
  const GrainDev& gj = P.grain[P.node_grain[j]];
  if (!(gj.flags & GF_MOVABLE) || P.clamped[j]) {
    for (int c = 0; c < D; ++c) Fb[c] = 0.0;
    return false;
  }
  double ab[D], vb[D];
  ldv<D>(A.ab, j, ab);
  ldv<D>(A.vb, j, vb);
  for (int c = 0; c < D; ++c) Fb[c] = gj.one_over_rho * (ab[c] + P.half_dt * vb[c]);
  return true;
}

// bond reference positions (hi/lo FP32, relative to the instance origin) from the mixed engine's
// bond record, and the displacement hi/lo pairs of a recorded step (same layout as the record's
// displacement part)
template <int D>
__device__ __forceinline__ void ld_xref(const float* __restrict__ bref, uint32_t N, uint32_t i, float (&xh)[D],
                                        float (&xl)[D]) {
  if constexpr (D == 2) {
    const float4 b = __ldg(reinterpret_cast<const float4*>(bref) + 2ull * i + 1);
    xh[0] = b.x;
    xh[1] = b.y;
    xl[0] = b.z;
    xl[1] = b.w;
  } else {
    for (int c = 0; c < D; ++c) {
      xh[c] = __ldg(bref + (size_t)(2 * D + c) * N + i);
      xl[c] = __ldg(bref + (size_t)(3 * D + c) * N + i);
    }
  }
}
template <int D>
__device__ __forceinline__ void ld_dhl(const float* __restrict__ df, uint32_t N, uint32_t i, float (&dh)[D],
                                       float (&dl)[D]) {
  if constexpr (D == 2) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(df) + i);
    dh[0] = a.x;
    dh[1] = a.y;
    dl[0] = a.z;
    dl[1] = a.w;
  } else {
    for (int c = 0; c < D; ++c) {
      dh[c] = __ldg(df + (size_t)c * N + i);
      dl[c] = __ldg(df + (size_t)(D + c) * N + i);
    }
  }
}
template <int D>
__device__ __forceinline__ void ldfv(const float* a, uint32_t i, float (&v)[D]) {
  if constexpr (D == 2) {
    const float2 t = reinterpret_cast<const float2*>(a)[i];
    v[0] = t.x;
    v[1] = t.y;
  } else {
    const float4 t = reinterpret_cast<const float4*>(a)[i];
    v[0] = t.x;
    v[1] = t.y;
    v[2] = t.z;
  }
}
template <int D>
__device__ __forceinline__ void stfv(float* a, uint32_t i, const float (&v)[D]) {
  if constexpr (D == 2) {
    reinterpret_cast<float2*>(a)[i] = make_float2(v[0], v[1]);
  } else {
    reinterpret_cast<float4*>(a)[i] = make_float4(v[0], v[1], v[2], 0.f);
  }
}

// Bond part of the reverse step: f_p = sum_j cnot vol_j s(eta) e(eta), eta = X_j - X_p; H =
// d(s e)/d(eta) is symmetric, so Xb_p = cnot sum_j H (vol_p Fb_j - vol_j Fb_p), and
// dF_p/dcnot = f_p / cnot. Writes the node's bond share of Xb (xbb) and of the cnot cotangent
// (pcb). F32: the mixed engine's form -- xi from the bond record's hi/lo reference positions,
// the displacement difference from the tape's hi/lo pairs, the cancellation-free stretch
// s = (2 xi.et + et.et) / (|xi| (|xi + et| + |xi|)), force cotangents from the FP32 array fbf.
template <int D, bool F32>
__global__ void __launch_bounds__(32 * SUB) k_adj_bonds(const Dev P, const AdjStep A) {
  pdl_enter();
  __shared__ double red[SUB][D + 1][32];
  const uint32_t lane = threadIdx.x & 31, sub = threadIdx.x >> 5;
  const uint32_t chunk = blockIdx.x;
  const uint32_t d = chunk * 32 + lane;
  const bool act = d < P.N;
  double part[D + 1];
  for (int v = 0; v <= D; ++v) part[v] = 0.0;
  const uint32_t g = act ? P.node_grain[d] : 0;
  const GrainDev& gr = P.grain[g];
  const bool mov = act && (gr.flags & GF_MOVABLE);
  if (mov) {
    const uint32_t t = *A.tstep;
    const uint32_t cdeg = P.chunk_deg[chunk];
    const uint32_t slot0 = P.chunk_slot[chunk] + lane;
    const uint32_t w0 = P.chunk_word[chunk];
    if constexpr (F32) {
      float dh[D], dl[D], xh[D], xl[D], Fb[D], xb[D], pc = 0.f;
      ld_dhl<D>(A.df, P.N, d, dh, dl);
      ld_xref<D>(P.bref, P.N, d, xh, xl);
      ldfv<D>(A.fbf, d, Fb);
      for (int c = 0; c < D; ++c) xb[c] = 0.f;
      const float volp = P.vol_f[d];
      for (uint32_t k = sub; k < cdeg; k += SUB) {
        const uint32_t s = slot0 + 32u * k;
        if (!bond_used(A.end_alive, A.break_step, w0 + k, lane, s, t)) continue;
        const uint32_t j = P.bcol[s];
        float jdh[D], jdl[D], jxh[D], jxl[D], Fj[D];
        ld_dhl<D>(A.df, P.N, j, jdh, jdl);
        ld_xref<D>(P.bref, P.N, j, jxh, jxl);
        ldfv<D>(A.fbf, j, Fj);
        const float volj = P.vol_f[j];
        float xi[D], et[D], y[D];
        for (int c = 0; c < D; ++c) {
          xi[c] = (jxh[c] - xh[c]) + (jxl[c] - xl[c]);
          et[c] = (jdh[c] - dh[c]) + (jdl[c] - dl[c]);
          y[c] = xi[c] + et[c];
        }
        float xx = 0.f, yy = 0.f, xe = 0.f, ee = 0.f;
        for (int c = 0; c < D; ++c) {
          xx = fmaf(xi[c], xi[c], xx);
          yy = fmaf(y[c], y[c], yy);
          xe = fmaf(xi[c], et[c], xe);
          ee = fmaf(et[c], et[c], ee);
        }
        const float ixn = rsqrtf(xx), iyn = rsqrtf(yy);
        const float str = __fdividef(fmaf(2.f, xe, ee) * ixn, fmaf(yy, iyn, xx * ixn));
        float e[D], w[D], ew = 0.f, eF = 0.f;
        for (int c = 0; c < D; ++c) {
          e[c] = y[c] * iyn;
          w[c] = volp * Fj[c] - volj * Fb[c];
          ew = fmaf(e[c], w[c], ew);
          eF = fmaf(e[c], Fb[c], eF);
        }
        for (int c = 0; c < D; ++c) xb[c] += e[c] * ew * ixn + str * (w[c] - e[c] * ew) * iyn;
        pc = fmaf(volj * str, eF, pc);
      }
      for (int c = 0; c < D; ++c) part[c] = gr.cnot * (double)xb[c];
      part[D] = (double)pc;
    } else {
      double Fb[D], xp[D];
      force_bar<D>(P, A, d, Fb);
      ldv<D>(A.X, d, xp);
      const double volp = P.vol[d];
      for (uint32_t k = sub; k < cdeg; k += SUB) {
        const uint32_t s = slot0 + 32u * k;
        if (!bond_used(A.end_alive, A.break_step, w0 + k, lane, s, t)) continue;
        const uint32_t j = P.bcol[s];
        const double xin = P.bxin[s];
        double xj[D], Fj[D], e[D];
        ldv<D>(A.X, j, xj);
        force_bar<D>(P, A, j, Fj);
        double n2 = 0.0;
        for (int c = 0; c < D; ++c) {
          e[c] = xj[c] - xp[c];
          n2 += e[c] * e[c];
        }
        const double en = sqrt(n2);
        const double ien = 1.0 / en, ixin = 1.0 / xin;
        for (int c = 0; c < D; ++c) e[c] *= ien;
        const double str = (en - xin) * ixin;
        const double volj = P.vol[j];
        double w[D], ew = 0.0, eF = 0.0;
        for (int c = 0; c < D; ++c) {
          w[c] = volp * Fj[c] - volj * Fb[c];
          ew += e[c] * w[c];
          eF += e[c] * Fb[c];
        }
        for (int c = 0; c < D; ++c) part[c] += gr.cnot * (e[c] * ew * ixin + str * (w[c] - e[c] * ew) * ien);
        part[D] += volj * str * eF;
      }
    }
  }
  // fixed-order sum of the SUB partial cotangents
  for (int v = 0; v <= D; ++v) red[sub][v][lane] = part[v];
  __syncthreads();
  if (sub != 0 || !act) return;
  double out[D];
  for (int c = 0; c < D; ++c) {
    double s = red[0][c][lane];
    for (int w = 1; w < SUB; ++w) s += red[w][c][lane];
    out[c] = s;
  }
  double pcs = red[0][D][lane];
  for (int w = 1; w < SUB; ++w) pcs += red[w][D][lane];
  stv<D>(A.xbb, d, out);
  A.pcb[d] = pcs;
}

// Contact, wall and integrator part of the reverse step: one block per 32-node chunk, SUB warps;
// warp w takes the node's contact entries i = w, w+SUB, ..., warp 0 also the walls; the partial
// cotangents are summed in shared memory in a fixed order and warp 0 adds the bond share from
// k_adj_bonds and runs the integrator. For the FP32 bond path it also writes the force cotangent
// of the next reverse step to fbf. In 2D at most 128 registers, 4 blocks per SM (138 unbounded,
// 3 per SM: a 592-chunk handle then ran 1.3 waves); 3D keeps its 168 registers, 3 blocks per SM.
template <int D>
__global__ void __launch_bounds__(32 * SUB, D == 2 ? 4 : 3) k_adj_rest(const Dev P, const AdjStep A) {
  pdl_enter();
  constexpr int NS = 2 * D;
  constexpr int NV = 2 * D + NPARAM;  // xb[D], vfb[D], pc[NPARAM]
  __shared__ double red[SUB][NV][32];
  const uint32_t lane = threadIdx.x & 31, sub = threadIdx.x >> 5;
  const uint32_t d = blockIdx.x * 32 + lane;
  const bool act = d < P.N;
  double acc[NV];
  for (int v = 0; v < NV; ++v) acc[v] = 0.0;
  double* xb = acc;
  double* vfb = acc + D;
  double* pc = acc + 2 * D;
  double Fb[D];
  uint32_t g = 0;
  bool live = false;
  if (act) {
    g = P.node_grain[d];
    live = force_bar<D>(P, A, d, Fb);
  }
  if (live) {
    const GrainDev gr = P.grain[g];
    const InstDev& in = P.inst[gr.inst];
    double xp[D], vp[D];
    ldv<D>(A.X, d, xp);
    ldv<D>(A.V, d, vp);
    const double volp = P.vol[d];

    // contacts: the node's own forces (its list) and the partners' forces from it (their lists)
    const bool damp = P.allow_damping, fric = P.allow_friction;
    const uint32_t o = A.off[d], n = A.cnt[d];
    for (uint32_t i = sub; i < n; i += SUB) {
      const uint32_t e = A.ent[o + i];
      const uint32_t q = e & ENT_NODE, fr = e >> 30;
      const uint32_t gqi = P.node_grain[q];
      const bool same = gqi == g;
      const GrainDev gq = P.grain[gqi];
      double Kn, Rc, zeta, mu;
      pair_params<D>(P, in, gr, gq, same, d, q, &Kn, &Rc, &zeta, &mu);
      double xq[D], vq[D], y[D], r[D];
      ldv<D>(A.X, q, xq);
      ldv<D>(A.V, q, vq);
      for (int c = 0; c < D; ++c) {
        y[c] = xq[c] - xp[c];
        r[c] = vp[c] - vq[c];
      }
      double yb[D], rb[D], pb[3] = {0.0, 0.0, 0.0};
      for (int c = 0; c < D; ++c) {
        yb[c] = 0.0;
        rb[c] = 0.0;
      }
      pair_vjp<D>(y, r, Fb, Kn, Rc, zeta, mu, P.vol[q], gr.rho, fr, damp, fric, P.dt, yb, rb, pb);
      for (int c = 0; c < D; ++c) {
        xb[c] -= yb[c];
        vfb[c] += rb[c];
      }
      if (same) {
        pc[0] += pb[0] / Rc;  // K_n' = cnot / R_c'
        pc[2] += pb[1];
        pc[3] += pb[2];
      } else {
        pc[1] += 0.5 * pb[0];
        pc[2] += 0.5 * pb[1];
        pc[3] += 0.5 * pb[2];
      }
      // the partner's force from this node, if the partner recorded it
      const uint32_t oq = A.off[q], nq = A.cnt[q];
      uint32_t frq = 4u;
      for (uint32_t k = 0; k < nq; ++k) {
        const uint32_t eq = A.ent[oq + k];
        if ((eq & ENT_NODE) == d) {
          frq = eq >> 30;
          break;
        }
      }
      if (frq == 4u) continue;
      double Fq[D];
      if (!force_bar<D>(P, A, q, Fq)) continue;
      double y2[D], r2[D], yb2[D], rb2[D], pb2[3] = {0.0, 0.0, 0.0};
      for (int c = 0; c < D; ++c) {
        y2[c] = xp[c] - xq[c];
        r2[c] = vq[c] - vp[c];
        yb2[c] = 0.0;
        rb2[c] = 0.0;
      }
      pair_vjp<D>(y2, r2, Fq, Kn, Rc, zeta, mu, volp, gq.rho, frq, damp, fric, P.dt, yb2, rb2, pb2);
      for (int c = 0; c < D; ++c) {
        xb[c] += yb2[c];
        vfb[c] -= rb2[c];
      }
      if (!same) {
        pc[1] += 0.5 * pb2[0];
        pc[2] += 0.5 * pb2[1];
        pc[3] += 0.5 * pb2[2];
      }
    }

    // walls: the node's force and, at the objective's step, its share of the wall reactions
    const uint32_t wbits = A.wall[d];
    if (sub == 0 && wbits) {
      const double R = in.contact_rad, Kn = gr.kn, rho = gr.rho;
      for (int k = 0; k < NS; ++k) {
        if (!wb_contact(wbits, k)) continue;
        int side, dir;
        wall_side<D>(k, &side, &dir);
        double gv[D];
        for (int c = 0; c < D; ++c) gv[c] = Fb[c];
        if (A.rbar) {
          // reaction[side] -= vol_p * (the node's wall force of this side)
          for (int c = 0; c < D; ++c) gv[c] -= volp * A.rbar[((size_t)gr.inst * NS + side) * D + c];
        }
        const double dist = xp[dir] - A.W[(size_t)gr.inst * NS + side];
        const double dd = fmin(fabs(dist), R);  // the replay's extension beyond R
        const double cs = dist > 0 ? 1.0 : -1.0;
        double Ar, Ap, FK, FKp;
        wall_geom<D>(R, dd, &Ar, &Ap, &FK, &FKp);
        const double F = Kn * FK, Fp = Kn * FKp;  // dF/d(dd); d(dd)/dX = cs
        // normal: f[dir] += cs F
        xb[dir] += gv[dir] * Fp;
        pc[1] += gv[dir] * cs * FK;
        double rv[D];
        for (int c = 0; c < D; ++c) rv[c] = vp[c];
        rv[dir] -= in.wall_speed[side];
        if (fric && wb_fric(wbits, k)) {
          const bool stick = wb_stick(wbits, k);
          const double sF = F > 0 ? 1.0 : (F < 0 ? -1.0 : 0.0);
          if constexpr (D == 2) {
            const int tg = (dir + 1) % 2;
            if (stick) {
              vfb[tg] += gv[tg] * (-rho / P.dt);
            } else {
              const double vts = wb_neg(wbits, k) ? -1.0 : 1.0;
              xb[dir] += gv[tg] * (-gr.mu * vts * sF * Fp * cs);
              pc[3] += gv[tg] * (-fabs(F) * vts);
              pc[1] += gv[tg] * (-gr.mu * vts * sF * FK);
            }
          } else {
            const int t1 = (dir + 1) % 3, t2 = (dir + 2) % 3;
            if (stick) {
              vfb[t1] += gv[t1] * (-1.0 / (rho * P.dt));
              vfb[t2] += gv[t2] * (-1.0 / (rho * P.dt));
            } else {
              const double v1 = rv[t1], v2 = rv[t2];
              const double vn = sqrt(v1 * v1 + v2 * v2);
              if (vn > 0) {
                const double u1 = v1 / vn, u2 = v2 / vn;
                const double a = gv[t1] * u1 + gv[t2] * u2;
                xb[dir] += -gr.mu * a * sF * Fp * cs;
                pc[3] += -fabs(F) * a;
                pc[1] += -gr.mu * a * sF * FK;
                vfb[t1] += -gr.mu * fabs(F) * (gv[t1] - a * u1) / vn;
                vfb[t2] += -gr.mu * fabs(F) * (gv[t2] - a * u2) / vn;
              }
            }
          }
        }
        if (damp) {
          // df = -dc rv[dir], dc = 2 zeta sqrt(K_n rho) sqrt(|Area|)
          const double sq = sqrt(Kn * rho);
          const double sa = sqrt(fabs(Ar));
          const double dc = 2.0 * gr.zeta * sq * sa;
          vfb[dir] += gv[dir] * (-dc);
          if (sa > 0) xb[dir] += gv[dir] * (-rv[dir]) * gr.zeta * sq * (Ap / sa) * cs;
          pc[2] += gv[dir] * (-rv[dir]) * 2.0 * sq * sa;
          if (Kn != 0.0) pc[1] += gv[dir] * (-rv[dir]) * dc / (2.0 * Kn);
        }
      }
    }
  }

  // fixed-order sum of the SUB partial cotangents, then the integrator (warp 0)
  for (int v = 0; v < NV; ++v) red[sub][v][lane] = acc[v];
  __syncthreads();
  if (sub != 0 || !act) return;
  if (!live) {
    // the state of this node does not depend on the parameters
    double zero[D];
    for (int c = 0; c < D; ++c) zero[c] = 0.0;
    stv<D>(A.db_o, d, zero);
    stv<D>(A.vb_o, d, zero);
    stv<D>(A.ab_o, d, zero);
    if (A.fbf) {
      float zf[D];
      for (int c = 0; c < D; ++c) zf[c] = 0.f;
      stfv<D>(A.fbf, d, zf);
    }
    return;
  }
  for (int v = 0; v < NV; ++v) {
    double sm = red[0][v][lane];
    for (int w = 1; w < SUB; ++w) sm += red[w][v][lane];
    acc[v] = sm;
  }
  double xbond[D];
  ldv<D>(A.xbb, d, xbond);
  for (int c = 0; c < D; ++c) xb[c] += xbond[c];
  pc[0] += A.pcb[d];
  const GrainDev& gr = P.grain[g];

  // integrator
  double db[D], vb[D], o1[D], o2[D], o3[D];
  ldv<D>(A.db, d, db);
  ldv<D>(A.vb, d, vb);
  for (int c = 0; c < D; ++c) {
    const double dtot = db[c] + xb[c];
    o1[c] = dtot;
    o2[c] = vb[c] + P.dt * dtot + vfb[c];
    o3[c] = P.half_dt * vb[c] + P.hdt2 * dtot;
  }
  stv<D>(A.db_o, d, o1);
  stv<D>(A.vb_o, d, o2);
  stv<D>(A.ab_o, d, o3);
  if (A.fbf) {
    // force cotangent of the previous step, for the FP32 bond kernel of the next reverse step
    float nf[D];
    for (int c = 0; c < D; ++c) nf[c] = (float)(gr.one_over_rho * (o3[c] + P.half_dt * o2[c]));
    stfv<D>(A.fbf, d, nf);
  }
  double* pa = A.pacc + (size_t)d * NPARAM;
  for (int k = 0; k < NPARAM; ++k) pa[k] += pc[k];
}

// force cotangents of the first reverse step from the seed cotangent (FP32 bond path)
template <int D>
__global__ void k_fb_init(const Dev P, const AdjStep A) {
  pdl_enter();
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= P.N) return;
  double Fb[D];
  force_bar<D>(P, A, d, Fb);
  float f[D];
  for (int c = 0; c < D; ++c) f[c] = (float)Fb[c];
  stfv<D>(A.fbf, d, f);
}

// per-grain sums of the per-node parameter cotangents, one block per grain, fixed order
__global__ void __launch_bounds__(256) k_grad_reduce(const Dev P, const double* pacc, double* grad) {
  __shared__ double sm[NPARAM][256];
  const uint32_t g = blockIdx.x;
  const GrainDev& gr = P.grain[g];
  double s[NPARAM] = {0.0, 0.0, 0.0, 0.0};
  for (uint32_t o = gr.node_begin + threadIdx.x; o < gr.node_end; o += blockDim.x) {  // input order
    const uint32_t i = at_of(P, o);
    for (int k = 0; k < NPARAM; ++k) s[k] += pacc[(size_t)i * NPARAM + k];
  }
  for (int k = 0; k < NPARAM; ++k) sm[k][threadIdx.x] = s[k];
  __syncthreads();
  for (uint32_t w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int k = 0; k < NPARAM; ++k) sm[k][threadIdx.x] += sm[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < NPARAM) grad[(size_t)g * NPARAM + threadIdx.x] = sm[threadIdx.x][0];
}

void launch_adjoint_step(const Dev& P, const AdjStep& A, cudaStream_t s, uint64_t* launches) {
  // programmatic dependent launch: each kernel waits on its predecessor in pdl_enter()
  const dim3 g(P.n_chunks), b(32 * SUB);
  if (P.dim == 2) {
    if (A.fbf) launch_k(k_adj_bonds<2, true>, g, b, 0, s, true, P, A);
    else launch_k(k_adj_bonds<2, false>, g, b, 0, s, true, P, A);
    launch_k(k_adj_rest<2>, g, b, 0, s, true, P, A);
  } else {
    if (A.fbf) launch_k(k_adj_bonds<3, true>, g, b, 0, s, true, P, A);
    else launch_k(k_adj_bonds<3, false>, g, b, 0, s, true, P, A);
    launch_k(k_adj_rest<3>, g, b, 0, s, true, P, A);
  }
  *launches += 2;
}

void launch_fb_init(const Dev& P, const AdjStep& A, cudaStream_t s, uint64_t* launches) {
  const uint32_t nb = (P.N + 127) / 128;
  if (P.dim == 2) {
    launch_k(k_fb_init<2>, nb, 128, 0, s, true, P, A);
  } else {
    launch_k(k_fb_init<3>, nb, 128, 0, s, true, P, A);
  }
  *launches += 1;
}

void launch_grad_reduce(const Dev& P, const double* pacc, double* grad, cudaStream_t s, uint64_t* launches) {
  if (P.G == 0) return;
  k_grad_reduce<<<P.G, 256, 0, s>>>(P, pacc, grad);
  *launches += 1;
}

}  // namespace pg
