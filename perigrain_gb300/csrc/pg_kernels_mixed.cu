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

// FP64 <-> FP32 moves done with integer instructions: GB300 executes FP64 arithmetic and the
// F2F conversions on its narrow FP64 pipe (~1/64 of the FP32 rate), so the per-node hi/lo split
// and the float->double widening below use bit manipulation on the INT pipe instead.
//
// trunc_f32: x truncated to 24 significant bits, as a float and (exactly) as a double. Values
// below the FP32 normal range become 0 (their size is < 1.2e-38); inf/NaN take the converting
// path so they propagate.
__device__ __forceinline__ float trunc_f32(double x, double* as_double) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned int hw = (unsigned int)(b >> 32);
  const int e = (int)((hw >> 20) & 0x7ffu);
  const unsigned int sgn = hw & 0x80000000u;
  if (e < 1023 - 126) {  // below the FP32 normal range: 0
    *as_double = 0.0;
    return __uint_as_float(sgn);
  }
  if (e > 1023 + 127) {  // beyond FP32 (inf/NaN included): inf or NaN, and lo = x - x
    *as_double = x;
    const bool nan = (e == 0x7ff) && ((b & 0xfffffffffffffull) != 0);
    return __uint_as_float(sgn | 0x7f800000u | (nan ? 0x400000u : 0u));
  }
  *as_double = __longlong_as_double((long long)(b & ~((1ull << 29) - 1)));
  return __uint_as_float(sgn | ((unsigned int)(e - 896) << 23) | (unsigned int)((b >> 29) & 0x7fffffu));
}
// Exact widening of a float; subnormal floats become a signed zero.
__device__ __forceinline__ double widen(float f) {
  const unsigned int b = __float_as_uint(f);
  const unsigned int e = (b >> 23) & 0xffu;
  const unsigned long long sgn = (unsigned long long)(b & 0x80000000u) << 32;
  if (e == 0) return __longlong_as_double((long long)sgn);
  const unsigned long long ee = (e == 0xff) ? 0x7ffull : (unsigned long long)(e + 896);
  return __longlong_as_double((long long)(sgn | (ee << 52) | ((unsigned long long)(b & 0x7fffffu) << 29)));
}
// hi/lo pair: x = hi + lo + O(2^-47 |x|); hi = trunc_f32(x), lo = trunc_f32(x - hi). When hi is an
// FP32 normal number the difference x - hi is exactly x's low 29 mantissa bits, so lo is formed
// from them with integer instructions (identical bits, no FP64 subtraction); otherwise the FP64
// route.
__device__ __forceinline__ void split_hl(double x, float* hi, float* lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned int hw = (unsigned int)(b >> 32);
  const int e = (int)((hw >> 20) & 0x7ffu);
  if (e < 1023 - 126 || e > 1023 + 127) {
    double hd, ld;
    *hi = trunc_f32(x, &hd);
    *lo = trunc_f32(x - hd, &ld);
    return;
  }
  const unsigned int sgn = hw & 0x80000000u;
  *hi = __uint_as_float(sgn | ((unsigned int)(e - 896) << 23) | (unsigned int)((b >> 29) & 0x7fffffu));
  const unsigned int r = (unsigned int)(b & ((1ull << 29) - 1));
  if (r == 0) {  // x - hi = +0
    *lo = 0.0f;
    return;
  }
  const int p = 31 - __clz(r);  // leading bit of the remainder
  const int ed = e + p - 52;     // biased FP64 exponent of x - hi
  if (ed < 1023 - 126) {         // below the FP32 normal range: signed zero
    *lo = __uint_as_float(sgn);
    return;
  }
  const unsigned int frac = (p <= 23) ? ((r << (23 - p)) & 0x7fffffu) : ((r >> (p - 23)) & 0x7fffffu);
  *lo = __uint_as_float(sgn | ((unsigned int)(ed - 896) << 23) | frac);
}

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
// bref layout. 2D: one 32-byte record per node, [disp hi.xy, disp lo.xy, xpos hi.xy, xpos lo.xy]
// (a neighbour gather touches one sector). 3D: 4*3 planes of N floats -- disp hi, disp lo, xpos
// hi, xpos lo (a padded 3D record would span two sectors; planes keep a warp's gather of the k-th
// neighbours of 32 consecutive nodes on consecutive entries).
template <int D>
__device__ __forceinline__ void ld_ref(const float* __restrict__ bref, uint32_t N, uint32_t i, float (&dh)[D],
                                       float (&dl)[D], float (&xh)[D], float (&xl)[D]) {
  if constexpr (D == 2) {
    const float4* p = reinterpret_cast<const float4*>(bref) + 2ull * i;
    const float4 a = __ldg(p), b = __ldg(p + 1);
    dh[0] = a.x;
    dh[1] = a.y;
    dl[0] = a.z;
    dl[1] = a.w;
    xh[0] = b.x;
    xh[1] = b.y;
    xl[0] = b.z;
    xl[1] = b.w;
  } else {
    for (int c = 0; c < D; ++c) {
      dh[c] = __ldg(bref + (size_t)c * N + i);
      dl[c] = __ldg(bref + (size_t)(D + c) * N + i);
      xh[c] = __ldg(bref + (size_t)(2 * D + c) * N + i);
      xl[c] = __ldg(bref + (size_t)(3 * D + c) * N + i);
    }
  }
}
template <int D>
__device__ __forceinline__ void st_ref_disp(float* bref, uint32_t N, uint32_t i, const double (&x)[D]) {
  float h[D], l[D];
  for (int c = 0; c < D; ++c) split_hl(x[c], &h[c], &l[c]);
  if constexpr (D == 2) {
    reinterpret_cast<float4*>(bref)[2ull * i] = make_float4(h[0], h[1], l[0], l[1]);
  } else {
    for (int c = 0; c < D; ++c) {
      bref[(size_t)c * N + i] = h[c];
      bref[(size_t)(D + c) * N + i] = l[c];
    }
  }
}

template <int D>
__device__ __forceinline__ void st_hl(float* a, uint32_t i, const double (&x)[D]) {
  float h[D], l[D];
  for (int c = 0; c < D; ++c) split_hl(x[c], &h[c], &l[c]);
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
  pdl_enter();
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31;
  const bool act = d < P.N;
  uint32_t g = 0;
  unsigned long long kmin[D], kmax[D];
  if (act) {
    // every per-node load is issued before the grain's flags are known, so they overlap
    g = P.node_grain[d];
    double dp[D], ps[D], cu[D], v[D];
    float a[D];
    ldv<D>(P.disp, d, dp);
    ldv<D>(P.vel_in, d, v);
    ldvf<D>(P.acc_f, d, a);
    ldv<D>(P.pos, d, ps);
    constexpr uint32_t SFB = (D == 2) ? 2 : 4;
    float db[D];
    for (int c = 0; c < D; ++c) db[c] = P.cand_q ? P.disp_b[(size_t)d * SFB + c] : 0.f;
    const bool pend = P.clamp_pending[d] != 0;
    const GrainDev& gr = P.grain[g];
    bool wrote = false;
    if (pend) {
      for (int c = 0; c < D; ++c) dp[c] = 0.0;
      P.clamp_pending[d] = 0;
      wrote = true;
    }
    if (gr.flags & GF_MOVABLE) {
      // the increment dt*v + (dt*dt/2)*a is formed in FP32 (relative error ~1e-7 of a step's
      // motion); the accumulation into disp stays FP64
      double vd;
      for (int c = 0; c < D; ++c) {
        const float vf = trunc_f32(v[c], &vd);
        dp[c] = dp[c] + widen(fmaf(P.dt_f, vf, P.hdt2_f * a[c]));
      }
      wrote = true;
    }
    if (wrote) {
      stv<D>(P.disp, d, dp);
      st_ref_disp<D>(P.bref, P.N, d, dp);
    }
    for (int c = 0; c < D; ++c) cu[c] = ps[c] + dp[c];
    stv<D>(P.cur, d, cu);
    const InstDev& in = P.inst[gr.inst];
    // the FP32 position image: offset from the fixed frame with candidate lists (independent of
    // the grid refit of the step before), else from this step's grid origin; formed in FP32 from
    // the truncated CurrPos (integer instructions) -- an FP64 subtraction here would run on the
    // narrow FP64 pipe, and the image only feeds the cell keys and the FP32 prefilter
    float rf[4] = {0.f, 0.f, 0.f, 0.f};
    bool ok = true;
    for (int c = 0; c < D; ++c) {
      if (((__double_as_longlong(cu[c]) >> 52) & 0x7ff) == 0x7ff) ok = false;  // inf or NaN
      double cut;
      rf[c] = trunc_f32(cu[c], &cut) - in.org_f[c];
    }
    if (!ok) set_status(P.status, PG_ENAN);
    if constexpr (D == 2) {
      reinterpret_cast<float2*>(P.curf)[d] = make_float2(rf[0], rf[1]);
    } else {
      reinterpret_cast<float4*>(P.curf)[d] = make_float4(rf[0], rf[1], rf[2], 0.f);
    }
    if (P.cand_q) {
      // candidate lists: keys only on rebuild steps (k_keys); rebuild once any node has moved
      // 0.45 skin since the last build. Nothing here reads the grid, which the previous step's
      // finalize may be refitting at the same time.
      float m2 = 0.f;
      for (int c = 0; c < D; ++c) {
        double dpt;
        const float dd = trunc_f32(dp[c], &dpt) - db[c];  // truncation (integer ops), not an FP64 conversion
        m2 += dd * dd;
      }
      if (m2 > in.skin_lim2) *P.rebuild = 1;
    } else {
      int32_t ci[3] = {0, 0, 0};
      for (int c = 0; c < D; ++c) ci[c] = cell_coord(rf[c] + in.frame_off_f[c], in.inv_cell_f, in.dims[c]);
      const uint32_t key =
          in.table_off + ((uint32_t)ci[2] * in.dims[1] + (uint32_t)ci[1]) * in.dims[0] + (uint32_t)ci[0];
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

// One bond: stretch s = (2 xi.eta + eta.eta) / (|xi| (|xi+eta| + |xi|)), force density
// cnot * s * vol_j * (xi+eta)/|xi+eta| added to f when `use`. cv = cnot * vol_j.
template <int D>
__device__ __forceinline__ void bond_term(const float (&dh)[D], const float (&dl)[D], const float (&xh)[D],
                                          const float (&xl)[D], const float (&jdh)[D], const float (&jdl)[D],
                                          const float (&jxh)[D], const float (&jxl)[D], float cv, bool use,
                                          float (&f)[D], float* str_out) {
  float xi[D], et[D], y[D];
  for (int c = 0; c < D; ++c) {
    xi[c] = (jxh[c] - xh[c]) + (jxl[c] - xl[c]);
    et[c] = (jdh[c] - dh[c]) + (jdl[c] - dl[c]);
    y[c] = xi[c] + et[c];
  }
  const float xx = dotf<D>(xi, xi), yy = dotf<D>(y, y);
  const float ixn = rsqrtf(xx), iyn = rsqrtf(yy);
  const float num = fmaf(2.f, dotf<D>(xi, et), dotf<D>(et, et));
  const float str = __fdividef(num * ixn, fmaf(yy, iyn, xx * ixn));
  const float sc = use ? cv * str * iyn : 0.f;
  for (int c = 0; c < D; ++c) f[c] = fmaf(sc, y[c], f[c]);
  *str_out = str;
}

// ---------------------------------------------------------------------------------------------
// fused force + integrate, FP32 forces
// ---------------------------------------------------------------------------------------------
// The input's index of device node i in a force kernel: PERM (the handle's node layout differs
// from the input order) looks it up, otherwise the layout is the input order and i is it.
template <bool PERM>
__device__ __forceinline__ uint32_t input_index(const Dev& P, uint32_t i) {
  if constexpr (PERM) return P.node_orig[i];
  return i;
}

template <int D, bool REC, bool GC, bool PERM>
__global__ void __launch_bounds__(128) k_force_mx(const Dev P) {
  pdl_enter();
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t chunk = d >> 5;
  if (chunk >= P.n_chunks) return;
  const bool act = d < P.N;
  const uint32_t t = *P.step;
  const uint32_t g = act ? P.node_grain[d] : 0;
  const GrainDev gr = P.grain[g];
  const bool mov = act && (gr.flags & GF_MOVABLE);

  float f[D];
  for (int c = 0; c < D; ++c) f[c] = 0.f;
  double vpd[D];
  if (act) ldv<D>(P.vel_in, d, vpd);
  // per-node inputs of the epilogue: in 2D loaded up front so their latency hides behind the bond
  // loop; in 3D where they are used (the extra live registers spill there and measured slower)
  constexpr int DE = (D == 2) ? D : 1;
  float ef_in[DE], ao_in[DE];
  bool clamped_in = false;
  if constexpr (D == 2) {
    if (mov) {
      ldvf<D>(P.extf_f, d, ef_in);
      ldvf<D>(P.acc_f, d, ao_in);
      clamped_in = P.clamped[d] != 0;
    }
  }

  const bool brk = P.enable_fracture && (gr.flags & GF_BREAKABLE) && (gr.flags & GF_BREAK_BONDS);
  const float cnot = gr.cnot_f, snot = gr.snot_f;
  const uint32_t cdeg = P.chunk_deg[chunk];
  const uint32_t slot0 = P.chunk_slot[chunk] + lane;
  const uint32_t w0 = P.chunk_word[chunk];
  {
    // bond forces and bond breaking (particle2.h:102-232): two bonds per iteration, both
    // neighbour gathers issued before either is used
    float dh[D], dl[D], xh[D], xl[D];
    if (mov) ld_ref<D>(P.bref, P.N, d, dh, dl, xh, xl);
    if constexpr (REC) {
      if (mov && P.rec_df) {
        if constexpr (D == 2) {
          reinterpret_cast<float4*>(P.rec_df)[d] = make_float4(dh[0], dh[1], dl[0], dl[1]);
        } else {
          for (int c = 0; c < D; ++c) {
            P.rec_df[(size_t)c * P.N + d] = dh[c];
            P.rec_df[(size_t)(D + c) * P.N + d] = dl[c];
          }
        }
      }
    }
    // the alive words and neighbour indices of the next pair are loaded one iteration ahead, so
    // only the neighbour gathers wait on memory in each iteration. A lane past the last node (d >= N
    // in the last chunk) gathers its own index for bonds it never uses: bref and vol_f are allocated
    // in whole chunks (zero padding), so those reads stay inside the arrays.
    uint32_t wa_n = 0u, wb_n = 0u, ca_n = d, cb_n = d;
    if (cdeg > 0) {
      wa_n = P.alive[w0];
      ca_n = P.bcol[slot0];
    }
    if (cdeg > 1) {
      wb_n = P.alive[w0 + 1];
      cb_n = P.bcol[slot0 + 32u];
    }
    for (uint32_t k = 0; k < cdeg; k += 2) {
      const bool two = (k + 1) < cdeg;
      const uint32_t wa = wa_n, wb = wb_n, ca = ca_n, cb = cb_n;
      if (k + 2 < cdeg) {
        wa_n = P.alive[w0 + k + 2];
        ca_n = P.bcol[slot0 + 32u * (k + 2)];
      }
      if (k + 3 < cdeg) {
        wb_n = P.alive[w0 + k + 3];
        cb_n = P.bcol[slot0 + 32u * (k + 3)];
      } else {
        wb_n = 0u;
        cb_n = d;
      }
      bool ba = (wa >> lane) & 1u, bb = (wb >> lane) & 1u;
      const bool ua = mov && ba, ub = mov && bb;
      const uint32_t sa = slot0 + 32u * k, sb = sa + 32u;
      const uint32_t ja = ua ? ca : d;
      const uint32_t jb = ub ? cb : d;
      float adh[D], adl[D], axh[D], axl[D], bdh[D], bdl[D], bxh[D], bxl[D];
      ld_ref<D>(P.bref, P.N, ja, adh, adl, axh, axl);
      ld_ref<D>(P.bref, P.N, jb, bdh, bdl, bxh, bxl);
      const float va = P.vol_f[ja], vb = P.vol_f[jb];
      float stra, strb;
      bond_term<D>(dh, dl, xh, xl, adh, adl, axh, axl, cnot * va, ua, f, &stra);
      bond_term<D>(dh, dl, xh, xl, bdh, bdl, bxh, bxl, cnot * vb, ub, f, &strb);
      if (brk && ua && stra > snot) {
        ba = false;
        P.break_step[sa] = t;
      }
      if (brk && ub && strb > snot) {
        bb = false;
        P.break_step[sb] = t;
      }
      const uint32_t na = __ballot_sync(0xffffffffu, ba);
      const uint32_t nb = __ballot_sync(0xffffffffu, bb);
      if (lane == 0) {
        if (na != wa) P.alive[w0 + k] = na;
        if (two && nb != wb) P.alive[w0 + k + 1] = nb;
      }
    }
  }
  __syncwarp();
  __syncwarp();

  unsigned long long my_pairs = 0, my_hash = 0, my_close = 0;
  uint32_t rent[REC ? MAX_CAND : 1];  // recorded contact entries of this node (REC only)
  uint32_t nrec = 0, wbits = 0;
  const InstDev& in = P.inst[gr.inst];
  const bool p_bdry = !P.nl_bdry_only || (act && P.bdry_rank[d] != NONE);
  const bool selfc = mov && P.enable_fracture && (gr.flags & GF_BREAKABLE) && P.self_contact;
  const bool other = mov && (P.worm || (gr.flags & GF_STOPPABLE));

  // with candidate lists a node whose list is empty has no contact this step
  const uint32_t ncl = (P.cand_q && act) ? (uint32_t)P.cand_n[d] : 0u;
  if ((selfc || other) && p_bdry && (!P.cand_q || ncl > 0)) {
    double bmn[D], bmx[D];
    grain_box<D>(P, g, bmn, bmx);
    float ph[D];
    ldf<D>(P.curf, d, ph);
    int32_t cc[3] = {0, 0, 0};
    for (int c = 0; c < D; ++c) cc[c] = cell_coord(ph[c] + in.frame_off_f[c], in.inv_cell_f, in.dims[c]);
    const float thr2 = in.pre_f * in.pre_f;
    unsigned long long keys[MAX_CAND];
    uint32_t idx[MAX_CAND];
    int nc = 0;
    // one candidate q of node d: the FP32 prefilter, the contact rules and the grain-box test,
    // then insertion in the reference's visit order
    auto consider = [&](uint32_t q) {
      float qf[D];
      ldf<D>(P.curf, q, qf);
      const uint32_t gq = P.node_grain[q];  // issued with the position, used after the prefilter
      float d2 = 0.f;
      for (int c = 0; c < D; ++c) {
        float dd = qf[c] - ph[c];
        d2 = fmaf(dd, dd, d2);
      }
      if (d2 > thr2) return;
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
      uint32_t qn = ncl ? P.cand_q[cbase] : d;  // the next entry is loaded one candidate ahead
      for (uint32_t k = 0; k < ncl; ++k) {
        const uint32_t q = qn;
        if (k + 1 < ncl) qn = P.cand_q[cbase + (size_t)(k + 1) * 32];
        consider(q);
      }
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
    // the pair log hashes input indices (the node's own looked up once; recorded runs only)
    const unsigned long long od_hash = P.record_pairs ? ((unsigned long long)input_index<PERM>(P, d) << 32) : 0ull;
    const float Kn0 = (float)in.normal_stiffness;
    const float mu0 = (float)in.friction_coefficient, zeta0 = (float)in.damping_ratio;
    const float rho = (float)gr.rho, dtf = (float)P.dt;
    double xp64[D];
    if (nc) ldv<D>(P.cur, d, xp64);
    for (int ci = 0; ci < nc; ++ci) {
      const uint32_t q = idx[ci];
      const bool same = (keys[ci] >> 63) == 0;
      // The contact decision |x_q - x_p| <= R_c' is made with the reference's FP64 arithmetic:
      // contact damping switches on at full strength at that boundary, so a decision flipped by
      // FP32 rounding would kick a node by metres per second.
      double xq64[D], dir64[D];
      ldv<D>(P.cur, q, xq64);
      for (int c = 0; c < D; ++c) dir64[c] = xq64[c] - xp64[c];
      double n2 = dir64[0] * dir64[0];
      for (int c = 1; c < D; ++c) n2 = n2 + dir64[c] * dir64[c];
      // dn64 <= R_c' <= contact_rad needs n2 <= contact_s_max (the same outcome as the sqrt
      // test): candidates beyond it skip the square root and the bonded-neighbour scan
      if (!(n2 <= in.contact_s_max)) continue;
      const double dn64 = sqrt(n2);
      double Rc64 = in.contact_rad;
      float Kn = Kn0, zeta = zeta0, mu = mu0;
      if constexpr (GC) {
        const GrainDev& gq = P.grain[(uint32_t)(keys[ci] >> 32) & 0x7fffffffu];
        Kn = (float)((gr.kn + gq.kn) * 0.5);
        zeta = (float)((gr.zeta + gq.zeta) * 0.5);
        mu = (float)((gr.mu + gq.mu) * 0.5);
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
        const double ref = sqrt(r2);
        Rc64 = ref < in.contact_rad ? ref : in.contact_rad;
        Kn = (float)(gr.cnot / Rc64);
      }
      if (!(dn64 <= Rc64)) continue;
      const float Rc = (float)Rc64, dn = (float)dn64;
      float dir[D];
      for (int c = 0; c < D; ++c) dir[c] = (float)dir64[c];
      if (P.record_pairs) {
        my_pairs += 1;
        my_hash += splitmix64(od_hash | input_index<PERM>(P, q));
      }
      if (dn == 0.f) my_close += 1;
      const float inv = 1.f / dn;
      float u[D];
      for (int c = 0; c < D; ++c) u[c] = dir[c] * inv;
      const float nvol = P.vol_f[q];
      const float s1 = -Kn * (Rc - dn) * nvol;
      for (int c = 0; c < D; ++c) f[c] = fmaf(s1, u[c], f[c]);
      const float cfn = fabsf(s1);
      uint32_t fr = 0;
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
            fr = (D == 2 && (tg[1] * u[0] - tg[0] * u[1]) < 0.f) ? FR_SLIDE_NEG : FR_SLIDE;
            if (tn < mu * cfn * dtf / rho) {
              sfr = -tn / rho / dtf;
              fr = FR_STICK;
            }
            const float it = sfr / tn;
            for (int c = 0; c < D; ++c) f[c] = fmaf(it, tg[c], f[c]);
          }
        }
      }
      if constexpr (REC) rent[nrec++] = q | (fr << 30);
    }
  }

  if (mov && other && p_bdry && in.allow_wall) {
    double bmn[D], bmx[D];
    grain_box<D>(P, g, bmn, bmx);
    if (!within_interior<D>(bmn, bmx, in.wall, in.contact_rad)) {
      double xc[D];
      ldv<D>(P.cur, d, xc);
      const double vol_i = (double)P.vol_f[d];
      const float R = (float)in.contact_rad;
      const float Kn = (float)(GC ? gr.kn : in.normal_stiffness);
      const float mu = (float)(GC ? gr.mu : in.friction_coefficient);
      const float zeta = (float)(GC ? gr.zeta : in.damping_ratio);
      const float rho = (float)gr.rho, dtf = (float)P.dt;
      constexpr int NS = 2 * D;
      const int order2[4][2] = {{3, 1}, {0, 0}, {1, 0}, {2, 1}};
      const int order3[6][2] = {{0, 0}, {3, 0}, {1, 1}, {4, 1}, {2, 2}, {5, 2}};
      for (int k = 0; k < NS; ++k) {
        const int side = (D == 2) ? order2[k][0] : order3[k][0];
        const int dir = (D == 2) ? order2[k][1] : order3[k][1];
        const float dist = (float)(xc[dir] - in.wall[side]);
        if (!(fabsf(dist) <= R)) continue;
        wbits |= 1u << (4 * k);
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
        rec.gid = P.nl_bdry_only ? (gr.node_begin + P.bdry_rank[d]) : input_index<PERM>(P, d);
        rec.side = (uint16_t)side;
        rec.has_fric = 0;
        rec.has_damp = 0;
        float rv[D];
        for (int c = 0; c < D; ++c) rv[c] = (float)vpd[c];
        rv[dir] -= (float)in.wall_speed[side];
        if (P.allow_friction) {
          if constexpr (D == 2) {
            const int tg = (dir + 1) % 2;
            if (fabsf(rv[tg]) > 0.f) {
              float ff = -mu * fabsf(F) * (rv[tg] > 0.f ? 1.f : -1.f);
              wbits |= (rv[tg] > 0.f ? 2u : 10u) << (4 * k);
              if (fabsf(rv[tg]) < mu * fabsf(F) * dtf / rho) {
                ff = -rv[tg] * rho / dtf;
                wbits |= 4u << (4 * k);
              }
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
              wbits |= 2u << (4 * k);
              if (vn < mu * fabsf(F) * dtf / rho) {
                sfr = -vn / rho / dtf;
                wbits |= 4u << (4 * k);
              }
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

  if (mov && P.worm) {
    float ef[D];
    if constexpr (D == 2) {
      for (int c = 0; c < D; ++c) ef[c] = ef_in[c];
    } else {
      ldvf<D>(P.extf_f, d, ef);
    }
    const float gate = (float)((worm_phase(t) + 1u) % 2u);
    for (int c = 0; c < D; ++c) f[c] = fmaf(gate, ef[c], f[c]);
  } else if (mov) {
    float ef[D];
    if constexpr (D == 2) {
      for (int c = 0; c < D; ++c) ef[c] = ef_in[c];
    } else {
      ldvf<D>(P.extf_f, d, ef);
    }
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
      if constexpr (D == 2) {
        for (int c = 0; c < D; ++c) ao[c] = ao_in[c];
      } else {
        ldvf<D>(P.acc_f, d, ao);
      }
      const float orho = gr.one_over_rho_f, hdt = P.half_dt_f;
      for (int c = 0; c < D; ++c) {
        a[c] = orho * f[c];
        v[c] = vpd[c] + widen((ao[c] + a[c]) * hdt);  // FP64 accumulation of an FP32 increment
      }
      if ((D == 2) ? clamped_in : (P.clamped[d] != 0)) {
        for (int c = 0; c < D; ++c) {
          a[c] = 0.f;
          v[c] = 0.0;
        }
        P.clamp_pending[d] = 1;
      }
      if (P.worm) worm_clamp<D>(input_index<PERM>(P, d) - gr.node_begin, worm_phase(t), a, v);
      stvf<D>(P.acc_f, d, a);
      stv<D>(P.vel_out, d, v);
    } else {
      stv<D>(P.vel_out, d, vpd);
    }
    stvf<D>(P.force_f, d, f);
  }

  if constexpr (REC) {
    record_masks(P, d, act, lane, rent, nrec, wbits);
    if (P.rec_x) {
      double xr[D];
      if (act) ldv<D>(P.cur, d, xr);
      record_tape<D>(P, d, act, t, xr, vpd);
    }
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

// The force kernel's variants: mask recording (REC), per-grain contact parameters (GC) and a node
// layout other than the input order (PERM) are compiled in only where used, so the plain kernel
// keeps its register budget.
template <int D>
static void launch_force_mx(const Dev& P, dim3 grid, dim3 block, cudaStream_t s, bool pdl, bool rec) {
  const bool perm = P.node_orig != nullptr;
  if (P.grain_contact) {
    if (rec) perm ? launch_k(k_force_mx<D, true, true, true>, grid, block, 0, s, pdl, P)
                  : launch_k(k_force_mx<D, true, true, false>, grid, block, 0, s, pdl, P);
    else perm ? launch_k(k_force_mx<D, false, true, true>, grid, block, 0, s, pdl, P)
              : launch_k(k_force_mx<D, false, true, false>, grid, block, 0, s, pdl, P);
  } else {
    if (rec) perm ? launch_k(k_force_mx<D, true, false, true>, grid, block, 0, s, pdl, P)
                  : launch_k(k_force_mx<D, true, false, false>, grid, block, 0, s, pdl, P);
    else perm ? launch_k(k_force_mx<D, false, false, true>, grid, block, 0, s, pdl, P)
              : launch_k(k_force_mx<D, false, false, false>, grid, block, 0, s, pdl, P);
  }
}

template <int D>
static void launch_mx(const Dev& P, const LaunchCfg& L, cudaStream_t s, uint64_t* launches, cudaEvent_t e0,
                      cudaEvent_t e1, bool rec) {
  const uint32_t nthr = P.n_chunks * 32;
  // programmatic dependent launch between the kernels of a step, except where events are
  // recorded between them (timed mode)
  const bool pdl = !e0 && !e1;
  launch_k(k_predict_mx<D>, cdiv(P.N, 256), 256, 0, s, pdl, P);
  *launches += 1;
  launch_grid_build<D>(P, s, launches, pdl);
  if (P.enable_torque) {
    launch_k(k_torque_center<D>, cdiv(P.G, 128), 128, 0, s, pdl, P);
    *launches += 1;
  }
  if (e0) cudaEventRecord(e0, s);
  const dim3 grid(cdiv(nthr, L.force_block)), block(L.force_block);
  launch_force_mx<D>(P, grid, block, s, pdl, rec);
  if (e1) cudaEventRecord(e1, s);
  launch_k(k_finalize<D>, finalize_blocks(P.I), FINAL_THREADS, P.wrec_smem ? FINAL_SMEM : 0, s, pdl, P);
  *launches += 2;
}

cudaError_t kernels_mixed_init() {
  cudaError_t e = cudaFuncSetAttribute(k_finalize<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, FINAL_SMEM);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_finalize<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, FINAL_SMEM);
  if (e != cudaSuccess) return e;
  // the recording variants of the force kernel have local frames of about 1.1 KB
  const void* fs[] = {
      (const void*)k_force_mx<2, false, false, false>, (const void*)k_force_mx<2, false, true, false>,
      (const void*)k_force_mx<2, true, false, false>,  (const void*)k_force_mx<2, true, true, false>,
      (const void*)k_force_mx<3, false, false, false>, (const void*)k_force_mx<3, false, true, false>,
      (const void*)k_force_mx<3, true, false, false>,  (const void*)k_force_mx<3, true, true, false>,
      (const void*)k_force_mx<2, false, false, true>,  (const void*)k_force_mx<2, false, true, true>,
      (const void*)k_force_mx<2, true, false, true>,   (const void*)k_force_mx<2, true, true, true>,
      (const void*)k_force_mx<3, false, false, true>,  (const void*)k_force_mx<3, false, true, true>,
      (const void*)k_force_mx<3, true, false, true>,   (const void*)k_force_mx<3, true, true, true>};
  size_t need = 0;
  e = max_local_bytes(fs, 16, &need);
  return e == cudaSuccess ? ensure_local_bytes(need) : e;
}

void launch_step_mixed(const Dev& P, const LaunchCfg& L, cudaStream_t s, uint64_t* launches, cudaEvent_t e0,
                       cudaEvent_t e1, bool rec) {
  if (P.dim == 2) {
    launch_mx<2>(P, L, s, launches, e0, e1, rec);
  } else {
    launch_mx<3>(P, L, s, launches, e0, e1, rec);
  }
}

void launch_mixed_predict(const Dev& P, cudaStream_t s, bool pdl, uint64_t* launches) {
  if (P.dim == 2) {
    launch_k(k_predict_mx<2>, cdiv(P.N, 256), 256, 0, s, pdl, P);
  } else {
    launch_k(k_predict_mx<3>, cdiv(P.N, 256), 256, 0, s, pdl, P);
  }
  *launches += 1;
}

template <int D>
static void launch_mx_body(const Dev& P, const LaunchCfg& L, cudaStream_t s, bool pdl, uint64_t* launches,
                           bool rec) {
  launch_grid_build<D>(P, s, launches, pdl);
  if (P.enable_torque) {
    launch_k(k_torque_center<D>, cdiv(P.G, 128), 128, 0, s, pdl, P);
    *launches += 1;
  }
  const dim3 grid(cdiv(P.n_chunks * 32, L.force_block)), block(L.force_block);
  launch_force_mx<D>(P, grid, block, s, pdl, rec);
  *launches += 1;
}

void launch_mixed_body(const Dev& P, const LaunchCfg& L, cudaStream_t s, bool pdl, uint64_t* launches, bool rec) {
  if (P.dim == 2) {
    launch_mx_body<2>(P, L, s, pdl, launches, rec);
  } else {
    launch_mx_body<3>(P, L, s, pdl, launches, rec);
  }
}

void launch_mixed_finalize(const Dev& P, cudaStream_t s, bool pdl, uint64_t* launches) {
  const uint32_t sm = P.wrec_smem ? FINAL_SMEM : 0;
  if (P.dim == 2) {
    launch_k(k_finalize<2>, finalize_blocks(P.I), FINAL_THREADS, sm, s, pdl, P);
  } else {
    launch_k(k_finalize<3>, finalize_blocks(P.I), FINAL_THREADS, sm, s, pdl, P);
  }
  *launches += 1;
}

}  // namespace pg
