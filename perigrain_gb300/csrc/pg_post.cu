// On-device post-processing of a snapshot (C ABI pg_postprocess of include/perigrain.h): the
// per-grain and per-instance quantities the reference's scripts compute by reading every
// tc_%05u.h5 / wall_%05u.h5 back into numpy --
//   damage per node (deg0 - deg) / deg0 and its grain mean   read_sim_output.py:126-133,
//                                                            gen_damage_data.py:55-66
//   grain means of vel, acc, CurrPos; grain sum of force     read_sim_output.py:201-232
//   sum of vol * rho * acc                                   read_sim_output.py:305-312
//   volume fraction = grain volume / wall box volume        read_sim_output.py:183-196
// -- from the state already in HBM, so a run's time series needs no snapshot download. One block
// per grain reduces its nodes in a fixed order (deterministic); only the per-grain sums leave the
// device.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "pg_common.cuh"
#include "pg_device.cuh"
#include "pg_handle.h"

using namespace pg;

namespace {

constexpr int POST_THREADS = 256;

// per grain: sum vel[D], sum acc[D], sum CurrPos[D], sum force[D], sum vol*rho*acc[D],
// sum damage, sum vol, node count
template <int D>
__host__ __device__ constexpr int post_nq() {
  return 5 * D + 3;
}

template <int D>
__global__ void __launch_bounds__(POST_THREADS) k_post(const Dev P, const double* vel, double* gsum,
                                                       double* node_damage) {
  constexpr int NQ = post_nq<D>();
  __shared__ double red[NQ][POST_THREADS];
  const uint32_t g = blockIdx.x, tid = threadIdx.x;
  const GrainDev& gr = P.grain[g];
  const bool mixed = P.acc_f != nullptr;
  double s[NQ];
  for (int k = 0; k < NQ; ++k) s[k] = 0.0;
  for (uint32_t o = gr.node_begin + tid; o < gr.node_end; o += POST_THREADS) {  // the input's order
    const uint32_t i = at_of(P, o);
    double v[D], x[D], a[D], f[D];
    ldv<D>(vel, i, v);
    ldv<D>(P.cur, i, x);
    if (mixed) {
      const uint32_t SF = (D == 2) ? 2 : 4;
      for (int c = 0; c < D; ++c) {
        a[c] = (double)P.acc_f[(size_t)i * SF + c];
        f[c] = (double)P.force_f[(size_t)i * SF + c];
      }
    } else {
      ldv<D>(P.acc, i, a);
      ldv<D>(P.force, i, f);
    }
    const double vol = P.vol[i];
    for (int c = 0; c < D; ++c) {
      s[c] += v[c];
      s[D + c] += a[c];
      s[2 * D + c] += x[c];
      s[3 * D + c] += f[c];
      s[4 * D + c] += (vol * gr.rho) * a[c];
    }
    // intact bonds now against bonds at creation (each bond sits in both endpoints' rows)
    const uint32_t c = i >> 5, lane = i & 31, deg0 = P.node_deg[i];
    uint32_t deg = 0;
    for (uint32_t k = 0; k < deg0; ++k) deg += (P.alive[P.chunk_word[c] + k] >> lane) & 1u;
    const double q = ((double)deg0 - (double)deg) / (double)deg0;  // 0/0 -> NaN, as numpy
    if (node_damage) node_damage[o] = q;
    s[5 * D] += q;
    s[5 * D + 1] += vol;
    s[5 * D + 2] += 1.0;
  }
  for (int k = 0; k < NQ; ++k) red[k][tid] = s[k];
  __syncthreads();
  for (uint32_t w = POST_THREADS / 2; w > 0; w >>= 1) {
    if (tid < w)
      for (int k = 0; k < NQ; ++k) red[k][tid] += red[k][tid + w];
    __syncthreads();
  }
  if (tid < (uint32_t)NQ) gsum[(size_t)g * NQ + tid] = red[tid][0];
}

}  // namespace

extern "C" int pg_postprocess(pg_handle* h, const pg_post* out) {
  if (!h || !out) return pg_fail(PG_EINVAL, "null argument");
  int rc = pg_synchronize(h);
  if (rc) return rc;
  const Dev& P = h->P;
  const uint32_t D = h->dim, G = P.G, I = P.I, N = P.N, NS = 2 * D;
  const int NQ = (D == 2) ? post_nq<2>() : post_nq<3>();
  if (!h->post_sum) CU(h->dalloc(&h->post_sum, (size_t)G * NQ));
  double* dmg = nullptr;
  if (out->node_damage) {
    if (!h->post_damage) CU(h->dalloc(&h->post_damage, N));
    dmg = h->post_damage;
  }
  const double* vel = h->vel_parity == 0 ? h->vel_a : h->vel_b;
  if (G) {
    if (D == 2) {
      k_post<2><<<G, POST_THREADS, 0, h->stream>>>(P, vel, h->post_sum, dmg);
    } else {
      k_post<3><<<G, POST_THREADS, 0, h->stream>>>(P, vel, h->post_sum, dmg);
    }
  }
  CU(cudaGetLastError());
  std::vector<double> gs((size_t)G * NQ);
  if (G) CU(cudaMemcpyAsync(gs.data(), h->post_sum, gs.size() * 8, cudaMemcpyDeviceToHost, h->stream));
  if (dmg) CU(cudaMemcpyAsync(out->node_damage, dmg, (size_t)N * 8, cudaMemcpyDeviceToHost, h->stream));
  CU(cudaStreamSynchronize(h->stream));
  std::vector<double> inert((size_t)I * D, 0.0), vol((size_t)I, 0.0);
  for (uint32_t g = 0; g < G; ++g) {
    const double* q = &gs[(size_t)g * NQ];
    const double n = q[5 * D + 2];
    for (uint32_t c = 0; c < D; ++c) {
      if (out->grain_mean_vel) out->grain_mean_vel[(size_t)g * D + c] = q[c] / n;
      if (out->grain_mean_acc) out->grain_mean_acc[(size_t)g * D + c] = q[D + c] / n;
      if (out->grain_mean_currpos) out->grain_mean_currpos[(size_t)g * D + c] = q[2 * D + c] / n;
      if (out->grain_force) out->grain_force[(size_t)g * D + c] = q[3 * D + c];
    }
    if (out->grain_damage) out->grain_damage[g] = q[5 * D] / n;
  }
  // per instance, grains in order
  std::vector<uint32_t> ginst(G);
  {
    std::vector<GrainDev> gd(G);
    if (G) CU(cudaMemcpy(gd.data(), P.grain, G * sizeof(GrainDev), cudaMemcpyDeviceToHost));
    for (uint32_t g = 0; g < G; ++g) ginst[g] = gd[g].inst;
  }
  for (uint32_t g = 0; g < G; ++g) {
    const double* q = &gs[(size_t)g * NQ];
    for (uint32_t c = 0; c < D; ++c) inert[(size_t)ginst[g] * D + c] += q[4 * D + c];
    vol[ginst[g]] += q[5 * D + 1];
  }
  if (out->inertial_force)
    for (size_t k = 0; k < inert.size(); ++k) out->inertial_force[k] = inert[k];
  if (out->volume_fraction) {
    std::vector<double> wall((size_t)I * NS);
    rc = pg_get_wall(h, wall.data());
    if (rc) return rc;
    for (uint32_t k = 0; k < I; ++k) {
      const double* wi = &wall[(size_t)k * NS];
      // the wall box volume of extract_bulk (read_sim_output.py:183-196), its index pairing kept
      const double wv = (D == 2) ? (wi[1] - wi[0]) * (wi[2] - wi[3])
                                 : (wi[1] - wi[0]) * (wi[3] - wi[2]) * (wi[5] - wi[4]);
      out->volume_fraction[k] = vol[k] / wv;
    }
  }
  return PG_OK;
}
