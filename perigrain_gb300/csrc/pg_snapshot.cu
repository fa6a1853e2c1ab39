// Asynchronous snapshots of the engine state (pg_snapshot / pg_wait / pg_host_alloc of
// include/perigrain.h): what the output step of run_timeloop (timeloop.h:881-1006) writes into
// tc_%05u.h5 and wall_%05u.h5, gathered on the device behind the steps already issued and
// copied to the host on a second stream while later steps compute.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>

#include "pg_device.cuh"
#include "pg_handle.h"

using namespace pg;

static int fail(int code, const std::string& msg) { return pg_fail(code, msg); }

namespace {

enum { SNAP_FIELDS = 5 };

struct SnapArgs {
  const void* src[SNAP_FIELDS];  // node fields, stride S per node
  double* dst[SNAP_FIELDS];      // [N][D] doubles
  uint32_t is32;                 // bit f: src[f] holds floats (mixed-precision acc / force)
  int nf;
  int disp_slot;                 // slot of the displacement field (-1: none)
  const uint8_t* clamp_pending;  // nodes whose clamp is applied at the next step read 0 there
  const uint32_t* node_at;       // device node of each input node (null: input order)
  uint32_t N, D, S;
  // bonds: alive bytes in CSR order
  const uint32_t *alive, *chunk_word, *node_deg;
  const uint64_t* bond_offset;
  uint8_t* alive_out;
  // per-instance items
  const double* reaction;
  double* reaction_out;
  uint32_t n_reaction;
  const InstDev* inst;
  double* wall_out;
  uint32_t I, NS;
  const int32_t* status;
  const unsigned long long* too_close;
  int64_t* status_out;
  unsigned long long* too_close_out;
};

// One grid-stride pass over every requested item.
__global__ void k_snap_gather(SnapArgs a) {
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nth = (size_t)gridDim.x * blockDim.x;
  const size_t ND = (size_t)a.N * a.D;
  for (int f = 0; f < a.nf; ++f) {
    const bool f32 = (a.is32 >> f) & 1u;
    const bool is_disp = f == a.disp_slot;
    for (size_t e = tid; e < ND; e += nth) {
      // element e of the output is component c of input node e / D
      const uint32_t o = (uint32_t)(e / a.D), c = (uint32_t)(e - (size_t)o * a.D);
      const uint32_t i = a.node_at ? a.node_at[o] : o;
      const size_t si = (size_t)i * a.S + c;
      double v = f32 ? (double)static_cast<const float*>(a.src[f])[si] : static_cast<const double*>(a.src[f])[si];
      if (is_disp && a.clamp_pending[i]) v = 0.0;
      a.dst[f][e] = v;
    }
  }
  if (a.alive_out) {
    for (size_t on = tid; on < a.N; on += nth) {  // input node on, in CSR order
      const uint32_t i = a.node_at ? a.node_at[on] : (uint32_t)on;
      const uint32_t c = (uint32_t)(i >> 5), lane = (uint32_t)(i & 31);
      const uint32_t* w = a.alive + a.chunk_word[c];
      uint8_t* o = a.alive_out + a.bond_offset[on];
      const uint32_t deg = a.node_deg[i];
      for (uint32_t k = 0; k < deg; ++k) o[k] = (uint8_t)((w[k] >> lane) & 1u);
    }
  }
  for (size_t k = tid; k < a.n_reaction; k += nth) a.reaction_out[k] = a.reaction[k];
  for (size_t k = tid; k < (size_t)a.I * a.NS; k += nth) a.wall_out[k] = a.inst[k / a.NS].wall[k % a.NS];
  if (tid == 0) {
    *a.status_out = *a.status;
    *a.too_close_out = *a.too_close;
  }
}

bool page_locked(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

extern "C" {

int pg_wait(pg_handle* h) {
  if (!h) return fail(PG_EINVAL, "null handle");
  SnapState* s = h->snap.get();
  if (!s || !s->pending) return PG_OK;
  s->pending = false;
  CU(cudaEventSynchronize(s->copied));
  for (const auto& o : s->out) std::memcpy(o.dst, o.src, o.bytes);
  s->out.clear();
  const uint32_t NS = 2 * h->dim;
  const size_t n_re = (size_t)h->P.I * NS * h->dim, n_wall = (size_t)h->P.I * NS;
  const char* sm = s->small_host;
  if (s->d.reaction) std::memcpy(s->d.reaction, sm, n_re * 8);
  if (s->d.wall) std::memcpy(s->d.wall, sm + align_up(n_re * 8), n_wall * 8);
  const size_t o_st = align_up(n_re * 8) + align_up(n_wall * 8);
  int64_t st = 0;
  uint64_t tc = 0;
  std::memcpy(&st, sm + o_st, 8);
  std::memcpy(&tc, sm + o_st + 8, 8);
  if (s->d.too_close_events) *s->d.too_close_events = tc;
  if (s->d.last_step) *s->d.last_step = s->last_step;
  if (st == PG_ETIMEOUT) h->halted = true;
  return device_status_fail((int32_t)st);
}

int pg_snapshot(pg_handle* h, const pg_snapshot_desc* d) {
  if (!h || !d) return fail(PG_EINVAL, "null argument");
  if (!h->snap) {
    std::unique_ptr<SnapState> s(new SnapState());
    CU(cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking));
    CU(cudaEventCreateWithFlags(&s->staged, cudaEventDisableTiming));
    CU(cudaEventCreateWithFlags(&s->copied, cudaEventDisableTiming));
    h->snap = std::move(s);
  }
  SnapState& s = *h->snap;
  if (s.pending) {
    int rc = pg_wait(h);
    if (rc) return rc;
  }
  const uint32_t N = h->P.N, D = h->dim, NS = 2 * D;
  const size_t field_bytes = (size_t)N * D * 8;
  const uint64_t n_bonds = h->bond_offset.empty() ? 0 : h->bond_offset[N];
  const bool mixed = h->precision == PG_MIXED;

  // requested node fields, in slot order
  struct Req {
    double* dst;
    const void* src;
    bool f32;
  } req[SNAP_FIELDS];
  int nf = 0, disp_slot = -1;
  auto add = [&](double* dst, const void* src, bool f32) {
    if (dst) req[nf++] = {dst, src, f32};
  };
  add(d->currpos, h->P.cur, false);
  add(d->vel, h->vel_parity == 0 ? h->vel_a : h->vel_b, false);
  add(d->acc, mixed ? (const void*)h->P.acc_f : (const void*)h->P.acc, mixed);
  add(d->force, mixed ? (const void*)h->P.force_f : (const void*)h->P.force, mixed);
  if (d->disp) {
    disp_slot = nf;
    add(d->disp, h->P.disp, false);
  }
  const bool want_alive = d->bond_alive && n_bonds;

  // device staging: fields, then alive bytes; the per-instance items in their own small area
  const size_t need = align_up((size_t)nf * field_bytes) + (want_alive ? align_up(n_bonds) : 0);
  if (need > s.stage_bytes) {
    cudaFree(s.stage);  // no snapshot is in flight: its copies completed in pg_wait
    s.stage = nullptr;
    s.stage_bytes = 0;
    CU(cudaMalloc((void**)&s.stage, need));
    s.stage_bytes = need;
  }
  const size_t n_re = (size_t)h->P.I * NS * D, n_wall = (size_t)h->P.I * NS;
  const size_t small = align_up(n_re * 8) + align_up(n_wall * 8) + 16;
  if (!s.small_dev) {
    CU(cudaMalloc((void**)&s.small_dev, small));
    CU(cudaHostAlloc((void**)&s.small_host, small, cudaHostAllocDefault));
    s.small_bytes = small;
  }
  if (want_alive && !s.bond_offset) {
    CU(cudaMalloc((void**)&s.bond_offset, (size_t)(N + 1) * 8));
    CU(cudaMemcpy(s.bond_offset, h->bond_offset.data(), (size_t)(N + 1) * 8, cudaMemcpyHostToDevice));
  }

  SnapArgs a{};
  for (int f = 0; f < nf; ++f) {
    a.src[f] = req[f].src;
    a.dst[f] = reinterpret_cast<double*>(s.stage + (size_t)f * field_bytes);
    if (req[f].f32) a.is32 |= 1u << f;
  }
  a.nf = nf;
  a.disp_slot = disp_slot;
  a.clamp_pending = h->P.clamp_pending;
  a.node_at = h->P.node_at;
  a.N = N;
  a.D = D;
  a.S = h->S;
  uint8_t* alive_stage = want_alive ? reinterpret_cast<uint8_t*>(s.stage + align_up((size_t)nf * field_bytes)) : nullptr;
  if (want_alive) {
    a.alive = h->P.alive;
    a.chunk_word = h->P.chunk_word;
    a.node_deg = h->P.node_deg;
    a.bond_offset = s.bond_offset;
    a.alive_out = alive_stage;
  }
  a.reaction = h->P.reaction;
  a.reaction_out = reinterpret_cast<double*>(s.small_dev);
  a.n_reaction = (uint32_t)n_re;
  a.inst = h->P.inst;
  a.wall_out = reinterpret_cast<double*>(s.small_dev + align_up(n_re * 8));
  a.I = h->P.I;
  a.NS = NS;
  a.status = h->P.status;
  a.too_close = h->P.too_close;
  const size_t o_st = align_up(n_re * 8) + align_up(n_wall * 8);
  a.status_out = reinterpret_cast<int64_t*>(s.small_dev + o_st);
  a.too_close_out = reinterpret_cast<unsigned long long*>(s.small_dev + o_st + 8);

  int sms = 0;
  CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device));
  const size_t work = std::max<size_t>({(size_t)N * D, n_re, n_wall, 1});
  const unsigned grid = (unsigned)std::min<size_t>((work + 255) / 256, (size_t)sms * 8);
  k_snap_gather<<<grid, 256, 0, h->stream>>>(a);
  CU(cudaGetLastError());
  CU(cudaEventRecord(s.staged, h->stream));
  CU(cudaStreamWaitEvent(s.copy, s.staged, 0));

  // copies: straight into page-locked caller buffers, else into the bounce buffer
  size_t bounce_need = 0;
  for (int f = 0; f < nf; ++f)
    if (!page_locked(req[f].dst)) bounce_need += align_up(field_bytes);
  const bool alive_direct = want_alive && page_locked(d->bond_alive);
  if (want_alive && !alive_direct) bounce_need += align_up(n_bonds);
  if (bounce_need > s.bounce_bytes) {
    if (s.bounce) cudaFreeHost(s.bounce);
    s.bounce = nullptr;
    s.bounce_bytes = 0;
    CU(cudaHostAlloc((void**)&s.bounce, bounce_need, cudaHostAllocDefault));
    s.bounce_bytes = bounce_need;
  }
  s.out.clear();
  size_t bo = 0;
  auto copy_out = [&](void* dst, const char* src, size_t bytes, bool direct) -> cudaError_t {
    if (direct) return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s.copy);
    char* b = s.bounce + bo;
    bo += align_up(bytes);
    s.out.push_back({dst, b, bytes});
    return cudaMemcpyAsync(b, src, bytes, cudaMemcpyDeviceToHost, s.copy);
  };
  cudaError_t e = cudaSuccess;
  if (field_bytes)
    for (int f = 0; f < nf && e == cudaSuccess; ++f)
      e = copy_out(req[f].dst, reinterpret_cast<const char*>(a.dst[f]), field_bytes, page_locked(req[f].dst));
  if (want_alive && e == cudaSuccess)
    e = copy_out(d->bond_alive, reinterpret_cast<const char*>(alive_stage), n_bonds, alive_direct);
  if (e == cudaSuccess) e = cudaMemcpyAsync(s.small_host, s.small_dev, s.small_bytes, cudaMemcpyDeviceToHost, s.copy);
  if (e == cudaSuccess) e = cudaEventRecord(s.copied, s.copy);
  if (e != cudaSuccess) {
    // copies already issued into the caller's buffers finish before the error returns
    cudaStreamSynchronize(s.copy);
    s.out.clear();
    CU(e);
  }
  s.d = *d;
  s.last_step = h->next_t - 1;
  s.pending = true;
  return PG_OK;
}

int pg_host_alloc(size_t bytes, void** out) {
  if (!out) return fail(PG_EINVAL, "null argument");
  *out = nullptr;
  CU(cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault));
  return PG_OK;
}

int pg_host_free(void* p) {
  if (p) CU(cudaFreeHost(p));
  return PG_OK;
}

}  // extern "C"
