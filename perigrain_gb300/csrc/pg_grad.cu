// Host driver of the gradient path (C ABI pg_grad_*, pg_masks_*, pg_set/get_grain_params of
// include/perigrain.h): checkpoints of the time-step state, mask recording, the frozen FP64
// replay forward, and the backward pass -- per segment, from the last to the first: restore the
// segment's checkpoint, recompute its steps recording CurrPos, velocity, walls and masks into a
// one-segment tape, then run the reverse steps (pg_adjoint_rev.cu) over the tape. Full-length
// segments are replayed from two CUDA graphs (recompute, reverse) captured once.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <string>
#include <vector>

#include "pg_adjoint.h"
#include "pg_handle.h"
#include "pg_kernels.h"
#include "pg_kernels_mixed.h"

using namespace pg;

static int fail(int code, const std::string& msg) { return pg_fail(code, msg); }

static GradState* grad_state(pg_handle* h) {
  if (!h->grad) h->grad.reset(new GradState);
  return h->grad.get();
}

// The device state one step reads and writes (everything else is rebuilt inside a step).
static int ensure_regions(pg_handle* h) {
  GradState* G = grad_state(h);
  if (!G->regions.empty()) return PG_OK;
  const Dev& P = h->P;
  const size_t N = P.N, S = h->S, D = h->dim, I = P.I, NC = P.n_chunks;
  auto add = [&](void* p, size_t bytes) {
    if (!bytes) return;
    G->regions.push_back({p, bytes});
    G->ckpt_bytes += (bytes + 255) & ~(size_t)255;
  };
  add(P.disp, N * S * 8);
  add(h->vel_a, N * S * 8);
  add(h->vel_b, N * S * 8);
  add(P.acc, N * S * 8);
  add(P.alive, (size_t)h->chunk_word[NC] * 4);
  add(P.inst, I * sizeof(InstDev));
  add(P.step, 4);
  add(P.clamp_pending, N);
  add(P.reaction, I * 2 * D * D * 8);
  if (h->precision == PG_MIXED) {
    const size_t SF = (D == 2) ? 2 : 4;
    add(P.acc_f, N * SF * 4);
    add(P.bref, N * 4 * D * 4);
  }
  CU(cudaEventCreate(&G->e0));
  CU(cudaEventCreate(&G->e1));
  return PG_OK;
}

static int ensure_slots(pg_handle* h, uint32_t slots) {
  GradState* G = grad_state(h);
  if (slots <= G->ckpt_slots) return PG_OK;
  char* nb = nullptr;
  CU(G->mem.alloc(&nb, (size_t)slots * G->ckpt_bytes));
  if (G->ckpt) {
    CU(cudaMemcpyAsync(nb, G->ckpt, (size_t)G->ckpt_slots * G->ckpt_bytes, cudaMemcpyDeviceToDevice, h->stream));
    CU(cudaStreamSynchronize(h->stream));
    G->mem.free_one(G->ckpt);
  }
  G->ckpt = nb;
  G->ckpt_slots = slots;
  G->ckpt_parity.resize(slots, 0);
  G->ckpt_t.resize(slots, 0);
  return PG_OK;
}

static int save_state(pg_handle* h, uint32_t slot) {
  GradState* G = h->grad.get();
  char* base = G->ckpt + (size_t)slot * G->ckpt_bytes;
  for (const auto& r : G->regions) {
    CU(cudaMemcpyAsync(base, r.first, r.second, cudaMemcpyDeviceToDevice, h->stream));
    base += (r.second + 255) & ~(size_t)255;
  }
  G->ckpt_parity[slot] = h->vel_parity;
  G->ckpt_t[slot] = h->next_t;
  return PG_OK;
}

static int restore_state(pg_handle* h, uint32_t slot) {
  GradState* G = h->grad.get();
  const char* base = G->ckpt + (size_t)slot * G->ckpt_bytes;
  for (const auto& r : G->regions) {
    CU(cudaMemcpyAsync(r.first, base, r.second, cudaMemcpyDeviceToDevice, h->stream));
    base += (r.second + 255) & ~(size_t)255;
  }
  h->vel_parity = G->ckpt_parity[slot];
  h->next_t = G->ckpt_t[slot];
  // the restored state is not the one the candidate lists were built for (the results do not
  // depend on when the lists are rebuilt)
  static const uint32_t one = 1;
  for (int p = 0; p < 2; ++p)
    if (h->rebuild_pp[p]) CU(cudaMemcpyAsync(h->rebuild_pp[p], &one, 4, cudaMemcpyHostToDevice, h->stream));
  return PG_OK;
}

static int read_status(pg_handle* h, int32_t* st) {
  CU(cudaMemcpyAsync(st, h->P.status, 4, cudaMemcpyDeviceToHost, h->stream));
  CU(cudaStreamSynchronize(h->stream));
  return PG_OK;
}

// one engine step with mask recording into (off, cnt, wall) of this step and the shared entry list
// (and, when x is set, the step's tape: CurrPos, velocity, walls, step number)
static Dev rec_dev(pg_handle* h, int parity, uint32_t* off, uint8_t* cnt, uint32_t* wall, uint32_t* ent,
                   uint32_t* ent_n, uint64_t cap, double* x, double* v, double* w, uint32_t* tstep, float* df) {
  Dev P = h->P;
  set_vel(h, P, parity);
  P.rec_off = off;
  P.rec_cnt = cnt;
  P.rec_wall = wall;
  P.rec_ent = ent;
  P.rec_n = ent_n;
  P.rec_cap = (uint32_t)std::min<uint64_t>(cap, 0xffffffffull);
  P.rec_x = x;
  P.rec_v = v;
  P.rec_w = w;
  P.rec_t = tstep;
  P.rec_df = df;
  return P;
}

static void enqueue_rec_step(pg_handle* h, int parity, uint32_t* off, uint8_t* cnt, uint32_t* wall, uint32_t* ent,
                             uint32_t* ent_n, uint64_t cap, uint64_t* launches, double* x = nullptr,
                             double* v = nullptr, double* w = nullptr, uint32_t* tstep = nullptr,
                             float* df = nullptr) {
  const Dev P = rec_dev(h, parity, off, cnt, wall, ent, ent_n, cap, x, v, w, tstep, df);
  if (h->precision == PG_MIXED) {
    launch_step_mixed(P, h->L, h->stream, launches, nullptr, nullptr, true);
  } else {
    launch_step(P, h->L, h->stream, launches, true);
  }
}

// one FP64 step replaying masks number `idx` of m
static void enqueue_replay_step(pg_handle* h, int parity, const pg_masks* m, uint32_t idx, const uint32_t* end_alive,
                                const uint32_t* break_step, double* wall_out, uint64_t* launches) {
  Dev P = h->P;
  set_vel(h, P, parity);
  ReplayStep R;
  const size_t N = P.N;
  R.off = m->off + (size_t)idx * N;
  R.cnt = m->cnt + (size_t)idx * N;
  R.wall = m->wall + (size_t)idx * N;
  R.ent = m->ent;
  R.end_alive = end_alive;
  R.break_step = break_step;
  R.wall_out = wall_out;
  launch_replay_step(P, R, h->stream, launches);
}

static int check_grad_ok(pg_handle* h) {
  if (h->P.enable_torque) return fail(PG_EINVAL, "torque is not differentiated (enable_torque must be 0)");
  if (h->P.worm) return fail(PG_EINVAL, "the worm time loop is not differentiated");
  std::vector<GrainDev> g(h->P.G);
  CU(cudaMemcpy(g.data(), h->P.grain, g.size() * sizeof(GrainDev), cudaMemcpyDeviceToHost));
  for (uint32_t k = 0; k < h->P.G; ++k)
    if ((g[k].flags & GF_MOVABLE) && !(g[k].flags & GF_STOPPABLE))
      return fail(PG_EINVAL, "grain " + std::to_string(k) + " is movable but not stoppable");
  return PG_OK;
}

// ---------------------------------------------------------------------------------------------
// segment tape and the two segment sequences
// ---------------------------------------------------------------------------------------------
static int ensure_tape(pg_handle* h, uint32_t C, bool masks, uint64_t ent_cap) {
  GradState* G = h->grad.get();
  const size_t N = h->P.N, S = h->S, I = h->P.I, NS = 2 * h->dim;
  const bool need_masks = masks && (!G->off || G->ent_cap < ent_cap);
  if (G->tape_steps >= C && !need_masks) return PG_OK;
  if (G->tape_steps < C) {
    G->drop_graphs();
    G->tape.release();
    G->off = G->wall = G->ent = G->ent_n = nullptr;
    G->cnt = nullptr;
    G->DF = nullptr;
    G->ent_cap = 0;
    CU(G->tape.alloc(&G->X, (size_t)C * N * S));
    CU(G->tape.alloc(&G->V, (size_t)C * N * S));
    CU(G->tape.alloc(&G->W, (size_t)C * I * NS));
    CU(G->tape.alloc(&G->tstep, C));
    if (h->precision == PG_MIXED) CU(G->tape.alloc(&G->DF, (size_t)C * N * (h->dim == 2 ? 4 : 6)));
    G->tape_steps = C;
  }
  if (masks && !G->off) {
    CU(G->tape.alloc(&G->off, (size_t)G->tape_steps * N));
    CU(G->tape.alloc(&G->cnt, (size_t)G->tape_steps * N));
    CU(G->tape.alloc(&G->wall, (size_t)G->tape_steps * N));
    CU(G->tape.alloc(&G->ent_n, 1));
  }
  if (masks && G->ent_cap < ent_cap) {
    G->drop_graphs();
    if (G->ent) G->tape.free_one(G->ent);
    CU(G->tape.alloc(&G->ent, ent_cap));
    G->ent_cap = ent_cap;
  }
  return PG_OK;
}

// Recompute `len` steps from the restored state, filling tape slots 0..len-1. Product mode
// records masks into the tape; frozen mode replays masks `first_idx`.. of G->frozen.
static int enqueue_recompute(pg_handle* h, int parity, uint32_t len, uint32_t first_idx, uint64_t* launches) {
  GradState* G = h->grad.get();
  const size_t N = h->P.N, S = h->S, I = h->P.I, NS = 2 * h->dim;
  if (!G->frozen) CU(cudaMemsetAsync(G->ent_n, 0, 4, h->stream));
  for (uint32_t i = 0; i < len; ++i) {
    double* X = G->X + (size_t)i * N * S;
    double* V = G->V + (size_t)i * N * S;
    double* W = G->W + (size_t)i * I * NS;
    if (G->frozen) {
      CU(cudaMemcpyAsync(G->tstep + i, h->P.step, 4, cudaMemcpyDeviceToDevice, h->stream));
      CU(cudaMemcpy2DAsync(W, NS * 8, (const char*)h->P.inst + offsetof(InstDev, wall), sizeof(InstDev), NS * 8, I,
                           cudaMemcpyDeviceToDevice, h->stream));
      enqueue_replay_step(h, parity, G->frozen, first_idx + i, G->frozen->end_alive, G->frozen->break_step, nullptr,
                          launches);
      const double* vin = parity == 0 ? h->vel_a : h->vel_b;
      CU(cudaMemcpyAsync(X, h->P.cur, N * S * 8, cudaMemcpyDeviceToDevice, h->stream));
      CU(cudaMemcpyAsync(V, vin, N * S * 8, cudaMemcpyDeviceToDevice, h->stream));
    } else if (h->overlap) {
      // the recording steps with each finalize beside the next position update, as in the
      // forward graphs (bit-identical to the serial order)
      float* DF = G->DF ? G->DF + (size_t)i * N * (h->dim == 2 ? 4 : 6) : nullptr;
      const Dev P = rec_dev(h, parity, G->off + (size_t)i * N, G->cnt + (size_t)i * N, G->wall + (size_t)i * N,
                            G->ent, G->ent_n, G->ent_cap, X, V, W, G->tstep + i, DF);
      if (i == 0) launch_mixed_predict(P, h->stream, true, launches);
      if (i > 0) cudaStreamWaitEvent(h->stream, h->ev_join, 0);
      launch_mixed_body(P, h->L, h->stream, true, launches, true);
      if (i + 1 < len) {
        cudaEventRecord(h->ev_fork, h->stream);
        cudaStreamWaitEvent(h->side, h->ev_fork, 0);
        launch_mixed_finalize(P, h->side, false, launches);
        cudaEventRecord(h->ev_join, h->side);
        Dev Pn = h->P;
        set_vel(h, Pn, parity ^ 1);
        launch_mixed_predict(Pn, h->stream, true, launches);
      } else {
        launch_mixed_finalize(P, h->stream, true, launches);
      }
    } else {
      // the recording force kernel writes the tape itself
      float* DF = G->DF ? G->DF + (size_t)i * N * (h->dim == 2 ? 4 : 6) : nullptr;
      enqueue_rec_step(h, parity, G->off + (size_t)i * N, G->cnt + (size_t)i * N, G->wall + (size_t)i * N, G->ent,
                       G->ent_n, G->ent_cap, launches, X, V, W, G->tstep + i, DF);
    }
    parity ^= 1;
  }
  return PG_OK;
}

// Reverse steps over tape slots len-1..0; cotangents move cot[cur] -> cot[cur^1] each step.
static void enqueue_reverse(pg_handle* h, int cur, uint32_t len, uint32_t first_idx, bool with_rbar,
                            uint64_t* launches) {
  GradState* G = h->grad.get();
  const size_t N = h->P.N, S = h->S, I = h->P.I, NS = 2 * h->dim;
  for (uint32_t ii = len; ii-- > 0;) {
    AdjStep A;
    A.X = G->X + (size_t)ii * N * S;
    A.V = G->V + (size_t)ii * N * S;
    A.W = G->W + (size_t)ii * I * NS;
    A.tstep = G->tstep + ii;
    if (G->frozen) {
      const size_t idx = first_idx + ii;
      A.off = G->frozen->off + idx * N;
      A.cnt = G->frozen->cnt + idx * N;
      A.wall = G->frozen->wall + idx * N;
      A.ent = G->frozen->ent;
      A.end_alive = G->frozen->end_alive;
      A.break_step = G->frozen->break_step;
    } else {
      A.off = G->off + (size_t)ii * N;
      A.cnt = G->cnt + (size_t)ii * N;
      A.wall = G->wall + (size_t)ii * N;
      A.ent = G->ent;
      A.end_alive = G->end_alive;
      A.break_step = h->P.break_step;
    }
    A.db = G->cot[cur][0];
    A.vb = G->cot[cur][1];
    A.ab = G->cot[cur][2];
    A.db_o = G->cot[cur ^ 1][0];
    A.vb_o = G->cot[cur ^ 1][1];
    A.ab_o = G->cot[cur ^ 1][2];
    A.pacc = G->pacc;
    A.rbar = (with_rbar && ii == len - 1) ? G->rbar : nullptr;
    A.xbb = G->xbb;
    A.pcb = G->pcb;
    const bool f32 = h->precision == PG_MIXED && !G->frozen;
    A.df = f32 ? G->DF + (size_t)ii * N * (h->dim == 2 ? 4 : 6) : nullptr;
    A.fbf = f32 ? G->fbf : nullptr;
    launch_adjoint_step(h->P, A, h->stream, launches);
    cur ^= 1;
  }
}

static int capture(pg_handle* h, cudaGraphExec_t* out, int which, int arg, uint32_t len, uint64_t* launches) {
  cudaGraph_t g = nullptr;
  CU(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  int rc = PG_OK;
  if (which == 0) {
    rc = enqueue_recompute(h, arg, len, 0, launches);
  } else {
    enqueue_reverse(h, arg, len, 0, false, launches);
  }
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  CU(e);
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  CU(e);
  return PG_OK;
}

extern "C" {

int pg_set_grain_params(pg_handle* h, const double* cnot, const double* snot, const double* kn, const double* zeta,
                        const double* mu) {
  if (!h) return fail(PG_EINVAL, "null handle");
  CU(cudaStreamSynchronize(h->stream));
  std::vector<GrainDev> g(h->P.G);
  CU(cudaMemcpy(g.data(), h->P.grain, g.size() * sizeof(GrainDev), cudaMemcpyDeviceToHost));
  for (uint32_t k = 0; k < h->P.G; ++k) {
    if (cnot) g[k].cnot = cnot[k];
    if (snot) g[k].snot = snot[k];
    if (kn) g[k].kn = kn[k];
    if (zeta) g[k].zeta = zeta[k];
    if (mu) g[k].mu = mu[k];
    set_grain_f(g[k]);
  }
  CU(cudaMemcpy(h->P.grain, g.data(), g.size() * sizeof(GrainDev), cudaMemcpyHostToDevice));
  if ((kn || zeta || mu) && !h->P.grain_contact) {
    h->P.grain_contact = 1;
    if (h->grad) h->grad->drop_graphs();
    return build_graphs(h);
  }
  return PG_OK;
}

int pg_get_grain_params(pg_handle* h, double* cnot, double* snot, double* kn, double* zeta, double* mu) {
  if (!h) return fail(PG_EINVAL, "null handle");
  CU(cudaStreamSynchronize(h->stream));
  std::vector<GrainDev> g(h->P.G);
  CU(cudaMemcpy(g.data(), h->P.grain, g.size() * sizeof(GrainDev), cudaMemcpyDeviceToHost));
  for (uint32_t k = 0; k < h->P.G; ++k) {
    if (cnot) cnot[k] = g[k].cnot;
    if (snot) snot[k] = g[k].snot;
    if (kn) kn[k] = g[k].kn;
    if (zeta) zeta[k] = g[k].zeta;
    if (mu) mu[k] = g[k].mu;
  }
  return PG_OK;
}

int pg_grad_begin(pg_handle* h) {
  if (!h) return fail(PG_EINVAL, "null handle");
  int rc = check_grad_ok(h);
  if (rc) return rc;
  rc = ensure_regions(h);
  if (rc) return rc;
  rc = ensure_slots(h, 1);
  if (rc) return rc;
  rc = save_state(h, 0);
  if (rc) return rc;
  CU(cudaStreamSynchronize(h->stream));
  h->grad->have_origin = true;
  h->grad->ready = false;
  return PG_OK;
}

int pg_grad_reset(pg_handle* h) {
  if (!h) return fail(PG_EINVAL, "null handle");
  if (!h->grad || !h->grad->have_origin) return fail(PG_EINVAL, "no origin: call pg_grad_begin first");
  int rc = restore_state(h, 0);
  if (rc) return rc;
  CU(cudaStreamSynchronize(h->stream));
  return PG_OK;
}

void pg_masks_free(pg_masks* m) { delete m; }

int pg_masks_record(pg_handle* h, uint32_t n_steps, pg_masks** out) {
  if (!h || !out) return fail(PG_EINVAL, "null argument");
  *out = nullptr;
  if (!h->grad || !h->grad->have_origin) return fail(PG_EINVAL, "no origin: call pg_grad_begin first");
  if (n_steps == 0) return fail(PG_EINVAL, "n_steps must be positive");
  int rc = check_grad_ok(h);
  if (rc) return rc;
  GradState* G = h->grad.get();
  const size_t N = h->P.N, NC = h->P.n_chunks;
  std::unique_ptr<pg_masks> m(new pg_masks);
  m->device = h->device;
  m->T = n_steps;
  m->N = (uint32_t)N;
  m->t0 = G->ckpt_t[0];
  CU(m->mem.alloc(&m->off, (size_t)n_steps * N));
  CU(m->mem.alloc(&m->cnt, (size_t)n_steps * N));
  CU(m->mem.alloc(&m->wall, (size_t)n_steps * N));
  CU(m->mem.alloc(&m->end_alive, h->chunk_word[NC]));
  CU(m->mem.alloc(&m->break_step, h->chunk_slot[NC]));
  uint32_t* ent_n = nullptr;
  CU(m->mem.alloc(&ent_n, 1));
  uint64_t cap = std::max<uint64_t>(1u << 20, (uint64_t)n_steps * N / 8);
  cap = std::min<uint64_t>(cap, 0x7fffffffull);
  for (int attempt = 0; attempt < 4; ++attempt) {
    if (m->ent) m->mem.free_one(m->ent);
    CU(m->mem.alloc(&m->ent, cap));
    rc = restore_state(h, 0);
    if (rc) return rc;
    CU(cudaMemsetAsync(ent_n, 0, 4, h->stream));
    CU(cudaMemsetAsync(h->P.status, 0, 4, h->stream));
    uint64_t launches = 0;
    for (uint32_t i = 0; i < n_steps; ++i) {
      enqueue_rec_step(h, h->vel_parity, m->off + (size_t)i * N, m->cnt + (size_t)i * N, m->wall + (size_t)i * N,
                       m->ent, ent_n, cap, &launches);
      h->vel_parity ^= 1;
      h->next_t += 1;
    }
    CU(cudaGetLastError());
    int32_t st = 0;
    rc = read_status(h, &st);
    if (rc) return rc;
    uint32_t need = 0;
    CU(cudaMemcpy(&need, ent_n, 4, cudaMemcpyDeviceToHost));
    if (st == PG_ECAPACITY && need > cap) {
      if (need >= 0x7fffffffu) return fail(PG_ECAPACITY, "too many recorded contact entries for one mask set");
      cap = std::min<uint64_t>((uint64_t)need + need / 4 + 1024, 0x7fffffffull);
      continue;
    }
    if (st) return fail(st, std::string("device reported: ") + pg_status_string(st));
    m->n_ent = need;
    CU(cudaMemcpy(m->end_alive, h->P.alive, (size_t)h->chunk_word[NC] * 4, cudaMemcpyDeviceToDevice));
    CU(cudaMemcpy(m->break_step, h->P.break_step, (size_t)h->chunk_slot[NC] * 4, cudaMemcpyDeviceToDevice));
    G->ready = false;
    *out = m.release();
    return PG_OK;
  }
  return fail(PG_ECAPACITY, "contact entries kept growing while recording masks");
}

int pg_grad_forward(pg_handle* h, uint32_t n_steps, uint32_t checkpoint_every, const pg_masks* frozen) {
  if (!h) return fail(PG_EINVAL, "null handle");
  if (!h->grad || !h->grad->have_origin) return fail(PG_EINVAL, "no origin: call pg_grad_begin first");
  if (n_steps == 0 || checkpoint_every == 0) return fail(PG_EINVAL, "n_steps and checkpoint_every must be positive");
  GradState* G = h->grad.get();
  if (frozen) {
    if (frozen->N != h->P.N || frozen->device != h->device) return fail(PG_EINVAL, "masks belong to another setup");
    if (frozen->t0 != G->ckpt_t[0]) return fail(PG_EINVAL, "masks were recorded from another origin");
    if (n_steps > frozen->T) return fail(PG_EINVAL, "n_steps exceeds the recorded masks");
  }
  int rc = check_grad_ok(h);
  if (rc) return rc;
  const uint32_t C = std::min(checkpoint_every, n_steps);
  const uint32_t nseg = (n_steps + C - 1) / C;
  rc = ensure_slots(h, nseg + 1);
  if (rc) return rc;
  const size_t NC = h->P.n_chunks;
  if (!G->end_alive) CU(G->mem.alloc(&G->end_alive, h->chunk_word[NC]));
  if (frozen && !G->wall_out) CU(G->mem.alloc(&G->wall_out, (size_t)h->P.N * 2 * h->dim * 4));
  if (G->frozen != frozen || G->C != C) G->drop_graphs();
  G->ready = false;
  G->frozen = frozen;
  G->T = n_steps;
  G->C = C;
  G->nseg = nseg;
  G->final_slot = nseg;
  rc = restore_state(h, 0);
  if (rc) return rc;
  CU(cudaMemsetAsync(h->P.status, 0, 4, h->stream));
  uint64_t launches = 0;
  CU(cudaEventRecord(G->e0, h->stream));
  for (uint32_t k = 0; k < nseg; ++k) {
    if (k > 0) {
      rc = save_state(h, k);
      if (rc) return rc;
    }
    const uint32_t len = std::min(C, n_steps - k * C);
    if (frozen) {
      for (uint32_t i = 0; i < len; ++i) {
        const bool last = (k == nseg - 1) && (i == len - 1);
        enqueue_replay_step(h, h->vel_parity, frozen, k * C + i, frozen->end_alive, frozen->break_step,
                            last ? G->wall_out : nullptr, &launches);
        h->vel_parity ^= 1;
        h->next_t += 1;
      }
    } else {
      uint32_t i = 0;
      while (i < len) {
        if (len - i >= (uint32_t)pg_handle::GRAPH_STEPS) {
          CU(cudaGraphLaunch(h->graph[h->vel_parity], h->stream));
          launches += h->graph_launches_per;
          i += pg_handle::GRAPH_STEPS;
        } else {
          enqueue_step(h, h->vel_parity, &launches);
          h->vel_parity ^= 1;
          ++i;
        }
      }
      h->next_t += len;
    }
  }
  rc = save_state(h, nseg);
  if (rc) return rc;
  CU(cudaEventRecord(G->e1, h->stream));
  if (!frozen)
    CU(cudaMemcpyAsync(G->end_alive, h->P.alive, (size_t)h->chunk_word[NC] * 4, cudaMemcpyDeviceToDevice,
                       h->stream));
  CU(cudaGetLastError());
  CU(cudaEventSynchronize(G->e1));
  float ms = 0;
  CU(cudaEventElapsedTime(&ms, G->e0, G->e1));
  G->fwd_ms = ms;
  G->fwd_launches = launches;
  h->last_launches = launches;
  rc = check_device_status(h);
  if (rc) return rc;
  G->ready = true;
  return PG_OK;
}

int pg_grad_backward(pg_handle* h, const double* disp_bar, const double* vel_bar, const double* reaction_bar,
                     double* grad) {
  if (!h || !grad) return fail(PG_EINVAL, "null argument");
  if (!h->grad || !h->grad->ready) return fail(PG_EINVAL, "no differentiable forward to go back through");
  GradState* G = h->grad.get();
  const size_t N = h->P.N, S = h->S, D = h->dim, I = h->P.I, NS = 2 * D, NG = h->P.G;
  const uint32_t C = G->C, nseg = G->nseg, T = G->T;
  if (!G->pacc) {
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 3; ++b) CU(G->mem.alloc(&G->cot[a][b], N * S));
    CU(G->mem.alloc(&G->pacc, N * NPARAM));
    CU(G->mem.alloc(&G->gradd, NG * NPARAM));
    CU(G->mem.alloc(&G->rbar, I * NS * D));
    CU(G->mem.alloc(&G->xbb, N * S));
    CU(G->mem.alloc(&G->pcb, N));
    CU(G->mem.alloc(&G->fbf, N * ((D == 2) ? 2 : 4)));
  }
  uint64_t cap = G->ent_cap ? G->ent_cap : std::max<uint64_t>(1u << 20, (uint64_t)C * N / 2);
  std::vector<uint32_t> need(nseg, 0);
  uint32_t* need_pinned = nullptr;
  CU(cudaMallocHost((void**)&need_pinned, nseg * 4));
  std::unique_ptr<uint32_t, decltype(&cudaFreeHost)> need_guard(need_pinned, &cudaFreeHost);
  // seeds (stride S on the device)
  std::vector<double> tmp(N * S, 0.0);
  auto upload = [&](const double* src, double* dst) -> int {
    std::fill(tmp.begin(), tmp.end(), 0.0);
    if (src)
      for (size_t i = 0; i < N; ++i)
        for (size_t c = 0; c < D; ++c) tmp[i * S + c] = src[(size_t)h->orig((uint32_t)i) * D + c];
    CU(cudaMemcpyAsync(dst, tmp.data(), tmp.size() * 8, cudaMemcpyHostToDevice, h->stream));
    CU(cudaStreamSynchronize(h->stream));
    return PG_OK;
  };
  for (int attempt = 0; attempt < 4; ++attempt) {
    int rc = ensure_tape(h, C, G->frozen == nullptr, cap);
    if (rc) return rc;
    if ((rc = upload(disp_bar, G->cot[0][0])) || (rc = upload(vel_bar, G->cot[0][1])) ||
        (rc = upload(nullptr, G->cot[0][2])))
      return rc;
    if (reaction_bar) CU(cudaMemcpyAsync(G->rbar, reaction_bar, I * NS * D * 8, cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemsetAsync(G->pacc, 0, N * NPARAM * 8, h->stream));
    CU(cudaMemsetAsync(h->P.status, 0, 4, h->stream));
    uint64_t launches = 0;
    CU(cudaEventRecord(G->e0, h->stream));
    if (h->precision == PG_MIXED && !G->frozen) {
      AdjStep A{};
      A.ab = G->cot[0][2];
      A.vb = G->cot[0][1];
      A.fbf = G->fbf;
      launch_fb_init(h->P, A, h->stream, &launches);
    }
    int cur = 0;
    for (uint32_t k = nseg; k-- > 0;) {
      const uint32_t len = std::min(C, T - k * C);
      rc = restore_state(h, k);
      if (rc) return rc;
      const bool full = (len == C) && (k != nseg - 1 || !reaction_bar);
      const int par = h->vel_parity;
      if (full && !G->frozen) {
        if (!G->g_rec[par]) {
          uint64_t n = 0;
          rc = capture(h, &G->g_rec[par], 0, par, C, &n);
          if (rc) return rc;
          G->g_rec_launches = n;
        }
        CU(cudaGraphLaunch(G->g_rec[par], h->stream));
        launches += G->g_rec_launches;
      } else {
        rc = enqueue_recompute(h, par, len, k * C, &launches);
        if (rc) return rc;
      }
      if (!G->frozen) CU(cudaMemcpyAsync(need_pinned + k, G->ent_n, 4, cudaMemcpyDeviceToHost, h->stream));
      if (full) {
        if (!G->g_adj[cur] && !G->frozen) {
          uint64_t n = 0;
          rc = capture(h, &G->g_adj[cur], 1, cur, C, &n);
          if (rc) return rc;
          G->g_adj_launches = n;
        }
        if (!G->frozen) {
          CU(cudaGraphLaunch(G->g_adj[cur], h->stream));
          launches += G->g_adj_launches;
        } else {
          enqueue_reverse(h, cur, len, k * C, false, &launches);
        }
      } else {
        enqueue_reverse(h, cur, len, k * C, k == nseg - 1 && reaction_bar != nullptr, &launches);
      }
      if (len & 1) cur ^= 1;
    }
    launch_grad_reduce(h->P, G->pacc, G->gradd, h->stream, &launches);
    CU(cudaEventRecord(G->e1, h->stream));
    CU(cudaGetLastError());
    CU(cudaEventSynchronize(G->e1));
    int32_t st = 0;
    rc = read_status(h, &st);
    if (rc) return rc;
    uint32_t mx = 0;
    for (uint32_t k = 0; k < nseg; ++k) mx = std::max(mx, need_pinned[k]);
    if (st == PG_ECAPACITY && !G->frozen && mx > G->ent_cap) {
      if (mx >= 0x7fffffffu) return fail(PG_ECAPACITY, "too many recorded contact entries in one segment");
      cap = (uint64_t)mx + mx / 4 + 1024;
      continue;
    }
    if (st) return fail(st, std::string("device reported: ") + pg_status_string(st));
    float ms = 0;
    CU(cudaEventElapsedTime(&ms, G->e0, G->e1));
    G->bwd_ms = ms;
    G->bwd_launches = launches;
    h->last_launches = launches;
    CU(cudaMemcpy(grad, G->gradd, NG * NPARAM * 8, cudaMemcpyDeviceToHost));
    rc = restore_state(h, G->final_slot);
    if (rc) return rc;
    CU(cudaStreamSynchronize(h->stream));
    return PG_OK;
  }
  return fail(PG_ECAPACITY, "contact entries kept growing in the backward pass");
}

int pg_grad_times(pg_handle* h, double* forward_ms, double* backward_ms, uint64_t* forward_launches,
                  uint64_t* backward_launches) {
  if (!h) return fail(PG_EINVAL, "null handle");
  const GradState* G = h->grad.get();
  if (forward_ms) *forward_ms = G ? G->fwd_ms : 0.0;
  if (backward_ms) *backward_ms = G ? G->bwd_ms : 0.0;
  if (forward_launches) *forward_launches = G ? G->fwd_launches : 0;
  if (backward_launches) *backward_launches = G ? G->bwd_launches : 0;
  return PG_OK;
}

}  // extern "C"
