// The engine handle (pg_handle of include/perigrain.h) and the host helpers shared by the
// engine (pg_engine.cu) and the gradient driver (pg_grad.cu).
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "pg_device.cuh"
#include "pg_kernels.h"

// Sets the thread's last error message and returns code.
int pg_fail(int code, const std::string& msg);

#define CU(call)                                                                       \
  do {                                                                                 \
    cudaError_t _e = (call);                                                           \
    if (_e != cudaSuccess)                                                             \
      return pg_fail(_e == cudaErrorMemoryAllocation ? PG_ENOMEM : PG_ECUDA,           \
                     std::string(#call) + ": " + cudaGetErrorString(_e));              \
  } while (0)

// Device memory owned by one object, freed with it.
struct DevPool {
  std::vector<void*> ptrs;
  ~DevPool() { release(); }
  void release() {
    for (void* p : ptrs) cudaFree(p);
    ptrs.clear();
  }
  template <class T>
  cudaError_t alloc(T** p, size_t count) {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e == cudaSuccess) ptrs.push_back((void*)*p);
    return e;
  }
  void free_one(void* p) {
    for (size_t i = 0; i < ptrs.size(); ++i)
      if (ptrs[i] == p) {
        cudaFree(p);
        ptrs.erase(ptrs.begin() + (long)i);
        return;
      }
  }
};

// Masks of a recorded run (pg_masks of include/perigrain.h): for steps t0+1 .. t0+T, per node
// the contact-entry offset and count and the wall bits (layout of Dev::rec_*), the entries, and
// the bond masks at the end of the run.
struct pg_masks {
  int device = 0;
  uint32_t T = 0, N = 0;
  uint64_t t0 = 0;
  uint32_t *off = nullptr, *wall = nullptr, *ent = nullptr, *end_alive = nullptr, *break_step = nullptr;
  uint8_t* cnt = nullptr;
  uint64_t n_ent = 0;
  DevPool mem;
};

// State of the differentiable run of a handle (pg_grad_* of include/perigrain.h).
struct GradState {
  // device state a checkpoint holds (the time-step state of the engine), and checkpoint storage
  std::vector<std::pair<void*, size_t>> regions;
  size_t ckpt_bytes = 0;
  char* ckpt = nullptr;  // slot 0 = origin, slot k = state after k*C steps, slot `final_slot` = end
  uint32_t ckpt_slots = 0;
  std::vector<int> ckpt_parity;
  std::vector<uint64_t> ckpt_t;
  bool have_origin = false;
  // last forward
  bool ready = false;
  uint32_t T = 0, C = 0, nseg = 0, final_slot = 0;
  const pg_masks* frozen = nullptr;
  uint32_t* end_alive = nullptr;
  // segment tape (C steps)
  uint32_t tape_steps = 0;
  double *X = nullptr, *V = nullptr, *W = nullptr;
  float* DF = nullptr;  // mixed precision: displacement hi/lo pairs per step
  uint32_t* tstep = nullptr;
  uint32_t *off = nullptr, *wall = nullptr, *ent = nullptr, *ent_n = nullptr;
  uint8_t* cnt = nullptr;
  uint64_t ent_cap = 0;
  // cotangents and parameter accumulators
  double* cot[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
  double *pacc = nullptr, *gradd = nullptr, *rbar = nullptr, *wall_out = nullptr;
  double *xbb = nullptr, *pcb = nullptr;
  float* fbf = nullptr;
  // graphs of one full segment: recording (per velocity parity) and reverse (per cotangent slot)
  cudaGraphExec_t g_rec[2] = {nullptr, nullptr};
  cudaGraphExec_t g_adj[2] = {nullptr, nullptr};
  uint64_t g_rec_launches = 0, g_adj_launches = 0;
  // timing and counts of the last forward / backward
  double fwd_ms = 0, bwd_ms = 0;
  uint64_t fwd_launches = 0, bwd_launches = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  DevPool mem, tape;

  void drop_graphs() {
    for (int i = 0; i < 2; ++i) {
      if (g_rec[i]) cudaGraphExecDestroy(g_rec[i]);
      if (g_adj[i]) cudaGraphExecDestroy(g_adj[i]);
      g_rec[i] = g_adj[i] = nullptr;
    }
  }
  ~GradState() {
    drop_graphs();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  }
};

// An asynchronous snapshot (pg_snapshot / pg_wait): device staging written on the handle's
// stream, copied to the host on `copy`.
struct SnapState {
  cudaStream_t copy = nullptr;
  cudaEvent_t staged = nullptr, copied = nullptr;
  char* stage = nullptr;  // device: requested fields, then alive bytes
  size_t stage_bytes = 0;
  char* small_dev = nullptr;   // device: reaction, wall, status, too_close
  char* small_host = nullptr;  // page-locked host copy of small_dev
  size_t small_bytes = 0;
  char* bounce = nullptr;  // page-locked host copy for caller buffers that are not page-locked
  size_t bounce_bytes = 0;
  uint64_t* bond_offset = nullptr;  // device copy of the CSR offsets (alive bytes in CSR order)
  bool pending = false;
  pg_snapshot_desc d{};
  uint64_t last_step = 0;
  struct CopyOut {
    void* dst;
    const char* src;
    size_t bytes;
  };
  std::vector<CopyOut> out;  // bounce -> caller, done by pg_wait

  ~SnapState() {
    if (copy) cudaStreamSynchronize(copy);
    if (staged) cudaEventDestroy(staged);
    if (copied) cudaEventDestroy(copied);
    if (copy) cudaStreamDestroy(copy);
    cudaFree(stage);
    cudaFree(small_dev);
    cudaFree(bond_offset);
    if (small_host) cudaFreeHost(small_host);
    if (bounce) cudaFreeHost(bounce);
  }
};

struct pg_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  pg::Dev P{};  // device pointers + config; vel_in/vel_out are set per launch
  pg::LaunchCfg L;
  uint32_t dim = 2, S = 2;
  int precision = PG_FP64;
  double contact_skin = 0.0;  // candidate-list skin in use (fraction of R_c; 0 = grid search)
  uint64_t next_t = 1;
  int vel_parity = 0;  // 0: current velocity in vel_a
  double* vel_a = nullptr;
  double* vel_b = nullptr;
  // per step parity (the parity of vel_in): grain boxes and the list-rebuild flag of the step's
  // positions, so the next step's position update can run beside this step's finalize
  unsigned long long* bbox_pp[2] = {nullptr, nullptr};
  uint32_t* rebuild_pp[2] = {nullptr, nullptr};
  // the finalize of one step beside the next step's position update (graphs of the mixed path)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  bool overlap = false;
  bool xpos_separate = false;
  // set when a status check saw PG_ETIMEOUT (a bounded device wait ran out): pg_step refuses
  bool halted = false;
  // node layout: node_orig[d] = the input's index of device node d (empty: input order)
  std::vector<uint32_t> node_orig;
  int32_t node_order = 0;  // pg_node_order asked for
  uint32_t orig(uint32_t d) const { return node_orig.empty() ? d : node_orig[d]; }
  std::vector<void*> allocs;
  // host copies needed for mapping
  std::vector<uint64_t> bond_offset;  // reference CSR
  std::vector<uint32_t> grain_node_offset;
  std::vector<uint32_t> node_deg;
  std::vector<uint32_t> chunk_slot, chunk_word;
  std::vector<pg::InstDev> inst_host;
  // graphs: one per velocity parity, each GRAPH_STEPS steps
  static const int GRAPH_STEPS = 8;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  uint64_t graph_launches_per = 0;
  uint64_t last_launches = 0;
  // timing
  bool timing = false;
  std::vector<cudaEvent_t> ev;
  double force_ms = 0, total_ms = 0;
  uint64_t force_launches = 0;
  cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr;
  // gradient path
  std::unique_ptr<GradState> grad;
  // post-processing scratch (pg_postprocess)
  double* post_sum = nullptr;
  double* post_damage = nullptr;
  double* field_scratch = nullptr;  // [N][D] doubles: FP32 fields widened for pg_get_field
  std::unique_ptr<SnapState> snap;

  ~pg_handle() {
    if (stream) cudaStreamSynchronize(stream);
    snap.reset();
    grad.reset();
    for (int i = 0; i < 2; ++i)
      if (graph[i]) cudaGraphExecDestroy(graph[i]);
    for (auto e : ev) cudaEventDestroy(e);
    if (ev_t0) cudaEventDestroy(ev_t0);
    if (ev_t1) cudaEventDestroy(ev_t1);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (side) cudaStreamDestroy(side);
    for (void* p : allocs) cudaFree(p);
    if (xpos_separate) cudaFree(P.xpos);
    if (stream) cudaStreamDestroy(stream);
  }

  template <class T>
  cudaError_t dalloc(T** p, size_t count) {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e == cudaSuccess) allocs.push_back((void*)*p);
    return e;
  }
};

void set_vel(pg_handle* h, pg::Dev& P, int parity);
// Enqueue one engine step with the current velocity parity `parity` (does not flip it).
void enqueue_step(pg_handle* h, int parity, uint64_t* launches);
int build_graphs(pg_handle* h);
int check_device_status(pg_handle* h);
// PG_OK for st == 0, else records the device status message and returns st.
int device_status_fail(int32_t st);
// Force a rebuild of the contact candidate lists at the next step (no-op without lists).
int request_list_rebuild(pg_handle* h);
