// kmc_host.h -- host-side internals of the GB300 kMC engine shared by its translation
// units (kmc_engine.cu: kernels, pool and trajectory API; kmc_state.cu: device-state
// images, .reload files and on-device sampling).  Not part of the C-ABI.
#pragma once
#include <cuda_runtime.h>

#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/kmc_gb300.h"
#include "kmc_device.cuh"

namespace kmc_host {
using namespace kmc;

extern thread_local std::string g_err;

// Records the error text (kmc_last_error) and returns the status code.
int fail(int code, const std::string &msg);

#define CK(call)                                                                           \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return fail(KMC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

struct ModelHost {
  std::vector<int32_t> prog;
  int32_t *d_prog = nullptr;
  ModelDev dev{};
};

struct SlotHost {
  bool used = false;
  size_t off = 0, bytes = 0;
  size_t samp_off = 0, samp_bytes = 0;  // on-device sampling record (samp_bytes 0: none)
  SlotDev dev{};
};

struct GraphKey {
  int64_t steps;
  std::vector<int32_t> slots;
  bool operator==(const GraphKey &o) const { return steps == o.steps && slots == o.slots; }
};
struct GraphKeyHash {
  size_t operator()(const GraphKey &k) const {
    size_t h = std::hash<int64_t>()(k.steps);
    for (int32_t s : k.slots) h = h * 1000003u ^ (size_t)s;
    return h;
  }
};
struct GraphEntry {
  int64_t nlaunch = 0;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  int32_t *d_list = nullptr;
  int64_t *d_steps = nullptr;
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Byte layout of one slot block.
struct Layout {
  size_t lat, as1, as2, rates, integ, accum, nsites, procstat, total;
};

// Stream-ordered device scratch, freed on its stream when it goes out of scope (on
// error returns too).
struct AsyncScratch {
  void *ptr = nullptr;
  cudaStream_t stream;
  explicit AsyncScratch(cudaStream_t s) : stream(s) {}
  AsyncScratch(const AsyncScratch &) = delete;
  AsyncScratch &operator=(const AsyncScratch &) = delete;
  cudaError_t alloc(size_t bytes) { return cudaMallocAsync(&ptr, bytes, stream); }
  template <class T> T *as() const { return static_cast<T *>(ptr); }
  ~AsyncScratch() {
    if (ptr) cudaFreeAsync(ptr, stream);
  }
};

inline Layout slot_layout(int P, int V) {
  Layout L;
  size_t o = 0;
  L.lat = o; o = align_up(o + (size_t)V, 16);
  L.as1 = o; o = align_up(o + (size_t)P * (V + 1) * 4, 16);
  L.as2 = o; o = align_up(o + (size_t)P * (V + 1) * 4, 16);
  L.rates = o; o += (size_t)P * 8;
  L.integ = o; o += (size_t)P * 8;
  L.accum = o; o += (size_t)P * 8;
  L.procstat = o; o += (size_t)P * 8;
  L.nsites = o; o = align_up(o + (size_t)P * 4, 16);
  L.total = o;
  return L;
}

}  // namespace kmc_host


struct kmc_pool {
  int device = 0;
  int num_sms = 1;
  cudaStream_t stream = nullptr;
  char *arena = nullptr;
  size_t arena_bytes = 0;
  std::map<size_t, size_t> free_blocks;  // offset -> size
  std::vector<kmc_host::SlotHost> slots;
  kmc::SlotDev *d_slots = nullptr;
  std::vector<kmc_host::ModelHost> models;
  kmc::ModelDev *d_models = nullptr;
  int max_models = 256;
  int32_t *d_list = nullptr;
  int64_t *d_steps = nullptr;
  int32_t *d_counter = nullptr;
  int32_t *d_cmd_out = nullptr;
  int32_t *h_cancel = nullptr;   // host-mapped
  int32_t *d_cancel = nullptr;
  // admission staging
  int32_t *d_adm_list = nullptr;
  kmc::SlotDev *d_adm_staged = nullptr;
  double *d_adm_rates = nullptr;
  int32_t *d_adm_roff = nullptr;
  size_t adm_rates_cap = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, tev0 = nullptr, tev1 = nullptr;
  bool timed = false;
  int64_t launches = 0;
  int warps_per_block = 4;
  int fast_path = 1;
  int stage_hot = 1;  // 1: a model's hot section goes to shared memory when it fits
  int blocks_per_sm = 0;  // 0 = occupancy maximum
  int traj_per_warp = 1;  // 2: two trajectories per warp, 16 lanes each (models of up to 64 processes)
  int tables_on_chip = 1; // 1: a launch's lattices and tables go to shared memory when they all fit
  int solo = 1;           // 1: launches of at most one trajectory per SM of models with up to 8
                          //    processes run the solo kernel (steps on one lane)
  std::unordered_map<kmc_host::GraphKey, kmc_host::GraphEntry, kmc_host::GraphKeyHash> graphs;
  std::mutex mu;
  unsigned long long *d_phase = nullptr;  // KMC_NPHASE cycle sums
  char *d_res = nullptr;   // results gather buffers
  char *h_res = nullptr;   // pinned
  // per-model launches of one run go to these streams (forked from and joined back to
  // `stream` with events) so one model's launch tail overlaps the others' work
  std::vector<cudaStream_t> aux;
  std::vector<cudaEvent_t> aux_ev;
  cudaEvent_t fork_ev = nullptr;
  size_t res_cap = 0;
};

struct kmc_handle {
  kmc_pool *pool = nullptr;
  int slot = -1;
  int model = -1;
  int P = 0, V = 0, spuck = 1, nspecies = 0;
  int32_t *d_trace = nullptr;
  int64_t trace_cap = 0;
  double walltime = 0.0;  // host seconds spent in kmc_do_steps (base.mpy's walltime)
};

namespace kmc_host {
int alloc_block(kmc_pool *p, size_t bytes, size_t *off);
void free_block(kmc_pool *p, size_t off, size_t bytes);
int read_slot(kmc_pool *p, int slot, SlotDev *out);
// Uploads the run list once and issues `rounds` runs of it on the pool stream, calling
// after(r) once round r is issued (it may enqueue more work; no host synchronisation).
int run_rounds(kmc_pool *p, const int32_t *slots, const int64_t *steps, int n, int rounds,
               const std::function<int(int)> &after);
int check_slot(kmc_pool *p, int slot);
// Checks a model program (header, op streams, fast streams, groups, tables) and fills m.
int validate_program(const int32_t *prog, int32_t len, ModelDev *m);
}  // namespace kmc_host
