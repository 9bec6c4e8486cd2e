// kmc_state.cu -- device-state images, kmos .reload files and on-device sampling for
// the GB300 kMC engine (C-ABI in include/kmc_gb300.h).
//
// State images.  kmos saves a trajectory with base.save_system and restores it with
// base.reload_system (base.mpy:363-578): an ASCII file with the clock, the counters,
// the lattice and both columns of avail_sites in full (2 * nr_of_proc * volume numbers).
// Here a trajectory is saved as a compact binary image instead: the scalars (clock,
// step, random stream, status), the P-vectors, the lattice, and for every process only
// the first nr_of_sites(p) entries of avail_sites(p, :, 1) -- the rest of that column
// is zero and avail_sites(p, :, 2) is its inverse, both rebuilt on the device when the
// image is loaded.  The image keeps integ_rates, kmc_time_step and the random stream,
// which the reference's file drops, so a restored trajectory continues bit for bit.
// Serving uses it to move trajectories between HBM and host memory.
//
// .reload files.  kmc_save_reload / kmc_load_reload write and read the reference's
// layout (save_system's edit descriptors, base.mpy:528-575), plus comment lines starting
// "#gb300" with what the reference's file cannot hold exactly (system size, kmc_time,
// rates and integ_rates to the last bit, kmc_time_step, the random stream).  The
// reference's reader skips comment lines, so either program reads either file.
//
// On-device sampling.  kmos.run.KMC_Model.get_std_sampled_data (run/__init__.py:
// 865-966) runs `samples` batches of kMC steps and after each one reads procstat,
// integ_rates, the clock and the occupation through the f2py getters.  Here the
// per-sample occupation (get_occupation, proclist_generic_subroutines.mpy:113-158),
// weighted by kmc_time_step as the reference weights it, is reduced on the device into
// a per-trajectory record in the arena; only the means and the counter differences come
// back to the host, once, at the end.
#include <cuda_runtime.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/kmc_gb300.h"
#include "kmc_device.cuh"
#include "kmc_host.h"
#include "kmc_reload.h"

using namespace kmc;
using namespace kmc_host;

namespace {

// ------------------------------------------------------------------ device kernels
// Copies avail_sites(p, 1..n_p, 1) of every process into one packed list.
__global__ void kmc_pack_tables_kernel(const int32_t *as1, int32_t stride, const int64_t *off, int32_t P,
                                       int32_t *out) {
  const int p = blockIdx.x;
  if (p >= P) return;
  const int64_t b = off[p];
  const int n = (int)(off[p + 1] - b);
  const int32_t *row = as1 + (size_t)p * stride;
  for (int k = threadIdx.x; k < n && k + 1 < stride; k += blockDim.x) out[b + k] = row[k + 1];
}

// Rebuilds both columns of avail_sites from the packed lists (the tables were zeroed).
__global__ void kmc_unpack_tables_kernel(int32_t *as1, int32_t *as2, int32_t stride, const int64_t *off, int32_t P,
                                         const int32_t *in) {
  const int p = blockIdx.x;
  if (p >= P) return;
  const int64_t b = off[p];
  const int n = (int)(off[p + 1] - b);
  int32_t *r1 = as1 + (size_t)p * stride;
  int32_t *r2 = as2 + (size_t)p * stride;
  for (int k = threadIdx.x; k < n && k + 1 < stride; k += blockDim.x) {
    const int s = in[b + k];
    if (s >= 1 && s < stride) {
      r1[k + 1] = s;
      r2[s] = k + 1;
    }
  }
}

// Sampling record of one trajectory, in 8-byte words:
//   [0] kmc_time at the start   [1] kmc_step at the start (int64)
//   [2] sum of the weights      [3] number of samples (int64)
//   [8, 8+P) procstat at the start (int64)   [8+P, 8+2P) integ_rates at the start
//   [8+2P, 8+2P+nocc) sum over samples of occupation * weight
constexpr int SAMP_HEAD = 8;
size_t samp_words(int P, int nocc) { return SAMP_HEAD + 2 * (size_t)P + nocc; }

struct SampleOut {
  int32_t occ_stride, proc_stride;
  double *occ;      // [n][occ_stride] occupation means
  int64_t *dps;     // [n][proc_stride] procstat differences
  double *dig;      // [n][proc_stride] integ_rates differences
  double *times;    // [n][2] total_time, simulated_time
  int64_t *steps;   // [n] kMC steps taken while sampling
  int32_t *status;  // [n]
};

enum SampleMode { SAMPLE_BEGIN = 0, SAMPLE_TAKE = 1, SAMPLE_END = 2 };

constexpr int OCC_BINS = 32 * 32;  // nspecies <= 30, spuck <= 32

// One block per listed trajectory.
//   BEGIN: snapshot the clock and counters, clear the sums.
//   TAKE:  occupation counts over the lattice (species != null species, per site index
//          within the unit cell), normalised by the number of cells, times the weight
//          kmc_time_step, added to the sums (np.average(occs, weights=step_ts)).
//   END:   means and differences to the output rows.
__global__ void __launch_bounds__(256) kmc_sample_kernel(const SlotDev *slots, const ModelDev *models,
                                                         const int32_t *list, double *const *recs, int32_t n,
                                                         int32_t mode, SampleOut out) {
  __shared__ unsigned int hist[OCC_BINS];
  const int item = blockIdx.x;
  if (item >= n) return;
  const SlotDev &S = slots[list[item]];
  const ModelDev M = models[S.model];
  const int P = S.P, ns = M.nspecies, sp = M.spuck, nocc = ns * sp;
  double *rec = recs[item];
  int64_t *irec = reinterpret_cast<int64_t *>(rec);
  int64_t *ps0 = irec + SAMP_HEAD;
  double *ig0 = rec + SAMP_HEAD + P;
  double *acc = rec + SAMP_HEAD + 2 * P;
  const int tid = threadIdx.x;

  if (mode == SAMPLE_BEGIN) {
    for (int i = tid; i < P; i += blockDim.x) {
      ps0[i] = S.procstat[i];
      ig0[i] = S.integ[i];
    }
    for (int i = tid; i < nocc; i += blockDim.x) acc[i] = 0.0;
    if (tid == 0) {
      rec[0] = S.kmc_time;
      irec[1] = S.kmc_step;
      rec[2] = 0.0;
      irec[3] = 0;
    }
    return;
  }
  if (mode == SAMPLE_END) {
    const double wsum = rec[2];
    for (int i = tid; i < out.proc_stride; i += blockDim.x) {
      const bool in = i < P;
      out.dps[(size_t)item * out.proc_stride + i] = in ? S.procstat[i] - ps0[i] : 0;
      out.dig[(size_t)item * out.proc_stride + i] = in ? __dadd_rn(S.integ[i], -ig0[i]) : 0.0;
    }
    for (int i = tid; i < out.occ_stride; i += blockDim.x)
      out.occ[(size_t)item * out.occ_stride + i] = i < nocc ? acc[i] / wsum : 0.0;
    if (tid == 0) {
      out.times[2 * item] = __dadd_rn(S.kmc_time, -rec[0]);
      out.times[2 * item + 1] = S.kmc_time;
      out.steps[item] = S.kmc_step - irec[1];
      out.status[item] = S.status;
    }
    return;
  }

  // SAMPLE_TAKE
  for (int i = tid; i < OCC_BINS; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  const int V = S.V;
  const int nvec = V / 16;  // the lattice starts the slot block: 256-byte aligned
  const uint4 *lv = reinterpret_cast<const uint4 *>(S.lat);
  for (int i = tid; i < nvec + (V - 16 * nvec); i += blockDim.x) {
    // run-length merge of equal bins within this thread's sites before the atomics
    int key = -1;
    unsigned int cnt = 0;
    auto count = [&](int spc, int type) {
      if (spc < 0 || spc >= ns) return;
      const int k = spc * sp + type;
      if (k == key) { cnt++; return; }
      if (cnt) atomicAdd(&hist[key], cnt);
      key = k;
      cnt = 1;
    };
    if (i < nvec) {
      const uint4 w = lv[i];
      const uint32_t words[4] = {w.x, w.y, w.z, w.w};
      int type = (16 * i) % sp;
#pragma unroll
      for (int j = 0; j < 16; j++) {
        count((int)(int8_t)(words[j >> 2] >> (8 * (j & 3))), type);
        type = (type + 1 == sp) ? 0 : type + 1;
      }
    } else {
      const int s = 16 * nvec + (i - nvec);
      count((int)S.lat[s], s % sp);
    }
    if (cnt) atomicAdd(&hist[key], cnt);
  }
  __syncthreads();
  const double cells = (double)S.X * (double)S.Y * (double)S.Z;
  const double w = S.kmc_time_step;
  for (int i = tid; i < nocc; i += blockDim.x)
    acc[i] = __dadd_rn(acc[i], __dmul_rn((double)hist[i] / cells, w));
  if (tid == 0) {
    rec[2] = __dadd_rn(rec[2], w);
    irec[3] += 1;
  }
}

// ------------------------------------------------------------------ image helpers
constexpr uint32_t IMAGE_MAGIC = 0x53434D4Bu;  // "KMCS"
constexpr uint32_t IMAGE_VERSION = 1;

struct ImageHeader {
  uint32_t magic, version;
  uint64_t program_hash;
  int32_t P, nspecies, spuck, backend;
  int32_t X, Y, Z, V;
  int32_t layer, status, rng_kind, accum_from;
  uint32_t seed, traj;
  double kmc_time, kmc_time_step;
  int64_t kmc_step;
  uint64_t rng[4];
  int64_t nentries;
  uint64_t bytes;
};

// Section offsets of an image: header, vectors (rates, integ, accum, procstat,
// nr_of_sites -- the slot block's own order), lattice, packed avail_sites entries.
struct ImageLayout {
  size_t vec, lat, ent, total;
};

ImageLayout image_layout(int P, int V, int64_t nentries) {
  ImageLayout L;
  L.vec = align_up(sizeof(ImageHeader), 16);
  L.lat = align_up(L.vec + (size_t)P * 36, 16);
  L.ent = align_up(L.lat + (size_t)V, 16);
  L.total = L.ent + (size_t)nentries * 4;
  return L;
}

uint64_t program_hash(const std::vector<int32_t> &prog) {  // FNV-1a over the words
  uint64_t h = 1469598103934665603ULL;
  for (int32_t w : prog)
    for (int b = 0; b < 4; b++) {
      h ^= ((uint32_t)w >> (8 * b)) & 0xffu;
      h *= 1099511628211ULL;
    }
  return h;
}

// Host-side copy of one trajectory's state (the unpacked form of an image).
struct HostState {
  ImageHeader h{};
  std::vector<double> rates, integ, accum;
  std::vector<int64_t> procstat;
  std::vector<int32_t> nsites;
  std::vector<int8_t> lat;
  std::vector<int32_t> entries;  // process-major avail_sites(p, 1..n_p, 1)
};

// Checks a state against the model and the lattice size before it reaches the device:
// every index the tables will hold stays inside the slot block.
int check_state(const HostState &st, const ModelDev &m) {
  const ImageHeader &h = st.h;
  if (h.P != m.P || h.nspecies != m.nspecies || h.spuck != m.spuck || h.backend != m.backend)
    return fail(KMC_ERR_ARG, "state belongs to another model (process/species/site counts differ)");
  if (h.X < 1 || h.Y < 1 || h.Z < 1 || (int64_t)h.X * h.Y * h.Z * h.spuck > (1 << 28) ||
      h.V != h.X * h.Y * h.Z * h.spuck)
    return fail(KMC_ERR_ARG, "state has a bad system size");
  if (h.rng_kind != RNG_GFORTRAN && h.rng_kind != RNG_PHILOX) return fail(KMC_ERR_ARG, "state has a bad rng kind");
  if (h.accum_from < 0 || h.accum_from > h.P) return fail(KMC_ERR_ARG, "state has a bad accum_from");
  if (h.status < 0 || h.status > ST_CANCELLED) return fail(KMC_ERR_ARG, "state has a bad status");
  const int V = h.V;
  for (int i = 0; i < V; i++)
    if (st.lat[i] < -1 || st.lat[i] > m.nspecies) return fail(KMC_ERR_ARG, "state lattice holds an unknown species");
  int64_t total = 0;
  for (int p = 0; p < h.P; p++) {
    if (st.nsites[p] < 0 || st.nsites[p] > V) return fail(KMC_ERR_TABLE, "state nr_of_sites out of range");
    total += st.nsites[p];
  }
  if (total != h.nentries || (int64_t)st.entries.size() != total)
    return fail(KMC_ERR_TABLE, "state avail_sites entries do not add up to nr_of_sites");
  std::vector<int32_t> seen(V + 1, 0);
  int64_t k = 0;
  for (int p = 0; p < h.P; p++)
    for (int i = 0; i < st.nsites[p]; i++, k++) {
      const int32_t s = st.entries[k];
      if (s < 1 || s > V) return fail(KMC_ERR_TABLE, "state avail_sites names a site outside the lattice");
      if (seen[s] == p + 1) return fail(KMC_ERR_TABLE, "state avail_sites lists a site twice for one process");
      seen[s] = p + 1;
    }
  return KMC_OK;
}

// Reads the state of an allocated slot (stream synchronised first).
int fetch_state(kmc_pool *p, int slot, HostState &st) {
  SlotDev d;
  int rc = read_slot(p, slot, &d);
  if (rc) return rc;
  const int P = d.P, V = d.V;
  const ModelHost &mh = p->models[d.model];
  ImageHeader &h = st.h;
  h.magic = IMAGE_MAGIC; h.version = IMAGE_VERSION; h.program_hash = program_hash(mh.prog);
  h.P = P; h.nspecies = mh.dev.nspecies; h.spuck = mh.dev.spuck; h.backend = mh.dev.backend;
  h.X = d.X; h.Y = d.Y; h.Z = d.Z; h.V = V;
  h.layer = d.layer; h.status = d.status; h.rng_kind = d.rng_kind; h.accum_from = d.accum_from;
  h.seed = d.seed; h.traj = d.traj;
  h.kmc_time = d.kmc_time; h.kmc_time_step = d.kmc_time_step; h.kmc_step = d.kmc_step;
  for (int i = 0; i < 4; i++) h.rng[i] = d.rng[i];
  std::vector<char> vec((size_t)P * 36);
  CK(cudaMemcpy(vec.data(), d.rates, vec.size(), cudaMemcpyDeviceToHost));
  st.rates.assign((const double *)vec.data(), (const double *)vec.data() + P);
  st.integ.assign((const double *)vec.data() + P, (const double *)vec.data() + 2 * P);
  st.accum.assign((const double *)vec.data() + 2 * P, (const double *)vec.data() + 3 * P);
  st.procstat.assign((const int64_t *)(vec.data() + 24 * (size_t)P), (const int64_t *)(vec.data() + 32 * (size_t)P));
  st.nsites.assign((const int32_t *)(vec.data() + 32 * (size_t)P), (const int32_t *)(vec.data() + 36 * (size_t)P));
  st.lat.resize(V);
  CK(cudaMemcpy(st.lat.data(), d.lat, V, cudaMemcpyDeviceToHost));
  std::vector<int64_t> off(P + 1, 0);
  for (int i = 0; i < P; i++) off[i + 1] = off[i] + std::max(0, std::min(st.nsites[i], V));
  h.nentries = off[P];
  st.entries.resize(off[P]);
  if (off[P] > 0) {
    AsyncScratch s_off(p->stream), s_ent(p->stream);
    CK(s_off.alloc(sizeof(int64_t) * (P + 1)));
    CK(s_ent.alloc(sizeof(int32_t) * off[P]));
    int64_t *d_off = s_off.as<int64_t>();
    int32_t *d_ent = s_ent.as<int32_t>();
    CK(cudaMemcpyAsync(d_off, off.data(), sizeof(int64_t) * (P + 1), cudaMemcpyHostToDevice, p->stream));
    kmc_pack_tables_kernel<<<P, 256, 0, p->stream>>>(d.as1, V + 1, d_off, P, d_ent);
    CK(cudaGetLastError());
    p->launches++;
    CK(cudaMemcpyAsync(st.entries.data(), d_ent, sizeof(int32_t) * off[P], cudaMemcpyDeviceToHost, p->stream));
    CK(cudaStreamSynchronize(p->stream));
  }
  h.bytes = image_layout(P, V, h.nentries).total;
  return KMC_OK;
}

// Writes a checked state into an allocated slot of the same model and size.
int store_state(kmc_pool *p, int slot, const HostState &st) {
  SlotHost &sh = p->slots[slot];
  const ImageHeader &h = st.h;
  const int P = h.P, V = h.V;
  SlotDev d = sh.dev;
  if (d.P != P || d.V != V) return fail(KMC_ERR_ARG, "state does not fit this slot");
  CK(cudaStreamSynchronize(p->stream));
  const size_t table_bytes = (size_t)((char *)d.rates - (char *)d.as1);
  CK(cudaMemsetAsync(d.as1, 0, table_bytes, p->stream));
  std::vector<char> vec((size_t)P * 36);
  memcpy(vec.data(), st.rates.data(), 8 * (size_t)P);
  memcpy(vec.data() + 8 * (size_t)P, st.integ.data(), 8 * (size_t)P);
  memcpy(vec.data() + 16 * (size_t)P, st.accum.data(), 8 * (size_t)P);
  memcpy(vec.data() + 24 * (size_t)P, st.procstat.data(), 8 * (size_t)P);
  memcpy(vec.data() + 32 * (size_t)P, st.nsites.data(), 4 * (size_t)P);
  CK(cudaMemcpyAsync(d.rates, vec.data(), vec.size(), cudaMemcpyHostToDevice, p->stream));
  CK(cudaMemcpyAsync(d.lat, st.lat.data(), V, cudaMemcpyHostToDevice, p->stream));
  std::vector<int64_t> off(P + 1, 0);
  for (int i = 0; i < P; i++) off[i + 1] = off[i] + st.nsites[i];
  AsyncScratch s_off(p->stream), s_ent(p->stream);
  if (off[P] > 0) {
    CK(s_off.alloc(sizeof(int64_t) * (P + 1)));
    CK(s_ent.alloc(sizeof(int32_t) * off[P]));
    int64_t *d_off = s_off.as<int64_t>();
    int32_t *d_ent = s_ent.as<int32_t>();
    CK(cudaMemcpyAsync(d_off, off.data(), sizeof(int64_t) * (P + 1), cudaMemcpyHostToDevice, p->stream));
    CK(cudaMemcpyAsync(d_ent, st.entries.data(), sizeof(int32_t) * off[P], cudaMemcpyHostToDevice, p->stream));
    kmc_unpack_tables_kernel<<<P, 256, 0, p->stream>>>(d.as1, d.as2, V + 1, d_off, P, d_ent);
    CK(cudaGetLastError());
    p->launches++;
  }
  d.layer = h.layer; d.status = h.status; d.rng_kind = h.rng_kind; d.accum_from = h.accum_from;
  d.seed = h.seed; d.traj = h.traj;
  d.kmc_time = h.kmc_time; d.kmc_time_step = h.kmc_time_step; d.kmc_step = h.kmc_step;
  for (int i = 0; i < 4; i++) d.rng[i] = h.rng[i];
  CK(cudaMemcpyAsync(p->d_slots + slot, &d, sizeof(SlotDev), cudaMemcpyHostToDevice, p->stream));
  CK(cudaStreamSynchronize(p->stream));
  sh.dev = d;
  return KMC_OK;
}

// Serialises a state into an image buffer of h.bytes bytes.
void write_image(const HostState &st, char *buf) {
  const ImageHeader &h = st.h;
  const ImageLayout L = image_layout(h.P, h.V, h.nentries);
  memset(buf, 0, L.total);
  memcpy(buf, &h, sizeof(h));
  const size_t P = h.P;
  memcpy(buf + L.vec, st.rates.data(), 8 * P);
  memcpy(buf + L.vec + 8 * P, st.integ.data(), 8 * P);
  memcpy(buf + L.vec + 16 * P, st.accum.data(), 8 * P);
  memcpy(buf + L.vec + 24 * P, st.procstat.data(), 8 * P);
  memcpy(buf + L.vec + 32 * P, st.nsites.data(), 4 * P);
  memcpy(buf + L.lat, st.lat.data(), h.V);
  if (h.nentries) memcpy(buf + L.ent, st.entries.data(), 4 * (size_t)h.nentries);
}

// Parses an image buffer (sizes checked; contents checked later by check_state).
int read_image(const void *buf, size_t bytes, HostState &st) {
  if (!buf || bytes < sizeof(ImageHeader)) return fail(KMC_ERR_ARG, "state image too short");
  memcpy(&st.h, buf, sizeof(ImageHeader));
  const ImageHeader &h = st.h;
  if (h.magic != IMAGE_MAGIC || h.version != IMAGE_VERSION) return fail(KMC_ERR_ARG, "not a state image (magic/version)");
  if (h.P < 1 || h.P > 256 || h.V < 1 || h.V > (1 << 28) || h.nentries < 0 || h.nentries > (int64_t)h.P * h.V)
    return fail(KMC_ERR_ARG, "state image header out of range");
  const ImageLayout L = image_layout(h.P, h.V, h.nentries);
  if (h.bytes != L.total || bytes < L.total) return fail(KMC_ERR_ARG, "state image size does not match its header");
  const char *b = static_cast<const char *>(buf);
  const size_t P = h.P;
  st.rates.resize(P); st.integ.resize(P); st.accum.resize(P); st.procstat.resize(P); st.nsites.resize(P);
  memcpy(st.rates.data(), b + L.vec, 8 * P);
  memcpy(st.integ.data(), b + L.vec + 8 * P, 8 * P);
  memcpy(st.accum.data(), b + L.vec + 16 * P, 8 * P);
  memcpy(st.procstat.data(), b + L.vec + 24 * P, 8 * P);
  memcpy(st.nsites.data(), b + L.vec + 32 * P, 4 * P);
  st.lat.resize(h.V);
  memcpy(st.lat.data(), b + L.lat, h.V);
  st.entries.resize(h.nentries);
  if (h.nentries) memcpy(st.entries.data(), b + L.ent, 4 * (size_t)h.nentries);
  return KMC_OK;
}

// Allocates a slot and its arena block for a state of (P, V).
int new_slot(kmc_pool *p, int model, const ImageHeader &h, int *slot_out) {
  int slot = -1;
  for (int s = 0; s < (int)p->slots.size(); s++)
    if (!p->slots[s].used) { slot = s; break; }
  if (slot < 0) return fail(KMC_ERR_NOMEM, "no free trajectory slot");
  const Layout L = slot_layout(h.P, h.V);
  size_t off;
  int rc = alloc_block(p, L.total, &off);
  if (rc) return rc;
  char *base = p->arena + off;
  SlotDev d{};
  d.lat = (int8_t *)(base + L.lat);
  d.as1 = (int32_t *)(base + L.as1);
  d.as2 = (int32_t *)(base + L.as2);
  d.rates = (double *)(base + L.rates);
  d.integ = (double *)(base + L.integ);
  d.accum = (double *)(base + L.accum);
  d.nsites = (int32_t *)(base + L.nsites);
  d.procstat = (int64_t *)(base + L.procstat);
  d.X = h.X; d.Y = h.Y; d.Z = h.Z; d.V = h.V;
  d.model = model; d.P = h.P;
  SlotHost &sh = p->slots[slot];
  sh = SlotHost();
  sh.used = true;
  sh.off = off;
  sh.bytes = L.total;
  sh.dev = d;
  *slot_out = slot;
  return KMC_OK;
}

void drop_slot(kmc_pool *p, int slot) {
  free_block(p, p->slots[slot].off, p->slots[slot].bytes);
  p->slots[slot] = SlotHost();
}

}  // namespace

// ===================================================================== C-ABI
extern "C" {

int kmc_pool_save_state(kmc_pool *p, int32_t slot, void *buf, size_t capacity, size_t *bytes) {
  int rc = check_slot(p, slot);
  if (rc) return rc;
  if (!bytes) return fail(KMC_ERR_ARG, "bad arguments");
  std::lock_guard<std::mutex> lock(p->mu);
  CK(cudaSetDevice(p->device));
  HostState st;
  rc = fetch_state(p, slot, st);
  if (rc) return rc;
  *bytes = st.h.bytes;
  if (!buf) return KMC_OK;
  if (capacity < st.h.bytes) return fail(KMC_ERR_ARG, "state image buffer too small");
  write_image(st, static_cast<char *>(buf));
  return KMC_OK;
}

int kmc_pool_restore_state(kmc_pool *p, int32_t model_id, const void *buf, size_t bytes, int32_t *slot) {
  if (!p || !slot || model_id < 0 || model_id >= (int)p->models.size()) return fail(KMC_ERR_ARG, "bad arguments");
  HostState st;
  int rc = read_image(buf, bytes, st);
  if (rc) return rc;
  const ModelHost &mh = p->models[model_id];
  if (st.h.program_hash != program_hash(mh.prog)) return fail(KMC_ERR_ARG, "state image was saved from another model program");
  rc = check_state(st, mh.dev);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(p->mu);
  CK(cudaSetDevice(p->device));
  int s = -1;
  rc = new_slot(p, model_id, st.h, &s);
  if (rc) return rc;
  rc = store_state(p, s, st);
  if (rc) { drop_slot(p, s); return rc; }
  *slot = s;
  return KMC_OK;
}

int kmc_check_image(const int32_t *program, int32_t program_len, const void *buf, size_t bytes) {
  ModelDev md{};
  int rc = validate_program(program, program_len, &md);
  if (rc) return rc;
  HostState st;
  rc = read_image(buf, bytes, st);
  if (rc) return rc;
  if (st.h.program_hash != program_hash(std::vector<int32_t>(program, program + program_len)))
    return fail(KMC_ERR_ARG, "state image was saved from another model program");
  return check_state(st, md);
}

int kmc_save_state(kmc_handle *h, void *buf, size_t capacity, size_t *bytes) {
  if (!h || !h->pool) return fail(KMC_ERR_ARG, "bad handle");
  return kmc_pool_save_state(h->pool, h->slot, buf, capacity, bytes);
}

int kmc_load_state(kmc_handle *h, const void *buf, size_t bytes) {
  if (!h || !h->pool) return fail(KMC_ERR_ARG, "bad handle");
  kmc_pool *p = h->pool;
  HostState st;
  int rc = read_image(buf, bytes, st);
  if (rc) return rc;
  const ModelHost &mh = p->models[h->model];
  if (st.h.program_hash != program_hash(mh.prog)) return fail(KMC_ERR_ARG, "state image was saved from another model program");
  rc = check_state(st, mh.dev);
  if (rc) return rc;
  const SlotDev &d = p->slots[h->slot].dev;
  if (st.h.X != d.X || st.h.Y != d.Y || st.h.Z != d.Z) return fail(KMC_ERR_ARG, "state image has another system size");
  std::lock_guard<std::mutex> lock(p->mu);
  CK(cudaSetDevice(p->device));
  return store_state(p, h->slot, st);
}

int kmc_save_reload(kmc_handle *h, const char *path) {
  if (!h || !h->pool || !path) return fail(KMC_ERR_ARG, "bad arguments");
  kmc_pool *p = h->pool;
  HostState st;
  {
    std::lock_guard<std::mutex> lock(p->mu);
    CK(cudaSetDevice(p->device));
    int rc = fetch_state(p, h->slot, st);
    if (rc) return rc;
  }
  const ImageHeader &hd = st.h;
  kmc_reload::ReloadData d;
  d.P = hd.P;
  d.V = hd.V;
  d.dims[0] = hd.X; d.dims[1] = hd.Y; d.dims[2] = hd.Z;
  d.kmc_time = hd.kmc_time;
  d.kmc_time_step = hd.kmc_time_step;
  d.walltime = h->walltime;
  d.kmc_step = hd.kmc_step;
  d.rng_kind = hd.rng_kind; d.seed = hd.seed; d.traj = hd.traj;
  for (int i = 0; i < 4; i++) d.rng[i] = hd.rng[i];
  d.rates.assign(st.rates.begin(), st.rates.begin() + hd.P);
  d.integ.assign(st.integ.begin(), st.integ.begin() + hd.P);
  d.procstat.assign(st.procstat.begin(), st.procstat.begin() + hd.P);
  d.nsites.assign(st.nsites.begin(), st.nsites.begin() + hd.P);
  d.lattice.assign(st.lat.begin(), st.lat.end());
  d.as1.resize(hd.P);
  int64_t k = 0;
  for (int q = 0; q < hd.P; q++) d.as1[q].assign(st.entries.begin() + k, st.entries.begin() + k + st.nsites[q]), k += st.nsites[q];
  return kmc_reload::write_reload(path, d);
}

int kmc_reload_info(const char *path, int32_t *nr_of_proc, int32_t *volume, int32_t dims[3]) {
  if (!path || !nr_of_proc || !volume || !dims) return fail(KMC_ERR_ARG, "bad arguments");
  kmc_reload::ReloadFile r;
  int rc = kmc_reload::parse_reload(path, r, true);
  if (rc) return rc;
  if (!r.have_proc || !r.have_volume) return fail(KMC_ERR_ARG, std::string(path) + ": no nr_of_proc / volume");
  *nr_of_proc = (int32_t)r.nr_of_proc;
  *volume = (int32_t)r.volume;
  for (int i = 0; i < 3; i++) dims[i] = r.dims[i];
  return KMC_OK;
}

int kmc_check_reload(const int32_t *program, int32_t program_len, const int32_t dims[3], const char *path) {
  if (!program || program_len < 7 || !dims || !path) return fail(KMC_ERR_ARG, "bad arguments");
  int P = 0, nspecies = 0, spuck = 0;
  if (program[2] == 2) {  // otf program: the checks kmc_otf_create makes
    int rc = kmc_otf_check_program(program, program_len);
    if (rc) return rc;
    P = program[3]; nspecies = program[4]; spuck = program[6];
  } else {
    ModelDev md{};
    int rc = validate_program(program, program_len, &md);
    if (rc) return rc;
    P = md.P; nspecies = md.nspecies; spuck = md.spuck;
  }
  if (dims[0] < 1 || dims[1] < 1 || dims[2] < 1) return fail(KMC_ERR_ARG, "bad system size");
  const int64_t V = (int64_t)dims[0] * dims[1] * dims[2] * spuck;
  if (V > (program[2] == 2 ? (1 << 24) : (1 << 28))) return fail(KMC_ERR_ARG, "lattice too large");
  kmc_reload::ReloadFile r;
  int rc = kmc_reload::parse_reload(path, r, false);
  if (rc) return rc;
  kmc_reload::ReloadData d;
  return kmc_reload::read_reload(r, P, (int)V, nspecies, d);
}

int kmc_load_reload(kmc_handle *h, const char *path) {
  if (!h || !h->pool || !path) return fail(KMC_ERR_ARG, "bad arguments");
  kmc_pool *p = h->pool;
  kmc_reload::ReloadFile r;
  int rc = kmc_reload::parse_reload(path, r, false);
  if (rc) return rc;
  const int P = h->P, V = h->V;
  kmc_reload::ReloadData d;
  rc = kmc_reload::read_reload(r, P, V, h->nspecies, d);
  if (rc) return rc;
  HostState st;
  {
    std::lock_guard<std::mutex> lock(p->mu);
    CK(cudaSetDevice(p->device));
    rc = fetch_state(p, h->slot, st);  // keeps the random stream when the file has none
    if (rc) return rc;
  }
  ImageHeader &hd = st.h;
  st.lat.resize(V);
  for (int i = 0; i < V; i++) st.lat[i] = (int8_t)d.lattice[i];
  st.entries.clear();
  for (int q = 0; q < P; q++) {
    st.entries.insert(st.entries.end(), d.as1[q].begin(), d.as1[q].end());
    st.nsites[q] = d.nsites[q];
    st.procstat[q] = d.procstat[q];
    st.rates[q] = d.rates[q];
    st.integ[q] = d.integ[q];
    st.accum[q] = 0.0;
  }
  hd.nentries = (int64_t)st.entries.size();
  hd.kmc_time = d.kmc_time;
  hd.kmc_step = d.kmc_step;
  hd.kmc_time_step = d.kmc_time_step;
  hd.status = ST_OK;
  hd.accum_from = 0;  // update_accum_rate on the next step
  if (r.have_rng) {
    hd.rng_kind = d.rng_kind;
    hd.seed = d.seed;
    hd.traj = d.traj;
    for (int i = 0; i < 4; i++) hd.rng[i] = d.rng[i];
  }
  const ModelHost &mh = p->models[h->model];
  rc = check_state(st, mh.dev);
  if (rc) return rc;
  {
    std::lock_guard<std::mutex> lock(p->mu);
    CK(cudaSetDevice(p->device));
    rc = store_state(p, h->slot, st);
    if (rc) return rc;
  }
  if (r.have_walltime) h->walltime = r.walltime;
  return KMC_OK;
}

// ------------------------------------------------------------ on-device sampling
static int sample_launch(kmc_pool *p, const int32_t *slots, int32_t n, int mode, const SampleOut &out) {
  std::vector<double *> recs(n);
  for (int i = 0; i < n; i++) {
    const SlotHost &sh = p->slots[slots[i]];
    if (!sh.samp_bytes) return fail(KMC_ERR_ARG, "slot is not sampling (kmc_pool_sample_begin first)");
    recs[i] = reinterpret_cast<double *>(p->arena + sh.samp_off);
  }
  AsyncScratch s_list(p->stream), s_recs(p->stream);
  CK(s_list.alloc(sizeof(int32_t) * n));
  CK(s_recs.alloc(sizeof(double *) * n));
  int32_t *d_list = s_list.as<int32_t>();
  double **d_recs = s_recs.as<double *>();
  CK(cudaMemcpyAsync(d_list, slots, sizeof(int32_t) * n, cudaMemcpyHostToDevice, p->stream));
  CK(cudaMemcpyAsync(d_recs, recs.data(), sizeof(double *) * n, cudaMemcpyHostToDevice, p->stream));
  kmc_sample_kernel<<<n, 256, 0, p->stream>>>(p->d_slots, p->d_models, d_list, d_recs, n, mode, out);
  CK(cudaGetLastError());
  p->launches++;
  return KMC_OK;
}

static int check_list(kmc_pool *p, const int32_t *slots, int32_t n) {
  if (!p || n < 1 || !slots) return fail(KMC_ERR_ARG, "bad arguments");
  std::vector<char> seen(p->slots.size(), 0);
  for (int i = 0; i < n; i++) {
    int rc = check_slot(p, slots[i]);
    if (rc) return rc;
    if (seen[slots[i]]) return fail(KMC_ERR_ARG, "slot listed twice");
    seen[slots[i]] = 1;
  }
  return KMC_OK;
}

int kmc_pool_sample_begin(kmc_pool *p, const int32_t *slots, int32_t n) {
  int rc = check_list(p, slots, n);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(p->mu);
  CK(cudaSetDevice(p->device));
  std::vector<int> fresh;
  for (int i = 0; i < n; i++) {
    SlotHost &sh = p->slots[slots[i]];
    if (sh.samp_bytes) continue;  // a running record restarts
    const ModelDev &m = p->models[sh.dev.model].dev;
    const size_t bytes = align_up(samp_words(m.P, m.nspecies * m.spuck) * 8, 256);
    size_t off;
    rc = alloc_block(p, bytes, &off);
    if (rc) {
      for (int s : fresh) {
        free_block(p, p->slots[s].samp_off, p->slots[s].samp_bytes);
        p->slots[s].samp_bytes = 0;
      }
      return rc;
    }
    sh.samp_off = off;
    sh.samp_bytes = bytes;
    fresh.push_back(slots[i]);
  }
  SampleOut none{};
  return sample_launch(p, slots, n, SAMPLE_BEGIN, none);
}

int kmc_pool_sample(kmc_pool *p, const int32_t *slots, int32_t n) {
  int rc = check_list(p, slots, n);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(p->mu);
  CK(cudaSetDevice(p->device));
  SampleOut none{};
  return sample_launch(p, slots, n, SAMPLE_TAKE, none);
}

static int sample_finish(kmc_pool *p, const int32_t *slots, int32_t n, int32_t occ_stride, int32_t proc_stride,
                         double *occ_mean, int64_t *procstat_delta, double *integ_delta, double *times,
                         int64_t *steps, int32_t *status) {
  const size_t nocc = (size_t)n * occ_stride, nps = (size_t)n * proc_stride;
  const size_t bytes = nocc * 8 + nps * 16 + (size_t)n * (16 + 8 + 4);
  AsyncScratch s_out(p->stream);
  CK(s_out.alloc(bytes));
  char *d = s_out.as<char>();
  SampleOut out;
  out.occ_stride = occ_stride;
  out.proc_stride = proc_stride;
  out.occ = reinterpret_cast<double *>(d);
  out.dps = reinterpret_cast<int64_t *>(d + nocc * 8);
  out.dig = reinterpret_cast<double *>(d + nocc * 8 + nps * 8);
  out.times = reinterpret_cast<double *>(d + nocc * 8 + nps * 16);
  out.steps = reinterpret_cast<int64_t *>(d + nocc * 8 + nps * 16 + (size_t)n * 16);
  out.status = reinterpret_cast<int32_t *>(d + nocc * 8 + nps * 16 + (size_t)n * 24);
  int rc = sample_launch(p, slots, n, SAMPLE_END, out);
  if (rc) return rc;
  std::vector<char> h(bytes);
  CK(cudaMemcpyAsync(h.data(), d, bytes, cudaMemcpyDeviceToHost, p->stream));
  CK(cudaStreamSynchronize(p->stream));
  if (occ_mean) memcpy(occ_mean, h.data(), nocc * 8);
  if (procstat_delta) memcpy(procstat_delta, h.data() + nocc * 8, nps * 8);
  if (integ_delta) memcpy(integ_delta, h.data() + nocc * 8 + nps * 8, nps * 8);
  if (times) memcpy(times, h.data() + nocc * 8 + nps * 16, (size_t)n * 16);
  if (steps) memcpy(steps, h.data() + nocc * 8 + nps * 16 + (size_t)n * 16, (size_t)n * 8);
  if (status) memcpy(status, h.data() + nocc * 8 + nps * 16 + (size_t)n * 24, (size_t)n * 4);
  for (int i = 0; i < n; i++) {
    SlotHost &sh = p->slots[slots[i]];
    free_block(p, sh.samp_off, sh.samp_bytes);
    sh.samp_off = sh.samp_bytes = 0;
  }
  return KMC_OK;
}

int kmc_pool_sample_end(kmc_pool *p, const int32_t *slots, int32_t n, int32_t occ_stride, int32_t proc_stride,
                        double *occ_mean, int64_t *procstat_delta, double *integ_delta, double *times, int64_t *steps,
                        int32_t *status) {
  int rc = check_list(p, slots, n);
  if (rc) return rc;
  if (occ_stride < 1 || proc_stride < 1) return fail(KMC_ERR_ARG, "bad strides");
  std::lock_guard<std::mutex> lock(p->mu);
  CK(cudaSetDevice(p->device));
  return sample_finish(p, slots, n, occ_stride, proc_stride, occ_mean, procstat_delta, integ_delta, times, steps,
                       status);
}

int kmc_pool_sample_run(kmc_pool *p, const int32_t *slots, int32_t n, int32_t samples, int64_t steps_per_sample,
                        int32_t occ_stride, int32_t proc_stride, double *occ_mean, int64_t *procstat_delta,
                        double *integ_delta, double *times, int64_t *steps, int32_t *status) {
  if (samples < 1 || steps_per_sample < 0) return fail(KMC_ERR_ARG, "bad sample counts");
  if (occ_stride < 1 || proc_stride < 1) return fail(KMC_ERR_ARG, "bad strides");
  int rc = kmc_pool_sample_begin(p, slots, n);
  if (rc) return rc;
  {
    std::lock_guard<std::mutex> lock(p->mu);
    std::vector<int64_t> st(n, steps_per_sample);
    SampleOut none{};
    rc = run_rounds(p, slots, st.data(), n, samples,
                    [&](int) { return sample_launch(p, slots, n, SAMPLE_TAKE, none); });
  }
  if (rc) return rc;
  return kmc_pool_sample_end(p, slots, n, occ_stride, proc_stride, occ_mean, procstat_delta, integ_delta, times,
                             steps, status);
}

}  // extern "C"
