// kmc_engine.cu -- GB300 (sm_103a) lattice-kMC step engine behind the C-ABI of
// include/kmc_gb300.h.
//
// Kernels
//   kmc_run_kernel     persistent do_kmc_steps (proclist_generic_subroutines.mpy:1-44),
//                      defined in kmc_run.cuh; this file builds its one-warp-per-
//                      trajectory variants, kmc_run_g16.cu the two-per-warp ones.
//   kmc_solo_kernel    do_kmc_steps for small launches of models with up to 8
//                      processes: one warp per trajectory, the steps on one lane
//                      (kmc_run.cuh, built in kmc_solo.cu).
//   kmc_init_kernel    device-side initialize_state (proclist_generic_subroutines.mpy:
//                      236-304): default species, then every touch-up in parallel
//                      (fresh touch-ups only append at their own site), then a
//                      per-process ballot compaction that lists sites in ascending
//                      order -- the order the reference's serial touch-up loop appends.
//   kmc_command_kernel single-warp commands on one trajectory: run_proc_nr, touchup,
//                      get_next_kmc_step, update_accum_rate, update_integ_rate,
//                      replace_species.
//   kmc_occupation_kernel  per-slot species counts per site index (get_occupation).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/kmc_gb300.h"
#include "kmc_device.cuh"
#include "kmc_host.h"
#include "kmc_run.cuh"

using namespace kmc;
using namespace kmc_host;

#define KMC_MAXK 16

// -------------------------------------------------------------------- init kernel
struct InitArgs {
  SlotDev *slots;
  const ModelDev *models;
  const SlotDev *staged;    // slot descriptors to install
  const int32_t *list;      // slot ids
  const double *rates;      // concatenated rate vectors
  const int32_t *rate_off;  // per item offset into rates
  int32_t n;
};

__global__ void __launch_bounds__(256) kmc_init_kernel(InitArgs a) {
  const int lane = threadIdx.x & 31;
  const int item = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (item >= a.n) return;
  const int slot = a.list[item];
  SlotDev &S = a.slots[slot];
  const SlotDev st = a.staged[item];
  const ModelDev M = a.models[st.model];
  const int P = M.P, V = st.V, stride = V + 1;
  const int32_t *site_layer = M.prog + M.off_site_layer;
  const int32_t *site_def = M.prog + M.off_site_default;

  // default species on the chosen layer, null species elsewhere
  for (int s = lane; s < V; s += 32) {
    const int n = s % M.spuck;
    st.lat[s] = (int8_t)(site_layer[n] == st.layer ? site_def[n] : M.null_species);
  }
  for (int i = lane; i < P; i += 32) {
    st.rates[i] = a.rates[a.rate_off[item] + i];
    st.integ[i] = 0.0;
    st.procstat[i] = 0;
    st.nsites[i] = 0;
  }
  __syncwarp();

  // every touch-up in collect mode: flag (p, site) in as2
  View v;
  v.lat = st.lat; v.as1 = st.as1; v.as2 = st.as2; v.ns = st.nsites; v.prog = M.prog;
  v.g.X = st.X; v.g.Y = st.Y; v.g.Z = st.Z; v.g.spuck = M.spuck;
  v.stride = stride; v.backend = M.backend; v.P = P; v.off_groups = M.off_groups;
  v.collect = true; v.err = ST_OK; v.minp = P;
  const int ncells = st.X * st.Y * st.Z;
  for (int c = lane; c < ncells; c += 32) {
    const int x = c % st.X, y = (c / st.X) % st.Y, z = c / (st.X * st.Y);
    if (M.backend == 1) {
      run_stream(v, M.prog[M.off_touch], x, y, z);
    } else {
      for (int n = 0; n < M.spuck; n++)
        if (site_layer[n] == st.layer) run_stream(v, M.prog[M.off_touch + n], x, y, z);
    }
  }
  const unsigned bad = __ballot_sync(0xffffffffu, v.err != ST_OK);
  __syncwarp();

  // compaction: as1[p] lists the flagged sites in ascending order
  const unsigned lt = (1u << lane) - 1u;
  for (int p = 0; p < P; p++) {
    int32_t *a1 = st.as1 + (size_t)p * stride;
    int32_t *a2 = st.as2 + (size_t)p * stride;
    int base = 0;
    for (int s0 = 1; s0 <= V; s0 += 32) {
      const int s = s0 + lane;
      const bool f = (s <= V) && a2[s] != 0;
      const unsigned b = __ballot_sync(0xffffffffu, f);
      if (f) {
        const int pos = base + __popc(b & lt) + 1;
        a1[pos] = s;
        a2[s] = pos;
      }
      base += __popc(b);
    }
    if (lane == 0) st.nsites[p] = base;
  }
  __syncwarp();
  if (lane == 0) {
    // update_accum_rate, as kmos.run.KMC_Model.reset does after set_rate_constants
    double acc = 0.0;
    for (int i = 0; i < P; i++) {
      const double term = __dmul_rn((double)st.nsites[i], st.rates[i]);
      acc = (i == 0) ? term : __dadd_rn(acc, term);
      st.accum[i] = acc;
    }
    SlotDev d = st;
    d.status = bad ? ST_PROGRAM : ST_OK;
    d.accum_from = P;
    d.kmc_time = 0.0;
    d.kmc_time_step = 0.0;
    d.kmc_step = 0;
    if (st.rng_kind == RNG_GFORTRAN) {
      gfortran_seed(d.rng, (int32_t)st.seed);
    } else {
      d.rng[0] = 0; d.rng[1] = d.rng[2] = d.rng[3] = 0;
    }
    S = d;
  }
}

// ----------------------------------------------------------------- command kernel
enum Cmd { CMD_RUN_PROC = 1, CMD_TOUCHUP = 2, CMD_GET_NEXT = 3, CMD_ACCUM = 4, CMD_INTEG = 5, CMD_REPLACE = 6,
           CMD_TOUCHUP_LIST = 7 };

struct CmdArgs {
  SlotDev *slots;
  const ModelDev *models;
  int32_t slot, cmd, a0, a1, a2;
  const int32_t *list;  // sites of CMD_TOUCHUP_LIST (a0 of them)
  int32_t *out;  // [status, proc, site]
};

__device__ void full_accum(SlotDev &S, int P) {
  double acc = 0.0;
  for (int i = 0; i < P; i++) {
    const double term = __dmul_rn((double)S.nsites[i], S.rates[i]);
    acc = (i == 0) ? term : __dadd_rn(acc, term);
    S.accum[i] = acc;
  }
  S.accum_from = P;
}

__global__ void kmc_command_kernel(CmdArgs a) {
  if (threadIdx.x != 0) return;
  SlotDev &S = a.slots[a.slot];
  const ModelDev M = a.models[S.model];
  const int P = M.P;
  View v;
  v.lat = S.lat; v.as1 = S.as1; v.as2 = S.as2; v.ns = S.nsites; v.prog = M.prog;
  v.g.X = S.X; v.g.Y = S.Y; v.g.Z = S.Z; v.g.spuck = M.spuck;
  v.stride = S.V + 1; v.backend = M.backend; v.P = P; v.off_groups = M.off_groups;
  v.collect = false; v.err = ST_OK; v.minp = S.accum_from;
  int status = ST_OK, proc = 0, site = 0;
  switch (a.cmd) {
    case CMD_RUN_PROC: {
      const int p = a.a0, s = a.a1;
      S.procstat[p - 1] += 1;
      int bx, by, bz, bn;
      v.g.coords(s, bx, by, bz, bn);
      run_stream(v, M.prog[M.off_proc + p - 1], bx, by, bz);
      status = v.err;
      S.accum_from = v.minp;
      break;
    }
    case CMD_TOUCHUP: {
      int bx, by, bz, bn;
      v.g.coords(a.a0, bx, by, bz, bn);
      run_stream(v, M.prog[M.off_touch + (M.backend == 1 ? 0 : bn - 1)], bx, by, bz);
      status = v.err;
      S.accum_from = v.minp;
      break;
    }
    case CMD_TOUCHUP_LIST: {  // the touch-ups of a0 sites, one after the other, in list order
      for (int k = 0; k < a.a0 && v.err == ST_OK; k++) {
        int bx, by, bz, bn;
        v.g.coords(a.list[k], bx, by, bz, bn);
        run_stream(v, M.prog[M.off_touch + (M.backend == 1 ? 0 : bn - 1)], bx, by, bz);
      }
      status = v.err;
      S.accum_from = v.minp;
      break;
    }
    case CMD_GET_NEXT: {
      // get_next_kmc_step: the time draw picks the site; no clock update
      double rt, rp, rs;
      draw3(S.rng_kind, S.rng, S.seed, S.traj, rt, rp, rs);
      full_accum(S, P);
      const double total = S.accum[P - 1];
      if (!(total > 0.0)) { status = ST_DEADLOCK; break; }
      const double val = __dmul_rn(rp, total);
      proc = 0;
      while (proc < P && !(S.accum[proc] > val || S.accum[proc] == total)) proc++;
      const int n = S.nsites[proc];
      if (n <= 0) { status = ST_DEADLOCK; break; }
      int idx = (int)__dadd_rn(1.0, __dmul_rn(rt, (double)n));
      if (idx > n) idx = n;
      site = S.as1[(size_t)proc * (S.V + 1) + idx];
      proc += 1;
      break;
    }
    case CMD_ACCUM:
      full_accum(S, P);
      break;
    case CMD_INTEG:
      for (int i = 0; i < P; i++)
        S.integ[i] = __dadd_rn(S.integ[i], __dmul_rn(__dmul_rn((double)S.nsites[i], S.rates[i]), S.kmc_time_step));
      break;
    case CMD_REPLACE: {
      const int s = a.a0;
      if (S.lat[s - 1] != a.a1) status = ST_SPECIES;
      else S.lat[s - 1] = (int8_t)a.a2;
      break;
    }
    default:
      status = ST_ARG;
  }
  a.out[0] = status;
  a.out[1] = proc;
  a.out[2] = site;
}

// -------------------------------------------------------------- occupation kernel
__global__ void kmc_occupation_kernel(const SlotDev *slots, const ModelDev *models, const int32_t *list,
                                      int32_t n, int32_t stride, unsigned long long *out) {
  __shared__ unsigned int hist[32 * 32];
  const int item = blockIdx.x;
  if (item >= n) return;
  const SlotDev &S = slots[list[item]];
  const ModelDev M = models[S.model];
  const int ns = M.nspecies, sp = M.spuck;
  for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  for (int s = threadIdx.x; s < S.V; s += blockDim.x) {
    const int spc = S.lat[s];
    if (spc >= 0 && spc < ns && spc < 32) atomicAdd(&hist[spc * 32 + (s % sp)], 1u);
  }
  __syncthreads();
  // a row holds `stride` counters: the host refuses strides below ns * sp, and the copy
  // stops at the row's end whatever it is given
  const int nc = min(ns * sp, stride);
  for (int i = threadIdx.x; i < nc; i += blockDim.x)
    out[(size_t)item * stride + i] = hist[(i / sp) * 32 + (i % sp)];
}

// ---------------------------------------------------------------- results gather
struct ResultRow {
  double kmc_time;
  int64_t kmc_step;
  int32_t status, pad;
};

__global__ void kmc_results_kernel(const SlotDev *slots, const int32_t *list, int32_t n, int32_t stride,
                                   int64_t *procstat, double *integ, ResultRow *rows) {
  const int item = blockIdx.x;
  if (item >= n) return;
  const SlotDev &S = slots[list[item]];
  for (int i = threadIdx.x; i < stride; i += blockDim.x) {
    const bool in = i < S.P;
    procstat[(size_t)item * stride + i] = in ? S.procstat[i] : 0;
    integ[(size_t)item * stride + i] = in ? S.integ[i] : 0.0;
  }
  if (threadIdx.x == 0) {
    ResultRow r;
    r.kmc_time = S.kmc_time;
    r.kmc_step = S.kmc_step;
    r.status = S.status;
    r.pad = 0;
    rows[item] = r;
  }
}

// ================================================================== host side
namespace kmc_host {
thread_local std::string g_err;

int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}


int alloc_block(kmc_pool *p, size_t bytes, size_t *off) {
  bytes = align_up(bytes, 256);
  for (auto it = p->free_blocks.begin(); it != p->free_blocks.end(); ++it) {
    if (it->second >= bytes) {
      *off = it->first;
      const size_t rest = it->second - bytes;
      const size_t noff = it->first + bytes;
      p->free_blocks.erase(it);
      if (rest) p->free_blocks[noff] = rest;
      return KMC_OK;
    }
  }
  return fail(KMC_ERR_NOMEM, "device arena has no free block of the requested size");
}

void free_block(kmc_pool *p, size_t off, size_t bytes) {
  bytes = align_up(bytes, 256);
  auto it = p->free_blocks.emplace(off, bytes).first;
  auto next = std::next(it);
  if (next != p->free_blocks.end() && it->first + it->second == next->first) {
    it->second += next->second;
    p->free_blocks.erase(next);
  }
  if (it != p->free_blocks.begin()) {
    auto prev = std::prev(it);
    if (prev->first + prev->second == it->first) {
      prev->second += it->second;
      p->free_blocks.erase(it);
    }
  }
}


int validate_program(const int32_t *prog, int32_t len, ModelDev *m) {
  if (!prog || len < 20) return fail(KMC_ERR_PROGRAM, "program too short");
  if ((uint32_t)prog[0] != 0x4B4D4331u || prog[1] != 1) return fail(KMC_ERR_PROGRAM, "bad program magic/version");
  m->backend = prog[2]; m->P = prog[3]; m->nspecies = prog[4]; m->null_species = prog[5];
  m->spuck = prog[6]; m->ngroups = prog[8];
  m->off_proc = prog[10]; m->off_touch = prog[11]; m->off_groups = prog[12];
  m->off_site_layer = prog[13]; m->off_site_default = prog[14]; m->len = len;
  if (prog[15] != len) return fail(KMC_ERR_PROGRAM, "program length mismatch");
  if (m->P < 1 || m->P > 256) return fail(KMC_ERR_PROGRAM, "process count must be in 1..256");
  if (m->spuck < 1 || m->spuck > 32) return fail(KMC_ERR_PROGRAM, "sites per unit cell must be in 1..32");
  if (m->nspecies < 1 || m->nspecies > 30) return fail(KMC_ERR_PROGRAM, "species count must be in 1..30");
  if (m->backend != 0 && m->backend != 1) return fail(KMC_ERR_PROGRAM, "unknown backend");
  if (m->ngroups < 0 || m->ngroups > len) return fail(KMC_ERR_PROGRAM, "bad group count");
  const int nt = m->backend == 1 ? 1 : m->spuck;
  // [start, start + count) inside [0, limit), in 64-bit so that no offset can wrap
  auto span_ok = [](int64_t start, int64_t count, int64_t limit) {
    return start >= 0 && count >= 0 && start + count <= limit;
  };
  if (!span_ok(m->off_proc, m->P + 1, len) || !span_ok(m->off_touch, nt + 1, len) ||
      !span_ok(m->off_groups, m->ngroups, len) || !span_ok(m->off_site_layer, m->spuck, len) ||
      !span_ok(m->off_site_default, m->spuck, len))
    return fail(KMC_ERR_PROGRAM, "program section outside the program");
  for (int i = 0; i <= m->P; i++)
    if (prog[m->off_proc + i] <= 0 || prog[m->off_proc + i] > len) return fail(KMC_ERR_PROGRAM, "bad op offset");
  for (int i = 0; i <= nt; i++)
    if (prog[m->off_touch + i] <= 0 || prog[m->off_touch + i] > len) return fail(KMC_ERR_PROGRAM, "bad touch-up offset");
  // walk every op stream: known ops, in-range processes/groups/sites/species, and an
  // OP_END before the end of the program
  auto coord_ok = [&](int32_t w) { const int n = (int)((uint32_t)w >> 24); return n >= 1 && n <= m->spuck; };
  auto species_ok = [&](int32_t s) { return s >= -1 && s <= m->nspecies; };
  auto walk = [&](int pos) -> bool {
    while (pos < len) {
      const uint32_t h = (uint32_t)prog[pos];
      const int op = h & 0xFF, cnt = (h >> 8) & 0xFF, arg = (h >> 16) & 0xFFFF;
      switch (op) {
        case OP_END: return true;
        case OP_REPLACE:
          if (pos + 3 >= len || !coord_ok(prog[pos + 1]) || !species_ok(prog[pos + 3])) return false;
          pos += 4; break;
        case OP_GDEL:
          if (pos + 1 >= len || arg < 1 || arg > m->P || !coord_ok(prog[pos + 1])) return false;
          pos += 2; break;
        case OP_ADD:
          if (pos + 1 + 2 * cnt >= len || arg < 1 || arg > m->P || !coord_ok(prog[pos + 1])) return false;
          for (int c = 0; c < cnt; c++) if (!coord_ok(prog[pos + 2 + 2 * c])) return false;
          pos += 2 + 2 * cnt; break;
        case OP_LI_DEL: case OP_LI_ADD:
          if (pos + 1 >= len || arg >= m->ngroups || !coord_ok(prog[pos + 1])) return false;
          pos += 2; break;
        case OP_STRIP:
          if (pos + 1 >= len || !coord_ok(prog[pos + 1])) return false;
          pos += 2; break;
        default: return false;
      }
    }
    return false;
  };
  for (int i = 0; i < m->P; i++)
    if (!walk(prog[m->off_proc + i])) return fail(KMC_ERR_PROGRAM, "malformed op stream of process " + std::to_string(i + 1));
  for (int i = 0; i < nt; i++)
    if (!walk(prog[m->off_touch + i])) return fail(KMC_ERR_PROGRAM, "malformed touch-up stream");
  if (m->off_site_layer < 0 || m->off_site_layer + m->spuck > len || m->off_site_default < 0 ||
      m->off_site_default + m->spuck > len)
    return fail(KMC_ERR_PROGRAM, "bad site tables");
  for (int n = 0; n < m->spuck; n++)
    if (!species_ok(prog[m->off_site_default + n])) return fail(KMC_ERR_PROGRAM, "bad default species");
  // hot section: fast streams with slot references below nlat, known edit kinds,
  // in-range processes / groups / species, table indices inside their tables, record
  // offsets inside the stream, 16-byte placement
  m->max_nedit = 0;
  m->off_hot = prog[21];
  m->hot_len = prog[20];
  m->hot_grp = prog[17];
  m->hot_tab = prog[18];
  m->reach_x = prog[19] & 0xFF; m->reach_y = (prog[19] >> 8) & 0xFF; m->reach_z = (prog[19] >> 16) & 0xFF;
  if (m->off_hot <= 0 || m->hot_len <= m->P || !span_ok(m->off_hot, m->hot_len, len)) {
    m->off_hot = 0;
  } else {
    const int32_t *hot = prog + m->off_hot;
    const int hl = m->hot_len, G = std::max(m->ngroups, 1);
    if (m->hot_grp < m->P + 1 || !span_ok(m->hot_grp, G, hl) || m->hot_tab < m->P + 1 || !span_ok(m->hot_tab, G, hl))
      return fail(KMC_ERR_PROGRAM, "bad hot-section tables");
    for (int g = 0; g < m->ngroups; g++) {
      const int off = hot[m->hot_grp + g];
      if (off <= 0 || !span_ok(off, 2, hl)) return fail(KMC_ERR_PROGRAM, "bad hot group record");
      const int M = hot[off], K = hot[off + 1];
      if (K > KMC_MAXK || K < 0 || M < 0 || !span_ok(off, 2 + K + (int64_t)M * (1 + K), hl))
        return fail(KMC_ERR_PROGRAM, "bad hot group record");
      for (int mm = 0; mm < M; mm++) {
        const int pid = hot[off + 2 + K + mm * (1 + K)];
        if (pid < 1 || pid > m->P) return fail(KMC_ERR_PROGRAM, "bad group member");
      }
      const int toff = hot[m->hot_tab + g];
      if (toff) {
        int64_t size = 1;
        for (int k = 0; k < K; k++) size *= (m->nspecies + 1);
        if (!span_ok(toff, size, hl)) return fail(KMC_ERR_PROGRAM, "nli table overruns program");
        for (int64_t i = 0; i < size; i++)
          if (hot[toff + i] < 0 || hot[toff + i] > m->P) return fail(KMC_ERR_PROGRAM, "bad nli table entry");
      }
    }
    if (m->off_hot % 4) return fail(KMC_ERR_PROGRAM, "hot section not on 16 bytes");
    for (int i = 0; i < m->P; i++) {
      const int off = hot[i];
      if (off == 0) continue;
      if (off < m->P + 1 || !span_ok(off, 4, hl) || off % 4) return fail(KMC_ERR_PROGRAM, "bad fast stream offset");
      const int nlat = hot[off], nchk = hot[off + 1], nwr = hot[off + 2];
      const uint32_t w3 = (uint32_t)hot[off + 3];
      const int nedit = w3 & 0xFFFF, nq = (w3 >> 16) & 0xF, dels_first = (w3 >> 20) & 0xF;
      if (nlat < 0 || nlat > FAST_SLOTS || nchk < 0 || nchk > nlat || nwr < 0 || nwr > nlat || nedit < 0 ||
          nedit > FAST_EDITS || nq > 3 || dels_first > 1 || (w3 >> 24))
        return fail(KMC_ERR_PROGRAM, "fast stream exceeds the on-chip limits");
      m->max_nedit = std::max(m->max_nedit, nedit);
      const int rec = fast_rec_offset(nlat, nchk, nwr);
      const int64_t head = (int64_t)rec + 4 * (1 + nq) * (int64_t)nedit;
      if (off + head > hl) return fail(KMC_ERR_PROGRAM, "fast stream overruns program");
      for (int c = 0; c < nlat; c++) if (!coord_ok(hot[off + 4 + c])) return fail(KMC_ERR_PROGRAM, "bad fast slot");
      const int32_t *chk = hot + off + 4 + nlat, *wr = chk + 2 * nchk;
      for (int c = 0; c < nchk; c++) if (chk[2 * c] < 0 || chk[2 * c] >= nlat) return fail(KMC_ERR_PROGRAM, "bad check");
      for (int c = 0; c < nwr; c++)
        if (wr[2 * c] < 0 || wr[2 * c] >= nlat || !species_ok(wr[2 * c + 1])) return fail(KMC_ERR_PROGRAM, "bad write");
      auto ref_ok = [&](int32_t r) { return r >= 0 ? r < nlat : species_ok(-r - 2); };
      const int32_t *q = hot + off + rec;  // quad j of edit k at q + 4 * (j * nedit + k)
      if (dels_first) {
        // the flag promises every del-kind edit before every add-kind edit, and adds that
        // cannot name one (process, site) twice: distinct (proc or group, target) and
        // not both the plain and the nli form
        bool seen_add = false, plain[2] = {false, false}, nli[2] = {false, false};
        for (int k = 0; k < nedit; k++) {
          const int32_t *a = q + 4 * k;
          const int op = a[0] & 0xFF;
          const bool add = op == 3 || op == 5 || op == 7;
          if (add) seen_add = true;
          else if (seen_add) return fail(KMC_ERR_PROGRAM, "fast stream marked dels-first has a del after an add");
          ((op == 2 || op == 3) ? plain : nli)[add] = true;
          for (int k2 = 0; k2 < k; k2++) {
            const int32_t *b = q + 4 * k2;
            const int op2 = b[0] & 0xFF;
            if ((op2 == 3 || op2 == 5 || op2 == 7) == add && ((uint32_t)b[0] >> 16) == ((uint32_t)a[0] >> 16) &&
                b[1] == a[1])
              return fail(KMC_ERR_PROGRAM, "fast stream marked dels-first names one target twice");
          }
        }
        if ((plain[0] && nli[0]) || (plain[1] && nli[1]))
          return fail(KMC_ERR_PROGRAM, "fast stream marked dels-first mixes edit forms");
      }
      for (int k = 0; k < nedit; k++) {
        const int32_t *q0 = q + 4 * k;
        const uint32_t h = (uint32_t)q0[0];
        const int op = h & 0xFF, cnt = (h >> 8) & 0xFF, arg = (h >> 16) & 0xFFFF;
        if (q0[1] < 0 || q0[1] >= nlat) return fail(KMC_ERR_PROGRAM, "bad edit target");
        if (op == 6 || op == 7) {
          // every index the table form can produce lies inside the group's table: all
          // 4 * nq packed references are summed, unused ones must be 0
          if (arg >= m->ngroups || cnt > 4 * nq) return fail(KMC_ERR_PROGRAM, "bad nli table edit");
          const int toff = hot[m->hot_tab + arg];
          const int K = hot[hot[m->hot_grp + arg] + 1];
          int64_t size = 1;
          for (int kk = 0; kk < K; kk++) size *= (m->nspecies + 1);
          int64_t lo = q0[2], hi = q0[2];
          for (int c = 0; c < 4 * nq; c++) {
            const int32_t w = q[4 * ((1 + c / 4) * nedit + k) + c % 4];
            if (c >= cnt ? w != 0 : (w < 0 || (w & 0xFF) >= nlat)) return fail(KMC_ERR_PROGRAM, "bad nli table edit");
            hi += (int64_t)m->nspecies * (w >> 8);
          }
          if (toff <= 0 || lo < toff || hi >= toff + size) return fail(KMC_ERR_PROGRAM, "nli table edit outside its table");
          continue;
        }
        if (op == 2) {
          if (arg < 1 || arg > m->P) return fail(KMC_ERR_PROGRAM, "bad edit process");
          continue;
        }
        if (op == 3 && cnt <= 1) {  // inline condition
          if (arg < 1 || arg > m->P || q0[2] < 0 || q0[2] >= nlat || (cnt == 0 && (q0[2] | q0[3])))
            return fail(KMC_ERR_PROGRAM, "bad add edit");
          continue;
        }
        // ops 3, 4, 5 keep their whole record in the stream's variable part
        const int64_t e = (int64_t)off + q0[2];
        if (q0[2] < head || e + 2 > hl || hot[e] != q0[0] || hot[e + 1] != q0[1])
          return fail(KMC_ERR_PROGRAM, "bad edit offset");
        if (op == 3) {
          if (arg < 1 || arg > m->P || e + 2 + 2 * cnt > hl) return fail(KMC_ERR_PROGRAM, "bad add edit");
          for (int c = 0; c < cnt; c++) if (!ref_ok(hot[e + 2 + c])) return fail(KMC_ERR_PROGRAM, "bad add ref");
        } else if (op == 4 || op == 5) {
          if (arg >= m->ngroups || e + 4 + cnt > hl || cnt != hot[hot[m->hot_grp + arg] + 1] ||
              hot[e + 2] != 0 || hot[e + 3] != hot[m->hot_grp + arg])
            return fail(KMC_ERR_PROGRAM, "bad nli edit");
          for (int c = 0; c < cnt; c++) if (!ref_ok(hot[e + 4 + c])) return fail(KMC_ERR_PROGRAM, "bad nli ref");
        } else {
          return fail(KMC_ERR_PROGRAM, "bad edit kind");
        }
      }
    }
  }
  m->max_k = 0;
  for (int g = 0; g < m->ngroups; g++) {
    const int off = prog[m->off_groups + g];
    if (off <= 0 || !span_ok(off, 2, len)) return fail(KMC_ERR_PROGRAM, "bad group offset");
    const int M = prog[off], K = prog[off + 1];
    if (K > KMC_MAXK) return fail(KMC_ERR_PROGRAM, "lateral-interaction group tests more than 16 sites");
    if (K < 0 || M < 0 || !span_ok(off, 2 + K + (int64_t)M * (1 + K), len))
      return fail(KMC_ERR_PROGRAM, "group record overruns program");
    for (int k = 0; k < K; k++)
      if (!coord_ok(prog[off + 2 + k])) return fail(KMC_ERR_PROGRAM, "bad group coordinate");
    for (int mm = 0; mm < M; mm++) {
      const int pid = prog[off + 2 + K + mm * (1 + K)];
      if (pid < 1 || pid > m->P) return fail(KMC_ERR_PROGRAM, "bad group member");
    }

    m->max_k = std::max(m->max_k, K);
  }
  return KMC_OK;
}

constexpr int STAGE_MAX_WORDS = 16384;  // hot sections up to 64 KB go to shared memory

// One launch of the run kernel: every listed slot runs `model`.
struct LaunchPlan {
  int model, first, count, blocks, threads, np, rounds, g;
  const void *fn;  // host stub of the kernel variant
  size_t smem;
  RunArgs a;
};

// Shared memory of one trajectory group of the (np, r, g) variant.
template <int NP, int R, int G>
constexpr size_t wsz() { return sizeof(WarpSmem<NP, R, G>); }
size_t warp_smem_bytes(int np, int r, int g) {
  switch (g * 1000 + np * 10 + r) {
    case 32013: return wsz<1, 3, 32>();
    case 32014: return wsz<1, 4, 32>();
    case 32023: return wsz<2, 3, 32>();
    case 32024: return wsz<2, 4, 32>();
    case 32043: return wsz<4, 3, 32>();
    case 32083: return wsz<8, 3, 32>();
    case 16013: return wsz<1, 3, 16>();
    case 16014: return wsz<1, 4, 16>();
    case 16023: return wsz<2, 3, 16>();
    case 16024: return wsz<2, 4, 16>();
    case 16043: return wsz<4, 3, 16>();
    case 16044: return wsz<4, 4, 16>();
    default: return 0;
  }
}

const void *run_kernel_g32(int np, int r) {
  switch (np * 10 + r) {
    case 13: return (const void *)kmc_run_kernel<1, 3, 32>;
    case 14: return (const void *)kmc_run_kernel<1, 4, 32>;
    case 23: return (const void *)kmc_run_kernel<2, 3, 32>;
    case 24: return (const void *)kmc_run_kernel<2, 4, 32>;
    case 43: return (const void *)kmc_run_kernel<4, 3, 32>;
    case 83: return (const void *)kmc_run_kernel<8, 3, 32>;
    default: return nullptr;
  }
}

// Launch shape of one model's launch with kernel variant (np, r, g).  ts_max: the
// largest ts_need of its trajectories; their lattice and tables go to shared memory when
// the pool allows it and every trajectory of the launch then still runs in one round.
int plan_kernel(kmc_pool *p, LaunchPlan &L, size_t hot_bytes, int np, int r, int g, size_t ts_max) {
  L.np = np;
  L.rounds = r;
  L.g = g;
  L.fn = g == 16 ? run_kernel_g16(np, r) : run_kernel_g32(np, r);
  const size_t wsm = warp_smem_bytes(np, r, g);
  if (!L.fn || !wsm) return fail(KMC_ERR_ARG, "no step kernel for this model and launch mode");
  // The attribute is a per-function cap shared by every plan (and pool) on the device:
  // raise it to the device's limit once rather than to this plan's size, which would
  // lower it under a plan made before this one.
  cudaFuncAttributes fa;
  CK(cudaFuncGetAttributes(&fa, L.fn));
  int optin = 0;
  CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device));
  const int64_t cap = optin - (int64_t)fa.sharedSizeBytes;
  if (fa.maxDynamicSharedSizeBytes < cap)
    CK(cudaFuncSetAttribute(L.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap));
  const int gpw = 32 / g;  // trajectory groups per warp
  const size_t ts = p->tables_on_chip ? align_up(ts_max, 16) : 0;
  auto smem_for = [&](int warps, bool on_chip) {
    return hot_bytes + (wsm + (on_chip ? ts : 0)) * (size_t)warps * gpw;
  };
  auto occupancy = [&](int warps, bool on_chip, int *nb) -> int {
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(nb, L.fn, 32 * warps, smem_for(warps, on_chip)));
    return KMC_OK;
  };
  if (p->warps_per_block > 0) {
    const int wpb = p->warps_per_block;
    const int gpb = wpb * gpw;
    L.threads = 32 * wpb;
    bool on_chip = false;
    int bps = 0;
    if (ts > 0 && (int64_t)smem_for(wpb, true) <= cap) {
      if (int rc_ = occupancy(wpb, true, &bps)) return rc_;
      if (p->blocks_per_sm > 0) bps = std::min(bps, p->blocks_per_sm);
      on_chip = bps >= 1 && (int64_t)L.count <= (int64_t)p->num_sms * bps * gpb;
    }
    if (!on_chip) {
      if ((int64_t)smem_for(wpb, false) > cap)
        return fail(KMC_ERR_ARG, "model's shared-memory section too large for one block");
      bps = p->blocks_per_sm;
      if (bps <= 0) { if (int rc_ = occupancy(wpb, false, &bps)) return rc_; }
    }
    if (bps <= 0) return fail(KMC_ERR_CUDA, "run kernel does not fit on an SM with this launch shape");
    L.smem = smem_for(wpb, on_chip);
    L.a.groups = gpb;
    L.a.ts_bytes = on_chip ? (int32_t)ts : 0;
    L.blocks = std::max(1, std::min((L.count + gpb - 1) / gpb, p->num_sms * bps));
    return KMC_OK;
  }
  // balanced: one block per SM, as many warps per block as fit (registers: 16 at 128
  // per thread; shared memory), and the fewest rounds of items per group with the
  // groups split evenly over the SMs
  const int regs = std::max(1, fa.numRegs);
  auto fit_warps = [&](bool on_chip, int *out) -> int {
    int maxw = std::min(16, 65536 / (regs * 32));
    const int64_t per_warp = (int64_t)(wsm + (on_chip ? ts : 0)) * gpw;
    maxw = (int)std::min<int64_t>(maxw, (cap - (int64_t)hot_bytes) / per_warp);
    // the occupancy calculator has the last word (register allocation granularity)
    while (maxw >= 1) {
      int nb = 0;
      if (int rc_ = occupancy(maxw, on_chip, &nb)) return rc_;
      if (nb >= 1) break;
      maxw--;
    }
    *out = maxw;
    return KMC_OK;
  };
  const int blocks = std::max(1, std::min(p->num_sms, (L.count + gpw - 1) / gpw));
  int maxw = 0;
  bool on_chip = false;
  if (ts > 0) {
    if (int rc_ = fit_warps(true, &maxw)) return rc_;
    on_chip = maxw >= 1 && (int64_t)L.count <= (int64_t)blocks * maxw * gpw;
  }
  if (!on_chip) { if (int rc_ = fit_warps(false, &maxw)) return rc_; }
  if (maxw < 1) return fail(KMC_ERR_ARG, "model's shared-memory section too large for one block");
  const int rounds = (L.count + blocks * maxw * gpw - 1) / (blocks * maxw * gpw);
  const int groups = (L.count + rounds - 1) / rounds;
  const int warps = (groups + gpw - 1) / gpw;
  const int wpb = std::min(maxw, (warps + blocks - 1) / blocks);
  L.threads = 32 * wpb;
  L.smem = smem_for(wpb, on_chip);
  L.blocks = blocks;
  L.a.groups = wpb * gpw;
  L.a.ts_bytes = on_chip ? (int32_t)ts : 0;
  return KMC_OK;
}

// The solo kernel: one block of one warp per trajectory, the program and (when they fit)
// the lattice and tables in shared memory.
int plan_solo(kmc_pool *p, LaunchPlan &L, size_t ts_max) {
  L.np = 1;
  L.rounds = 0;
  L.g = 32;
  // the variant is chosen below, once the placement is known; none has static shared
  // memory, so any of them gives the dynamic limit
  cudaFuncAttributes fa;
  CK(cudaFuncGetAttributes(&fa, solo_kernel(1, false)));
  int optin = 0;
  CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device));
  const int64_t cap = optin - (int64_t)fa.sharedSizeBytes;
  const ModelHost &mh = p->models[L.model];
  const size_t prog_b = align_up((size_t)mh.dev.len * 4, 16);
  const size_t ts = p->tables_on_chip ? align_up(ts_max, 16) : 0;
  size_t smem = sizeof(SoloSmem);
  L.a.prog_words = 0;
  L.a.ts_bytes = 0;
  if ((int64_t)(smem + prog_b) <= cap) { smem += prog_b; L.a.prog_words = mh.dev.len; }
  if (ts > 0 && (int64_t)(smem + ts) <= cap) { smem += ts; L.a.ts_bytes = (int32_t)ts; }
  // on chip: the program and every trajectory's lattice and tables (ts covers the largest)
  const bool onchip = L.a.prog_words > 0 && L.a.ts_bytes > 0;
  L.fn = solo_kernel(mh.dev.P, onchip);
  if (!L.fn) return fail(KMC_ERR_ARG, "solo kernel: more processes than it is built for");
  // raise the chosen variant's dynamic shared-memory limit to the device's
  CK(cudaFuncGetAttributes(&fa, L.fn));
  if (fa.maxDynamicSharedSizeBytes < cap)
    CK(cudaFuncSetAttribute(L.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap));
  L.a.groups = 1;
  L.threads = 32;
  L.blocks = L.count;
  L.smem = smem;
  return KMC_OK;
}

int ensure_aux(kmc_pool *p, size_t n);

// Sorts the run list by model (stable) into ls / st and plans one launch per model.
int plan_run(kmc_pool *p, const int32_t *slots, const int64_t *steps, int n, std::vector<int32_t> &ls,
             std::vector<int64_t> &st, std::vector<LaunchPlan> &plans) {
  std::vector<int32_t> order(n);
  for (int i = 0; i < n; i++) order[i] = i;
  // by model, then longest first (steps, then lattice size), so that the kernel's strided
  // first assignment spreads the long trajectories over the blocks
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    const SlotDev &a = p->slots[slots[x]].dev, &b = p->slots[slots[y]].dev;
    if (a.model != b.model) return a.model < b.model;
    if (steps[x] != steps[y]) return steps[x] > steps[y];
    return a.V > b.V;
  });
  ls.resize(n);
  st.resize(n);
  for (int i = 0; i < n; i++) { ls[i] = slots[order[i]]; st[i] = steps[order[i]]; }
  plans.clear();
  int i = 0;
  while (i < n) {
    const int model = p->slots[ls[i]].dev.model;
    int j = i;
    while (j < n && p->slots[ls[j]].dev.model == model) j++;
    LaunchPlan L;
    L.model = model;
    L.first = i;
    L.count = j - i;
    const ModelDev &md = p->models[model].dev;
    RunArgs &a = L.a;
    a.slots = p->d_slots;
    a.models = p->d_models;
    a.n = L.count;
    a.counter = p->d_counter + plans.size();
    a.cancel = p->d_cancel;
    a.fast = p->fast_path;
    a.model = model;
    a.stage_words = (p->stage_hot && md.off_hot && md.hot_len <= STAGE_MAX_WORDS) ? md.hot_len : 0;
    a.prog_words = 0;
    a.phase = p->d_phase;
    const size_t hot_bytes = ((size_t)a.stage_words * 4 + 15) / 16 * 16;
    // fast streams of more than 96 edits run in the 4-round kernel (built for up to 64
    // processes); a larger model with such streams takes the serial interpreter
    const bool big = md.max_nedit > 96;
    if (big && md.P > 64) a.fast = 0;
    // two trajectories per warp (16 lanes each) for models of up to 64 processes
    const int g = (p->traj_per_warp == 2 && md.P <= 64) ? 16 : 32;
    int np = 1;
    while (np * g < md.P) np *= 2;
    const int r = (big && md.P <= 64) ? 4 : 3;
    size_t ts_max = 0;
    for (int k = i; k < j; k++) {
      const SlotDev &d = p->slots[ls[k]].dev;
      ts_max = std::max(ts_max, ts_need(md.P, d.V));
    }
    int rc = (p->solo && md.P <= SOLO_PMAX && L.count <= p->num_sms) ? plan_solo(p, L, ts_max)
                                                                       : plan_kernel(p, L, hot_bytes, np, r, g, ts_max);
    if (rc) return rc;
    plans.push_back(L);
    i = j;
  }
  if ((int)plans.size() > p->max_models) return fail(KMC_ERR_ARG, "too many models in one run");
  return ensure_aux(p, plans.size());
}

// Issues the planned launches on the pool stream (capturable: no host copies).
// Streams and events for n concurrent per-model launches (created outside any capture).
int ensure_aux(kmc_pool *p, size_t n) {
  if (n > 1 && !p->fork_ev) CK(cudaEventCreateWithFlags(&p->fork_ev, cudaEventDisableTiming));
  while (n > 1 && p->aux.size() < n) {
    cudaStream_t st;
    cudaEvent_t ev;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    p->aux.push_back(st);
    p->aux_ev.push_back(ev);
  }
  return KMC_OK;
}

int issue_run(kmc_pool *p, std::vector<LaunchPlan> &plans, const int32_t *d_list, const int64_t *d_steps,
              int32_t *d_trace) {
  CK(cudaMemsetAsync(p->d_counter, 0, sizeof(int32_t) * plans.size(), p->stream));
  const bool fork = plans.size() > 1 && p->aux.size() >= plans.size();
  if (fork) CK(cudaEventRecord(p->fork_ev, p->stream));
  for (size_t i = 0; i < plans.size(); i++) {
    LaunchPlan &L = plans[i];
    L.a.list = d_list + L.first;
    L.a.steps = d_steps + L.first;
    L.a.trace = d_trace;
    cudaStream_t st = p->stream;
    if (fork) {
      st = p->aux[i];
      CK(cudaStreamWaitEvent(st, p->fork_ev, 0));
    }
    void *args[] = {&L.a};
    CK(cudaLaunchKernel(L.fn, dim3(L.blocks), dim3(L.threads), args, L.smem, st));
    CK(cudaGetLastError());
    p->launches++;
    if (fork) CK(cudaEventRecord(p->aux_ev[i], st));
  }
  if (fork)
    for (size_t i = 0; i < plans.size(); i++) CK(cudaStreamWaitEvent(p->stream, p->aux_ev[i], 0));
  return KMC_OK;
}

// Plans, copies the sorted list to d_list / d_steps and issues the launches.
int launch_run(kmc_pool *p, const int32_t *slots, const int64_t *steps, int n, int32_t *d_list, int64_t *d_steps,
               int32_t *d_trace) {
  std::vector<int32_t> ls;
  std::vector<int64_t> st;
  std::vector<LaunchPlan> plans;
  int rc = plan_run(p, slots, steps, n, ls, st, plans);
  if (rc) return rc;
  // pageable sources: the copies have read them when cudaMemcpyAsync returns
  CK(cudaMemcpyAsync(d_list, ls.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, p->stream));
  CK(cudaMemcpyAsync(d_steps, st.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, p->stream));
  return issue_run(p, plans, d_list, d_steps, d_trace);
}

int run_rounds(kmc_pool *p, const int32_t *slots, const int64_t *steps, int n, int rounds,
               const std::function<int(int)> &after) {
  std::vector<int32_t> ls;
  std::vector<int64_t> st;
  std::vector<LaunchPlan> plans;
  int rc = plan_run(p, slots, steps, n, ls, st, plans);
  if (rc) return rc;
  CK(cudaMemcpyAsync(p->d_list, ls.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, p->stream));
  CK(cudaMemcpyAsync(p->d_steps, st.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, p->stream));
  *p->h_cancel = 0;
  for (int r = 0; r < rounds; r++) {
    rc = issue_run(p, plans, p->d_list, p->d_steps, nullptr);
    if (rc) return rc;
    rc = after(r);
    if (rc) return rc;
  }
  return KMC_OK;
}

// Every slot of a run list admitted, and none listed twice (two warps would step one
// trajectory at once).
int check_run_list(kmc_pool *p, const int32_t *slots, int n) {
  std::vector<char> seen(p->slots.size(), 0);
  for (int i = 0; i < n; i++) {
    int rc = check_slot(p, slots[i]);
    if (rc) return rc;
    if (seen[slots[i]]) return fail(KMC_ERR_ARG, "slot listed twice in one run");
    seen[slots[i]] = 1;
  }
  return KMC_OK;
}

void clear_graphs(kmc_pool *p) {
  if (p->graphs.empty()) return;
  cudaStreamSynchronize(p->stream);  // no captured launch may still be running
  for (auto &kv : p->graphs) {
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
    cudaFree(kv.second.d_list);
    cudaFree(kv.second.d_steps);
  }
  p->graphs.clear();
}

int read_slot(kmc_pool *p, int slot, SlotDev *out) {
  CK(cudaStreamSynchronize(p->stream));
  CK(cudaMemcpy(out, p->d_slots + slot, sizeof(SlotDev), cudaMemcpyDeviceToHost));
  return KMC_OK;
}

int check_slot(kmc_pool *p, int slot) {
  if (!p || slot < 0 || slot >= (int)p->slots.size() || !p->slots[slot].used) return fail(KMC_ERR_ARG, "bad slot");
  return KMC_OK;
}

// Occupation rows of `stride` counters: every listed slot admitted and its model's
// nspecies * spuck counters fitting in one row (get_occupation's (0:nspecies-1, 1:spuck)
// matrix, proclist_generic_subroutines.mpy:113-158).
int check_occupation_list(kmc_pool *p, const int32_t *slots, int n, int stride) {
  for (int i = 0; i < n; i++) {
    int rc = check_slot(p, slots[i]);
    if (rc) return rc;
    const ModelDev &m = p->models[p->slots[slots[i]].dev.model].dev;
    if (stride < m.nspecies * m.spuck)
      return fail(KMC_ERR_ARG, "occupation stride " + std::to_string(stride) + " below nspecies * spuck = " +
                                   std::to_string(m.nspecies * m.spuck) + " of slot " + std::to_string(slots[i]));
  }
  return KMC_OK;
}

int run_command(kmc_pool *p, int slot, int cmd, int a0, int a1, int a2, int32_t *proc, int32_t *site,
                const int32_t *d_list) {
  CmdArgs c;
  c.slots = p->d_slots; c.models = p->d_models; c.slot = slot; c.cmd = cmd;
  c.a0 = a0; c.a1 = a1; c.a2 = a2; c.list = d_list; c.out = p->d_cmd_out;
  kmc_command_kernel<<<1, 32, 0, p->stream>>>(c);
  CK(cudaGetLastError());
  p->launches++;
  int32_t out[3];
  CK(cudaMemcpyAsync(out, p->d_cmd_out, sizeof(out), cudaMemcpyDeviceToHost, p->stream));
  CK(cudaStreamSynchronize(p->stream));
  if (proc) *proc = out[1];
  if (site) *site = out[2];
  if (out[0]) return fail(out[0], "command failed with status " + std::to_string(out[0]));
  return KMC_OK;
}

}  // namespace kmc_host

// ===================================================================== C-ABI
extern "C" {

const char *kmc_last_error(void) { return g_err.c_str(); }
const char *kmc_version(void) { return "kmc_gb300 1.0 (sm_103a)"; }

int kmc_check_program(const int32_t *program, int32_t program_len) {
  ModelDev md{};
  return validate_program(program, program_len, &md);
}

int kmc_pool_create(int32_t device, size_t arena_bytes, int32_t max_slots, kmc_pool **out) {
  if (!out || max_slots < 1) return fail(KMC_ERR_ARG, "bad arguments");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(KMC_ERR_NODEVICE, "no CUDA device");
  if (device < 0 || device >= ndev) return fail(KMC_ERR_ARG, "bad device");
  CK(cudaSetDevice(device));
  kmc_pool *p = new kmc_pool();
  p->device = device;
  CK(cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, device));
  CK(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
  arena_bytes = align_up(std::max<size_t>(arena_bytes, 256), 256);
  CK(cudaMalloc(&p->arena, arena_bytes));
  p->arena_bytes = arena_bytes;
  p->free_blocks[0] = arena_bytes;
  p->slots.resize(max_slots);
  CK(cudaMalloc(&p->d_slots, sizeof(SlotDev) * max_slots));
  CK(cudaMemset(p->d_slots, 0, sizeof(SlotDev) * max_slots));
  CK(cudaMalloc(&p->d_models, sizeof(ModelDev) * p->max_models));
  CK(cudaMalloc(&p->d_list, sizeof(int32_t) * max_slots));
  CK(cudaMalloc(&p->d_steps, sizeof(int64_t) * max_slots));
  CK(cudaMalloc(&p->d_counter, sizeof(int32_t) * p->max_models));
  CK(cudaMalloc(&p->d_cmd_out, sizeof(int32_t) * 4));
  CK(cudaMalloc(&p->d_phase, sizeof(unsigned long long) * KMC_NPHASE));
  CK(cudaMemset(p->d_phase, 0, sizeof(unsigned long long) * KMC_NPHASE));
  CK(cudaHostAlloc(&p->h_cancel, sizeof(int32_t), cudaHostAllocMapped));
  *p->h_cancel = 0;
  CK(cudaHostGetDevicePointer(&p->d_cancel, p->h_cancel, 0));
  CK(cudaMalloc(&p->d_adm_list, sizeof(int32_t) * max_slots));
  CK(cudaMalloc(&p->d_adm_staged, sizeof(SlotDev) * max_slots));
  CK(cudaMalloc(&p->d_adm_roff, sizeof(int32_t) * max_slots));
  CK(cudaEventCreate(&p->ev0));
  CK(cudaEventCreate(&p->ev1));
  CK(cudaEventCreate(&p->tev0));
  CK(cudaEventCreate(&p->tev1));
  *out = p;
  return KMC_OK;
}

int kmc_pool_destroy(kmc_pool *p) {
  if (!p) return KMC_OK;
  cudaSetDevice(p->device);
  cudaStreamSynchronize(p->stream);
  for (auto &kv : p->graphs) {
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
    cudaFree(kv.second.d_list);
    cudaFree(kv.second.d_steps);
  }
  for (auto &m : p->models) cudaFree(m.d_prog);
  cudaFree(p->arena); cudaFree(p->d_slots); cudaFree(p->d_models); cudaFree(p->d_list);
  cudaFree(p->d_steps); cudaFree(p->d_counter); cudaFree(p->d_cmd_out); cudaFreeHost(p->h_cancel);
  cudaFree(p->d_res); cudaFreeHost(p->h_res); cudaFree(p->d_phase);
  cudaFree(p->d_adm_list); cudaFree(p->d_adm_staged); cudaFree(p->d_adm_rates); cudaFree(p->d_adm_roff);
  cudaEventDestroy(p->ev0); cudaEventDestroy(p->ev1); cudaEventDestroy(p->tev0); cudaEventDestroy(p->tev1);
  for (size_t i = 0; i < p->aux.size(); i++) {
    cudaStreamDestroy(p->aux[i]);
    cudaEventDestroy(p->aux_ev[i]);
  }
  if (p->fork_ev) cudaEventDestroy(p->fork_ev);
  cudaStreamDestroy(p->stream);
  delete p;
  return KMC_OK;
}

int kmc_pool_add_model(kmc_pool *p, const int32_t *program, int32_t len, int32_t *model_id) {
  if (!p || !model_id) return fail(KMC_ERR_ARG, "bad arguments");
  if ((int)p->models.size() >= p->max_models) return fail(KMC_ERR_ARG, "too many models");
  ModelHost m;
  int rc = validate_program(program, len, &m.dev);
  if (rc) return rc;
  m.prog.assign(program, program + len);
  CK(cudaSetDevice(p->device));
  CK(cudaMalloc(&m.d_prog, sizeof(int32_t) * len));
  CK(cudaMemcpy(m.d_prog, program, sizeof(int32_t) * len, cudaMemcpyHostToDevice));
  m.dev.prog = m.d_prog;
  const int id = (int)p->models.size();
  CK(cudaMemcpy(p->d_models + id, &m.dev, sizeof(ModelDev), cudaMemcpyHostToDevice));
  p->models.push_back(std::move(m));
  *model_id = id;
  return KMC_OK;
}

int kmc_pool_slot_bytes(kmc_pool *p, int32_t model_id, const int32_t dims[3], size_t *bytes) {
  if (!p || model_id < 0 || model_id >= (int)p->models.size() || !dims || !bytes) return fail(KMC_ERR_ARG, "bad arguments");
  const int V = dims[0] * dims[1] * dims[2] * p->models[model_id].dev.spuck;
  *bytes = align_up(slot_layout(p->models[model_id].dev.P, V).total, 256);
  return KMC_OK;
}

int kmc_pool_free_bytes(kmc_pool *p, size_t *total, size_t *largest) {
  if (!p) return fail(KMC_ERR_ARG, "bad pool");
  size_t t = 0, l = 0;
  for (auto &kv : p->free_blocks) { t += kv.second; l = std::max(l, kv.second); }
  if (total) *total = t;
  if (largest) *largest = l;
  return KMC_OK;
}

int kmc_pool_admit_many(kmc_pool *p, int32_t n, const int32_t *model_ids, const int32_t *dims3, int32_t layer,
                        const int32_t *seeds, int32_t rng_kind, const uint32_t *traj_ids, const double *rates,
                        const int32_t *rate_offsets, int32_t *slots_out) {
  if (!p || n < 1 || !model_ids || !dims3 || !seeds || !rates || !rate_offsets || !slots_out)
    return fail(KMC_ERR_ARG, "bad arguments");
  if (rng_kind != RNG_GFORTRAN && rng_kind != RNG_PHILOX) return fail(KMC_ERR_ARG, "bad rng kind");
  std::lock_guard<std::mutex> lock(p->mu);
  CK(cudaSetDevice(p->device));
  std::vector<int32_t> got;
  std::vector<SlotDev> staged;
  size_t nrates = 0;
  for (int i = 0; i < n; i++) {
    const int mid = model_ids[i];
    if (mid < 0 || mid >= (int)p->models.size()) return fail(KMC_ERR_ARG, "bad model id");
    if (rate_offsets[i] < 0) return fail(KMC_ERR_ARG, "negative rate offset");
    nrates = std::max(nrates, (size_t)rate_offsets[i] + p->models[mid].dev.P);
  }
  int rc = KMC_OK;
  for (int i = 0; i < n && rc == KMC_OK; i++) {
    const ModelDev &m = p->models[model_ids[i]].dev;
    const int X = dims3[3 * i], Y = dims3[3 * i + 1], Z = dims3[3 * i + 2];
    if (X < 1 || Y < 1 || Z < 1 || (int64_t)X * Y * Z * m.spuck > (1 << 28)) { rc = fail(KMC_ERR_ARG, "bad system size"); break; }
    const int V = X * Y * Z * m.spuck;
    int slot = -1;
    for (int s = 0; s < (int)p->slots.size(); s++)
      if (!p->slots[s].used) { slot = s; break; }
    if (slot < 0) { rc = fail(KMC_ERR_NOMEM, "no free trajectory slot"); break; }
    const Layout L = slot_layout(m.P, V);
    size_t off;
    rc = alloc_block(p, L.total, &off);
    if (rc) break;
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
    d.X = X; d.Y = Y; d.Z = Z; d.V = V;
    d.model = model_ids[i]; d.P = m.P; d.layer = layer; d.status = ST_OK;
    d.rng_kind = rng_kind; d.seed = (uint32_t)seeds[i]; d.traj = traj_ids ? traj_ids[i] : (uint32_t)i;
    p->slots[slot].used = true;
    p->slots[slot].off = off;
    p->slots[slot].bytes = L.total;
    p->slots[slot].dev = d;
    // tables start at zero
    CK(cudaMemsetAsync(base + L.as1, 0, L.rates - L.as1, p->stream));
    got.push_back(slot);
    staged.push_back(d);
  }
  if (rc) {
    for (int s : got) { free_block(p, p->slots[s].off, p->slots[s].bytes); p->slots[s].used = false; }
    return rc;
  }
  if (nrates > p->adm_rates_cap) {
    cudaFree(p->d_adm_rates);
    CK(cudaMalloc(&p->d_adm_rates, sizeof(double) * nrates));
    p->adm_rates_cap = nrates;
  }
  CK(cudaMemcpyAsync(p->d_adm_list, got.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, p->stream));
  CK(cudaMemcpyAsync(p->d_adm_staged, staged.data(), sizeof(SlotDev) * n, cudaMemcpyHostToDevice, p->stream));
  CK(cudaMemcpyAsync(p->d_adm_rates, rates, sizeof(double) * nrates, cudaMemcpyHostToDevice, p->stream));
  CK(cudaMemcpyAsync(p->d_adm_roff, rate_offsets, sizeof(int32_t) * n, cudaMemcpyHostToDevice, p->stream));
  InitArgs a;
  a.slots = p->d_slots; a.models = p->d_models; a.staged = p->d_adm_staged; a.list = p->d_adm_list;
  a.rates = p->d_adm_rates; a.rate_off = p->d_adm_roff; a.n = n;
  const int threads = 256;
  const int blocks = (n * 32 + threads - 1) / threads;
  kmc_init_kernel<<<blocks, threads, 0, p->stream>>>(a);
  CK(cudaGetLastError());
  p->launches++;
  // the staging buffers are reused by the next admission: wait for this one
  CK(cudaStreamSynchronize(p->stream));
  for (int i = 0; i < n; i++) slots_out[i] = got[i];
  return KMC_OK;
}

int kmc_pool_admit(kmc_pool *p, int32_t model_id, const int32_t dims[3], int32_t layer, int32_t seed,
                   int32_t rng_kind, uint32_t traj_id, const double *rates, int32_t *slot) {
  const int32_t roff = 0;
  return kmc_pool_admit_many(p, 1, &model_id, dims, layer, &seed, rng_kind, &traj_id, rates, &roff, slot);
}

int kmc_pool_release(kmc_pool *p, int32_t slot) {
  int rc = check_slot(p, slot);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(p->mu);
  CK(cudaStreamSynchronize(p->stream));
  free_block(p, p->slots[slot].off, p->slots[slot].bytes);
  if (p->slots[slot].samp_bytes) free_block(p, p->slots[slot].samp_off, p->slots[slot].samp_bytes);
  p->slots[slot] = SlotHost();
  return KMC_OK;
}

int kmc_pool_run(kmc_pool *p, const int32_t *slots, const int64_t *steps, int32_t n) {
  if (!p || n < 0 || (n && (!slots || !steps))) return fail(KMC_ERR_ARG, "bad arguments");
  if (n == 0) return KMC_OK;
  if (n > (int)p->slots.size()) return fail(KMC_ERR_ARG, "too many slots");
  int rc = check_run_list(p, slots, n);
  if (rc) return rc;
  for (int i = 0; i < n; i++)
    if (steps[i] < 0) return fail(KMC_ERR_ARG, "negative step count");
  CK(cudaSetDevice(p->device));
  *p->h_cancel = 0;
  CK(cudaEventRecord(p->ev0, p->stream));
  rc = launch_run(p, slots, steps, n, p->d_list, p->d_steps, nullptr);
  CK(cudaEventRecord(p->ev1, p->stream));
  p->timed = true;
  return rc;
}

int kmc_pool_run_graph(kmc_pool *p, const int32_t *slots, int64_t steps, int32_t n) {
  if (!p || n < 1 || !slots || steps < 0) return fail(KMC_ERR_ARG, "bad arguments");
  if (n > (int)p->slots.size()) return fail(KMC_ERR_ARG, "too many slots");
  int rc0 = check_run_list(p, slots, n);
  if (rc0) return rc0;
  CK(cudaSetDevice(p->device));
  GraphKey key{steps, std::vector<int32_t>(slots, slots + n)};
  auto it = p->graphs.find(key);
  if (it == p->graphs.end() && p->graphs.size() >= 64) {
    // bounded cache: drop every captured graph when a 65th run list arrives
    CK(cudaStreamSynchronize(p->stream));
    clear_graphs(p);
  }
  if (it == p->graphs.end()) {
    GraphEntry e;
    CK(cudaMalloc(&e.d_list, sizeof(int32_t) * n));
    CK(cudaMalloc(&e.d_steps, sizeof(int64_t) * n));
    std::vector<int64_t> st0(n, steps), st;
    std::vector<int32_t> ls;
    std::vector<LaunchPlan> plans;
    // sort, set kernel attributes and query occupancy outside the capture
    int rc = plan_run(p, slots, st0.data(), n, ls, st, plans);
    if (rc) return rc;
    CK(cudaMemcpy(e.d_list, ls.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(e.d_steps, st.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice));
    CK(cudaStreamSynchronize(p->stream));
    CK(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
    const int64_t before = p->launches;
    rc = issue_run(p, plans, e.d_list, e.d_steps, nullptr);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(p->stream, &g);
    e.nlaunch = p->launches - before;
    p->launches = before;
    if (rc) return rc;
    if (ce != cudaSuccess) return fail(KMC_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
    e.graph = g;
    CK(cudaGraphInstantiate(&e.exec, g, 0));
    it = p->graphs.emplace(key, e).first;
  }
  *p->h_cancel = 0;
  CK(cudaEventRecord(p->ev0, p->stream));
  CK(cudaGraphLaunch(it->second.exec, p->stream));
  CK(cudaEventRecord(p->ev1, p->stream));
  p->timed = true;
  p->launches += it->second.nlaunch;
  return KMC_OK;
}

int kmc_pool_sync(kmc_pool *p) {
  if (!p) return fail(KMC_ERR_ARG, "bad pool");
  CK(cudaStreamSynchronize(p->stream));
  return KMC_OK;
}

int kmc_pool_cancel(kmc_pool *p) {
  if (!p) return fail(KMC_ERR_ARG, "bad pool");
  *(volatile int32_t *)p->h_cancel = 1;
  return KMC_OK;
}

int kmc_pool_last_kernel_ms(kmc_pool *p, float *ms) {
  if (!p || !ms || !p->timed) return fail(KMC_ERR_ARG, "no timed launch");
  CK(cudaEventSynchronize(p->ev1));
  CK(cudaEventElapsedTime(ms, p->ev0, p->ev1));
  return KMC_OK;
}

int kmc_pool_timer_start(kmc_pool *p) {
  if (!p) return fail(KMC_ERR_ARG, "bad pool");
  CK(cudaEventRecord(p->tev0, p->stream));
  return KMC_OK;
}

int kmc_pool_timer_stop(kmc_pool *p, float *ms) {
  if (!p || !ms) return fail(KMC_ERR_ARG, "bad arguments");
  CK(cudaEventRecord(p->tev1, p->stream));
  CK(cudaEventSynchronize(p->tev1));
  CK(cudaEventElapsedTime(ms, p->tev0, p->tev1));
  return KMC_OK;
}

int kmc_pool_phase_cycles(kmc_pool *p, uint64_t *out, int32_t reset) {
  if (!p || !out) return fail(KMC_ERR_ARG, "bad arguments");
  CK(cudaStreamSynchronize(p->stream));
  CK(cudaMemcpy(out, p->d_phase, sizeof(unsigned long long) * KMC_NPHASE, cudaMemcpyDeviceToHost));
  if (reset) CK(cudaMemset(p->d_phase, 0, sizeof(unsigned long long) * KMC_NPHASE));
#ifdef KMC_PHASE_TIMING
  return KMC_OK;
#else
  return fail(KMC_ERR_ARG, "library built without KMC_PHASE_TIMING");
#endif
}

int kmc_pool_launch_count(kmc_pool *p, int64_t *count) {
  if (!p || !count) return fail(KMC_ERR_ARG, "bad arguments");
  *count = p->launches;
  return KMC_OK;
}

int kmc_pool_set_launch(kmc_pool *p, int32_t warps_per_block, int32_t blocks_per_sm) {
  if (!p || warps_per_block < 0 || warps_per_block > 16 || blocks_per_sm < 0) return fail(KMC_ERR_ARG, "bad launch shape");
  p->warps_per_block = warps_per_block;
  p->blocks_per_sm = blocks_per_sm;
  clear_graphs(p);
  return KMC_OK;
}

int kmc_pool_set_trajectories_per_warp(kmc_pool *p, int32_t n) {
  if (!p || (n != 1 && n != 2)) return fail(KMC_ERR_ARG, "trajectories per warp must be 1 or 2");
  p->traj_per_warp = n;
  clear_graphs(p);
  return KMC_OK;
}

int kmc_pool_set_solo(kmc_pool *p, int32_t enable) {
  if (!p) return fail(KMC_ERR_ARG, "bad pool");
  p->solo = enable ? 1 : 0;
  clear_graphs(p);
  return KMC_OK;
}

int kmc_pool_set_tables_on_chip(kmc_pool *p, int32_t enable) {
  if (!p) return fail(KMC_ERR_ARG, "bad pool");
  p->tables_on_chip = enable ? 1 : 0;
  clear_graphs(p);
  return KMC_OK;
}

int kmc_pool_set_table_placement(kmc_pool *p, int32_t shared) {
  if (!p) return fail(KMC_ERR_ARG, "bad pool");
  p->stage_hot = shared ? 1 : 0;
  clear_graphs(p);
  return KMC_OK;
}

int kmc_pool_set_fast_path(kmc_pool *p, int32_t enable) {
  if (!p) return fail(KMC_ERR_ARG, "bad pool");
  p->fast_path = enable ? 1 : 0;
  clear_graphs(p);
  return KMC_OK;
}

int kmc_pool_get_status(kmc_pool *p, int32_t slot, int32_t *status) {
  int rc = check_slot(p, slot);
  if (rc) return rc;
  SlotDev d;
  rc = read_slot(p, slot, &d);
  if (rc) return rc;
  *status = d.status;
  return KMC_OK;
}

int kmc_pool_get_clock(kmc_pool *p, int32_t slot, double *t, int64_t *step) {
  int rc = check_slot(p, slot);
  if (rc) return rc;
  SlotDev d;
  rc = read_slot(p, slot, &d);
  if (rc) return rc;
  if (t) *t = d.kmc_time;
  if (step) *step = d.kmc_step;
  return KMC_OK;
}

#define POOL_VEC_GETTER(NAME, FIELD, TYPE)                                                   \
  int NAME(kmc_pool *p, int32_t slot, TYPE *out) {                                           \
    int rc = check_slot(p, slot);                                                            \
    if (rc) return rc;                                                                       \
    CK(cudaStreamSynchronize(p->stream));                                                    \
    const SlotDev &d = p->slots[slot].dev;                                                   \
    CK(cudaMemcpy(out, d.FIELD, sizeof(TYPE) * d.P, cudaMemcpyDeviceToHost));                 \
    return KMC_OK;                                                                           \
  }
POOL_VEC_GETTER(kmc_pool_get_procstat, procstat, int64_t)
POOL_VEC_GETTER(kmc_pool_get_integ_rates, integ, double)
POOL_VEC_GETTER(kmc_pool_get_nr_of_sites, nsites, int32_t)

int kmc_pool_get_lattice(kmc_pool *p, int32_t slot, int32_t *out) {
  int rc = check_slot(p, slot);
  if (rc) return rc;
  CK(cudaStreamSynchronize(p->stream));
  const SlotDev &d = p->slots[slot].dev;
  std::vector<int8_t> tmp(d.V);
  CK(cudaMemcpy(tmp.data(), d.lat, d.V, cudaMemcpyDeviceToHost));
  for (int i = 0; i < d.V; i++) out[i] = tmp[i];
  return KMC_OK;
}

int kmc_pool_set_rates(kmc_pool *p, int32_t slot, const double *rates) {
  int rc = check_slot(p, slot);
  if (rc) return rc;
  if (!rates) return fail(KMC_ERR_ARG, "bad arguments");
  std::lock_guard<std::mutex> lock(p->mu);
  CK(cudaSetDevice(p->device));
  CK(cudaStreamSynchronize(p->stream));
  SlotHost &sh = p->slots[slot];
  CK(cudaMemcpy(sh.dev.rates, rates, sizeof(double) * sh.dev.P, cudaMemcpyHostToDevice));
  // the next step recomputes every n*r term and the whole prefix sum (update_accum_rate)
  const int32_t zero = 0;
  CK(cudaMemcpy(&p->d_slots[slot].accum_from, &zero, sizeof(int32_t), cudaMemcpyHostToDevice));
  sh.dev.accum_from = 0;
  return KMC_OK;
}

int kmc_pool_get_tables(kmc_pool *p, int32_t slot, int32_t *as1, int32_t *as2) {
  int rc = check_slot(p, slot);
  if (rc) return rc;
  CK(cudaStreamSynchronize(p->stream));
  const SlotDev &d = p->slots[slot].dev;
  const size_t bytes = sizeof(int32_t) * (size_t)d.P * (d.V + 1);
  if (as1) CK(cudaMemcpy(as1, d.as1, bytes, cudaMemcpyDeviceToHost));
  if (as2) CK(cudaMemcpy(as2, d.as2, bytes, cudaMemcpyDeviceToHost));
  return KMC_OK;
}

int kmc_pool_occupation_counts(kmc_pool *p, const int32_t *slots, int32_t n, int32_t stride, int64_t *out) {
  if (!p || n < 1 || !slots || !out || stride < 1) return fail(KMC_ERR_ARG, "bad arguments");
  {
    int rc = check_occupation_list(p, slots, n, stride);
    if (rc) return rc;
  }
  AsyncScratch s_list(p->stream), s_out(p->stream);
  CK(s_list.alloc(sizeof(int32_t) * n));
  CK(s_out.alloc(sizeof(unsigned long long) * (size_t)n * stride));
  int32_t *d_list = s_list.as<int32_t>();
  unsigned long long *d_out = s_out.as<unsigned long long>();
  CK(cudaMemsetAsync(d_out, 0, sizeof(unsigned long long) * (size_t)n * stride, p->stream));
  CK(cudaMemcpyAsync(d_list, slots, sizeof(int32_t) * n, cudaMemcpyHostToDevice, p->stream));
  kmc_occupation_kernel<<<n, 256, 0, p->stream>>>(p->d_slots, p->d_models, d_list, n, stride, d_out);
  CK(cudaGetLastError());
  p->launches++;
  CK(cudaMemcpyAsync(out, d_out, sizeof(unsigned long long) * (size_t)n * stride, cudaMemcpyDeviceToHost, p->stream));
  CK(cudaStreamSynchronize(p->stream));
  return KMC_OK;
}

int kmc_pool_get_results(kmc_pool *p, const int32_t *slots, int32_t n, int32_t stride, int64_t *procstat,
                         double *integ, double *times, int64_t *steps, int32_t *status) {
  if (!p || n < 1 || !slots || stride < 1) return fail(KMC_ERR_ARG, "bad arguments");
  for (int i = 0; i < n; i++) {
    int rc = check_slot(p, slots[i]);
    if (rc) return rc;
  }
  CK(cudaSetDevice(p->device));
  const size_t nps = (size_t)n * stride;
  const size_t bytes = sizeof(int32_t) * n + nps * 16 + sizeof(ResultRow) * n + 256;
  if (bytes > p->res_cap) {
    CK(cudaStreamSynchronize(p->stream));
    cudaFree(p->d_res);
    cudaFreeHost(p->h_res);
    CK(cudaMalloc(&p->d_res, bytes));
    CK(cudaMallocHost(&p->h_res, bytes));
    p->res_cap = bytes;
  }
  char *d = p->d_res;
  int32_t *d_list = (int32_t *)d;
  int64_t *d_ps = (int64_t *)(d + align_up(sizeof(int32_t) * n, 16));
  double *d_ig = (double *)((char *)d_ps + nps * 8);
  ResultRow *d_rows = (ResultRow *)((char *)d_ig + nps * 8);
  const size_t used = (char *)(d_rows + n) - d;
  memcpy(p->h_res, slots, sizeof(int32_t) * n);
  CK(cudaMemcpyAsync(d_list, p->h_res, sizeof(int32_t) * n, cudaMemcpyHostToDevice, p->stream));
  kmc_results_kernel<<<n, 64, 0, p->stream>>>(p->d_slots, d_list, n, stride, d_ps, d_ig, d_rows);
  CK(cudaGetLastError());
  p->launches++;
  const size_t off = align_up(sizeof(int32_t) * n, 16);
  CK(cudaMemcpyAsync(p->h_res + off, d + off, used - off, cudaMemcpyDeviceToHost, p->stream));
  CK(cudaStreamSynchronize(p->stream));
  const int64_t *h_ps = (const int64_t *)(p->h_res + off);
  const double *h_ig = (const double *)((const char *)h_ps + nps * 8);
  const ResultRow *h_rows = (const ResultRow *)((const char *)h_ig + nps * 8);
  if (procstat) memcpy(procstat, h_ps, nps * 8);
  if (integ) memcpy(integ, h_ig, nps * 8);
  for (int i = 0; i < n; i++) {
    if (times) times[i] = h_rows[i].kmc_time;
    if (steps) steps[i] = h_rows[i].kmc_step;
    if (status) status[i] = h_rows[i].status;
  }
  return KMC_OK;
}

// ------------------------------------------------- occupation counts without allocating
// Scratch of kmc_pool_occupation_counts_static: the slot list (int32) followed by the
// counters (unsigned 64-bit), for at most KMC_STATIC_OCC_MAX_SLOTS slots of at most
// KMC_STATIC_OCC_MAX_STRIDE counters.  Every GPU that loads the library holds it until
// the process exits.  Host code may not use the name as an address: the per-device
// address comes from cudaGetSymbolAddress below.
constexpr size_t kOccListBytes = sizeof(int32_t) * KMC_STATIC_OCC_MAX_SLOTS;
constexpr size_t kOccCountBytes = sizeof(unsigned long long) * KMC_STATIC_OCC_MAX_SLOTS * KMC_STATIC_OCC_MAX_STRIDE;
static __device__ __align__(256) unsigned char g_occ_scratch[kOccListBytes + kOccCountBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_occ_mu;
void *g_occ_addr[kMaxDevices];  // device address of g_occ_scratch, per device
}  // namespace

int kmc_pool_occupation_counts_static(kmc_pool *p, const int32_t *slots, int32_t n, int32_t stride, int64_t *out) {
  if (!p || !slots || !out) return fail(KMC_ERR_ARG, "bad arguments");
  if (n < 1 || n > KMC_STATIC_OCC_MAX_SLOTS)
    return fail(KMC_ERR_ARG, "kmc_pool_occupation_counts_static: slot count must be 1.." +
                                 std::to_string(KMC_STATIC_OCC_MAX_SLOTS));
  if (stride < 1 || stride > KMC_STATIC_OCC_MAX_STRIDE)
    return fail(KMC_ERR_ARG, "kmc_pool_occupation_counts_static: stride must be 1.." +
                                 std::to_string(KMC_STATIC_OCC_MAX_STRIDE));
  {
    int rc = check_occupation_list(p, slots, n, stride);
    if (rc) return rc;
  }
  if (p->device < 0 || p->device >= kMaxDevices) return fail(KMC_ERR_ARG, "device index beyond the static table");
  CK(cudaSetDevice(p->device));
  void *base = nullptr;
  {
    // one-time set-up per device, with that device current
    std::lock_guard<std::mutex> lock(g_occ_mu);
    if (!g_occ_addr[p->device]) {
      void *addr = nullptr;
      CK(cudaGetSymbolAddress(&addr, g_occ_scratch));
      g_occ_addr[p->device] = addr;
    }
    base = g_occ_addr[p->device];
  }
  int32_t *d_list = reinterpret_cast<int32_t *>(base);
  unsigned long long *d_out = reinterpret_cast<unsigned long long *>(static_cast<char *>(base) + kOccListBytes);
  const size_t count_bytes = sizeof(unsigned long long) * (size_t)n * stride;
  // the counters keep the previous call's values: clear the part this call uses
  CK(cudaMemsetAsync(d_out, 0, count_bytes, p->stream));
  CK(cudaMemcpyAsync(d_list, slots, sizeof(int32_t) * n, cudaMemcpyHostToDevice, p->stream));
  kmc_occupation_kernel<<<n, 256, 0, p->stream>>>(p->d_slots, p->d_models, d_list, n, stride, d_out);
  CK(cudaGetLastError());
  p->launches++;
  CK(cudaMemcpyAsync(out, d_out, count_bytes, cudaMemcpyDeviceToHost, p->stream));
  CK(cudaStreamSynchronize(p->stream));
  return KMC_OK;
}

// ---------------------------------------------------------- single trajectory API
int kmc_create(const int32_t *program, int32_t program_len, const int32_t dims[3], int32_t layer, int32_t seed,
               int32_t rng_kind, uint32_t traj_id, kmc_handle **out) {
  if (!program || !dims || !out) return fail(KMC_ERR_ARG, "bad arguments");
  ModelDev md;
  int rc = validate_program(program, program_len, &md);
  if (rc) return rc;
  if (dims[0] < 1 || dims[1] < 1 || dims[2] < 1) return fail(KMC_ERR_ARG, "bad system size");
  const int V = dims[0] * dims[1] * dims[2] * md.spuck;
  const size_t bytes = align_up(slot_layout(md.P, V).total, 256);
  kmc_pool *p = nullptr;
  rc = kmc_pool_create(0, bytes, 1, &p);
  if (rc) return rc;
  kmc_handle *h = new kmc_handle();
  h->pool = p;
  rc = kmc_pool_add_model(p, program, program_len, &h->model);
  if (rc) { kmc_pool_destroy(p); delete h; return rc; }
  std::vector<double> zeros(md.P, 0.0);
  rc = kmc_pool_admit(p, h->model, dims, layer, seed, rng_kind, traj_id, zeros.data(), &h->slot);
  if (rc) { kmc_pool_destroy(p); delete h; return rc; }
  h->P = md.P; h->V = V; h->spuck = md.spuck; h->nspecies = md.nspecies;
  int32_t st = 0;
  rc = kmc_pool_get_status(p, h->slot, &st);
  if (rc || st) { kmc_pool_destroy(p); delete h; return rc ? rc : fail(st, "initialize_state failed"); }
  *out = h;
  return KMC_OK;
}

int kmc_destroy(kmc_handle *h) {
  if (!h) return KMC_OK;
  if (h->d_trace) cudaFree(h->d_trace);
  kmc_pool_destroy(h->pool);
  delete h;
  return KMC_OK;
}

#define HCHECK(h) \
  if (!(h) || !(h)->pool) return fail(KMC_ERR_ARG, "bad handle");

int kmc_set_rate_const(kmc_handle *h, int32_t proc, double rate) {
  HCHECK(h);
  if (proc < 1 || proc > h->P) return fail(KMC_ERR_ARG, "proc out of range");
  const SlotDev &d = h->pool->slots[h->slot].dev;
  CK(cudaStreamSynchronize(h->pool->stream));
  CK(cudaMemcpy(d.rates + proc - 1, &rate, sizeof(double), cudaMemcpyHostToDevice));
  const int32_t zero = 0;
  CK(cudaMemcpy(&h->pool->d_slots[h->slot].accum_from, &zero, sizeof(int32_t), cudaMemcpyHostToDevice));
  return KMC_OK;
}

int kmc_update_accum_rate(kmc_handle *h) {
  HCHECK(h);
  return run_command(h->pool, h->slot, CMD_ACCUM, 0, 0, 0, nullptr, nullptr, nullptr);
}

int kmc_update_integ_rate(kmc_handle *h) {
  HCHECK(h);
  return run_command(h->pool, h->slot, CMD_INTEG, 0, 0, 0, nullptr, nullptr, nullptr);
}

static int finish_run(kmc_handle *h) {
  int32_t st = 0;
  int rc = kmc_pool_get_status(h->pool, h->slot, &st);
  if (rc) return rc;
  if (st) {
    // keep the trajectory usable for inspection: clear the status word
    const int32_t zero = 0;
    CK(cudaMemcpy(&h->pool->d_slots[h->slot].status, &zero, sizeof(int32_t), cudaMemcpyHostToDevice));
    return fail(st, "kMC step failed with status " + std::to_string(st));
  }
  return KMC_OK;
}

int kmc_do_steps(kmc_handle *h, int64_t n) {
  HCHECK(h);
  if (n < 0) return fail(KMC_ERR_ARG, "negative step count");
  const auto t0 = std::chrono::steady_clock::now();
  int rc = kmc_pool_run(h->pool, &h->slot, &n, 1);
  if (rc) return rc;
  rc = finish_run(h);
  h->walltime += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

int kmc_get_walltime(kmc_handle *h, double *t) {
  HCHECK(h);
  if (!t) return fail(KMC_ERR_ARG, "bad arguments");
  *t = h->walltime;
  return KMC_OK;
}

int kmc_trace_steps(kmc_handle *h, int64_t n, int32_t *out) {
  HCHECK(h);
  if (n < 0 || !out) return fail(KMC_ERR_ARG, "bad arguments");
  if (n == 0) return KMC_OK;
  kmc_pool *p = h->pool;
  if (h->trace_cap < n) {
    if (h->d_trace) cudaFree(h->d_trace);
    CK(cudaMalloc(&h->d_trace, sizeof(int32_t) * 2 * n));
    h->trace_cap = n;
  }
  *p->h_cancel = 0;
  int rc = launch_run(p, &h->slot, &n, 1, p->d_list, p->d_steps, h->d_trace);
  if (rc) return rc;
  CK(cudaMemcpyAsync(out, h->d_trace, sizeof(int32_t) * 2 * n, cudaMemcpyDeviceToHost, p->stream));
  return finish_run(h);
}

int kmc_get_next_step(kmc_handle *h, int32_t *proc, int32_t *site) {
  HCHECK(h);
  return run_command(h->pool, h->slot, CMD_GET_NEXT, 0, 0, 0, proc, site, nullptr);
}

int kmc_run_proc_nr(kmc_handle *h, int32_t proc, int32_t site) {
  HCHECK(h);
  if (proc < 1 || proc > h->P || site < 1 || site > h->V) return fail(KMC_ERR_ARG, "proc or site out of range");
  return run_command(h->pool, h->slot, CMD_RUN_PROC, proc, site, 0, nullptr, nullptr, nullptr);
}

int kmc_touchup(kmc_handle *h, int32_t site) {
  HCHECK(h);
  if (site < 1 || site > h->V) return fail(KMC_ERR_ARG, "site out of range");
  return run_command(h->pool, h->slot, CMD_TOUCHUP, site, 0, 0, nullptr, nullptr, nullptr);
}

int kmc_touchup_many(kmc_handle *h, const int32_t *sites, int32_t n) {
  HCHECK(h);
  if (n < 0 || (n > 0 && !sites)) return fail(KMC_ERR_ARG, "bad arguments");
  for (int k = 0; k < n; k++)
    if (sites[k] < 1 || sites[k] > h->V) return fail(KMC_ERR_ARG, "site out of range");
  if (n == 0) return KMC_OK;
  kmc_pool *p = h->pool;
  AsyncScratch list(p->stream);
  CK(list.alloc(sizeof(int32_t) * n));
  CK(cudaMemcpyAsync(list.as<int32_t>(), sites, sizeof(int32_t) * n, cudaMemcpyHostToDevice, p->stream));
  return run_command(p, h->slot, CMD_TOUCHUP_LIST, n, 0, 0, nullptr, nullptr, list.as<int32_t>());
}

int kmc_replace_species(kmc_handle *h, int32_t site, int32_t old_species, int32_t new_species) {
  HCHECK(h);
  if (site < 1 || site > h->V) return fail(KMC_ERR_ARG, "site out of range");
  // the species a lattice can hold: 0..nspecies-1 and null_species (-1 or nspecies), the
  // range state images and .reload files are checked against
  if (new_species < -1 || new_species > h->nspecies) return fail(KMC_ERR_ARG, "unknown species");
  return run_command(h->pool, h->slot, CMD_REPLACE, site, old_species, new_species, nullptr, nullptr, nullptr);
}

int kmc_get_species(kmc_handle *h, int32_t site, int32_t *species) {
  HCHECK(h);
  if (site < 1 || site > h->V || !species) return fail(KMC_ERR_ARG, "site out of range");
  CK(cudaStreamSynchronize(h->pool->stream));
  int8_t s;
  CK(cudaMemcpy(&s, h->pool->slots[h->slot].dev.lat + site - 1, 1, cudaMemcpyDeviceToHost));
  *species = s;
  return KMC_OK;
}

int kmc_get_kmc_time(kmc_handle *h, double *t) {
  HCHECK(h);
  return kmc_pool_get_clock(h->pool, h->slot, t, nullptr);
}

int kmc_set_kmc_time(kmc_handle *h, double t) {
  HCHECK(h);
  CK(cudaStreamSynchronize(h->pool->stream));
  CK(cudaMemcpy(&h->pool->d_slots[h->slot].kmc_time, &t, sizeof(double), cudaMemcpyHostToDevice));
  return KMC_OK;
}

int kmc_get_kmc_time_step(kmc_handle *h, double *dt) {
  HCHECK(h);
  SlotDev d;
  int rc = read_slot(h->pool, h->slot, &d);
  if (rc) return rc;
  *dt = d.kmc_time_step;
  return KMC_OK;
}

int kmc_get_kmc_step(kmc_handle *h, int64_t *step) {
  HCHECK(h);
  return kmc_pool_get_clock(h->pool, h->slot, nullptr, step);
}

int kmc_get_volume(kmc_handle *h, int32_t *volume) {
  HCHECK(h);
  *volume = h->V;
  return KMC_OK;
}

int kmc_get_nr_of_proc(kmc_handle *h, int32_t *nproc) {
  HCHECK(h);
  *nproc = h->P;
  return KMC_OK;
}

int kmc_get_procstat(kmc_handle *h, int64_t *out) { HCHECK(h); return kmc_pool_get_procstat(h->pool, h->slot, out); }
int kmc_get_integ_rates(kmc_handle *h, double *out) { HCHECK(h); return kmc_pool_get_integ_rates(h->pool, h->slot, out); }
int kmc_get_nr_of_sites(kmc_handle *h, int32_t *out) { HCHECK(h); return kmc_pool_get_nr_of_sites(h->pool, h->slot, out); }

int kmc_get_rates(kmc_handle *h, double *out) {
  HCHECK(h);
  CK(cudaStreamSynchronize(h->pool->stream));
  CK(cudaMemcpy(out, h->pool->slots[h->slot].dev.rates, sizeof(double) * h->P, cudaMemcpyDeviceToHost));
  return KMC_OK;
}

int kmc_get_accum_rates(kmc_handle *h, double *out) {
  HCHECK(h);
  CK(cudaStreamSynchronize(h->pool->stream));
  CK(cudaMemcpy(out, h->pool->slots[h->slot].dev.accum, sizeof(double) * h->P, cudaMemcpyDeviceToHost));
  return KMC_OK;
}

int kmc_get_avail_site(kmc_handle *h, int32_t proc, int32_t idx, int32_t sw, int32_t *out) {
  HCHECK(h);
  if (proc < 1 || proc > h->P || idx < 1 || idx > h->V || (sw != 1 && sw != 2) || !out)
    return fail(KMC_ERR_ARG, "index out of range");
  CK(cudaStreamSynchronize(h->pool->stream));
  const SlotDev &d = h->pool->slots[h->slot].dev;
  const int32_t *tab = sw == 1 ? d.as1 : d.as2;
  CK(cudaMemcpy(out, tab + (size_t)(proc - 1) * (h->V + 1) + idx, sizeof(int32_t), cudaMemcpyDeviceToHost));
  return KMC_OK;
}

int kmc_get_lattice(kmc_handle *h, int32_t *out) { HCHECK(h); return kmc_pool_get_lattice(h->pool, h->slot, out); }
int kmc_get_tables(kmc_handle *h, int32_t *as1, int32_t *as2) { HCHECK(h); return kmc_pool_get_tables(h->pool, h->slot, as1, as2); }

int kmc_get_occupation(kmc_handle *h, double *out) {
  HCHECK(h);
  const int stride = h->nspecies * h->spuck;
  std::vector<int64_t> counts(stride);
  int rc = kmc_pool_occupation_counts(h->pool, &h->slot, 1, stride, counts.data());
  if (rc) return rc;
  const SlotDev &d = h->pool->slots[h->slot].dev;
  const double cells = (double)d.X * d.Y * d.Z;
  for (int i = 0; i < stride; i++) out[i] = (double)counts[i] / cells;
  return KMC_OK;
}

}  // extern "C"
