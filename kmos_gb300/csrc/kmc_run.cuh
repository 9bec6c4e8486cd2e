// kmc_run.cuh -- the persistent kMC step kernel (do_kmc_steps,
// proclist_generic_subroutines.mpy:1-44) of the GB300 engine, shared by the translation
// units that instantiate its variants.
//
// A *group* of G lanes owns one trajectory at a time: G = 32 is one warp per trajectory,
// G = 16 puts two trajectories on one warp (each half runs its own steps; the two halves
// share an instruction stream wherever their steps take the same branches, so one warp
// instruction advances both).  Every warp-level collective of the step names only its
// group's lanes.  Groups pull trajectories from a work counter, so thousands of uneven
// trajectories share one launch.  Per step:
//   * three FP64 draws (gfortran xoshiro256** or Philox), G steps' worth at a time,
//   * accum_rates prefix sum in the reference's serial order (base.mpy:603-623),
//     recomputed only from the first process whose nr_of_sites changed (bit-identical
//     to a full recompute),
//   * kmc_time += -log(r)/accum(P) (base.mpy:1123-1161),
//   * integ_rates update, one process per lane (base.mpy:626-645),
//   * the bisection of interval_search_real (base.mpy:1234-1338) as group ballots:
//     proc = min(first i with accum(i) > v, first i with accum(i) == accum(P)),
//   * site = avail_sites(proc, min(n, int(1 + r*n)), 1),
//   * run_proc_nr: the op program of that process.
// FP64 adds and multiplies use explicit _rn intrinsics (and the files are built with
// -fmad=false) so nothing is contracted into an FMA.
//
// With RunArgs::ts_bytes > 0 a trajectory whose lattice and avail_sites tables fit in
// ts_bytes runs with them in the group's region of shared memory: copied in when the
// group takes the trajectory, every step's reads and writes on chip, copied back when it
// is done (for the plain one-trajectory drop-in and other small launches).
#pragma once
#include <cuda_runtime.h>

#include "kmc_device.cuh"

namespace kmc {

constexpr int KMC_NPHASE = 16;

// The lanes of one trajectory group and its collectives.  For G = 32 these are the
// plain full-warp forms.
template <int G>
struct Group {
  int gl;         // lane within the group
  int base;       // first lane of the group within the warp
  unsigned mask;  // the group's lanes as a warp mask
  __device__ __forceinline__ Group() {
    const int lane = threadIdx.x & 31;
    if constexpr (G == 32) {
      gl = lane; base = 0; mask = 0xffffffffu;
    } else {
      gl = lane & (G - 1); base = lane & ~(G - 1); mask = ((1u << G) - 1u) << base;
    }
  }
  // bit i = lane i of the group
  __device__ __forceinline__ unsigned ballot(bool p) const {
    if constexpr (G == 32) return __ballot_sync(0xffffffffu, p);
    else return __ballot_sync(mask, p) >> base;
  }
  __device__ __forceinline__ bool any(bool p) const {
    if constexpr (G == 32) return __any_sync(0xffffffffu, p);
    else return __any_sync(mask, p);
  }
  template <class T>
  __device__ __forceinline__ T shfl(T v, int src) const {
    if constexpr (G == 32) return __shfl_sync(0xffffffffu, v, src);
    else return __shfl_sync(mask, v, src, G);
  }
  __device__ __forceinline__ void sync() const {
    if constexpr (G == 32) __syncwarp();
    else __syncwarp(mask);
  }
  __device__ __forceinline__ unsigned reduce_max(unsigned v) const {
    if constexpr (G == 32) return __reduce_max_sync(0xffffffffu, v);
    else return __reduce_max_sync(mask, v);
  }
};

// Cycle accounting per step phase (builds with -DKMC_PHASE_TIMING only): lane 0 of the
// group adds the clock64() time since the previous mark to phase i.
#ifdef KMC_PHASE_TIMING
#define KMC_PHASE(sm, i, grp)                          \
  do {                                                 \
    (grp).sync();                                      \
    if ((grp).gl == 0) {                               \
      const long long now_ = clock64();                \
      (sm).ph[i] += now_ - (sm).tprev;                 \
      (sm).tprev = now_;                               \
    }                                                  \
  } while (0)
#else
#define KMC_PHASE(sm, i, grp) \
  do {                        \
  } while (0)
#endif

// Shared memory of one trajectory group: NP processes per lane, NP * G in all.
template <int NP, int R, int G>
struct WarpSmem {
  double rates[NP * G];
  double accum[NP * G];
  double term[NP * G];  // nr_of_sites(i) * rates(i), refreshed when nr_of_sites(i) changes
  int32_t ns[NP * G];
  uint32_t pmask[NP * G][R];  // edits of each process this step, one bit per edit
  int32_t ndel[NP * G];       // del edits of each process so far this step (0 between steps)
  long long ph[KMC_NPHASE];   // phase cycle accounting (KMC_PHASE_TIMING builds)
  long long tprev;
  FastSmem<R, G, NP * G> f;  // list tails for every process the kernel holds
};

// Replays the edits of process p (bits of pmask[p], in program order).  Lane-private;
// returns a status.  Clears pmask[p] and ndel[p].  The loads it needs were issued
// group-parallel while the edits were evaluated: em[k] = avail_sites(p, site_k, 2) for
// every del edit k, and tail[p][j] = avail_sites(p, n0 - j, 1) for
// j < min(nd, TAIL_MAX), nd = its del edits.  In a dels-first stream (every del before
// every add, no (process, site) named by two dels or by two adds) only the moves of
// the dels are read back, so the cleared position entries and the adds are not logged.
template <int NP, int R, int G>
__device__ int replay_process(FastSmem<R, G, NP * G> &f, int32_t *ns, uint32_t (*pmask)[R], int32_t *ndel,
                              const View &v, int p, int rounds, bool dels_first, int gl) {
  const size_t row = (size_t)p * v.stride;
  int32_t *a1 = v.as1 + row;
  int32_t *a2 = v.as2 + row;
  const int n0 = ns[p];
  if (!KMC_IN(n0, 0, v.stride - 1)) return ST_TABLE;
  uint32_t bits[R];
#pragma unroll
  for (int r = 0; r < R; r++) {
    bits[r] = r < rounds ? pmask[p][r] : 0u;
    pmask[p][r] = 0u;
  }
  ndel[p] = 0;
  // apply the edits; reads look in the write log, then at the prefetched values.  The
  // log is append-only (a later entry for a key shadows earlier ones) and is searched
  // newest first, four keys per shared-memory load; once full, reads go to memory, which
  // every write reaches too.
  int nlog = 0;
  bool logok = true;
  auto put = [&](int table, int index, int32_t val) {
    if (table) a2[index] = val; else a1[index] = val;
    if (!logok) return;
    if (nlog < LOG_MAX) {
      reinterpret_cast<uint32_t *>(&f.lkey4[nlog >> 2][gl])[nlog & 3] = ((uint32_t)table << 31) | (uint32_t)index;
      f.lval[nlog][gl] = val;
      nlog++;
    } else {
      logok = false;
    }
  };
  auto logged = [&](int table, int index, int32_t &val) -> bool {
    const uint32_t key = ((uint32_t)table << 31) | (uint32_t)index;
    for (int g = (nlog - 1) >> 2; g >= 0; g--) {
      const uint4 k4 = f.lkey4[g][gl];
      const int b = 4 * g;
      int i = -1;
      if (b + 3 < nlog && k4.w == key) i = b + 3;
      else if (b + 2 < nlog && k4.z == key) i = b + 2;
      else if (b + 1 < nlog && k4.y == key) i = b + 1;
      else if (k4.x == key) i = b;
      if (i >= 0) { val = f.lval[i][gl]; return true; }
    }
    return false;
  };
  int n = n0;
#pragma unroll
  for (int r = 0; r < R; r++) {
    uint32_t b = bits[r];
    while (b) {
      const int k = 32 * r + __ffs(b) - 1;
      b &= b - 1;
      const int kind = f.ekind[k], site = f.esite[k];
      if (kind == E_ADD) {  // add_proc (base.mpy:268-302)
        if (n + 1 >= v.stride) return ST_TABLE;  // full list: tables out of step with the lattice
        n += 1;
        if (dels_first) {  // no del of this process follows, so nothing reads these back
          a1[n] = site;
          a2[site] = n;
          continue;
        }
        put(0, n, site);
        put(1, site, n);
        continue;
      }
      // del_proc (base.mpy:211-265)
      int m;
      if (!logok) m = a2[site];
      else if (nlog == 0 || !logged(1, site, m)) m = f.em[k];
      if (m == 0) {
        if (kind == E_DEL) return ST_TABLE;  // nli names a process that is not there
        continue;                            // guarded del of an absent entry
      }
      if (!KMC_IN(m, 1, n)) return ST_TABLE;
      if (m < n) {
        int last;
        if (!logok) last = a1[n];
        else if (nlog == 0 || !logged(0, n, last))
          last = (n0 - n < TAIL_MAX && n <= n0) ? f.tail[p][n0 - n] : a1[n];
        if (!KMC_IN(last, 1, v.stride - 1)) return ST_TABLE;
        put(0, m, last);
        a1[n] = 0;  // vacated top entry: read again only after an add (logged) refills it
        put(1, last, m);
      } else {
        a1[m] = 0;  // the same, m being the top
      }
      if (dels_first) a2[site] = 0;  // no later del of this process names this site
      else put(1, site, 0);
      n -= 1;
    }
  }
  ns[p] = n;
  return ST_OK;
}

// The serial interpreter (run_stream) for the step kernel's steps without a fast stream,
// out of line on a copy of the view: a single copy of its code away from the step loop,
// and the caller's view stays in registers.  Returns the status.
static __device__ __noinline__ int run_stream_copy(View v, int pos, int bx, int by, int bz) {
  v.minp = v.P;
  v.err = ST_OK;
  run_stream(v, pos, bx, by, bz);
  return v.err;
}

// One kMC step's run_proc_nr through the gather / evaluate / replay path.  All lanes of
// the group call it and get the status.
template <int NP, int R, int G>
__device__ int fast_step(WarpSmem<NP, R, G> &sm, const Hot &H, View &v, const int32_t *fs, int bx, int by, int bz,
                         const Group<G> &grp) {
  constexpr int RR = 32 * R / G;  // evaluation rounds of G edits
  const int gl = grp.gl;
  FastSmem<R, G, NP * G> &f = sm.f;
  const int nlat = fs[0], nchk = fs[1], nwr = fs[2];
  const uint32_t w3 = (uint32_t)fs[3];
  const int nedit = w3 & 0xFFFF, nq = (w3 >> 16) & 0xF;
  const bool dels_first = (w3 >> 20) & 1;
  const int32_t *coords = fs + 4;
  const int32_t *chk = coords + nlat;
  const int32_t *wr = chk + 2 * nchk;
  // edit k's quads, nedit quads apart: [h, target slot, x, 0], then packed references
  const int4 *quad = reinterpret_cast<const int4 *>(fs + fast_rec_offset(nlat, nchk, nwr));
  const unsigned lt = (1u << gl) - 1u;
  // 1. gather every slot (all lattice loads in flight together); check the old species
  //    of first replaces
  int32_t lvv[FAST_SLOTS / G];
  bool off_lattice = false;  // (KMC_DEBUG builds)
#pragma unroll
  for (int rr = 0; rr < FAST_SLOTS / G; rr++) {
    const int i = gl + G * rr;
    lvv[rr] = 0;
    if (i < nlat) {
      int site = v.g.site_near(bx, by, bz, coords[i]);
      if (!KMC_IN(site, 1, v.stride - 1)) { site = 1; off_lattice = true; }
      f.latsite[i] = site;
      lvv[rr] = v.lat[site - 1];
    }
  }
#ifdef KMC_DEBUG
  if (grp.any(off_lattice)) return ST_TABLE;
#endif
  KMC_PHASE(sm, 11, grp);
#pragma unroll
  for (int rr = 0; rr < FAST_SLOTS / G; rr++)
    if (gl + G * rr < nlat) f.latv[gl + G * rr] = lvv[rr];
  grp.sync();
  bool bad = false;
  for (int i = gl; i < nchk; i += G) bad |= !in_mask(f.latv[chk[2 * i]], chk[2 * i + 1]);
  if (grp.any(bad)) return ST_SPECIES;
  KMC_PHASE(sm, 4, grp);
  // 2. evaluate every edit in parallel; compact the ones that happen, in order.  The
  //    loads the replay needs are issued here and land in shared memory afterwards: a
  //    del edit's avail_sites(p, site, 2), and the list entry avail_sites(p, n0 - j, 1)
  //    its swap-remove can move, j = its rank among the process's dels this step.
  int ne = 0;
  int32_t emv[RR], tv[RR];
  int empos[RR], tslot[RR];
#pragma unroll
  for (int rr = 0; rr < RR; rr++) {
    emv[rr] = 0;
    empos[rr] = -1;
    tv[rr] = 0;
    tslot[rr] = -1;
    if (G * rr >= nedit) continue;
    const int k = G * rr + gl;
    bool on = false;
    int kind = E_GDEL, p = 0, site = 0, tgt = 0;
    if (k < nedit) {
      // all of the edit's quads in flight together; the table index is the base plus
      // code(slot) * mul over every packed reference (unused ones are 0: slot 0 times 0)
      const int4 q0 = quad[k];
      int4 q1 = make_int4(0, 0, 0, 0), q2 = q1, q3 = q1;
      if (nq >= 1) q1 = quad[nedit + k];
      if (nq >= 2) q2 = quad[2 * nedit + k];
      if (nq >= 3) q3 = quad[3 * nedit + k];
      const uint32_t h = (uint32_t)q0.x;
      const int op = h & 0xFF, cnt = (h >> 8) & 0xFF, arg = (h >> 16) & 0xFFFF;
      tgt = q0.y;
      if (op >= 6) {
        const int ns = H.nspecies;
        auto tref = [&](int32_t w) { return species_code(f.latv[w & 0xFF], ns) * (w >> 8); };
        int idx = q0.z + ((tref(q1.x) + tref(q1.y)) + (tref(q1.z) + tref(q1.w)));
        if (nq >= 2) idx += (tref(q2.x) + tref(q2.y)) + (tref(q2.z) + tref(q2.w));
        if (nq >= 3) idx += (tref(q3.x) + tref(q3.y)) + (tref(q3.z) + tref(q3.w));
        p = H.h[idx];
        on = p != 0;
        kind = op == 6 ? E_DEL : E_ADD;
      } else if (op == 2) {
        on = true; p = arg;
      } else if (op == 3) {
        if (cnt <= 1) {  // the condition is in the quad: [h, target, slot, mask]
          on = cnt == 0 || in_mask(f.latv[q0.z], q0.w);
        } else {
          const int32_t *e = fs + q0.z;  // [h, target, ref * cnt, mask * cnt]
          on = true;
          for (int c = 0; c < cnt && on; c++) on = in_mask(ref_value(e[2 + c], f.latv), e[2 + cnt + c]);
        }
        p = arg; kind = E_ADD;
      } else {
        const int32_t *e = fs + q0.z;  // [h, target, 0, record offset, ref * cnt]
        p = nli_refs(H, cnt, e[2], e[3], e + 4, f.latv);
        on = p != 0;
        kind = op == 4 ? E_DEL : E_ADD;
      }
    }
    KMC_PHASE(sm, 12, grp);
    if (on) {
      site = f.latsite[tgt];
      if (kind != E_ADD) emv[rr] = v.as2[(size_t)(p - 1) * v.stride + site];
    }
    KMC_PHASE(sm, 13, grp);
    // a del's rank among its process's dels picks which list entry it loads; the ranks
    // only have to be distinct, so a shared-memory counter gives them in any order
    if (on && kind != E_ADD) {
      const int q = p - 1;
      const int rank = atomicAdd(&sm.ndel[q], 1);
      if (rank < TAIL_MAX) {
        const int n0 = sm.ns[q];
        tslot[rr] = q * TAIL_MAX + rank;
        if (n0 - rank >= 1) tv[rr] = v.as1[(size_t)q * v.stride + n0 - rank];
      }
    }
    KMC_PHASE(sm, 14, grp);
    const unsigned b = grp.ballot(on);
    if (on) {
      const int pos = ne + __popc(b & lt);
      f.ekind[pos] = (int8_t)kind;
      f.ep[pos] = (int16_t)(p - 1);
      f.esite[pos] = site;
      atomicOr(&sm.pmask[p - 1][pos >> 5], 1u << (pos & 31));  // the process's edit mask
      if (kind != E_ADD) empos[rr] = pos;
    }
    ne += __popc(b);
    KMC_PHASE(sm, 15, grp);
  }
  const int rounds = (ne + 31) >> 5;
  KMC_PHASE(sm, 5, grp);
  // the loads issued during evaluation land now
#pragma unroll
  for (int rr = 0; rr < RR; rr++) {
    if (empos[rr] >= 0) f.em[empos[rr]] = emv[rr];
    if (tslot[rr] >= 0) (&f.tail[0][0])[tslot[rr]] = tv[rr];
  }
  grp.sync();
  KMC_PHASE(sm, 6, grp);
  // 3. every process with edits replays them on its own lane (process j on lane j % G)
  int err = ST_OK;
  for (int j = gl; j < v.P; j += G) {
    uint32_t any = 0;
#pragma unroll
    for (int r = 0; r < R; r++) any |= r < rounds ? sm.pmask[j][r] : 0u;
    if (any) {
      const int e = replay_process<NP, R, G>(f, sm.ns, sm.pmask, sm.ndel, v, j, rounds, dels_first, gl);
      if (e) err = e;
    }
  }
  KMC_PHASE(sm, 7, grp);
  // 4. the final species of every replaced slot
  if (!grp.any(err != ST_OK))
    for (int i = gl; i < nwr; i += G) v.lat[f.latsite[wr[2 * i]] - 1] = (int8_t)wr[2 * i + 1];
  const int e0 = grp.reduce_max((unsigned)err);
  grp.sync();
  KMC_PHASE(sm, 8, grp);
  return e0;
}

// --------------------------------------------------------------------- run kernel
struct RunArgs {
  SlotDev *slots;
  const ModelDev *models;
  const int32_t *list;
  const int64_t *steps;
  int32_t n;
  int32_t *counter;
  int32_t *trace;                 // (proc, site) per step of a single-slot run, or null
  const volatile int32_t *cancel; // host-mapped cancel flag, or null
  int32_t fast;                   // 1: use the gather / replay path where it applies
  int32_t model;                  // every listed slot runs this model
  int32_t stage_words;            // hot-section words copied to shared memory (0 = read it from global)
  int32_t groups;                 // trajectory groups per block
  int32_t ts_bytes;               // shared memory per group for lattice and tables (0 = none)
  int32_t prog_words;             // solo kernel: program words copied to shared memory (0 = none)
  unsigned long long *phase;      // KMC_NPHASE cycle sums (KMC_PHASE_TIMING builds)
};

// Bytes of shared memory a trajectory's lattice and avail_sites tables take in a
// group's region: the lattice, then as1 and as2, each on a 16-byte boundary.
__host__ __device__ inline size_t ts_need(int P, int V) {
  const size_t lat = ((size_t)V + 15) / 16 * 16;
  const size_t tab = ((size_t)P * (V + 1) * 4 + 15) / 16 * 16;
  return lat + 2 * tab;
}

// Copies n bytes between 16-byte aligned buffers with the group's lanes.
template <int G>
__device__ inline void group_copy(void *dst, const void *src, size_t n, const Group<G> &grp) {
  const size_t n16 = n / 16;
  int4 *d4 = reinterpret_cast<int4 *>(dst);
  const int4 *s4 = reinterpret_cast<const int4 *>(src);
  for (size_t i = grp.gl; i < n16; i += G) d4[i] = s4[i];
  unsigned char *d1 = reinterpret_cast<unsigned char *>(dst);
  const unsigned char *s1 = reinterpret_cast<const unsigned char *>(src);
  for (size_t i = 16 * n16 + grp.gl; i < n; i += G) d1[i] = s1[i];
}

template <int NP, int R, int G>
__global__ void __launch_bounds__(512, 1) kmc_run_kernel(RunArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Group<G> grp;
  const int gl = grp.gl;
  const int gib = threadIdx.x / G;  // group in block
  const ModelDev M = a.models[a.model];
  const int P = M.P;
  // stage the model's hot section (fast streams, group records, nli tables)
  int32_t *hot_s = reinterpret_cast<int32_t *>(smem_raw);
  const int stage = a.stage_words;
  for (int i = threadIdx.x; i < stage; i += blockDim.x) hot_s[i] = M.prog[M.off_hot + i];
  Hot H;
  H.h = stage ? hot_s : M.prog + M.off_hot;
  H.grp = M.hot_grp;
  H.tab = M.hot_tab;
  H.nspecies = M.nspecies;
  const size_t hot_bytes = ((size_t)stage * 4 + 15) / 16 * 16;
  WarpSmem<NP, R, G> &sm = reinterpret_cast<WarpSmem<NP, R, G> *>(smem_raw + hot_bytes)[gib];
  unsigned char *ts = smem_raw + hot_bytes + sizeof(WarpSmem<NP, R, G>) * a.groups + (size_t)a.ts_bytes * gib;
  for (int i = gl; i < NP * G * R; i += G) (&sm.pmask[0][0])[i] = 0u;
  for (int i = gl; i < NP * G; i += G) sm.ndel[i] = 0;
  for (int i = gl; i < KMC_NPHASE; i += G) sm.ph[i] = 0;
  __syncthreads();

  // Work: every group first takes item (group in block) * gridDim.x + block -- the list
  // is sorted by cost, so each block gets an even share of long and short trajectories
  // -- then pulls further items from the counter.
  const int nstatic = gridDim.x * a.groups;
  for (int round = 0;; round++) {
    int item = gib * gridDim.x + blockIdx.x;
    if (round > 0) {
      if (gl == 0) item = nstatic + atomicAdd(a.counter, 1);
      item = grp.shfl(item, 0);
    }
    if (item >= a.n) break;
    const int slot = a.list[item];
    const int64_t nsteps = a.steps[item];
    SlotDev &S = a.slots[slot];
    if (S.status != ST_OK || S.model != a.model) continue;
    const int stride = S.V + 1;

    View v;
    v.lat = S.lat;
    v.as1 = S.as1;
    v.as2 = S.as2;
    // lattice and tables on chip when they fit in the group's region
    const bool on_chip = a.ts_bytes > 0 && ts_need(P, S.V) <= (size_t)a.ts_bytes;
    const size_t lat_b = ((size_t)S.V + 15) / 16 * 16, tab_b = (size_t)P * stride * 4;
    if (on_chip) {
      v.lat = reinterpret_cast<int8_t *>(ts);
      v.as1 = reinterpret_cast<int32_t *>(ts + lat_b);
      v.as2 = reinterpret_cast<int32_t *>(ts + lat_b + (tab_b + 15) / 16 * 16);
      group_copy(v.lat, S.lat, S.V, grp);
      group_copy(v.as1, S.as1, tab_b, grp);
      group_copy(v.as2, S.as2, tab_b, grp);
      grp.sync();
    }
    v.ns = sm.ns;
    v.prog = M.prog;
    v.g.X = S.X; v.g.Y = S.Y; v.g.Z = S.Z; v.g.spuck = M.spuck;
    FastDiv div_spuck, div_x, div_y;  // calculate_nr2lattice without hardware division
    div_spuck.init(M.spuck);
    div_x.init(S.X);
    div_y.init(S.Y);
    v.stride = stride;
    v.backend = M.backend;
    v.P = P;
    v.off_groups = M.off_groups;
    v.collect = false;

    const bool fast_ok = a.fast && M.off_hot != 0 && S.V <= FAST_MAXV && P <= 256 &&
                         (M.reach_x == 0 || S.X > 2 * M.reach_x) && (M.reach_y == 0 || S.Y > 2 * M.reach_y) &&
                         (M.reach_z == 0 || S.Z > 2 * M.reach_z);
    double ig[NP];
    int64_t ps[NP];
    int32_t n0[NP];
#pragma unroll
    for (int j = 0; j < NP; j++) {
      const int i = gl + G * j;
      if (i < P) {
        const double r = S.rates[i];
        const int n = S.nsites[i];
        sm.rates[i] = r;
        sm.accum[i] = S.accum[i];
        sm.ns[i] = n;
        sm.term[i] = __dmul_rn((double)n, r);
        n0[j] = n;
        ig[j] = S.integ[i];
        ps[j] = S.procstat[i];
      } else {
        n0[j] = 0;
        ig[j] = 0.0;
        ps[j] = 0;
      }
    }
    // with every rate >= +0 every term n*r is >= +0, so is every partial sum, and adding
    // a +0 term leaves a sum >= +0 unchanged bit for bit: the chain skips those adds
    bool neg_rate = false;
#pragma unroll
    for (int j = 0; j < NP; j++) {
      const int i = gl + G * j;
      neg_rate |= i < P && (__double_as_longlong(sm.rates[i]) < 0);
    }
    const bool skip_zero = !grp.any(neg_rate);
    double t = S.kmc_time, dt = S.kmc_time_step;
    int64_t kstep = S.kmc_step;
    // random numbers: every G steps, lane j draws step k + j's (ran_time, ran_proc,
    // ran_site) and -log(ran_time); steps take them with shuffles
    uint64_t rbase[4] = {S.rng[0], S.rng[1], S.rng[2], S.rng[3]};
    const int rng_kind = S.rng_kind;
    const uint32_t seed = S.seed, traj = S.traj;
    double my_nl = 0.0, my_rp = 0.0, my_rs = 0.0;
    int bidx = G;
    int from = S.accum_from;
    int status = ST_OK;
    int64_t k = 0;
    grp.sync();
    if (gl == 0) sm.tprev = clock64();

    for (; k < nsteps; k++) {
      // the flag as one group-wide decision, so that no lane leaves the loop alone
      if (a.cancel && (k & 1023) == 0 && grp.any(*a.cancel != 0)) { status = ST_CANCELLED; break; }
      if (bidx == G) {
        if (k > 0) {  // advance the base state past the batch just used
          if (rng_kind == RNG_GFORTRAN) {
            for (int d = 0; d < 3 * G; d++) xoshiro_next(rbase[0], rbase[1], rbase[2], rbase[3]);
          } else {
            rbase[0] += G;
          }
        }
        uint64_t st[4] = {rbase[0], rbase[1], rbase[2], rbase[3]};
        double rt;
        if (rng_kind == RNG_GFORTRAN) {
          for (int d = 0; d < 3 * gl; d++) xoshiro_next(st[0], st[1], st[2], st[3]);
        } else {
          st[0] += gl;
        }
        draw3(rng_kind, st, seed, traj, rt, my_rp, my_rs);
        my_nl = -log(rt);
        bidx = 0;
      }
      const double nl = grp.shfl(my_nl, bidx);
      const double ran_proc = grp.shfl(my_rp, bidx);
      const double ran_site = grp.shfl(my_rs, bidx);
      bidx++;
      KMC_PHASE(sm, 0, grp);

      // update_accum_rate from the first stale entry: entries before it are the same
      // sums of the same terms, so the result equals a full recompute bit for bit
      if (gl == 0 && from < P) {
        double acc = from > 0 ? sm.accum[from - 1] : 0.0;
        int i = from;
        if (i == 0) { acc = sm.term[0]; sm.accum[0] = acc; i = 1; }
        for (; i < P; i += 8) {
          double t8[8];  // load a chunk of terms before the dependent adds
#pragma unroll
          for (int j = 0; j < 8; j++) t8[j] = (i + j < P) ? sm.term[i + j] : 0.0;
#pragma unroll
          for (int j = 0; j < 8; j++)
            if (i + j < P) {
              if (!(skip_zero && __double_as_longlong(t8[j]) == 0)) acc = __dadd_rn(acc, t8[j]);
              sm.accum[i + j] = acc;
            }
        }
      }
      from = P;
      grp.sync();
      KMC_PHASE(sm, 1, grp);
      const double total = sm.accum[P - 1];
      const long long tbits = __double_as_longlong(total);
      if (!(tbits > 0 && tbits < 0x7FF0000000000000LL)) { status = ST_DEADLOCK; break; }

      // determine_procsite: for non-negative doubles the order of the bit patterns is
      // the order of the values
      const long long vbits = __double_as_longlong(__dmul_rn(ran_proc, total));
      int proc = -1;
#pragma unroll
      for (int j = 0; j < NP; j++) {
        const int i = gl + G * j;
        const long long ab = i < P ? __double_as_longlong(sm.accum[i]) : 0;
        const bool pred = (i < P) && (ab > vbits || ab == tbits);
        const unsigned b = grp.ballot(pred);
        if (proc < 0 && b) proc = G * j + __ffs(b) - 1;
      }
      const int n = sm.ns[proc];
      if (n <= 0) { status = ST_DEADLOCK; break; }
      // idx = int(1 + ran_site * n): the int -> double and the truncation by bit
      // manipulation (exact for 1 <= n < 2^31 and 1 <= q < 2^32), the product and the sum
      // in FP64 as the reference rounds them
      const long long qb = __double_as_longlong(__dadd_rn(1.0, __dmul_rn(ran_site, int_to_double(n))));
      const int qe = (int)(qb >> 52) - 1023;
      int idx = (int)((((unsigned long long)qb & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull) >> (52 - qe));
      if (idx > n) idx = n;
      if (!KMC_IN(n, 1, S.V)) { status = ST_TABLE; break; }

#pragma unroll
      for (int j = 0; j < NP; j++)
        if (proc == gl + G * j) ps[j] += 1;  // increment_procstat

      KMC_PHASE(sm, 2, grp);
      int err = ST_OK;
      const int fs_off = fast_ok ? H.h[proc] : 0;
      int site = 0;
      if (gl == 0) site = v.as1[(size_t)proc * stride + idx];

      // while the site load is in flight: update_clocks, kmc_time += -log(r)/accum(P)
      // with the quotient as -log(r) times the reciprocal of accum(P) (within 2 ulp),
      // and update_integ_rate, integ(i) = integ(i) + n(i)*r(i)*dt
      dt = __dmul_rn(nl, __drcp_rn(total));
      t = __dadd_rn(t, dt);
      kstep += 1;
#pragma unroll
      for (int j = 0; j < NP; j++) {
        const int i = gl + G * j;
        if (i < P) ig[j] = __dadd_rn(ig[j], __dmul_rn(sm.term[i], dt));
      }

      if (gl == 0 && a.trace) { a.trace[2 * k] = proc + 1; a.trace[2 * k + 1] = site; }
      site = grp.shfl(site, 0);
      if (site < 1 || site > S.V) { status = ST_TABLE; break; }  // list entry outside the lattice
      int bx, by, bz, bn;
      {  // calculate_nr2lattice (lattice.mpy:177-210)
        const unsigned c = div_spuck.div((unsigned)(site - 1));
        bn = site - M.spuck * (int)c;
        const unsigned r = div_x.div(c);
        bx = (int)(c - (unsigned)S.X * r);
        const unsigned zq = div_y.div(r);
        by = (int)(r - (unsigned)S.Y * zq);
        bz = (int)zq;
      }
      KMC_PHASE(sm, 3, grp);
      if (fs_off) {
        err = fast_step<NP, R, G>(sm, H, v, H.h + fs_off, bx, by, bz, grp);
      } else {
        if (gl == 0) err = run_stream_copy(v, M.prog[M.off_proc + proc], bx, by, bz);
        err = grp.shfl(err, 0);
        grp.sync();
        KMC_PHASE(sm, 9, grp);
      }
      if (err) { status = err; break; }
      // refresh the terms of processes whose nr_of_sites changed; accum restarts at
      // the first of them
      int first = P;
#pragma unroll
      for (int j = 0; j < NP; j++) {
        const int i = gl + G * j;
        const int nn = i < P ? sm.ns[i] : 0;
        const bool ch = i < P && nn != n0[j];
        if (ch) { sm.term[i] = __dmul_rn(int_to_double(nn), sm.rates[i]); n0[j] = nn; }
        const unsigned b = grp.ballot(ch);
        if (first == P && b) first = G * j + __ffs(b) - 1;
      }
      from = first;
      grp.sync();
      KMC_PHASE(sm, 10, grp);
    }
    // random state after the draws actually used: bidx draws of the current batch
    // (a step that found no process has drawn its numbers, as in the reference)
    if (bidx < G || k > 0) {
      const int used = bidx;
      if (rng_kind == RNG_GFORTRAN) {
        for (int d = 0; d < 3 * used; d++) xoshiro_next(rbase[0], rbase[1], rbase[2], rbase[3]);
      } else {
        rbase[0] += used;
      }
    }

#pragma unroll
    for (int j = 0; j < NP; j++) {
      const int i = gl + G * j;
      if (i < P) {
        S.integ[i] = ig[j];
        S.procstat[i] = ps[j];
        S.nsites[i] = sm.ns[i];
        S.accum[i] = sm.accum[i];
      }
    }
    if (on_chip) {  // the lattice and tables back to the slot
      grp.sync();
      group_copy(S.lat, v.lat, S.V, grp);
      group_copy(S.as1, v.as1, tab_b, grp);
      group_copy(S.as2, v.as2, tab_b, grp);
    }
    if (gl == 0) {
      S.kmc_time = t;
      S.kmc_time_step = dt;
      S.kmc_step = kstep;
      S.rng[0] = rbase[0]; S.rng[1] = rbase[1]; S.rng[2] = rbase[2]; S.rng[3] = rbase[3];
      S.accum_from = from;
      S.status = status;
    }
    grp.sync();
  }
#ifdef KMC_PHASE_TIMING
  if (gl == 0 && a.phase)
    for (int i = 0; i < KMC_NPHASE; i++) atomicAdd(&a.phase[i], (unsigned long long)sm.ph[i]);
#endif
}

// --------------------------------------------------------------- solo kernel
// One trajectory per block of one warp, for models of at most SOLO_PMAX processes (the
// plain one-trajectory drop-in and other small launches).  The steps run on lane 0
// alone, as the reference's loop runs them: no warp collective per step, the process
// vectors (rates, accum, terms, integ, procstat) in lane 0's registers.  The other lanes
// draw the random numbers of the next 32 steps at once (the same streams as
// kmc_run_kernel: lane j takes step k + j) and copy the state on and off chip.  The
// program, the lattice and the avail_sites tables sit in shared memory when they fit
// (RunArgs::prog_words, RunArgs::ts_bytes).  run_proc_nr evaluates the process's resolved
// fast stream serially (every condition on the values before the step, then the table
// edits in program order, then the lattice writes: the serial interpreter's result) and
// falls back to the interpreter where the fast form does not apply.  Arithmetic and
// order are kmc_run_kernel's, so results are the same bit for bit.
constexpr int SOLO_PMAX = 8;

struct SoloSmem {
  double nl[32], rp[32], rs[32];  // -log(ran_time), ran_proc, ran_site of the batch's steps
  double tot[32], dtb[32];        // each step's total rate and kmc_time_step
  double thist[32][SOLO_PMAX];    // each step's terms nr_of_sites * rate (before its edits)
  int32_t latv[FAST_SLOTS];       // slot species before the step
  int32_t latsite[FAST_SLOTS];    // slot sites
  int32_t ns[SOLO_PMAX];          // nr_of_sites
  int32_t status, used, from, nclk;
};

// run_proc_nr of one step through the process's resolved fast stream, serially: the
// slots' species, the old-species checks, every edit's condition on the values before the
// step and its table operation in program order (add_proc / del_proc / guarded del_proc,
// base.mpy:211-302, written out here so that the view stays in registers), then the
// replaced slots' final species.
__device__ __forceinline__ int solo_fast_stream(View &v, const Hot &H, const int32_t *fs, int bx, int by, int bz,
                                                int32_t *latv, int32_t *latsite) {
  const int nlat = fs[0], nchk = fs[1], nwr = fs[2];
  const uint32_t w3 = (uint32_t)fs[3];
  const int nedit = w3 & 0xFFFF, nq = (w3 >> 16) & 0xF;
  const int32_t *coords = fs + 4;
  const int32_t *chk = coords + nlat;
  const int32_t *wr = chk + 2 * nchk;
  const int4 *quad = reinterpret_cast<const int4 *>(fs + fast_rec_offset(nlat, nchk, nwr));
  for (int i = 0; i < nlat; i++) {
    const int site = v.g.site_near(bx, by, bz, coords[i]);
    if (!KMC_IN(site, 1, v.stride - 1)) return ST_TABLE;
    latsite[i] = site;
    latv[i] = v.lat[site - 1];
  }
  for (int i = 0; i < nchk; i++)
    if (!in_mask(latv[chk[2 * i]], chk[2 * i + 1])) return ST_SPECIES;
  for (int k = 0; k < nedit; k++) {
    const int4 q0 = quad[k];
    const uint32_t h = (uint32_t)q0.x;
    const int op = h & 0xFF, cnt = (h >> 8) & 0xFF, arg = (h >> 16) & 0xFFFF;
    int p, kind;
    if (op >= 6) {
      const int ns = H.nspecies;
      auto tref = [&](int32_t w) { return species_code(latv[w & 0xFF], ns) * (w >> 8); };
      int idx = q0.z;
      if (nq >= 1) { const int4 q = quad[nedit + k]; idx += (tref(q.x) + tref(q.y)) + (tref(q.z) + tref(q.w)); }
      if (nq >= 2) { const int4 q = quad[2 * nedit + k]; idx += (tref(q.x) + tref(q.y)) + (tref(q.z) + tref(q.w)); }
      if (nq >= 3) { const int4 q = quad[3 * nedit + k]; idx += (tref(q.x) + tref(q.y)) + (tref(q.z) + tref(q.w)); }
      p = H.h[idx];
      kind = op == 6 ? E_DEL : E_ADD;
    } else if (op == 2) {
      p = arg;
      kind = E_GDEL;
    } else if (op == 3) {
      bool on;
      if (cnt <= 1) {
        on = cnt == 0 || in_mask(latv[q0.z], q0.w);
      } else {
        const int32_t *e = fs + q0.z;
        on = true;
        for (int c = 0; c < cnt && on; c++) on = in_mask(ref_value(e[2 + c], latv), e[2 + cnt + c]);
      }
      p = on ? arg : 0;
      kind = E_ADD;
    } else {
      const int32_t *e = fs + q0.z;
      p = nli_refs(H, cnt, e[2], e[3], e + 4, latv);
      kind = op == 4 ? E_DEL : E_ADD;
    }
    if (p == 0) continue;
    const int site = latsite[q0.y];
    int32_t *a1 = v.as1 + (size_t)(p - 1) * v.stride;
    int32_t *a2 = v.as2 + (size_t)(p - 1) * v.stride;
    if (kind == E_ADD) {  // add_proc (base.mpy:268-302)
      const int n = v.ns[p - 1] + 1;
      if (n >= v.stride) return ST_TABLE;  // a full list: tables out of step with the lattice
      v.ns[p - 1] = n;
      a1[n] = site;
      a2[site] = n;
    } else {  // del_proc (base.mpy:211-265), guarded or not
      const int m = a2[site];
      if (m == 0) {
        if (kind == E_DEL) return ST_TABLE;  // nli names a process that is not there
        continue;
      }
      const int n = v.ns[p - 1];
      if (!KMC_IN(m, 1, n)) return ST_TABLE;
      if (m < n) {
        const int last = a1[n];
        if (!KMC_IN(last, 1, v.stride - 1)) return ST_TABLE;
        a1[m] = last;
        a1[n] = 0;
        a2[last] = m;
      } else {
        a1[m] = 0;
      }
      a2[site] = 0;
      v.ns[p - 1] = n - 1;
    }
    if (p - 1 < v.minp) v.minp = p - 1;
  }
  for (int i = 0; i < nwr; i++) v.lat[latsite[wr[2 * i]] - 1] = (int8_t)wr[2 * i + 1];
  return ST_OK;
}

// Defined in the one translation unit that defines KMC_DEFINE_SOLO_KERNEL (kmc_solo.cu).
// PP = the model's process count exactly, so every loop over processes unrolls to its
// true length and the vectors stay in registers; __maxnreg__ gives the one warp of the
// block the registers that takes without spills.  ONCHIP: the launch staged the program
// and every trajectory's lattice and tables in shared memory, so every table pointer is
// a shared-memory one and its accesses compile to shared-memory loads and stores.
#ifdef KMC_DEFINE_SOLO_KERNEL
template <int PP, bool ONCHIP>
__global__ void __maxnreg__(224) kmc_solo_kernel(RunArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Group<32> grp;
  const int lane = grp.gl;
  const int item = blockIdx.x;
  if (item >= a.n) return;
  const ModelDev M = a.models[a.model];
  constexpr int P = PP;
  const int slot = a.list[item];
  const int64_t nsteps = a.steps[item];
  SlotDev &S = a.slots[slot];
  if (S.status != ST_OK || S.model != a.model || M.P != PP) return;
  SoloSmem &sm = *reinterpret_cast<SoloSmem *>(smem_raw);
  const size_t prog_b = ((size_t)a.prog_words * 4 + 15) / 16 * 16;
  int32_t *prog_s = reinterpret_cast<int32_t *>(smem_raw + sizeof(SoloSmem));
  unsigned char *ts = smem_raw + sizeof(SoloSmem) + prog_b;
  for (int i = lane; i < a.prog_words; i += 32) prog_s[i] = M.prog[i];
  const int stride = S.V + 1;
  View v;
  v.lat = S.lat;
  v.as1 = S.as1;
  v.as2 = S.as2;
  // the host plans ONCHIP only when the program and every listed trajectory fit
  constexpr bool on_chip = ONCHIP;
  const size_t lat_b = ((size_t)S.V + 15) / 16 * 16, tab_b = (size_t)P * stride * 4;
  if (on_chip) {
    v.lat = reinterpret_cast<int8_t *>(ts);
    v.as1 = reinterpret_cast<int32_t *>(ts + lat_b);
    v.as2 = reinterpret_cast<int32_t *>(ts + lat_b + (tab_b + 15) / 16 * 16);
    group_copy(v.lat, S.lat, S.V, grp);
    group_copy(v.as1, S.as1, tab_b, grp);
    group_copy(v.as2, S.as2, tab_b, grp);
  }
  const int32_t *prog = ONCHIP ? prog_s : (a.prog_words ? prog_s : M.prog);
  v.ns = sm.ns;
  v.prog = prog;
  v.g.X = S.X; v.g.Y = S.Y; v.g.Z = S.Z; v.g.spuck = M.spuck;
  v.stride = stride;
  v.backend = M.backend;
  v.P = P;
  v.off_groups = M.off_groups;
  v.collect = false;
  v.minp = P;
  v.err = ST_OK;
  Hot H;
  H.h = prog + M.off_hot;
  H.grp = M.hot_grp;
  H.tab = M.hot_tab;
  H.nspecies = M.nspecies;
  const bool fast_ok = a.fast && M.off_hot != 0 && S.V <= FAST_MAXV &&
                       (M.reach_x == 0 || S.X > 2 * M.reach_x) && (M.reach_y == 0 || S.Y > 2 * M.reach_y) &&
                       (M.reach_z == 0 || S.Z > 2 * M.reach_z);
  // the process vectors in registers (every index a compile-time constant)
  double rates_r[PP], accum_r[PP], term_r[PP];
  long long ps_r[PP];
  int32_t n0_r[PP];
  bool neg_rate = false;
#pragma unroll
  for (int i = 0; i < PP; i++) {
    rates_r[i] = S.rates[i];
    accum_r[i] = S.accum[i];
    n0_r[i] = S.nsites[i];
    term_r[i] = __dmul_rn((double)n0_r[i], rates_r[i]);
    ps_r[i] = S.procstat[i];
    neg_rate |= __double_as_longlong(rates_r[i]) < 0;
  }
  // the running sums of the clock and integ_rates: lane 0 kmc_time, lane 1 + i process
  // i's integ_rates, advanced once per batch of steps (kmc_time is read by no step)
  double run_sum = lane == 0 ? S.kmc_time : (lane <= P ? S.integ[lane - 1] : 0.0);
  // with every rate >= +0 every term n*r is >= +0, so is every partial sum, and adding
  // a +0 term leaves a sum >= +0 unchanged bit for bit: the chain skips those adds
  const bool skip_zero = !neg_rate;
  if (lane < P) sm.ns[lane] = S.nsites[lane];
  if (lane == 0) {
    sm.status = ST_OK;
    sm.used = 0;
    sm.from = S.accum_from;
  }
  FastDiv div_spuck, div_x, div_y;
  div_spuck.init(M.spuck);
  div_x.init(S.X);
  div_y.init(S.Y);
  double dt = S.kmc_time_step;
  int64_t kstep = S.kmc_step;
  uint64_t rbase[4] = {S.rng[0], S.rng[1], S.rng[2], S.rng[3]};
  const int rng_kind = S.rng_kind;
  grp.sync();

  int64_t k = 0;
  int status = ST_OK;
  int used = 0;  // draws of the current batch taken
#ifdef KMC_PHASE_TIMING
  // lane 0's cycles per phase of the step (builds with KMC_PHASE_TIMING only): 0 draws
  // and the previous batch's clock and integ, 1 accum, 2 bisection and site, 3 trace,
  // 4 site coordinates, 5 run_proc_nr, 6 term refresh
  long long ph[7] = {0, 0, 0, 0, 0, 0, 0};
  long long tp = clock64();
#define SOLO_PHASE(i)                 \
  do {                                \
    const long long now_ = clock64(); \
    ph[i] += now_ - tp;               \
    tp = now_;                        \
  } while (0)
#else
#define SOLO_PHASE(i) \
  do {                \
  } while (0)
#endif
  while (k < nsteps && status == ST_OK) {
    if (a.cancel && grp.any(*a.cancel != 0)) { status = ST_CANCELLED; break; }  // one decision for the warp
    // every lane draws one step of the next batch
    if (k > 0) {
      if (rng_kind == RNG_GFORTRAN) {
        for (int d = 0; d < 96; d++) xoshiro_next(rbase[0], rbase[1], rbase[2], rbase[3]);
      } else {
        rbase[0] += 32;
      }
    }
    {
      uint64_t st[4] = {rbase[0], rbase[1], rbase[2], rbase[3]};
      if (rng_kind == RNG_GFORTRAN) {
        for (int d = 0; d < 3 * lane; d++) xoshiro_next(st[0], st[1], st[2], st[3]);
      } else {
        st[0] += lane;
      }
      double rt, rp, rs;
      draw3(rng_kind, st, S.seed, S.traj, rt, rp, rs);
      sm.nl[lane] = -log(rt);
      sm.rp[lane] = rp;
      sm.rs[lane] = rs;
    }
    grp.sync();
    const int nb = (int)min((int64_t)32, nsteps - k);
    if (lane == 0) {
      int from = sm.from, b = 0, nclk = 0;
      SOLO_PHASE(0);
      for (; b < nb; b++) {
        const double ran_proc = sm.rp[b], ran_site = sm.rs[b];
        used = b + 1;
        // update_accum_rate from the first stale entry (base.mpy:603-623)
        if (from < P) {
          double acc = 0.0;
#pragma unroll
          for (int i = 0; i < PP; i++) {
            if (i >= from) {
              if (i == 0) {
                acc = term_r[0];
              } else {
                if (i == from) acc = accum_r[i - 1];
                if (!(skip_zero && __double_as_longlong(term_r[i]) == 0)) acc = __dadd_rn(acc, term_r[i]);
              }
              accum_r[i] = acc;
            }
          }
        }
        from = P;
        const double total = accum_r[PP - 1];
        const long long tbits = __double_as_longlong(total);
        if (!(tbits > 0 && tbits < 0x7FF0000000000000LL)) { status = ST_DEADLOCK; break; }
        SOLO_PHASE(1);
        // determine_procsite (base.mpy:1075-1120, 1234-1338): the first process whose
        // accumulated rate exceeds ran_proc * total, or reaches total
        const long long vbits = __double_as_longlong(__dmul_rn(ran_proc, total));
        int proc = P - 1;
#pragma unroll
        for (int i = PP - 1; i >= 0; i--) {
          const long long ab = __double_as_longlong(accum_r[i]);
          if (ab > vbits || ab == tbits) proc = i;
        }
        const int n = sm.ns[proc];
        if (n <= 0) { status = ST_DEADLOCK; break; }
        const long long qb = __double_as_longlong(__dadd_rn(1.0, __dmul_rn(ran_site, int_to_double(n))));
        const int qe = (int)(qb >> 52) - 1023;
        int idx = (int)((((unsigned long long)qb & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull) >> (52 - qe));
        if (idx > n) idx = n;
        if (!KMC_IN(n, 1, S.V)) { status = ST_TABLE; break; }
        const int site = v.as1[(size_t)proc * stride + idx];
        const int fs_off = fast_ok ? H.h[proc] : 0;
#pragma unroll
        for (int i = 0; i < PP; i++)
          if (i == proc) ps_r[i] += 1;  // increment_procstat
        SOLO_PHASE(2);
        // update_clocks and update_integ_rate: this step's total rate and terms are kept,
        // and the sums are advanced for the whole batch after it (below), in step order
        auto clock_integ = [&]() {
          sm.tot[b] = total;
#pragma unroll
          for (int i = 0; i < PP; i++) sm.thist[b][i] = term_r[i];
          kstep += 1;
          nclk = b + 1;
        };
        if (a.trace) { a.trace[2 * (k + b)] = proc + 1; a.trace[2 * (k + b) + 1] = site; }
        if (site < 1 || site > S.V) { clock_integ(); status = ST_TABLE; break; }
        SOLO_PHASE(3);
        int bx, by, bz;
        {  // calculate_nr2lattice (lattice.mpy:177-210)
          const unsigned c = div_spuck.div((unsigned)(site - 1));
          const unsigned r = div_x.div(c);
          bx = (int)(c - (unsigned)S.X * r);
          const unsigned zq = div_y.div(r);
          by = (int)(r - (unsigned)S.Y * zq);
          bz = (int)zq;
        }
        SOLO_PHASE(4);
        int err;
        int minp;
        if (fs_off) {
          v.minp = P;
          v.err = ST_OK;
          err = solo_fast_stream(v, H, H.h + fs_off, bx, by, bz, sm.latv, sm.latsite);
          minp = v.minp;
        } else {
          View vv = v;  // the interpreter takes its view by reference: a copy keeps v in registers
          vv.minp = P;
          vv.err = ST_OK;
          run_stream(vv, prog[M.off_proc + proc], bx, by, bz);
          err = vv.err;
          minp = vv.minp;
        }
        SOLO_PHASE(5);
        clock_integ();
        if (err) { status = err; break; }
        int first = P;
#pragma unroll
        for (int i = 0; i < PP; i++) {
          if (i >= minp) {
            const int nn = sm.ns[i];
            if (nn != n0_r[i]) {
              term_r[i] = __dmul_rn(int_to_double(nn), rates_r[i]);
              n0_r[i] = nn;
              if (first == P) first = i;
            }
          }
        }
        from = first;
        SOLO_PHASE(6);
      }
      sm.from = from;
      sm.status = status;
      sm.used = used;
      sm.nclk = nclk;
    }
    grp.sync();
    status = sm.status;
    used = sm.used;
    {
      // the batch's clock and integ_rates (base.mpy:626-645, 1123-1161), as
      // kmc_run_kernel computes them: kmc_time_step = -log(r) times the reciprocal of the
      // total rate, one step per lane; then, step by step, kmc_time += kmc_time_step on
      // lane 0 (its term is 1, and 1 * x is x exactly) and integ(i) += term(i) *
      // kmc_time_step on lane 1 + i, one instruction stream for both
      const int nclk = sm.nclk;
      if (lane < nclk) sm.dtb[lane] = __dmul_rn(sm.nl[lane], __drcp_rn(sm.tot[lane]));
      grp.sync();
      const int ti = lane >= 1 && lane <= P ? lane - 1 : 0;
      for (int j = 0; j < nclk; j++) {
        const double d = sm.dtb[j];
        const double term = lane == 0 ? 1.0 : sm.thist[j][ti];
        run_sum = __dadd_rn(run_sum, __dmul_rn(term, d));
      }
      if (nclk > 0) dt = sm.dtb[nclk - 1];
      grp.sync();
    }
    k += nb;
  }
  // random state after the draws actually used: `used` draws of the last batch
  if (k > 0 || used > 0) {
    if (rng_kind == RNG_GFORTRAN) {
      for (int d = 0; d < 3 * used; d++) xoshiro_next(rbase[0], rbase[1], rbase[2], rbase[3]);
    } else {
      rbase[0] += used;
    }
  }
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < PP; i++) {
      S.procstat[i] = ps_r[i];
      S.nsites[i] = sm.ns[i];
      S.accum[i] = accum_r[i];
    }
  }
  if (lane >= 1 && lane <= P) S.integ[lane - 1] = run_sum;
  if (on_chip) {
    group_copy(S.lat, v.lat, S.V, grp);
    group_copy(S.as1, v.as1, tab_b, grp);
    group_copy(S.as2, v.as2, tab_b, grp);
  }
#ifdef KMC_PHASE_TIMING
  if (lane == 0 && a.phase)
    for (int i = 0; i < 7; i++) atomicAdd(&a.phase[i], (unsigned long long)ph[i]);
#endif
#undef SOLO_PHASE
  if (lane == 0) {
    S.kmc_time = run_sum;
    S.kmc_time_step = dt;
    S.kmc_step = kstep;
    S.rng[0] = rbase[0]; S.rng[1] = rbase[1]; S.rng[2] = rbase[2]; S.rng[3] = rbase[3];
    S.accum_from = sm.from;
    S.status = status;
  }
}
#endif  // KMC_DEFINE_SOLO_KERNEL

}  // namespace kmc

namespace kmc_host {
// Host stubs of the step kernel variants, by processes per lane (np), edit rounds (r) and
// lanes per trajectory; null for a variant that is not built.
const void *run_kernel_g32(int np, int r);
const void *run_kernel_g16(int np, int r);
// Host stub of the solo kernel for a model of P processes (null beyond SOLO_PMAX).
const void *solo_kernel(int P, bool onchip);
}  // namespace kmc_host
