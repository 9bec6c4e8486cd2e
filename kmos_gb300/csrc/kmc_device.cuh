// kmc_device.cuh -- device data structures and the op-program interpreter of the
// GB300 lattice-kMC step engine.
//
// State of one trajectory ("slot") lives in one block of the pool's HBM arena:
//   lat     int8   [V]          species per site (null species -1 or nspecies)
//   as1     int32  [P][V+1]     avail_sites(p, i, 1): the i-th site that can do p
//   as2     int32  [P][V+1]     avail_sites(p, s, 2): position of site s in as1[p], 0 = absent
//   rates, integ, accum double [P];  nsites int32 [P];  procstat int64 [P]
// The reference keeps avail_sites(nr_of_proc, volume, 2) column-major with the process
// index fastest (base.mpy:648-744); here each process owns two contiguous rows so a
// trajectory's edits for one process stay within one row.  Values and the order of
// entries are exactly the reference's (1-based sites and positions).
#pragma once
#include <stdint.h>

namespace kmc {

enum Op { OP_END = 0, OP_REPLACE = 1, OP_GDEL = 2, OP_ADD = 3, OP_LI_DEL = 4, OP_LI_ADD = 5, OP_STRIP = 6 };

enum Status {
  ST_OK = 0, ST_ARG = 1, ST_SPECIES = 2, ST_DEADLOCK = 3, ST_TABLE = 4, ST_PROGRAM = 5,
  ST_CANCELLED = 8
};

enum Rng { RNG_GFORTRAN = 0, RNG_PHILOX = 1 };

// Every table and lattice index a step computes from table contents is checked in builds
// with KMC_DEBUG: out of range, the step stops with ST_TABLE instead of touching memory
// outside its slot.  The device-side counterpart of the host's program and state checks
// (which make these indices in range by construction); off in the product build.
#ifdef KMC_DEBUG
#define KMC_IN(x, lo, hi) ((x) >= (lo) && (x) <= (hi))
#else
#define KMC_IN(x, lo, hi) true
#endif

struct ModelDev {
  const int32_t *prog;
  int32_t len, backend, P, nspecies, null_species, spuck, ngroups;
  int32_t off_proc, off_touch, off_groups, off_site_layer, off_site_default, max_k;
  int32_t off_hot, hot_len, hot_grp, hot_tab, reach_x, reach_y, reach_z;
  int32_t max_nedit;  // most edits of any fast stream (selects the 3- or 4-round kernel)
};

struct __align__(16) SlotDev {
  int8_t *lat;
  int32_t *as1;
  int32_t *as2;
  double *rates;
  double *integ;
  double *accum;
  int32_t *nsites;
  int64_t *procstat;
  int32_t X, Y, Z, V;
  int32_t model, P, layer, status;
  double kmc_time, kmc_time_step;
  int64_t kmc_step;
  uint64_t rng[4];          // xoshiro256** state, or rng[0] = Philox draw counter
  int32_t rng_kind, accum_from;
  uint32_t seed, traj;
};

// ------------------------------------------------------------------ random numbers
// gfortran stream: xoshiro256** (Blackman & Vigna 2018) with the state libgfortran's
// RANDOM_SEED(PUT=) builds from 32-bit seed words all equal to the kmos seed
// (libgfortran/intrinsics/random.c, GCC >= 7); a real(8) draw is (next() >> 11) * 2^-53.
__host__ __device__ inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

__host__ __device__ inline uint64_t xoshiro_next(uint64_t &s0, uint64_t &s1, uint64_t &s2, uint64_t &s3) {
  const uint64_t result = rotl64(s1 * 5, 7) * 9;
  const uint64_t t = s1 << 17;
  s2 ^= s0;
  s3 ^= s1;
  s1 ^= s2;
  s0 ^= s3;
  s2 ^= t;
  s3 = rotl64(s3, 45);
  return result;
}

__host__ __device__ inline void gfortran_seed(uint64_t s[4], int32_t seed) {
  const uint64_t w = ((uint64_t)(uint32_t)seed << 32) | (uint64_t)(uint32_t)seed;
  s[0] = w ^ 0xbd0c5b6e50c2df49ULL;
  s[1] = w ^ 0xd46061cd46e1df38ULL;
  s[2] = w ^ 0xbb4f4d4ed6103544ULL;
  s[3] = w ^ 0x114a583d0756ad39ULL;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
// 1, 2, 3", SC'11).
__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
#ifdef __CUDA_ARCH__
    const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
#else
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

__host__ __device__ inline double u53_closed0(uint64_t x) {  // [0, 1): gfortran real(8)
  return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}
__host__ __device__ inline double u53_open(uint32_t hi, uint32_t lo) {  // (0, 1)
  const uint64_t x = ((uint64_t)hi << 32) | lo;
  return ((double)(x >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

// Three draws (ran_time, ran_proc, ran_site) of one step.
__host__ __device__ inline void draw3(int kind, uint64_t rng[4], uint32_t seed, uint32_t traj,
                                      double &r0, double &r1, double &r2) {
  if (kind == RNG_GFORTRAN) {
    r0 = u53_closed0(xoshiro_next(rng[0], rng[1], rng[2], rng[3]));
    r1 = u53_closed0(xoshiro_next(rng[0], rng[1], rng[2], rng[3]));
    r2 = u53_closed0(xoshiro_next(rng[0], rng[1], rng[2], rng[3]));
  } else {
    uint32_t a[4] = {(uint32_t)rng[0], (uint32_t)(rng[0] >> 32), 0u, 0u};
    uint32_t b[4] = {(uint32_t)rng[0], (uint32_t)(rng[0] >> 32), 1u, 0u};
    philox4x32_10(a, seed, traj);
    philox4x32_10(b, seed, traj);
    r0 = u53_open(a[0], a[1]);
    r1 = u53_open(a[2], a[3]);
    r2 = u53_open(b[0], b[1]);
    rng[0] += 1;
  }
}

// ---------------------------------------------------------------- lattice mapping
__host__ __device__ inline int wrapc(int v, int n) {
  if (v >= n) { v -= n; if (v >= n) v %= n; }
  else if (v < 0) { v += n; if (v < 0) { v %= n; if (v < 0) v += n; } }
  return v;
}

// Unpacks a program coordinate (dx, dy, dz as signed bytes, n as an unsigned byte)
// relative to base cell (bx, by, bz) into a 1-based site index
// (lattice.mpy:146-175 calculate_lattice2nr with periodic modulo).
struct Geometry {
  int X, Y, Z, spuck;
  __host__ __device__ inline int site(int bx, int by, int bz, int32_t w) const {
    const uint32_t u = (uint32_t)w;
    const int dx = (int8_t)(u & 0xFF), dy = (int8_t)((u >> 8) & 0xFF), dz = (int8_t)((u >> 16) & 0xFF);
    const int n = (int)(u >> 24);
    return spuck * (wrapc(bx + dx, X) + X * (wrapc(by + dy, Y) + Y * wrapc(bz + dz, Z))) + n;
  }
  // site() for offsets smaller than the lattice in every axis (the fast path's
  // precondition): one conditional add or subtract per axis instead of a modulo
  __host__ __device__ inline int site_near(int bx, int by, int bz, int32_t w) const {
    const uint32_t u = (uint32_t)w;
    int x = bx + (int8_t)(u & 0xFF), y = by + (int8_t)((u >> 8) & 0xFF), z = bz + (int8_t)((u >> 16) & 0xFF);
    x += x < 0 ? X : 0;
    x -= x >= X ? X : 0;
    y += y < 0 ? Y : 0;
    y -= y >= Y ? Y : 0;
    z += z < 0 ? Z : 0;
    z -= z >= Z ? Z : 0;
    return spuck * (x + X * (y + Y * z)) + (int)(u >> 24);
  }
  __host__ __device__ inline void cell(int bx, int by, int bz, int32_t w, int &cx, int &cy, int &cz) const {
    const uint32_t u = (uint32_t)w;
    cx = bx + (int8_t)(u & 0xFF);
    cy = by + (int8_t)((u >> 8) & 0xFF);
    cz = bz + (int8_t)((u >> 16) & 0xFF);
  }
  // calculate_nr2lattice (lattice.mpy:177-210)
  __host__ __device__ inline void coords(int nr, int &x, int &y, int &z, int &n) const {
    const int c = (nr - 1) / spuck;
    n = nr - spuck * c;
    x = c % X;
    const int r = c / X;
    y = r % Y;
    z = r / Y;
  }
};

// n / d by a multiply and a shift for 0 <= n < 2^31 (Granlund & Montgomery, "Division by
// invariant integers using multiplication", PLDI 1994): with p = 32 + ceil(log2 d) and
// m = ceil(2^p / d), m*d - 2^p < d <= 2^(p-32), so floor(n*m / 2^p) = floor(n / d) for
// every n < 2^32; n < 2^31 keeps n*m below 2^64.
struct FastDiv {
  unsigned long long m;
  int p;
  __host__ __device__ inline void init(unsigned d) {
    int l = 0;
    while (l < 31 && (1u << l) < d) l++;
    p = 32 + l;
    m = ((1ull << p) + d - 1) / d;
  }
  __host__ __device__ inline unsigned div(unsigned n) const { return (unsigned)(((unsigned long long)n * m) >> p); }
};

// (double)n for 0 <= n < 2^31 from its bit pattern: integer instructions only, so the
// conversion takes no slot of the FP64 pipe.
__device__ inline double int_to_double(int n) {
  if (n <= 0) return 0.0;
  const int e = 31 - __clz(n);
  return __longlong_as_double((long long)(((unsigned long long)(1023 + e) << 52) |
                                          (((unsigned long long)n << (52 - e)) & 0xFFFFFFFFFFFFFull)));
}

__host__ __device__ inline bool in_mask(int species, int32_t mask) {
  const int bit = species < 0 ? 31 : species;
  return ((uint32_t)mask >> bit) & 1u;
}

// One trajectory's tables as seen by the serial interpreter.
struct View {
  int8_t *lat;
  int32_t *as1;
  int32_t *as2;
  int32_t *ns;          // nr_of_sites (shared memory in the step kernel)
  const int32_t *prog;
  Geometry g;
  int stride;           // V + 1
  int backend, P, off_groups;
  int minp;             // smallest 0-based process whose nr_of_sites changed
  int err;
  bool collect;         // initialisation: only flag (p, site) in as2
};

// add_proc (base.mpy:268-302; base_lat_int.mpy:292-311 takes proc 0 as a no-op)
__device__ inline void add_proc(View &v, int p, int site) {
  if (p == 0) return;
  int32_t *a1 = v.as1 + (size_t)(p - 1) * v.stride;
  int32_t *a2 = v.as2 + (size_t)(p - 1) * v.stride;
  if (!KMC_IN(site, 1, v.stride - 1)) { v.err = ST_TABLE; return; }
  if (v.collect) { a2[site] = 1; return; }
  const int n = v.ns[p - 1] + 1;
  // a list can hold every site once; more entries mean the tables no longer match the
  // lattice (a species replaced without a touch-up): stop instead of leaving the row
  if (n >= v.stride) { v.err = ST_TABLE; return; }
  v.ns[p - 1] = n;
  a1[n] = site;
  a2[site] = n;
  if (p - 1 < v.minp) v.minp = p - 1;
}

// del_proc (base.mpy:211-265): swap-remove, in the reference's order of writes.
__device__ inline void del_proc(View &v, int p, int site) {
  if (p == 0) return;
  int32_t *a1 = v.as1 + (size_t)(p - 1) * v.stride;
  int32_t *a2 = v.as2 + (size_t)(p - 1) * v.stride;
  if (!KMC_IN(site, 1, v.stride - 1)) { v.err = ST_TABLE; return; }
  const int m = a2[site];
  if (m == 0) { v.err = ST_TABLE; return; }
  const int n = v.ns[p - 1];
  if (!KMC_IN(n, m, v.stride - 1)) { v.err = ST_TABLE; return; }
  if (m < n) {
    const int last = a1[n];
    if (!KMC_IN(last, 1, v.stride - 1)) { v.err = ST_TABLE; return; }
    a1[m] = last;
    a1[n] = 0;
    a2[last] = m;
  } else {
    a1[m] = 0;
  }
  a2[site] = 0;
  v.ns[p - 1] = n - 1;
  if (p - 1 < v.minp) v.minp = p - 1;
}

__device__ inline bool can_do(const View &v, int p, int site) {
  return v.as2[(size_t)(p - 1) * v.stride + site] != 0;
}

// nli_<group>(cell) (kmos/io/__init__.py:1985-2057): the member of the group whose
// conditions all hold (the last one on identical paths), or 0.
__device__ inline int nli(const View &v, int g, int cx, int cy, int cz) {
  const int32_t *rec = v.prog + v.prog[v.off_groups + g];
  const int M = rec[0], K = rec[1];
  const int32_t *coords = rec + 2;
  uint32_t bits[16];
  for (int k = 0; k < K && k < 16; k++) {
    const int s = v.lat[v.g.site(cx, cy, cz, coords[k]) - 1];
    bits[k] = 1u << (s < 0 ? 31 : s);
  }
  int result = 0;
  const int32_t *mem = coords + K;
  for (int m = 0; m < M; m++, mem += 1 + K) {
    bool ok = true;
    for (int k = 0; k < K; k++) ok = ok && ((uint32_t)mem[1 + k] & bits[k]);
    if (ok) result = mem[0];
  }
  return result;
}

// Executes one op stream (a process's run_proc_nr body or a touch-up) at base cell
// (bx, by, bz), in program order.
__device__ inline void run_stream(View &v, int pos, int bx, int by, int bz) {
  const int32_t *w = v.prog;
  for (;;) {
    if (v.err) return;
    const uint32_t h = (uint32_t)w[pos];
    const int op = h & 0xFF, cnt = (h >> 8) & 0xFF, arg = (h >> 16) & 0xFFFF;
    switch (op) {
      case OP_END:
        return;
      case OP_REPLACE: {
        const int site = v.g.site(bx, by, bz, w[pos + 1]);
        if (!in_mask(v.lat[site - 1], w[pos + 2])) { v.err = ST_SPECIES; return; }
        v.lat[site - 1] = (int8_t)w[pos + 3];
        pos += 4;
        break;
      }
      case OP_GDEL: {
        const int site = v.g.site(bx, by, bz, w[pos + 1]);
        if (can_do(v, arg, site)) del_proc(v, arg, site);
        pos += 2;
        break;
      }
      case OP_ADD: {
        const int site = v.g.site(bx, by, bz, w[pos + 1]);
        bool ok = true;
        for (int c = 0; c < cnt && ok; c++)
          ok = in_mask(v.lat[v.g.site(bx, by, bz, w[pos + 2 + 2 * c]) - 1], w[pos + 3 + 2 * c]);
        if (ok) add_proc(v, arg, site);
        pos += 2 + 2 * cnt;
        break;
      }
      case OP_LI_DEL:
      case OP_LI_ADD: {
        int cx, cy, cz;
        v.g.cell(bx, by, bz, w[pos + 1], cx, cy, cz);
        const int p = nli(v, arg, cx, cy, cz);
        const int site = v.g.site(bx, by, bz, w[pos + 1]);
        if (op == OP_LI_DEL) del_proc(v, p, site); else add_proc(v, p, site);
        pos += 2;
        break;
      }
      case OP_STRIP: {
        const int site = v.g.site(bx, by, bz, w[pos + 1]);
        if (!v.collect)
          for (int p = 1; p <= v.P; p++)
            if (can_do(v, p, site)) del_proc(v, p, site);
        pos += 2;
        break;
      }
      default:
        v.err = ST_PROGRAM;
        return;
    }
  }
}

}  // namespace kmc

// ==================================================================================
// Fast step: gather -> parallel evaluation -> per-process replay
// ==================================================================================
// A process's resolved fast stream (kmos_gb300/program.py) lists every lattice
// coordinate it reads or writes as a slot; every condition reads a slot's value from
// before the step or a constant, so the edits of one step are evaluated in parallel:
//   1. lanes load every slot's species and check the old species of the replaces;
//   2. lanes evaluate the edits (guarded dels, adds, nli dels / adds; one edit per lane,
//      its record read as 16-byte quads), issue the loads the dels will need
//      (avail_sites(p, site, 2) and the top entries of avail_sites(p, :, 1)), and a
//      ballot compacts the edits that happen into a list in program order;
//   3. edits of different processes touch different rows of avail_sites, so each lane
//      takes one process and replays that process's edits in program order with the
//      reference's add_proc / del_proc arithmetic, writing through to memory and
//      remembering the writes later reads need in a small lane-private log (in a
//      dels-first stream only the entries its dels move);
//   4. lanes write the final species of the replaced slots.
// The edits and their order within each process are those of the serial interpreter;
// edits of different processes commute.
namespace kmc {

constexpr int FAST_SLOTS = 128;
constexpr int FAST_EDITS = 128;  // largest fast stream: 4 rounds of 32 edits
constexpr int LOG_MAX = 8;    // lane-private write log entries (a multiple of 4)
constexpr int TAIL_MAX = 6;   // prefetched list-tail entries per process
constexpr int FAST_MAXV = (1 << 23) - 1;

enum EditKind { E_GDEL = 0, E_DEL = 1, E_ADD = 2 };

// Start of a fast stream's edit quads (stream-relative words): after the head, rounded
// up to 16 bytes.
__host__ __device__ inline int fast_rec_offset(int nlat, int nchk, int nwr) {
  return (4 + nlat + 2 * nchk + 2 * nwr + 3) & ~3;
}

// R rounds of 32 edits: the step kernel comes in R = 3 (streams of up to 96 edits, the
// common case) and R = 4 (up to 128, large lateral-interaction groups).  G lanes run one
// trajectory (32: a warp; 16: half a warp), each with its own write log.
template <int R, int G = 32, int TP = 32>
struct FastSmem {
  int32_t latv[FAST_SLOTS];
  int32_t latsite[FAST_SLOTS];
  int8_t ekind[32 * R];    // E_GDEL / E_DEL / E_ADD
  int16_t ep[32 * R];      // process, 0-based
  int32_t esite[32 * R];   // target site
  int32_t em[32 * R];      // prefetched avail_sites(p, site, 2) of del edits
  int32_t tail[TP][TAIL_MAX];  // avail_sites(p, n0 - j, 1), j < TAIL_MAX, for the TP processes of the kernel
  uint4 lkey4[LOG_MAX / 4][G];  // lane-private write logs, four keys per 16 bytes (lane-minor)
  int32_t lval[LOG_MAX][G];
};

// The hot section of a model program: fast streams, group records and nli tables with
// offsets relative to its start (shared memory when the block staged it).
struct Hot {
  const int32_t *h;
  int grp, tab, nspecies;
};

__device__ inline int ref_value(int32_t ref, const int32_t *latv) { return ref >= 0 ? latv[ref] : -ref - 2; }

// nli table code of a species: the species, or ns for the null species (-1); a value
// above ns (a lattice holding no valid species) maps to ns too, so a table index built
// from codes stays inside its table.
__device__ inline int species_code(int s, int ns) { return (int)min((unsigned)s, (unsigned)ns); }

// nli of one edit: table lookup when the group has one, else a member scan.  The edit
// carries the group's table and record offsets (hot-relative) and its K references.
__device__ inline int nli_refs(const Hot &H, int K, int toff, int roff, const int32_t *refs, const int32_t *latv) {
  if (toff) {
    const int base = H.nspecies + 1;
    int idx = 0, mul = 1;
#pragma unroll 4
    for (int k = 0; k < K; k++) {
      idx += species_code(ref_value(refs[k], latv), H.nspecies) * mul;
      mul *= base;
    }
    return H.h[toff + idx];
  }
  const int32_t *rec = H.h + roff;
  const int M = rec[0];
  int result = 0;
  const int32_t *mem = rec + 2 + K;
  for (int m = 0; m < M; m++, mem += 1 + K) {
    bool ok = true;
    for (int k = 0; k < K && ok; k++) ok = in_mask(ref_value(refs[k], latv), mem[1 + k]);
    if (ok) result = mem[0];
  }
  return result;
}

}  // namespace kmc
