// kmc_otf.cu -- the otf ("on-the-fly" rates) backend's step engine: the C-ABI
// kmc_otf_* (include/kmc_gb300.h) over a batch of independent trajectories of one model.
//
// Reference: kmos/fortran_src/base_otf.f90 and the otf code generator
// (kmos/io/__init__.py:2657-3723); the model program is kmos_gb300/otf.py's.
//
// State of trajectory t, process p (0-based), list position i (1-based), in HBM:
//   lat   int8   [T][V]            species per site
//   as1   int32  [T][P][V+1]       avail_sites(p, i, 1)
//   as2   int32  [T][P][V+1]       avail_sites(p, s, 2)
//   rm    double [T][P][V+1]       rates_matrix(p, i): the rate of list entry i
//   pm    double [T][P][V+1]       running sums of rm left to right: pm(i) = pm(i-1) + rm(i)
//   dirty int32  [T][P]            first position whose running sum is stale
//   ns, procstat, integ, accum, tot [T][P];  rates, userpar shared by the batch
// update_accum_rate (base_otf.f90:687-716) re-sums every list from its first entry each
// step; a running sum depends only on the entries before it, so only the sums from the
// first entry an event changed onwards are recomputed -- the values are the reference's
// left-to-right sums bit for bit, and pm is at once the accum_rates_proc array
// determine_procsite (base_otf.f90:1213-1277) searches.
//
// One warp per trajectory, eight per block; each block first copies the image -- the
// program, then the rate tables -- to its shared memory.  A step: lanes re-sum the stale
// lists (one process per lane, a serial chain each; a constant-rate process's sums come
// from its one-table row instead), lane 0 chains the process totals into accum_rates,
// every lane advances the clock and integ_rates of its processes, lane 0 picks the
// process and the entry (interval_search_real on accum_rates and on the chosen list's
// running sums), and the event runs (run_event): lane 0 writes the lattice, the lanes
// load the table positions and evaluate the add conditions and the rates (gr_<name>,
// io:2800-2965: a table lookup by bystander counts, or the rate program) in parallel,
// then every lane replays the guarded dels, rate updates and adds of its own processes
// in program order (ops of different processes touch different rows).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/kmc_gb300.h"
#include "kmc_device.cuh"
#include "kmc_host.h"
#include "kmc_reload.h"

namespace otfdev {
using namespace kmc;

constexpr int OTF_PMAX = 256;
constexpr int OTF_WARPS = 8;  // trajectories per block (two blocks per SM at 128 registers)
constexpr int OTF_NRMAX = 64;
constexpr int OTF_STACK = 16;
constexpr int OTF_AUX = 8;
enum { OP_UPDATE = 7 };
enum { I_END = 0, I_PUSH_BASE = 1, I_PUSH_PAR = 2, I_PUSH_NR = 3, I_PUSH_INT = 4, I_PUSH_CONST = 5,
       I_LOAD_AUX = 6, I_STORE_AUX = 7, I_STORE_RESULT = 8, I_ADD = 10, I_SUB = 11, I_MUL = 12,
       I_DIV = 13, I_NEG = 14, I_POWI = 15, I_POW = 16, I_EXP = 17, I_LOG = 18, I_SQRT = 19,
       I_ABS = 20, I_CVT = 21 };
enum { K_INT = 0, K_F32 = 1, K_F64 = 2 };

struct Traj {
  double kmc_time, kmc_time_step;
  int64_t kmc_step;
  uint64_t rng[4];
  uint32_t seed, traj;
  int32_t rng_kind, status;
};

struct Dev {
  const int32_t *prog;
  int P, nspecies, null_species, spuck, nuser, off_proc, off_touch, off_rate, off_site_layer, off_site_default;
  int X, Y, Z, V, T;
  int8_t *lat;
  int32_t *as1, *as2, *dirty, *ns;
  double *rm, *pm, *integ, *accum, *tot;
  int64_t *procstat;
  const double *rates, *userpar;
  Traj *traj;
  unsigned long long *phase;  // OTF_NPHASE cycle sums (KMC_PHASE_TIMING builds)
  int32_t prog_len;           // words of the image: the program, then the rate tables
  int32_t prog_staged;        // 1: each block copies the image to shared memory
  int32_t tab_index;          // image word of the P table-record offsets (-1: no table)
  int32_t tab_values;         // image word of the table values (doubles, 16-byte aligned)
  int32_t tab_entries;        // table values
  int32_t tab_on;             // 1: rate_of reads the tables
  int32_t uni_index;          // image word of the P constant-rate row numbers (-1: none)
  int32_t uni_on;             // 1: constant-rate processes' running sums come from usum
  double *usum;               // per constant-rate process: its running sums of 0..V entries
  int32_t ev_index;           // image word of the P event records (built by build_image)
};

// Cycle accounting of the step loop (builds with -DKMC_PHASE_TIMING only): lane 0 adds
// the clock64() time since its previous mark to phase i: 0 draws, 1 running sums and
// accum_rates, 2 clock and integ, 3 process and entry pick, 4 event: replaces and op list,
// 5 event: conditions and rates evaluated in parallel, 6 event: table replay.
constexpr int OTF_NPHASE = 8;
#ifdef KMC_PHASE_TIMING
#define OTF_MARK(i)                     \
  do {                                  \
    if ((threadIdx.x & 31) == 0) {      \
      const long long now_ = clock64(); \
      oph[i] += now_ - otp;             \
      otp = now_;                       \
    }                                   \
  } while (0)
#define OTF_PH_PARAMS , long long *oph, long long &otp
#define OTF_PH_ARGS , oph, otp
#else
#define OTF_MARK(i) \
  do {              \
  } while (0)
#define OTF_PH_PARAMS
#define OTF_PH_ARGS
#endif

// One trajectory's view.
struct View {
  const Dev *d;
  const int32_t *prog;  // the program: the block's shared-memory copy when staged
  int8_t *lat;
  int32_t *as1, *as2, *dirty, *ns;
  double *rm, *pm, *integ, *accum, *tot;
  int64_t *procstat;
  Geometry g;
  int stride, err;
  __device__ inline size_t row(int p) const { return (size_t)p * stride; }  // p 0-based
};

__device__ inline View view_of(const Dev &d, int t) {
  View v;
  v.d = &d;
  v.prog = d.prog;
  const size_t PV = (size_t)d.P * (d.V + 1);
  v.lat = d.lat + (size_t)t * d.V;
  v.as1 = d.as1 + (size_t)t * PV;
  v.as2 = d.as2 + (size_t)t * PV;
  v.rm = d.rm + (size_t)t * PV;
  v.pm = d.pm + (size_t)t * PV;
  v.dirty = d.dirty + (size_t)t * d.P;
  v.ns = d.ns + (size_t)t * d.P;
  v.integ = d.integ + (size_t)t * d.P;
  v.accum = d.accum + (size_t)t * d.P;
  v.tot = d.tot + (size_t)t * d.P;
  v.procstat = d.procstat + (size_t)t * d.P;
  v.g = Geometry{d.X, d.Y, d.Z, d.spuck};
  v.stride = d.V + 1;
  v.err = ST_OK;
  return v;
}

// ---------------------------------------------------------------- rate programs
// x ** m for an integer m by libgcc's __powidf2 / __powisf2 (right-to-left binary
// powering in the base's precision, the reciprocal for m < 0); integers as gfortran's
// pow_i4_i4.
__device__ inline double powi_kind(double xd, int32_t m, int kind) {
  uint32_t n = m < 0 ? 0u - (uint32_t)m : (uint32_t)m;
  if (kind == K_F32) {
    float x = (float)xd, y = (n & 1u) ? x : 1.0f;
    while (n >>= 1) { x = __fmul_rn(x, x); if (n & 1u) y = __fmul_rn(y, x); }
    return m < 0 ? (double)__fdiv_rn(1.0f, y) : (double)y;
  }
  if (kind == K_F64) {
    double x = xd, y = (n & 1u) ? x : 1.0;
    while (n >>= 1) { x = __dmul_rn(x, x); if (n & 1u) y = __dmul_rn(y, x); }
    return m < 0 ? __ddiv_rn(1.0, y) : y;
  }
  int32_t x = (int32_t)xd, y = (n & 1u) ? x : 1;
  while (n >>= 1) { x = (int32_t)((uint32_t)x * (uint32_t)x); if (n & 1u) y = (int32_t)((uint32_t)y * (uint32_t)x); }
  if (m < 0) return (y == 1 || y == -1) ? (double)((((uint32_t)0 - (uint32_t)m) & 1u) ? y : 1) : 0.0;
  return (double)y;
}

// The rate program of process p (code) with base_rate = rates(p) and the bystander
// counts nr: the body of gr_<p> (io:2800-2965) after its counting loop.
__device__ double rate_program(const Dev &d, const int32_t *code, int p, const int32_t *nr, int &err) {
  double st[OTF_STACK], aux[OTF_AUX], result = 0.0;
  for (int k = 0; k < OTF_AUX; k++) aux[k] = 0.0;
  int sp = 0;
  for (int pc = 0;;) {
    const uint32_t w = (uint32_t)code[pc++];
    const int op = w & 0xFF, kind = (w >> 8) & 0xFF, arg = (int)(w >> 16);
    switch (op) {
      case I_END: return result;
      case I_PUSH_BASE: st[sp++] = d.rates[p - 1]; break;
      case I_PUSH_PAR: st[sp++] = d.userpar[arg]; break;
      case I_PUSH_NR: st[sp++] = (double)nr[arg]; break;
      case I_PUSH_INT: st[sp++] = (double)code[pc++]; break;
      case I_PUSH_CONST:
        st[sp++] = __hiloint2double(code[pc + 1], code[pc]);
        pc += 2;
        break;
      case I_LOAD_AUX: st[sp++] = aux[arg]; break;
      case I_STORE_AUX: aux[arg] = st[--sp]; break;
      case I_STORE_RESULT: result = st[--sp]; break;
      case I_ADD: case I_SUB: case I_MUL: case I_DIV: {
        const double b2 = st[--sp], a = st[sp - 1];
        double r2;
        if (kind == K_INT) {
          const int32_t ia = (int32_t)a, ib = (int32_t)b2;
          r2 = op == I_ADD ? (double)(int32_t)((uint32_t)ia + (uint32_t)ib)
             : op == I_SUB ? (double)(int32_t)((uint32_t)ia - (uint32_t)ib)
             : op == I_MUL ? (double)(int32_t)((uint32_t)ia * (uint32_t)ib)
             : (ib == 0 ? 0.0 : (ib == -1 ? (double)(int32_t)(0u - (uint32_t)ia) : (double)(ia / ib)));
        } else if (kind == K_F32) {
          const float fa = (float)a, fb = (float)b2;
          r2 = op == I_ADD ? __fadd_rn(fa, fb) : op == I_SUB ? __fsub_rn(fa, fb)
             : op == I_MUL ? __fmul_rn(fa, fb) : __fdiv_rn(fa, fb);
        } else {
          r2 = op == I_ADD ? __dadd_rn(a, b2) : op == I_SUB ? __dsub_rn(a, b2)
             : op == I_MUL ? __dmul_rn(a, b2) : __ddiv_rn(a, b2);
        }
        st[sp - 1] = r2;
        break;
      }
      case I_NEG:
        st[sp - 1] = kind == K_INT ? (double)(int32_t)(0u - (uint32_t)(int32_t)st[sp - 1]) : -st[sp - 1];
        break;
      case I_POWI: { const double m = st[--sp]; st[sp - 1] = powi_kind(st[sp - 1], (int32_t)m, kind); break; }
      case I_POW: {
        const double b2 = st[--sp], a = st[sp - 1];
        st[sp - 1] = kind == K_F32 ? (double)powf((float)a, (float)b2) : pow(a, b2);
        break;
      }
      case I_EXP: st[sp - 1] = kind == K_F32 ? (double)expf((float)st[sp - 1]) : exp(st[sp - 1]); break;
      case I_LOG: st[sp - 1] = kind == K_F32 ? (double)logf((float)st[sp - 1]) : log(st[sp - 1]); break;
      case I_SQRT: st[sp - 1] = kind == K_F32 ? (double)__fsqrt_rn((float)st[sp - 1]) : __dsqrt_rn(st[sp - 1]); break;
      case I_ABS: st[sp - 1] = fabs(st[sp - 1]); break;
      case I_CVT:
        if (kind == K_INT && arg == K_F32) st[sp - 1] = (double)(float)(int32_t)st[sp - 1];
        break;
      default: err = ST_PROGRAM; return 0.0;
    }
  }
}

// The first word of process p's rate program (past its bystander list).
__device__ inline const int32_t *rate_code(const int32_t *prog, const Dev &d, int p) {
  const int32_t *r = prog + prog[d.off_rate + p - 1];
  const int nb = r[0];
  const int32_t *b = r + 4;
  for (int k = 0; k < nb; k++) b += 2 + 2 * b[1];
  return b;
}

// A site of the event's neighbourhood: Geometry::site_near when every offset of the
// program (an op's plus its bystanders') stays within one lattice period (NEAR, chosen on
// the host), Geometry::site otherwise.
template <bool NEAR>
__device__ __forceinline__ int gsite(const Geometry &g, int bx, int by, int bz, int32_t w) {
  return NEAR ? g.site_near(bx, by, bz, w) : g.site(bx, by, bz, w);
}

// gr_<p>(cell) evaluated: the bystander counts, then the rate program.  Out of line:
// with rate tables it runs only for the processes that have none, and a single copy
// keeps the step loop's code small.
__device__ __noinline__ double rate_counted(const Dev *dp, const int32_t *prog, const int8_t *lat, Geometry g, int p,
                                            int cx, int cy, int cz, int *err) {
  const Dev &d = *dp;
  const int32_t *r = prog + prog[d.off_rate + p - 1];
  const int nb = r[0], nv = r[1];
  int32_t nr[OTF_NRMAX];
  for (int k = 0; k < nv; k++) nr[k] = 0;
  const int32_t *b = r + 4;
  for (int k = 0; k < nb; k++) {
    const int sp = lat[g.site(cx, cy, cz, b[0]) - 1];
    const int npairs = b[1];
    for (int j = 0; j < npairs; j++)
      if (sp == b[2 + 2 * j]) nr[b[3 + 2 * j]] += 1;
    b += 2 + 2 * npairs;
  }
  int e = ST_OK;
  const double rate = rate_program(d, b, p, nr, e);
  *err = e;
  return rate;
}

// gr_<p>(cell).  With rate tables: a process's rate depends only on its bystander counts
// (rates and user parameters are fixed between launches), so the counts select an entry
// of the process's table, which otf_table_kernel filled with rate_program's value for
// those counts -- the same double the program gives here.  The table index is the counts
// in mixed radix: each bystander matching a pair adds the stride of that pair's
// variable.  Otherwise the counts are taken and the program run.
template <bool NEAR = false>
__device__ double rate_of(View &v, int p, int cx, int cy, int cz) {
  const Dev &d = *v.d;
  if (d.tab_on) {
    const int rec = v.prog[d.tab_index + p - 1];
    if (rec >= 0) {
      const int32_t *m = v.prog + rec;
      const int nv = m[1];
      const int nb = m[2 + nv];
      const int32_t *b = m + 3 + nv;
      int idx = m[0];
      for (int k = 0; k < nb; k++) {
        const int sp = v.lat[gsite<NEAR>(v.g, cx, cy, cz, b[0]) - 1];
        const int npairs = b[1];
        for (int j = 0; j < npairs; j++)
          if (sp == b[2 + 2 * j]) idx += b[3 + 2 * j];
        b += 2 + 2 * npairs;
      }
      return reinterpret_cast<const double *>(v.prog + d.tab_values)[idx];
    }
  }
  int err = ST_OK;
  const double rate = rate_counted(v.d, v.prog, v.lat, v.g, p, cx, cy, cz, &err);
  if (err) v.err = err;
  return rate;
}

// Fills the rate tables: thread e computes entry e -- the process whose table holds it,
// the counts its index encodes (mixed radix, first variable fastest), the program's rate.
__global__ void otf_table_kernel(Dev d, int32_t *img) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.tab_entries) return;
  for (int p0 = 0; p0 < d.P; p0++) {
    const int rec = img[d.tab_index + p0];
    if (rec < 0) continue;
    const int32_t *m = img + rec;
    const int nv = m[1];
    int size = 1;
    for (int k = 0; k < nv; k++) size *= m[2 + k];
    if (e < m[0] || e >= m[0] + size) continue;
    int32_t nr[OTF_NRMAX];
    int rem = e - m[0];
    for (int k = 0; k < nv; k++) {
      nr[k] = rem % m[2 + k];
      rem /= m[2 + k];
    }
    int err = 0;
    const double r = rate_program(d, rate_code(img, d, p0 + 1), p0 + 1, nr, err);
    reinterpret_cast<double *>(img + d.tab_values)[e] = r;
    return;
  }
}

// A process whose rate program reads no bystander count gives every list entry the same
// rate c, so while every entry holds the current c its running sums are
// pm(i) = fl(pm(i-1) + c) from pm(0) = 0: the same numbers for every trajectory and step.
// Row r of usum holds them for i = 0..V, filled here (one thread per such process) when
// the rates or user parameters change.
__global__ void otf_uniform_kernel(Dev d, const int32_t *img) {
  const int p0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (p0 >= d.P || d.uni_index < 0) return;
  const int row = img[d.uni_index + p0];
  if (row < 0) return;
  const int32_t none[1] = {0};
  int err = 0;
  const double c = rate_program(d, rate_code(img, d, p0 + 1), p0 + 1, none, err);
  double *u = d.usum + (size_t)row * (d.V + 1);
  double s = 0.0;
  u[0] = 0.0;
  for (int i = 1; i <= d.V; i++) {
    s = __dadd_rn(s, c);
    u[i] = s;
  }
}

// ---------------------------------------------------------------- table operations
__device__ inline void mark(View &v, int p0, int pos) {
  if (pos < v.dirty[p0]) v.dirty[p0] = pos;
}

// add_proc (base_otf.f90:286-331); m0 = avail_sites(p, site, 2) as the caller read it
__device__ inline void add_at(View &v, int p, int site, double rate, int m0) {
  const int p0 = p - 1;
  int32_t *a1 = v.as1 + v.row(p0), *a2 = v.as2 + v.row(p0);
  if (site < 1 || site > v.d->V || m0 != 0) { v.err = ST_TABLE; return; }
  const int n = v.ns[p0] + 1;
  if (n > v.d->V) { v.err = ST_TABLE; return; }
  v.ns[p0] = n;
  a1[n] = site;
  a2[site] = n;
  v.tot[p0] = __dadd_rn(v.tot[p0], rate);  // the running rates_matrix(p, V+1)
  v.rm[v.row(p0) + n] = rate;
  mark(v, p0, n);
}

__device__ inline void add_entry(View &v, int p, int site, double rate) {
  if (site < 1 || site > v.d->V) { v.err = ST_TABLE; return; }
  add_at(v, p, site, rate, v.as2[v.row(p - 1) + site]);
}

// del_proc (base_otf.f90:221-283): the last entry and its rate fill the hole; m =
// avail_sites(p, site, 2) as the caller read it.
__device__ inline void del_at(View &v, int p, int site, int m) {
  const int p0 = p - 1;
  int32_t *a1 = v.as1 + v.row(p0), *a2 = v.as2 + v.row(p0);
  double *r = v.rm + v.row(p0);
  const int n = v.ns[p0];
  if (m < 1 || m > n) { v.err = ST_TABLE; return; }
  v.tot[p0] = __dsub_rn(v.tot[p0], r[m]);
  if (m < n) {
    const int last = a1[n];
    if (last < 1 || last > v.d->V) { v.err = ST_TABLE; return; }
    a1[m] = last;
    a1[n] = 0;
    r[m] = r[n];
    r[n] = 0.0;
    a2[last] = m;
  } else {
    a1[m] = 0;
    r[m] = 0.0;
  }
  a2[site] = 0;
  v.ns[p0] = n - 1;
  mark(v, p0, m);
}

__device__ inline void del_entry(View &v, int p, int site) { del_at(v, p, site, v.as2[v.row(p - 1) + site]); }

__device__ inline bool can_do(const View &v, int p, int site) { return v.as2[v.row(p - 1) + site] != 0; }

// One op stream (run_proc_<name> or touchup_cell) at cell (bx, by, bz), serially.
__device__ void run_stream(View &v, int pos, int bx, int by, int bz) {
  const int32_t *w = v.prog;
  for (;;) {
    if (v.err) return;
    const uint32_t h = (uint32_t)w[pos];
    const int op = h & 0xFF, cnt = (h >> 8) & 0xFF, arg = (h >> 16) & 0xFFFF;
    switch (op) {
      case OP_END: return;
      case OP_REPLACE: {
        const int site = v.g.site(bx, by, bz, w[pos + 1]);
        if (!in_mask(v.lat[site - 1], w[pos + 2])) { v.err = ST_SPECIES; return; }
        v.lat[site - 1] = (int8_t)w[pos + 3];
        pos += 4;
        break;
      }
      case OP_GDEL: {
        const int site = v.g.site(bx, by, bz, w[pos + 1]);
        if (can_do(v, arg, site)) del_entry(v, arg, site);
        pos += 2;
        break;
      }
      case OP_ADD: {
        const int site = v.g.site(bx, by, bz, w[pos + 1]);
        bool ok = true;
        for (int c = 0; c < cnt && ok; c++)
          ok = in_mask(v.lat[v.g.site(bx, by, bz, w[pos + 2 + 2 * c]) - 1], w[pos + 3 + 2 * c]);
        if (ok) {
          int cx, cy, cz;
          v.g.cell(bx, by, bz, w[pos + 1], cx, cy, cz);
          add_entry(v, arg, site, rate_of(v, arg, cx, cy, cz));
        }
        pos += 2 + 2 * cnt;
        break;
      }
      case OP_UPDATE: {  // update_rates_matrix (base_otf.f90:333-364)
        const int site = v.g.site(bx, by, bz, w[pos + 1]);
        if (can_do(v, arg, site)) {
          int cx, cy, cz;
          v.g.cell(bx, by, bz, w[pos + 1], cx, cy, cz);
          const int m = v.as2[v.row(arg - 1) + site];
          const double rate = rate_of(v, arg, cx, cy, cz);
          double *r = v.rm + v.row(arg - 1);
          v.tot[arg - 1] = __dsub_rn(__dadd_rn(v.tot[arg - 1], rate), r[m]);
          r[m] = rate;
          mark(v, arg - 1, m);
        }
        pos += 2;
        break;
      }
      case OP_STRIP: {
        const int site = v.g.site(bx, by, bz, w[pos + 1]);
        for (int p = 1; p <= v.d->P; p++)
          if (can_do(v, p, site)) del_entry(v, p, site);
        pos += 2;
        break;
      }
      default: v.err = ST_PROGRAM; return;
    }
  }
}

constexpr int OTF_RATE_OPS = 128;  // rate evaluations of one event done warp-parallel
constexpr int OTF_PMASK_PROCS = 64; // models of up to 64 processes replay through per-process masks

struct EventSmem {
  double rate[OTF_RATE_OPS];
  int32_t off[OTF_RATE_OPS];  // program offsets of the stream's table ops
  int32_t m0[OTF_RATE_OPS];   // avail_sites(p, site, 2) before the event
  int32_t site[OTF_RATE_OPS]; // the op's site
  int16_t p0[OTF_RATE_OPS];   // the op's process, 0-based
  int8_t ok[OTF_RATE_OPS];
  uint32_t pmask[OTF_PMASK_PROCS][OTF_RATE_OPS / 32];  // each process's ops, one bit per op
};

// run_proc_<name> of a step with the whole warp.  Every rate and every add condition
// of the stream reads the lattice only after all of the stream's replaces (the
// generator puts the replaces after the dels and before the updates and adds, and dels
// do not read the lattice), so: (1) lane 0 applies the replaces and lists the table
// ops; (2) lanes load each op's avail_sites(p, site, 2) as it stands before the event
// and evaluate the add conditions and the rates in parallel, from the final lattice;
// (3) the table operations are replayed with those values: every op touches only its
// own process's rows, running total, list length and stale mark, so ops of different
// processes commute, and lane j replays the ops of processes j, j + 32, ... in program
// order.  A position loaded in (2) is used while no earlier op of the event has deleted
// or added an entry of that process (updates move no entry); after that the replay
// reads the table.  Updates come before adds in every stream, so an update whose entry
// was absent before the event is absent at its turn too and needs no rate.  A stream of
// more than OTF_RATE_OPS ops is replayed by lane 0 alone, in program order, the ops past
// the listed ones evaluated there.
template <bool NEAR>
__device__ void run_event(View &v, EventSmem &es, int proc0, int pos, int bx, int by, int bz, int lane,
                          bool keep_tot OTF_PH_PARAMS) {
  const int32_t *w = v.prog;
  int32_t *offs = es.off;
  int nops, ntab;
  {
    // the process's event record (built on the host): its replaces, applied by lane 0,
    // and the offsets of its table ops, copied to offs by all lanes
    const int32_t *rec = w + w[v.d->ev_index + proc0];
    const int nrep = rec[0];
    ntab = rec[1];
    nops = min(ntab, OTF_RATE_OPS);
    if (lane == 0)
      for (int i = 0; i < nrep; i++) {
        const int p = rec[2 + i];
        const int site = gsite<NEAR>(v.g, bx, by, bz, w[p + 1]);
        if (!in_mask(v.lat[site - 1], w[p + 2])) { v.err = ST_SPECIES; break; }
        v.lat[site - 1] = (int8_t)w[p + 3];
      }
    for (int k = lane; k < nops; k += 32) offs[k] = rec[2 + nrep + k];
  }
  const bool over = ntab > OTF_RATE_OPS;
  const int err0 = __shfl_sync(0xFFFFFFFFu, v.err, 0);
  __syncwarp();
  OTF_MARK(4);
  if (err0) return;
  for (int k = lane; k < nops; k += 32) {
    const int p = offs[k];
    const uint32_t h = (uint32_t)w[p];
    const int op = h & 0xFF, cnt = (h >> 8) & 0xFF, arg = (h >> 16) & 0xFFFF;
    const int site = gsite<NEAR>(v.g, bx, by, bz, w[p + 1]);
    const int m0 = v.as2[v.row(arg - 1) + site];
    bool ok = op == OP_ADD || (op == OP_UPDATE && m0 != 0);
    if (op == OP_ADD)
      for (int c = 0; c < cnt && ok; c++)
        ok = in_mask(v.lat[gsite<NEAR>(v.g, bx, by, bz, w[p + 2 + 2 * c]) - 1], w[p + 3 + 2 * c]);
    double rate = 0.0;
    if (ok) {
      int cx, cy, cz;
      v.g.cell(bx, by, bz, w[p + 1], cx, cy, cz);
      rate = rate_of<NEAR>(v, arg, cx, cy, cz);
    }
    es.m0[k] = m0;
    es.rate[k] = rate;
    es.ok[k] = ok ? 1 : 0;
    es.site[k] = site;
    es.p0[k] = (int16_t)(arg - 1);
    if (arg - 1 < OTF_PMASK_PROCS) atomicOr(&es.pmask[arg - 1][k >> 5], 1u << (k & 31));
  }
  __syncwarp();
  OTF_MARK(5);
  if (!over) {
    // one process per lane: its ops in program order (base_otf.f90:221-364)
    uint32_t moved = 0;  // bit (p0 >> 5): an op of this event deleted or added an entry of p0
    auto apply = [&](int k) {
      const int p0 = es.p0[k];
      const int p = es.off[k];
      const int op = (uint32_t)w[p] & 0xFF;
      const int site = es.site[k];
      const uint32_t bit = 1u << (p0 >> 5);
      const int m = (moved & bit) ? v.as2[v.row(p0) + site] : es.m0[k];
      if (op == OP_GDEL) {
        if (m != 0) {
          del_at(v, p0 + 1, site, m);
          moved |= bit;
        }
      } else if (op == OP_ADD) {
        if (es.ok[k]) {
          add_at(v, p0 + 1, site, es.rate[k], m);
          moved |= bit;
        }
      } else if (m != 0) {  // OP_UPDATE (base_otf.f90:333-364)
        double rate = es.rate[k];
        if (!es.ok[k]) {  // absent before the event, present now
          int cx, cy, cz;
          v.g.cell(bx, by, bz, w[p + 1], cx, cy, cz);
          rate = rate_of<NEAR>(v, p0 + 1, cx, cy, cz);
        }
        double *r = v.rm + v.row(p0);
        v.tot[p0] = __dsub_rn(__dadd_rn(v.tot[p0], rate), r[m]);
        r[m] = rate;
        mark(v, p0, m);
      }
    };
    if (v.d->P <= OTF_PMASK_PROCS) {
      // each lane walks only its own processes' ops (bits of their masks, cleared as
      // read), so the lanes' replays run side by side.  A process's list length, stale
      // mark and running total stay in registers over its ops: add_proc, del_proc and
      // update_rates_matrix (base_otf.f90:221-364) on them, then one write back.  The
      // total rates_matrix(p, V+1) is only kept where it is read before the next
      // update_accum_rate overwrites it (keep_tot: the last step of a launch).
      const int V = v.d->V;
      for (int q = lane; q < v.d->P; q += 32) {
        uint32_t any = 0;
        for (int wd = 0; wd < OTF_RATE_OPS / 32; wd++) any |= es.pmask[q][wd];
        if (!any) continue;
        int32_t *a1 = v.as1 + v.row(q), *a2 = v.as2 + v.row(q);
        double *r = v.rm + v.row(q);
        int n = v.ns[q], dq = v.dirty[q];
        double tq = keep_tot ? v.tot[q] : 0.0;
        bool mv = false;  // an op of this event deleted or added an entry of q
        int err = ST_OK;
#pragma unroll 1
        for (int wd = 0; wd < OTF_RATE_OPS / 32; wd++) {
          uint32_t b = es.pmask[q][wd];
          es.pmask[q][wd] = 0u;
          while (b && err == ST_OK) {
            const int k = 32 * wd + __ffs(b) - 1;
            b &= b - 1;
            const int op = (uint32_t)w[es.off[k]] & 0xFF;
            const int site = es.site[k];
            const int m = mv ? a2[site] : es.m0[k];
            if (op == OP_GDEL) {
              if (m == 0) continue;
              if (m < 1 || m > n) { err = ST_TABLE; break; }
              if (keep_tot) tq = __dsub_rn(tq, r[m]);
              if (m < n) {
                const int last = a1[n];
                if (last < 1 || last > V) { err = ST_TABLE; break; }
                a1[m] = last;
                a1[n] = 0;
                r[m] = r[n];
                r[n] = 0.0;
                a2[last] = m;
              } else {
                a1[m] = 0;
                r[m] = 0.0;
              }
              a2[site] = 0;
              n -= 1;
              dq = min(dq, m);
              mv = true;
            } else if (op == OP_ADD) {
              if (!es.ok[k]) continue;
              if (site < 1 || site > V || m != 0 || n + 1 > V) { err = ST_TABLE; break; }
              n += 1;
              a1[n] = site;
              a2[site] = n;
              if (keep_tot) tq = __dadd_rn(tq, es.rate[k]);
              r[n] = es.rate[k];
              dq = min(dq, n);
              mv = true;
            } else if (m != 0) {  // OP_UPDATE (base_otf.f90:333-364)
              double rate = es.rate[k];
              if (!es.ok[k]) {  // absent before the event, present now
                int cx, cy, cz;
                v.g.cell(bx, by, bz, w[es.off[k] + 1], cx, cy, cz);
                rate = rate_of<NEAR>(v, q + 1, cx, cy, cz);
              }
              if (keep_tot) tq = __dsub_rn(__dadd_rn(tq, rate), r[m]);
              r[m] = rate;
              dq = min(dq, m);
            }
          }
        }
        v.ns[q] = n;
        v.dirty[q] = dq;
        if (keep_tot) v.tot[q] = tq;
        if (err) v.err = err;
        // bits of later words left unread after an error: cleared above already
      }
    } else {
      for (int k = 0; k < nops && !v.err; k++)
        if ((es.p0[k] & 31) == lane) apply(k);
    }
    v.err = (int)__reduce_max_sync(0xFFFFFFFFu, (unsigned)v.err);
    return;
  }
  // more ops than listed: lane 0 replays the stream alone; the masks are emptied first
  for (int q = lane; q < v.d->P && q < OTF_PMASK_PROCS; q += 32)
    for (int wd = 0; wd < OTF_RATE_OPS / 32; wd++) es.pmask[q][wd] = 0u;
  __syncwarp();
  if (lane != 0) return;
  uint64_t moved = 0;  // processes (0-based, < 64) an op of this event deleted or added
  int k = 0;
  for (int p = pos;;) {
    if (v.err) return;
    const uint32_t h = (uint32_t)w[p];
    const int op = h & 0xFF, cnt = (h >> 8) & 0xFF, arg = (h >> 16) & 0xFFFF;
    if (op == OP_END) return;
    if (op == OP_REPLACE) { p += 4; continue; }
    const int site = gsite<NEAR>(v.g, bx, by, bz, w[p + 1]);
    const int p0 = arg - 1;
    const bool pre = k < nops && p0 < 64 && !((moved >> p0) & 1ull);
    const int m = pre ? es.m0[k] : v.as2[v.row(p0) + site];
    const bool have = k < nops;
    const bool ok0 = have && es.ok[k] != 0;
    const double rate0 = have ? es.rate[k] : 0.0;
    k++;
    if (op == OP_GDEL) {
      if (m != 0) {
        del_at(v, arg, site, m);
        if (p0 < 64) moved |= 1ull << p0;
      }
      p += 2;
      continue;
    }
    if (op == OP_ADD) {
      bool ok = ok0;
      double rate = rate0;
      if (!have) {
        ok = true;
        for (int c = 0; c < cnt && ok; c++)
          ok = in_mask(v.lat[gsite<NEAR>(v.g, bx, by, bz, w[p + 2 + 2 * c]) - 1], w[p + 3 + 2 * c]);
        int cx, cy, cz;
        v.g.cell(bx, by, bz, w[p + 1], cx, cy, cz);
        rate = ok ? rate_of<NEAR>(v, arg, cx, cy, cz) : 0.0;
      }
      if (ok) {
        add_at(v, arg, site, rate, m);
        if (p0 < 64) moved |= 1ull << p0;
      }
      p += 2 + 2 * cnt;
      continue;
    }
    // OP_UPDATE (base_otf.f90:333-364)
    if (m != 0) {
      double rate = rate0;
      if (!ok0) {  // not evaluated ahead (past the listed ops)
        int cx, cy, cz;
        v.g.cell(bx, by, bz, w[p + 1], cx, cy, cz);
        rate = rate_of<NEAR>(v, arg, cx, cy, cz);
      }
      double *r = v.rm + v.row(p0);
      v.tot[p0] = __dsub_rn(__dadd_rn(v.tot[p0], rate), r[m]);
      r[m] = rate;
      mark(v, p0, m);
    }
    p += 2;
  }
}

// interval_search_real (base_otf.f90:1386-1490) on arr[1..size]: bisection, the scan
// right past zeros, the scan left over equal values; 0 when no entry is positive.
__device__ inline int interval_search(const double *arr, int size, double value) {
  int left = 1, right = size, mid;
  for (;;) {
    mid = (right + left) >> 1;
    if (left >= right) break;
    if (value < arr[mid]) right = mid; else left = mid + 1;
  }
  if (arr[mid] == 0.0) {
    for (;;) {
      if (arr[mid] > 0.0) break;
      if (mid >= size) return 0;
      mid = mid + 1;
    }
  }
  while (mid != 1 && arr[mid - 1] >= arr[mid]) mid = mid - 1;
  return mid;
}

// The running sums of process p0's list (1-based): its usum row while the constant-rate
// sums hold (see otf_uniform_kernel), else the list's own pm row.
__device__ inline const double *sums_of(const View &v, int p0) {
  const Dev &d = *v.d;
  if (d.uni_on) {
    const int row = v.prog[d.uni_index + p0];
    if (row >= 0) return d.usum + (size_t)row * (d.V + 1);
  }
  return v.pm + v.row(p0);
}

// interval_search with the whole warp, for arr[1..size] non-decreasing (running sums of
// non-negative rates).  The bisection above returns the first index i with
// value < arr[i], arr[size] never tested (as if true); here that index comes from a
// 32-way search -- each round every lane tests one of 32 evenly spaced indices of the
// remaining range and a ballot keeps the part holding the first true one -- and then the
// same scans right past zeros and left over equal values, by every lane alike.
__device__ int interval_search_warp(const double *arr, int size, double value, int lane) {
  int lo = 1, hi = size;  // the answer lies in [lo, hi]; the test at hi is true
  while (lo < hi) {
    const int step = (hi - lo + 32) >> 5;  // ceil((hi - lo + 1) / 32)
    const int p = lo + lane * step;
    const bool t = p >= hi || value < arr[p];
    const unsigned b = __ballot_sync(0xFFFFFFFFu, t);
    if (!b) {
      lo += 31 * step + 1;  // every tested index false: the answer is past the last
      continue;
    }
    const int j = __ffs(b) - 1;
    if (j == 0) { hi = lo; break; }
    const int pj = lo + j * step;
    lo = lo + (j - 1) * step + 1;
    hi = pj < hi ? pj : hi;
  }
  int mid = lo;
  if (arr[mid] == 0.0) {
    for (;;) {
      if (arr[mid] > 0.0) break;
      if (mid >= size) return 0;
      mid = mid + 1;
    }
  }
  while (mid != 1 && arr[mid - 1] >= arr[mid]) mid = mid - 1;
  return mid;
}

// update_accum_rate: stale running sums re-summed (lanes: processes), then the totals
// chained into accum_rates on lane 0.  sacc is the warp's accum_rates (1-based).  A
// constant-rate process's total is read from its usum row; its pm row is left stale,
// with dirty still marking the first entry changed since it was last summed.
__device__ void accum_step(View &v, double *sacc, double *stot, int lane) {
  const int P = v.d->P;
  for (int p0 = lane; p0 < P; p0 += 32) {
    const int n = v.ns[p0];
    const double *us = sums_of(v, p0);
    double *pm = v.pm + v.row(p0);
    if (us != pm) {
      const double t = n > 0 ? us[n] : 0.0;
      stot[p0] = t;
      v.tot[p0] = t;
      continue;
    }
    const int lo = v.dirty[p0];
    if (lo <= n) {
      // the chain is serial; its loads are not: 16 entries are fetched before their adds
      const double *rm = v.rm + v.row(p0);
      double s = lo > 1 ? pm[lo - 1] : 0.0;
      int j = lo;
      for (; j + 15 <= n; j += 16) {
        double r[16];
#pragma unroll
        for (int u = 0; u < 16; u++) r[u] = rm[j + u];
#pragma unroll
        for (int u = 0; u < 16; u++) {
          s = __dadd_rn(s, r[u]);
          pm[j + u] = s;
        }
      }
      for (; j <= n; j++) {
        s = __dadd_rn(s, rm[j]);
        pm[j] = s;
      }
    }
    v.dirty[p0] = 0x7FFFFFFF;
    const double t = n > 0 ? pm[n] : 0.0;
    stot[p0] = t;
    v.tot[p0] = t;
  }
  __syncwarp();
  if (lane == 0) {
    double acc = stot[0];
    sacc[1] = acc;
    for (int p0 = 1; p0 < P; p0++) {
      acc = __dadd_rn(acc, stot[p0]);
      sacc[p0 + 1] = acc;
    }
  }
  __syncwarp();
}

struct Smem {
  EventSmem ev[OTF_WARPS];
};

// Dynamic shared memory of a block: the image (when staged; its size rounded to 16
// bytes), then each warp's accum_rates (P + 1 doubles, 1-based) and process totals (P).
// Sized by the model's P rather than OTF_PMAX, a block of eight intZGB trajectories takes
// 54 KB in all, so the two blocks of an SM leave most of its on-chip memory to the L1
// cache of the tables (and hold two copies of the image, not four as blocks of four).
__host__ __device__ inline size_t otf_image_bytes(int prog_len, int staged) {
  return staged ? ((size_t)prog_len * 4 + 15) / 16 * 16 : 0;
}
__host__ __device__ inline size_t otf_dyn_bytes(int prog_len, int staged, int P) {
  return otf_image_bytes(prog_len, staged) + (size_t)OTF_WARPS * (2 * P + 1) * 8;
}

// cmd: 0 = do_kmc_steps(n) on every trajectory (trace: only trajectory `only`, pairs to
// trace); 1 = update_accum_rate; 2 = update_integ_rate; 3 = get_next_kmc_step of `only`
// (out[0..1]); 4 = run_proc_nr(out[0], out[1]) on `only`; 5 = initialize_state(layer = n);
// 6 = recalculate_rates_matrix; 7 = touchup_cell of the n cells (x, y, z) in io, in
// order, on `only`.
template <bool NEAR>
__global__ void __launch_bounds__(32 * OTF_WARPS, 2) otf_kernel(Dev d, int cmd, int64_t n, int only, int32_t *io) {
  __shared__ Smem sm;
  extern __shared__ __align__(16) unsigned char dyn_s[];
  int32_t *prog_s = reinterpret_cast<int32_t *>(dyn_s);  // the image, when staged
  double *sums_s = reinterpret_cast<double *>(dyn_s + otf_image_bytes(d.prog_len, d.prog_staged));
  // the block copies the image to shared memory first (every thread is still here)
  if (d.prog_staged) {
    for (int i = threadIdx.x; i < d.prog_len; i += blockDim.x) prog_s[i] = d.prog[i];
    __syncthreads();
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = blockIdx.x * OTF_WARPS + warp;
  if (t >= d.T || (only >= 0 && t != only)) return;
  View v = view_of(d, t);
  if (d.prog_staged) v.prog = prog_s;
  Traj tr = d.traj[t];
  if (tr.status && cmd != 5) return;
  const int P = d.P;
  double *sacc = sums_s + (size_t)warp * (P + 1), *stot = sums_s + (size_t)OTF_WARPS * (P + 1) + (size_t)warp * P;
  if (cmd == 5) {  // initialize_state (proclist_generic_subroutines.mpy:236-304), the cell touch-up
    if (lane == 0) {
      const int32_t *site_layer = v.prog + d.off_site_layer, *site_def = v.prog + d.off_site_default;
      for (int s = 1; s <= d.V; s++) {
        const int nr = (s - 1) % d.spuck + 1;
        v.lat[s - 1] = (int8_t)(site_layer[nr - 1] == (int)n ? site_def[nr - 1] : d.null_species);
      }
      for (int k = 0; k < d.Z && !v.err; k++)
        for (int j = 0; j < d.Y && !v.err; j++)
          for (int i = 0; i < d.X && !v.err; i++) run_stream(v, v.prog[d.off_touch], i, j, k);
      tr.status = v.err;
      d.traj[t] = tr;
    }
    return;
  }
  if (cmd == 6) {  // recalculate_rates_matrix: every entry's rate from the current lattice
    for (int p0 = 0; p0 < P; p0++) {
      const int nn = v.ns[p0];
      for (int i = 1 + lane; i <= nn; i += 32) {
        int x, y, z, s;
        v.g.coords(v.as1[v.row(p0) + i], x, y, z, s);
        v.rm[v.row(p0) + i] = rate_of<NEAR>(v, p0 + 1, x, y, z);
      }
      if (lane == 0) v.dirty[p0] = 1;
    }
    __syncwarp();
    // reaccumulate_rates_matrix (base_otf.f90:366-387): the totals re-summed
    accum_step(v, sacc, stot, lane);
    if (lane == 0 && v.err) { tr.status = v.err; d.traj[t] = tr; }
    return;
  }
  if (cmd == 1 || cmd == 3) {
    double r0 = 0, r1 = 0, r2 = 0;
    if (cmd == 3) draw3(tr.rng_kind, tr.rng, tr.seed, tr.traj, r0, r1, r2);
    accum_step(v, sacc, stot, lane);
    for (int p0 = lane; p0 < P; p0 += 32) v.accum[p0] = sacc[p0 + 1];
    if (cmd == 3 && lane == 0) {  // get_next_kmc_step: the time draw picks the entry
      int proc = interval_search(sacc, P, __dmul_rn(r1, sacc[P]));
      int site = 0;
      if (proc) {
        const int nn = v.ns[proc - 1];
        const double *pm = sums_of(v, proc - 1);
        const int k = nn > 0 ? interval_search(pm, nn, __dmul_rn(r0, pm[nn])) : 0;
        site = k ? v.as1[v.row(proc - 1) + k] : 0;
      }
      io[0] = proc;
      io[1] = site;
      d.traj[t] = tr;
    }
    return;
  }
  if (cmd == 2) {
    for (int p0 = lane; p0 < P; p0 += 32)
      v.integ[p0] = __dadd_rn(v.integ[p0], __dmul_rn(v.tot[p0], tr.kmc_time_step));
    return;
  }
  if (cmd == 7) {  // touchup_cell (io:3240-3284): the cell's first site stripped, its adds
    if (lane == 0) {
      for (int64_t i = 0; i < n && !v.err; i++) run_stream(v, v.prog[d.off_touch], io[3 * i], io[3 * i + 1], io[3 * i + 2]);
      tr.status = v.err;
      d.traj[t] = tr;
    }
    return;
  }
  if (cmd == 4) {
    if (lane == 0) {
      const int proc = io[0], site = io[1];
      v.procstat[proc - 1] += 1;
      int x, y, z, s;
      v.g.coords(site, x, y, z, s);
      run_stream(v, v.prog[d.off_proc + proc - 1], x, y, z);
      tr.status = v.err;
      d.traj[t] = tr;
    }
    return;
  }
  // cmd 0: do_kmc_steps (proclist_generic_subroutines.mpy:1-44); the event masks start
  // empty and every event's replay leaves them empty
  for (int i = lane; i < OTF_PMASK_PROCS * (OTF_RATE_OPS / 32); i += 32) (&sm.ev[warp].pmask[0][0])[i] = 0u;
  __syncwarp();
#ifdef KMC_PHASE_TIMING
  long long oph[OTF_NPHASE] = {0, 0, 0, 0, 0, 0, 0, 0};
  long long otp = clock64();
#endif
  // random numbers: every 32 steps lane j draws step k + j's (ran_time, ran_proc,
  // ran_site) and -log(ran_time); steps take them with shuffles
  uint64_t rbase[4] = {tr.rng[0], tr.rng[1], tr.rng[2], tr.rng[3]};
  double my_nl = 0.0, my_r1 = 0.0, my_r2 = 0.0;
  int bidx = 32;
  int64_t step = 0;
  for (; step < n; step++) {
    if (bidx == 32) {
      if (step > 0) {  // past the batch just used
        if (tr.rng_kind == RNG_GFORTRAN) {
          for (int dd = 0; dd < 96; dd++) xoshiro_next(rbase[0], rbase[1], rbase[2], rbase[3]);
        } else {
          rbase[0] += 32;
        }
      }
      uint64_t st[4] = {rbase[0], rbase[1], rbase[2], rbase[3]};
      if (tr.rng_kind == RNG_GFORTRAN) {
        for (int dd = 0; dd < 3 * lane; dd++) xoshiro_next(st[0], st[1], st[2], st[3]);
      } else {
        st[0] += lane;
      }
      double q0;
      draw3(tr.rng_kind, st, tr.seed, tr.traj, q0, my_r1, my_r2);
      my_nl = -log(q0);
      bidx = 0;
    }
    const double nl = __shfl_sync(0xFFFFFFFFu, my_nl, bidx);
    const double r1 = __shfl_sync(0xFFFFFFFFu, my_r1, bidx);
    const double r2 = __shfl_sync(0xFFFFFFFFu, my_r2, bidx);
    bidx++;
    OTF_MARK(0);
    accum_step(v, sacc, stot, lane);
    OTF_MARK(1);
    const double total = sacc[P];
    if (!(total > 0.0)) { tr.status = ST_DEADLOCK; break; }
    // update_clocks (base_otf.f90:1280-1320), update_integ_rate (719-738)
    tr.kmc_time_step = __ddiv_rn(nl, total);
    tr.kmc_time = __dadd_rn(tr.kmc_time, tr.kmc_time_step);
    tr.kmc_step += 1;
    for (int p0 = lane; p0 < P; p0 += 32)
      v.integ[p0] = __dadd_rn(v.integ[p0], __dmul_rn(stot[p0], tr.kmc_time_step));
    OTF_MARK(2);
    // determine_procsite: the process on lane 0 (accum_rates in shared memory), the entry
    // with the whole warp (the list's running sums in device memory)
    int proc = 0, site = 0;
    if (lane == 0) proc = interval_search(sacc, P, __dmul_rn(r1, total));
    proc = __shfl_sync(0xFFFFFFFFu, proc, 0);
    const int nn = proc ? v.ns[proc - 1] : 0;
    int err = !proc || nn <= 0 ? ST_DEADLOCK : ST_OK;
    if (!err) {
      const double *pm = sums_of(v, proc - 1);
      const int k = interval_search_warp(pm, nn, __dmul_rn(r2, pm[nn]), lane);
      if (!k) {
        err = ST_DEADLOCK;
      } else if (lane == 0) {
        site = v.as1[v.row(proc - 1) + k];
        if (io) { io[2 * step] = proc; io[2 * step + 1] = site; }
        v.procstat[proc - 1] += 1;
      }
    }
    if (err) { tr.status = err; break; }
    site = __shfl_sync(0xFFFFFFFFu, site, 0);
    OTF_MARK(3);
    {
      int x, y, z, s;
      v.g.coords(site, x, y, z, s);
      run_event<NEAR>(v, sm.ev[warp], proc - 1, v.prog[d.off_proc + proc - 1], x, y, z, lane, step + 1 == n OTF_PH_ARGS);
    }
    err = __shfl_sync(0xFFFFFFFFu, v.err, 0);
    __syncwarp();
    OTF_MARK(6);
    if (err) { tr.status = err; break; }
  }
#ifdef KMC_PHASE_TIMING
  if (lane == 0 && d.phase)
    for (int i = 0; i < OTF_NPHASE; i++) atomicAdd(&d.phase[i], (unsigned long long)oph[i]);
#endif
  // the random state after the draws actually used: bidx draws of the current batch (a
  // step that found no process has drawn its numbers, as in the reference)
  if (bidx < 32 || step > 0) {
    if (tr.rng_kind == RNG_GFORTRAN) {
      for (int dd = 0; dd < 3 * bidx; dd++) xoshiro_next(rbase[0], rbase[1], rbase[2], rbase[3]);
    } else {
      rbase[0] += bidx;
    }
  }
  tr.rng[0] = rbase[0]; tr.rng[1] = rbase[1]; tr.rng[2] = rbase[2]; tr.rng[3] = rbase[3];

  for (int p0 = lane; p0 < P; p0 += 32) v.accum[p0] = sacc[p0 + 1];
  if (lane == 0) d.traj[t] = tr;
}

}  // namespace otfdev

// ==================================================================================
// host side
// ==================================================================================
using namespace kmc_host;
using otfdev::Dev;
using otfdev::Traj;

struct kmc_otf {
  cudaStream_t stream = nullptr;
  std::vector<int32_t> prog;  // the image: the program, then the rate-table records
  bool tab_stale = true;      // rates or user parameters changed since the tables were filled
  bool uni_ok = true;         // every entry of a constant-rate process holds the current rate
  bool uni_enabled = true;    // kmc_otf_set_constant_rate_sums
  int uni_rows = 0;           // constant-rate processes
  bool near = false;          // every offset of the program within one lattice period
  Dev d{};
  std::vector<double> rates, userpar;
  double *d_rates = nullptr, *d_userpar = nullptr;
  int32_t *d_io = nullptr;
  size_t io_cap = 0;
  void *mem = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.0f;
  int64_t launches = 0;
};

namespace {

bool span_ok(int64_t off, int64_t len, int64_t total) { return off >= 0 && len >= 0 && off + len <= total; }

// Simulates a rate program's stack on the host: every instruction known, every index in
// range, depth within the device stack, exactly one final END.
int check_code(const int32_t *c, int64_t len, int nvars, int nuser) {
  int depth = 0;
  for (int64_t pc = 0; pc < len;) {
    const uint32_t w = (uint32_t)c[pc++];
    const int op = w & 0xFF, kind = (w >> 8) & 0xFF, arg = (int)(w >> 16);
    if (kind > 2) return 0;
    switch (op) {
      case otfdev::I_END: return depth >= 0 && pc == len;
      case otfdev::I_PUSH_BASE: depth++; break;
      case otfdev::I_PUSH_PAR: if (arg >= nuser) return 0; depth++; break;
      case otfdev::I_PUSH_NR: if (arg >= nvars) return 0; depth++; break;
      case otfdev::I_PUSH_INT: if (pc + 1 > len) return 0; pc += 1; depth++; break;
      case otfdev::I_PUSH_CONST: if (pc + 2 > len) return 0; pc += 2; depth++; break;
      case otfdev::I_LOAD_AUX: if (arg >= otfdev::OTF_AUX) return 0; depth++; break;
      case otfdev::I_STORE_AUX: if (arg >= otfdev::OTF_AUX || depth < 1) return 0; depth--; break;
      case otfdev::I_STORE_RESULT: if (depth < 1) return 0; depth--; break;
      case otfdev::I_ADD: case otfdev::I_SUB: case otfdev::I_MUL: case otfdev::I_DIV:
      case otfdev::I_POWI: case otfdev::I_POW:
        if (depth < 2) return 0; depth--; break;
      case otfdev::I_NEG: case otfdev::I_EXP: case otfdev::I_LOG: case otfdev::I_SQRT:
      case otfdev::I_ABS: case otfdev::I_CVT:
        if (depth < 1) return 0; break;
      default: return 0;
    }
    if (depth > otfdev::OTF_STACK) return 0;
  }
  return 0;
}

bool coord_ok(int32_t w, int spuck) {
  const int n = (int)((uint32_t)w >> 24);
  return n >= 1 && n <= spuck;
}

// An op stream of the otf program: ops known, arguments and coordinates in range,
// ending inside the program.
bool check_stream(const int32_t *w, int64_t len, int64_t pos, int P, int ns, int spuck, bool touch) {
  for (int guard = 0; guard < 1 << 20; guard++) {
    if (!span_ok(pos, 1, len)) return false;
    const uint32_t h = (uint32_t)w[pos];
    const int op = h & 0xFF, cnt = (h >> 8) & 0xFF, arg = (h >> 16) & 0xFFFF;
    switch (op) {
      case OP_END: return true;
      case OP_REPLACE:
        if (!span_ok(pos, 4, len) || !coord_ok(w[pos + 1], spuck) || w[pos + 3] < -1 || w[pos + 3] > ns) return false;
        pos += 4;
        break;
      case OP_GDEL: case otfdev::OP_UPDATE:
        if (!span_ok(pos, 2, len) || arg < 1 || arg > P || !coord_ok(w[pos + 1], spuck)) return false;
        pos += 2;
        break;
      case OP_ADD:
        if (!span_ok(pos, 2 + 2 * (int64_t)cnt, len) || arg < 1 || arg > P || !coord_ok(w[pos + 1], spuck)) return false;
        for (int c = 0; c < cnt; c++) if (!coord_ok(w[pos + 2 + 2 * c], spuck)) return false;
        pos += 2 + 2 * cnt;
        break;
      case OP_STRIP:
        if (!touch || !span_ok(pos, 2, len) || !coord_ok(w[pos + 1], spuck)) return false;
        pos += 2;
        break;
      default: return false;
    }
  }
  return false;
}

int validate_otf(const int32_t *w, int32_t len) {
  if (!w || len < 24) return fail(KMC_ERR_PROGRAM, "program too short");
  if ((uint32_t)w[0] != 0x4B4D4331u || w[1] != 1 || w[2] != 2) return fail(KMC_ERR_PROGRAM, "not an otf program");
  const int P = w[3], ns = w[4], spuck = w[6], nuser = w[23];
  if (P < 1 || P > otfdev::OTF_PMAX || ns < 1 || ns > 30 || spuck < 1 || spuck > 255 || nuser < 0 || nuser > 4096)
    return fail(KMC_ERR_PROGRAM, "otf program sizes out of range");
  if (w[5] != -1 && w[5] != ns) return fail(KMC_ERR_PROGRAM, "bad null species");
  const int64_t off_proc = w[10], off_touch = w[11], off_sl = w[13], off_sd = w[14], off_rate = w[22];
  if (!span_ok(off_proc, P + 1, len) || !span_ok(off_touch, 2, len) || !span_ok(off_sl, spuck, len) ||
      !span_ok(off_sd, spuck, len) || !span_ok(off_rate, P + 1, len))
    return fail(KMC_ERR_PROGRAM, "otf program section out of range");
  for (int s = 0; s < spuck; s++)
    if (w[off_sd + s] < -1 || w[off_sd + s] > ns) return fail(KMC_ERR_PROGRAM, "bad default species");
  for (int p = 0; p < P; p++)
    if (!check_stream(w, len, w[off_proc + p], P, ns, spuck, false)) return fail(KMC_ERR_PROGRAM, "bad process stream");
  if (!check_stream(w, len, w[off_touch], P, ns, spuck, true)) return fail(KMC_ERR_PROGRAM, "bad touch-up stream");
  for (int p = 0; p < P; p++) {
    const int64_t r = w[off_rate + p];
    if (!span_ok(r, 4, len)) return fail(KMC_ERR_PROGRAM, "bad rate record");
    const int nb = w[r], nv = w[r + 1], nc = w[r + 2];
    if (nb < 0 || nb > 4096 || nv < 0 || nv > otfdev::OTF_NRMAX || nc < 1) return fail(KMC_ERR_PROGRAM, "bad rate record");
    int64_t pos = r + 4;
    for (int k = 0; k < nb; k++) {
      if (!span_ok(pos, 2, len) || !coord_ok(w[pos], spuck)) return fail(KMC_ERR_PROGRAM, "bad bystander");
      const int np = w[pos + 1];
      if (np < 0 || !span_ok(pos + 2, 2 * (int64_t)np, len)) return fail(KMC_ERR_PROGRAM, "bad bystander");
      for (int j = 0; j < np; j++)
        if (w[pos + 2 + 2 * j] < -1 || w[pos + 2 + 2 * j] > ns || w[pos + 3 + 2 * j] < 0 || w[pos + 3 + 2 * j] >= nv)
          return fail(KMC_ERR_PROGRAM, "bad bystander species or variable");
      pos += 2 + 2 * (int64_t)np;
    }
    if (!span_ok(pos, nc, len) || !check_code(w + pos, nc, nv, nuser)) return fail(KMC_ERR_PROGRAM, "bad rate program");
  }
  return KMC_OK;
}

// The largest |offset| per axis an event's site computations reach: an op's coordinate
// plus, for the rates it evaluates, a bystander's (process streams and rate records).
void otf_reach(const int32_t *w, int r[3]) {
  const int P = w[3];
  const int64_t off_proc = w[10], off_rate = w[22];
  int op_r[3] = {0, 0, 0}, by_r[3] = {0, 0, 0};
  auto take = [](int32_t c, int *m) {
    const uint32_t u = (uint32_t)c;
    const int d[3] = {(int8_t)(u & 0xFF), (int8_t)((u >> 8) & 0xFF), (int8_t)((u >> 16) & 0xFF)};
    for (int a = 0; a < 3; a++) m[a] = std::max(m[a], std::abs(d[a]));
  };
  for (int p = 0; p < P; p++) {
    for (int64_t pos = w[off_proc + p];;) {
      const uint32_t h = (uint32_t)w[pos];
      const int op = h & 0xFF, cnt = (h >> 8) & 0xFF;
      if (op == OP_END) break;
      take(w[pos + 1], op_r);
      if (op == OP_REPLACE) { pos += 4; continue; }
      if (op == OP_ADD) {
        for (int c = 0; c < cnt; c++) take(w[pos + 2 + 2 * c], op_r);
        pos += 2 + 2 * cnt;
        continue;
      }
      pos += 2;
    }
    const int64_t rr = w[off_rate + p];
    const int nb = w[rr];
    int64_t b = rr + 4;
    for (int k = 0; k < nb; k++) {
      take(w[b], by_r);
      b += 2 + 2 * (int64_t)w[b + 1];
    }
  }
  for (int a = 0; a < 3; a++) r[a] = op_r[a] + by_r[a];
}

constexpr int64_t OTF_TABLE_MAX = 4096;  // table entries of one model (32 KB of doubles)

// Appends the rate-table records to a checked program: for each process whose counts
// take at most OTF_TABLE_MAX combinations in all, the record [first entry, nv,
// radix(nv), nb, then per bystander: coordinate, npairs, (species, stride of the
// variable) x npairs], where radix(k) = 1 + the pairs counting into variable k (the
// most it can reach) and stride(k) = radix(0) ... radix(k - 1).  The index array of the
// P record offsets (-1: no table) follows the program; then the records, the P usum row
// numbers of the constant-rate processes (-1: not one), and the values.
void build_image(const int32_t *w, int32_t len, std::vector<int32_t> &img, Dev &d, int &uni_rows) {
  const int P = w[3];
  const int64_t off_rate = w[22];
  img.assign(w, w + len);
  img.resize(align_up((size_t)len, 2), 0);
  d.tab_index = (int32_t)img.size();
  img.resize(img.size() + P, -1);
  int64_t entries = 0;
  for (int p = 0; p < P; p++) {
    const int64_t r = w[off_rate + p];
    const int nb = w[r], nv = w[r + 1];
    std::vector<int64_t> radix(nv, 1);
    int64_t pos = r + 4;
    for (int k = 0; k < nb; k++) {
      const int np = w[pos + 1];
      for (int j = 0; j < np; j++) radix[w[pos + 3 + 2 * j]] += 1;
      pos += 2 + 2 * (int64_t)np;
    }
    int64_t size = 1;
    std::vector<int64_t> stride(nv);
    for (int k = 0; k < nv && size <= OTF_TABLE_MAX; k++) {
      stride[k] = size;
      size *= radix[k];
    }
    if (size > OTF_TABLE_MAX || entries + size > OTF_TABLE_MAX) continue;
    img[d.tab_index + p] = (int32_t)img.size();
    img.push_back((int32_t)entries);
    img.push_back(nv);
    for (int k = 0; k < nv; k++) img.push_back((int32_t)radix[k]);
    img.push_back(nb);
    pos = r + 4;
    for (int k = 0; k < nb; k++) {
      const int np = w[pos + 1];
      img.push_back(w[pos]);
      img.push_back(np);
      for (int j = 0; j < np; j++) {
        img.push_back(w[pos + 2 + 2 * j]);
        img.push_back((int32_t)stride[w[pos + 3 + 2 * j]]);
      }
      pos += 2 + 2 * (int64_t)np;
    }
    entries += size;
  }
  d.tab_entries = (int32_t)entries;
  // the constant-rate processes (rate programs reading no count): their usum rows
  d.uni_index = (int32_t)img.size();
  img.resize(img.size() + P, -1);
  int rows = 0;
  for (int p = 0; p < P; p++)
    if (w[w[off_rate + p] + 1] == 0) img[d.uni_index + p] = rows++;
  if (!rows) d.uni_index = -1;
  uni_rows = rows;
  d.ev_index = (int32_t)img.size();
  img.resize(img.size() + P, 0);
  const int64_t off_proc = w[10];
  for (int p = 0; p < P; p++) {
    std::vector<int32_t> reps, tab;
    int64_t ntab = 0;
    for (int64_t pos = w[off_proc + p];;) {
      const uint32_t h = (uint32_t)w[pos];
      const int op = h & 0xFF, cnt = (h >> 8) & 0xFF;
      if (op == OP_END) break;
      if (op == OP_REPLACE) {
        reps.push_back((int32_t)pos);
        pos += 4;
      } else {
        if (ntab < otfdev::OTF_RATE_OPS) tab.push_back((int32_t)pos);
        ntab++;
        pos += op == OP_ADD ? 2 + 2 * cnt : 2;
      }
    }
    img[d.ev_index + p] = (int32_t)img.size();
    img.push_back((int32_t)reps.size());
    img.push_back((int32_t)ntab);
    img.insert(img.end(), reps.begin(), reps.end());
    img.insert(img.end(), tab.begin(), tab.end());
  }
  img.resize(align_up(img.size(), 4), 0);
  d.tab_values = (int32_t)img.size();
  img.resize(img.size() + 2 * (size_t)entries, 0);
  d.tab_on = entries > 0 ? 1 : 0;
  if (!entries) d.tab_index = -1;
}

int launch(kmc_otf *h, int cmd, int64_t n, int only, int32_t *d_io) {
  const int blocks = only >= 0 ? 1 : (h->d.T + otfdev::OTF_WARPS - 1) / otfdev::OTF_WARPS;
  Dev d = h->d;
  if (only >= 0) {
    // one block whose first warp is trajectory `only`: shift the trajectory base
    const size_t PV = (size_t)d.P * (d.V + 1);
    d.lat += (size_t)only * d.V; d.as1 += only * PV; d.as2 += only * PV; d.rm += only * PV; d.pm += only * PV;
    d.dirty += (size_t)only * d.P; d.ns += (size_t)only * d.P; d.integ += (size_t)only * d.P;
    d.accum += (size_t)only * d.P; d.tot += (size_t)only * d.P; d.procstat += (size_t)only * d.P;
    d.traj += only; d.T = 1;
  }
  // site_near for programs whose every offset stays within one period of this lattice
  const void *kfn = h->near ? (const void *)otfdev::otf_kernel<true> : (const void *)otfdev::otf_kernel<false>;
  // the image goes to every block's shared memory when it fits beside the static part
  // and the warps' accum_rates and totals
  size_t dyn = 0;
  {
    cudaFuncAttributes fa;
    CK(cudaFuncGetAttributes(&fa, kfn));
    int optin = 0, dev = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const int64_t cap = optin - (int64_t)fa.sharedSizeBytes;
    d.prog_staged = (int64_t)otfdev::otf_dyn_bytes(d.prog_len, 1, d.P) <= cap ? 1 : 0;
    dyn = otfdev::otf_dyn_bytes(d.prog_len, d.prog_staged, d.P);
    if ((int64_t)dyn > cap) return fail(KMC_ERR_ARG, "otf: too many processes for shared memory");
    if (fa.maxDynamicSharedSizeBytes < (int)dyn)
      CK(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap));
  }
  if (h->tab_stale) {
    if (h->d.tab_entries > 0) {
      otfdev::otf_table_kernel<<<(h->d.tab_entries + 127) / 128, 128, 0, h->stream>>>(h->d, const_cast<int32_t *>(h->d.prog));
      CK(cudaGetLastError());
    }
    if (h->d.uni_index >= 0) {
      otfdev::otf_uniform_kernel<<<(h->d.P + 31) / 32, 32, 0, h->stream>>>(h->d, h->d.prog);
      CK(cudaGetLastError());
    }
    h->tab_stale = false;
  }
  // recalculate_rates_matrix gives every entry the current rate before it sums
  if (cmd == 6) h->uni_ok = true;
  d.uni_on = h->uni_enabled && h->uni_ok && d.uni_index >= 0 ? 1 : 0;
  CK(cudaEventRecord(h->ev0, h->stream));
  int only_arg = only >= 0 ? 0 : -1;
  void *args[] = {&d, &cmd, &n, &only_arg, &d_io};
  CK(cudaLaunchKernel(kfn, dim3(blocks), dim3(32 * otfdev::OTF_WARPS), args, dyn, h->stream));
  CK(cudaGetLastError());
  CK(cudaEventRecord(h->ev1, h->stream));
  h->launches++;
  return KMC_OK;
}

int sync_timed(kmc_otf *h) {
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  return KMC_OK;
}

int io_buffer(kmc_otf *h, size_t words) {
  if (words <= h->io_cap) return KMC_OK;
  if (h->d_io) CK(cudaFree(h->d_io));
  h->d_io = nullptr;
  CK(cudaMalloc(&h->d_io, words * 4));
  h->io_cap = words;
  return KMC_OK;
}

int traj_status(kmc_otf *h, int traj) {
  Traj tr;
  CK(cudaMemcpy(&tr, h->d.traj + traj, sizeof(Traj), cudaMemcpyDeviceToHost));
  return tr.status ? fail(tr.status, "trajectory stopped with a table, species or dead-lock error") : KMC_OK;
}

// A trajectory's state from the host (reload_system, base_otf.f90:448-599): lattice,
// avail_sites(:, :, 1) as [P][V+1] (entry 0 unused), nr_of_sites, procstat, integ_rates
// (NULL: zero), the clock, kmc_step, and the random stream when rng is given.  Checked
// first: species in range, each list's entries distinct sites.  avail_sites(:, :, 2) is
// rebuilt as the inverse; rates_matrix is zero as after allocate_system (the reference's
// file does not hold it) until recalculate_rates_matrix.
int otf_store(kmc_otf *h, int traj, const int32_t *lattice, const int32_t *as1, const int32_t *nsites,
              const int64_t *procstat, const double *integ, const double clock[2], int64_t kmc_step, const Traj *rng) {
  const Dev &d = h->d;
  const int P = d.P, V = d.V;
  const size_t PV = (size_t)P * (V + 1);
  std::vector<int8_t> lat(V);
  for (int i = 0; i < V; i++) {
    if (lattice[i] < -1 || lattice[i] > d.nspecies) return fail(KMC_ERR_ARG, "state: unknown species");
    lat[i] = (int8_t)lattice[i];
  }
  std::vector<int32_t> a1(PV, 0), a2(PV, 0), dirty(P, 1);
  for (int q = 0; q < P; q++) {
    const int n = nsites[q];
    if (n < 0 || n > V) return fail(KMC_ERR_TABLE, "state: nr_of_sites out of range");
    for (int i = 1; i <= n; i++) {
      const int s = as1[(size_t)q * (V + 1) + i];
      if (s < 1 || s > V || a2[(size_t)q * (V + 1) + s] != 0) return fail(KMC_ERR_TABLE, "state: avail_sites entry");
      a1[(size_t)q * (V + 1) + i] = s;
      a2[(size_t)q * (V + 1) + s] = i;
    }
  }
  std::vector<double> zeros(PV, 0.0), integ0(P, 0.0);
  Traj tr;
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(&tr, d.traj + traj, sizeof(Traj), cudaMemcpyDeviceToHost));
  tr.kmc_time = clock[0];
  tr.kmc_time_step = clock[1];
  tr.kmc_step = kmc_step;
  tr.status = 0;
  if (rng) {
    tr.rng_kind = rng->rng_kind; tr.seed = rng->seed; tr.traj = rng->traj;
    for (int i = 0; i < 4; i++) tr.rng[i] = rng->rng[i];
  }
  CK(cudaMemcpy(d.lat + (size_t)traj * V, lat.data(), V, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d.as1 + traj * PV, a1.data(), PV * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d.as2 + traj * PV, a2.data(), PV * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d.rm + traj * PV, zeros.data(), PV * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d.pm + traj * PV, zeros.data(), PV * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d.dirty + (size_t)traj * P, dirty.data(), P * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d.ns + (size_t)traj * P, nsites, P * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d.procstat + (size_t)traj * P, procstat, P * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d.integ + (size_t)traj * P, integ ? integ : integ0.data(), P * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d.accum + (size_t)traj * P, integ0.data(), P * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d.tot + (size_t)traj * P, integ0.data(), P * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d.traj + traj, &tr, sizeof(Traj), cudaMemcpyHostToDevice));
  h->uni_ok = false;  // the entries' rates are zero, not the constant-rate processes' rates
  return KMC_OK;
}

}  // namespace

extern "C" {

int kmc_otf_check_program(const int32_t *program, int32_t len) { return validate_otf(program, len); }

int kmc_otf_create(const int32_t *program, int32_t len, const int32_t dims[3], int32_t layer, int32_t ntraj,
                   int32_t seed, int32_t rng_kind, uint32_t traj0, kmc_otf **out) {
  if (!program || !dims || !out || ntraj < 1 || (rng_kind != 0 && rng_kind != 1)) return fail(KMC_ERR_ARG, "bad arguments");
  int rc = validate_otf(program, len);
  if (rc) return rc;
  if (dims[0] < 1 || dims[1] < 1 || dims[2] < 1) return fail(KMC_ERR_ARG, "bad system size");
  const int64_t V = (int64_t)dims[0] * dims[1] * dims[2] * program[6];
  if (V > (1 << 24)) return fail(KMC_ERR_ARG, "lattice too large");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(KMC_ERR_NODEVICE, "no CUDA device");
  kmc_otf *h = new kmc_otf();
  const int P = program[3], T = ntraj;
  Dev &d = h->d;
  build_image(program, len, h->prog, d, h->uni_rows);
  const int32_t img_len = (int32_t)h->prog.size();
  {
    int reach[3];
    otf_reach(program, reach);
    h->near = reach[0] <= dims[0] && reach[1] <= dims[1] && reach[2] <= dims[2];
  }
  d.P = P; d.nspecies = program[4]; d.null_species = program[5]; d.spuck = program[6];
  d.nuser = program[23]; d.off_proc = program[10]; d.off_touch = program[11]; d.off_rate = program[22];
  d.off_site_layer = program[13]; d.off_site_default = program[14];
  d.X = dims[0]; d.Y = dims[1]; d.Z = dims[2]; d.V = (int)V; d.T = T;
  const size_t PV = (size_t)P * (V + 1), TP = (size_t)T * P;
  // constant-rate running sums for lattices of up to 65536 sites (512 KB per process)
  const bool use_usum = h->uni_rows > 0 && V <= 65536;
  if (!use_usum) d.uni_index = -1;
  const size_t sizes[] = {(size_t)img_len * 4, (size_t)T * V, T * PV * 4, T * PV * 4, T * PV * 8, T * PV * 8,
                          TP * 4, TP * 4, TP * 8, TP * 8, TP * 8, TP * 8, (size_t)T * sizeof(Traj),
                          (size_t)P * 8, (size_t)(d.nuser > 0 ? d.nuser : 1) * 8,
                          (size_t)otfdev::OTF_NPHASE * 8,
                          use_usum ? (size_t)h->uni_rows * (V + 1) * 8 : 0};
  size_t offs[17], total = 0;
  for (int i = 0; i < 17; i++) { offs[i] = total; total = align_up(total + sizes[i], 256); }
  auto cleanup = [&](int code) { if (h->mem) cudaFree(h->mem); if (h->stream) cudaStreamDestroy(h->stream);
                                 if (h->ev0) cudaEventDestroy(h->ev0); if (h->ev1) cudaEventDestroy(h->ev1);
                                 delete h; return code; };
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess)
    return cleanup(fail(KMC_ERR_CUDA, "stream or event creation failed"));
  if (cudaMalloc(&h->mem, total) != cudaSuccess) return cleanup(fail(KMC_ERR_NOMEM, "device memory"));
  if (cudaMemsetAsync(h->mem, 0, total, h->stream) != cudaSuccess) return cleanup(fail(KMC_ERR_CUDA, "memset"));
  char *base = (char *)h->mem;
  int32_t *dprog = (int32_t *)(base + offs[0]);
  d.prog = dprog;
  d.prog_len = img_len;
  d.prog_staged = 0;
  d.lat = (int8_t *)(base + offs[1]);
  d.as1 = (int32_t *)(base + offs[2]); d.as2 = (int32_t *)(base + offs[3]);
  d.rm = (double *)(base + offs[4]); d.pm = (double *)(base + offs[5]);
  d.dirty = (int32_t *)(base + offs[6]); d.ns = (int32_t *)(base + offs[7]);
  d.integ = (double *)(base + offs[8]); d.accum = (double *)(base + offs[9]);
  d.tot = (double *)(base + offs[10]); d.procstat = (int64_t *)(base + offs[11]);
  d.traj = (Traj *)(base + offs[12]);
  h->d_rates = (double *)(base + offs[13]); h->d_userpar = (double *)(base + offs[14]);
  d.rates = h->d_rates; d.userpar = h->d_userpar;
  d.phase = (unsigned long long *)(base + offs[15]);
  d.usum = use_usum ? (double *)(base + offs[16]) : nullptr;
  d.uni_on = 0;
  h->rates.assign(P, 0.0);
  h->userpar.assign(d.nuser, 0.0);
  std::vector<Traj> tr(T);
  for (int t = 0; t < T; t++) {
    std::memset(&tr[t], 0, sizeof(Traj));
    tr[t].seed = (uint32_t)seed; tr[t].traj = traj0 + (uint32_t)t; tr[t].rng_kind = rng_kind;
    if (rng_kind == RNG_GFORTRAN) gfortran_seed(tr[t].rng, seed);
  }
  if (cudaMemcpyAsync(dprog, h->prog.data(), (size_t)img_len * 4, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
      cudaMemcpyAsync(d.traj, tr.data(), (size_t)T * sizeof(Traj), cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
    return cleanup(fail(KMC_ERR_CUDA, "upload"));
  std::vector<int32_t> dirty(TP, 0x7FFFFFFF);
  if (cudaMemcpyAsync(d.dirty, dirty.data(), TP * 4, cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
    return cleanup(fail(KMC_ERR_CUDA, "upload"));
  rc = launch(h, 5, layer, -1, nullptr);
  if (rc) return cleanup(rc);
  rc = sync_timed(h);
  if (rc) return cleanup(rc);
  for (int t = 0; t < T; t++) {
    rc = traj_status(h, t);
    if (rc) return cleanup(rc);
  }
  *out = h;
  return KMC_OK;
}

int kmc_otf_destroy(kmc_otf *h) {
  if (!h) return KMC_OK;
  if (h->d_io) cudaFree(h->d_io);
  if (h->mem) cudaFree(h->mem);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return KMC_OK;
}

int kmc_otf_set_rate_const(kmc_otf *h, int32_t proc, double rate) {
  if (!h || proc < 1 || proc > h->d.P) return fail(KMC_ERR_ARG, "bad process");
  h->rates[proc - 1] = rate;
  h->tab_stale = true;
  h->uni_ok = false;
  CK(cudaMemcpyAsync(h->d_rates, h->rates.data(), h->rates.size() * 8, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return KMC_OK;
}

int kmc_otf_set_user_parameter(kmc_otf *h, int32_t k, double value) {
  if (!h || k < 1 || k > h->d.nuser) return fail(KMC_ERR_ARG, "bad user parameter");
  h->userpar[k - 1] = value;
  h->tab_stale = true;
  h->uni_ok = false;
  CK(cudaMemcpyAsync(h->d_userpar, h->userpar.data(), h->userpar.size() * 8, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return KMC_OK;
}

int kmc_otf_recalculate_rates_matrix(kmc_otf *h) {
  if (!h) return fail(KMC_ERR_ARG, "bad handle");
  int rc = launch(h, 6, 0, -1, nullptr);
  return rc ? rc : sync_timed(h);
}

int kmc_otf_update_accum_rate(kmc_otf *h) {
  if (!h) return fail(KMC_ERR_ARG, "bad handle");
  int rc = launch(h, 1, 0, -1, nullptr);
  return rc ? rc : sync_timed(h);
}

int kmc_otf_update_integ_rate(kmc_otf *h) {
  if (!h) return fail(KMC_ERR_ARG, "bad handle");
  int rc = launch(h, 2, 0, -1, nullptr);
  return rc ? rc : sync_timed(h);
}

int kmc_otf_do_steps(kmc_otf *h, int64_t n) {
  if (!h || n < 0) return fail(KMC_ERR_ARG, "bad arguments");
  int rc = launch(h, 0, n, -1, nullptr);
  if (rc) return rc;
  rc = sync_timed(h);
  if (rc) return rc;
  std::vector<Traj> tr(h->d.T);
  CK(cudaMemcpy(tr.data(), h->d.traj, tr.size() * sizeof(Traj), cudaMemcpyDeviceToHost));
  for (const Traj &x : tr)
    if (x.status) return fail(x.status, "a trajectory stopped with a table, species or dead-lock error");
  return KMC_OK;
}

int kmc_otf_trace_steps(kmc_otf *h, int32_t traj, int64_t n, int32_t *out) {
  if (!h || traj < 0 || traj >= h->d.T || n < 0 || !out) return fail(KMC_ERR_ARG, "bad arguments");
  int rc = io_buffer(h, (size_t)(2 * n + 2));
  if (rc) return rc;
  rc = launch(h, 0, n, traj, h->d_io);
  if (rc) return rc;
  rc = sync_timed(h);
  if (rc) return rc;
  CK(cudaMemcpy(out, h->d_io, (size_t)n * 8, cudaMemcpyDeviceToHost));
  return traj_status(h, traj);
}

int kmc_otf_get_next_step(kmc_otf *h, int32_t traj, int32_t *proc, int32_t *site) {
  if (!h || traj < 0 || traj >= h->d.T || !proc || !site) return fail(KMC_ERR_ARG, "bad arguments");
  int rc = io_buffer(h, 2);
  if (rc) return rc;
  rc = launch(h, 3, 0, traj, h->d_io);
  if (rc) return rc;
  rc = sync_timed(h);
  if (rc) return rc;
  int32_t v[2];
  CK(cudaMemcpy(v, h->d_io, 8, cudaMemcpyDeviceToHost));
  if (!v[0] || !v[1]) return fail(KMC_ERR_DEADLOCK, "no process available");
  *proc = v[0];
  *site = v[1];
  return KMC_OK;
}

int kmc_otf_run_proc_nr(kmc_otf *h, int32_t traj, int32_t proc, int32_t site) {
  if (!h || traj < 0 || traj >= h->d.T || proc < 1 || proc > h->d.P || site < 1 || site > h->d.V)
    return fail(KMC_ERR_ARG, "bad arguments");
  int rc = io_buffer(h, 2);
  if (rc) return rc;
  const int32_t v[2] = {proc, site};
  CK(cudaMemcpyAsync(h->d_io, v, 8, cudaMemcpyHostToDevice, h->stream));
  rc = launch(h, 4, 0, traj, h->d_io);
  if (rc) return rc;
  rc = sync_timed(h);
  return rc ? rc : traj_status(h, traj);
}

int kmc_otf_get_state(kmc_otf *h, int32_t traj, int32_t *lattice, int32_t *as1, int32_t *as2, int32_t *nsites,
                      int64_t *procstat, double *integ, double *accum, double *rates_matrix, double *totals,
                      double clock[2], int64_t *kmc_step) {
  if (!h || traj < 0 || traj >= h->d.T) return fail(KMC_ERR_ARG, "bad arguments");
  const Dev &d = h->d;
  const size_t PV = (size_t)d.P * (d.V + 1);
  CK(cudaStreamSynchronize(h->stream));
  if (lattice) {
    std::vector<int8_t> l(d.V);
    CK(cudaMemcpy(l.data(), d.lat + (size_t)traj * d.V, d.V, cudaMemcpyDeviceToHost));
    for (int i = 0; i < d.V; i++) lattice[i] = l[i];
  }
  if (as1) CK(cudaMemcpy(as1, d.as1 + traj * PV, PV * 4, cudaMemcpyDeviceToHost));
  if (as2) CK(cudaMemcpy(as2, d.as2 + traj * PV, PV * 4, cudaMemcpyDeviceToHost));
  if (rates_matrix) CK(cudaMemcpy(rates_matrix, d.rm + traj * PV, PV * 8, cudaMemcpyDeviceToHost));
  if (nsites) CK(cudaMemcpy(nsites, d.ns + (size_t)traj * d.P, d.P * 4, cudaMemcpyDeviceToHost));
  if (procstat) CK(cudaMemcpy(procstat, d.procstat + (size_t)traj * d.P, d.P * 8, cudaMemcpyDeviceToHost));
  if (integ) CK(cudaMemcpy(integ, d.integ + (size_t)traj * d.P, d.P * 8, cudaMemcpyDeviceToHost));
  if (accum) CK(cudaMemcpy(accum, d.accum + (size_t)traj * d.P, d.P * 8, cudaMemcpyDeviceToHost));
  if (totals) CK(cudaMemcpy(totals, d.tot + (size_t)traj * d.P, d.P * 8, cudaMemcpyDeviceToHost));
  if (clock || kmc_step) {
    Traj tr;
    CK(cudaMemcpy(&tr, d.traj + traj, sizeof(Traj), cudaMemcpyDeviceToHost));
    if (clock) { clock[0] = tr.kmc_time; clock[1] = tr.kmc_time_step; }
    if (kmc_step) *kmc_step = tr.kmc_step;
  }
  return KMC_OK;
}

int kmc_otf_set_rate_tables(kmc_otf *h, int32_t on) {
  if (!h) return fail(KMC_ERR_ARG, "bad handle");
  h->d.tab_on = on && h->d.tab_entries > 0 ? 1 : 0;
  return KMC_OK;
}

int kmc_otf_get_rate_consts(kmc_otf *h, double *rates) {
  if (!h || !rates) return fail(KMC_ERR_ARG, "bad arguments");
  std::copy(h->rates.begin(), h->rates.end(), rates);
  return KMC_OK;
}

int kmc_otf_set_kmc_time(kmc_otf *h, int32_t traj, double kmc_time) {
  if (!h || traj < 0 || traj >= h->d.T) return fail(KMC_ERR_ARG, "bad arguments");
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(&h->d.traj[traj].kmc_time, &kmc_time, sizeof(double), cudaMemcpyHostToDevice));
  return KMC_OK;
}

int kmc_otf_replace_species(kmc_otf *h, int32_t traj, int32_t site, int32_t old_species, int32_t new_species) {
  if (!h || traj < 0 || traj >= h->d.T || site < 1 || site > h->d.V) return fail(KMC_ERR_ARG, "bad arguments");
  if (new_species < -1 || new_species > h->d.nspecies) return fail(KMC_ERR_ARG, "unknown species");
  int8_t *cell = h->d.lat + (size_t)traj * h->d.V + (site - 1);
  int8_t cur;
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(&cur, cell, 1, cudaMemcpyDeviceToHost));
  if (cur != old_species) return fail(KMC_ERR_SPECIES, "replace_species: the site holds another species");
  const int8_t nw = (int8_t)new_species;
  CK(cudaMemcpy(cell, &nw, 1, cudaMemcpyHostToDevice));
  return KMC_OK;
}

int kmc_otf_touchup_cells(kmc_otf *h, int32_t traj, int32_t n, const int32_t *cells) {
  if (!h || traj < 0 || traj >= h->d.T || n < 0 || (n > 0 && !cells)) return fail(KMC_ERR_ARG, "bad arguments");
  if (n == 0) return KMC_OK;
  for (int32_t i = 0; i < n; i++)
    if (cells[3 * i] < 0 || cells[3 * i] >= h->d.X || cells[3 * i + 1] < 0 || cells[3 * i + 1] >= h->d.Y ||
        cells[3 * i + 2] < 0 || cells[3 * i + 2] >= h->d.Z)
      return fail(KMC_ERR_ARG, "cell out of range");
  int rc = io_buffer(h, (size_t)3 * n);
  if (rc) return rc;
  CK(cudaMemcpyAsync(h->d_io, cells, (size_t)12 * n, cudaMemcpyHostToDevice, h->stream));
  rc = launch(h, 7, n, traj, h->d_io);
  if (rc) return rc;
  rc = sync_timed(h);
  return rc ? rc : traj_status(h, traj);
}

int kmc_otf_set_state(kmc_otf *h, int32_t traj, const int32_t *lattice, const int32_t *as1, const int32_t *nr_of_sites,
                      const int64_t *procstat, const double *integ_rates, const double clock[2], int64_t kmc_step) {
  if (!h || traj < 0 || traj >= h->d.T || !lattice || !as1 || !nr_of_sites || !procstat || !clock || kmc_step < 0)
    return fail(KMC_ERR_ARG, "bad arguments");
  return otf_store(h, traj, lattice, as1, nr_of_sites, procstat, integ_rates, clock, kmc_step, nullptr);
}

int kmc_otf_save_reload(kmc_otf *h, int32_t traj, const char *path, double walltime) {
  if (!h || traj < 0 || traj >= h->d.T || !path) return fail(KMC_ERR_ARG, "bad arguments");
  const Dev &dv = h->d;
  const int P = dv.P, V = dv.V;
  const size_t PV = (size_t)P * (V + 1);
  std::vector<int8_t> lat(V);
  std::vector<int32_t> a1(PV), ns(P);
  kmc_reload::ReloadData d;
  d.P = P;
  d.V = V;
  d.procstat.resize(P);
  d.integ.resize(P);
  Traj tr;
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(lat.data(), dv.lat + (size_t)traj * V, V, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(a1.data(), dv.as1 + traj * PV, PV * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(ns.data(), dv.ns + (size_t)traj * P, P * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(d.procstat.data(), dv.procstat + (size_t)traj * P, P * 8, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(d.integ.data(), dv.integ + (size_t)traj * P, P * 8, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&tr, dv.traj + traj, sizeof(Traj), cudaMemcpyDeviceToHost));
  d.dims[0] = dv.X; d.dims[1] = dv.Y; d.dims[2] = dv.Z;
  d.kmc_time = tr.kmc_time;
  d.kmc_time_step = tr.kmc_time_step;
  d.walltime = walltime;
  d.kmc_step = tr.kmc_step;
  d.rng_kind = tr.rng_kind; d.seed = tr.seed; d.traj = tr.traj;
  for (int i = 0; i < 4; i++) d.rng[i] = tr.rng[i];
  d.rates = h->rates;
  d.nsites = ns;
  d.lattice.assign(lat.begin(), lat.end());
  d.as1.resize(P);
  for (int q = 0; q < P; q++) d.as1[q].assign(a1.begin() + (size_t)q * (V + 1) + 1, a1.begin() + (size_t)q * (V + 1) + 1 + ns[q]);
  return kmc_reload::write_reload(path, d);
}

int kmc_otf_load_reload(kmc_otf *h, int32_t traj, const char *path, double *walltime) {
  if (!h || traj < 0 || traj >= h->d.T || !path) return fail(KMC_ERR_ARG, "bad arguments");
  kmc_reload::ReloadFile r;
  int rc = kmc_reload::parse_reload(path, r, false);
  if (rc) return rc;
  kmc_reload::ReloadData d;
  rc = kmc_reload::read_reload(r, h->d.P, h->d.V, h->d.nspecies, d);
  if (rc) return rc;
  const int P = h->d.P, V = h->d.V;
  std::vector<int32_t> a1((size_t)P * (V + 1), 0);
  for (int q = 0; q < P; q++)
    std::copy(d.as1[q].begin(), d.as1[q].end(), a1.begin() + (size_t)q * (V + 1) + 1);
  const double clock[2] = {d.kmc_time, d.kmc_time_step};
  Traj rng{};
  if (r.have_rng) {
    rng.rng_kind = d.rng_kind; rng.seed = d.seed; rng.traj = d.traj;
    for (int i = 0; i < 4; i++) rng.rng[i] = d.rng[i];
  }
  rc = otf_store(h, traj, d.lattice.data(), a1.data(), d.nsites.data(), d.procstat.data(), d.integ.data(), clock,
                 d.kmc_step, r.have_rng ? &rng : nullptr);
  if (rc) return rc;
  // the file's rate constants (base.reload_system reads `rates`)
  h->rates = d.rates;
  h->tab_stale = true;
  CK(cudaMemcpyAsync(h->d_rates, h->rates.data(), h->rates.size() * 8, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (walltime) *walltime = d.walltime;
  return KMC_OK;
}

int kmc_otf_set_constant_rate_sums(kmc_otf *h, int32_t on) {
  if (!h) return fail(KMC_ERR_ARG, "bad handle");
  h->uni_enabled = on != 0;
  return KMC_OK;
}

int kmc_otf_rate_table_entries(kmc_otf *h, int32_t *entries) {
  if (!h || !entries) return fail(KMC_ERR_ARG, "bad arguments");
  *entries = h->d.tab_entries;
  return KMC_OK;
}

int kmc_otf_last_kernel_ms(kmc_otf *h, float *ms) {
  if (!h || !ms) return fail(KMC_ERR_ARG, "bad arguments");
  *ms = h->last_ms;
  return KMC_OK;
}

int kmc_otf_phase_cycles(kmc_otf *h, uint64_t *out, int32_t reset) {
  if (!h || !out) return fail(KMC_ERR_ARG, "bad arguments");
#ifdef KMC_PHASE_TIMING
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(out, h->d.phase, sizeof(unsigned long long) * otfdev::OTF_NPHASE, cudaMemcpyDeviceToHost));
  if (reset) CK(cudaMemset(h->d.phase, 0, sizeof(unsigned long long) * otfdev::OTF_NPHASE));
  return KMC_OK;
#else
  (void)reset;
  return fail(KMC_ERR_ARG, "library built without KMC_PHASE_TIMING");
#endif
}

int kmc_otf_launch_count(kmc_otf *h, int64_t *n) {
  if (!h || !n) return fail(KMC_ERR_ARG, "bad arguments");
  *n = h->launches;
  return KMC_OK;
}

}  // extern "C"
