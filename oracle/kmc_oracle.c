/*
 * kmc_oracle.c -- CPU restatement of the kmos compiled step loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm may load it,
 * and only as the oracle or as the timed CPU baseline.  The product (kmos_gb300/)
 * never links or calls it.
 *
 * What it restates (mhoffman/kmos, paths relative to the project root):
 *   base.mpy:211-265     del_proc       (swap-remove of avail_sites, literal order)
 *   base.mpy:268-302     add_proc       (append)
 *   base.mpy:304-321     can_do
 *   base.mpy:603-623     update_accum_rate  (serial prefix sum, left to right)
 *   base.mpy:626-645     update_integ_rate  (integ += n*r*dt, left to right)
 *   base.mpy:1075-1120   determine_procsite
 *   base.mpy:1123-1161   update_clocks      (kmc_time += -log(r)/accum(P))
 *   base.mpy:1187-1231   replace_species    (old species check)
 *   base.mpy:1234-1338   interval_search_real (bisection, non-zero scan, left-most scan)
 *   base_lat_int.mpy:243-311 add/del with proc == 0 as a no-op
 *   lattice.mpy:146-210  lattice2nr / nr2lattice (periodic modulo mapping)
 *   proclist_generic_subroutines.mpy:1-110 do_kmc_steps / do_kmc_step /
 *                        get_next_kmc_step (which uses the *time* draw as the site draw)
 *   proclist_generic_subroutines.mpy:113-158 get_occupation
 *   proclist_generic_subroutines.mpy:236-304 initialize_state (reset, defaults, touch-ups)
 * and, for the otf backend (backend 2), kmos/fortran_src/base_otf.f90:
 *   221-283 del_proc (the entry's rate moves with it)    286-331 add_proc (with a rate)
 *   333-364 update_rates_matrix     366-387 reaccumulate_rates_matrix
 *   687-716 update_accum_rate (each list re-summed left to right every step)
 *   719-738 update_integ_rate       1213-1277 determine_procsite (process, then the
 *   entry from the running sum of the chosen list)
 * with the generated gr_<name> rate functions (kmos/io/__init__.py:2657-2965) run from
 * the rate programs of kmos_gb300/otf.py by an evaluator written here (otf_eval), the
 * cell touch-up (io:3240-3285) and recalculate_rates_matrix (proclist_generic_subroutines.mpy:307-325).
 * The process-specific code (generated proclist.f90 / run_proc_*.f90 / nli_*.f90) is
 * taken from the op program that kmos_gb300.program compiles; the op semantics below
 * follow kmos/io/__init__.py:305-465, 1732-2057, 2219-2655.
 *
 * avail_sites is kept in the reference's own column-major layout
 * avail_sites(proc, idx, sw) -> (proc-1) + P*(idx-1) + P*V*(sw-1), independently of the
 * engine's per-process layout.
 *
 * Random numbers: two streams.
 *   ORACLE_RNG_GFORTRAN: the stream gfortran's RANDOM_NUMBER gives for real(8) after
 *     RANDOM_SEED(PUT=seed_arr) with every seed word equal to the kmos seed (libgfortran
 *     of GCC >= 7, libgfortran/intrinsics/random.c): xoshiro256** (Blackman & Vigna,
 *     "Scrambled linear pseudorandom number generators", 2018) whose 256-bit state is
 *     the PUT words XOR-ed with libgfortran's four fixed 64-bit keys; a real(8) draw is
 *     (next() >> 11) * 2^-53.  This is the stream the reference's golden trajectory
 *     (tests/test_run/_tmp_export_BACKEND/ref_procs_sites_BACKEND.log) was produced with.
 *   ORACLE_RNG_PHILOX: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), key
 *     (seed, trajectory), counter (draw counter lo, hi, block, 0); three draws per step
 *     from two blocks, u = ((w_hi:w_lo) >> 11 + 0.5) * 2^-53 in (0, 1).
 *
 * Built with -ffp-contract=off so that n*r and the prefix-sum adds round separately,
 * as gfortran's x86-64 code does.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_OK 0
#define ORACLE_ERR_ARG 1
#define ORACLE_ERR_SPECIES 2     /* replace_species: old species mismatch */
#define ORACLE_ERR_DEADLOCK 3    /* interval_search_real: no available process */
#define ORACLE_ERR_TABLE 4       /* avail_sites inconsistency (add twice / del absent) */
#define ORACLE_ERR_PROGRAM 5

#define ORACLE_RNG_GFORTRAN 0
#define ORACLE_RNG_PHILOX 1

enum { OP_END = 0, OP_REPLACE = 1, OP_GDEL = 2, OP_ADD = 3, OP_LI_DEL = 4, OP_LI_ADD = 5, OP_STRIP = 6,
       OP_UPDATE = 7 };

typedef struct {
    /* program */
    int32_t *prog;
    int prog_len;
    int backend, P, nspecies, null_species, spuck, dim, ngroups, nlayers;
    int off_proc, off_touch, off_groups, off_site_layer, off_site_default;
    /* system */
    int X, Y, Z, V;
    int32_t *lattice;        /* lattice(V), 1-based through lat() */
    int32_t *avail_sites;    /* avail_sites(P, V, 2), column-major */
    int32_t *nr_of_sites;    /* (P) */
    double *rates, *accum_rates, *integ_rates;
    int64_t *procstat;
    double kmc_time, kmc_time_step;
    int64_t kmc_step;
    /* rng */
    int rng_kind;
    uint64_t xs[4];
    uint32_t seed, traj;
    uint64_t ctr;
    /* instrumentation: int32 avail_sites / nr_of_sites accesses made by run_proc_nr
     * (add_proc, del_proc, can_do) and occupation reads/writes, as the Fortran does them */
    int64_t n_as, n_occ;
    int err;
    /* otf: rates_matrix(P, V+1) column-major like avail_sites, user parameters,
     * the rate-record table and the running-sum scratch of determine_procsite */
    double *rm, *userpar, *accum_proc;
    int nuser, off_rate;
} oracle_t;

/* ----------------------------------------------------------------- random numbers */
static uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t xoshiro_next(uint64_t *s)
{
    const uint64_t result = rotl64(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return result;
}

static void gfortran_seed(uint64_t *s, int32_t seed)
{
    /* libgfortran scrambles the PUT words with four fixed keys before using them */
    static const uint64_t keys[4] = {
        0xbd0c5b6e50c2df49ULL, 0xd46061cd46e1df38ULL, 0xbb4f4d4ed6103544ULL, 0x114a583d0756ad39ULL};
    uint64_t w = ((uint64_t)(uint32_t)seed << 32) | (uint64_t)(uint32_t)seed;
    for (int i = 0; i < 4; i++) s[i] = w ^ keys[i];
}

static void philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static double u53_open(uint32_t hi, uint32_t lo)
{
    uint64_t x = ((uint64_t)hi << 32) | lo;
    return ((double)(x >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

static void draw3(oracle_t *o, double *r0, double *r1, double *r2)
{
    if (o->rng_kind == ORACLE_RNG_GFORTRAN) {
        *r0 = (double)(xoshiro_next(o->xs) >> 11) * (1.0 / 9007199254740992.0);
        *r1 = (double)(xoshiro_next(o->xs) >> 11) * (1.0 / 9007199254740992.0);
        *r2 = (double)(xoshiro_next(o->xs) >> 11) * (1.0 / 9007199254740992.0);
    } else {
        uint32_t key[2] = {o->seed, o->traj};
        uint32_t c[4] = {(uint32_t)o->ctr, (uint32_t)(o->ctr >> 32), 0u, 0u};
        uint32_t a[4], b[4];
        philox4x32_10(c, key, a);
        c[2] = 1u;
        philox4x32_10(c, key, b);
        *r0 = u53_open(a[0], a[1]);
        *r1 = u53_open(a[2], a[3]);
        *r2 = u53_open(b[0], b[1]);
        o->ctr++;
    }
}

/* ------------------------------------------------------------------ table access */
#define AS(o, p, i, sw) (o)->avail_sites[((p) - 1) + (int64_t)(o)->P * ((i) - 1) + (int64_t)(o)->P * (o)->V * ((sw) - 1)]

static int lat_get(oracle_t *o, int site) { o->n_occ++; return o->lattice[site - 1]; }
static void lat_set(oracle_t *o, int site, int s) { o->n_occ++; o->lattice[site - 1] = s; }

static int can_do(oracle_t *o, int p, int site) { o->n_as++; return AS(o, p, site, 2) != 0; }

#define RM(o, p, i) (o)->rm[((p) - 1) + (int64_t)(o)->P * ((i) - 1)]

static void add_proc_rate(oracle_t *o, int p, int site, double rate);

static void add_proc(oracle_t *o, int p, int site)
{
    if (o->backend == 2) { add_proc_rate(o, p, site, 0.0); return; }
    if (o->backend == 1 && p == 0) return; /* lat_int: nli found no member */
    if (AS(o, p, site, 2) != 0) { o->err = ORACLE_ERR_TABLE; return; }
    o->nr_of_sites[p - 1] += 1;
    AS(o, p, o->nr_of_sites[p - 1], 1) = site;
    AS(o, p, site, 2) = o->nr_of_sites[p - 1];
    o->n_as += 4; /* n read+write, two table writes */
}

static void del_proc(oracle_t *o, int p, int site)
{
    if (o->backend == 1 && p == 0) return;
    int m = AS(o, p, site, 2);
    o->n_as += 2;
    if (m == 0) { o->err = ORACLE_ERR_TABLE; return; }
    int n = o->nr_of_sites[p - 1];
    if (m < n) {
        AS(o, p, m, 1) = AS(o, p, n, 1);
        AS(o, p, n, 1) = 0;
        if (o->backend == 2) {
            RM(o, p, o->V + 1) = RM(o, p, o->V + 1) - RM(o, p, m);
            RM(o, p, m) = RM(o, p, n);
            RM(o, p, n) = 0.0;
        }
        AS(o, p, AS(o, p, m, 1), 2) = m;
        o->n_as += 5;
    } else {
        AS(o, p, m, 1) = 0;
        if (o->backend == 2) {
            RM(o, p, o->V + 1) = RM(o, p, o->V + 1) - RM(o, p, m);
            RM(o, p, m) = 0.0;
        }
        o->n_as += 1;
    }
    AS(o, p, site, 2) = 0;
    o->nr_of_sites[p - 1] = n - 1;
    o->n_as += 2;
}

static void add_proc_rate(oracle_t *o, int p, int site, double rate)
{
    if (AS(o, p, site, 2) != 0) { o->err = ORACLE_ERR_TABLE; return; }
    o->nr_of_sites[p - 1] += 1;
    int n = o->nr_of_sites[p - 1];
    AS(o, p, n, 1) = site;
    AS(o, p, site, 2) = n;
    RM(o, p, o->V + 1) = RM(o, p, o->V + 1) + rate;
    RM(o, p, n) = rate;
}

static void update_rates_matrix(oracle_t *o, int p, int site, double rate)
{
    int m = AS(o, p, site, 2);
    if (m == 0) { o->err = ORACLE_ERR_TABLE; return; }
    RM(o, p, o->V + 1) = RM(o, p, o->V + 1) + rate - RM(o, p, m);
    RM(o, p, m) = rate;
}

/* -------------------------------------------------------------- lattice mapping */
static int modp(int a, int b) { int r = a % b; return r < 0 ? r + b : r; }

static int lattice2nr(oracle_t *o, int x, int y, int z, int n)
{
    return o->spuck * (modp(x, o->X) + o->X * (modp(y, o->Y) + o->Y * modp(z, o->Z))) + n;
}

static void nr2lattice(oracle_t *o, int nr, int *x, int *y, int *z, int *n)
{
    int c = (nr - 1) / o->spuck;
    *n = nr - o->spuck * c;
    *x = c % o->X;
    *y = (c / o->X) % o->Y;
    *z = c / (o->X * o->Y);
}

static void unpack(int32_t w, int *dx, int *dy, int *dz, int *n)
{
    uint32_t u = (uint32_t)w;
    *dx = (int8_t)(u & 0xFF);
    *dy = (int8_t)((u >> 8) & 0xFF);
    *dz = (int8_t)((u >> 16) & 0xFF);
    *n = (int)((u >> 24) & 0xFF);
}

static int coord_site(oracle_t *o, int bx, int by, int bz, int32_t w)
{
    int dx, dy, dz, n;
    unpack(w, &dx, &dy, &dz, &n);
    return lattice2nr(o, bx + dx, by + dy, bz + dz, n);
}

static int in_mask(int species, int32_t mask)
{
    int bit = species < 0 ? 31 : species;
    return ((uint32_t)mask >> bit) & 1u;
}

/* nli_<group>: the member whose conditions all hold, the last one on identical paths;
 * 0 when none holds (kmos/io/__init__.py:1985-2057). */
static int nli(oracle_t *o, int g, int cx, int cy, int cz)
{
    const int32_t *rec = o->prog + o->prog[o->off_groups + g];
    int M = rec[0], K = rec[1];
    const int32_t *coords = rec + 2;
    int sp[64];
    if (K > 64) { o->err = ORACLE_ERR_PROGRAM; return 0; }
    for (int k = 0; k < K; k++) sp[k] = lat_get(o, coord_site(o, cx, cy, cz, coords[k]));
    int result = 0;
    const int32_t *mem = coords + K;
    for (int m = 0; m < M; m++, mem += 1 + K) {
        int ok = 1;
        for (int k = 0; k < K && ok; k++) ok = in_mask(sp[k], mem[1 + k]);
        if (ok) result = mem[0];
    }
    return result;
}

/* --------------------------------------------------------- otf rate programs */
enum { I_END = 0, I_PUSH_BASE = 1, I_PUSH_PAR = 2, I_PUSH_NR = 3, I_PUSH_INT = 4, I_PUSH_CONST = 5,
       I_LOAD_AUX = 6, I_STORE_AUX = 7, I_STORE_RESULT = 8, I_ADD = 10, I_SUB, I_MUL, I_DIV, I_NEG,
       I_POWI, I_POW, I_EXP, I_LOG, I_SQRT, I_ABS, I_CVT };
enum { K_INT = 0, K_F32 = 1, K_F64 = 2 };

static int32_t wrap32(int64_t v) { return (int32_t)(uint32_t)(uint64_t)v; }

/* x ** m for an integer m: libgcc's __powidf2 / __powisf2 (right-to-left binary powering
 * in the base's precision, the reciprocal for m < 0); gfortran's pow_i4_i4 for integers. */
static double powi_kind(double xd, int32_t m, int kind)
{
    uint32_t n = m < 0 ? -(uint32_t)m : (uint32_t)m;
    if (kind == K_F32) {
        float x = (float)xd, y = (n % 2) ? x : 1.0f;
        while (n >>= 1) { x = x * x; if (n % 2) y = y * x; }
        return m < 0 ? (double)(1.0f / y) : (double)y;
    }
    if (kind == K_F64) {
        double x = xd, y = (n % 2) ? x : 1.0;
        while (n >>= 1) { x = x * x; if (n % 2) y = y * x; }
        return m < 0 ? 1.0 / y : y;
    }
    int64_t x = (int64_t)xd, y = (n % 2) ? x : 1;
    while (n >>= 1) { x = wrap32(x * x); if (n % 2) y = wrap32(y * x); }
    if (m < 0) return (y == 1 || y == -1) ? (double)((-(int64_t)m) % 2 ? y : 1) : 0.0;
    return (double)y;
}

/* Runs a rate program (kmos_gb300/otf.py) on the stack machine: values are held as
 * doubles and rounded to their Fortran kind by each instruction. */
static double otf_eval(oracle_t *o, const int32_t *code, double base, const int32_t *nr)
{
    double st[32], aux[8] = {0}, result = 0.0;
    int sp = 0;
    for (int pc = 0;;) {
        uint32_t w = (uint32_t)code[pc++];
        int op = w & 0xFF, kind = (w >> 8) & 0xFF, arg = (int)(w >> 16);
        if (sp > 30) { o->err = ORACLE_ERR_PROGRAM; return 0.0; }
        switch (op) {
        case I_END: return result;
        case I_PUSH_BASE: st[sp++] = base; break;
        case I_PUSH_PAR: st[sp++] = arg < o->nuser ? o->userpar[arg] : 0.0; break;
        case I_PUSH_NR: st[sp++] = (double)nr[arg]; break;
        case I_PUSH_INT: st[sp++] = (double)code[pc++]; break;
        case I_PUSH_CONST: {
            uint64_t bits = (uint64_t)(uint32_t)code[pc] | ((uint64_t)(uint32_t)code[pc + 1] << 32);
            double v;
            memcpy(&v, &bits, 8);
            st[sp++] = v;
            pc += 2;
            break;
        }
        case I_LOAD_AUX: st[sp++] = aux[arg & 7]; break;
        case I_STORE_AUX: aux[arg & 7] = st[--sp]; break;
        case I_STORE_RESULT: result = st[--sp]; break;
        case I_ADD: case I_SUB: case I_MUL: case I_DIV: {
            double b = st[--sp], a = st[sp - 1], r;
            if (kind == K_INT) {
                int64_t ia = (int64_t)a, ib = (int64_t)b;
                r = op == I_ADD ? wrap32(ia + ib) : op == I_SUB ? wrap32(ia - ib) : op == I_MUL ? wrap32(ia * ib)
                  : (ib == 0 ? 0 : wrap32(ia / ib));
            } else if (kind == K_F32) {
                float fa = (float)a, fb = (float)b;
                r = op == I_ADD ? fa + fb : op == I_SUB ? fa - fb : op == I_MUL ? fa * fb : fa / fb;
            } else {
                r = op == I_ADD ? a + b : op == I_SUB ? a - b : op == I_MUL ? a * b : a / b;
            }
            st[sp - 1] = r;
            break;
        }
        case I_NEG: st[sp - 1] = kind == K_INT ? (double)wrap32(-(int64_t)st[sp - 1]) : -st[sp - 1]; break;
        case I_POWI: { double m = st[--sp]; st[sp - 1] = powi_kind(st[sp - 1], (int32_t)m, kind); break; }
        case I_POW: {
            double b = st[--sp], a = st[sp - 1];
            st[sp - 1] = kind == K_F32 ? (double)powf((float)a, (float)b) : pow(a, b);
            break;
        }
        case I_EXP: st[sp - 1] = kind == K_F32 ? (double)expf((float)st[sp - 1]) : exp(st[sp - 1]); break;
        case I_LOG: st[sp - 1] = kind == K_F32 ? (double)logf((float)st[sp - 1]) : log(st[sp - 1]); break;
        case I_SQRT: st[sp - 1] = kind == K_F32 ? (double)sqrtf((float)st[sp - 1]) : sqrt(st[sp - 1]); break;
        case I_ABS: st[sp - 1] = fabs(st[sp - 1]); break;
        case I_CVT:
            if (kind == K_INT && arg == K_F32) st[sp - 1] = (double)(float)(int32_t)st[sp - 1];
            break;  /* int -> double and float -> double are exact */
        default: o->err = ORACLE_ERR_PROGRAM; return 0.0;
        }
    }
}

/* gr_<p>(cell) (kmos/io/__init__.py:2800-2965): count the bystanders' species into the
 * nr variables, then the rate program with base_rate = rates(p). */
static double gr(oracle_t *o, int p, int cx, int cy, int cz)
{
    const int32_t *r = o->prog + o->prog[o->off_rate + p - 1];
    int nb = r[0], nv = r[1];
    int32_t nr[64] = {0};
    if (nv > 64) { o->err = ORACLE_ERR_PROGRAM; return 0.0; }
    const int32_t *b = r + 4;
    for (int k = 0; k < nb; k++) {
        int sp = lat_get(o, coord_site(o, cx, cy, cz, b[0]));
        int npairs = b[1];
        for (int j = 0; j < npairs; j++)
            if (sp == b[2 + 2 * j]) nr[b[3 + 2 * j]] += 1;
        b += 2 + 2 * npairs;
    }
    return otf_eval(o, b, o->rates[p - 1], nr);
}

static void run_stream(oracle_t *o, int pos, int bx, int by, int bz)
{
    const int32_t *w = o->prog;
    for (;;) {
        if (o->err) return;
        uint32_t h = (uint32_t)w[pos];
        int op = h & 0xFF, cnt = (h >> 8) & 0xFF, arg = (h >> 16) & 0xFFFF;
        switch (op) {
        case OP_END:
            return;
        case OP_REPLACE: {
            int site = coord_site(o, bx, by, bz, w[pos + 1]);
            if (!in_mask(lat_get(o, site), w[pos + 2])) { o->err = ORACLE_ERR_SPECIES; return; }
            lat_set(o, site, w[pos + 3]);
            pos += 4;
            break;
        }
        case OP_GDEL: {
            int site = coord_site(o, bx, by, bz, w[pos + 1]);
            if (can_do(o, arg, site)) del_proc(o, arg, site);
            pos += 2;
            break;
        }
        case OP_ADD: {
            int site = coord_site(o, bx, by, bz, w[pos + 1]);
            int ok = 1;
            for (int c = 0; c < cnt && ok; c++) {
                int s2 = coord_site(o, bx, by, bz, w[pos + 2 + 2 * c]);
                ok = in_mask(lat_get(o, s2), w[pos + 3 + 2 * c]);
            }
            if (ok) {
                if (o->backend == 2) {
                    int dx, dy, dz, n;
                    unpack(w[pos + 1], &dx, &dy, &dz, &n);
                    add_proc_rate(o, arg, site, gr(o, arg, bx + dx, by + dy, bz + dz));
                } else {
                    add_proc(o, arg, site);
                }
            }
            pos += 2 + 2 * cnt;
            break;
        }
        case OP_UPDATE: {
            int dx, dy, dz, n;
            unpack(w[pos + 1], &dx, &dy, &dz, &n);
            int site = lattice2nr(o, bx + dx, by + dy, bz + dz, n);
            if (can_do(o, arg, site)) update_rates_matrix(o, arg, site, gr(o, arg, bx + dx, by + dy, bz + dz));
            pos += 2;
            break;
        }
        case OP_LI_DEL:
        case OP_LI_ADD: {
            int dx, dy, dz, n;
            unpack(w[pos + 1], &dx, &dy, &dz, &n);
            int p = nli(o, arg, bx + dx, by + dy, bz + dz);
            int site = lattice2nr(o, bx + dx, by + dy, bz + dz, n);
            if (op == OP_LI_DEL) del_proc(o, p, site); else add_proc(o, p, site);
            pos += 2;
            break;
        }
        case OP_STRIP: {
            int site = coord_site(o, bx, by, bz, w[pos + 1]);
            for (int p = 1; p <= o->P; p++)
                if (can_do(o, p, site)) del_proc(o, p, site);
            pos += 2;
            break;
        }
        default:
            o->err = ORACLE_ERR_PROGRAM;
            return;
        }
    }
}

/* ---------------------------------------------------------------- base routines */
static void update_accum_rate(oracle_t *o)
{
    if (o->backend == 2) {  /* base_otf.f90:687-716 */
        for (int i = 1; i <= o->P; i++) {
            RM(o, i, o->V + 1) = 0.0;
            for (int j = 1; j <= o->nr_of_sites[i - 1]; j++) RM(o, i, o->V + 1) = RM(o, i, o->V + 1) + RM(o, i, j);
            o->accum_rates[i - 1] = i == 1 ? RM(o, 1, o->V + 1) : o->accum_rates[i - 2] + RM(o, i, o->V + 1);
        }
        return;
    }
    o->accum_rates[0] = (double)o->nr_of_sites[0] * o->rates[0];
    for (int i = 1; i < o->P; i++)
        o->accum_rates[i] = o->accum_rates[i - 1] + (double)o->nr_of_sites[i] * o->rates[i];
}

static void update_integ_rate(oracle_t *o)
{
    if (o->backend == 2) {  /* base_otf.f90:719-738 */
        for (int i = 0; i < o->P; i++)
            o->integ_rates[i] = o->integ_rates[i] + RM(o, i + 1, o->V + 1) * o->kmc_time_step;
        return;
    }
    for (int i = 0; i < o->P; i++)
        o->integ_rates[i] = o->integ_rates[i] + (double)o->nr_of_sites[i] * o->rates[i] * o->kmc_time_step;
}

static void update_clocks(oracle_t *o, double ran_time)
{
    o->kmc_time_step = -log(ran_time) / o->accum_rates[o->P - 1];
    o->kmc_time = o->kmc_time + o->kmc_time_step;
    o->kmc_step = o->kmc_step + 1;
}

/* interval_search_real, literally: bisection, then a scan right past zeros, then a
 * scan left over equal values.  Returns 1-based index, 0 on dead lock. */
static int interval_search_real(const double *arr, int size, double value)
{
    int left = 1, right = size, mid;
    for (;;) {
        mid = (right + left) >> 1;
        if (left >= right) break;
        if (value < arr[mid - 1]) right = mid; else left = mid + 1;
    }
    if (arr[mid - 1] == 0.0) {
        for (;;) {
            if (arr[mid - 1] > 0.0) break;
            if (mid >= size) return 0; /* the reference stops here ("dead-lock") */
            mid = mid + 1;
        }
    }
    while (mid != 1 && arr[mid - 2] >= arr[mid - 1]) mid = mid - 1;
    return mid;
}

static int determine_procsite(oracle_t *o, double ran_proc, double ran_site, int *proc, int *site)
{
    int p = interval_search_real(o->accum_rates, o->P, ran_proc * o->accum_rates[o->P - 1]);
    if (p == 0) return ORACLE_ERR_DEADLOCK;
    int n = o->nr_of_sites[p - 1];
    if (n <= 0) return ORACLE_ERR_DEADLOCK;
    if (o->backend == 2) {  /* base_otf.f90:1213-1277 */
        o->accum_proc[0] = RM(o, p, 1);
        for (int i = 2; i <= n; i++) o->accum_proc[i - 1] = o->accum_proc[i - 2] + RM(o, p, i);
        int k = interval_search_real(o->accum_proc, n, ran_site * o->accum_proc[n - 1]);
        if (k == 0) return ORACLE_ERR_DEADLOCK;
        *proc = p;
        *site = AS(o, p, k, 1);
        return ORACLE_OK;
    }
    int idx = (int)(1.0 + ran_site * (double)n);
    if (idx > n) idx = n;
    *proc = p;
    *site = AS(o, p, idx, 1);
    return ORACLE_OK;
}

/* ----------------------------------------------------------------- exported API */
void oracle_destroy(oracle_t *o)
{
    if (!o) return;
    free(o->prog); free(o->lattice); free(o->avail_sites); free(o->nr_of_sites);
    free(o->rates); free(o->accum_rates); free(o->integ_rates); free(o->procstat);
    free(o->rm); free(o->userpar); free(o->accum_proc);
    free(o);
}

int oracle_run_proc_nr(oracle_t *o, int proc, int site)
{
    if (proc < 1 || proc > o->P || site < 1 || site > o->V) return ORACLE_ERR_ARG;
    int x, y, z, n;
    o->procstat[proc - 1] += 1;
    nr2lattice(o, site, &x, &y, &z, &n);
    run_stream(o, o->prog[o->off_proc + proc - 1], x, y, z);
    return o->err;
}

int oracle_touchup(oracle_t *o, int site)
{
    int x, y, z, n;
    if (site < 1 || site > o->V) return ORACLE_ERR_ARG;
    nr2lattice(o, site, &x, &y, &z, &n);
    int idx = o->backend >= 1 ? 0 : n - 1;  /* lat_int: one touch-up per cell; otf: touchup_cell */
    run_stream(o, o->prog[o->off_touch + idx], x, y, z);
    return o->err;
}

/* initialize_state (proclist_generic_subroutines.mpy:236-304) for layer `layer`. */
static int initialize_state(oracle_t *o, int layer)
{
    const int32_t *site_layer = o->prog + o->off_site_layer;
    const int32_t *site_def = o->prog + o->off_site_default;
    for (int k = 0; k < o->Z; k++)
        for (int j = 0; j < o->Y; j++)
            for (int i = 0; i < o->X; i++) {
                for (int nr = 1; nr <= o->spuck; nr++) {
                    int s = lattice2nr(o, i, j, k, nr);
                    /* reset_site(site, null_species): species is null already */
                    if (lat_get(o, s) != o->null_species) return ORACLE_ERR_SPECIES;
                    lat_set(o, s, o->null_species);
                    for (int p = 1; p <= o->P; p++)
                        if (can_do(o, p, s)) del_proc(o, p, s);
                }
                for (int nr = 1; nr <= o->spuck; nr++)
                    if (site_layer[nr - 1] == layer) {
                        int s = lattice2nr(o, i, j, k, nr);
                        lat_set(o, s, site_def[nr - 1]);
                    }
            }
    for (int k = 0; k < o->Z; k++)
        for (int j = 0; j < o->Y; j++)
            for (int i = 0; i < o->X; i++) {
                if (o->backend >= 1) {
                    run_stream(o, o->prog[o->off_touch], i, j, k);
                } else {
                    for (int nr = 1; nr <= o->spuck; nr++)
                        if (site_layer[nr - 1] == layer)
                            run_stream(o, o->prog[o->off_touch + nr - 1], i, j, k);
                }
                if (o->err) return o->err;
            }
    return o->err;
}

oracle_t *oracle_create(const int32_t *prog, int prog_len, int X, int Y, int Z, int layer,
                        int32_t seed, int rng_kind, uint32_t traj, int *status)
{
    *status = ORACLE_ERR_ARG;
    if (prog_len < 20 || (uint32_t)prog[0] != 0x4B4D4331u || prog[1] != 1) return NULL;
    oracle_t *o = (oracle_t *)calloc(1, sizeof(oracle_t));
    o->prog = (int32_t *)malloc(sizeof(int32_t) * prog_len);
    memcpy(o->prog, prog, sizeof(int32_t) * prog_len);
    o->prog_len = prog_len;
    o->backend = prog[2]; o->P = prog[3]; o->nspecies = prog[4]; o->null_species = prog[5];
    o->spuck = prog[6]; o->dim = prog[7]; o->ngroups = prog[8]; o->nlayers = prog[9];
    o->off_proc = prog[10]; o->off_touch = prog[11]; o->off_groups = prog[12];
    o->off_site_layer = prog[13]; o->off_site_default = prog[14];
    if (X < 1 || Y < 1 || Z < 1 || o->P < 1) { oracle_destroy(o); return NULL; }
    o->X = X; o->Y = Y; o->Z = Z;
    o->V = X * Y * Z * o->spuck;
    o->lattice = (int32_t *)malloc(sizeof(int32_t) * o->V);
    for (int i = 0; i < o->V; i++) o->lattice[i] = o->null_species;
    o->avail_sites = (int32_t *)calloc((size_t)o->P * o->V * 2, sizeof(int32_t));
    o->nr_of_sites = (int32_t *)calloc(o->P, sizeof(int32_t));
    o->rates = (double *)calloc(o->P, sizeof(double));
    o->accum_rates = (double *)calloc(o->P, sizeof(double));
    o->integ_rates = (double *)calloc(o->P, sizeof(double));
    o->procstat = (int64_t *)calloc(o->P, sizeof(int64_t));
    if (o->backend == 2) {
        o->off_rate = prog[22];
        o->nuser = prog[23];
        o->rm = (double *)calloc((size_t)o->P * (o->V + 1), sizeof(double));
        o->userpar = (double *)calloc(o->nuser > 0 ? o->nuser : 1, sizeof(double));
        o->accum_proc = (double *)calloc(o->V, sizeof(double));
    }
    o->rng_kind = rng_kind;
    o->seed = (uint32_t)seed;
    o->traj = traj;
    gfortran_seed(o->xs, seed);
    *status = initialize_state(o, layer);
    o->n_as = o->n_occ = 0;
    return o;
}

/* The tables of a given lattice from scratch: every table emptied, then the touch-up of
 * every site (of every site type; lat_int: of every cell) as initialize_state runs them
 * (proclist_generic_subroutines.mpy:236-304).  A touch-up lists exactly the processes
 * whose conditions hold at its site, so the entries are the processes the lattice enables
 * -- in touch-up order, which need not be the order an incremental run reaches.  Used by
 * the tests as a size-independent invariant of long runs. */
int oracle_rebuild_tables(oracle_t *o, const int32_t *lattice)
{
    for (int i = 0; i < o->V; i++) o->lattice[i] = lattice[i];
    memset(o->avail_sites, 0, sizeof(int32_t) * (size_t)o->P * o->V * 2);
    memset(o->nr_of_sites, 0, sizeof(int32_t) * o->P);
    if (o->backend == 2) memset(o->rm, 0, sizeof(double) * (size_t)o->P * (o->V + 1));
    o->err = 0;
    for (int k = 0; k < o->Z; k++)
        for (int j = 0; j < o->Y; j++)
            for (int i = 0; i < o->X; i++) {
                if (o->backend >= 1) {
                    run_stream(o, o->prog[o->off_touch], i, j, k);
                } else {
                    for (int nr = 1; nr <= o->spuck; nr++) run_stream(o, o->prog[o->off_touch + nr - 1], i, j, k);
                }
                if (o->err) return o->err;
            }
    return o->err;
}

void oracle_set_rate_const(oracle_t *o, int proc, double rate) { o->rates[proc - 1] = rate; }

/* otf: update_user_parameter (proclist_pars, io:2755-2762) */
void oracle_set_user_parameter(oracle_t *o, int k, double v) { if (k >= 1 && k <= o->nuser) o->userpar[k - 1] = v; }

/* otf: recalculate_rates_matrix (proclist_generic_subroutines.mpy:307-325): every available entry's rate re-evaluated,
 * then reaccumulate_rates_matrix (base_otf.f90:366-387). */
int oracle_recalculate_rates_matrix(oracle_t *o)
{
    if (o->backend != 2) return ORACLE_ERR_ARG;
    for (int p = 1; p <= o->P; p++)
        for (int i = 1; i <= o->nr_of_sites[p - 1]; i++) {
            int x, y, z, n;
            nr2lattice(o, AS(o, p, i, 1), &x, &y, &z, &n);
            RM(o, p, i) = gr(o, p, x, y, z);
        }
    for (int p = 1; p <= o->P; p++) {
        RM(o, p, o->V + 1) = 0.0;
        for (int i = 1; i <= o->V; i++) {
            if (AS(o, p, i, 1) > 0) RM(o, p, o->V + 1) = RM(o, p, o->V + 1) + RM(o, p, i);
            else RM(o, p, i) = 0.0;
        }
    }
    return o->err;
}

/* otf: get_rate (base_otf.f90:1121-1145): rates_matrix(p, idx), idx = V+1 the total */
double oracle_get_rates_matrix(oracle_t *o, int p, int idx) { return o->backend == 2 ? RM(o, p, idx) : 0.0; }
void oracle_update_accum_rate(oracle_t *o) { update_accum_rate(o); }
void oracle_update_integ_rate(oracle_t *o) { update_integ_rate(o); }

/* do_kmc_steps(n) (proclist_generic_subroutines.mpy:1-44) */
int oracle_do_kmc_steps(oracle_t *o, int64_t n)
{
    for (int64_t i = 0; i < n; i++) {
        double ran_time, ran_proc, ran_site;
        int proc, site;
        draw3(o, &ran_time, &ran_proc, &ran_site);
        update_accum_rate(o);
        if (!(o->accum_rates[o->P - 1] > 0.0)) return ORACLE_ERR_DEADLOCK;
        update_clocks(o, ran_time);
        update_integ_rate(o);
        int st = determine_procsite(o, ran_proc, ran_site, &proc, &site);
        if (st) return st;
        st = oracle_run_proc_nr(o, proc, site);
        if (st) return st;
    }
    return ORACLE_OK;
}

/* get_next_kmc_step (proclist_generic_subroutines.mpy:85-110): note the time draw
 * selects the site and no clock is advanced. */
int oracle_get_next_kmc_step(oracle_t *o, int *proc, int *site)
{
    double ran_time, ran_proc, ran_site;
    draw3(o, &ran_time, &ran_proc, &ran_site);
    update_accum_rate(o);
    return determine_procsite(o, ran_proc, ran_time, proc, site);
}

/* Records (proc, site) of n do_kmc_step calls into out[2*i], out[2*i+1]. */
int oracle_trace_steps(oracle_t *o, int64_t n, int32_t *out)
{
    for (int64_t i = 0; i < n; i++) {
        double ran_time, ran_proc, ran_site;
        int proc, site;
        draw3(o, &ran_time, &ran_proc, &ran_site);
        update_accum_rate(o);
        if (!(o->accum_rates[o->P - 1] > 0.0)) return ORACLE_ERR_DEADLOCK;
        update_clocks(o, ran_time);
        update_integ_rate(o);
        int st = determine_procsite(o, ran_proc, ran_site, &proc, &site);
        if (st) return st;
        out[2 * i] = proc;
        out[2 * i + 1] = site;
        st = oracle_run_proc_nr(o, proc, site);
        if (st) return st;
    }
    return ORACLE_OK;
}

int oracle_replace_species(oracle_t *o, int site, int old_species, int new_species)
{
    if (site < 1 || site > o->V) return ORACLE_ERR_ARG;
    if (o->lattice[site - 1] != old_species) return ORACLE_ERR_SPECIES;
    o->lattice[site - 1] = new_species;
    return ORACLE_OK;
}

int oracle_get_species(oracle_t *o, int site) { return o->lattice[site - 1]; }
int oracle_get_volume(oracle_t *o) { return o->V; }
int oracle_get_nrofsites(oracle_t *o, int proc) { return o->nr_of_sites[proc - 1]; }
int oracle_get_avail_site(oracle_t *o, int proc, int idx, int sw) { return AS(o, proc, idx, sw); }
double oracle_get_kmc_time(oracle_t *o) { return o->kmc_time; }
double oracle_get_kmc_time_step(oracle_t *o) { return o->kmc_time_step; }
int64_t oracle_get_kmc_step(oracle_t *o) { return o->kmc_step; }
double oracle_get_rate(oracle_t *o, int proc) { return o->rates[proc - 1]; }
double oracle_get_accum_rate(oracle_t *o, int proc) { return o->accum_rates[proc - 1]; }
double oracle_get_integ_rate(oracle_t *o, int proc) { return o->integ_rates[proc - 1]; }
int64_t oracle_get_procstat(oracle_t *o, int proc) { return o->procstat[proc - 1]; }
void oracle_get_counters(oracle_t *o, int64_t *n_as, int64_t *n_occ) { *n_as = o->n_as; *n_occ = o->n_occ; }
void oracle_reset_counters(oracle_t *o) { o->n_as = 0; o->n_occ = 0; }

/* Copies the state out in the engine's export layout: lattice (V int32), per-process
 * site lists as1[p][0..V] and positions as2[p][0..V] (index 0 unused, 1-based values),
 * nr_of_sites (P), procstat (P), rates/integ (P). */
void oracle_export(oracle_t *o, int32_t *lattice, int32_t *as1, int32_t *as2, int32_t *nsites,
                   int64_t *procstat, double *integ)
{
    int V = o->V, P = o->P;
    for (int i = 0; i < V; i++) lattice[i] = o->lattice[i];
    for (int p = 1; p <= P; p++) {
        as1[(int64_t)(p - 1) * (V + 1)] = 0;
        as2[(int64_t)(p - 1) * (V + 1)] = 0;
        for (int i = 1; i <= V; i++) {
            as1[(int64_t)(p - 1) * (V + 1) + i] = AS(o, p, i, 1);
            as2[(int64_t)(p - 1) * (V + 1) + i] = AS(o, p, i, 2);
        }
        nsites[p - 1] = o->nr_of_sites[p - 1];
        procstat[p - 1] = o->procstat[p - 1];
        integ[p - 1] = o->integ_rates[p - 1];
    }
}

/* get_occupation (proclist_generic_subroutines.mpy:113-158): counts per (species,
 * site index) divided by the number of cells; out is [nspecies_out][spuck]. */
void oracle_get_occupation(oracle_t *o, int nspecies_out, double *out)
{
    memset(out, 0, sizeof(double) * nspecies_out * o->spuck);
    for (int s = 1; s <= o->V; s++) {
        int sp = o->lattice[s - 1];
        int n = (s - 1) % o->spuck;
        if (sp != o->null_species && sp >= 0 && sp < nspecies_out) out[sp * o->spuck + n] += 1.0;
    }
    double cells = (double)(o->X * o->Y * o->Z);
    for (int i = 0; i < nspecies_out * o->spuck; i++) out[i] = out[i] / cells;
}

/* Philox4x32-10 block, exported for the known-answer test. */
void oracle_philox(const uint32_t *ctr, const uint32_t *key, uint32_t *out) { philox4x32_10(ctr, key, out); }

/* Raw draws of either stream, exported for tests. */
void oracle_draws(oracle_t *o, int64_t n, double *out)
{
    for (int64_t i = 0; i < n; i++) draw3(o, &out[3 * i], &out[3 * i + 1], &out[3 * i + 2]);
}
