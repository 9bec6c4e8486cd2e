/*
 * kmc_gb300.h -- C-ABI of the GB300 lattice-kMC step engine (libkmcgb300.so).
 *
 * The engine replaces the compiled step loop of kmos's local_smart and lat_int
 * backends: the f2py extension module ``kmc_model`` with submodules base, lattice and
 * proclist, built by kmos/utils/__init__.py:406-521 and imported by
 * kmos/run/__init__.py:86-114 (mhoffman/kmos; paths relative to that project).  Every
 * entry point returns an int status (KMC_OK or an error below) where the Fortran code
 * would ``stop`` the whole process.  No torch types cross this boundary: plain
 * pointers, sizes and host buffers.
 *
 * Two levels:
 *   - kmc_* on a kmc_handle: one trajectory, the plain drop-in behind the f2py module
 *     interface (one model per handle; handles are independent and re-entrant).
 *   - kmc_pool_*: a device arena holding many resident trajectories of possibly
 *     different models and lattice sizes, run together by one persistent kernel
 *     (batching) and admitted / released while others run (serving).
 *
 * Model programs are int32 arrays produced by kmos_gb300.program.compile_model; their
 * layout is documented there and checked here (magic 0x4B4D4331, version 1).
 *
 * Threads: different handles and pools are independent; one handle or pool is driven
 * by one host thread at a time (kmc_pool_cancel excepted, which any thread may call
 * while a run is in flight).
 */
#ifndef KMC_GB300_H
#define KMC_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define KMC_API __attribute__((visibility("default")))
#else
#define KMC_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define KMC_OK 0
#define KMC_ERR_ARG 1       /* bad argument (proc/site/size out of range, bad handle) */
#define KMC_ERR_SPECIES 2   /* replace_species found another species (base.mpy:1205-1228) */
#define KMC_ERR_DEADLOCK 3  /* no process available (base.mpy:1293-1311) */
#define KMC_ERR_TABLE 4     /* avail_sites inconsistency (del of an absent entry) */
#define KMC_ERR_PROGRAM 5   /* malformed model program */
#define KMC_ERR_NOMEM 6     /* device arena full (serving admission refuses) */
#define KMC_ERR_CUDA 7      /* a CUDA call failed; kmc_last_error() has the text */
#define KMC_ERR_CANCELLED 8 /* the host cancelled a running batch */
#define KMC_ERR_NODEVICE 9  /* no CUDA device visible */

/* random-number streams */
#define KMC_RNG_GFORTRAN 0  /* gfortran RANDOM_NUMBER stream after RANDOM_SEED(PUT=seed words):
                               reproduces the reference's own trajectories */
#define KMC_RNG_PHILOX 1    /* Philox4x32-10 keyed by (seed, trajectory id): counter based,
                               independent of batching and placement */

typedef struct kmc_handle kmc_handle;
typedef struct kmc_pool kmc_pool;

/* Text of the last error on this thread (static storage). */
KMC_API const char *kmc_last_error(void);
/* Library version string. */
KMC_API const char *kmc_version(void);
/* Checks a model program (kmos_gb300.program.compile_model's words) the way
 * kmc_create and kmc_pool_add_model do before anything reaches the device: header,
 * op streams, fast streams (slot references, table indices inside their tables,
 * 16-byte placement), group records and nli tables.  KMC_OK or KMC_ERR_PROGRAM with
 * kmc_last_error() naming the fault.  Needs no GPU. */
KMC_API int kmc_check_program(const int32_t *program, int32_t program_len);

/* ------------------------------------------------------------------------------
 * One trajectory (plain drop-in)
 * ------------------------------------------------------------------------------ */

/* proclist.init(input_system_size, system_name, layer, seed_in, no_banner)
 * (proclist_generic_subroutines.mpy:166-230) -> allocate_system (lattice.mpy:212-317,
 * base.mpy:648-744) + initialize_state (proclist_generic_subroutines.mpy:236-304).
 * dims: system size per axis (unused axes 1).  layer: layer id whose sites get their
 * default species.  rng_kind: KMC_RNG_*.  traj_id: Philox key word (ignored for
 * KMC_RNG_GFORTRAN).  The initial state is built on the device. */
KMC_API int kmc_create(const int32_t *program, int32_t program_len, const int32_t dims[3], int32_t layer,
               int32_t seed, int32_t rng_kind, uint32_t traj_id, kmc_handle **out);
/* lattice.deallocate_system (lattice.mpy:324-340, base.mpy:753) */
KMC_API int kmc_destroy(kmc_handle *h);

/* base.set_rate_const(proc, rate) (base.mpy:581-601); proc is 1-based. */
KMC_API int kmc_set_rate_const(kmc_handle *h, int32_t proc, double rate);
/* base.update_accum_rate (base.mpy:603-623) */
KMC_API int kmc_update_accum_rate(kmc_handle *h);
/* base.update_integ_rate (base.mpy:626-645) */
KMC_API int kmc_update_integ_rate(kmc_handle *h);

/* proclist.do_kmc_steps(n) (proclist_generic_subroutines.mpy:1-44) */
KMC_API int kmc_do_steps(kmc_handle *h, int64_t n);
/* do_kmc_steps(n) that also records the (proc, site) of every step into out[2n]
 * (a host buffer); used to check step-by-step parity. */
KMC_API int kmc_trace_steps(kmc_handle *h, int64_t n, int32_t *out);
/* proclist.get_next_kmc_step (proclist_generic_subroutines.mpy:85-110) */
KMC_API int kmc_get_next_step(kmc_handle *h, int32_t *proc, int32_t *site);
/* proclist.run_proc_nr(proc, site) (generated proclist.f90 / kmos/io/__init__.py:305-465,
 * 1732-1764); proc 1-based, site 1-based. */
KMC_API int kmc_run_proc_nr(kmc_handle *h, int32_t proc, int32_t site);
/* proclist.touchup_<layer>_<site>(site) / touchup_cell(cell) (kmos/io/__init__.py:
 * 2411-2443, 1766-1791); site is the 1-based site index of the site (local_smart) or
 * of any site of the cell (lat_int). */
KMC_API int kmc_touchup(kmc_handle *h, int32_t site);
/* The touch-ups of n sites, in list order, in one launch: what kmos.run's
 * _adjust_database (kmos/run/__init__.py:1439-1457) does with one touchup call per site.
 * Sites as for kmc_touchup; all are checked before any runs. */
KMC_API int kmc_touchup_many(kmc_handle *h, const int32_t *sites, int32_t n);
/* base.get_species(site) (base.mpy:1164-1184) */
KMC_API int kmc_get_species(kmc_handle *h, int32_t site, int32_t *species);
/* base.replace_species(site, old, new) (base.mpy:1187-1231): KMC_ERR_SPECIES unless the
 * site holds old; KMC_ERR_ARG for a new species outside -1..nspecies (the reference does
 * not check it). */
KMC_API int kmc_replace_species(kmc_handle *h, int32_t site, int32_t old_species, int32_t new_species);

/* base.get_kmc_time / set_kmc_time / get_kmc_time_step / get_kmc_step (base.mpy:854-1072) */
KMC_API int kmc_get_kmc_time(kmc_handle *h, double *t);
KMC_API int kmc_set_kmc_time(kmc_handle *h, double t);
KMC_API int kmc_get_kmc_time_step(kmc_handle *h, double *dt);
KMC_API int kmc_get_kmc_step(kmc_handle *h, int64_t *step);
/* base.get_volume (base.mpy:1042), base.nr_of_proc (base.mpy:189) */
KMC_API int kmc_get_volume(kmc_handle *h, int32_t *volume);
KMC_API int kmc_get_nr_of_proc(kmc_handle *h, int32_t *nproc);
/* Whole P-vectors: base.get_procstat(i), get_integ_rate(i), get_rate(i),
 * get_accum_rate(i), get_nrofsites(i) for i = 1..P (base.mpy:888, 968, 991, 945, 907),
 * copied into host arrays. */
KMC_API int kmc_get_procstat(kmc_handle *h, int64_t *out);
KMC_API int kmc_get_integ_rates(kmc_handle *h, double *out);
KMC_API int kmc_get_rates(kmc_handle *h, double *out);
KMC_API int kmc_get_accum_rates(kmc_handle *h, double *out);
KMC_API int kmc_get_nr_of_sites(kmc_handle *h, int32_t *out);
/* base.get_avail_site(proc, idx, sw) (avail_sites(proc, idx, sw), base.mpy:925-942) */
KMC_API int kmc_get_avail_site(kmc_handle *h, int32_t proc, int32_t idx, int32_t sw, int32_t *out);
/* The whole lattice (V species ids) and both book-keeping tables in the engine's
 * per-process layout: as1[p][i] = avail_sites(p+1, i, 1), as2[p][s] = avail_sites(p+1, s, 2)
 * for i, s = 0..V (index 0 unused); buffers of V and P*(V+1) int32. */
KMC_API int kmc_get_lattice(kmc_handle *h, int32_t *out);
KMC_API int kmc_get_tables(kmc_handle *h, int32_t *as1, int32_t *as2);
/* proclist.get_occupation (proclist_generic_subroutines.mpy:113-158): out is
 * [nspecies][spuck] doubles. */
KMC_API int kmc_get_occupation(kmc_handle *h, double *out);

/* ------------------------------------------------------------------------------
 * Many resident trajectories (batching and serving)
 * ------------------------------------------------------------------------------ */

/* A pool owns one device arena of arena_bytes and room for max_slots trajectories. */
KMC_API int kmc_pool_create(int32_t device, size_t arena_bytes, int32_t max_slots, kmc_pool **out);
KMC_API int kmc_pool_destroy(kmc_pool *pool);
/* Registers a model program; returns its id. */
KMC_API int kmc_pool_add_model(kmc_pool *pool, const int32_t *program, int32_t program_len, int32_t *model_id);
/* Device bytes one trajectory of this model and size needs (for admission control). */
KMC_API int kmc_pool_slot_bytes(kmc_pool *pool, int32_t model_id, const int32_t dims[3], size_t *bytes);
/* Free bytes left in the arena (largest contiguous block in *largest). */
KMC_API int kmc_pool_free_bytes(kmc_pool *pool, size_t *total, size_t *largest);
/* Admits one trajectory: allocates its state in the arena and queues its device-side
 * initialisation (initialize_state + rates + update_accum_rate) on the pool stream.
 * rates: P doubles.  Returns KMC_ERR_NOMEM when the arena has no room. */
KMC_API int kmc_pool_admit(kmc_pool *pool, int32_t model_id, const int32_t dims[3], int32_t layer,
                   int32_t seed, int32_t rng_kind, uint32_t traj_id, const double *rates,
                   int32_t *slot);
/* Admits n trajectories at once (one initialisation launch); slots receives n ids. */
KMC_API int kmc_pool_admit_many(kmc_pool *pool, int32_t n, const int32_t *model_ids, const int32_t *dims3,
                        int32_t layer, const int32_t *seeds, int32_t rng_kind, const uint32_t *traj_ids,
                        const double *rates, const int32_t *rate_offsets, int32_t *slots);
/* Frees a trajectory's arena block. */
KMC_API int kmc_pool_release(kmc_pool *pool, int32_t slot);
/* Runs steps[i] kMC steps on slots[i] for i < n in one persistent launch (asynchronous
 * on the pool stream; kmc_pool_sync waits and returns the first error status). */
KMC_API int kmc_pool_run(kmc_pool *pool, const int32_t *slots, const int64_t *steps, int32_t n);
/* Like kmc_pool_run with one step count for every listed slot, replayed from a CUDA
 * graph captured on first use for this (slots, steps) list. */
KMC_API int kmc_pool_run_graph(kmc_pool *pool, const int32_t *slots, int64_t steps, int32_t n);
KMC_API int kmc_pool_sync(kmc_pool *pool);
/* Sets the cancel flag a running batch polls; the batch ends with KMC_ERR_CANCELLED in
 * the slots it did not finish. */
KMC_API int kmc_pool_cancel(kmc_pool *pool);
/* Per-slot results: status, kmc_time, kmc_step, procstat (P), integ_rates (P),
 * nr_of_sites (P), occupation counts ([nspecies][spuck] int64). */
KMC_API int kmc_pool_get_status(kmc_pool *pool, int32_t slot, int32_t *status);
KMC_API int kmc_pool_get_clock(kmc_pool *pool, int32_t slot, double *kmc_time, int64_t *kmc_step);
KMC_API int kmc_pool_get_procstat(kmc_pool *pool, int32_t slot, int64_t *out);
KMC_API int kmc_pool_get_integ_rates(kmc_pool *pool, int32_t slot, double *out);
KMC_API int kmc_pool_get_nr_of_sites(kmc_pool *pool, int32_t slot, int32_t *out);
KMC_API int kmc_pool_get_lattice(kmc_pool *pool, int32_t slot, int32_t *out);
KMC_API int kmc_pool_get_tables(kmc_pool *pool, int32_t slot, int32_t *as1, int32_t *as2);
/* base.set_rate_const for every process of a resident trajectory (rates[P], base.mpy:
 * 581-601) followed by update_accum_rate before its next step: new parameters (T,
 * partial pressures) for a trajectory that keeps its lattice, tables and clock. */
KMC_API int kmc_pool_set_rates(kmc_pool *pool, int32_t slot, const double *rates);
/* Occupation counts of many slots at once, reduced on the device: out[i] holds the
 * [nspecies][spuck] counts of slots[i] (int64), with stride `stride` int64 per slot.
 * A stride below nspecies * spuck of any listed slot's model returns KMC_ERR_ARG.
 * Replaces get_occupation (proclist_generic_subroutines.mpy:113-158) for many slots. */
KMC_API int kmc_pool_occupation_counts(kmc_pool *pool, const int32_t *slots, int32_t n, int32_t stride, int64_t *out);
/* Results of many slots in one device gather and one copy: for slots[i], procstat
 * (int64) and integ_rates (double) into rows of `stride` entries, kmc_time and
 * kmc_step into times[i] / steps[i], status into status[i].  Any output may be null. */
KMC_API int kmc_pool_get_results(kmc_pool *pool, const int32_t *slots, int32_t n, int32_t stride,
                                 int64_t *procstat, double *integ, double *times, int64_t *steps,
                                 int32_t *status);
/* kmc_pool_occupation_counts for callers that must not allocate device memory: code
 * running under a fixed device-memory budget that is already spent (a serving process
 * that has given all of it to resident trajectories), or a real-time loop where a
 * cudaMalloc would synchronise the device.  It has no counterpart in the reference.  Its
 * scratch (slot list and counters) is one static device array of about 2 MB that every
 * call shares: at most KMC_STATIC_OCC_MAX_SLOTS slots and KMC_STATIC_OCC_MAX_STRIDE
 * counters per slot (larger requests, and strides below nspecies * spuck of a listed
 * slot's model, return KMC_ERR_ARG).  The first call on a device looks the array's
 * address up (cudaGetSymbolAddress).  Every call copies to and from host memory and
 * synchronises the pool's stream, so it must not be made during a stream capture or
 * from a CUDA host callback.  Calls whose work overlaps on the GPU (other threads, other
 * pools' streams) race on the array: serialise them. */
#define KMC_STATIC_OCC_MAX_SLOTS 4096
#define KMC_STATIC_OCC_MAX_STRIDE 64
KMC_API int kmc_pool_occupation_counts_static(kmc_pool *pool, const int32_t *slots, int32_t n, int32_t stride,
                                              int64_t *out);
/* Launch configuration used by kmc_pool_run: warps per block (1..16) with blocks_per_sm
 * blocks per SM (0 = as many as fit), or warps_per_block 0 = balanced: one block per SM,
 * the run's trajectories split evenly over the SMs in the fewest rounds per warp. */
KMC_API int kmc_pool_set_launch(kmc_pool *pool, int32_t warps_per_block, int32_t blocks_per_sm);
/* Trajectories per warp of kmc_pool_run: 1 (default, 32 lanes per trajectory) or 2
 * (16 lanes each, for models of up to 64 processes; larger models keep one).  Two per
 * warp double the trajectories an SM holds at a given register budget and let one warp
 * instruction advance both wherever their steps take the same branches.  Results do not
 * depend on it.  The reference has one trajectory per process (one do_kmc_steps loop,
 * proclist_generic_subroutines.mpy:1-44); this is a batching knob of this library. */
KMC_API int kmc_pool_set_trajectories_per_warp(kmc_pool *pool, int32_t n);
/* 1 (default): when every trajectory of a launch fits, each one's lattice and
 * avail_sites tables are copied to shared memory when its group takes it, stepped there
 * and copied back (launches of few, small trajectories: the plain one-trajectory
 * drop-in); 0: always stepped in device memory.  Results do not depend on it. */
KMC_API int kmc_pool_set_tables_on_chip(kmc_pool *pool, int32_t enable);
/* 1 (default): a launch of at most one trajectory per SM whose model has at most 8
 * processes (the plain one-trajectory drop-in of small models) runs each trajectory on
 * one warp of its own with the steps on one lane, as the reference's loop runs them
 * (proclist_generic_subroutines.mpy:1-44), the program, lattice and tables in shared
 * memory; 0: such launches take the group-parallel step kernel.  Results do not depend
 * on it. */
KMC_API int kmc_pool_set_solo(kmc_pool *pool, int32_t enable);
/* 1 (default): steps whose process has a fast stream run through the gather /
 * replay / scatter path; 0: every step runs the serial interpreter (same results). */
KMC_API int kmc_pool_set_fast_path(kmc_pool *pool, int32_t enable);
/* Table placement: 1 (default) copies each model's hot section (fast streams, group
 * records, nli tables; up to 64 KB) into every block's shared memory, 0 reads it from
 * global memory through L1 (more shared memory left for warps). */
KMC_API int kmc_pool_set_table_placement(kmc_pool *pool, int32_t shared);
/* Device time (ms, CUDA events on the pool stream) of the last kmc_pool_run launch. */
KMC_API int kmc_pool_last_kernel_ms(kmc_pool *pool, float *ms);
/* CUDA events on the pool stream around a region of work: start, then stop waits for
 * the region to finish and returns its device time in ms. */
KMC_API int kmc_pool_timer_start(kmc_pool *pool);
KMC_API int kmc_pool_timer_stop(kmc_pool *pool, float *ms);
/* Cycles the step kernel spent per phase, summed over warps, in builds compiled with
 * KMC_PHASE_TIMING (16 entries: draws, accum, clock/integ/bisection, site pick, slot
 * gather, end of edit evaluation, table-load stores, replay, lattice writes, serial
 * interpreter, term refresh, slot sites, then per evaluation round: edit decode and nli,
 * del-position load, del rank and list-entry load, compaction); other builds return
 * KMC_ERR_ARG.  reset != 0 clears the sums. */
KMC_API int kmc_pool_phase_cycles(kmc_pool *pool, uint64_t *out, int32_t reset);
/* Kernel launches issued by this pool since creation. */
KMC_API int kmc_pool_launch_count(kmc_pool *pool, int64_t *count);

/* ------------------------------------------------------------------------------
 * Saving and restoring trajectories (base.save_system / base.reload_system,
 * base.mpy:363-578)
 * ------------------------------------------------------------------------------ */

/* Compact binary image of one trajectory: clock, step, random stream, status,
 * rates / integ_rates / accum_rates / procstat / nr_of_sites, the lattice and the first
 * nr_of_sites(p) entries of avail_sites(p, :, 1) per process (the rest of the tables is
 * rebuilt on load).  *bytes receives the image size; with buf NULL nothing else is done,
 * and a capacity below it returns KMC_ERR_ARG.  Unlike the reference's .reload file the
 * image keeps integ_rates, kmc_time_step and the random stream, so a restored trajectory
 * continues bit for bit. */
KMC_API int kmc_pool_save_state(kmc_pool *pool, int32_t slot, void *buf, size_t capacity, size_t *bytes);
/* Admits a trajectory from an image saved from the same model program (checked by a
 * hash); the image is validated (sizes, species, every table index) before it reaches
 * the device.  The new slot id goes to *slot. */
KMC_API int kmc_pool_restore_state(kmc_pool *pool, int32_t model_id, const void *buf, size_t bytes, int32_t *slot);
/* Checks a state image against a model program without a device: the checks
 * kmc_pool_restore_state / kmc_load_state make before anything reaches the GPU (magic,
 * sizes, program hash, species, every avail_sites entry in 1..volume and listed once per
 * process).  KMC_OK, KMC_ERR_PROGRAM (bad program), KMC_ERR_ARG or KMC_ERR_TABLE (bad
 * image). */
KMC_API int kmc_check_image(const int32_t *program, int32_t program_len, const void *buf, size_t bytes);
/* The same on a handle; kmc_load_state needs an image of the handle's model and size. */
KMC_API int kmc_save_state(kmc_handle *h, void *buf, size_t capacity, size_t *bytes);
KMC_API int kmc_load_state(kmc_handle *h, const void *buf, size_t bytes);
/* base.save_system (base.mpy:489-575): writes the reference's <system_name>.reload
 * layout to `path`, plus "#gb300" comment lines (system size, exact kmc_time, rates and
 * integ_rates, kmc_time_step, random stream) that the reference's reader skips. */
KMC_API int kmc_save_reload(kmc_handle *h, const char *path);
/* First pass of base.reload_system (base.mpy:363-440): nr_of_proc, volume and, from a
 * "#gb300 system_size" line, the system size (zeros when the file has none). */
KMC_API int kmc_reload_info(const char *path, int32_t *nr_of_proc, int32_t *volume, int32_t dims[3]);
/* Checks a .reload file against a model program (lattice or otf) and a system size
 * without a device: the checks kmc_load_reload / kmc_otf_load_reload make before anything
 * reaches the GPU (the counts, every vector's length, species in -1..nspecies, each
 * process's avail_sites columns inverse to each other over its nr_of_sites entries, a
 * known random stream).  No reference counterpart (base.mpy:363-578 reads without
 * checks).  KMC_OK, KMC_ERR_PROGRAM (bad program), KMC_ERR_ARG or KMC_ERR_TABLE (bad
 * file). */
KMC_API int kmc_check_reload(const int32_t *program, int32_t program_len, const int32_t dims[3], const char *path);
/* Second pass of base.reload_system (base.mpy:442-486) into an allocated handle of the
 * same model and volume: kmc_time, walltime, kmc_step, lattice, nr_of_sites, rates,
 * procstat, avail_sites and avail_sites_back, checked for consistency (KMC_ERR_TABLE).
 * Without "#gb300" lines integ_rates and kmc_time_step restart at zero and the handle's
 * random stream continues, as in the reference. */
KMC_API int kmc_load_reload(kmc_handle *h, const char *path);
/* base.get_walltime: host seconds spent in kmc_do_steps (the reference adds CPU_TIME
 * every step, base.mpy:1123-1161). */
KMC_API int kmc_get_walltime(kmc_handle *h, double *walltime);

/* ------------------------------------------------------------------------------
 * On-device sampling (kmos.run.KMC_Model.get_std_sampled_data, run/__init__.py:865-966)
 * ------------------------------------------------------------------------------ */

/* Starts a sampling record for each listed slot (arena memory; KMC_ERR_NOMEM when full):
 * kmc_time, kmc_step, procstat and integ_rates now. */
KMC_API int kmc_pool_sample_begin(kmc_pool *pool, const int32_t *slots, int32_t n);
/* One sample per listed slot, on the pool stream after the work queued before it: the
 * occupation (get_occupation) weighted by kmc_time_step is added to the record. */
KMC_API int kmc_pool_sample(kmc_pool *pool, const int32_t *slots, int32_t n);
/* Ends the records: per slot i, occ_mean[i][occ_stride] = the kmc_time_step-weighted
 * mean occupation ([nspecies][spuck], NaN when every weight was zero),
 * procstat_delta / integ_delta[i][proc_stride] = the change since kmc_pool_sample_begin,
 * times[i] = {total_time, simulated_time}, steps[i] = kMC steps taken, status[i]. */
KMC_API int kmc_pool_sample_end(kmc_pool *pool, const int32_t *slots, int32_t n, int32_t occ_stride,
                                int32_t proc_stride, double *occ_mean, int64_t *procstat_delta,
                                double *integ_delta, double *times, int64_t *steps, int32_t *status);
/* begin, then `samples` times (run steps_per_sample kMC steps on every listed slot,
 * sample), then end -- all queued on the device without a host round trip. */
KMC_API int kmc_pool_sample_run(kmc_pool *pool, const int32_t *slots, int32_t n, int32_t samples,
                                int64_t steps_per_sample, int32_t occ_stride, int32_t proc_stride,
                                double *occ_mean, int64_t *procstat_delta, double *integ_delta, double *times,
                                int64_t *steps, int32_t *status);

/* ------------------------------------------------------------------------------
 * otf backend (kmos/fortran_src/base_otf.f90 + the otf generator, kmos/io/__init__.py:
 * 2657-3723): per-entry rates from bystanders.  A handle holds ntraj independent
 * trajectories of one otf program (kmos_gb300.otf), trajectory t keyed (seed, traj0 + t)
 * on the Philox stream, or all on the gfortran stream of `seed`.  Rate constants and
 * user parameters are shared by the batch.  The f2py module of an otf build exposes the
 * same routines per trajectory: base.set_rate_const, proclist_pars.update_user_parameter,
 * proclist.recalculate_rates_matrix, base.update_accum_rate / update_integ_rate,
 * proclist.do_kmc_steps / get_next_kmc_step / run_proc_nr, base.get_rate.
 * ------------------------------------------------------------------------------ */
typedef struct kmc_otf kmc_otf;

/* The checks kmc_otf_create makes on an otf program (no device needed). */
KMC_API int kmc_otf_check_program(const int32_t *program, int32_t program_len);
/* proclist.init for ntraj trajectories: base.allocate_system (base_otf.f90:741-865) +
 * initialize_state(layer) (proclist_generic_subroutines.mpy:166-304, the cell touch-ups);
 * kmc_otf_destroy is deallocate_system (base_otf.f90:874-932). */
KMC_API int kmc_otf_create(const int32_t *program, int32_t program_len, const int32_t dims[3], int32_t layer,
                           int32_t ntraj, int32_t seed, int32_t rng_kind, uint32_t traj0, kmc_otf **out);
KMC_API int kmc_otf_destroy(kmc_otf *h);
/* base.set_rate_const (base_otf.f90:665-685) */
KMC_API int kmc_otf_set_rate_const(kmc_otf *h, int32_t proc, double rate);
/* proclist_pars.update_user_parameter (kmos/io/__init__.py:2756-2765): k = 1.. in sorted
 * parameter-name order */
KMC_API int kmc_otf_set_user_parameter(kmc_otf *h, int32_t k, double value);
/* proclist.recalculate_rates_matrix + reaccumulate_rates_matrix (proclist_generic_subroutines.mpy:307-325) */
KMC_API int kmc_otf_recalculate_rates_matrix(kmc_otf *h);
/* base.update_accum_rate (base_otf.f90:687-716) / update_integ_rate (719-738) */
KMC_API int kmc_otf_update_accum_rate(kmc_otf *h);
KMC_API int kmc_otf_update_integ_rate(kmc_otf *h);
/* proclist.do_kmc_steps(n) (proclist_generic_subroutines.mpy:1-44) on every trajectory,
 * one launch */
KMC_API int kmc_otf_do_steps(kmc_otf *h, int64_t n);
/* n steps of trajectory traj alone, its (proc, site) pairs to out[2n] */
KMC_API int kmc_otf_trace_steps(kmc_otf *h, int32_t traj, int64_t n, int32_t *out);
/* proclist.get_next_kmc_step (proclist_generic_subroutines.mpy:85-110) / run_proc_nr
 * (kmos/io/__init__.py:3292-3326) of one trajectory */
KMC_API int kmc_otf_get_next_step(kmc_otf *h, int32_t traj, int32_t *proc, int32_t *site);
KMC_API int kmc_otf_run_proc_nr(kmc_otf *h, int32_t traj, int32_t proc, int32_t site);
/* State of one trajectory (NULL skips a field): lattice[V], avail_sites as1/as2[P][V+1],
 * nr_of_sites[P], procstat[P], integ_rates[P], accum_rates[P], rates_matrix[P][V+1]
 * (base.get_rate(p, i) of list position i), totals[P] (get_rate(p, -1) as the last
 * update_accum_rate summed it), clock = {kmc_time, kmc_time_step}, kmc_step. */
KMC_API int kmc_otf_get_state(kmc_otf *h, int32_t traj, int32_t *lattice, int32_t *as1, int32_t *as2,
                              int32_t *nr_of_sites, int64_t *procstat, double *integ_rates, double *accum_rates,
                              double *rates_matrix, double *totals, double clock[2], int64_t *kmc_step);
/* base.set_kmc_time (base_otf.f90:968-982) of one trajectory. */
KMC_API int kmc_otf_set_kmc_time(kmc_otf *h, int32_t traj, double kmc_time);
/* base.replace_species (base_otf.f90:1344-1383): KMC_ERR_SPECIES unless the site holds
 * old_species; the tables are not touched (kmos.run's put then touches up every cell). */
KMC_API int kmc_otf_replace_species(kmc_otf *h, int32_t traj, int32_t site, int32_t old_species,
                                    int32_t new_species);
/* proclist.touchup_cell (io:3240-3284) of n cells, cells[3i..3i+2] = (x, y, z), in the
 * given order (kmos.run's _adjust_database runs x outermost, run/__init__.py:1439-1457),
 * one launch. */
KMC_API int kmc_otf_touchup_cells(kmc_otf *h, int32_t traj, int32_t n, const int32_t *cells);
/* A trajectory's state from the host, as reload_system restores it (base_otf.f90:448-599):
 * lattice[V], avail_sites(:, :, 1) as as1[P][V+1] (entry 0 unused; column 2 is rebuilt as
 * its inverse), nr_of_sites[P], procstat[P], integ_rates[P] (NULL: zero), clock =
 * {kmc_time, kmc_time_step}, kmc_step.  rates_matrix is zero, as the reference's file does
 * not hold it, until kmc_otf_recalculate_rates_matrix.  KMC_ERR_ARG / KMC_ERR_TABLE for a
 * species out of range or a list that names a site twice. */
KMC_API int kmc_otf_set_state(kmc_otf *h, int32_t traj, const int32_t *lattice, const int32_t *as1,
                              const int32_t *nr_of_sites, const int64_t *procstat, const double *integ_rates,
                              const double clock[2], int64_t kmc_step);
/* base.save_system / reload_system of one trajectory (base_otf.f90:448-663): the
 * reference's .reload layout with the same "#gb300" comment lines kmc_save_reload writes
 * (exact clock, rate constants, integ_rates, random stream).  Loading sets the batch's
 * rate constants from the file; walltime: the file's (may be NULL). */
KMC_API int kmc_otf_save_reload(kmc_otf *h, int32_t traj, const char *path, double walltime);
KMC_API int kmc_otf_load_reload(kmc_otf *h, int32_t traj, const char *path, double *walltime);
/* The batch's rate constants (base.rates, base_otf.f90:152, set by set_rate_const,
 * base_otf.f90:665-685), P values. */
KMC_API int kmc_otf_get_rate_consts(kmc_otf *h, double *rates);
/* Rate tables (no reference counterpart; results are the same either way): a process's
 * rate depends only on its bystander counts, so for models whose counts take at most
 * 4096 combinations in all, each combination's rate is computed once by the process's
 * rate program after the rates or user parameters change, and steps look it up.  on = 0
 * evaluates every rate (gr_<name>, io:2800-2965) instead. */
KMC_API int kmc_otf_set_rate_tables(kmc_otf *h, int32_t on);
/* Constant-rate running sums (no reference counterpart; results are the same either
 * way): every entry of a process whose rate program reads no bystander count holds the
 * same rate c once recalculate_rates_matrix has run, so the running sums of its list
 * (update_accum_rate, base_otf.f90:687-716) are fl(pm(i-1) + c) from 0 -- one table per
 * process, filled after the rates or user parameters change, replaces re-summing the
 * list.  Used between recalculate_rates_matrix and the next rate or parameter change,
 * for lattices of up to 65536 sites; on = 0 always sums the lists. */
KMC_API int kmc_otf_set_constant_rate_sums(kmc_otf *h, int32_t on);
/* entries: the rate tables' size in values, whether or not they are in use (0: the model
 * has none). */
KMC_API int kmc_otf_rate_table_entries(kmc_otf *h, int32_t *entries);
/* Device time of the last launch (CUDA events on the handle's stream) and launch count. */
KMC_API int kmc_otf_last_kernel_ms(kmc_otf *h, float *ms);
KMC_API int kmc_otf_launch_count(kmc_otf *h, int64_t *n);
/* Cycles the otf step loop spent per phase, summed over trajectories (8 entries: draws,
 * running sums and accum_rates, clock and integ, pick, event op list, event evaluation,
 * event replay, unused), in builds compiled with KMC_PHASE_TIMING; KMC_ERR_ARG
 * otherwise.  reset != 0 clears them. */
KMC_API int kmc_otf_phase_cycles(kmc_otf *h, uint64_t *out, int32_t reset);

#ifdef __cplusplus
}
#endif
#endif /* KMC_GB300_H */
