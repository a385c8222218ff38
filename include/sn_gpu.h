/*
 * sn_gpu.h -- C ABI of the GB300 Metropolis dipole-lattice sweep.
 *
 * Drop-in boundary for the StarryNight hot loop.  The reference has no
 * library API: its sweep is MC_moves(MCMinorSteps) (src/starrynight-main.c:222,
 * :248) acting on global state -- the lattice `struct dipole ***lattice`
 * (src/starrynight-config.c:32-36), the neighbour list (src/starrynight-
 * montecarlo-core.c:29-36), beta/Efield/CageStrain/K/ConstrainToX
 * (src/starrynight-config.c:62-85) and the ACCEPT/REJECT counters (:26-27).
 * This ABI replaces that region: the host keeps the reference's config keys
 * and driver loop and calls these functions instead.
 *
 * Conventions
 *   - Plain C types only; no CUDA or torch types cross the boundary.
 *   - The caller owns every host buffer; the handle owns all device memory.
 *   - Every function returns sn_status (SN_OK == 0); none calls exit().
 *     sn_gpu_last_error() gives a one-line reason for the last failure.
 *   - One handle is driven by one host thread; its work runs on the handle's
 *     own CUDA stream, in order.
 *   - Lattice arrays are site-major with z fastest: site (x,y,z) is at
 *     index (x*Y + y)*Z + z, the element order of the reference's
 *     lattice[x][y][z].  Dipoles are float triples (x,y,z); lengths are
 *     floats.  A site of length 0 is a vacancy and holds the zero vector.
 *   - Temperatures are float Kelvin; beta = 300/T (energies in units of
 *     k_B * 300 K, src/starrynight-main.c:215).
 */
#ifndef SN_GPU_H
#define SN_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum sn_status {
    SN_OK = 0,
    SN_ERR_ARG = 1,         /* NULL handle/buffer, index out of range, bad value  */
    SN_ERR_CONFIG = 2,      /* parameters the model cannot take (cutoff, species) */
    SN_ERR_SCHEDULE = 3,    /* lattice shape admits no conflict-free block/colour schedule */
    SN_ERR_CUDA = 4,        /* CUDA runtime error (no device, launch failure, ...) */
    SN_ERR_NOMEM = 5,       /* device or host allocation failed */
    SN_ERR_TIMEOUT = 6,     /* a bounded device-side wait ran out */
    SN_ERR_UNSUPPORTED = 7  /* valid request outside what this build implements */
} sn_status;

#define SN_MAX_SPECIES 10 /* dipoles[10], src/starrynight-config.c:39-43 */
#define SN_MAX_CUTOFF 6   /* largest DipoleCutOff with a tiled kernel in this build */

/* Model parameters shared by all replicas: the starrynight.cfg keys of the
 * hot path (src/starrynight-config.c:123-166). */
typedef struct sn_params {
    int cutoff;                      /* DipoleCutOff (lattice units)                    */
    int dim;                         /* 3: sphere proposals; 2: circle (DIM<3 branch)   */
    int constrain_to_x;              /* ConstrainToX: proposals along +-x,+-y,+-z       */
    double cage_strain;              /* CageStrain (double, as the reference holds it)  */
    double K;                        /* K, epitaxial term; applied only when K > 0      */
    float efield[3];                 /* Efield.{x,y,z}; replicas may override           */
    int n_species;                   /* length of Dipoles / Prevalence                  */
    float dipoles[SN_MAX_SPECIES];   /* Dipoles: species lengths (0 = vacancy)          */
    float prevalence[SN_MAX_SPECIES];/* Prevalence: species probabilities               */
    uint64_t seed;                   /* default Philox key for replicas with seed 0     */
    int sweep_method;                /* SN_SWEEP_AUTO / _STENCIL / _CACHED (below)      */
} sn_params;

/* How the sweep forms a move's energy change (sn_params.sweep_method).  Both
 * give the Metropolis sweep of site_energy (src/starrynight-montecarlo-core.c:
 * 76-141); they differ in work and in the last bits of dE.
 *   SN_SWEEP_STENCIL: every attempted move sums the cutoff stencil over the
 *     neighbours' dipoles (the reference's way, on a shared-memory tile).
 *   SN_SWEEP_CACHED: the local field of every site is kept in HBM as exact
 *     fixed-point sums (each neighbour's contribution rounded to 2^-k on its
 *     own, k about 20); an attempt reads it, an accepted move adds its
 *     neighbours' changes.  Work per attempt no longer grows with the
 *     cutoff, only per accepted move.  Needs every 3D block side >= 2 cutoff,
 *     Z a multiple of 4 and dipoles with |components| <= 1; 2D replicas always
 *     use the stencil.
 *   SN_SWEEP_AUTO (0): CACHED where every 3D replica of the table admits it,
 *     else STENCIL.  The environment variable SN_SWEEP=stencil|cached
 *     overrides the choice. */
enum { SN_SWEEP_AUTO = 0, SN_SWEEP_STENCIL = 1, SN_SWEEP_CACHED = 2 };

/* One lattice of the replica table (batched mode: many per handle). */
typedef struct sn_replica_desc {
    int X, Y, Z;           /* lattice size (reference keys X, Y, Z)        */
    float T;               /* temperature in Kelvin (reference key T)     */
    int has_efield;        /* 1: efield below replaces sn_params.efield    */
    float efield[3];
    uint64_t seed;         /* Philox key of this replica; 0 -> params.seed + replica */
    int block[3];          /* block shape to use (from sn_plan_candidates or a
                              tuner); 0,0,0 -> the planner's first choice     */
} sn_replica_desc;

/* The block/colour schedule chosen for one replica (what the CPU oracle
 * mirrors).  A site (x,y,z) belongs to block (x/bx, y/by, z/bz) of block
 * colour (block index mod m per axis) and to site colour (cx,cy,cz) =
 * (local coordinate mod s).  A sweep visits block colours (cbx,cby,cbz)
 * lexicographically; inside one it visits colour groups lexicographically
 * by their representative (cx,cy,cz).  Without merging a group is one site
 * colour.  With merge = 1 the representatives have cx < s/2 and a group is
 * the pair c, c + (s/2,s/2,s/2) mod s: sites of the two colours are at least
 * s/2 apart along every axis, farther than the cutoff, so they are updated
 * together.  Sites updated together never interact, so the order inside a
 * group does not matter. */
typedef struct sn_schedule_info {
    int bx, by, bz;        /* block dimensions                          */
    int nbx, nby, nbz;     /* blocks per axis                           */
    int mx, my, mz;        /* block colours per axis                    */
    int s;                 /* site-colour stride = cutoff + 1           */
    int halo;              /* halo width = cutoff (0 along z in 2D)     */
    int tile_slots;        /* shared-memory slots per tile (padded)     */
    int smem_bytes;        /* dynamic shared memory per block           */
    int merge;             /* 1: colour pairs c, c + (s/2,s/2,s/2)      */
    int threads;           /* threads per block of the sweep kernel     */
    int field_cache;       /* 1: the cached-field sweep (SN_SWEEP_CACHED) */
} sn_schedule_info;

/* Initial lattice patterns (InitialLattice, src/starrynight-main.c:184-203). */
enum {
    SN_LATTICE_RANDOM = 0,        /* uniform on the sphere, then solid solution   */
    SN_LATTICE_FERROELECTRIC = 1  /* all along +x, then solid solution            */
};

/* Energy precision for sn_gpu_energy / sn_gpu_recompute. */
enum {
    SN_ENERGY_FP32 = 0,   /* FP32 local fields, FP64 site products and sums  */
    SN_ENERGY_FP64 = 1    /* every operation in FP64                          */
};

typedef struct sn_handle sn_handle;

/* ---- lifecycle --------------------------------------------------------- */

/* Allocates the replica table in HBM, builds the neighbour offsets
 * (replaces gen_neighbour, src/starrynight-montecarlo-core.c:38-72) and the
 * per-replica schedule.  Lattices start as all-vacancy until
 * sn_gpu_init_lattice or sn_gpu_upload_lattice.  Replaces the setup part of
 * main(), src/starrynight-main.c:153-180. */
sn_status sn_gpu_init(const sn_params *params, int n_replicas, const sn_replica_desc *replicas,
                      sn_handle **out);
sn_status sn_gpu_destroy(sn_handle *h);
const char *sn_gpu_status_string(sn_status s);
const char *sn_gpu_last_error(const sn_handle *h);

/* ---- lattice ----------------------------------------------------------- */

/* Pattern + solid solution on the device from (seed, site) Philox draws.
 * Replaces initialise_lattice_random/_ferroelectric + solid_solution
 * (src/starrynight-lattice.c:25-47, :139-171); vacancies get the zero
 * vector.  seed 0 -> the replica's seed. */
sn_status sn_gpu_init_lattice(sn_handle *h, int replica, int pattern, uint64_t seed);

/* xyz: 3N floats interleaved; len: N floats or NULL (every site gets
 * Dipoles[0]).  Sites with len == 0 are stored as zero vectors.  Replaces
 * the host writes into lattice[x][y][z]. */
sn_status sn_gpu_upload_lattice(sn_handle *h, int replica, const float *xyz, const float *len);
/* xyz: 3N floats; len: N floats or NULL.  For the analysis writers that read
 * lattice[x][y][z] between megasteps (src/starrynight-main.c:51-103). */
sn_status sn_gpu_download_lattice(sn_handle *h, int replica, float *xyz, float *len);

/* ---- sweep --------------------------------------------------------------- */

/* n_sweeps Metropolis sweeps of every replica (each occupied site attempted
 * once per sweep), as CUDA-graph launches.  accept/reject (nullable) receive
 * the totals of this call over all replicas.  Replaces MC_moves(X*Y*Z*n)
 * (src/starrynight-montecarlo-core.c:143-191) and the ACCEPT/REJECT counters.
 * The call returns when its sweeps have finished on the GPU, with their own
 * status: SN_ERR_TIMEOUT when a block of the dataflow schedule gave up
 * waiting for a neighbour (sn_gpu_set_wait_limit).  The lattice is then not a
 * valid Metropolis state: upload or initialise it again before sweeping on
 * (the handle itself stays usable). */
sn_status sn_gpu_sweep(sn_handle *h, int n_sweeps, uint64_t *accept, uint64_t *reject);

/* Polls a block of the dataflow sweep spends on one neighbour's done flag
 * before it records SN_ERR_TIMEOUT and goes on (default 4194304 polls, about
 * 1-4 s; >= 1).  Every device-side wait is bounded by it, so a sweep launch
 * always ends.  The reference has no waits: it exit()s on its own errors
 * (src/starrynight-config.c:113-121). */
sn_status sn_gpu_set_wait_limit(sn_handle *h, uint32_t polls);

/* sn_gpu_sweep, then the lattice of every replica r with xyz[r] != NULL
 * written to xyz[r] (3 floats per site, as sn_gpu_download_lattice with a
 * NULL len); xyz has one entry per replica.  A buffer in pinned or
 * registered host memory (or device memory) is written by the last sweep
 * itself, each block's sites as soon as that block is final, so the
 * transfer overlaps the sweep; any other buffer is filled by the staged
 * download afterwards.  The same lattice either way.  Replaces MC_moves on
 * the host lattice followed by the read of lattice[x][y][z] by the output
 * routines (src/starrynight-main.c:222-227, :248). */
sn_status sn_gpu_sweep_download(sn_handle *h, int n_sweeps, float *const *xyz, uint64_t *accept, uint64_t *reject);

/* Page-locked host memory for the lattice buffers of the calls above, for C
 * hosts that do not include the CUDA headers: uploads and downloads from it
 * run at the full host-link rate and sn_gpu_sweep_download writes it from
 * the sweep itself.  NULL on failure; free with sn_gpu_host_free.  (The
 * reference allocates its lattice with malloc, src/starrynight-main.c:155-161.) */
void *sn_gpu_host_alloc(size_t bytes);
void sn_gpu_host_free(void *p);

/* Total sweeps done so far (the Philox sweep counter). */
sn_status sn_gpu_sweep_count(const sn_handle *h, uint64_t *sweeps);

/* Sets the sweep counter (what sn_gpu_sweep_count reports and what keys the
 * sweep's random stream) -- used to resume from a checkpoint so that the
 * continued run is the run that never stopped.  No reference counterpart. */
sn_status sn_gpu_set_sweep_count(sn_handle *h, uint64_t sweeps);

/* ---- energies and observables -------------------------------------------- */

/* Full recompute of one replica's energy (FP64 total).  site_E (nullable,
 * N doubles) receives the site energies e_i = p_i.(len_i h_i - C nn_i + E)
 * - K(|p_ix|+|p_iy|)[K>0], whose differences are site_energy()'s dE
 * (src/starrynight-montecarlo-core.c:76-141). */
sn_status sn_gpu_energy(sn_handle *h, int replica, int precision, double *E_total, double *site_E);

/* Per replica (arrays of n_replicas): E/site and |P|/site from the running
 * FP64 totals, P = sum_i len_i p_i (P_vec nullable, 3 per replica).  N is
 * X*Y*Z, as polarisation() divides (src/starrynight-analysis.c:48-62). */
sn_status sn_gpu_observables(sn_handle *h, double *E_per_site, double *P_abs, double *P_vec);

/* Per-sweep log of one replica since the last call: E/site and |P|/site
 * after each sweep.  *n_out = entries written (<= max). */
sn_status sn_gpu_history(sn_handle *h, int replica, int max, double *E_per_site, double *P_abs,
                         int *n_out);

/* Recompute every replica's energy, compare with the running total, and
 * restart the running total from the recompute.  *max_rel_drift (nullable)
 * = max over replicas of |E_running - E_recompute| / max(|E_recompute|, 1). */
sn_status sn_gpu_recompute(sn_handle *h, int precision, double *max_rel_drift);

/* Make sn_gpu_sweep recompute every `every` sweeps (0 = never) and keep the
 * largest relative drift seen; read it with sn_gpu_drift. */
sn_status sn_gpu_set_recompute(sn_handle *h, int every, int precision);
sn_status sn_gpu_drift(const sn_handle *h, double *max_rel_drift, int *n_checks);

/* ---- run control ---------------------------------------------------------- */

sn_status sn_gpu_set_field(sn_handle *h, int replica, const float efield[3]);
sn_status sn_gpu_set_temperature(sn_handle *h, int replica, float T);
sn_status sn_gpu_get_temperature(const sn_handle *h, int replica, float *T);

/* Replica exchange between adjacent temperatures every `every` sweeps
 * (0 = off); pairs alternate even/odd, swap accepted with probability
 * min(1, exp((beta_a - beta_b)(E_a - E_b))).  The reference runs independent
 * temperatures as separate processes (Makefile:48-62); this is the in-GPU
 * form of that batch. */
sn_status sn_gpu_set_exchange(sn_handle *h, int every);
sn_status sn_gpu_exchange_stats(sn_handle *h, uint64_t *attempted, uint64_t *accepted);

/* ---- differentiation ------------------------------------------------------- */

/* Adjoint of the total energy of one replica: dE_dp (nullable, 3N floats) =
 * dE/dp_i = len_i h_i - C nn_i + E - K(sgn p_ix, sgn p_iy, 0)[K>0] (zero at
 * vacancies); dE_dparams (nullable, 5 doubles) = dE/d(Dipole, CageStrain,
 * Ex, Ey, Ez) with dE/dDipole = 2 E_dd / Dipoles[0]; E_total nullable. */
sn_status sn_gpu_adjoint(sn_handle *h, int replica, float *dE_dp, double *dE_dparams, double *E_total);

/* T=0 projected-gradient descent on the sphere: n_steps of
 * p <- normalize(p - step (g - (g.p) p)) at every occupied site.  E_trace
 * (nullable, n_steps+1 doubles) receives E before and after each step. */
sn_status sn_gpu_quench(sn_handle *h, int replica, int n_steps, float step, double *E_trace);

/* ---- analysis on the resident lattice ------------------------------------
 * The per-site maps and order parameters of src/starrynight-analysis.c,
 * computed on the device; the caller's buffers are host memory.
 *
 * sn_gpu_potential: dipole_potential(x,y,z) (:65-94, called with MAX = 6 by
 *   every writer) for all N sites into pot[N], index (x*Y+y)*Z+z.  Bit-equal
 *   to the reference's value (same float terms, same double sum order).
 * sn_gpu_efield: |E| of dipole_electricfield(cutoff,x,y,z) (:393-450, cutoff 4
 *   in lattice_Efield_XYZ) or, with half_offset = 1, of
 *   dipole_electricfieldoffset (:310-380, cutoff 2 in
 *   lattice_Efieldoffset_XYZ) for all sites into magnitude[N]; bit-equal.
 * sn_gpu_radial_order: the histograms of radial_order_parameter (:528-598,
 *   cutoff 9): per bin b = |r|^2 in [0, cutoff^2], fe_sum[b] = sum over sites
 *   and offsets of p_i.p_j, afe_sum[b] = sum of p_i.p_j - 3(n.p_i)(n.p_j),
 *   count[b] = number of terms; arrays of cutoff^2+1 entries (any may be
 *   NULL).  Summed in FP64 (the reference sums in float).
 * sn_gpu_order_parameters: polarisation() (:48-62) = sum p_x / N and
 *   landau_order() (:506-526) = |sum p|^2, both unweighted by length, and the
 *   orientation sum itself (orientation_sum[3]); any output may be NULL.
 * Cutoffs are limited to 1..32.  Lattice sides shorter than the cutoff wrap
 * periodically (the reference indexes out of bounds there). */
sn_status sn_gpu_potential(sn_handle *h, int replica, int cutoff, double *pot);
sn_status sn_gpu_efield(sn_handle *h, int replica, int cutoff, int half_offset, double *magnitude);
sn_status sn_gpu_radial_order(sn_handle *h, int replica, int cutoff, double *fe_sum, double *afe_sum,
                              int64_t *count);
sn_status sn_gpu_order_parameters(sn_handle *h, int replica, double *polarisation_x, double *landau,
                                  double *orientation_sum);

/* ---- energy without device allocation -------------------------------------------
 * No counterpart in the reference, which has no library API at all.  For
 * callers that may not allocate device memory (a plugin whose host framework
 * owns the device memory pool, a process that has reserved nearly all device
 * memory for its lattices, a long run that must not risk an out-of-memory
 * failure between sweeps): the total energy of a lattice held in the
 * CALLER's device memory -- d_px, d_py, d_pz, d_len are device pointers to
 * N = X*Y*Z floats each, index (x*Y+y)*Z+z, vacancies as zero vectors of
 * length 0 -- computed like sn_gpu_energy(SN_ENERGY_FP32) without any device
 * allocation.  efield may be NULL (params->efield is used); *E_total is a
 * host double; stream is a cudaStream_t or NULL (the default stream), and the
 * call returns after the result is on the host.
 * All scratch lives in one fixed device array inside the library (about
 * 1 MiB, on every GPU that loads it, until exit): the lattice may split into
 * at most 65536 tiles (512^3 at cutoff 3 needs 32768); larger lattices are
 * rejected with SN_ERR_ARG.  Every call reuses that array, so calls whose GPU
 * work overlaps race and return wrong energies: keep them ordered on one
 * stream.  The first call on each device looks up the array's device
 * address (with that device current) and should come before any stream
 * capture begins. */
sn_status sn_gpu_energy_noalloc(const float *d_px, const float *d_py, const float *d_pz, const float *d_len,
                                int X, int Y, int Z, const sn_params *params, const float *efield,
                                double *E_total, void *stream);

/* ---- random streams ---------------------------------------------------------- */

/* Philox4x32-10 of n (counter, key) pairs on the device: ctr 4n words,
 * key 2n words, out 4n words (host buffers).  The stream behind every
 * proposal, for checking against a CPU restatement. */
sn_status sn_gpu_philox(const uint32_t *ctr, const uint32_t *key, uint32_t *out, int n);
/* The proposals the sweep draws in one replica for sites[i] at sweep index
 * `sweep`: out4[4i..4i+3] = (p'x, p'y, p'z, u); NaN p' when every Marsaglia
 * try was rejected (the move then keeps the old dipole). */
sn_status sn_gpu_proposals(const sn_handle *h, int replica, const uint32_t *sites, int n, uint32_t sweep,
                           float *out4);

/* ---- introspection ---------------------------------------------------------- */

sn_status sn_gpu_schedule(const sn_handle *h, int replica, sn_schedule_info *out);
/* Host-only: the schedule sn_gpu_init would pick (no GPU needed). */
sn_status sn_plan_schedule(int X, int Y, int Z, int cutoff, int mixed_lengths, sn_schedule_info *out);
/* Host-only: up to max_out feasible schedules in the planner's order of
 * preference (the first is sn_plan_schedule's); *n_out receives the count.
 * An autotuner times them and passes the winner's block shape in
 * sn_replica_desc.block. */
sn_status sn_plan_candidates(int X, int Y, int Z, int cutoff, int mixed_lengths, sn_schedule_info *out,
                             int max_out, int *n_out);
/* The empirical autotuner: times the first max_candidates of
 * sn_plan_candidates for this replica's lattice size (one temporary handle
 * each, a random lattice at the replica's temperature and field, 2 warm-up
 * sweeps, then `sweeps` sweeps timed with CUDA events) and writes the
 * fastest shape to block[3] and its time to *ms_per_sweep (nullable).  Put
 * block into sn_replica_desc.block; every shape gives an exact sweep, the
 * choice only changes speed and the order of the moves. */
sn_status sn_gpu_autotune(const sn_params *params, const sn_replica_desc *replica, int max_candidates, int sweeps,
                          int block[3], double *ms_per_sweep);
/* Host-only: 1 if no two sites updated together interact under periodic
 * boundaries (same block colour and site colour within the cutoff). */
int sn_check_schedule(int X, int Y, int Z, int cutoff, const sn_schedule_info *sched);
/* Host-only check of the dataflow schedule of a replica table (no GPU
 * needed): plans every replica's blocks as sn_gpu_init would and verifies,
 * independently of how the lists were built, that every block appears once
 * and waits exactly on its periodically adjacent blocks of earlier colour,
 * all earlier in the list (so the persistent sweep cannot deadlock).
 * stats (nullable, 3 entries): blocks, dependencies, largest dependency
 * count.  No reference counterpart. */
sn_status sn_check_flow(const sn_params *params, int n_replicas, const sn_replica_desc *replicas, uint64_t *stats);
/* Kernel launches issued by this handle so far. */
sn_status sn_gpu_launch_count(const sn_handle *h, uint64_t *launches);
/* The handle's CUDA stream as an opaque pointer (for event timing). */
void *sn_gpu_stream(const sn_handle *h);
/* Runs n_sweeps sweeps WITHOUT the graph, timing every block-colour launch
 * of the sweep kernel with CUDA events on the handle's stream:
 * *avg_launch_ms = mean duration of one launch, *avg_sweep_ms = mean sweep.
 * The sweeps are real (they advance the lattice and the sweep counter). */
/* Dataflow schedule statistics since the last call: stats[0] = 1 when the
 * sweep runs as one dataflow launch per kernel variant (0: one launch per
 * block colour), stats[1] = its resident grid (3D variant), stats[2] = blocks
 * that had to wait for a neighbour, stats[3] = polls spent waiting.
 * Measurement hook; no reference counterpart. */
sn_status sn_gpu_flow_stats(sn_handle *h, uint64_t *stats);
sn_status sn_gpu_phase_times(sn_handle *h, int n_sweeps, double *avg_launch_ms, double *avg_sweep_ms,
                             int *launches_per_sweep);
/* sn_gpu_sweep(h, n_sweeps, NULL, NULL) with *ms = the device time of those
 * sweeps (CUDA events on the handle's stream around the graph launches and
 * any periodic recompute, taken before the call's status read).
 * Measurement hook; no reference counterpart. */
sn_status sn_gpu_sweep_timed(sn_handle *h, int n_sweeps, double *ms);
/* Checks the field cache of a replica that uses the cached-field sweep: the
 * cache as the sweeps maintained it is compared with a fresh field-cache pass
 * over the current lattice; *mismatches = differing int32 entries (0 when
 * the incremental updates are exact, as designed).  The cache holds the
 * fresh values afterwards.  SN_ERR_UNSUPPORTED for a stencil-sweep replica.
 * Test and self-check hook; no reference counterpart. */
sn_status sn_gpu_field_cache_check(sn_handle *h, int replica, uint64_t *mismatches);
/* Test hook for the bounded waits: makes dataflow item `item` of the 3D
 * variant wait, in every later sweep, on a flag that no block ever publishes
 * (so that wait runs out and the sweep reports SN_ERR_TIMEOUT); item = -1
 * restores the planned dependency list.  Nothing faults or hangs: the wait
 * gives up after the limit of sn_gpu_set_wait_limit.  No reference
 * counterpart. */
sn_status sn_gpu_test_stall_block(sn_handle *h, int item);
/* Measured FP32 FMA throughput of the current device (TFLOP/s, an FMA
 * counted as 2) and its nominal maximum SM clock; the roofline denominator
 * for the sweep kernel, which runs on CUDA cores. */
sn_status sn_gpu_fp32_peak(double *tflops, double *sm_clock_mhz);
/* Number of neighbour offsets (gen_neighbour's count) for a cutoff. */
int sn_neighbour_count(int cutoff, int Z);

#ifdef __cplusplus
}
#endif

#endif
