/*
 * sn_oracle.h -- CPU oracle for the StarryNight Metropolis dipole-lattice
 * sweep.  TEST INFRASTRUCTURE ONLY: this library is the checker for the CUDA
 * path and the CPU baseline in bench.py.  Nothing in the product links,
 * loads or calls it.
 *
 * Contents (each function cites the reference code it restates; paths are
 * relative to the StarryNight source tree):
 *   - MT19937 (Matsumoto & Nishimura 1998), the generator the reference
 *     vendors in src/mt19937ar-cok.c (init_genrand :63, genrand_int32 :130,
 *     genrand_real1 :164, genrand_real2 :182).
 *   - Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11, "Parallel random
 *     numbers: as easy as 1, 2, 3"), the counter-based stream of the GPU path.
 *   - gen_neighbour (src/starrynight-montecarlo-core.c:38-72).
 *   - A reference-faithful random-sequential engine: site_energy
 *     (src/starrynight-montecarlo-core.c:76-141), MC_move / MC_moves (:143-191),
 *     random_sphere_point / random_X_point (src/starrynight-config.c:203-263),
 *     initialise_lattice_random + solid_solution (src/starrynight-lattice.c:25-37,
 *     139-171).  Same float/double mix and the same RNG call order, so it
 *     reproduces the reference binary's trajectory bit for bit.
 *   - The Philox colour-sweep mirror of the GPU schedule (oracle a), with the
 *     energy change evaluated in FP64 (oracle b).
 *   - FP64 site energies, total energy, local field and parameter gradients.
 *
 * Build with -ffp-contract=off so that x86-64 and aarch64 hosts give the same
 * bits (the reference is compiled without FMA contraction on x86-64).
 */
#ifndef SN_ORACLE_H
#define SN_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- MT19937 ---------------- */
typedef struct {
    uint32_t mt[624];
    int32_t mti; /* index of the next word; 624 => regenerate before use */
} sno_mt;

void sno_mt_seed(sno_mt *g, uint32_t seed);
uint32_t sno_mt_u32(sno_mt *g);
double sno_mt_real1(sno_mt *g); /* [0,1]  y/(2^32-1) */
double sno_mt_real2(sno_mt *g); /* [0,1)  y/2^32     */

/* ---------------- Philox4x32-10 ---------------- */
void sno_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* ---------------- neighbour table ---------------- */
/* Offsets (dx,dy,dz) with 0 < |r| <= cutoff in the reference's loop order;
 * 2D (dz == 0 only) when Z == 1.  Returns the count, or -1 if max is too small. */
int sno_gen_neighbours(int cutoff, int Z, int *dx, int *dy, int *dz, float *d, int max);

/* ---------------- model ---------------- */
typedef struct {
    int X, Y, Z;
    int cutoff;          /* DipoleCutOff */
    int dim;             /* 3: sphere proposals; 2: circle proposals (DIM<3) */
    int constrain_to_x;  /* ConstrainToX */
    double beta;         /* 1/kT in units of k_B*300 K */
    float efield[3];
    double K;
    double cage_strain;
} sno_model;

/* ---------------- reference-faithful random-sequential engine ----------------
 * Lattice: AoS float4 (x, y, z, length) per site, index (x*Y + y)*Z + z,
 * exactly the reference's struct dipole. */
void sno_ref_init_random(const sno_model *m, float *lat4, sno_mt *g,
                         int n_species, const float *lengths, const float *prevalence);
double sno_ref_site_energy(const sno_model *m, const float *lat4, int x, int y, int z,
                           const float newd[4], const float oldd[4]);
/* Runs `moves` MC_move() calls; adds to accept/reject. */
void sno_ref_mc_moves(const sno_model *m, float *lat4, sno_mt *g, long long moves,
                      uint64_t *accept, uint64_t *reject);

/* ---------------- GPU-schedule mirror (oracle a) ---------------- */
typedef struct {
    int bx, by, bz;      /* block dims */
    int nbx, nby, nbz;   /* blocks per axis */
    int mx, my, mz;      /* block colours per axis */
    int s;               /* site-colour stride (cutoff + 1) */
    int merge;           /* 1: colours c and c + (s/2,s/2,s/2) form one group */
} sno_schedule;

typedef struct {
    uint64_t seed;       /* Philox key */
    float beta;          /* beta as the GPU holds it */
    float length;        /* uniform dipole length (0 = per-site lengths used) */
} sno_stream;

/* One sweep in the GPU's block-colour / site-colour order.  px/py/pz/len are
 * SoA site arrays (index (x*Y+y)*Z+z), updated in place.
 *   gpu_after (nullable, 3 arrays packed [px|py|pz] of the GPU's state after
 *     this sweep): when the oracle's decision differs from the GPU's at a site
 *     whose margin is inside `tol`, the GPU's decision is adopted (borderline);
 *     a difference outside the band is counted as hard and also adopted so the
 *     comparison can continue.
 *   margin_out (nullable, N doubles): dE64 - (-ln u)/beta per site (NaN for
 *     vacancies); accept_out (nullable, N bytes).
 * Returns the number of accepted moves. */
uint64_t sno_colour_sweep(const sno_model *m, const sno_schedule *sc, const sno_stream *st,
                          uint32_t sweep, float *px, float *py, float *pz, const float *len,
                          const float *gpu_after, double tol,
                          uint64_t *n_borderline, uint64_t *n_hard,
                          double *dE_sum, double *margin_out, uint8_t *accept_out);

/* The FP32 proposal the GPU draws for (site, sweep): writes p[3]; returns the
 * uniform used by the accept test in *u. */
void sno_proposal(const sno_model *m, const sno_stream *st, uint32_t site, uint32_t sweep,
                  float p[3], float *u);

/* ---------------- FP64 energies and gradients (oracle b, adjoint) ----------------
 * site energy e_i = p_i . (len_i h_i - C nn_i + E) - K(|p_ix| + |p_iy|)[K>0]
 * with h_i = sum_j len_j (p_j - 3 n (n.p_j)) / d^3 over the cutoff sphere and
 * nn_i = sum over the six unit offsets of p_j.  Total
 * E = sum_i [ 1/2 p_i.(len_i h_i - C nn_i) + p_i.E - K(|p_ix|+|p_iy|)[K>0] ].
 * Any output pointer may be NULL.
 *   site_e: N doubles; grad: 3N doubles (dE/dp_i); dparams[5]: dE/d(Dipole,
 *   CageStrain, Ex, Ey, Ez) with dE/dDipole = 2 E_dd / dipole. */
double sno_energy64(const sno_model *m, const float *px, const float *py, const float *pz,
                    const float *len, double dipole, double *site_e, double *grad,
                    double *dparams, double *E_dd_out);

/* dE for replacing site i's dipole by newp, in FP64. */
double sno_delta_energy64(const sno_model *m, const float *px, const float *py, const float *pz,
                          const float *len, int site, const float newp[3]);

#ifdef __cplusplus
}
#endif

#endif

/* ---- analysis (src/starrynight-analysis.c) ----------------------------------
 * SoA lattice, index (x*Y+y)*Z+z.  Each follows the reference function it names
 * statement by statement in float/double as the reference types them, so the
 * per-site maps equal the reference's bit for bit; the histogram sums are
 * FP64 (the reference's are float). */
void sno_potential_map(const float *px, const float *py, const float *pz, const float *len, int X, int Y, int Z,
                       int cutoff, double *out);
void sno_efield_map(const float *px, const float *py, const float *pz, int X, int Y, int Z, int cutoff, int half,
                    double *out);
void sno_radial_order(const float *px, const float *py, const float *pz, int X, int Y, int Z, int cutoff,
                      int float_sums, double *fe, double *afe, long long *count);
void sno_order_params(const float *px, const float *py, const float *pz, long long n, double *pol_x,
                      double *landau, double *sum3);
