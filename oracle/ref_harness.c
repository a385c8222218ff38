/*
 * ref_harness.c -- drives the UNMODIFIED reference sources as a library.
 * TEST INFRASTRUCTURE ONLY: built by oracle/Makefile into oracle/_ref/ from
 * the reference tree (REF=<path to StarryNight>), never shipped.
 *
 * The reference is one translation unit (src/starrynight-main.c:18-26
 * #includes the other files).  This harness includes the same files in the
 * same order, minus starrynight-main.c, and replaces main() with small
 * entry points that set the globals main() would set
 * (src/starrynight-main.c:137-215) and call the reference's own
 * gen_neighbour / initialise_lattice_random / solid_solution / MC_moves /
 * site_energy.  It is used to generate golden vectors that pin the CPU
 * oracle (sn_oracle.c) to the reference bit for bit.
 */
#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "libconfig.h"

#include "mt19937ar-cok.c"

static int rand_int(int SPAN);

#include "starrynight-config.c"
#include "starrynight-lattice.c"
#include "starrynight-analysis.c"
#include "starrynight-montecarlo-core.c"

#define EXPORT __attribute__((visibility("default")))

static int quiet_fd = -1;

static void mute(void)
{
    fflush(stderr);
    quiet_fd = dup(2);
    if (freopen("/dev/null", "w", stderr) == NULL) quiet_fd = -1;
}

static void unmute(void)
{
    if (quiet_fd >= 0) {
        fflush(stderr);
        dup2(quiet_fd, 2);
        close(quiet_fd);
        quiet_fd = -1;
    }
}

static void free_lattice(void)
{
    int x, y;
    if (!lattice) return;
    for (x = 0; x < X; x++) {
        for (y = 0; y < Y; y++) free(lattice[x][y]);
        free(lattice[x]);
    }
    free(lattice);
    lattice = NULL;
}

/* Sets the globals that load_config()/main() would set, allocates the
 * lattice as main() does (:155-161), seeds MT (:172-176), builds the
 * neighbour list and the random + solid-solution initial lattice. */
EXPORT int refh_setup(int X_, int Y_, int Z_, int cutoff, double cage, double K_, const float *E,
                      int constrain, int T_, int n_species, const float *lens, const float *prevs,
                      unsigned int seed)
{
    int x, y, i;
    free_lattice();
    X = X_;
    Y = Y_;
    Z = Z_;
    DipoleCutOff = cutoff;
    CageStrain = cage;
    K = K_;
    Efield.x = E[0];
    Efield.y = E[1];
    Efield.z = E[2];
    ConstrainToX = constrain;
    T = T_;
    if (n_species > 10) return -1;
    dipolecount = n_species;
    for (i = 0; i < 10; i++) {
        dipoles[i].length = i < n_species ? lens[i] : 0.0f;
        dipoles[i].prevalence = i < n_species ? prevs[i] : 0.0f;
    }
    lattice = (struct dipole ***)malloc(sizeof(struct dipole **) * X);
    for (x = 0; x < X; x++) {
        lattice[x] = (struct dipole **)malloc(sizeof(struct dipole *) * Y);
        for (y = 0; y < Y; y++) lattice[x][y] = (struct dipole *)malloc(sizeof(struct dipole) * Z);
    }
    init_genrand(seed);
    mute();
    neighbour = 0;
    gen_neighbour();
    initialise_lattice_random();
    solid_solution();
    unmute();
    beta = 1 / ((float)T / 300.0);
    ACCEPT = 0;
    REJECT = 0;
    return neighbour;
}

EXPORT void refh_get_lattice(float *out4)
{
    int x, y, z;
    for (x = 0; x < X; x++)
        for (y = 0; y < Y; y++)
            for (z = 0; z < Z; z++) {
                struct dipole *d = &lattice[x][y][z];
                float *o = &out4[4 * (((long)x * Y + y) * Z + z)];
                o[0] = d->x;
                o[1] = d->y;
                o[2] = d->z;
                o[3] = d->length;
            }
}

EXPORT void refh_set_lattice(const float *in4)
{
    int x, y, z;
    for (x = 0; x < X; x++)
        for (y = 0; y < Y; y++)
            for (z = 0; z < Z; z++) {
                struct dipole *d = &lattice[x][y][z];
                const float *o = &in4[4 * (((long)x * Y + y) * Z + z)];
                d->x = o[0];
                d->y = o[1];
                d->z = o[2];
                d->length = o[3];
            }
}

/* MC_moves takes an int (src/starrynight-montecarlo-core.c:143); chunk. */
EXPORT void refh_mc_moves(long long n)
{
    while (n > 0) {
        int chunk = n > INT_MAX ? INT_MAX : (int)n;
        MC_moves(chunk);
        n -= chunk;
    }
}

EXPORT void refh_counts(unsigned long long *acc, unsigned long long *rej)
{
    *acc = ACCEPT;
    *rej = REJECT;
}

EXPORT double refh_beta(void) { return beta; }

EXPORT double refh_site_energy(int x, int y, int z, const float *nw)
{
    struct dipole d;
    d.x = nw[0];
    d.y = nw[1];
    d.z = nw[2];
    d.length = lattice[x][y][z].length;
    return site_energy(x, y, z, &d, &lattice[x][y][z]);
}

EXPORT int refh_neighbours(int *dxyz, float *d, int max)
{
    int i;
    for (i = 0; i < neighbour && i < max; i++) {
        dxyz[3 * i + 0] = neighbours[i].dx;
        dxyz[3 * i + 1] = neighbours[i].dy;
        dxyz[3 * i + 2] = neighbours[i].dz;
        d[i] = neighbours[i].d;
    }
    return neighbour;
}

/* The reference's own observables on the current lattice:
 * polarisation() (src/starrynight-analysis.c:48-62) and landau_order()
 * (:506-526). */
EXPORT void refh_observables(double *pol_x, double *landau)
{
    *pol_x = polarisation();
    *landau = landau_order();
}

EXPORT unsigned int refh_mt_next(void) { return (unsigned int)genrand_int32(); }
