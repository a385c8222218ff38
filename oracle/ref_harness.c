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

/* ---- analysis entry points: the reference's own functions on the current
 * lattice (src/starrynight-analysis.c). ---- */

/* Orientation patterns of src/starrynight-lattice.c:39-137 by InitialLattice
 * name (what main() selects, src/starrynight-main.c:180-200); lengths untouched. */
EXPORT int refh_init_pattern(const char *name)
{
    if (!strcmp(name, "random")) initialise_lattice_random();
    else if (!strcmp(name, "ferroelectric")) initialise_lattice_ferroelectric();
    else if (!strcmp(name, "buckled")) initialise_lattice_buckled();
    else if (!strcmp(name, "antiferro_wall")) initialise_lattice_antiferro_wall();
    else if (!strcmp(name, "ferro_wall")) initialise_lattice_ferro_wall();
    else if (!strcmp(name, "antiferro_slip")) initialise_lattice_antiferro_slip();
    else if (!strcmp(name, "spectrum")) initialise_lattice_spectrum();
    else if (!strcmp(name, "slab_delete")) initialise_lattice_slab_delete();
    else return -1;
    return 0;
}

/* dipole_potential (:65-94) at every site, index (x*Y+y)*Z+z */
EXPORT void refh_potential_map(double *out)
{
    int x, y, z;
    for (x = 0; x < X; x++)
        for (y = 0; y < Y; y++)
            for (z = 0; z < Z; z++) out[((long)x * Y + y) * Z + z] = dipole_potential(x, y, z);
}

/* |E| of dipole_electricfield (:393-450) or, half = 1, of
 * dipole_electricfieldoffset (:310-380; its per-term stderr trace muted) */
EXPORT void refh_efield_map(int cutoff, int half, double *out)
{
    int x, y, z;
    if (half) mute();
    for (x = 0; x < X; x++)
        for (y = 0; y < Y; y++)
            for (z = 0; z < Z; z++)
                out[((long)x * Y + y) * Z + z] =
                    half ? dipole_electricfieldoffset(cutoff, x, y, z) : dipole_electricfield(cutoff, x, y, z);
    if (half) unmute();
}

/* The reference's writers, by name, on the current lattice. */
EXPORT int refh_write(const char *kind, const char *path)
{
    char buf[512];
    snprintf(buf, sizeof(buf), "%s", path);
    if (!strcmp(kind, "potential_xyz")) lattice_potential_XYZ(buf);
    else if (!strcmp(kind, "potential_cube")) lattice_potential_cube(buf);
    else if (!strcmp(kind, "efield_xyz")) lattice_Efield_XYZ(buf);
    else if (!strcmp(kind, "efieldoffset_xyz")) {
        mute();
        lattice_Efieldoffset_XYZ(buf);
        unmute();
    } else if (!strcmp(kind, "potential_pgm")) outputpotential_png(buf);
    else if (!strcmp(kind, "dipoles_xyz")) outputlattice_xyz(buf);
    else if (!strcmp(kind, "dipoles_ppm")) outputlattice_ppm_hsv(buf);
    else if (!strcmp(kind, "dipoles_svg")) outputlattice_svg(buf);
    else if (!strcmp(kind, "rdf")) radial_order_parameter(buf);
    else if (!strcmp(kind, "recombination")) {
        FILE *fo = fopen(buf, "w");
        if (!fo) return -2;
        mute();
        recombination_calculator(fo);
        unmute();
        fclose(fo);
    } else return -1;
    fflush(NULL); /* outputlattice_xyz leaves its file open */
    return 0;
}

/* stderr output of outputlattice_dumb_terminal (:820-925) or of
 * recombination_calculator(stderr) (:97-230, as analysis_initial calls it)
 * captured into a file */
EXPORT int refh_capture(const char *kind, const char *path)
{
    int saved, rc = 0;
    fflush(stderr);
    saved = dup(2);
    if (saved < 0 || freopen(path, "w", stderr) == NULL) return -2;
    if (!strcmp(kind, "dumb_terminal")) outputlattice_dumb_terminal();
    else if (!strcmp(kind, "recombination")) recombination_calculator(stderr);
    else rc = -1;
    fflush(stderr);
    dup2(saved, 2);
    close(saved);
    return rc;
}
