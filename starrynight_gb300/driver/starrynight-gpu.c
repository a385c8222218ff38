/*
 * starrynight-gpu.c -- host driver: the reference program's main loop
 * (src/starrynight-main.c:125-277) on top of the GB300 C ABI.
 *
 * Reads ./starrynight.cfg with the same keys and lookup rules as
 * load_config() (src/starrynight-config.c:98-182) through the project's
 * libconfig-subset reader, honours the same command-line overrides
 * (argv[1] = T, argv[2] = CageStrain, src/starrynight-main.c:142-151), builds
 * the initial lattice named by InitialLattice, then runs MCEqmSteps
 * equilibration megasteps and MCMegaSteps production megasteps of MCMoves
 * sweeps each (MCMinorSteps = X*Y*Z*MCMoves single-site moves in the
 * reference, src/starrynight-config.c:166).
 *
 * Output: stderr carries the reference's progress lines, including
 * "MC Moves (per second): %f MHz" per megastep (src/starrynight-main.c:255)
 * and the final ACCEPT/REJECT line (:273); stdout carries one line of
 * observables per megastep: megastep, sweeps, E/site, |P|/site, P_x, P_y,
 * P_z.  The analysis flags (DisplayDumbTerminal, CalculateRecombination,
 * CalculateRadialOrderParameter, CalculatePotential, CalculateEfield,
 * SaveDipolesXYZ/PNG/SVG, SavePotentialCube) write the same files at the same
 * points as analysis_initial / analysis_midpoint and the post-equilibration
 * block (src/starrynight-main.c:29-103, :225-231), from maps computed on the
 * GPU (sn_gpu_potential, sn_gpu_efield, sn_gpu_radial_order) and written by
 * libsn_io; the recombination log is Recombination_T_%04d.log (:164-168).
 *
 * Additional keys: Dipole (single species length) and DipoleFraction
 * (occupancy p: Dipoles = [Dipole, 0], Prevalence = [p, 1-p]), Seed
 * (Philox key; default 0xDEADBEEF + T as the reference seeds MT,
 * src/starrynight-main.c:172), ResumeFrom (a checkpoint file that replaces
 * InitialLattice and restores the sweep counter), CheckpointFile and
 * CheckpointEvery (write a checkpoint every that many production
 * megasteps, and at the end), AutoTune (time that many of the planner's
 * block shapes with sn_gpu_autotune and run with the fastest; 0 = the
 * planner's choice).  Options: --config FILE, --seed N,
 * --print-config (parse, print, exit without touching the GPU).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "libconfig.h"
#include "sn_gpu.h"
#include "sn_io.h"

typedef struct {
    double T;
    int X, Y, Z;
    float efield[3];
    double K, cage_strain;
    int n_species;
    float dipoles[SN_MAX_SPECIES], prevalence[SN_MAX_SPECIES];
    int constrain_to_x;
    int cutoff;
    char initial[64];
    int eqm_steps, mega_steps;
    double mc_moves;
    int save_xyz, save_png, save_svg, save_cube;
    int dumb_terminal, recombination, radial, potential, calc_efield;
    int has_seed;
    unsigned long long seed;
    char resume[256], checkpoint[256];
    int checkpoint_every;
    int autotune;
} cfg_t;

/* Defaults of src/starrynight-config.c:12-93 (the reference leaves T and
 * the Dipoles list to the file). */
static void cfg_defaults(cfg_t *c)
{
    memset(c, 0, sizeof(*c));
    c->T = 300.0;
    c->X = c->Y = c->Z = 20;
    c->K = 1.0;
    c->cage_strain = 1.0;
    c->n_species = 1;
    c->dipoles[0] = 1.0f;
    c->prevalence[0] = 1.0f;
    c->cutoff = 3;
    strcpy(c->initial, "random");
    c->mega_steps = 400;
    c->eqm_steps = 10;
    c->mc_moves = 1.0;
    c->dumb_terminal = 1;   /* src/starrynight-config.c:81-82 */
    c->recombination = 1;
}

static int cfg_load(const char *path, cfg_t *c)
{
    config_t cf;
    const config_setting_t *st;
    double tmp;
    int itmp, i, n;
    const char *str;
    config_init(&cf);
    if (!config_read_file(&cf, path)) {
        fprintf(stderr, "%s:%d - %s\n", config_error_file(&cf), config_error_line(&cf), config_error_text(&cf));
        config_destroy(&cf);
        return 0;
    }
    if (config_lookup_int(&cf, "T", &itmp)) c->T = itmp;
    else if (config_lookup_float(&cf, "T", &tmp)) c->T = tmp;
    config_lookup_int(&cf, "X", &c->X);
    config_lookup_int(&cf, "Y", &c->Y);
    config_lookup_int(&cf, "Z", &c->Z);
    if (config_lookup_float(&cf, "Efield.x", &tmp)) c->efield[0] = (float)tmp;
    if (config_lookup_float(&cf, "Efield.y", &tmp)) c->efield[1] = (float)tmp;
    if (config_lookup_float(&cf, "Efield.z", &tmp)) c->efield[2] = (float)tmp;
    config_lookup_float(&cf, "K", &c->K);
    config_lookup_float(&cf, "CageStrain", &c->cage_strain);
    st = config_lookup(&cf, "Dipoles");
    if (st && (n = config_setting_length(st)) > 0) {
        if (n > SN_MAX_SPECIES) n = SN_MAX_SPECIES;
        c->n_species = n;
        for (i = 0; i < n; i++) c->dipoles[i] = (float)config_setting_get_float_elem(st, i);
        st = config_lookup(&cf, "Prevalence");
        for (i = 0; i < n; i++) c->prevalence[i] = st ? (float)config_setting_get_float_elem(st, i) : 0.0f;
    }
    /* single-species spelling: Dipole = D, DipoleFraction = p */
    if (config_lookup_float(&cf, "Dipole", &tmp)) {
        c->n_species = 1;
        c->dipoles[0] = (float)tmp;
        c->prevalence[0] = 1.0f;
    }
    if (config_lookup_float(&cf, "DipoleFraction", &tmp)) {
        c->n_species = 2;
        c->dipoles[1] = 0.0f;
        c->prevalence[0] = (float)tmp;
        c->prevalence[1] = (float)(1.0 - tmp);
    }
    config_lookup_bool(&cf, "ConstrainToX", &c->constrain_to_x);
    config_lookup_int(&cf, "DipoleCutOff", &c->cutoff);
    if (config_lookup_string(&cf, "InitialLattice", &str)) snprintf(c->initial, sizeof(c->initial), "%s", str);
    config_lookup_int(&cf, "MCEqmSteps", &c->eqm_steps);
    config_lookup_int(&cf, "MCMegaSteps", &c->mega_steps);
    config_lookup_float(&cf, "MCMoves", &c->mc_moves);
    config_lookup_bool(&cf, "DisplayDumbTerminal", &c->dumb_terminal);
    config_lookup_bool(&cf, "CalculateRecombination", &c->recombination);
    config_lookup_bool(&cf, "CalculateRadialOrderParameter", &c->radial);
    config_lookup_bool(&cf, "CalculatePotential", &c->potential);
    config_lookup_bool(&cf, "CalculateEfield", &c->calc_efield);
    config_lookup_bool(&cf, "SaveDipolesSVG", &c->save_svg);
    config_lookup_bool(&cf, "SaveDipolesPNG", &c->save_png);
    config_lookup_bool(&cf, "SaveDipolesXYZ", &c->save_xyz);
    config_lookup_bool(&cf, "SavePotentialCube", &c->save_cube);
    if (config_lookup_string(&cf, "ResumeFrom", &str)) snprintf(c->resume, sizeof(c->resume), "%s", str);
    if (config_lookup_string(&cf, "CheckpointFile", &str)) snprintf(c->checkpoint, sizeof(c->checkpoint), "%s", str);
    config_lookup_int(&cf, "CheckpointEvery", &c->checkpoint_every);
    config_lookup_int(&cf, "AutoTune", &c->autotune);
    {
        long long s;
        if (config_lookup_int64(&cf, "Seed", &s)) {
            c->seed = (unsigned long long)s;
            c->has_seed = 1;
        }
    }
    config_destroy(&cf);
    return 1;
}

/* Orientation patterns of src/starrynight-lattice.c:39-137 (the random
 * pattern is drawn on the device).  Index (x*Y+y)*Z+z. */
static void pattern(const cfg_t *c, float *xyz)
{
    const int X = c->X, Y = c->Y, Z = c->Z;
    int x, y, z;
    for (x = 0; x < X; x++)
        for (y = 0; y < Y; y++)
            for (z = 0; z < Z; z++) {
                float *p = &xyz[3 * (((size_t)x * Y + y) * Z + z)];
                float px = 0.0f, py = 0.0f, pz = 0.0f;
                if (!strcmp(c->initial, "ferroelectric")) {
                    px = 1.0f;
                } else if (!strcmp(c->initial, "buckled")) {
                    px = (float)(x % 2);
                    py = (float)(y % 2);
                    pz = (float)(z % 2);
                } else if (!strcmp(c->initial, "antiferro_wall")) {
                    if ((y < Y / 2) ^ (x > X / 2)) px = (float)(2. * ((z + y) % 2) - 1.0);
                    else py = (float)(2. * ((x + z) % 2) - 1.0);
                } else if (!strcmp(c->initial, "ferro_wall")) {
                    py = x < X / 2 ? -1.0f : 1.0f;
                } else if (!strcmp(c->initial, "antiferro_slip")) {
                    px = x < X / 2 ? (float)(2. * ((z + y) % 2) - 1.0) : (float)(2. * ((z + y + 1) % 2) - 1.0);
                } else if (!strcmp(c->initial, "spectrum")) {
                    const float angle = (float)(2 * M_PI * (x * X + y) / ((float)X * Y));
                    px = (float)sin(angle);
                    py = (float)cos(angle);
                }
                p[0] = px;
                p[1] = py;
                p[2] = pz;
            }
}

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* ---- analysis points (src/starrynight-main.c:29-103): lattice and maps are
 * fetched from the GPU once per point and shared by the writers ---- */
typedef struct {
    sn_handle *h;
    const cfg_t *c;
    size_t N;
    float *xyz, *len;
    double *pot, *map;
    int have_lattice, have_pot;
    float dmax;
    FILE *log;
    int pinned; /* xyz and len from sn_gpu_host_alloc */
} ana_t;

static int ana_fail(ana_t *a, const char *what, sn_status s)
{
    fprintf(stderr, "%s failed: %s (%s)\n", what, sn_gpu_status_string(s), sn_gpu_last_error(a->h));
    return -1;
}

static int ana_lattice(ana_t *a)
{
    sn_status s;
    if (a->have_lattice) return 0;
    if ((s = sn_gpu_download_lattice(a->h, 0, a->xyz, a->len)) != SN_OK) return ana_fail(a, "download", s);
    a->have_lattice = 1;
    return 0;
}

static int ana_potential(ana_t *a)
{
    sn_status s;
    if (a->have_pot) return 0;
    if (!a->pot && !(a->pot = (double *)malloc(a->N * sizeof(double)))) return -1;
    /* every writer calls dipole_potential with MAX = 6 (src/starrynight-analysis.c:68) */
    if ((s = sn_gpu_potential(a->h, 0, 6, a->pot)) != SN_OK) return ana_fail(a, "sn_gpu_potential", s);
    a->have_pot = 1;
    return 0;
}

static int ana_io(int rc, const char *name)
{
    if (rc) fprintf(stderr, "cannot write %s\n", name);
    return rc;
}

static int ana_field(ana_t *a, const char *name, int cutoff, int half)
{
    sn_status s;
    if (!a->map && !(a->map = (double *)malloc(a->N * sizeof(double)))) return -1;
    if ((s = sn_gpu_efield(a->h, 0, cutoff, half, a->map)) != SN_OK) return ana_fail(a, "sn_gpu_efield", s);
    return ana_io(sn_io_write_field_xyz(name, a->c->X, a->c->Y, a->c->Z, a->map), name);
}

static int ana_pot_xyz(ana_t *a, const char *name)
{
    if (ana_potential(a)) return -1;
    return ana_io(sn_io_write_potential_xyz(name, a->c->X, a->c->Y, a->c->Z, a->pot), name);
}

static int ana_cube(ana_t *a, const char *name)
{
    if (ana_potential(a)) return -1;
    return ana_io(sn_io_write_potential_cube(name, a->c->X, a->c->Y, a->c->Z, a->pot), name);
}

static int ana_pgm(ana_t *a, const char *name)
{
    if (ana_potential(a)) return -1;
    return ana_io(sn_io_write_potential_pgm(name, a->c->X, a->c->Y, a->c->Z, a->pot), name);
}

static int ana_dipoles(ana_t *a, const char *name, int kind)
{
    const cfg_t *c = a->c;
    if (ana_lattice(a)) return -1;
    if (kind == 0) return ana_io(sn_io_write_dipoles_xyz(name, c->X, c->Y, c->Z, a->xyz), name);
    if (kind == 1) return ana_io(sn_io_write_dipoles_ppm(name, c->X, c->Y, c->Z, a->xyz), name);
    return ana_io(sn_io_write_dipoles_svg(name, c->X, c->Y, c->Z, a->xyz), name);
}

static int ana_rdf(ana_t *a, const char *name)
{
    enum { C = 9 }; /* radial_order_parameter's CUTOFF (src/starrynight-analysis.c:538) */
    double fe[C * C + 1], afe[C * C + 1];
    int64_t cnt[C * C + 1];
    sn_status s = sn_gpu_radial_order(a->h, 0, C, fe, afe, cnt);
    if (s != SN_OK) return ana_fail(a, "sn_gpu_radial_order", s);
    return ana_io(sn_io_append_rdf(name, C, fe, afe, cnt, (int)a->c->T), name);
}

static int ana_terminal(ana_t *a)
{
    if (ana_lattice(a) || ana_potential(a)) return -1;
    return sn_io_dumb_terminal(stderr, a->c->X, a->c->Y, a->c->Z, a->xyz, a->len, a->pot, (int)a->c->T, &a->dmax);
}

static int ana_recombination(ana_t *a, FILE *log)
{
    if (ana_potential(a)) return -1;
    return sn_io_recombination(log, stderr, a->c->X, a->c->Y, a->c->Z, a->pot, (int)a->c->T);
}

/* analysis_initial, src/starrynight-main.c:29-53 */
static int analysis_initial(ana_t *a)
{
    const cfg_t *c = a->c;
    int rc = 0;
    a->have_lattice = a->have_pot = 0;
    if (c->calc_efield) rc |= ana_field(a, "initial_lattice_efield.xyz", 4, 0);
    if (c->calc_efield) rc |= ana_field(a, "initial_lattice_efieldoffset.xyz", 2, 1);
    if (c->potential) rc |= ana_pot_xyz(a, "initial_lattice_potential.xyz");
    if (c->save_cube) rc |= ana_cube(a, "initial_lattice_potential.cube");
    if (c->save_svg) rc |= ana_dipoles(a, "initial-SVG.svg", 2);
    if (c->potential) rc |= ana_pgm(a, "initial_pot.png");
    if (c->save_xyz) rc |= ana_dipoles(a, "initial_dipoles.xyz", 0);
    if (c->radial) rc |= ana_rdf(a, "rdf.dat");
    if (c->save_png) rc |= ana_dipoles(a, "initial.png", 1);
    if (c->potential) rc |= ana_pgm(a, "initial_pot.png");
    if (c->dumb_terminal) rc |= ana_terminal(a);
    if (c->recombination) rc |= ana_recombination(a, stderr);
    return rc;
}

/* analysis_midpoint, src/starrynight-main.c:56-103 */
static int analysis_midpoint(ana_t *a, int step)
{
    const cfg_t *c = a->c;
    char prefix[64], name[128];
    int rc = 0;
    a->have_lattice = a->have_pot = 0;
    snprintf(prefix, sizeof(prefix), "T_%04d_%d_%03d", (int)c->T, (int)c->cage_strain, step);
    if (c->dumb_terminal) rc |= ana_terminal(a);
    if (c->recombination) rc |= ana_recombination(a, a->log);
    snprintf(name, sizeof(name), "%s-RDF.dat", prefix);
    if (c->radial) rc |= ana_rdf(a, name);
    snprintf(name, sizeof(name), "%s_efield.xyz", prefix);
    if (c->calc_efield) rc |= ana_field(a, name, 4, 0);
    snprintf(name, sizeof(name), "%s_potential.xyz", prefix);
    if (c->potential) rc |= ana_pot_xyz(a, name);
    snprintf(name, sizeof(name), "%s_potential.cube", prefix);
    if (c->save_cube) rc |= ana_cube(a, name);
    snprintf(name, sizeof(name), "%s_potential.png", prefix);
    if (c->potential) rc |= ana_pgm(a, name);
    snprintf(name, sizeof(name), "%s_MC-PNG.png", prefix);
    if (c->save_png) rc |= ana_dipoles(a, name, 1);
    snprintf(name, sizeof(name), "%s_MC-SVG.svg", prefix);
    if (c->save_svg) rc |= ana_dipoles(a, name, 2);
    return rc;
}

static int write_checkpoint(ana_t *a, unsigned long long accept, unsigned long long attempt)
{
    const cfg_t *c = a->c;
    sn_checkpoint k;
    uint64_t sweeps = 0;
    sn_status s;
    a->have_lattice = 0;
    if (ana_lattice(a)) return -1;
    if ((s = sn_gpu_sweep_count(a->h, &sweeps)) != SN_OK) return ana_fail(a, "sn_gpu_sweep_count", s);
    memset(&k, 0, sizeof(k));
    k.X = c->X;
    k.Y = c->Y;
    k.Z = c->Z;
    k.cutoff = c->cutoff;
    k.sweeps = sweeps;
    k.seed = c->seed;
    k.T = c->T;
    k.efield[0] = c->efield[0];
    k.efield[1] = c->efield[1];
    k.efield[2] = c->efield[2];
    k.accept = accept;
    k.attempt = attempt;
    return ana_io(sn_io_write_checkpoint(c->checkpoint, &k, a->xyz, a->len), c->checkpoint);
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        sn_status s_ = (call);                                                                    \
        if (s_ != SN_OK) {                                                                        \
            fprintf(stderr, "%s failed: %s (%s)\n", #call, sn_gpu_status_string(s_), sn_gpu_last_error(h)); \
            if (h) sn_gpu_destroy(h);                                                             \
            return 2;                                                                             \
        }                                                                                         \
    } while (0)

#define CKA(call)                                                                                 \
    do {                                                                                          \
        if ((call) != 0) {                                                                        \
            sn_gpu_destroy(h);                                                                    \
            return 2;                                                                             \
        }                                                                                         \
    } while (0)

int main(int argc, char **argv)
{
    cfg_t c;
    const char *cfg_path = "starrynight.cfg";
    int print_only = 0, npos = 0, i;
    const char *pos[2] = {NULL, NULL};
    long long seed_opt = -1;
    sn_handle *h = NULL;
    cfg_defaults(&c);
    for (i = 1; i < argc; i++) {
        if (!strcmp(argv[i], "--config") && i + 1 < argc) cfg_path = argv[++i];
        else if (!strcmp(argv[i], "--seed") && i + 1 < argc) seed_opt = strtoll(argv[++i], NULL, 0);
        else if (!strcmp(argv[i], "--print-config")) print_only = 1;
        else if (npos < 2) pos[npos++] = argv[i];
    }
    fprintf(stderr, "starrynight-gpu: loading %s\n", cfg_path);
    if (!cfg_load(cfg_path, &c)) return EXIT_FAILURE;
    if (pos[0]) c.T = atof(pos[0]);            /* src/starrynight-main.c:142-146 */
    if (pos[1]) c.cage_strain = atof(pos[1]);  /* :147-151 */
    if (seed_opt >= 0) {
        c.seed = (unsigned long long)seed_opt;
        c.has_seed = 1;
    }
    if (!c.has_seed) c.seed = (unsigned long long)(uint32_t)(0xDEADBEEFu + (uint32_t)(int)c.T);
    if (print_only) {
        printf("T %g\nX %d\nY %d\nZ %d\nEfield %g %g %g\nK %g\nCageStrain %g\nDipoleCutOff %d\n", c.T, c.X, c.Y,
               c.Z, c.efield[0], c.efield[1], c.efield[2], c.K, c.cage_strain, c.cutoff);
        printf("Dipoles");
        for (i = 0; i < c.n_species; i++) printf(" %g", c.dipoles[i]);
        printf("\nPrevalence");
        for (i = 0; i < c.n_species; i++) printf(" %g", c.prevalence[i]);
        printf("\nConstrainToX %d\nInitialLattice %s\nMCEqmSteps %d\nMCMegaSteps %d\nMCMoves %g\nSeed %llu\n",
               c.constrain_to_x, c.initial, c.eqm_steps, c.mega_steps, c.mc_moves, c.seed);
        printf("DisplayDumbTerminal %d\nCalculateRecombination %d\nCalculateRadialOrderParameter %d\n"
               "CalculatePotential %d\nCalculateEfield %d\nSaveDipolesXYZ %d\nSaveDipolesPNG %d\n"
               "SaveDipolesSVG %d\nSavePotentialCube %d\nResumeFrom %s\nCheckpointFile %s\nCheckpointEvery %d\n"
               "AutoTune %d\n",
               c.dumb_terminal, c.recombination, c.radial, c.potential, c.calc_efield, c.save_xyz, c.save_png,
               c.save_svg, c.save_cube, c.resume, c.checkpoint, c.checkpoint_every, c.autotune);
        return 0;
    }
    {
        sn_params P;
        sn_replica_desc R;
        ana_t a;
        char logname[64];
        const size_t N = (size_t)c.X * c.Y * c.Z;
        const int sweeps = c.mc_moves >= 1.0 ? (int)lround(c.mc_moves) : 1;
        unsigned long long ACCEPT = 0, REJECT = 0;
        memset(&P, 0, sizeof(P));
        memset(&R, 0, sizeof(R));
        memset(&a, 0, sizeof(a));
        P.cutoff = c.cutoff;
        P.dim = 3;
        P.constrain_to_x = c.constrain_to_x;
        P.cage_strain = c.cage_strain;
        P.K = c.K;
        memcpy(P.efield, c.efield, sizeof(P.efield));
        P.n_species = c.n_species;
        memcpy(P.dipoles, c.dipoles, sizeof(P.dipoles));
        memcpy(P.prevalence, c.prevalence, sizeof(P.prevalence));
        P.seed = c.seed;
        R.X = c.X;
        R.Y = c.Y;
        R.Z = c.Z;
        R.T = (float)c.T;
        R.seed = c.seed;
        if (c.mc_moves != (double)sweeps)
            fprintf(stderr, "MCMoves %g rounded to %d whole sweeps per megastep\n", c.mc_moves, sweeps);
        /* the log file of src/starrynight-main.c:163-177 */
        snprintf(logname, sizeof(logname), "Recombination_T_%04d.log", (int)c.T);
        a.log = fopen(logname, "w");
        if (!a.log) {
            fprintf(stderr, "cannot open %s\n", logname);
            return 2;
        }
        fprintf(a.log, "# Starrynight - simulation run on time(NULL)= %ld\n# Philox seed: %llX\n", (long)time(NULL),
                c.seed);
        if (c.autotune > 0) {
            double ms = 0.0;
            CK(sn_gpu_autotune(&P, &R, c.autotune, 5, R.block, &ms));
            fprintf(stderr, "AutoTune: block %dx%dx%d, %.3f ms per sweep\n", R.block[0], R.block[1], R.block[2], ms);
        }
        CK(sn_gpu_init(&P, 1, &R, &h));
        a.h = h;
        a.c = &c;
        a.N = N;
        a.dmax = 55.0f;
        /* page-locked when the device allows: lattice downloads at the host-link rate */
        a.xyz = (float *)sn_gpu_host_alloc(3 * N * sizeof(float));
        a.len = (float *)sn_gpu_host_alloc(N * sizeof(float));
        a.pinned = a.xyz && a.len;
        if (!a.pinned) {
            sn_gpu_host_free(a.xyz);
            sn_gpu_host_free(a.len);
            a.xyz = (float *)malloc(3 * N * sizeof(float));
            a.len = (float *)malloc(N * sizeof(float));
        }
        if (!a.xyz || !a.len) {
            fprintf(stderr, "out of host memory\n");
            sn_gpu_destroy(h);
            return 2;
        }
        if (c.resume[0]) {
            sn_checkpoint k;
            int rc;
            memset(&k, 0, sizeof(k));
            k.X = c.X;
            k.Y = c.Y;
            k.Z = c.Z;
            rc = sn_io_read_checkpoint(c.resume, &k, a.xyz, a.len);
            if (rc) {
                fprintf(stderr, "cannot resume from %s (%s)\n", c.resume,
                        rc == -3 ? "lattice size differs" : rc == -2 ? "not a valid checkpoint" : "cannot read");
                sn_gpu_destroy(h);
                return 2;
            }
            if (k.seed != c.seed)
                fprintf(stderr, "warning: checkpoint seed %llX differs from the run's seed %llX\n",
                        (unsigned long long)k.seed, c.seed);
            CK(sn_gpu_upload_lattice(h, 0, a.xyz, a.len));
            CK(sn_gpu_set_sweep_count(h, k.sweeps));
            fprintf(stderr, "Resumed from %s at sweep %llu\n", c.resume, (unsigned long long)k.sweeps);
        } else if (!strcmp(c.initial, "random")) {
            CK(sn_gpu_init_lattice(h, 0, SN_LATTICE_RANDOM, 0));
        } else {
            /* species from the device solid solution, orientation from the pattern */
            CK(sn_gpu_init_lattice(h, 0, SN_LATTICE_FERROELECTRIC, 0));
            CK(sn_gpu_download_lattice(h, 0, NULL, a.len));
            pattern(&c, a.xyz);
            if (!strcmp(c.initial, "slab_delete")) { /* src/starrynight-lattice.c:126-137 */
                size_t k;
                CK(sn_gpu_init_lattice(h, 0, SN_LATTICE_RANDOM, 0));
                CK(sn_gpu_download_lattice(h, 0, a.xyz, a.len));
                for (k = 0; k < (size_t)(c.X < 6 ? c.X : 6) * c.Y * c.Z; k++)
                    a.xyz[3 * k] = a.xyz[3 * k + 1] = a.xyz[3 * k + 2] = 0.0f;
            }
            CK(sn_gpu_upload_lattice(h, 0, a.xyz, a.len));
        }
        a.have_lattice = a.have_pot = 0;
        if (c.dumb_terminal) CKA(ana_terminal(&a)); /* src/starrynight-main.c:208 */
        CKA(analysis_initial(&a));
        fprintf(stderr, "'.' is %e MC moves attempted.\n", (double)N * sweeps);
        for (i = 0; i < c.eqm_steps; i++) {
            fprintf(stderr, ",");
            CK(sn_gpu_sweep(h, sweeps, NULL, NULL));
        }
        fprintf(stderr, "\n");
        /* after equilibration, src/starrynight-main.c:225-227 */
        a.have_lattice = a.have_pot = 0;
        if (c.calc_efield) CKA(ana_field(&a, "equilib_lattice_efield.xyz", 4, 0));
        if (c.save_svg) CKA(ana_dipoles(&a, "equilib-SVG.svg", 2));
        if (c.potential) CKA(ana_pgm(&a, "equilib_pot.png"));
        printf("# megastep sweeps E_per_site P_abs_per_site Px Py Pz\n");
        for (i = 0; i < c.mega_steps; i++) {
            uint64_t acc = 0, rej = 0;
            double E, Pabs, Pv[3];
            const double t0 = now_s();
            CK(sn_gpu_sweep(h, sweeps, &acc, &rej));
            const double t1 = now_s();
            CK(sn_gpu_observables(h, &E, &Pabs, Pv));
            ACCEPT += acc;
            REJECT += rej;
            CKA(analysis_midpoint(&a, i));
            printf("%d %d %.10f %.10f %.6f %.6f %.6f\n", i, (c.eqm_steps + i + 1) * sweeps, E, Pabs, Pv[0], Pv[1], Pv[2]);
            fflush(stdout);
            {
                const double t2 = now_s();
                fprintf(stderr, "MC Moves (per second): %f MHz\n", 1e-6 * (double)(acc + rej) / (t1 - t0));
                fprintf(stderr, "Output routines: %f s ; Efficiency of MC moves vs. analysis %.2f%%\n", t2 - t1,
                        100.0 * (t1 - t0) / (t2 - t0));
            }
            if (c.checkpoint[0] && c.checkpoint_every > 0 && (i + 1) % c.checkpoint_every == 0)
                CKA(write_checkpoint(&a, ACCEPT, ACCEPT + REJECT));
        }
        if (c.checkpoint[0]) CKA(write_checkpoint(&a, ACCEPT, ACCEPT + REJECT));
        fprintf(stderr, "\n");
        fprintf(stderr, "Monte Carlo moves - ACCEPT: %llu REJECT: %llu ratio: %f\n", ACCEPT, REJECT,
                (float)ACCEPT / (float)(REJECT + ACCEPT));
        fclose(a.log);
        if (a.pinned) {
            sn_gpu_host_free(a.xyz);
            sn_gpu_host_free(a.len);
        } else {
            free(a.xyz);
            free(a.len);
        }
        free(a.pot);
        free(a.map);
        sn_gpu_destroy(h);
    }
    return 0;
}
