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
 * P_z.  SaveDipolesXYZ writes initial_dipoles.xyz in the format of
 * outputlattice_xyz (src/starrynight-analysis.c:710-728).
 *
 * Additional keys: Dipole (single species length) and DipoleFraction
 * (occupancy p: Dipoles = [Dipole, 0], Prevalence = [p, 1-p]), and Seed
 * (Philox key; default 0xDEADBEEF + T as the reference seeds MT,
 * src/starrynight-main.c:172).  Options: --config FILE, --seed N,
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
    int save_xyz;
    int has_seed;
    unsigned long long seed;
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
    config_lookup_bool(&cf, "SaveDipolesXYZ", &c->save_xyz);
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

/* outputlattice_xyz, src/starrynight-analysis.c:710-728 */
static void write_xyz(const char *name, const cfg_t *c, const float *xyz)
{
    const float r = 1.6f / 2, d = 4.0f, zs = 5.0f;
    int x, y, z;
    FILE *fo = fopen(name, "w");
    if (!fo) {
        fprintf(stderr, "cannot write %s\n", name);
        return;
    }
    fprintf(fo, "%d\n\n", c->X * c->Y * c->Z * 2);
    for (x = 0; x < c->X; x++)
        for (y = 0; y < c->Y; y++)
            for (z = 0; z < c->Z; z++) {
                const float *p = &xyz[3 * (((size_t)x * c->Y + y) * c->Z + z)];
                fprintf(fo, "C %f %f %f\n", d * x + r * p[0], d * y + r * p[1], zs * (d * z) + r * p[2]);
                fprintf(fo, "N %f %f %f\n", d * x - r * p[0], d * y - r * p[1], zs * (d * z) - r * p[2]);
            }
    fclose(fo);
}

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
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
        return 0;
    }
    {
        sn_params P;
        sn_replica_desc R;
        const size_t N = (size_t)c.X * c.Y * c.Z;
        const int sweeps = c.mc_moves >= 1.0 ? (int)lround(c.mc_moves) : 1;
        unsigned long long ACCEPT = 0, REJECT = 0;
        float *xyz = NULL, *len = NULL;
        memset(&P, 0, sizeof(P));
        memset(&R, 0, sizeof(R));
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
        CK(sn_gpu_init(&P, 1, &R, &h));
        xyz = (float *)malloc(3 * N * sizeof(float));
        len = (float *)malloc(N * sizeof(float));
        if (!xyz || !len) {
            fprintf(stderr, "out of host memory\n");
            sn_gpu_destroy(h);
            return 2;
        }
        if (!strcmp(c.initial, "random")) {
            CK(sn_gpu_init_lattice(h, 0, SN_LATTICE_RANDOM, 0));
        } else {
            /* species from the device solid solution, orientation from the pattern */
            CK(sn_gpu_init_lattice(h, 0, SN_LATTICE_FERROELECTRIC, 0));
            CK(sn_gpu_download_lattice(h, 0, NULL, len));
            pattern(&c, xyz);
            if (!strcmp(c.initial, "slab_delete")) { /* src/starrynight-lattice.c:126-137 */
                size_t k;
                CK(sn_gpu_init_lattice(h, 0, SN_LATTICE_RANDOM, 0));
                CK(sn_gpu_download_lattice(h, 0, xyz, len));
                for (k = 0; k < (size_t)(c.X < 6 ? c.X : 6) * c.Y * c.Z; k++) xyz[3 * k] = xyz[3 * k + 1] = xyz[3 * k + 2] = 0.0f;
            }
            CK(sn_gpu_upload_lattice(h, 0, xyz, len));
        }
        if (c.save_xyz) {
            CK(sn_gpu_download_lattice(h, 0, xyz, NULL));
            write_xyz("initial_dipoles.xyz", &c, xyz);
        }
        fprintf(stderr, "'.' is %e MC moves attempted.\n", (double)N * sweeps);
        for (i = 0; i < c.eqm_steps; i++) {
            fprintf(stderr, ",");
            CK(sn_gpu_sweep(h, sweeps, NULL, NULL));
        }
        fprintf(stderr, "\n");
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
            printf("%d %d %.10f %.10f %.6f %.6f %.6f\n", i, (c.eqm_steps + i + 1) * sweeps, E, Pabs, Pv[0], Pv[1], Pv[2]);
            fflush(stdout);
            fprintf(stderr, "MC Moves (per second): %f MHz\n", 1e-6 * (double)(acc + rej) / (t1 - t0));
        }
        fprintf(stderr, "Monte Carlo moves - ACCEPT: %llu REJECT: %llu ratio: %f\n", ACCEPT, REJECT,
                (float)ACCEPT / (float)(REJECT + ACCEPT));
        free(xyz);
        free(len);
        sn_gpu_destroy(h);
    }
    return 0;
}
