/*
 * sn_oracle.c -- CPU oracle for the Metropolis dipole-lattice sweep.
 * TEST INFRASTRUCTURE ONLY (checker for the CUDA path, CPU baseline for
 * bench.py).  See sn_oracle.h for what each part restates.
 *
 * Compile with -ffp-contract=off: every float/double operation below must be
 * rounded individually, as in the reference's x86-64 build, so the same bits
 * come out on x86-64 and aarch64 hosts.
 */
#include "sn_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ====================================================================== */
/* MT19937: Matsumoto & Nishimura, ACM TOMACS 8(1), 1998.  The reference
 * vendors it as src/mt19937ar-cok.c (Cokus' ordering of the same sequence). */
enum { MT_N = 624, MT_M = 397 };

void sno_mt_seed(sno_mt *g, uint32_t seed)
{
    int i;
    g->mt[0] = seed;
    for (i = 1; i < MT_N; i++)
        g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
    g->mti = MT_N;
}

static void mt_refill(sno_mt *g)
{
    int i;
    for (i = 0; i < MT_N; i++) {
        uint32_t y = (g->mt[i] & 0x80000000u) | (g->mt[(i + 1) % MT_N] & 0x7fffffffu);
        uint32_t v = g->mt[(i + MT_M) % MT_N] ^ (y >> 1);
        if (y & 1u) v ^= 0x9908b0dfu;
        g->mt[i] = v;
    }
    g->mti = 0;
}

uint32_t sno_mt_u32(sno_mt *g)
{
    uint32_t y;
    if (g->mti >= MT_N) mt_refill(g);
    y = g->mt[g->mti++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

double sno_mt_real1(sno_mt *g) { return (double)sno_mt_u32(g) * (1.0 / 4294967295.0); }
double sno_mt_real2(sno_mt *g) { return (double)sno_mt_u32(g) * (1.0 / 4294967296.0); }

/* ====================================================================== */
/* Philox4x32-10: Salmon, Moraes, Dror, Shaw, SC'11.  Ten rounds of the
 * 4x32 S-box with the published multipliers and Weyl key increments. */
void sno_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    int r;
    for (r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* ====================================================================== */
/* gen_neighbour, src/starrynight-montecarlo-core.c:38-72 (same loop order,
 * same float distance computation, same Z==1 special case). */
int sno_gen_neighbours(int cutoff, int Z, int *odx, int *ody, int *odz, float *od, int max)
{
    int n = 0, dx, dy, dz;
    int zc = (Z == 1) ? 0 : cutoff;
    for (dx = -cutoff; dx <= cutoff; dx++)
        for (dy = -cutoff; dy <= cutoff; dy++)
            for (dz = -zc; dz <= zc; dz++) {
                float d;
                if (dx == 0 && dy == 0 && dz == 0) continue;
                d = (float)sqrt((float)dx * dx + dy * dy + dz * dz);
                if (d > (float)cutoff) continue;
                if (n >= max) return -1;
                odx[n] = dx;
                ody[n] = dy;
                odz[n] = dz;
                od[n] = d;
                n++;
            }
    return n;
}

typedef struct {
    int n;
    int *dx, *dy, *dz;
    float *d;
} nbtab;

static int nbtab_build(nbtab *t, int cutoff, int Z)
{
    int side = 2 * cutoff + 1;
    int max = side * side * side;
    t->dx = (int *)malloc(sizeof(int) * (size_t)max);
    t->dy = (int *)malloc(sizeof(int) * (size_t)max);
    t->dz = (int *)malloc(sizeof(int) * (size_t)max);
    t->d = (float *)malloc(sizeof(float) * (size_t)max);
    if (!t->dx || !t->dy || !t->dz || !t->d) return 0;
    t->n = sno_gen_neighbours(cutoff, Z, t->dx, t->dy, t->dz, t->d, max);
    return t->n >= 0;
}

static void nbtab_free(nbtab *t)
{
    free(t->dx);
    free(t->dy);
    free(t->dz);
    free(t->d);
}

static inline long site_index(const sno_model *m, int x, int y, int z)
{
    return ((long)x * m->Y + y) * m->Z + z;
}

static inline int wrap(int v, int L) { return ((v % L) + L) % L; }

/* ====================================================================== */
/* Reference-faithful engine.  The float/double mix of every expression
 * follows the reference line by line; comments give the line restated. */

/* dot(), src/starrynight-config.c:189-199: float accumulation from 0. */
static float ref_dot(const float *a, const float *b)
{
    float sum = 0.0f;
    sum += a[0] * b[0];
    sum += a[1] * b[1];
    sum += a[2] * b[2];
    return sum;
}

/* random_sphere_point, src/starrynight-config.c:203-227 (DIM<3 circle branch
 * :213-219, sphere branch :221-226). */
static void ref_sphere_point(const sno_model *m, sno_mt *g, float *p)
{
    float x1, x2;
    do {
        x1 = (float)(2.0 * sno_mt_real1(g) - 1.0);
        x2 = (float)(2.0 * sno_mt_real1(g) - 1.0);
    } while ((double)(x1 * x1 + x2 * x2) > 1.0);
    if (m->dim < 3) {
        p[0] = (x1 * x1 - x2 * x2) / (x1 * x1 + x2 * x2);
        p[1] = 2 * x1 * x2 / (x1 * x1 + x2 * x2);
        p[2] = 0.0f;
    } else {
        float s1 = 1 - x1 * x1 - x2 * x2;
        p[0] = (float)((double)(2 * x1) * sqrt((double)s1));
        p[1] = (float)((double)(2 * x2) * sqrt((double)s1));
        p[2] = (float)(1.0 - 2.0 * (double)(x1 * x1 + x2 * x2));
    }
}

/* random_X_point, src/starrynight-config.c:230-263. */
static void ref_x_point(sno_mt *g, float *p)
{
    int i = (int)(sno_mt_u32(g) % 6u);
    p[0] = p[1] = p[2] = 0.0f;
    switch (i) {
    case 0: p[0] = 1.0f; break;
    case 1: p[0] = -1.0f; break;
    case 2: p[1] = 1.0f; break;
    case 3: p[1] = -1.0f; break;
    case 4: p[2] = 1.0f; break;
    default: p[2] = -1.0f; break;
    }
}

void sno_ref_init_random(const sno_model *m, float *lat4, sno_mt *g,
                         int n_species, const float *lengths, const float *prevalence)
{
    int x, y, z;
    /* initialise_lattice_random, src/starrynight-lattice.c:25-37 */
    for (x = 0; x < m->X; x++)
        for (y = 0; y < m->Y; y++)
            for (z = 0; z < m->Z; z++)
                ref_sphere_point(m, g, &lat4[4 * site_index(m, x, y, z)]);
    /* solid_solution, src/starrynight-lattice.c:139-171 */
    for (x = 0; x < m->X; x++)
        for (y = 0; y < m->Y; y++)
            for (z = 0; z < m->Z; z++) {
                float sample = (float)sno_mt_real1(g);
                int i = 0;
                while (i < n_species - 1 && sample > prevalence[i]) {
                    sample -= prevalence[i];
                    i++;
                }
                lat4[4 * site_index(m, x, y, z) + 3] = lengths[i];
            }
}

/* site_energy, src/starrynight-montecarlo-core.c:76-141. */
static double ref_site_energy_tab(const sno_model *m, const nbtab *nb, const float *lat4,
                                  int x, int y, int z, const float *newd, const float *oldd)
{
    double dE = 0.0;
    int i;
    for (i = 0; i < nb->n; i++) {
        int dx = nb->dx[i], dy = nb->dy[i], dz = nb->dz[i];
        float d = nb->d[i];
        const float *t = &lat4[4 * site_index(m, (m->X + x + dx) % m->X, (m->Y + y + dy) % m->Y,
                                              (m->Z + z + dz) % m->Z)];
        float n[3];
        float dnt, term;
        n[0] = (float)dx / d;
        n[1] = (float)dy / d;
        n[2] = (float)dz / d;
        dnt = ref_dot(n, t);
        /* :102-106 */
        term = (oldd[3] * t[3]) *
               ((ref_dot(newd, t) - 3 * ref_dot(n, newd) * dnt) -
                (ref_dot(oldd, t) - 3 * ref_dot(n, oldd) * dnt)) /
               (d * d * d);
        dE += term;
        /* :113-115, cage strain on the six unit offsets */
        if (dx * dx + dy * dy + dz * dz == 1)
            dE += -m->cage_strain * (double)ref_dot(newd, t) + m->cage_strain * (double)ref_dot(oldd, t);
    }
    /* :120-121 */
    dE += (double)(ref_dot(newd, m->efield) - ref_dot(oldd, m->efield));
    /* :124-134 */
    if (m->K > 0.0) {
        float ex[3] = {1.0f, 0.0f, 0.0f}, ey[3] = {0.0f, 1.0f, 0.0f};
        dE += -m->K * fabs((double)ref_dot(newd, ex)) + m->K * fabs((double)ref_dot(oldd, ex));
        dE += -m->K * fabs((double)ref_dot(newd, ey)) + m->K * fabs((double)ref_dot(oldd, ey));
    }
    return dE;
}

double sno_ref_site_energy(const sno_model *m, const float *lat4, int x, int y, int z,
                           const float newd[4], const float oldd[4])
{
    nbtab nb;
    double r = 0.0;
    if (nbtab_build(&nb, m->cutoff, m->Z)) r = ref_site_energy_tab(m, &nb, lat4, x, y, z, newd, oldd);
    nbtab_free(&nb);
    return r;
}

/* MC_moves / MC_move, src/starrynight-montecarlo-core.c:143-191, with
 * rand_int at :18-21. */
void sno_ref_mc_moves(const sno_model *m, float *lat4, sno_mt *g, long long moves,
                      uint64_t *accept, uint64_t *reject)
{
    nbtab nb;
    long long k;
    if (!nbtab_build(&nb, m->cutoff, m->Z)) {
        nbtab_free(&nb);
        return;
    }
    for (k = 0; k < moves; k++) {
        int x = (int)(sno_mt_u32(g) % (uint32_t)m->X);
        int y = (int)(sno_mt_u32(g) % (uint32_t)m->Y);
        int z = (int)(sno_mt_u32(g) % (uint32_t)m->Z);
        float *old = &lat4[4 * site_index(m, x, y, z)];
        float nw[4];
        float dE;
        if (old[3] == 0.0f) continue; /* :163 vacancy */
        if (m->constrain_to_x)
            ref_x_point(g, nw);
        else
            ref_sphere_point(m, g, nw);
        nw[3] = old[3];
        dE = (float)ref_site_energy_tab(m, &nb, lat4, x, y, z, nw, old);
        if (dE < 0.0 || exp((double)(-dE) * m->beta) > sno_mt_real2(g)) { /* :179 */
            old[0] = nw[0];
            old[1] = nw[1];
            old[2] = nw[2];
            (*accept)++;
        } else {
            (*reject)++;
        }
    }
    nbtab_free(&nb);
}

/* ====================================================================== */
/* Philox proposal of the GPU path.  The exact float operations here are the
 * contract the CUDA kernel follows: only correctly rounded + - * / sqrt. */
static const float TWO_M23 = 1.1920928955078125e-07f; /* 2^-23 */
static const float TWO_M24 = 5.9604644775390625e-08f; /* 2^-24 */

static int try_point(const sno_model *m, uint32_t ra, uint32_t rb, float p[3])
{
    float x1 = (float)(ra >> 8) * TWO_M23 - 1.0f;
    float x2 = (float)(rb >> 8) * TWO_M23 - 1.0f;
    float a = x1 * x1;
    float b = x2 * x2;
    float q = a + b;
    if (q > 1.0f) return 0;
    if (m->dim < 3) {
        if (q == 0.0f) return 0;
        p[0] = (a - b) / q;
        p[1] = ((2.0f * x1) * x2) / q;
        p[2] = 0.0f;
    } else {
        float t = sqrtf(1.0f - q);
        p[0] = (2.0f * x1) * t;
        p[1] = (2.0f * x2) * t;
        p[2] = 1.0f - 2.0f * q;
    }
    return 1;
}

enum { PROPOSAL_MAX_CALLS = 16 };

/* Returns 1 with p set, or 0 if every try was rejected (then the move keeps
 * the old dipole). */
static int proposal(const sno_model *m, const sno_stream *st, uint32_t site, uint32_t sweep,
                    float p[3], float *u)
{
    uint32_t key[2] = {(uint32_t)st->seed, (uint32_t)(st->seed >> 32)};
    uint32_t ctr[4] = {site, sweep, 0u, 0u};
    uint32_t r[4];
    uint32_t k;
    sno_philox4x32_10(ctr, key, r);
    *u = (float)(r[0] >> 8) * TWO_M24;
    if (m->constrain_to_x) {
        uint32_t c = (uint32_t)(((uint64_t)r[3] * 6u) >> 32);
        p[0] = p[1] = p[2] = 0.0f;
        p[c >> 1] = (c & 1u) ? -1.0f : 1.0f;
        return 1;
    }
    if (try_point(m, r[1], r[2], p)) return 1;
    for (k = 1; k < PROPOSAL_MAX_CALLS; k++) {
        ctr[2] = k;
        sno_philox4x32_10(ctr, key, r);
        if (try_point(m, r[0], r[1], p)) return 1;
        if (try_point(m, r[2], r[3], p)) return 1;
    }
    return 0;
}

void sno_proposal(const sno_model *m, const sno_stream *st, uint32_t site, uint32_t sweep,
                  float p[3], float *u)
{
    if (!proposal(m, st, site, sweep, p, u)) p[0] = p[1] = p[2] = NAN;
}

/* ====================================================================== */
/* FP64 local field of site i: h = sum_j len_j T_o p_j, nn = sum_{|o|=1} p_j */
typedef struct {
    int n;
    int *dx, *dy, *dz;
    double *T; /* 6 per offset: xx yy zz xy xz yz */
    int *unit;
} tab64;

static int tab64_build(tab64 *t, int cutoff, int Z)
{
    nbtab nb;
    int i;
    if (!nbtab_build(&nb, cutoff, Z)) {
        nbtab_free(&nb);
        return 0;
    }
    t->n = nb.n;
    t->dx = nb.dx;
    t->dy = nb.dy;
    t->dz = nb.dz;
    free(nb.d);
    t->T = (double *)malloc(sizeof(double) * 6 * (size_t)(t->n > 0 ? t->n : 1));
    t->unit = (int *)malloc(sizeof(int) * (size_t)(t->n > 0 ? t->n : 1));
    if (!t->T || !t->unit) return 0;
    for (i = 0; i < t->n; i++) {
        double ox = t->dx[i], oy = t->dy[i], oz = t->dz[i];
        double r2 = ox * ox + oy * oy + oz * oz;
        double d = sqrt(r2);
        double inv3 = 1.0 / (r2 * d);
        double nx = ox / d, ny = oy / d, nz = oz / d;
        t->T[6 * i + 0] = (1.0 - 3.0 * nx * nx) * inv3;
        t->T[6 * i + 1] = (1.0 - 3.0 * ny * ny) * inv3;
        t->T[6 * i + 2] = (1.0 - 3.0 * nz * nz) * inv3;
        t->T[6 * i + 3] = -3.0 * nx * ny * inv3;
        t->T[6 * i + 4] = -3.0 * nx * nz * inv3;
        t->T[6 * i + 5] = -3.0 * ny * nz * inv3;
        t->unit[i] = (t->dx[i] * t->dx[i] + t->dy[i] * t->dy[i] + t->dz[i] * t->dz[i]) == 1;
    }
    return 1;
}

static void tab64_free(tab64 *t)
{
    free(t->dx);
    free(t->dy);
    free(t->dz);
    free(t->T);
    free(t->unit);
}

static void field64(const sno_model *m, const tab64 *t, const float *px, const float *py,
                    const float *pz, const float *len, int x, int y, int z, double h[3], double nn[3])
{
    int i;
    h[0] = h[1] = h[2] = 0.0;
    nn[0] = nn[1] = nn[2] = 0.0;
    for (i = 0; i < t->n; i++) {
        long j = site_index(m, wrap(x + t->dx[i], m->X), wrap(y + t->dy[i], m->Y), wrap(z + t->dz[i], m->Z));
        double lj = len[j];
        double qx = px[j], qy = py[j], qz = pz[j];
        const double *T = &t->T[6 * i];
        h[0] += lj * (T[0] * qx + T[3] * qy + T[4] * qz);
        h[1] += lj * (T[3] * qx + T[1] * qy + T[5] * qz);
        h[2] += lj * (T[4] * qx + T[5] * qy + T[2] * qz);
        if (t->unit[i]) {
            nn[0] += qx;
            nn[1] += qy;
            nn[2] += qz;
        }
    }
}

static double k_term(const sno_model *m, double x, double y)
{
    return m->K > 0.0 ? -m->K * (fabs(x) + fabs(y)) : 0.0;
}

double sno_delta_energy64(const sno_model *m, const float *px, const float *py, const float *pz,
                          const float *len, int site, const float newp[3])
{
    tab64 t;
    double h[3], nn[3], g[3], dE;
    int x, y, z;
    if (!tab64_build(&t, m->cutoff, m->Z)) {
        tab64_free(&t);
        return NAN;
    }
    x = site / (m->Y * m->Z);
    y = (site / m->Z) % m->Y;
    z = site % m->Z;
    field64(m, &t, px, py, pz, len, x, y, z, h, nn);
    g[0] = len[site] * h[0] - m->cage_strain * nn[0] + m->efield[0];
    g[1] = len[site] * h[1] - m->cage_strain * nn[1] + m->efield[1];
    g[2] = len[site] * h[2] - m->cage_strain * nn[2] + m->efield[2];
    dE = ((double)newp[0] - px[site]) * g[0] + ((double)newp[1] - py[site]) * g[1] +
         ((double)newp[2] - pz[site]) * g[2];
    dE += k_term(m, newp[0], newp[1]) - k_term(m, px[site], py[site]);
    tab64_free(&t);
    return dE;
}

uint64_t sno_colour_sweep(const sno_model *m, const sno_schedule *sc, const sno_stream *st,
                          uint32_t sweep, float *px, float *py, float *pz, const float *len,
                          const float *gpu_after, double tol,
                          uint64_t *n_borderline, uint64_t *n_hard,
                          double *dE_sum, double *margin_out, uint8_t *accept_out)
{
    tab64 t;
    long N = (long)m->X * m->Y * m->Z;
    int two_d = (m->Z == 1);
    int szc = two_d ? 1 : sc->s;
    int cbx, cby, cbz, cx, cy, cz;
    uint64_t n_acc = 0;
    double beta = (double)st->beta;
    if (!tab64_build(&t, m->cutoff, m->Z)) {
        tab64_free(&t);
        return 0;
    }
    if (margin_out)
        for (long i = 0; i < N; i++) margin_out[i] = NAN;
    if (accept_out) memset(accept_out, 0, (size_t)N);
    /* colour groups: representative (gx,gy,gz) and, when merged, the
     * partner shifted by s/2 along every axis (the two never interact) */
    for (cbx = 0; cbx < sc->mx; cbx++)
        for (cby = 0; cby < sc->my; cby++)
            for (cbz = 0; cbz < sc->mz; cbz++)
                for (int gx = 0; gx < (sc->merge ? sc->s / 2 : sc->s); gx++)
                    for (int gy = 0; gy < sc->s; gy++)
                        for (int gz = 0; gz < szc; gz++)
                            for (int half = 0; half < (sc->merge ? 2 : 1); half++) {
                            int ibx, iby, ibz;
                            cx = half ? (gx + sc->s / 2) % sc->s : gx;
                            cy = half ? (gy + sc->s / 2) % sc->s : gy;
                            cz = half ? (gz + sc->s / 2) % sc->s : gz;
                            for (ibx = cbx; ibx < sc->nbx; ibx += sc->mx)
                                for (iby = cby; iby < sc->nby; iby += sc->my)
                                    for (ibz = cbz; ibz < sc->nbz; ibz += sc->mz) {
                                        int lx, ly, lz;
                                        for (lx = cx; lx < sc->bx; lx += sc->s)
                                            for (ly = cy; ly < sc->by; ly += sc->s)
                                                for (lz = cz; lz < sc->bz; lz += szc) {
                                                    int x = ibx * sc->bx + lx;
                                                    int y = iby * sc->by + ly;
                                                    int z = ibz * sc->bz + lz;
                                                    long i = site_index(m, x, y, z);
                                                    float p[3], u;
                                                    double h[3], nn[3], g[3], dE, thr, margin;
                                                    int acc, gacc;
                                                    if (len[i] == 0.0f) continue;
                                                    if (!proposal(m, st, (uint32_t)i, sweep, p, &u)) {
                                                        p[0] = px[i];
                                                        p[1] = py[i];
                                                        p[2] = pz[i];
                                                    }
                                                    field64(m, &t, px, py, pz, len, x, y, z, h, nn);
                                                    g[0] = len[i] * h[0] - m->cage_strain * nn[0] + m->efield[0];
                                                    g[1] = len[i] * h[1] - m->cage_strain * nn[1] + m->efield[1];
                                                    g[2] = len[i] * h[2] - m->cage_strain * nn[2] + m->efield[2];
                                                    dE = ((double)p[0] - px[i]) * g[0] + ((double)p[1] - py[i]) * g[1] +
                                                         ((double)p[2] - pz[i]) * g[2];
                                                    dE += k_term(m, p[0], p[1]) - k_term(m, px[i], py[i]);
                                                    thr = (u > 0.0f) ? -log((double)u) / beta : INFINITY;
                                                    margin = dE - thr;
                                                    acc = (dE < 0.0) || (exp(-beta * dE) > (double)u);
                                                    if (margin_out) margin_out[i] = margin;
                                                    if (gpu_after) {
                                                        const float *gx = gpu_after, *gy = gpu_after + N, *gz = gpu_after + 2 * N;
                                                        gacc = (gx[i] != px[i]) || (gy[i] != py[i]) || (gz[i] != pz[i]);
                                                        /* a proposal equal to the current dipole leaves the
                                                         * lattice unchanged either way: nothing to compare */
                                                        if (p[0] == px[i] && p[1] == py[i] && p[2] == pz[i]) gacc = acc;
                                                        if (gacc != acc) {
                                                            if (fabs(margin) <= tol) {
                                                                if (n_borderline) (*n_borderline)++;
                                                            } else {
                                                                if (n_hard) (*n_hard)++;
                                                            }
                                                            acc = gacc;
                                                        }
                                                        if (acc && (gx[i] != p[0] || gy[i] != p[1] || gz[i] != p[2])) {
                                                            /* GPU moved the site to something other than the proposal */
                                                            if (n_hard) (*n_hard)++;
                                                        }
                                                    }
                                                    if (acc) {
                                                        px[i] = p[0];
                                                        py[i] = p[1];
                                                        pz[i] = p[2];
                                                        n_acc++;
                                                        if (dE_sum) *dE_sum += dE;
                                                        if (accept_out) accept_out[i] = 1;
                                                    }
                                                }
                                    }
                        }
    tab64_free(&t);
    return n_acc;
}

double sno_energy64(const sno_model *m, const float *px, const float *py, const float *pz,
                    const float *len, double dipole, double *site_e, double *grad,
                    double *dparams, double *E_dd_out)
{
    tab64 t;
    double E = 0.0, E_dd = 0.0, E_cs = 0.0;
    double Psum[3] = {0.0, 0.0, 0.0};
    int x, y, z;
    if (!tab64_build(&t, m->cutoff, m->Z)) {
        tab64_free(&t);
        return NAN;
    }
    for (x = 0; x < m->X; x++)
        for (y = 0; y < m->Y; y++)
            for (z = 0; z < m->Z; z++) {
                long i = site_index(m, x, y, z);
                double h[3], nn[3], p[3], li = len[i];
                double dd, cs, fe, kk;
                field64(m, &t, px, py, pz, len, x, y, z, h, nn);
                p[0] = px[i];
                p[1] = py[i];
                p[2] = pz[i];
                dd = li * (p[0] * h[0] + p[1] * h[1] + p[2] * h[2]);
                cs = -m->cage_strain * (p[0] * nn[0] + p[1] * nn[1] + p[2] * nn[2]);
                fe = p[0] * m->efield[0] + p[1] * m->efield[1] + p[2] * m->efield[2];
                kk = k_term(m, p[0], p[1]);
                if (site_e) site_e[i] = dd + cs + fe + kk;
                if (grad) {
                    double sx = 0.0, sy = 0.0;
                    if (m->K > 0.0) {
                        sx = p[0] > 0 ? 1.0 : (p[0] < 0 ? -1.0 : 0.0);
                        sy = p[1] > 0 ? 1.0 : (p[1] < 0 ? -1.0 : 0.0);
                    }
                    grad[3 * i + 0] = li * h[0] - m->cage_strain * nn[0] + m->efield[0] - m->K * sx * (m->K > 0.0);
                    grad[3 * i + 1] = li * h[1] - m->cage_strain * nn[1] + m->efield[1] - m->K * sy * (m->K > 0.0);
                    grad[3 * i + 2] = li * h[2] - m->cage_strain * nn[2] + m->efield[2];
                }
                E_dd += 0.5 * dd;
                E_cs += 0.5 * cs;
                E += 0.5 * dd + 0.5 * cs + fe + kk;
                Psum[0] += p[0];
                Psum[1] += p[1];
                Psum[2] += p[2];
            }
    if (dparams) {
        dparams[0] = dipole != 0.0 ? 2.0 * E_dd / dipole : 0.0;
        dparams[1] = m->cage_strain != 0.0 ? E_cs / m->cage_strain : 0.0;
        dparams[2] = Psum[0];
        dparams[3] = Psum[1];
        dparams[4] = Psum[2];
        if (m->cage_strain == 0.0) {
            /* dE/dC = -1/2 sum_i p_i . nn_i, evaluated directly */
            double s = 0.0;
            for (x = 0; x < m->X; x++)
                for (y = 0; y < m->Y; y++)
                    for (z = 0; z < m->Z; z++) {
                        long i = site_index(m, x, y, z);
                        double h[3], nn[3];
                        field64(m, &t, px, py, pz, len, x, y, z, h, nn);
                        s += px[i] * nn[0] + py[i] * nn[1] + pz[i] * nn[2];
                    }
            dparams[1] = -0.5 * s;
        }
    }
    if (E_dd_out) *E_dd_out = E_dd;
    tab64_free(&t);
    return E;
}

/* ------------------------------------------------------------------------ */
/* Analysis maps and order parameters (src/starrynight-analysis.c).          */

/* dot() of src/starrynight-config.c:189-199: float sum from 0, x then y then z */
static float an_dot(float ax, float ay, float az, float bx, float by, float bz)
{
    float s = 0.0f;
    s += ax * bx;
    s += ay * by;
    s += az * bz;
    return s;
}

static long an_wrap(int v, int L)
{
    v %= L;
    return v < 0 ? v + L : v;
}

/* dipole_potential, src/starrynight-analysis.c:65-94 */
void sno_potential_map(const float *px, const float *py, const float *pz, const float *len, int X, int Y, int Z,
                       int cutoff, double *out)
{
    int x, y, z, dx, dy, dz;
    for (x = 0; x < X; x++)
        for (y = 0; y < Y; y++)
            for (z = 0; z < Z; z++) {
                double pot = 0.0;
                for (dx = -cutoff; dx <= cutoff; dx++)
                    for (dy = -cutoff; dy <= cutoff; dy++)
                        for (dz = -cutoff; dz <= cutoff; dz++) {
                            float rx, ry, rz, d, term;
                            long j;
                            if (dx == 0 && dy == 0 && dz == 0) continue;
                            rx = (float)dx;
                            ry = (float)dy;
                            rz = (float)dz;
                            d = (float)sqrt((double)(rx * rx + ry * ry + rz * rz));
                            if (d > (float)cutoff) continue;
                            j = (an_wrap(x + dx, X) * Y + an_wrap(y + dy, Y)) * Z + an_wrap(z + dz, Z);
                            term = len[j] * an_dot(px[j], py[j], pz[j], rx, ry, rz) / (d * d * d);
                            pot += term;
                        }
                out[((long)x * Y + y) * Z + z] = pot;
            }
}

/* dipole_electricfield (half = 0), :393-450, and dipole_electricfieldoffset
 * (half = 1), :310-380; returns |E| = sqrt(dot(E, E)) per site. */
void sno_efield_map(const float *px, const float *py, const float *pz, int X, int Y, int Z, int cutoff, int half,
                    double *out)
{
    const int lo = half ? -cutoff - 1 : -cutoff, hi = half ? cutoff - 1 : cutoff;
    int x, y, z, dx, dy, dz;
    for (x = 0; x < X; x++)
        for (y = 0; y < Y; y++)
            for (z = 0; z < Z; z++) {
                const long i = ((long)x * Y + y) * Z + z;
                float ex = 0.0f, ey = 0.0f, ez = 0.0f;
                for (dx = lo; dx <= hi; dx++)
                    for (dy = lo; dy <= hi; dy++)
                        for (dz = lo; dz <= hi; dz++) {
                            float rx, ry, rz, d, nx, ny, nz, cx, cy, cz;
                            double radial;
                            long j;
                            if (!half && dx == 0 && dy == 0 && dz == 0) continue;
                            if (half) {
                                rx = (float)dx + 0.5;
                                ry = (float)dy + 0.5;
                                rz = (float)dz + 0.5;
                            } else {
                                rx = (float)dx;
                                ry = (float)dy;
                                rz = (float)dz;
                            }
                            d = (float)sqrt((double)(rx * rx + ry * ry + rz * rz));
                            if (d > (float)cutoff) continue;
                            nx = rx / d;
                            ny = ry / d;
                            nz = rz / d;
                            j = (an_wrap(x + dx, X) * Y + an_wrap(y + dy, Y)) * Z + an_wrap(z + dz, Z);
                            radial = an_dot(nx, ny, nz, px[j], py[j], pz[j]);
                            cx = 3 * nx * radial - px[j];
                            cy = 3 * ny * radial - py[j];
                            cz = 3 * nz * radial - pz[j];
                            cx /= d * d * d;
                            cy /= d * d * d;
                            cz /= d * d * d;
                            ex += cx;
                            ey += cy;
                            ez += cz;
                        }
                if (!half) {
                    ex -= 1 / 3.0 * px[i];
                    ey -= 1 / 3.0 * py[i];
                    ez -= 1 / 3.0 * pz[i];
                }
                out[i] = sqrt(an_dot(ex, ey, ez, ex, ey, ez));
            }
}

/* radial_order_parameter, :528-598; arrays of cutoff^2+1.  Bin sums in FP64,
 * or with float_sums in float in the reference's order (its own histogram
 * arithmetic, :576-577), returned as doubles. */
#define SNO_MAX_BINS 1025
void sno_radial_order(const float *px, const float *py, const float *pz, int X, int Y, int Z, int cutoff,
                      int float_sums, double *fe, double *afe, long long *count)
{
    const int nb = cutoff * cutoff + 1;
    static float ffe[SNO_MAX_BINS], fafe[SNO_MAX_BINS];
    int x, y, z, dx, dy, dz, b;
    if (nb > SNO_MAX_BINS) return;
    for (b = 0; b < nb; b++) {
        fe[b] = afe[b] = 0.0;
        ffe[b] = fafe[b] = 0.0f;
        count[b] = 0;
    }
    for (x = 0; x < X; x++)
        for (y = 0; y < Y; y++)
            for (z = 0; z < Z; z++) {
                const long i = ((long)x * Y + y) * Z + z;
                for (dx = -cutoff; dx <= cutoff; dx++)
                    for (dy = -cutoff; dy <= cutoff; dy++)
                        for (dz = -cutoff; dz <= cutoff; dz++) {
                            const int ds = dx * dx + dy * dy + dz * dz;
                            float c, a, d, nx, ny, nz;
                            long j;
                            if (ds > cutoff * cutoff) continue;
                            j = (an_wrap(x + dx, X) * Y + an_wrap(y + dy, Y)) * Z + an_wrap(z + dz, Z);
                            c = an_dot(px[i], py[i], pz[i], px[j], py[j], pz[j]);
                            d = (float)sqrt((double)((float)dx * dx + dy * dy + dz * dz));
                            if (d == 0) d = 1;
                            nx = (float)dx / d;
                            ny = (float)dy / d;
                            nz = (float)dz / d;
                            a = c - 3 * an_dot(nx, ny, nz, px[i], py[i], pz[i]) * an_dot(nx, ny, nz, px[j], py[j], pz[j]);
                            if (float_sums) {
                                ffe[ds] += c;
                                fafe[ds] += a;
                            } else {
                                fe[ds] += c;
                                afe[ds] += a;
                            }
                            count[ds]++;
                        }
            }
    if (float_sums)
        for (b = 0; b < nb; b++) {
            fe[b] = ffe[b];
            afe[b] = fafe[b];
        }
}

/* polarisation() (:48-62) and landau_order() (:506-526), in FP64 */
void sno_order_params(const float *px, const float *py, const float *pz, long long n, double *pol_x,
                      double *landau, double *sum3)
{
    double s[3] = {0.0, 0.0, 0.0};
    long long k;
    for (k = 0; k < n; k++) {
        s[0] += px[k];
        s[1] += py[k];
        s[2] += pz[k];
    }
    if (pol_x) *pol_x = s[0] / (double)n;
    if (landau) *landau = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
    if (sum3) {
        sum3[0] = s[0];
        sum3[1] = s[1];
        sum3[2] = s[2];
    }
}
