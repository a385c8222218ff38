/*
 * sn_io.c -- the reference program's analysis output formats, written from
 * caller-supplied arrays, and the checkpoint format (include/sn_io.h).
 *
 * Each writer follows the reference routine named beside it in
 * src/starrynight-analysis.c: the same format strings, the same traversal
 * order and the same float/double types in the arithmetic that feeds the
 * printed numbers, so the same input values give byte-identical files.
 * Index (x*Y+y)*Z+z throughout; xyz holds x,y,z per site.
 */
#include "sn_io.h"

#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static size_t site(int Y, int Z, int x, int y, int z) { return ((size_t)x * Y + y) * Z + z; }

static int finish(FILE *fo)
{
    int bad = ferror(fo);
    if (fclose(fo) != 0) bad = 1;
    return bad ? -1 : 0;
}

/* outputlattice_xyz, src/starrynight-analysis.c:710-728 */
int sn_io_write_dipoles_xyz(const char *path, int X, int Y, int Z, const float *xyz)
{
    const float r = 1.6 / 2, d = 4.0;
    const double zscale = 5.0;
    int x, y, z;
    FILE *fo = fopen(path, "w");
    if (!fo) return -1;
    fprintf(fo, "%d\n\n", X * Y * Z * 2);
    for (x = 0; x < X; x++)
        for (y = 0; y < Y; y++)
            for (z = 0; z < Z; z++) {
                const float *p = xyz + 3 * site(Y, Z, x, y, z);
                fprintf(fo, "C %f %f %f\n", d * x + r * p[0], d * y + r * p[1], zscale * (d * z) + r * p[2]);
                fprintf(fo, "N %f %f %f\n", d * x - r * p[0], d * y - r * p[1], zscale * (d * z) - r * p[2]);
            }
    return finish(fo);
}

/* outputlattice_ppm_hsv, :620-673: hue = pi + atan2(y, x), value and
 * saturation from z, black for zero vectors; one RGB byte triple per site of
 * the z = 0 plane in x-major order. */
int sn_io_write_dipoles_ppm(const char *path, int X, int Y, int Z, const float *xyz)
{
    float r = 0.0f, g = 0.0f, b = 0.0f, h, s, v, p, t, q, f;
    int i, k, hp;
    FILE *fo = fopen(path, "w");
    if (!fo) return -1;
    fprintf(fo, "P6\n%d %d\n255\n", X, Y);
    for (i = 0; i < X; i++)
        for (k = 0; k < Y; k++) {
            const float *d = xyz + 3 * site(Y, Z, i, k, 0);
            h = M_PI + atan2(d[1], d[0]);
            v = 0.5 + 0.4 * d[2];
            s = 0.6 - 0.6 * fabs(d[2]);
            hp = (int)floor(h / (M_PI / 3.0));
            f = h / (M_PI / 3.0) - (float)hp;
            p = v * (1.0 - s);
            q = v * (1.0 - f * s);
            t = v * (1.0 - (1.0 - f) * s);
            switch (hp) { /* hp = 6 (h = 2 pi) keeps the previous colour, as in the reference */
            case 0: r = v; g = t; b = p; break;
            case 1: r = q; g = v; b = p; break;
            case 2: r = p; g = v; b = t; break;
            case 3: r = p; g = q; b = v; break;
            case 4: r = t; g = p; b = v; break;
            case 5: r = v; g = p; b = q; break;
            }
            if (d[0] == 0.0 && d[1] == 0.0 && d[2] == 0.0) r = g = b = 0.0f;
            fputc((unsigned char)(int)(254.0 * r), fo);
            fputc((unsigned char)(int)(254.0 * g), fo);
            fputc((unsigned char)(int)(254.0 * b), fo);
        }
    return finish(fo);
}

/* outputlattice_svg, :675-708: x and y swapped so it overlays the PPM */
int sn_io_write_dipoles_svg(const char *path, int X, int Y, int Z, const float *xyz)
{
    int x, y;
    FILE *fo = fopen(path, "w");
    if (!fo) return -1;
    fprintf(fo, "<svg xmlns=\"http://www.w3.org/2000/svg\" version=\"1.1\" height=\"%d\" width=\"%d\">\n", X, Y);
    fprintf(fo, " <marker id=\"triangle\" viewBox=\"0 0 10 10\" refX=\"7\" refY=\"5\" markerUnits=\"strokeWidth\" "
                "markerWidth=\"2\" markerHeight=\"2\" orient=\"auto\"><path d=\"M 0 0 L 10 5 L 0 10 z\" /></marker>\n");
    for (x = 0; x < X; x++)
        for (y = 0; y < Y; y++) {
            const float *d = xyz + 3 * site(Y, Z, x, y, 0);
            const int grey = (int)((-d[2] + 1.0) * 127.0);
            fprintf(fo,
                    " <line x1=\"%f\" y1=\"%f\" x2=\"%f\" y2=\"%f\" style=\"stroke:rgb(%d,%d,%d);stroke-width:0.17\" "
                    "marker-end=\"url(#triangle)\" />\n",
                    y + 0.5 + 0.4 * d[1], x + 0.5 + 0.4 * d[0], y + 0.5 - 0.4 * d[1], x + 0.5 - 0.4 * d[0], grey, grey,
                    grey);
        }
    fprintf(fo, "</svg>\n");
    return finish(fo);
}

/* lattice_potential_XYZ, :264-278 */
int sn_io_write_potential_xyz(const char *path, int X, int Y, int Z, const double *pot)
{
    int x, y, z;
    FILE *fo = fopen(path, "w");
    if (!fo) return -1;
    for (x = 0; x < X; x++)
        for (y = 0; y < Y; y++)
            for (z = 0; z < Z; z++) fprintf(fo, "%d %d %d %f\n", x, y, z, pot[site(Y, Z, x, y, z)]);
    return finish(fo);
}

/* lattice_potential_cube, :280-308: unit voxels, one dummy atom at the origin,
 * six values per line and a line break after every (x, y) column */
int sn_io_write_potential_cube(const char *path, int X, int Y, int Z, const double *pot)
{
    int x, y, z;
    FILE *fo = fopen(path, "w");
    if (!fo) return -1;
    fprintf(fo, "Starrynight Cube file: %d %d %d\n\n", X, Y, Z);
    fprintf(fo, "1 0.0 0.0 0.0\n");
    fprintf(fo, "%d 1.0 0.0 0.0\n", X);
    fprintf(fo, "%d 0.0 1.0 0.0\n", Y);
    fprintf(fo, "%d 0.0 0.0 1.0\n", Z);
    fprintf(fo, "1 0.0 0.0 0.0 0.0 0.0\n");
    for (x = 0; x < X; x++)
        for (y = 0; y < Y; y++) {
            for (z = 0; z < Z; z++) {
                fprintf(fo, "%g ", pot[site(Y, Z, x, y, z)]);
                if (z % 6 == 5) fprintf(fo, "\n");
            }
            fprintf(fo, "\n");
        }
    return finish(fo);
}

/* outputpotential_png, :481-504 (a text greymap despite the name) */
int sn_io_write_potential_pgm(const char *path, int X, int Y, int Z, const double *pot)
{
    int i, k, pixel;
    FILE *fo = fopen(path, "w");
    if (!fo) return -1;
    fprintf(fo, "P2\n%d %d\n%d\n", X, Y, SHRT_MAX);
    for (i = 0; i < X; i++) {
        for (k = 0; k < Y; k++) {
            pixel = SHRT_MAX / 2 + (int)(SHRT_MAX * 0.1 * pot[site(Y, Z, i, k, 0)]);
            if (pixel < 0) pixel = 0;
            if (pixel > SHRT_MAX) pixel = SHRT_MAX;
            fprintf(fo, "%d ", pixel);
        }
        fprintf(fo, "\n");
    }
    return finish(fo);
}

/* lattice_Efield_XYZ, :468-479, and lattice_Efieldoffset_XYZ, :379-391 */
int sn_io_write_field_xyz(const char *path, int X, int Y, int Z, const double *magnitude)
{
    int x, y, z;
    FILE *fo = fopen(path, "w");
    if (!fo) return -1;
    for (x = 0; x < X; x++)
        for (y = 0; y < Y; y++)
            for (z = 0; z < Z; z++) fprintf(fo, "%d %d %d %f\n", x, y, z, magnitude[site(Y, Z, x, y, z)]);
    return finish(fo);
}

/* output of radial_order_parameter, :581-597: float means per bin, bins
 * 0 .. cutoff^2 - 1 (the last bin, |r|^2 = cutoff^2, is not printed) */
int sn_io_append_rdf(const char *path, int cutoff, const double *fe_sum, const double *afe_sum,
                     const int64_t *count, int T)
{
    int i;
    FILE *fo = fopen(path, "a");
    if (!fo) return -1;
    fprintf(fo, "# r^2 r orientational_FE_correlation[r^2] orientational_AFE_correlation[r^2] "
                "orientational_count[r^2] T\n");
    for (i = 0; i < cutoff * cutoff; i++) {
        if (count[i] > 0) {
            const float fe = (float)(fe_sum[i] / (double)count[i]);
            const float afe = (float)(afe_sum[i] / (double)count[i]);
            fprintf(fo, "%d %f %f %f %d %d\n", i, sqrt(i), fe, afe, (int)count[i], T);
        }
    }
    fprintf(fo, "\n");
    return finish(fo);
}

/* recombination_calculator, :97-230: Boltzmann and Fermi-Dirac partition
 * functions of electrons and holes in the potential (scaled by 0.165/5 eV at
 * kT = 25 meV), the Fermi-Dirac densities and their overlap. */
int sn_io_recombination(FILE *log, FILE *art, int X, int Y, int Z, const double *pot, int T)
{
    const double BETA = 1 / (0.025);
    const double potentialeV = 0.165 / 5;
    const size_t N = (size_t)X * Y * Z;
    const double N2 = (double)((long long)N * (long long)N);
    double ZBe = 0.0, ZBh = 0.0, ZFDe = 0.0, ZFDh = 0.0;
    double eMAX = 0.0, hMAX = 0.0, RMAX = 0.0, e_total = 0.0, h_total = 0.0, r_total = 0.0;
    double *el = NULL, *ho = NULL;
    size_t k;
    int x, y;
    if (!log) return -1;
    for (k = 0; k < N; k++) {
        const double p = potentialeV * pot[k];
        ZBe += exp(-p * BETA);
        ZBh += exp(p * BETA);
        ZFDe += 1.0 / (exp(p * BETA) + 1.0);
        ZFDh += 1.0 / (exp(-p * BETA) + 1.0);
    }
    fprintf(log, "T: %d ZBe: %e ZBh: %e ZFDe: %e ZFDh: %e R_Boltz: %e ", T, ZBe, ZBh, ZFDe, ZFDh, N2 / (ZBe * ZBh));
    el = (double *)malloc(2 * (size_t)X * Y * sizeof(double));
    if (!el) return -1;
    ho = el + (size_t)X * Y;
    for (k = 0; k < N; k++) {
        const double p = potentialeV * pot[k];
        const double e = 1.0 / (exp(p * BETA) + 1.0) / ZFDe;
        const double h = 1.0 / (exp(-p * BETA) + 1.0) / ZFDh;
        if (k % Z == 0) { /* the z = 0 plane feeds the maxima and the pictures */
            el[k / Z] = e;
            ho[k / Z] = h;
            if (e > eMAX) eMAX = e;
            if (h > hMAX) hMAX = h;
            if (e * h > RMAX) RMAX = e * h;
        }
        e_total += e;
        h_total += h;
        r_total += e * h;
    }
    fprintf(log, "R_FD: %e FD-Total-electron: %e FD-Total-hole: %e\n", (double)N * r_total, e_total, h_total);
    fflush(log);
    if (art) {
        fprintf(art, "%*s%*s\n", X + 3, "ELECTRONS", (2 * X) + 4, "HOLES");
        fprintf(art, "Density eMAX: %f hMAX: %f\n", eMAX, hMAX);
        for (y = 0; y < Y; y++) {
            for (x = 0; x < X; x++) {
                const double e = el[(size_t)x * Y + y];
                fprintf(art, "%c[48;5;%d", 27, 232 + (int)(23.0 / eMAX * e));
                fprintf(art, "m%c%c%c[0m", (int)(10.0 / eMAX * e) + '0', '.', 27);
            }
            fprintf(art, "    ");
            for (x = 0; x < X; x++) {
                const double h = ho[(size_t)x * Y + y];
                fprintf(art, "%c[48;5;%d", 27, 232 + (int)(23.0 / hMAX * h));
                fprintf(art, "m%c%c%c[0m", (int)(10.0 / hMAX * h) + '0', '.', 27);
            }
            fprintf(art, "\n");
        }
        fprintf(art, "RMAX: %e\n", RMAX);
        fprintf(art, "%*s\n", 2 + X + X + X, "<<< RECOMBINATION <<<");
        for (y = 0; y < Y; y++) {
            fprintf(art, "%*s", 2 + X, " ");
            for (x = 0; x < X; x++) {
                const double r = el[(size_t)x * Y + y] * ho[(size_t)x * Y + y];
                fprintf(art, "%c[48;5;%d", 27, 232 + (int)(23.0 * r / RMAX));
                fprintf(art, "m%c%c%c[0m", (int)(10.0 * r / RMAX) + '0', '.', 27);
            }
            fprintf(art, "\n");
        }
        fprintf(art, "T: %d ZBe: %e ZBh: %e ZFDe: %e ZFDh: %e R_Boltz: %e \n", T, ZBe, ZBh, ZFDe, ZFDh,
                N2 / (ZBe * ZBh));
        fprintf(art, "R_FD: %e FD-Total-electron: %e FD-Total-hole: %e\n", (double)N * r_total, e_total, h_total);
    }
    free(el);
    return ferror(log) ? -1 : 0;
}

/* outputlattice_dumb_terminal, :820-925: one character cell per site of the
 * z = 0 plane, arrow and colour from the in-plane angle ('o' / 'x' out of the
 * plane, '#' for vacancies), then the potential as grey levels and digits. */
int sn_io_dumb_terminal(FILE *out, int X, int Y, int Z, const float *xyz, const float *len, const double *pot,
                        int T, float *dmax)
{
    const char *arrows = "-\\|/-\\|/";
    const char *density = "012345689";
    float new_dmax = 0.0f, potential, variance = 0.0f, mean = 0.0f, a, DMAX;
    int x, y;
    if (!out) return -1;
    fprintf(out, "%*s%*s\n", X + 3, "DIPOLES", (2 * X) + 4, "POTENTIAL");
    for (y = 0; y < Y; y++)
        for (x = 0; x < X; x++) {
            potential = pot[site(Y, Z, x, y, 0)];
            if (fabs(potential) > new_dmax) new_dmax = fabs(potential);
        }
    DMAX = new_dmax;
    for (y = 0; y < Y; y++) {
        for (x = 0; x < X; x++) {
            const size_t k = site(Y, Z, x, y, 0);
            const float *p = xyz + 3 * k;
            const int vacant = len ? len[k] == 0.0f : 0;
            char arrow;
            a = atan2(p[1], p[0]);
            a = a / (M_PI);
            a = a + 1.0;
            a = a + 0.125;
            if (a > 2.0) a = a - 2.0;
            a *= 4;
            if (vacant) a = 7;
            fprintf(out, "%c[%d", 27, 31 + ((int)a) % 8);
            if (a < 4.0) fprintf(out, ";7");
            arrow = arrows[(int)a];
            if (p[2] > sqrt(2) / 2.0) arrow = 'o';
            if (p[2] < -sqrt(2) / 2.0) arrow = 'x';
            if (vacant) arrow = '#';
            fprintf(out, "m%c %c[0m", arrow, 27);
            fprintf(out, "%c[37m%c[0m", 27, 27);
        }
        fprintf(out, "    ");
        for (x = 0; x < X; x++) {
            const float *p = xyz + 3 * site(Y, Z, x, y, 0);
            char arrow;
            potential = pot[site(Y, Z, x, y, 0)];
            variance += potential * potential;
            mean += potential;
            if (fabs(potential) > new_dmax) new_dmax = fabs(potential);
            /* an all-zero plane gives DMAX = 0: level 0 instead of a division by zero */
            fprintf(out, "%c[48;5;%d", 27, 232 + 12 + (DMAX > 0.0f ? (int)(11.0 * potential / DMAX) : 0));
            a = atan2(p[1], p[0]);
            a = a / (M_PI);
            a = a + 1.0;
            a = a + 0.125;
            if (a > 2.0) a = a - 2.0;
            a *= 4;
            arrow = arrows[(int)a];
            if (p[2] > sqrt(2) / 2.0) arrow = 'o';
            if (p[2] < -sqrt(2) / 2.0) arrow = 'x';
            fprintf(out, "m%c%c%c[0m", density[DMAX > 0.0f ? (int)(8.0 * fabs(potential) / DMAX) : 0], arrow, 27);
        }
        fprintf(out, "\n");
    }
    mean = mean / (X * Y);
    variance = variance / (X * Y);
    fprintf(out, "T: %d DMAX: %f new_DMAX: %f variance: %f mean: %f\n", T, DMAX, new_dmax, variance, mean);
    if (dmax) *dmax = new_dmax;
    return ferror(out) ? -1 : 0;
}

/* ---- checkpoint ---- */

static const char kMagic[8] = {'S', 'N', 'C', 'K', 'P', 'T', '0', '1'};

typedef struct {
    FILE *f;
    uint64_t h;  /* FNV-1a 64 of every byte after the magic */
    int bad;
} ck_stream;

static void ck_bytes(ck_stream *s, const void *p, size_t n, int writing)
{
    unsigned char *b = (unsigned char *)p;
    size_t i;
    if (s->bad) return;
    if (writing ? fwrite(p, 1, n, s->f) != n : fread((void *)p, 1, n, s->f) != n) {
        s->bad = 1;
        return;
    }
    for (i = 0; i < n; i++) s->h = (s->h ^ b[i]) * 1099511628211ull;
}

/* little-endian integers and IEEE values regardless of the host's byte order */
static void ck_u64(ck_stream *s, uint64_t *v, int writing)
{
    unsigned char b[8] = {0};
    int i;
    if (writing)
        for (i = 0; i < 8; i++) b[i] = (unsigned char)(*v >> (8 * i));
    ck_bytes(s, b, 8, writing);
    if (!writing) {
        *v = 0;
        for (i = 0; i < 8; i++) *v |= (uint64_t)b[i] << (8 * i);
    }
}

static void ck_i32(ck_stream *s, int32_t *v, int writing)
{
    uint64_t u = (uint64_t)(uint32_t)*v;
    unsigned char b[4] = {0};
    int i;
    if (writing)
        for (i = 0; i < 4; i++) b[i] = (unsigned char)(u >> (8 * i));
    ck_bytes(s, b, 4, writing);
    if (!writing) {
        uint32_t w = 0;
        for (i = 0; i < 4; i++) w |= (uint32_t)b[i] << (8 * i);
        *v = (int32_t)w;
    }
}

static void ck_f64(ck_stream *s, double *v, int writing)
{
    uint64_t u;
    memcpy(&u, v, 8);
    ck_u64(s, &u, writing);
    if (!writing) memcpy(v, &u, 8);
}

static void ck_f32s(ck_stream *s, float *v, size_t n, int writing)
{
    size_t i;
    for (i = 0; i < n && !s->bad; i++) {
        uint32_t u;
        unsigned char b[4] = {0};
        int j;
        memcpy(&u, &v[i], 4);
        if (writing)
            for (j = 0; j < 4; j++) b[j] = (unsigned char)(u >> (8 * j));
        ck_bytes(s, b, 4, writing);
        if (!writing) {
            u = 0;
            for (j = 0; j < 4; j++) u |= (uint32_t)b[j] << (8 * j);
            memcpy(&v[i], &u, 4);
        }
    }
}

static void ck_header(ck_stream *s, sn_checkpoint *h, int writing)
{
    int c;
    ck_i32(s, &h->X, writing);
    ck_i32(s, &h->Y, writing);
    ck_i32(s, &h->Z, writing);
    ck_i32(s, &h->cutoff, writing);
    ck_u64(s, &h->sweeps, writing);
    ck_u64(s, &h->seed, writing);
    ck_f64(s, &h->T, writing);
    for (c = 0; c < 3; c++) ck_f64(s, &h->efield[c], writing);
    ck_u64(s, &h->accept, writing);
    ck_u64(s, &h->attempt, writing);
}

int sn_io_write_checkpoint(const char *path, const sn_checkpoint *hdr, const float *xyz, const float *len)
{
    ck_stream s;
    sn_checkpoint h = *hdr;
    size_t N;
    uint64_t sum;
    if (!xyz || !len || h.X < 1 || h.Y < 1 || h.Z < 1) return -1;
    N = (size_t)h.X * h.Y * h.Z;
    s.f = fopen(path, "wb");
    if (!s.f) return -1;
    s.h = 1469598103934665603ull;
    s.bad = fwrite(kMagic, 1, 8, s.f) != 8;
    ck_header(&s, &h, 1);
    ck_f32s(&s, (float *)xyz, 3 * N, 1);
    ck_f32s(&s, (float *)len, N, 1);
    sum = s.h;
    ck_u64(&s, &sum, 1);
    if (s.bad) {
        fclose(s.f);
        return -1;
    }
    return finish(s.f);
}

int sn_io_read_checkpoint(const char *path, sn_checkpoint *hdr, float *xyz, float *len)
{
    ck_stream s;
    sn_checkpoint h;
    char magic[8];
    uint64_t sum, want;
    size_t N;
    if (!hdr) return -1;
    s.f = fopen(path, "rb");
    if (!s.f) return -1;
    s.h = 1469598103934665603ull;
    s.bad = 0;
    if (fread(magic, 1, 8, s.f) != 8 || memcmp(magic, kMagic, 8) != 0) {
        fclose(s.f);
        return -2;
    }
    memset(&h, 0, sizeof(h));
    ck_header(&s, &h, 0);
    if (s.bad || h.X < 1 || h.Y < 1 || h.Z < 1) {
        fclose(s.f);
        return -2;
    }
    if (!xyz) {
        fclose(s.f);
        *hdr = h;
        return 0;
    }
    if ((hdr->X && hdr->X != h.X) || (hdr->Y && hdr->Y != h.Y) || (hdr->Z && hdr->Z != h.Z) || !len) {
        fclose(s.f);
        return -3;
    }
    N = (size_t)h.X * h.Y * h.Z;
    ck_f32s(&s, xyz, 3 * N, 0);
    ck_f32s(&s, len, N, 0);
    want = s.h;
    ck_u64(&s, &sum, 0);
    fclose(s.f);
    if (s.bad || sum != want) return -2;
    *hdr = h;
    return 0;
}
