/*
 * sn_io.h -- the reference program's output formats and a checkpoint format,
 * as a host-only C library (starrynight_gb300/lib/libsn_io.so).
 *
 * The reference writes its analysis files from the global lattice inside
 * src/starrynight-analysis.c; here each writer takes the data as arguments
 * (host arrays, index (x*Y+y)*Z+z, xyz interleaved as x,y,z per site), so a
 * host can write them from what sn_gpu_download_lattice, sn_gpu_potential,
 * sn_gpu_efield and sn_gpu_radial_order return.  Given the same values the
 * files are byte-identical to the reference's.  Every function returns 0 on
 * success and -1 when the file cannot be opened or written.
 */
#ifndef SN_IO_H
#define SN_IO_H

#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* outputlattice_xyz (src/starrynight-analysis.c:710-728): a C and an N atom per site. */
int sn_io_write_dipoles_xyz(const char *path, int X, int Y, int Z, const float *xyz);

/* outputlattice_ppm_hsv (:620-673): binary PPM of the z = 0 plane, hue from the in-plane angle. */
int sn_io_write_dipoles_ppm(const char *path, int X, int Y, int Z, const float *xyz);

/* outputlattice_svg (:675-708): one line per site of the z = 0 plane. */
int sn_io_write_dipoles_svg(const char *path, int X, int Y, int Z, const float *xyz);

/* lattice_potential_XYZ (:264-278): "x y z pot" per site. */
int sn_io_write_potential_xyz(const char *path, int X, int Y, int Z, const double *pot);

/* lattice_potential_cube (:280-308): Gaussian cube file of the potential map. */
int sn_io_write_potential_cube(const char *path, int X, int Y, int Z, const double *pot);

/* outputpotential_png (:481-504): plain-text greymap (PGM "P2") of the z = 0 plane. */
int sn_io_write_potential_pgm(const char *path, int X, int Y, int Z, const double *pot);

/* lattice_Efield_XYZ (:468-479) / lattice_Efieldoffset_XYZ (:379-391): "x y z |E|" per site. */
int sn_io_write_field_xyz(const char *path, int X, int Y, int Z, const double *magnitude);

/* The output half of radial_order_parameter (:528-600): appends the header, one
 * line per bin b < cutoff^2 with count[b] > 0 (means fe_sum/count,
 * afe_sum/count) and a blank line.  T is printed as an integer. */
int sn_io_append_rdf(const char *path, int cutoff, const double *fe_sum, const double *afe_sum,
                     const int64_t *count, int T);

/* recombination_calculator (:97-230) from a potential map: writes the two
 * log lines to log and, when art is not NULL, the density pictures of the
 * z = 0 plane to art. */
int sn_io_recombination(FILE *log, FILE *art, int X, int Y, int Z, const double *pot, int T);

/* outputlattice_dumb_terminal (:820-925): coloured arrows and potential of
 * the z = 0 plane (len may be NULL: no vacancies).  *dmax, when not NULL,
 * receives the colour scale used (the reference's global DMAX). */
int sn_io_dumb_terminal(FILE *out, int X, int Y, int Z, const float *xyz, const float *len, const double *pot,
                        int T, float *dmax);

/* ---- checkpoint / resume (no counterpart in the reference) ----
 * One replica: its lattice, the sweep counter that keys the sweep's random
 * stream, its Philox key, temperature and field.  Resuming from a checkpoint
 * (upload the lattice, sn_gpu_set_sweep_count, same seed) continues the run
 * exactly as if it had not stopped.  The file is little-endian with a
 * 64-bit FNV-1a checksum; sn_io_read_checkpoint returns -2 for a file that is
 * not a checkpoint or fails the checksum, and -3 when xyz/len are given but
 * the lattice size differs from hdr->X/Y/Z as passed in (set them to 0 to
 * accept any size; a NULL xyz reads the header only). */
typedef struct {
    int32_t X, Y, Z;
    int32_t cutoff;
    uint64_t sweeps;
    uint64_t seed;
    double T;
    double efield[3];
    uint64_t accept, attempt;
} sn_checkpoint;

int sn_io_write_checkpoint(const char *path, const sn_checkpoint *hdr, const float *xyz, const float *len);
int sn_io_read_checkpoint(const char *path, sn_checkpoint *hdr, float *xyz, float *len);

#ifdef __cplusplus
}
#endif
#endif
