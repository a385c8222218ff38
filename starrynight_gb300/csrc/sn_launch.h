// sn_launch.h -- host-side entry points of the kernels, one set per cutoff
// (sn_sweep_inst.cu is compiled once per cutoff with -DSN_RC=<rc>) plus the
// small kernels of sn_kernels.cu.
#pragma once

#include <cuda_runtime.h>

#include "sn_internal.h"

namespace sn_sweep {
struct SnFieldArgs;
}

struct SnFieldArgsHost;

typedef cudaError_t (*sn_sweep_launch_fn)(bool two_d, bool mixed, bool cached, const SnPhaseArgs &a, int grid,
                                          int threads, int smem, cudaStream_t st);
typedef cudaError_t (*sn_field_launch_fn)(bool fp64, bool two_d, bool mixed, const void *field_args, int grid,
                                          int threads, int smem, cudaStream_t st);
typedef void (*sn_geo_fn)(bool two_d, int *S, int *SZ, int *NS, int *NF, int *merge);
typedef cudaError_t (*sn_flow_launch_fn)(bool two_d, bool mixed, bool cached, const SnFlowArgs &a, int grid,
                                         int threads, int smem, cudaStream_t st, int *max_grid);
typedef int (*sn_cached_smem_fn)(int cslots, int tg, int pc, bool mixed, int ng);
typedef cudaError_t (*sn_gfield_launch_fn)(bool mixed, const void *field_args, int grid, int smem, cudaStream_t st);

#define SN_DECLARE_RC(N)                                                                                     \
    cudaError_t sn_launch_sweep_rc##N(bool, bool, bool, const SnPhaseArgs &, int, int, int, cudaStream_t);  \
    cudaError_t sn_launch_flow_rc##N(bool, bool, bool, const SnFlowArgs &, int, int, int, cudaStream_t,     \
                                     int *);                                                               \
    int sn_cached_smem_rc##N(int, int, int, bool, int);                                                         \
    cudaError_t sn_launch_gfield_rc##N(bool, const void *, int, int, cudaStream_t);                        \
    cudaError_t sn_launch_field_rc##N(bool, bool, bool, const void *, int, int, int, cudaStream_t);        \
    cudaError_t sn_launch_field64_rc##N(bool, bool, const void *, int, int, int, cudaStream_t);            \
    void sn_geo_rc##N(bool, int *, int *, int *, int *, int *);
SN_DECLARE_RC(1)
SN_DECLARE_RC(2)
SN_DECLARE_RC(3)
SN_DECLARE_RC(4)
SN_DECLARE_RC(5)
SN_DECLARE_RC(6)

// Field-pass arguments as the host fills them (layout identical to
// sn_sweep::SnFieldArgs).
struct SnFieldArgsHost {
    const SnWork *work;
    const SnReplicaDev *reps;
    const SnTile *geoms;
    double cage;
    double K;
    double *site_e;
    float *grad;
    double *red;
    int red_stride;
    int write_g;
};

// Exchange bookkeeping on the device.
struct SnExchange {
    int every;
    int pad;
    unsigned long long attempted;
    unsigned long long accepted;
    uint32_t seed_lo, seed_hi;
};

struct SnInitArgs {
    float *px, *py, *pz, *len;
    long long n;
    int pattern;
    int dim;
    int n_species;
    float dipoles[10];
    float prevalence[10];
    uint32_t seed_lo, seed_hi;
};

cudaError_t sn_launch_init_lattice(const SnInitArgs &a, cudaStream_t st);

// Planner, field-pass launcher and error slot of sn_gpu.cu, for sn_noalloc.cu.
void sn_internal_set_error(const char *msg);
bool sn_internal_plan(int X, int Y, int Z, int rc, bool mixed, SnTile *out, char *why, size_t why_len);
cudaError_t sn_internal_field_launch(int rc, bool fp64, bool two_d, bool mixed, const SnFieldArgsHost &a, int grid,
                                     int threads, int smem, cudaStream_t st);
cudaError_t sn_launch_upload_convert(const float *stage_xyz, const float *stage_len, float *px, float *py, float *pz,
                                     float *len, long long n, float uniform_len, int mixed, float default_len,
                                     int *flags, cudaStream_t st);
cudaError_t sn_launch_download_convert(const float *px, const float *py, const float *pz, const float *len,
                                       float *stage_xyz, float *stage_len, long long n, cudaStream_t st);
// reps[r].out_xyz = out (nullptr: the sweep writes no copy), in stream order.
cudaError_t sn_launch_set_out(SnReplicaDev *reps, int r, float *out, cudaStream_t st);
cudaError_t sn_launch_sweep_end(SnAccum *acc, SnState *state, double *hist, SnReplicaDev *reps, int nrep,
                                uint32_t *sweep, SnExchange *ex, int *order, uint32_t *queues, cudaStream_t st);
cudaError_t sn_launch_recompute_finish(const double *red, SnState *state, const SnReplicaDev *reps, int rep,
                                       double cage, double *drift_max, int record, cudaStream_t st);
// The coming sweep's proposals of every replica with a proposal buffer
// (SnReplicaDev::prop); sms = multiprocessors of the device (grid sizing).
cudaError_t sn_launch_sweep_proposals(const SnReplicaDev *reps, int nrep, const uint32_t *sweep, int dim,
                                      int constrain, int sms, cudaStream_t st);
// *count += number of i < n with a[i] != b[i].
cudaError_t sn_launch_count_diff(const int *a, const int *b, long long n, unsigned long long *count, cudaStream_t st);
cudaError_t sn_launch_quench_step(float *px, float *py, float *pz, const float *len, const float *grad,
                                  long long n, float step, cudaStream_t st);
cudaError_t sn_launch_fma_peak(float *out, int blocks, int threads, int iters, cudaStream_t st);
cudaError_t sn_launch_philox_batch(const uint32_t *ctr, const uint32_t *key, uint32_t *out, int n, cudaStream_t st);
cudaError_t sn_launch_proposal_batch(const uint32_t *site, uint32_t sweep, uint32_t seed_lo, uint32_t seed_hi,
                                     int dim, int constrain, float *out4, int n, cudaStream_t st);

// ---- analysis stencils (sn_analysis.cu) ----

// One replica's lattice arrays (z fastest) as the analysis kernels read them.
struct SnLatticeView {
    const float *px, *py, *pz, *len;
    int X, Y, Z;
    long long n;
};

// One displacement of an analysis stencil, with the per-offset constants the
// reference computes on the fly: a = r (potential) or r/d (field, correlation),
// b = 3 r/d (field), d3 = d*d*d in float, bin = |r|^2 (correlation).
struct SnAnalysisOffset {
    int dx, dy, dz, bin;
    float a[3];
    float d3;
    float b[3];
    float pad;
};

cudaError_t sn_launch_potential(const SnLatticeView &L, const SnAnalysisOffset *off, int n_off, double *out,
                                cudaStream_t st);
cudaError_t sn_launch_efield(const SnLatticeView &L, const SnAnalysisOffset *off, int n_off, int self_term,
                             double *out, cudaStream_t st);
cudaError_t sn_launch_radial(const SnLatticeView &L, const SnAnalysisOffset *off, int n_off, int n_bins,
                             double *fe, double *afe, cudaStream_t st);
cudaError_t sn_launch_orient_sum(const SnLatticeView &L, double *out3, cudaStream_t st);
