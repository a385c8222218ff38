// sn_kernels.cu -- the small kernels around the sweep: lattice
// initialisation, host-layout conversion, the end-of-sweep fold with replica
// exchange, recompute bookkeeping and the quench step.
#include <algorithm>
#include <cmath>

#include "../../include/sn_gpu.h"
#include "sn_device.cuh"
#include "sn_launch.h"

namespace {

// initialise_lattice_random / _ferroelectric + solid_solution
// (src/starrynight-lattice.c:25-47, :139-171), drawn from Philox with
// counter (site, 0, k, SN_STREAM_INIT).  Draw 0 word 0 picks the species by
// walking the Prevalence list as solid_solution does; words 1,2 and later
// draws feed the same Marsaglia tries as the sweep proposal.  Vacancies hold
// the zero vector.
__global__ void init_lattice_kernel(const SnInitArgs a)
{
    const uint2 key = make_uint2(a.seed_lo, a.seed_hi);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < a.n;
         i += (long long)gridDim.x * blockDim.x) {
        uint4 r = sn_philox(make_uint4((uint32_t)i, 0u, 0u, SN_STREAM_INIT), key);
        float sample = sn_uniform24(r.x);
        int s = 0;
        while (s < a.n_species - 1 && sample > a.prevalence[s]) {
            sample = __fsub_rn(sample, a.prevalence[s]);
            s++;
        }
        const float L = a.dipoles[s];
        float3 p = make_float3(1.0f, 0.0f, 0.0f);
        if (a.pattern == SN_LATTICE_RANDOM) {
            bool ok = sn_try_point(r.y, r.z, a.dim, p);
            for (uint32_t k = 1; !ok && k < SN_PROPOSAL_MAX_DRAWS; k++) {
                r = sn_philox(make_uint4((uint32_t)i, 0u, k, SN_STREAM_INIT), key);
                ok = sn_try_point(r.x, r.y, a.dim, p) || sn_try_point(r.z, r.w, a.dim, p);
            }
            if (!ok) p = make_float3(0.0f, 0.0f, 1.0f);
        }
        if (L == 0.0f) p = make_float3(0.0f, 0.0f, 0.0f);
        a.px[i] = p.x;
        a.py[i] = p.y;
        a.pz[i] = p.z;
        a.len[i] = L;
    }
}

// flags[0]: a length that differs from the uniform length (uniform mode)
// flags[2]: a negative or non-finite length
// (an occupied site may hold any orientation, the zero vector included, as
// the reference's buckled and slab_delete patterns produce)
__global__ void upload_convert_kernel(const float *__restrict__ sxyz, const float *__restrict__ slen, float *px,
                                      float *py, float *pz, float *len, long long n, float uniform_len, int mixed,
                                      float default_len, int *flags)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        float x = sxyz[3 * i + 0], y = sxyz[3 * i + 1], z = sxyz[3 * i + 2];
        const float L = slen ? slen[i] : default_len;
        if (!(L >= 0.0f) || isinf(L)) atomicOr(&flags[2], 1);
        if (L == 0.0f) {
            x = y = z = 0.0f;
        } else {
            if (!mixed && L != uniform_len) atomicOr(&flags[0], 1);
            // the field cache's fixed-point range assumes unit (or shorter) dipole components
            if (!(fabsf(x) <= 1.0001f && fabsf(y) <= 1.0001f && fabsf(z) <= 1.0001f)) atomicOr(&flags[3], 1);
        }
        px[i] = x;
        py[i] = y;
        pz[i] = z;
        len[i] = L;
    }
}

__global__ void download_convert_kernel(const float *__restrict__ px, const float *__restrict__ py,
                                        const float *__restrict__ pz, const float *__restrict__ len, float *sxyz,
                                        float *slen, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        sxyz[3 * i + 0] = px[i];
        sxyz[3 * i + 1] = py[i];
        sxyz[3 * i + 2] = pz[i];
        if (slen) slen[i] = len[i];
    }
}

__global__ void set_out_kernel(SnReplicaDev *reps, int r, float *out)
{
    if (threadIdx.x == 0) reps[r].out_xyz = out;
}

// End of one sweep: fold the per-sweep accumulators into the running FP64
// totals, log E/site and |P|/site, advance the sweep counter and, when due,
// run one round of replica exchange between adjacent temperatures.
__global__ void sweep_end_kernel(SnAccum *acc, SnState *state, double *hist, SnReplicaDev *reps, int nrep,
                                 uint32_t *sweep, SnExchange *ex, int *order, uint32_t *queues)
{
    if (queues && threadIdx.x < 2) queues[threadIdx.x] = 0u;  // dataflow queues of the next sweep
    for (int r = threadIdx.x; r < nrep; r += blockDim.x) {
        SnState &s = state[r];
        SnAccum &A = acc[r];
        s.E += A.dE;
        s.P[0] += A.dP[0];
        s.P[1] += A.dP[1];
        s.P[2] += A.dP[2];
        s.acc_total += A.acc;
        s.att_total += A.att;
        A.dE = 0.0;
        A.dP[0] = A.dP[1] = A.dP[2] = 0.0;
        A.acc = 0ull;
        A.att = 0ull;
        const double N = (double)reps[r].n_sites;
        const double Pm = sqrt(s.P[0] * s.P[0] + s.P[1] * s.P[1] + s.P[2] * s.P[2]);
        double *hr = hist + 2 * ((size_t)r * SN_HIST_CAP + (size_t)(s.hist_head % SN_HIST_CAP));
        hr[0] = s.E / N;
        hr[1] = Pm / N;
        s.hist_head++;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t s = *sweep + 1u;
        if (ex->every > 0 && nrep > 1 && (s % (uint32_t)ex->every) == 0u) {
            const uint32_t round = s / (uint32_t)ex->every;
            const uint2 key = make_uint2(ex->seed_lo, ex->seed_hi);
            for (int k = (int)(round & 1u); k + 1 < nrep; k += 2) {
                const int ra = order[k], rb = order[k + 1];
                const double d = ((double)reps[ra].beta - (double)reps[rb].beta) * (state[ra].E - state[rb].E);
                const uint4 q = sn_philox(make_uint4((uint32_t)k, round, 0u, SN_STREAM_EXCHANGE), key);
                const double u = (double)sn_uniform24(q.x);
                ex->attempted++;
                if (d >= 0.0 || u < exp(d)) {
                    const float tb = reps[ra].beta, tt = reps[ra].T;
                    reps[ra].beta = reps[rb].beta;
                    reps[ra].T = reps[rb].T;
                    reps[rb].beta = tb;
                    reps[rb].T = tt;
                    order[k] = rb;
                    order[k + 1] = ra;
                    ex->accepted++;
                }
            }
        }
        *sweep = s;
    }
}

// red (10 doubles, see SnFieldArgs) -> running E and P of one replica.
__global__ void recompute_finish_kernel(const double *red, SnState *state, const SnReplicaDev *reps, int rep,
                                        double cage, double *drift_max, int record)
{
    const double E = red[0] - 0.5 * cage * red[1] + red[2] + red[3];
    SnState &s = state[rep];
    if (record) {
        const double d = fabs(s.E - E) / fmax(fabs(E), 1.0);
        if (d > drift_max[rep]) drift_max[rep] = d;
    }
    s.E = E;
    s.P[0] = red[4];
    s.P[1] = red[5];
    s.P[2] = red[6];
    (void)reps;
}

// One projected-gradient step on the sphere at every occupied site:
// p <- normalize(p - step (g - (g.p) p)).
__global__ void quench_step_kernel(float *px, float *py, float *pz, const float *__restrict__ len,
                                   const float *__restrict__ grad, long long n, float step)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        if (len[i] == 0.0f) continue;
        const float x = px[i], y = py[i], z = pz[i];
        const float gx = grad[3 * i], gy = grad[3 * i + 1], gz = grad[3 * i + 2];
        const float gp = gx * x + gy * y + gz * z;
        float nx = x - step * (gx - gp * x);
        float ny = y - step * (gy - gp * y);
        float nz = z - step * (gz - gp * z);
        const float inv = rsqrtf(nx * nx + ny * ny + nz * nz);
        px[i] = nx * inv;
        py[i] = ny * inv;
        pz[i] = nz * inv;
    }
}

__global__ void philox_batch_kernel(const uint32_t *ctr, const uint32_t *key, uint32_t *out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint4 r = sn_philox(make_uint4(ctr[4 * i], ctr[4 * i + 1], ctr[4 * i + 2], ctr[4 * i + 3]),
                              make_uint2(key[2 * i], key[2 * i + 1]));
    out[4 * i + 0] = r.x;
    out[4 * i + 1] = r.y;
    out[4 * i + 2] = r.z;
    out[4 * i + 3] = r.w;
}

__global__ void proposal_batch_kernel(const uint32_t *site, uint32_t sweep, uint2 key, int dim, int constrain,
                                      float *out4, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 p;
    float u;
    if (!sn_proposal(site[i], sweep, SN_STREAM_SWEEP, key, dim, constrain, p, u))
        p = make_float3(NAN, NAN, NAN);
    out4[4 * i + 0] = p.x;
    out4[4 * i + 1] = p.y;
    out4[4 * i + 2] = p.z;
    out4[4 * i + 3] = u;
}

// The proposals and accept thresholds of one sweep for every site of the
// replicas that use the cached-field sweep (blockIdx.y = replica; replicas
// without a proposal buffer are skipped): the move the sweep will attempt at
// each site depends only on (seed, sweep, site), so all of them are drawn
// here with full parallelism instead of inside the sweep's block schedule.
// Thresholds are -ln(u)/beta (accept iff dE < threshold); vacancies get -1.
// A proposal whose Marsaglia tries all fail keeps the old dipole.
//
// Lanes are kept busy by compaction: a warp takes a chunk of 256 sites,
// writes the vacancies at once and queues the occupied sites (warp ballot),
// draws the first try for 32 queued sites at a time, and queues the ~21 % of
// sites whose first try was rejected; those are redrawn 32 at a time, the
// remainder carried to the warp's next chunk.  Without it a warp pays for
// its vacant lanes and runs a second draw whenever any one lane needs it,
// which is almost always.
#define SN_PROP_CHUNK 256
#define SN_PROP_WARPS 8

__device__ __forceinline__ void proposal_retry_out(const SnReplicaDev &R, float4 *out, uint32_t site, float thr,
                                                   uint32_t sweep, uint2 key, int dim)
{
    float3 p;
    if (!sn_proposal_retry(site, sweep, SN_STREAM_SWEEP, key, dim, p))
        p = make_float3(R.px[site], R.py[site], R.pz[site]);
    out[site] = make_float4(p.x, p.y, p.z, thr);
}

__global__ void __launch_bounds__(SN_PROP_WARPS * 32, 4)
    sweep_proposals_kernel(const SnReplicaDev *reps, const uint32_t *sweep_ctr, int dim, int constrain)
{
    __shared__ uint32_t qsite[SN_PROP_WARPS][SN_PROP_CHUNK];
    __shared__ uint32_t fsite[SN_PROP_WARPS][SN_PROP_CHUNK + 32];
    __shared__ float fthr[SN_PROP_WARPS][SN_PROP_CHUNK + 32];
    const SnReplicaDev &R = reps[blockIdx.y];
    float4 *out = R.prop;
    if (!out) return;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const unsigned below = (1u << lane) - 1u;
    const uint32_t sweep = *sweep_ctr;
    const uint2 key = make_uint2(R.seed_lo, R.seed_hi);
    const float beta = R.beta;
    const long long n = R.n_sites;
    const float *__restrict__ len = R.len;
    uint32_t *q = qsite[wib], *fs = fsite[wib];
    float *ft = fthr[wib];
    int nf = 0;  // rejected first tries queued in fs/ft (warp-uniform)
    const long long stride = (long long)gridDim.x * SN_PROP_WARPS * SN_PROP_CHUNK;
    for (long long c0 = ((long long)blockIdx.x * SN_PROP_WARPS + wib) * SN_PROP_CHUNK; c0 < n; c0 += stride) {
        // 1. occupied sites of the chunk into q, in site order; vacancies written here
        float lv[SN_PROP_CHUNK / 32];
#pragma unroll
        for (int j = 0; j < SN_PROP_CHUNK / 32; j++) {
            const long long i = c0 + 32 * j + lane;
            lv[j] = i < n ? __ldg(len + i) : 0.0f;
        }
        int nq = 0;
#pragma unroll
        for (int j = 0; j < SN_PROP_CHUNK / 32; j++) {
            const long long i = c0 + 32 * j + lane;
            const bool occ = lv[j] != 0.0f;
            if (i < n && !occ) out[i] = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
            const unsigned m = __ballot_sync(0xffffffffu, occ);
            if (occ) q[nq + __popc(m & below)] = (uint32_t)i;
            nq += __popc(m);
        }
        __syncwarp();
        // 2. draw 0 for the queued sites, 64 at a time (two independent draws
        // per lane, interleaved by the compiler); rejected tries to fs/ft
        for (int b = 0; b < nq; b += 64) {
            const bool v1 = b + lane < nq, v2 = b + 32 + lane < nq;
            const uint32_t s1 = v1 ? q[b + lane] : 0u, s2 = v2 ? q[b + 32 + lane] : 0u;
            float3 p1, p2;
            float u1, u2;
            const bool ok1 = sn_proposal_first(s1, sweep, SN_STREAM_SWEEP, key, dim, constrain, p1, u1);
            const bool ok2 = sn_proposal_first(s2, sweep, SN_STREAM_SWEEP, key, dim, constrain, p2, u2);
            const float thr1 = u1 > 0.0f ? -logf(u1) / beta : INFINITY;
            const float thr2 = u2 > 0.0f ? -logf(u2) / beta : INFINITY;
            if (v1 && ok1) out[s1] = make_float4(p1.x, p1.y, p1.z, thr1);
            if (v2 && ok2) out[s2] = make_float4(p2.x, p2.y, p2.z, thr2);
            const bool r1 = v1 && !ok1, r2 = v2 && !ok2;
            const unsigned m1 = __ballot_sync(0xffffffffu, r1), m2 = __ballot_sync(0xffffffffu, r2);
            if (r1) {
                const int e = nf + __popc(m1 & below);
                fs[e] = s1;
                ft[e] = thr1;
            }
            nf += __popc(m1);
            if (r2) {
                const int e = nf + __popc(m2 & below);
                fs[e] = s2;
                ft[e] = thr2;
            }
            nf += __popc(m2);
        }
        __syncwarp();
        // 3. full rounds of retries
        while (nf >= 32) {
            nf -= 32;
            proposal_retry_out(R, out, fs[nf + lane], ft[nf + lane], sweep, key, dim);
            __syncwarp();
        }
    }
    if (lane < nf) proposal_retry_out(R, out, fs[lane], ft[lane], sweep, key, dim);
}

// FP32 FMA throughput probe: 8 independent chains per thread, no memory
// traffic in the loop; one result per thread keeps the work live.
__global__ void fma_peak_kernel(float *out, int iters, float a, float b)
{
    float v[8];
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = (float)(threadIdx.x + k) * 1e-3f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = fmaf(v[k], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) s += v[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int grid_for(long long n, int threads)
{
    long long g = (n + threads - 1) / threads;
    if (g > 152LL * 32) g = 152LL * 32;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

cudaError_t sn_launch_init_lattice(const SnInitArgs &a, cudaStream_t st)
{
    init_lattice_kernel<<<grid_for(a.n, 256), 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t sn_launch_upload_convert(const float *stage_xyz, const float *stage_len, float *px, float *py, float *pz,
                                     float *len, long long n, float uniform_len, int mixed, float default_len,
                                     int *flags, cudaStream_t st)
{
    upload_convert_kernel<<<grid_for(n, 256), 256, 0, st>>>(stage_xyz, stage_len, px, py, pz, len, n, uniform_len,
                                                           mixed, default_len, flags);
    return cudaGetLastError();
}

cudaError_t sn_launch_download_convert(const float *px, const float *py, const float *pz, const float *len,
                                       float *stage_xyz, float *stage_len, long long n, cudaStream_t st)
{
    download_convert_kernel<<<grid_for(n, 256), 256, 0, st>>>(px, py, pz, len, stage_xyz, stage_len, n);
    return cudaGetLastError();
}

cudaError_t sn_launch_set_out(SnReplicaDev *reps, int r, float *out, cudaStream_t st)
{
    set_out_kernel<<<1, 32, 0, st>>>(reps, r, out);
    return cudaGetLastError();
}

cudaError_t sn_launch_sweep_end(SnAccum *acc, SnState *state, double *hist, SnReplicaDev *reps, int nrep,
                                uint32_t *sweep, SnExchange *ex, int *order, uint32_t *queues, cudaStream_t st)
{
    sweep_end_kernel<<<1, 256, 0, st>>>(acc, state, hist, reps, nrep, sweep, ex, order, queues);
    return cudaGetLastError();
}

__global__ void count_diff_kernel(const int *__restrict__ a, const int *__restrict__ b, long long n,
                                  unsigned long long *count)
{
    unsigned long long c = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        c += a[i] != b[i];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

cudaError_t sn_launch_count_diff(const int *a, const int *b, long long n, unsigned long long *count, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    count_diff_kernel<<<grid_for(n, 256), 256, 0, st>>>(a, b, n, count);
    return cudaGetLastError();
}

cudaError_t sn_launch_recompute_finish(const double *red, SnState *state, const SnReplicaDev *reps, int rep,
                                       double cage, double *drift_max, int record, cudaStream_t st)
{
    recompute_finish_kernel<<<1, 1, 0, st>>>(red, state, reps, rep, cage, drift_max, record);
    return cudaGetLastError();
}

cudaError_t sn_launch_quench_step(float *px, float *py, float *pz, const float *len, const float *grad,
                                  long long n, float step, cudaStream_t st)
{
    quench_step_kernel<<<grid_for(n, 256), 256, 0, st>>>(px, py, pz, len, grad, n, step);
    return cudaGetLastError();
}

cudaError_t sn_launch_philox_batch(const uint32_t *ctr, const uint32_t *key, uint32_t *out, int n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    philox_batch_kernel<<<(n + 255) / 256, 256, 0, st>>>(ctr, key, out, n);
    return cudaGetLastError();
}

cudaError_t sn_launch_fma_peak(float *out, int blocks, int threads, int iters, cudaStream_t st)
{
    fma_peak_kernel<<<blocks, threads, 0, st>>>(out, iters, 0.999999f, 1e-6f);
    return cudaGetLastError();
}

cudaError_t sn_launch_proposal_batch(const uint32_t *site, uint32_t sweep, uint32_t seed_lo, uint32_t seed_hi,
                                     int dim, int constrain, float *out4, int n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    proposal_batch_kernel<<<(n + 255) / 256, 256, 0, st>>>(site, sweep, make_uint2(seed_lo, seed_hi), dim, constrain,
                                                           out4, n);
    return cudaGetLastError();
}

cudaError_t sn_launch_sweep_proposals(const SnReplicaDev *reps, int nrep, const uint32_t *sweep, int dim,
                                      int constrain, int sms, cudaStream_t st)
{
    if (nrep <= 0) return cudaSuccess;
    // one wave of resident blocks (the blocks stride over the sites); the
    // occupancy is looked up once per device
    static int per_sm_dev[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
    int per_sm = per_sm_dev[dev];
    if (per_sm == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_proposals_kernel, SN_PROP_WARPS * 32, 0) !=
                cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        per_sm_dev[dev] = per_sm;
    }
    const int bx = std::max(1, per_sm * sms / nrep);
    sweep_proposals_kernel<<<dim3(bx, nrep), SN_PROP_WARPS * 32, 0, st>>>(reps, sweep, dim, constrain);
    return cudaGetLastError();
}
