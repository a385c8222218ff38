// sn_analysis.cu -- analysis stencils on the resident lattice: the per-site
// dipole potential and dipole electric-field maps and the orientational
// correlation histogram of the reference's analysis code, plus the plain
// orientation sums behind polarisation() and landau_order().
//
// The maps reproduce the reference's arithmetic operation for operation
// (src/starrynight-analysis.c:65-94 dipole_potential, :310-380
// dipole_electricfieldoffset, :393-450 dipole_electricfield): the per-offset
// terms in FP32 with the reference's evaluation order and no contraction,
// summed in the reference's offset order in the reference's accumulator type,
// so each site's value is the reference's value bit for bit.  The offset
// tables (displacement, d^3, r/d) are built on the host with the reference's
// own float/double conversions.  The correlation histogram
// (:528-598 radial_order_parameter) sums in FP64 where the reference sums in
// FP32 (the reference's float sums over N x offsets terms lose digits).
//
// These kernels run once per analysis call, not per sweep: a thread per site
// walking the offset list, neighbours read through the read-only cache.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "sn_launch.h"

namespace {

// dot() of the reference (src/starrynight-config.c:189-199): a float sum
// started at 0 and added x, y, z in that order.
__device__ __forceinline__ float ref_dot(float ax, float ay, float az, float bx, float by, float bz)
{
    float s = __fadd_rn(0.0f, __fmul_rn(ax, bx));
    s = __fadd_rn(s, __fmul_rn(ay, by));
    return __fadd_rn(s, __fmul_rn(az, bz));
}

__device__ __forceinline__ int wrap(int v, int L)
{
    v %= L;
    return v < 0 ? v + L : v;
}

__device__ __forceinline__ void site_xyz(long long k, int Y, int Z, int &x, int &y, int &z)
{
    z = (int)(k % Z);
    const long long r = k / Z;
    y = (int)(r % Y);
    x = (int)(r / Y);
}

// pot_i = sum_j len_j (p_j . r) / d^3 over the offset list (double sum of
// float terms, src/starrynight-analysis.c:87-89).
__global__ void potential_kernel(SnLatticeView L, const SnAnalysisOffset *__restrict__ off, int n_off,
                                 double *__restrict__ out)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L.n) return;
    int x, y, z;
    site_xyz(k, L.Y, L.Z, x, y, z);
    double pot = 0.0;
    for (int i = 0; i < n_off; i++) {
        const SnAnalysisOffset o = off[i];
        const long long j = ((long long)wrap(x + o.dx, L.X) * L.Y + wrap(y + o.dy, L.Y)) * L.Z + wrap(z + o.dz, L.Z);
        const float dt = ref_dot(__ldg(L.px + j), __ldg(L.py + j), __ldg(L.pz + j), o.a[0], o.a[1], o.a[2]);
        const float t = __fdiv_rn(__fmul_rn(__ldg(L.len + j), dt), o.d3);
        pot = __dadd_rn(pot, (double)t);
    }
    out[k] = pot;
}

// |E_i| with E_i = sum_j (3 n (n . p_j) - p_j) / d^3 accumulated in float,
// minus p_i / 3 when self_term (the Kronecker contribution of
// src/starrynight-analysis.c:446-449); returns sqrt(dot(E, E)).
__global__ void efield_kernel(SnLatticeView L, const SnAnalysisOffset *__restrict__ off, int n_off, int self_term,
                              double *__restrict__ out)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L.n) return;
    int x, y, z;
    site_xyz(k, L.Y, L.Z, x, y, z);
    float ex = 0.0f, ey = 0.0f, ez = 0.0f;
    for (int i = 0; i < n_off; i++) {
        const SnAnalysisOffset o = off[i];
        const long long j = ((long long)wrap(x + o.dx, L.X) * L.Y + wrap(y + o.dy, L.Y)) * L.Z + wrap(z + o.dz, L.Z);
        const float qx = __ldg(L.px + j), qy = __ldg(L.py + j), qz = __ldg(L.pz + j);
        const double radial = (double)ref_dot(o.a[0], o.a[1], o.a[2], qx, qy, qz);
        // (3 n_x) radial - p_x in double, stored to float, then / d^3 in float
        float cx = (float)__dsub_rn(__dmul_rn((double)o.b[0], radial), (double)qx);
        float cy = (float)__dsub_rn(__dmul_rn((double)o.b[1], radial), (double)qy);
        float cz = (float)__dsub_rn(__dmul_rn((double)o.b[2], radial), (double)qz);
        cx = __fdiv_rn(cx, o.d3);
        cy = __fdiv_rn(cy, o.d3);
        cz = __fdiv_rn(cz, o.d3);
        ex = __fadd_rn(ex, cx);
        ey = __fadd_rn(ey, cy);
        ez = __fadd_rn(ez, cz);
    }
    if (self_term) {
        const double third = 1.0 / 3.0;
        ex = (float)__dsub_rn((double)ex, __dmul_rn(third, (double)L.px[k]));
        ey = (float)__dsub_rn((double)ey, __dmul_rn(third, (double)L.py[k]));
        ez = (float)__dsub_rn((double)ez, __dmul_rn(third, (double)L.pz[k]));
    }
    out[k] = __dsqrt_rn((double)ref_dot(ex, ey, ez, ex, ey, ez));
}

__device__ __forceinline__ double warp_sum_d(double v)
{
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Orientational correlation histogram: for every site i and every offset of
// bin b = |r|^2, FE = p_i . p_j and AFE = FE - 3 (n . p_i)(n . p_j).  The
// offset list is sorted by bin; each thread sums its site's terms of a bin in
// FP64, and at the end of a bin the warp's sums go to shared FP64 bins.
__global__ void radial_kernel(SnLatticeView L, const SnAnalysisOffset *__restrict__ off, int n_off, int n_bins,
                              double *__restrict__ fe_out, double *__restrict__ afe_out)
{
    extern __shared__ double sbin[];  // 2 * n_bins
    for (int i = threadIdx.x; i < 2 * n_bins; i += blockDim.x) sbin[i] = 0.0;
    __syncthreads();
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = k < L.n;
    int x = 0, y = 0, z = 0;
    float ix = 0.0f, iy = 0.0f, iz = 0.0f;
    if (live) {
        site_xyz(k, L.Y, L.Z, x, y, z);
        ix = L.px[k];
        iy = L.py[k];
        iz = L.pz[k];
    }
    double fe = 0.0, afe = 0.0;
    for (int i = 0; i < n_off; i++) {
        const SnAnalysisOffset o = off[i];
        if (live) {
            const long long j =
                ((long long)wrap(x + o.dx, L.X) * L.Y + wrap(y + o.dy, L.Y)) * L.Z + wrap(z + o.dz, L.Z);
            const float qx = __ldg(L.px + j), qy = __ldg(L.py + j), qz = __ldg(L.pz + j);
            const float c = ref_dot(ix, iy, iz, qx, qy, qz);
            const float ni = ref_dot(o.a[0], o.a[1], o.a[2], ix, iy, iz);
            const float nj = ref_dot(o.a[0], o.a[1], o.a[2], qx, qy, qz);
            const float a = __fsub_rn(c, __fmul_rn(__fmul_rn(3.0f, ni), nj));
            fe += (double)c;
            afe += (double)a;
        }
        if (i + 1 == n_off || off[i + 1].bin != o.bin) {  // uniform across the block
            const double wf = warp_sum_d(fe), wa = warp_sum_d(afe);
            if ((threadIdx.x & 31) == 0) {
                atomicAdd(&sbin[2 * o.bin], wf);
                atomicAdd(&sbin[2 * o.bin + 1], wa);
            }
            fe = 0.0;
            afe = 0.0;
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < n_bins; b += blockDim.x) {
        if (sbin[2 * b] != 0.0) atomicAdd(fe_out + b, sbin[2 * b]);
        if (sbin[2 * b + 1] != 0.0) atomicAdd(afe_out + b, sbin[2 * b + 1]);
    }
}

// Unweighted orientation sums sum_i p_i (polarisation(), landau_order()).
__global__ void orient_sum_kernel(SnLatticeView L, double *__restrict__ out3)
{
    double s[3] = {0.0, 0.0, 0.0};
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < L.n;
         k += (long long)gridDim.x * blockDim.x) {
        s[0] += (double)L.px[k];
        s[1] += (double)L.py[k];
        s[2] += (double)L.pz[k];
    }
    __shared__ double part[3][32];
    for (int c = 0; c < 3; c++) {
        const double w = warp_sum_d(s[c]);
        if ((threadIdx.x & 31) == 0) part[c][threadIdx.x >> 5] = w;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int nw = blockDim.x >> 5;
        for (int c = 0; c < 3; c++) {
            const double v = warp_sum_d(threadIdx.x < nw ? part[c][threadIdx.x] : 0.0);
            if (threadIdx.x == 0) atomicAdd(out3 + c, v);
        }
    }
}

unsigned grid_for(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

cudaError_t sn_launch_potential(const SnLatticeView &L, const SnAnalysisOffset *off, int n_off, double *out,
                                cudaStream_t st)
{
    if (L.n <= 0) return cudaSuccess;
    potential_kernel<<<grid_for(L.n, 256), 256, 0, st>>>(L, off, n_off, out);
    return cudaGetLastError();
}

cudaError_t sn_launch_efield(const SnLatticeView &L, const SnAnalysisOffset *off, int n_off, int self_term,
                             double *out, cudaStream_t st)
{
    if (L.n <= 0) return cudaSuccess;
    efield_kernel<<<grid_for(L.n, 256), 256, 0, st>>>(L, off, n_off, self_term, out);
    return cudaGetLastError();
}

cudaError_t sn_launch_radial(const SnLatticeView &L, const SnAnalysisOffset *off, int n_off, int n_bins,
                             double *fe, double *afe, cudaStream_t st)
{
    if (L.n <= 0) return cudaSuccess;
    radial_kernel<<<grid_for(L.n, 256), 256, 2 * n_bins * sizeof(double), st>>>(L, off, n_off, n_bins, fe, afe);
    return cudaGetLastError();
}

cudaError_t sn_launch_orient_sum(const SnLatticeView &L, double *out3, cudaStream_t st)
{
    if (L.n <= 0) return cudaSuccess;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const unsigned g = (unsigned)std::min<long long>(grid_for(L.n, 256), 4LL * (nsm > 0 ? nsm : 1));
    orient_sum_kernel<<<g, 256, 0, st>>>(L, out3);
    return cudaGetLastError();
}
