// sn_device.cuh -- device helpers: Philox4x32-10, the Metropolis proposal,
// and the compile-time cutoff stencil.
#pragma once

#include <cstdint>
#include <utility>

#include "sn_internal.h"

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): ten rounds of the 4x32
// S-box with the published multipliers and Weyl key increments.
__device__ __forceinline__ uint4 sn_philox(uint4 c, uint2 k)
{
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

// ---------------------------------------------------------------------------
// Proposal.  Counter (site, sweep, k, stream), key = replica seed.  Only
// correctly rounded + - * / sqrt are used, so the CPU oracle reproduces the
// proposal bit for bit.  Draw 0: word 0 -> accept uniform u in [0,1);
// words 1,2 -> first Marsaglia try; word 3 -> axis choice (ConstrainToX).
// Draws k >= 1: two tries each.  Marsaglia (1972) as in random_sphere_point
// (src/starrynight-config.c:203-227): x1,x2 uniform in [-1,1) until
// q = x1^2 + x2^2 <= 1, then p = (2 x1 sqrt(1-q), 2 x2 sqrt(1-q), 1 - 2q);
// the DIM<3 branch maps to the circle ((x1^2-x2^2)/q, 2 x1 x2 / q, 0).
#define SN_PROPOSAL_MAX_DRAWS 16
#define SN_STREAM_SWEEP 0u
#define SN_STREAM_INIT 1u
#define SN_STREAM_EXCHANGE 2u

__device__ __forceinline__ float sn_unit_m1(uint32_t r)  // [-1, 1) in 2^-23 steps
{
    return __fsub_rn(__fmul_rn((float)(r >> 8), 1.1920928955078125e-07f), 1.0f);
}

__device__ __forceinline__ float sn_uniform24(uint32_t r)  // [0, 1) in 2^-24 steps
{
    return __fmul_rn((float)(r >> 8), 5.9604644775390625e-08f);
}

__device__ __forceinline__ bool sn_try_point(uint32_t ra, uint32_t rb, int dim, float3 &p)
{
    const float x1 = sn_unit_m1(ra), x2 = sn_unit_m1(rb);
    const float a = __fmul_rn(x1, x1), b = __fmul_rn(x2, x2);
    const float q = __fadd_rn(a, b);
    if (q > 1.0f) return false;
    if (dim < 3) {
        if (q == 0.0f) return false;
        p.x = __fdiv_rn(__fsub_rn(a, b), q);
        p.y = __fdiv_rn(__fmul_rn(__fmul_rn(2.0f, x1), x2), q);
        p.z = 0.0f;
    } else {
        const float t = __fsqrt_rn(__fsub_rn(1.0f, q));
        p.x = __fmul_rn(__fmul_rn(2.0f, x1), t);
        p.y = __fmul_rn(__fmul_rn(2.0f, x2), t);
        p.z = __fsub_rn(1.0f, __fmul_rn(2.0f, q));
    }
    return true;
}

// Draw 0 of a proposal: the accept uniform u, and the first try (or the axis
// for ConstrainToX).  False when the try was rejected: sn_proposal_retry then
// continues with draws 1, 2, ...
__device__ __forceinline__ bool sn_proposal_first(uint32_t site, uint32_t sweep, uint32_t stream, uint2 key,
                                                  int dim, int constrain, float3 &p, float &u)
{
    const uint4 r = sn_philox(make_uint4(site, sweep, 0u, stream), key);
    u = sn_uniform24(r.x);
    if (constrain) {
        const uint32_t c = (uint32_t)(((uint64_t)r.w * 6ull) >> 32);
        const float v = (c & 1u) ? -1.0f : 1.0f;
        p = make_float3(c >> 1 == 0 ? v : 0.0f, c >> 1 == 1 ? v : 0.0f, c >> 1 == 2 ? v : 0.0f);
        return true;
    }
    return sn_try_point(r.y, r.z, dim, p);
}

__device__ __forceinline__ bool sn_proposal_retry(uint32_t site, uint32_t sweep, uint32_t stream, uint2 key,
                                                  int dim, float3 &p)
{
    for (uint32_t k = 1; k < SN_PROPOSAL_MAX_DRAWS; k++) {
        const uint4 r = sn_philox(make_uint4(site, sweep, k, stream), key);
        if (sn_try_point(r.x, r.y, dim, p)) return true;
        if (sn_try_point(r.z, r.w, dim, p)) return true;
    }
    return false;
}

// Returns false when every try was rejected (the move then keeps the old dipole).
__device__ __forceinline__ bool sn_proposal(uint32_t site, uint32_t sweep, uint32_t stream, uint2 key,
                                            int dim, int constrain, float3 &p, float &u)
{
    return sn_proposal_first(site, sweep, stream, key, dim, constrain, p, u) ||
           sn_proposal_retry(site, sweep, stream, key, dim, p);
}

// ---------------------------------------------------------------------------
// Compile-time cutoff stencil.  The offsets with 0 < |o|^2 <= rc^2 (the
// sphere of gen_neighbour, src/starrynight-montecarlo-core.c:38-72; 2D when
// Z == 1) come in +-o pairs; the kernels enumerate the "positive" half
// (first nonzero component > 0) and use T_o = T_{-o}.
namespace sn_stencil {

constexpr bool positive(int x, int y, int z) { return x > 0 || (x == 0 && (y > 0 || (y == 0 && z > 0))); }

constexpr int npairs(int rc, bool two_d)
{
    int n = 0;
    const int zc = two_d ? 0 : rc;
    for (int x = -rc; x <= rc; x++)
        for (int y = -rc; y <= rc; y++)
            for (int z = -zc; z <= zc; z++)
                if (x * x + y * y + z * z <= rc * rc && positive(x, y, z)) n++;
    return n;
}

struct Off {
    int x, y, z;
};

constexpr Off pair_offset(int rc, bool two_d, int idx)
{
    int n = 0;
    const int zc = two_d ? 0 : rc;
    for (int x = -rc; x <= rc; x++)
        for (int y = -rc; y <= rc; y++)
            for (int z = -zc; z <= zc; z++)
                if (x * x + y * y + z * z <= rc * rc && positive(x, y, z)) {
                    if (n == idx) return Off{x, y, z};
                    n++;
                }
    return Off{0, 0, 0};
}

constexpr double csqrt(double v)
{
    double r = v > 1.0 ? v : 1.0;
    for (int i = 0; i < 64; i++) r = 0.5 * (r + v / r);
    return r;
}

// Entry e of T_o = (I - 3 n n^T)/d^3, e in {xx, yy, zz, xy, xz, yz}.
constexpr double tensor_d(int x, int y, int z, int e)
{
    const double r2 = double(x * x + y * y + z * z);
    const double d = csqrt(r2);
    const double inv5 = 1.0 / (r2 * r2 * d);
    const double inv3 = 1.0 / (r2 * d);
    const int a[6] = {x, y, z, x, x, y};
    const int b[6] = {x, y, z, y, z, z};
    const double diag = e < 3 ? inv3 : 0.0;
    return diag - 3.0 * double(a[e] * b[e]) * inv5;
}

}  // namespace sn_stencil
