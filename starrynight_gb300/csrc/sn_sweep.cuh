// sn_sweep.cuh -- the Metropolis sweep kernels and the field (energy) pass.
//
// Schedule.  A replica's lattice is cut into blocks of B = (bx,by,bz) sites;
// blocks get a checkerboard colour (block index mod 2 per axis).  Blocks of
// one colour never interact (two of them are at least one block, >= cutoff
// sites, apart); a block's halo (cutoff sites around it) lies in blocks of
// other colours.  sweep_phase runs one launch per block colour, one CTA per
// block; sweep_flow runs a whole sweep as one persistent launch in which a
// block waits only for its adjacent blocks of earlier colours -- the same
// reads and writes for every block.  Inside the block the CTA visits the s^3 site
// colours (local coordinate mod s, s = cutoff + 1) in order; sites of one
// site colour are >= s apart and are updated together.  Every occupied site
// is attempted exactly once per sweep: the same set of moves as MC_moves
// over X*Y*Z steps (src/starrynight-montecarlo-core.c:143-191), in a
// different but fixed order.
//
// Per site-colour group (one colour, or two colours that cannot interact):
//   1. (split) NS warp groups each sum a slice of the cutoff stencil into
//      partial local fields h = sum T_o p_j and nearest-neighbour sums
//      nn = sum_{|o|=1} p_j; T_o = (I - 3 n n^T)/d^3 is a compile-time
//      constant and +o/-o neighbours share it (the FP32 form of the
//      dipole-dipole sum of site_energy, src/starrynight-montecarlo-core.c:91-106).
//   2. (finalize) one thread per target adds the partials, forms
//      g = len_i h - C nn + E (+ the K term), dE = (p' - p).g
//      (src/starrynight-montecarlo-core.c:102-134) and applies the accept
//      test dE < 0 || exp(-beta dE) > u (:179) with a Philox uniform.
//
// Shared memory.  The tile (block + halo) is stored as float triples, each
// axis permuted class-major (pi(u) = start[u mod s] + u / s), so the targets
// of one site colour occupy consecutive slots and every stencil offset is one
// uniform slot delta for all of them: with the padded strides chosen on the
// host, the 32 lanes of a warp hit 32 distinct banks.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <type_traits>

#include "sn_device.cuh"

namespace sn_sweep {

template <int RC, bool TWO_D>
struct Geo {
    static constexpr int S = RC + 1;                 // site-colour stride
    static constexpr int H = RC;                     // halo (x, y)
    static constexpr int HZ = TWO_D ? 0 : RC;        // halo (z)
    static constexpr int SZ = TWO_D ? 1 : S;         // site colours along z
    static constexpr int NF = 2 * RC + 1;            // offsets per axis
    static constexpr int NP = sn_stencil::npairs(RC, TWO_D);
    // neighbour-list splits: about SN_PAIRS_PER_SPLIT +-o pairs per thread, at most 8
    static constexpr int NSR = (NP + SN_PAIRS_PER_SPLIT / 2) / SN_PAIRS_PER_SPLIT;
    static constexpr int NS = NSR < 1 ? 1 : (NSR > 8 ? 8 : NSR);
    // Site colours c and c + (s/2, s/2, s/2) never interact when every
    // component of the displacement between their sites is >= s/2, i.e. when
    // 3 (s/2)^2 > cutoff^2 (cutoff 1, 3, 5 in 3D).  They are then updated
    // together, halving the number of sequential sub-phases.
    static constexpr bool MERGE = !TWO_D && (S % 2 == 0) && 3 * (S / 2) * (S / 2) > RC * RC;
    static constexpr int NH = MERGE ? 2 : 1;         // colours per group
    static constexpr int HX = MERGE ? S / 2 : S;     // representative colours along x
    static constexpr int NG = HX * S * SZ;           // colour groups per block
};

__device__ __forceinline__ float sn_fma(float a, float b, float c) { return fmaf(a, b, c); }

// Round to the nearest integer (ties to even), saturating at the int32 range.
__device__ __forceinline__ int fixed_point(float v) { return __float2int_rn(v); }
__device__ __forceinline__ int fixed_point(double v) { return __double2int_rn(v); }

// Sum of component c over the accumulator sets, in set order.
template <typename R>
__device__ __forceinline__ R sum_sets(const R (&h)[SN_ACC_SETS][3], int c)
{
    R s = h[0][c];
#pragma unroll
    for (int k = 1; k < SN_ACC_SETS; k++) s += h[k][c];
    return s;
}
__device__ __forceinline__ double sn_fma(double a, double b, double c) { return fma(a, b, c); }

// ---------------------------------------------------------------------------
// One +-o pair of the stencil.
template <typename R, int RC, bool TWO_D, bool MIXED, int I>
__device__ __forceinline__ void pair_step(const unsigned char *__restrict__ base, uint32_t tb,
                                          const int (&FX)[2 * RC + 1], const int (&FY)[2 * RC + 1],
                                          const float *__restrict__ tlen, uint32_t tslot, R (&h)[SN_ACC_SETS][3],
                                          R (&nn)[3])
{
    constexpr sn_stencil::Off o = sn_stencil::pair_offset(RC, TWO_D, I);
    constexpr int H = RC;
    // x, y: class-major axes, per-colour byte deltas FX, FY (one column base
    // tb + FX + FY per (ox, oy), shared by the column's loads); z: plain
    // axis, a compile-time delta of 12 bytes per site.  Signed arithmetic:
    // neighbours below the target have negative deltas, and every neighbour
    // lies inside the tile because |o| <= halo.
    const int ao = FX[H + o.x] + FY[H + o.y];
    const int bo = FX[H - o.x] + FY[H - o.y];
    const float *pa = reinterpret_cast<const float *>(base + ((int)tb + ao) + 12 * o.z);
    const float *pb = reinterpret_cast<const float *>(base + ((int)tb + bo) - 12 * o.z);
    const R ax = pa[0], ay = pa[1], az = pa[2];
    const R bx = pb[0], by = pb[1], bz = pb[2];
    R qx, qy, qz;
    if constexpr (MIXED) {
        // the tile holds unit p; weight each neighbour by its length here,
        // in the accumulator's precision
        const R la = tlen[(int)tslot + ao / 12 + o.z], lb = tlen[(int)tslot + bo / 12 - o.z];
        qx = sn_fma(la, ax, lb * bx);
        qy = sn_fma(la, ay, lb * by);
        qz = sn_fma(la, az, lb * bz);
    } else {
        qx = ax + bx;
        qy = ay + by;
        qz = az + bz;
    }
    constexpr R txx = (R)sn_stencil::tensor_d(o.x, o.y, o.z, 0);
    constexpr R tyy = (R)sn_stencil::tensor_d(o.x, o.y, o.z, 1);
    constexpr R tzz = (R)sn_stencil::tensor_d(o.x, o.y, o.z, 2);
    constexpr R txy = (R)sn_stencil::tensor_d(o.x, o.y, o.z, 3);
    constexpr R txz = (R)sn_stencil::tensor_d(o.x, o.y, o.z, 4);
    constexpr R tyz = (R)sn_stencil::tensor_d(o.x, o.y, o.z, 5);
    R(&a)[3] = h[I % SN_ACC_SETS];  // independent accumulator chains for consecutive pairs
    a[0] = sn_fma(txx, qx, a[0]);
    if constexpr (txy != 0.0f) a[0] = sn_fma(txy, qy, a[0]);
    if constexpr (txz != 0.0f) a[0] = sn_fma(txz, qz, a[0]);
    if constexpr (txy != 0.0f) a[1] = sn_fma(txy, qx, a[1]);
    a[1] = sn_fma(tyy, qy, a[1]);
    if constexpr (tyz != 0.0f) a[1] = sn_fma(tyz, qz, a[1]);
    if constexpr (txz != 0.0f) a[2] = sn_fma(txz, qx, a[2]);
    if constexpr (tyz != 0.0f) a[2] = sn_fma(tyz, qy, a[2]);
    a[2] = sn_fma(tzz, qz, a[2]);
    if constexpr (o.x * o.x + o.y * o.y + o.z * o.z == 1) {
        // cage strain: unweighted sum of the six nearest dipoles
        if constexpr (MIXED) {
            nn[0] += ax + bx;
            nn[1] += ay + by;
            nn[2] += az + bz;
        } else {
            nn[0] += qx;
            nn[1] += qy;
            nn[2] += qz;
        }
    }
}

template <typename R, int RC, bool TWO_D, bool MIXED, int LO, int... Is>
__device__ __forceinline__ void run_pairs(std::integer_sequence<int, Is...>, const unsigned char *base, uint32_t tb,
                                          const int (&FX)[2 * RC + 1], const int (&FY)[2 * RC + 1],
                                          const float *tlen, uint32_t tslot, R (&h)[SN_ACC_SETS][3], R (&nn)[3])
{
    (pair_step<R, RC, TWO_D, MIXED, LO + Is>(base, tb, FX, FY, tlen, tslot, h, nn), ...);
}

template <typename R, int RC, bool TWO_D, bool MIXED, int J>
__device__ __forceinline__ void dispatch_split(int j, const unsigned char *base, uint32_t tb,
                                               const int (&FX)[2 * RC + 1], const int (&FY)[2 * RC + 1],
                                               const float *tlen, uint32_t tslot, R (&h)[SN_ACC_SETS][3], R (&nn)[3])
{
    using G = Geo<RC, TWO_D>;
    if constexpr (J < G::NS) {
        if (j == J) {
            constexpr int lo = J * G::NP / G::NS, hi = (J + 1) * G::NP / G::NS;
            run_pairs<R, RC, TWO_D, MIXED, lo>(std::make_integer_sequence<int, hi - lo>{}, base, tb, FX, FY, tlen,
                                                tslot, h, nn);
        } else {
            dispatch_split<R, RC, TWO_D, MIXED, J + 1>(j, base, tb, FX, FY, tlen, tslot, h, nn);
        }
    }
}

__device__ __forceinline__ int sn_wrap(int v, int L) { return v < 0 ? v + L : (v >= L ? v - L : v); }

template <int S>
__device__ __forceinline__ int sn_pi(const int *start, int u) { return start[u % S] + u / S; }

__host__ __device__ inline int sn_count(int B, int c, int S) { return c < B ? (B - c + S - 1) / S : 0; }

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Compensated (Kahan) FP32 running sum: error independent of the number of
// terms to first order, so a thread's few dozen accepted moves per block
// keep FP64-grade totals without using the (slow) FP64 pipe per move.
struct KahanF {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float v)
    {
        const float y = __fsub_rn(v, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

__device__ __forceinline__ void cp_async4(void *smem_dst, const void *gsrc)
{
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gsrc) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// Shared-memory carve-up, identical on host (sizing) and device.
struct Carve {
    uint32_t tile, tlen, props, parts, ftab, start, red, total;
};

__host__ __device__ inline uint32_t sn_align16(uint32_t v) { return (v + 15u) & ~15u; }

// pc > 0: sweep kernel (pc staged proposal groups, 3 float partials);
// pc == 0: field kernel (6 partials of rbytes each).
__host__ __device__ inline Carve sn_carve(int slots, int tg, int pc, int NS, int S, int NF, bool mixed, int rbytes)
{
    Carve c;
    uint32_t o = 0;
    c.tile = o;
    o += sn_align16((uint32_t)slots * 12u);
    c.tlen = o;
    if (mixed) o += sn_align16((uint32_t)slots * 4u);
    c.props = o;
    o += (uint32_t)(pc * tg) * 16u;
    c.parts = o;
    o += sn_align16((uint32_t)(NS * (pc > 0 ? 3 : 6) * tg * rbytes));
    c.ftab = o;
    o += sn_align16((uint32_t)(3 * S * NF) * 4u);
    c.start = o;
    o += sn_align16(3u * SN_MAX_S * 4u);
    c.red = o;
    o += (SN_MAX_THREADS / 32) * 16u * 8u;
    c.total = o;
    return c;
}

// Colour (cx, cy, cz) of half `h` of group g (h = 1: the merged partner).
template <int S, int SZ, bool MERGE>
__device__ __forceinline__ void group_colour(int g, int h, int &cx, int &cy, int &cz)
{
    cx = g / (S * SZ);
    cy = (g / SZ) % S;
    cz = g % SZ;
    if (MERGE && h) {
        cx = (cx + S / 2) % S;
        cy = (cy + S / 2) % S;
        cz = (cz + S / 2) % S;
    }
}

// Tables every block needs: class starts of the x and y axes and, per axis
// and site colour c, the byte delta of each offset o from a target of
// colour c (z is stored plainly: its deltas are compile-time).
template <int RC, bool TWO_D>
__device__ __forceinline__ void build_tables(const SnTile &Gm, int *start, int *ftab, int tid, int nthreads)
{
    using G = Geo<RC, TWO_D>;
    constexpr int S = G::S, H = G::H, NF = G::NF;
    if (tid < 3 * SN_MAX_S) start[tid] = Gm.start[tid / SN_MAX_S][tid % SN_MAX_S];
    __syncthreads();
    for (int i = tid; i < 2 * S * NF; i += nthreads) {
        const int ax = i / (S * NF), c = (i / NF) % S, o = i % NF - H;
        int v = 0;
        const int T = Gm.T[ax];
        const int u0 = c + H, u = u0 + o;
        if (u >= 0 && u < T && u0 < T) {
            const int *st = start + ax * SN_MAX_S;
            const int d = sn_pi<S>(st, u) - sn_pi<S>(st, u0);
            v = d * (ax == 0 ? Gm.Sx : Gm.Sy) * 12;
        }
        ftab[i] = v;
    }
}

// Copy of block + halo (periodic wrap) into the class-major tile by
// asynchronous copies.  The dataflow kernel reads blocks other SMs wrote
// during the same launch; its acquire of their done flags followed by a
// gpu-scope fence orders those writes before these copies.
template <int RC, bool TWO_D, bool MIXED>
__device__ __forceinline__ void stage_tile(const SnReplicaDev &R, const SnTile &Gm, const SnWork &w, float *tile,
                                           float *tlen, const int *start, int tid, int nthreads)
{
    using G = Geo<RC, TWO_D>;
    constexpr int S = G::S, H = G::H, HZ = G::HZ;
    const int lane = tid & 31, warp = tid >> 5, nwarps = nthreads >> 5;
    const int X = R.X, Y = R.Y, Z = R.Z;
    const int Tx = Gm.T[0], Ty = Gm.T[1], Tz = Gm.T[2];
    for (int row = warp; row < Tx * Ty; row += nwarps) {
        const int ux = row / Ty, uy = row - (row / Ty) * Ty;
        const int gx = sn_wrap(w.x0 - H + ux, X), gy = sn_wrap(w.y0 - H + uy, Y);
        const int rslot = sn_pi<S>(start, ux) * Gm.Sx + sn_pi<S>(start + SN_MAX_S, uy) * Gm.Sy;
        const long long gb = ((long long)gx * Y + gy) * Z;
        for (int uz = lane; uz < Tz; uz += 32) {
            const int gz = TWO_D ? 0 : sn_wrap(w.z0 - HZ + uz, Z);
            const long long g = gb + gz;
            const int slot = rslot + uz;  // z is stored plainly
            cp_async4(&tile[3 * slot + 0], R.px + g);
            cp_async4(&tile[3 * slot + 1], R.py + g);
            cp_async4(&tile[3 * slot + 2], R.pz + g);
            if constexpr (MIXED) cp_async4(&tlen[slot], R.len + g);
        }
    }
}

// ---------------------------------------------------------------------------
// Sweep kernel.  Thread tid owns split j = tid / tg of the stencil for target
// tt = tid % tg of every colour group: half h = tt / tp of the group, target
// t = tt % tp = (qx, qy, qz) of that colour (inactive where the colour has
// fewer targets).  Threads with j == 0 also finalize their target.
template <int RC, bool TWO_D, bool MIXED, bool FLOW>
__device__ __forceinline__ void sweep_block(const SnWork w, const SnPhaseArgs &a, unsigned char *smem)
{
    using G = Geo<RC, TWO_D>;
    constexpr int S = G::S, H = G::H, HZ = G::HZ, SZ = G::SZ, NF = G::NF, NS = G::NS;
    constexpr bool MERGE = G::MERGE;

    const int tid = threadIdx.x, nthreads = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5;
    const SnReplicaDev &R = a.reps[w.rep];
    const SnTile &Gm = a.geoms[R.geom];

    const int Y = R.Y, Z = R.Z;
    float *__restrict__ gpx = R.px;
    float *__restrict__ gpy = R.py;
    float *__restrict__ gpz = R.pz;
    const float *__restrict__ glen = R.len;
    const int Bx = Gm.B[0], By = Gm.B[1], Bz = Gm.B[2];
    const int Sy = Gm.Sy, Sx = Gm.Sx;
    const int tp = Gm.tp, tg = Gm.tg, ng = Gm.ng, pc = Gm.pc;
    const int nqy = Gm.nq[1], nqz = Gm.nq[2];
    const uint32_t sweep = *a.sweep;
    const uint2 key = make_uint2(R.seed_lo, R.seed_hi);
    const float beta = R.beta;
    const float Ex = R.E[0], Ey = R.E[1], Ez = R.E[2];
    const float C = a.cage, Kk = a.K;
    const float Lu = R.length;

    const Carve cv = sn_carve(Gm.slots, tg, pc, NS, S, NF, MIXED, 4);
    float *tile = reinterpret_cast<float *>(smem + cv.tile);
    float *tlen = reinterpret_cast<float *>(smem + cv.tlen);
    float4 *props = reinterpret_cast<float4 *>(smem + cv.props);
    float *parts = reinterpret_cast<float *>(smem + cv.parts);
    int *ftab = reinterpret_cast<int *>(smem + cv.ftab);
    int *start = reinterpret_cast<int *>(smem + cv.start);
    double *red = reinterpret_cast<double *>(smem + cv.red);

    build_tables<RC, TWO_D>(Gm, start, ftab, tid, nthreads);
    stage_tile<RC, TWO_D, MIXED>(R, Gm, w, tile, tlen, start, tid, nthreads);

    // this thread's fixed role
    const int j = tid / tg, tt = tid - (tid / tg) * tg;
    const int hh = tt / tp, t = tt - (tt / tp) * tp;
    const int qz = t % nqz, qy = (t / nqz) % nqy, qx = t / (nqz * nqy);
    // a launch shared by replicas of different geometry runs with the largest
    // block size: threads past splits * targets have no stencil role
    const bool tvalid = tid < NS * tg && qx < Gm.nq[0];
    const int trel = qx * Sx + qy * Sy + S * qz;  // z plain: targets S apart
    const int srel = ((S * qx) * Y + S * qy) * Z + (TWO_D ? 0 : S * qz);

    KahanF sdE, sPx, sPy, sPz;
    unsigned int sacc = 0, satt = 0;

    int FX[NF], FY[NF];
    int pcx = -1, pcy = -1;
    int gchunk = 0, gnext = 0;  // first group of the staged chunk, first group of the next
    // groups in which this thread's target exists (bit g), computed once
    unsigned long long amask = 0ull;
    for (int g = 0; g < ng && g < 64; g++) {
        int cx, cy, cz;
        group_colour<S, SZ, MERGE>(g, hh, cx, cy, cz);
        if (tvalid && qx < sn_count(Bx, cx, S) && qy < sn_count(By, cy, S) && (TWO_D || qz < sn_count(Bz, cz, S)))
            amask |= 1ull << g;
    }
    for (int g = 0; g < ng; g++) {
        // ---- proposals and accept thresholds of the next pc groups ------------
        // Thread (j, tt) draws for its own target tt in groups g0+j, g0+j+NS, ...
        if (g == gnext) {
            __syncthreads();  // previous chunk fully consumed
            gchunk = g;
            gnext = min(g + pc, ng);
            if (tid < NS * tg) {
                for (int k = j; k < gnext - g; k += NS) {
                    int cx, cy, cz;
                    group_colour<S, SZ, MERGE>(g + k, hh, cx, cy, cz);
                    float4 pr = make_float4(0.0f, 0.0f, 0.0f, -2.0f);  // no target here
                    if ((g + k < 64) ? ((amask >> (g + k)) & 1ull)
                                     : (tvalid && qx < sn_count(Bx, cx, S) && qy < sn_count(By, cy, S) &&
                                        (TWO_D || qz < sn_count(Bz, cz, S)))) {
                        const int site = ((w.x0 + cx) * Y + (w.y0 + cy)) * Z + (TWO_D ? 0 : w.z0 + cz) + srel;
                        pr.w = -1.0f;  // vacancy
                        if (glen[site] != 0.0f) {
                            float3 p;
                            float u;
                            if (!sn_proposal((uint32_t)site, sweep, SN_STREAM_SWEEP, key, a.dim, a.constrain, p, u))
                                p = make_float3(FLOW ? __ldcg(gpx + site) : gpx[site],
                                                FLOW ? __ldcg(gpy + site) : gpy[site],
                                                FLOW ? __ldcg(gpz + site) : gpz[site]);
                            // accept iff dE < -ln(u)/beta  <=>  dE < 0 || exp(-beta dE) > u
                            const float thr = u > 0.0f ? -logf(u) / beta : INFINITY;
                            pr = make_float4(p.x, p.y, p.z, thr);
                        }
                    }
                    props[k * tg + tt] = pr;
                }
            }
            if (g == 0) cp_async_wait_all();
            __syncthreads();
        }

        int cx, cy, cz;
        group_colour<S, SZ, MERGE>(g, hh, cx, cy, cz);
        const bool active = (g < 64) ? ((amask >> g) & 1ull) != 0ull
                                     : (tvalid && qx < sn_count(Bx, cx, S) && qy < sn_count(By, cy, S) &&
                                        (TWO_D || qz < sn_count(Bz, cz, S)));
        if (cx != pcx) {
#pragma unroll
            for (int o = 0; o < NF; o++) FX[o] = ftab[(0 * S + cx) * NF + o];
            pcx = cx;
        }
        if (cy != pcy) {
#pragma unroll
            for (int o = 0; o < NF; o++) FY[o] = ftab[(1 * S + cy) * NF + o];
            pcy = cy;
        }
        const int tslot = sn_pi<S>(start, cx + H) * Sx + sn_pi<S>(start + SN_MAX_S, cy + H) * Sy +
                          (TWO_D ? 0 : cz + HZ) + trel;

        // ---- 1. partial g = len_i h - C nn of this split ---------------------------
        if (active) {
            float hacc[SN_ACC_SETS][3] = {};
            float nn[3] = {0.f, 0.f, 0.f};
            dispatch_split<float, RC, TWO_D, MIXED, 0>(j, smem + cv.tile, (uint32_t)tslot * 12u, FX, FY, tlen,
                                                       (uint32_t)tslot, hacc, nn);
            const float sc = MIXED ? tlen[tslot] : Lu * Lu;
            float *pp = parts + (j * 3) * tg + tt;
            pp[0 * tg] = fmaf(sc, sum_sets(hacc, 0), -C * nn[0]);
            pp[1 * tg] = fmaf(sc, sum_sets(hacc, 1), -C * nn[1]);
            pp[2 * tg] = fmaf(sc, sum_sets(hacc, 2), -C * nn[2]);
        }
        __syncthreads();

        // ---- 2. finalize: dE, accept, update ------------------------------------------
        if (j == 0 && active) {
            const float4 pr = props[(g - gchunk) * tg + tt];
            if (pr.w >= 0.0f) {
                float gx = Ex, gy = Ey, gz = Ez;
#pragma unroll
                for (int k = 0; k < NS; k++) {
                    const float *pp = parts + (k * 3) * tg + tt;
                    gx += pp[0 * tg];
                    gy += pp[1 * tg];
                    gz += pp[2 * tg];
                }
                const int site = ((w.x0 + cx) * Y + (w.y0 + cy)) * Z + (TWO_D ? 0 : w.z0 + cz) + srel;
                const float Li = MIXED ? tlen[tslot] : Lu;
                const float ox = tile[3 * tslot + 0], oy = tile[3 * tslot + 1], oz = tile[3 * tslot + 2];
                const float dx = pr.x - ox, dy = pr.y - oy, dz = pr.z - oz;
                float dE = fmaf(dx, gx, fmaf(dy, gy, dz * gz));
                if (Kk > 0.0f) dE -= Kk * ((fabsf(pr.x) - fabsf(ox)) + (fabsf(pr.y) - fabsf(oy)));
                satt++;
                if (dE < pr.w) {
                    tile[3 * tslot + 0] = pr.x;
                    tile[3 * tslot + 1] = pr.y;
                    tile[3 * tslot + 2] = pr.z;
                    gpx[site] = pr.x;
                    gpy[site] = pr.y;
                    gpz[site] = pr.z;
                    sacc++;
                    sdE.add(dE);
                    sPx.add(Li * dx);
                    sPy.add(Li * dy);
                    sPz.add(Li * dz);
                }
            }
        }
        __syncthreads();
    }

    // ---- the block's final sites to the caller's buffer -------------------------
    // No other block writes these sites during the sweep, so the tile's
    // interior is final now.  A row of the block (fixed x, y) is 3*Bz floats
    // contiguous both in the tile (z stored plainly) and in the buffer.
    if (float *out = R.out_xyz) {
        const int w3 = 3 * Bz;
        for (int row = warp; row < Bx * By; row += nthreads >> 5) {
            const int lx = row / By, ly = row - (row / By) * By;
            const int s0 = sn_pi<S>(start, lx + H) * Sx + sn_pi<S>(start + SN_MAX_S, ly + H) * Sy + HZ;
            const long long o0 = 3ll * ((((long long)(w.x0 + lx)) * Y + (w.y0 + ly)) * Z + (TWO_D ? 0 : w.z0));
            for (int e = lane; e < w3; e += 32) out[o0 + e] = tile[3 * s0 + e];
        }
    }

    // ---- block reduction of the move statistics ---------------------------------
    double v[6] = {sdE.value(), sPx.value(), sPy.value(), sPz.value(), (double)sacc, (double)satt};
#pragma unroll
    for (int k = 0; k < 6; k++) v[k] = warp_sum(v[k]);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 6; k++) red[warp * 16 + k] = v[k];
    }
    __syncthreads();
    if (tid < 6) {
        double s = 0.0;
        for (int q = 0; q < (nthreads >> 5); q++) s += red[q * 16 + tid];
        SnAccum *A = a.acc + w.rep;
        if (tid == 0) atomicAdd(&A->dE, s);
        else if (tid < 4) atomicAdd(&A->dP[tid - 1], s);
        else if (tid == 4) atomicAdd(&A->acc, (unsigned long long)s);
        else atomicAdd(&A->att, (unsigned long long)s);
    }
}

// ---------------------------------------------------------------------------
// Full local-field pass (energy recompute, site energies, adjoint).  Same
// tiles, stencil and thread roles as the sweep, read-only, every block of
// the replica in one launch.  R = float: FP32 local fields, FP64 site
// products and sums; R = double: every operation in FP64.
//   red[rep*red_stride + k]: 0 E_dd = 1/2 sum len_i p_i.H_i   1 sum p_i.nn_i
//                    2 sum p_i.E                       3 sum K term
//                    4..6 sum len_i p_i                7..9 sum p_i
// where H_i = sum_j len_j T_o p_j is the dipole field at site i.
struct SnFieldArgs {
    const SnWork *work;
    const SnReplicaDev *reps;
    const SnTile *geoms;
    double cage;
    double K;
    double *site_e;  // nullable: N doubles
    float *grad;     // nullable: 3N floats (interleaved)
    double *red;     // 10 doubles per replica
    int red_stride;  // doubles between replicas in red (0: all replicas share one slot)
    int write_g;     // 1: refresh the replica's local-field cache (SnReplicaDev::gcache)
};

}  // namespace sn_sweep

#include "sn_sweep_cached.cuh"

namespace sn_sweep {

// Block size limits of a sweep kernel variant: the stencil-sum sweep (its
// thread count varies with the block shape) or the cached-field sweep (fixed).
template <bool CACHED>
struct SweepBounds {
    static constexpr int threads = CACHED ? SN_CACHED_THREADS : SN_SWEEP_MAX_THREADS;
    static constexpr int min_blocks = CACHED ? 2 : SN_SWEEP_MIN_BLOCKS;
};

template <int RC, bool TWO_D, bool MIXED, bool CACHED, bool FLOW>
__device__ __forceinline__ void sweep_block_any(const SnWork w, const SnPhaseArgs &a, unsigned char *smem, bool first,
                                                CStats *cst = nullptr)
{
    if constexpr (CACHED && !TWO_D) sweep_block_cached<RC, MIXED, FLOW>(w, a, smem, first, cst);
    else sweep_block<RC, TWO_D, MIXED, FLOW>(w, a, smem);
}

// One block colour per launch, one CTA per block.
template <int RC, bool TWO_D, bool MIXED, bool CACHED>
__global__ void __launch_bounds__(SweepBounds<CACHED>::threads, SweepBounds<CACHED>::min_blocks)
    sweep_phase(const SnPhaseArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    sweep_block_any<RC, TWO_D, MIXED, CACHED, false>(a.work[blockIdx.x], a, smem, true);
}

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t *p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_gpu(uint32_t *p, uint32_t v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Dataflow sweep: one persistent launch per sweep.  Every CTA is resident
// (the host sizes the grid with the occupancy API) and takes blocks from a
// queue ordered by block colour.  Before updating a block it waits until
// each adjacent block of an earlier colour has finished this sweep (a spin
// bounded by err[3] polls; on time-out it records SN_ERR_TIMEOUT in err[0]
// and goes on, so the launch always ends).
// Adjacent blocks of later colours wait for this one in turn, so every block
// sees exactly the lattice the phase-by-phase order gives it.  Deadlock
// cannot occur: a block waited on was taken from the queue earlier by a CTA
// that is running, and it only waits on blocks taken before it.
template <int RC, bool TWO_D, bool MIXED, bool CACHED>
__global__ void __launch_bounds__(SweepBounds<CACHED>::threads, SweepBounds<CACHED>::min_blocks)
    sweep_flow(const SnFlowArgs f)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_item;
    // cached sweep: each thread's move statistics over the CTA's blocks of
    // replica cur_rep, added to the replica's totals when the replica changes
    // and at the end (not reduced and added on every block)
    CStats st;
    int cur_rep = -1;
    const int tid = threadIdx.x;
    const uint32_t epoch = *f.base.sweep + 1u;
    bool first = true;  // this CTA's first block (per-CTA shared-memory tables)
    const bool reserve = f.base.n_work >= 16 * (int)gridDim.x;
    if (tid == 0) s_item = (int)atomicAdd(f.queue, 1u);
    __syncthreads();
    int item = s_item;
    for (;;) {
        __syncthreads();  // every thread has read s_item
        if (item >= f.base.n_work) break;
        // With many blocks per CTA the next block is taken now, so the
        // queue's latency overlaps this block (no deadlock: the earliest
        // unfinished block in queue order waits on finished blocks only, and
        // its CTA is done with any earlier one).  With few, a block taken
        // early holds up the blocks that depend on it, so it is taken after
        // this one (1.02 against 0.82 ms per sweep at 128^3, cutoff 4).
        if (reserve && tid == 0) s_item = (int)atomicAdd(f.queue, 1u);
        const int *dl = f.deps + (size_t)item * SN_MAX_DEPS;
        if (tid < dl[0]) {
            const uint32_t *flag = f.done + dl[1 + tid];
            const uint32_t limit = __ldcg(f.err + 3);
            uint32_t it = 0;
            for (; ld_acquire_gpu(flag) < epoch; it++) {
                if (it >= limit) {
                    atomicOr(f.err, 1u);
                    break;
                }
                __nanosleep(100);
            }
            if (it) {  // dependency stall statistics
                atomicAdd(f.err + 1, 1u);
                atomicAdd(f.err + 2, (unsigned)it);
            }
        }
        if constexpr (CACHED && !TWO_D) {
            const int rep = f.base.work[item].rep;  // the same for every thread
            if (rep != cur_rep) {
                if (cur_rep >= 0) flush_cstats(st, reinterpret_cast<double *>(smem), f.base.acc + cur_rep);
                cur_rep = rep;
            }
        }
        // Ordering: the waiting threads' acquire loads of the dependencies'
        // flags, then the barrier, make the producers' writes visible to
        // every thread's later loads.  The cached sweep reads other blocks'
        // data only through L2 (its tile by cp.async.cg, or by TMA after
        // fence.proxy.async); the stencil sweep stages neighbours' dipoles
        // through L1 (cp.async.ca), so each of its threads also fences.
        // After the block, the barrier and thread 0's release store publish
        // the whole CTA's writes (release is cumulative over the barrier).
        __syncthreads();
        if constexpr (!CACHED) __threadfence();
        sweep_block_any<RC, TWO_D, MIXED, CACHED, true>(f.base.work[item], f.base, smem, first, &st);
        first = false;
        __syncthreads();
        if (tid == 0) st_release_gpu(f.done + item, epoch);
        if (!reserve && tid == 0) s_item = (int)atomicAdd(f.queue, 1u);
        __syncthreads();
        item = s_item;
    }
    if constexpr (CACHED && !TWO_D) {
        if (cur_rep >= 0) flush_cstats(st, reinterpret_cast<double *>(smem), f.base.acc + cur_rep);
    }
}

template <typename R, int RC, bool TWO_D, bool MIXED>
__global__ void __launch_bounds__(SN_MAX_THREADS, 1) field_tiled(const SnFieldArgs a)
{
    using G = Geo<RC, TWO_D>;
    constexpr int S = G::S, H = G::H, HZ = G::HZ, SZ = G::SZ, NF = G::NF, NP = G::NP;
    constexpr bool MERGE = G::MERGE;
    extern __shared__ __align__(16) unsigned char smem[];

    const int tid = threadIdx.x, nthreads = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5;
    const SnWork w = a.work[blockIdx.x];
    const SnReplicaDev &Rp = a.reps[w.rep];
    const SnTile &Gm = a.geoms[Rp.geom];
    const int Y = Rp.Y, Z = Rp.Z;
    const float *__restrict__ gpx = Rp.px;
    const float *__restrict__ gpy = Rp.py;
    const float *__restrict__ gpz = Rp.pz;
    const float *__restrict__ glen = Rp.len;
    const int Bx = Gm.B[0], By = Gm.B[1], Bz = Gm.B[2];
    const int Sy = Gm.Sy, Sx = Gm.Sx;
    const int tp = Gm.tp, tg = Gm.tg, ng = Gm.ng;
    const int nqy = Gm.nq[1], nqz = Gm.nq[2];
    const R C = (R)a.cage, Kk = (R)a.K;
    const R Ex = (R)Rp.E[0], Ey = (R)Rp.E[1], Ez = (R)Rp.E[2];
    const R Lu = (R)Rp.length;

    const Carve cv = sn_carve(Gm.slots, tg, 0, G::NS, S, NF, MIXED, (int)sizeof(R));
    float *tlen = reinterpret_cast<float *>(smem + cv.tlen);
    int *ftab = reinterpret_cast<int *>(smem + cv.ftab);
    int *start = reinterpret_cast<int *>(smem + cv.start);
    double *red = reinterpret_cast<double *>(smem + cv.red);

    build_tables<RC, TWO_D>(Gm, start, ftab, tid, nthreads);
    stage_tile<RC, TWO_D, MIXED>(Rp, Gm, w, reinterpret_cast<float *>(smem + cv.tile), tlen, start, tid, nthreads);
    cp_async_wait_all();
    __syncthreads();

    // Read-only pass: every (colour group, target) of the block is an
    // independent item; a thread runs the whole stencil of its items, so the
    // loop needs no barrier.  Lanes of a warp take consecutive targets of one
    // group, the conflict-free pattern of the tile layout.
    // Sums 0 (1/2) L p.H, 1 p.nn, 2 p.E, 3 K term, 4-6 L p, 7-9 p: in FP64 for
    // the FP64 pass; for the FP32 pass compensated FP32 sums per thread
    // (FP64 is a slow pipe on this GPU), combined by TwoSum within warps.
    double acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    KahanF facc[10];
    auto add = [&](int k, R v) {
        if constexpr (sizeof(R) == 4) facc[k].add(v);
        else acc[k] += (double)v;
    };
    const int items = ng * tg;
    for (int it = tid; it < items; it += nthreads) {
        const int g = it / tg, tt = it - (it / tg) * tg;
        const int hh = tt / tp, t = tt - (tt / tp) * tp;
        const int qz = t % nqz, qy = (t / nqz) % nqy, qx = t / (nqz * nqy);
        int cx, cy, cz;
        group_colour<S, SZ, MERGE>(g, hh, cx, cy, cz);
        if (!(qx < Gm.nq[0] && qx < sn_count(Bx, cx, S) && qy < sn_count(By, cy, S) &&
              (TWO_D || qz < sn_count(Bz, cz, S))))
            continue;
        int FX[NF], FY[NF];
#pragma unroll
        for (int o = 0; o < NF; o++) {
            FX[o] = ftab[(0 * S + cx) * NF + o];
            FY[o] = ftab[(1 * S + cy) * NF + o];
        }
        const int tslot = sn_pi<S>(start, cx + H) * Sx + sn_pi<S>(start + SN_MAX_S, cy + H) * Sy +
                          (TWO_D ? 0 : cz + HZ) + qx * Sx + qy * Sy + S * qz;
        R hacc[SN_ACC_SETS][3] = {};
        R nnv[3] = {0, 0, 0};
        if constexpr (sizeof(R) == 4) {
            run_pairs<R, RC, TWO_D, MIXED, 0>(std::make_integer_sequence<int, NP>{}, smem + cv.tile,
                                              (uint32_t)tslot * 12u, FX, FY, tlen, (uint32_t)tslot, hacc, nnv);
        } else {
            // FP64 validation mode: one stencil slice at a time keeps the double registers in check
#pragma unroll 1
            for (int j = 0; j < G::NS; j++)
                dispatch_split<R, RC, TWO_D, MIXED, 0>(j, smem + cv.tile, (uint32_t)tslot * 12u, FX, FY, tlen,
                                                       (uint32_t)tslot, hacc, nnv);
        }
        const R hx = sum_sets(hacc, 0), hy = sum_sets(hacc, 1), hz = sum_sets(hacc, 2);
        const long long site = ((long long)(w.x0 + cx + S * qx) * Y + (w.y0 + cy + S * qy)) * Z +
                               (TWO_D ? 0 : w.z0 + cz + S * qz);
        const R px = (R)gpx[site], py = (R)gpy[site], pz = (R)gpz[site];
        const R Li = (R)glen[site];  // 0 at vacancies in both modes
        if (a.write_g && Rp.gcache) {
            // the cached-field sweep's g = len_i H_i - C nn_i (no applied field), fixed point
            const R scl = MIXED ? R(1) : Lu;
            const R s = (R)Rp.gscale;
            const size_t Nn = (size_t)Rp.n_sites;
            Rp.gcache[site] = fixed_point(s * (Li * scl * hx - C * nnv[0]));
            Rp.gcache[Nn + site] = fixed_point(s * (Li * scl * hy - C * nnv[1]));
            Rp.gcache[2 * Nn + site] = fixed_point(s * (Li * scl * hz - C * nnv[2]));
        }
        if (Li == R(0)) {
            if (a.site_e) a.site_e[site] = 0.0;
            if (a.grad) {
                a.grad[3 * site + 0] = 0.0f;
                a.grad[3 * site + 1] = 0.0f;
                a.grad[3 * site + 2] = 0.0f;
            }
            continue;
        }
        // H = sum_j len_j T p_j: uniform tiles hold unit p (H = L h).  Site
        // products in R (FP32 fields: FP32 products, FP64 sums)
        const R sc = MIXED ? R(1) : Lu;
        const R Hx = sc * hx, Hy = sc * hy, Hz = sc * hz;
        const R gx = Li * Hx - C * nnv[0] + Ex;
        const R gy = Li * Hy - C * nnv[1] + Ey;
        const R gz = Li * Hz - C * nnv[2] + Ez;
        const R kt = Kk > R(0) ? -Kk * (fabs(px) + fabs(py)) : R(0);
        const R pH = px * Hx + py * Hy + pz * Hz;
        const R pn = px * nnv[0] + py * nnv[1] + pz * nnv[2];
        const R pE = px * Ex + py * Ey + pz * Ez;
        if (a.site_e) a.site_e[site] = (double)(px * gx + py * gy + pz * gz + kt);
        if (a.grad) {
            const R sx = Kk > R(0) ? (px > R(0) ? R(1) : (px < R(0) ? R(-1) : R(0))) : R(0);
            const R sy = Kk > R(0) ? (py > R(0) ? R(1) : (py < R(0) ? R(-1) : R(0))) : R(0);
            a.grad[3 * site + 0] = (float)(gx - Kk * sx);
            a.grad[3 * site + 1] = (float)(gy - Kk * sy);
            a.grad[3 * site + 2] = (float)gz;
        }
        add(0, Li * pH);  // halved below
        add(1, pn);
        add(2, pE);
        add(3, kt);
        add(4, Li * px);
        add(5, Li * py);
        add(6, Li * pz);
        add(7, px);
        add(8, py);
        add(9, pz);
    }
    if constexpr (sizeof(R) == 4) {
        float hs[10], hc[10];
#pragma unroll
        for (int k = 0; k < 10; k++) {
            hs[k] = facc[k].s;
            hc[k] = -facc[k].c;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int k = 0; k < 10; k++) {
                const float bs = __shfl_xor_sync(0xffffffffu, hs[k], o), bc = __shfl_xor_sync(0xffffffffu, hc[k], o);
                const float t2 = __fadd_rn(hs[k], bs);
                const float bb = __fsub_rn(t2, hs[k]);
                const float err = __fadd_rn(__fsub_rn(hs[k], __fsub_rn(t2, bb)), __fsub_rn(bs, bb));
                hs[k] = t2;
                hc[k] = __fadd_rn(__fadd_rn(hc[k], bc), err);
            }
        }
#pragma unroll
        for (int k = 0; k < 10; k++) acc[k] = (double)hs[k] + (double)hc[k];
    } else {
#pragma unroll
        for (int k = 0; k < 10; k++) acc[k] = warp_sum(acc[k]);
    }
    acc[0] *= 0.5;
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 10; k++) red[warp * 16 + k] = acc[k];
    }
    __syncthreads();
    if (tid < 10) {
        double s = 0.0;
        for (int q = 0; q < (nthreads >> 5); q++) s += red[q * 16 + tid];
        atomicAdd(&a.red[a.red_stride * w.rep + tid], s);
    }
}

// The dynamic shared-memory limit of a kernel is a per-device attribute: it
// is set once per (kernel variant, device), tracked by one bit per variant in
// a per-device mask (a second host thread may set it again: harmless).
#define SN_ATTR_MAX_DEVICES 64
struct SnAttrOnce {
    std::atomic<uint32_t> mask[SN_ATTR_MAX_DEVICES];
};

template <typename F>
cudaError_t set_smem_once(SnAttrOnce &once, int idx, F fn, int static_bytes)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint32_t bit = 1u << idx;
    const bool tracked = dev >= 0 && dev < SN_ATTR_MAX_DEVICES;
    if (tracked && (once.mask[dev].load(std::memory_order_acquire) & bit)) return cudaSuccess;
    if (static_bytes < 0) {  // static shared memory of the kernel comes off the 227 KB
        cudaFuncAttributes fa;
        e = cudaFuncGetAttributes(&fa, fn);
        if (e != cudaSuccess) return e;
        static_bytes = (int)fa.sharedSizeBytes;
    }
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024 - static_bytes);
    if (e == cudaSuccess && tracked) once.mask[dev].fetch_or(bit, std::memory_order_release);
    return e;
}

template <typename R, int RC>
cudaError_t launch_field_rc(bool two_d, bool mixed, const SnFieldArgs &args, int grid, int threads, int smem_bytes,
                            cudaStream_t st)
{
    static SnAttrOnce once;
    const int idx = (two_d ? 2 : 0) + (mixed ? 1 : 0);
    void (*fn)(const SnFieldArgs);
    if (two_d) fn = mixed ? field_tiled<R, RC, true, true> : field_tiled<R, RC, true, false>;
    else fn = mixed ? field_tiled<R, RC, false, true> : field_tiled<R, RC, false, false>;
    if (cudaError_t e = set_smem_once(once, idx, fn, 0)) return e;
    if (grid <= 0) return cudaSuccess;
    fn<<<grid, threads, smem_bytes, st>>>(args);
    return cudaGetLastError();
}

// The cached-field variants exist for 3D lattices only.
template <int RC>
cudaError_t launch_rc(bool two_d, bool mixed, bool cached, const SnPhaseArgs &args, int grid, int threads,
                      int smem_bytes, cudaStream_t st)
{
    static SnAttrOnce once;
    if (cached && two_d) return cudaErrorNotSupported;
    const int idx = (cached ? 4 : 0) + (two_d ? 2 : 0) + (mixed ? 1 : 0);
    void (*fn)(const SnPhaseArgs);
    if (cached) fn = mixed ? sweep_phase<RC, false, true, true> : sweep_phase<RC, false, false, true>;
    else if (two_d) fn = mixed ? sweep_phase<RC, true, true, false> : sweep_phase<RC, true, false, false>;
    else fn = mixed ? sweep_phase<RC, false, true, false> : sweep_phase<RC, false, false, false>;
    if (cudaError_t e = set_smem_once(once, idx, fn, 0)) return e;
    if (grid <= 0) return cudaSuccess;
    fn<<<grid, threads, smem_bytes, st>>>(args);
    return cudaGetLastError();
}

template <int RC>
cudaError_t launch_flow_rc(bool two_d, bool mixed, bool cached, const SnFlowArgs &args, int grid, int threads,
                           int smem_bytes, cudaStream_t st, int *max_grid)
{
    static SnAttrOnce once;
    if (cached && two_d) return cudaErrorNotSupported;
    const int idx = (cached ? 4 : 0) + (two_d ? 2 : 0) + (mixed ? 1 : 0);
    void (*fn)(const SnFlowArgs);
    if (cached) fn = mixed ? sweep_flow<RC, false, true, true> : sweep_flow<RC, false, false, true>;
    else if (two_d) fn = mixed ? sweep_flow<RC, true, true, false> : sweep_flow<RC, true, false, false>;
    else fn = mixed ? sweep_flow<RC, false, true, false> : sweep_flow<RC, false, false, false>;
    // the queue slot is static shared memory: the dynamic limit is what remains of 227 KB
    if (cudaError_t e = set_smem_once(once, idx, fn, -1)) return e;
    if (max_grid) {
        int per_sm = 0, dev = 0, nsm = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem_bytes);
        if (e == cudaSuccess) e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        *max_grid = per_sm * nsm;
    }
    if (grid <= 0) return cudaSuccess;
    fn<<<grid, threads, smem_bytes, st>>>(args);
    return cudaGetLastError();
}

template <int RC>
cudaError_t launch_gfield_rc(bool mixed, const SnFieldArgs &args, int grid, int smem_bytes, cudaStream_t st)
{
    static SnAttrOnce once;
    void (*fn)(const SnFieldArgs) = mixed ? gfield_tiled<RC, true> : gfield_tiled<RC, false>;
    if (cudaError_t e = set_smem_once(once, mixed ? 1 : 0, fn, 0)) return e;
    if (grid <= 0) return cudaSuccess;
    fn<<<grid, SN_GFIELD_THREADS, smem_bytes, st>>>(args);
    return cudaGetLastError();
}

// Compile-time sizes the host planner needs.
template <int RC>
inline void geo_sizes(bool two_d, int &S, int &SZ, int &NS, int &NF, int &merge)
{
    if (two_d) {
        S = Geo<RC, true>::S;
        SZ = Geo<RC, true>::SZ;
        NS = Geo<RC, true>::NS;
        NF = Geo<RC, true>::NF;
        merge = Geo<RC, true>::MERGE;
    } else {
        S = Geo<RC, false>::S;
        SZ = Geo<RC, false>::SZ;
        NS = Geo<RC, false>::NS;
        NF = Geo<RC, false>::NF;
        merge = Geo<RC, false>::MERGE;
    }
}

}  // namespace sn_sweep
