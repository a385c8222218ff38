// sn_sweep.cuh -- the Metropolis sweep kernel (one block colour per launch).
//
// Schedule.  A replica's lattice is cut into blocks of B = (bx,by,bz) sites;
// blocks get a checkerboard colour (block index mod 2 per axis).  One launch
// handles every block of one block colour, one CTA per block.  Two blocks of
// the same colour are at least one block (>= cutoff sites) apart, so they
// never interact and their CTAs run independently; each CTA reads its halo
// (cutoff sites around the block) from blocks of other colours, which no
// CTA of this launch writes.  Inside the block the CTA visits the s^3 site
// colours (local coordinate mod s, s = cutoff + 1) in order; sites of one
// site colour are >= s apart and are updated together.  Every occupied site
// is attempted exactly once per sweep: the same set of moves as MC_moves
// over X*Y*Z steps (src/starrynight-montecarlo-core.c:143-191), in a
// different but fixed order.
//
// Per site colour:
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
    static constexpr int NS = (NP + 7) / 15 < 1 ? 1 : ((NP + 7) / 15 > 16 ? 16 : (NP + 7) / 15);
};

__device__ __forceinline__ float sn_fma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double sn_fma(double a, double b, double c) { return fma(a, b, c); }

// ---------------------------------------------------------------------------
// One +-o pair of the stencil.
template <typename R, int RC, bool TWO_D, bool MIXED, int I>
__device__ __forceinline__ void pair_step(const unsigned char *__restrict__ base, uint32_t tb,
                                          const int (&FX)[2 * RC + 1], const int (&FY)[2 * RC + 1],
                                          const int (&FZ)[2 * RC + 1], const float *__restrict__ tlen,
                                          uint32_t tslot, R (&h)[2][3], R (&nn)[3])
{
    constexpr sn_stencil::Off o = sn_stencil::pair_offset(RC, TWO_D, I);
    constexpr int H = RC;
    // signed byte offsets: neighbours below the target give negative deltas;
    // tb + delta stays inside the tile because |o| <= halo.
    const int ao = FX[H + o.x] + FY[H + o.y] + FZ[H + o.z];
    const int bo = FX[H - o.x] + FY[H - o.y] + FZ[H - o.z];
    const float *pa = reinterpret_cast<const float *>(base + ((int)tb + ao));
    const float *pb = reinterpret_cast<const float *>(base + ((int)tb + bo));
    const R ax = pa[0], ay = pa[1], az = pa[2];
    const R bx = pb[0], by = pb[1], bz = pb[2];
    const R qx = ax + bx, qy = ay + by, qz = az + bz;
    constexpr R txx = (R)sn_stencil::tensor_d(o.x, o.y, o.z, 0);
    constexpr R tyy = (R)sn_stencil::tensor_d(o.x, o.y, o.z, 1);
    constexpr R tzz = (R)sn_stencil::tensor_d(o.x, o.y, o.z, 2);
    constexpr R txy = (R)sn_stencil::tensor_d(o.x, o.y, o.z, 3);
    constexpr R txz = (R)sn_stencil::tensor_d(o.x, o.y, o.z, 4);
    constexpr R tyz = (R)sn_stencil::tensor_d(o.x, o.y, o.z, 5);
    R(&a)[3] = h[I & 1];
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
        if constexpr (MIXED) {
            // the tile holds len*p; the cage-strain term wants unit p
            const R la = tlen[(int)tslot + ao / 12], lb = tlen[(int)tslot + bo / 12];
            const R ia = la > R(0) ? R(1) / la : R(0), ib = lb > R(0) ? R(1) / lb : R(0);
            nn[0] += ax * ia + bx * ib;
            nn[1] += ay * ia + by * ib;
            nn[2] += az * ia + bz * ib;
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
                                          const int (&FZ)[2 * RC + 1], const float *tlen, uint32_t tslot,
                                          R (&h)[2][3], R (&nn)[3])
{
    (pair_step<R, RC, TWO_D, MIXED, LO + Is>(base, tb, FX, FY, FZ, tlen, tslot, h, nn), ...);
}

template <typename R, int RC, bool TWO_D, bool MIXED, int J>
__device__ __forceinline__ void dispatch_split(int j, const unsigned char *base, uint32_t tb,
                                               const int (&FX)[2 * RC + 1], const int (&FY)[2 * RC + 1],
                                               const int (&FZ)[2 * RC + 1], const float *tlen, uint32_t tslot,
                                               R (&h)[2][3], R (&nn)[3])
{
    using G = Geo<RC, TWO_D>;
    if constexpr (J < G::NS) {
        if (j == J) {
            constexpr int lo = J * G::NP / G::NS, hi = (J + 1) * G::NP / G::NS;
            run_pairs<R, RC, TWO_D, MIXED, lo>(std::make_integer_sequence<int, hi - lo>{}, base, tb, FX, FY, FZ,
                                                tlen, tslot, h, nn);
        } else {
            dispatch_split<R, RC, TWO_D, MIXED, J + 1>(j, base, tb, FX, FY, FZ, tlen, tslot, h, nn);
        }
    }
}

__device__ __forceinline__ int sn_wrap(int v, int L) { return v < 0 ? v + L : (v >= L ? v - L : v); }

template <int S>
__device__ __forceinline__ int sn_pi(const int *start, int u) { return start[u % S] + u / S; }

__device__ __forceinline__ int sn_count(int B, int c, int S) { return c < B ? (B - c + S - 1) / S : 0; }

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Shared-memory carve-up, identical on host (sizing) and device.
struct Carve {
    uint32_t tile, tlen, props, psite, parts, ftab, start, red, total;
};

__host__ __device__ inline uint32_t sn_align16(uint32_t v) { return (v + 15u) & ~15u; }

__host__ __device__ inline Carve sn_carve(int slots, int maxt, int S, int SZ, int NS, int NF, bool mixed)
{
    Carve c;
    uint32_t o = 0;
    c.tile = o;
    o += sn_align16((uint32_t)slots * 12u);
    c.tlen = o;
    if (mixed) o += sn_align16((uint32_t)slots * 4u);
    c.props = o;
    o += (uint32_t)(S * SZ * maxt) * 16u;
    c.psite = o;
    o += sn_align16((uint32_t)(S * SZ * maxt) * 4u);
    c.parts = o;
    o += sn_align16((uint32_t)(NS * 6 * maxt) * 8u);  // room for FP64 partials (field kernel)
    c.ftab = o;
    o += sn_align16((uint32_t)(3 * S * NF) * 4u);
    c.start = o;
    o += sn_align16(3u * SN_MAX_S * 4u);
    c.red = o;
    o += (SN_THREADS / 32) * 16u * 8u;
    c.total = o;
    return c;
}

// ---------------------------------------------------------------------------
template <int RC, bool TWO_D, bool MIXED>
__global__ void __launch_bounds__(SN_THREADS, 1) sweep_phase(const SnPhaseArgs a)
{
    using G = Geo<RC, TWO_D>;
    constexpr int S = G::S, H = G::H, HZ = G::HZ, SZ = G::SZ, NF = G::NF, NS = G::NS;
    extern __shared__ __align__(16) unsigned char smem[];

    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const SnWork w = a.work[blockIdx.x];
    const SnReplicaDev &R = a.reps[w.rep];
    const SnTile &Gm = a.geoms[R.geom];

    const int X = R.X, Y = R.Y, Z = R.Z;
    float *__restrict__ gpx = R.px;
    float *__restrict__ gpy = R.py;
    float *__restrict__ gpz = R.pz;
    const float *__restrict__ glen = R.len;
    const int Bx = Gm.B[0], By = Gm.B[1], Bz = Gm.B[2];
    const int Tx = Gm.T[0], Ty = Gm.T[1], Tz = Gm.T[2];
    const int Sy = Gm.Sy, Sx = Gm.Sx, maxt = Gm.maxt;
    const uint32_t sweep = *a.sweep;
    const uint2 key = make_uint2(R.seed_lo, R.seed_hi);
    const float beta = R.beta;
    const float Ex = R.E[0], Ey = R.E[1], Ez = R.E[2];
    const float C = a.cage, Kk = a.K;
    const float Lu = R.length;
    const float gscale = MIXED ? 1.0f : Lu * Lu;

    const Carve cv = sn_carve(Gm.slots, maxt, S, SZ, NS, NF, MIXED);
    float *tile = reinterpret_cast<float *>(smem + cv.tile);
    float *tlen = reinterpret_cast<float *>(smem + cv.tlen);
    float4 *props = reinterpret_cast<float4 *>(smem + cv.props);
    int *psite = reinterpret_cast<int *>(smem + cv.psite);
    float *parts = reinterpret_cast<float *>(smem + cv.parts);
    int *ftab = reinterpret_cast<int *>(smem + cv.ftab);
    int *start = reinterpret_cast<int *>(smem + cv.start);
    double *red = reinterpret_cast<double *>(smem + cv.red);

    // ---- geometry tables ---------------------------------------------------
    if (tid < 3 * SN_MAX_S) start[tid] = Gm.start[tid / SN_MAX_S][tid % SN_MAX_S];
    __syncthreads();
    for (int i = tid; i < 3 * S * NF; i += SN_THREADS) {
        const int ax = i / (S * NF), c = (i / NF) % S, o = i % NF - H;
        int v = 0;
        const int Ha = ax == 2 ? HZ : H;
        const int T = Gm.T[ax];
        const int u0 = c + Ha, u = u0 + o;
        if (!(ax == 2 && TWO_D) && u >= 0 && u < T && u0 < T) {
            const int *st = start + ax * SN_MAX_S;
            const int d = sn_pi<S>(st, u) - sn_pi<S>(st, u0);
            const int stride = ax == 0 ? Sx : (ax == 1 ? Sy : 1);
            v = d * stride * 12;
        }
        ftab[i] = v;
    }

    // ---- stage block + halo (periodic wrap) ------------------------------------
    for (int row = warp; row < Tx * Ty; row += SN_THREADS / 32) {
        const int ux = row / Ty, uy = row - (row / Ty) * Ty;
        const int gx = sn_wrap(w.x0 - H + ux, X), gy = sn_wrap(w.y0 - H + uy, Y);
        const int rslot = sn_pi<S>(start, ux) * Sx + sn_pi<S>(start + SN_MAX_S, uy) * Sy;
        const long long gb = ((long long)gx * Y + gy) * Z;
        for (int uz = lane; uz < Tz; uz += 32) {
            const int gz = TWO_D ? 0 : sn_wrap(w.z0 - HZ + uz, Z);
            const long long g = gb + gz;
            const int slot = rslot + (TWO_D ? 0 : sn_pi<S>(start + 2 * SN_MAX_S, uz));
            float x = gpx[g], y = gpy[g], z = gpz[g];
            if constexpr (MIXED) {
                const float L = glen[g];
                tlen[slot] = L;
                x *= L;
                y *= L;
                z *= L;
            }
            tile[3 * slot + 0] = x;
            tile[3 * slot + 1] = y;
            tile[3 * slot + 2] = z;
        }
    }
    __syncthreads();

    double sdE = 0.0, sPx = 0.0, sPy = 0.0, sPz = 0.0;
    unsigned int sacc = 0, satt = 0;

    for (int cx = 0; cx < S; cx++) {
        const int nxc = sn_count(Bx, cx, S);
        if (nxc == 0) continue;
        // ---- proposals for every (cy, cz) of this cx: independent of the lattice
        for (int i = tid; i < S * SZ * maxt; i += SN_THREADS) {
            const int k = i / maxt, t = i - k * maxt;
            const int cy = k / SZ, cz = k - cy * SZ;
            const int nyc = sn_count(By, cy, S), nzc = TWO_D ? 1 : sn_count(Bz, cz, S);
            if (t >= nxc * nyc * nzc) continue;
            const int qz = t % nzc, r = t / nzc, qy = r % nyc, qx = r / nyc;
            const int lx = cx + S * qx, ly = cy + S * qy, lz = TWO_D ? 0 : cz + S * qz;
            const int site = ((w.x0 + lx) * Y + (w.y0 + ly)) * Z + (w.z0 + lz);
            const int slot = sn_pi<S>(start, lx + H) * Sx + sn_pi<S>(start + SN_MAX_S, ly + H) * Sy +
                             (TWO_D ? 0 : sn_pi<S>(start + 2 * SN_MAX_S, lz + HZ));
            bool occ;
            if constexpr (MIXED) occ = tlen[slot] != 0.0f;
            else occ = tile[3 * slot] != 0.0f || tile[3 * slot + 1] != 0.0f || tile[3 * slot + 2] != 0.0f;
            float4 pr = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
            if (occ) {
                float3 p;
                float u;
                if (!sn_proposal((uint32_t)site, sweep, SN_STREAM_SWEEP, key, a.dim, a.constrain, p, u))
                    p = make_float3(gpx[site], gpy[site], gpz[site]);
                pr = make_float4(p.x, p.y, p.z, u);
            }
            props[i] = pr;
            psite[i] = site;
        }
        __syncthreads();
        int FX[NF];
#pragma unroll
        for (int o = 0; o < NF; o++) FX[o] = ftab[(0 * S + cx) * NF + o];
        const int bx0 = sn_pi<S>(start, cx + H);

        for (int cy = 0; cy < S; cy++) {
            const int nyc = sn_count(By, cy, S);
            if (nyc == 0) continue;
            int FY[NF];
#pragma unroll
            for (int o = 0; o < NF; o++) FY[o] = ftab[(1 * S + cy) * NF + o];
            const int by0 = sn_pi<S>(start + SN_MAX_S, cy + H);

            for (int cz = 0; cz < SZ; cz++) {
                const int nzc = TWO_D ? 1 : sn_count(Bz, cz, S);
                const int nt = nxc * nyc * nzc;
                if (nt == 0) continue;
                int FZ[NF];
#pragma unroll
                for (int o = 0; o < NF; o++) FZ[o] = TWO_D ? 0 : ftab[(2 * S + cz) * NF + o];
                const int bz0 = TWO_D ? 0 : sn_pi<S>(start + 2 * SN_MAX_S, cz + HZ);
                const int ntp = (nt + 31) & ~31;

                // ---- 1. partial local fields ----------------------------------
                for (int wi = tid; wi < NS * ntp; wi += SN_THREADS) {
                    const int j = wi / ntp, t = wi - j * ntp;
                    if (t < nt) {
                        const int qz = t % nzc, r = t / nzc, qy = r % nyc, qx = r / nyc;
                        const uint32_t tslot = (uint32_t)((bx0 + qx) * Sx + (by0 + qy) * Sy + bz0 + qz);
                        float hacc[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
                        float nn[3] = {0.f, 0.f, 0.f};
                        dispatch_split<float, RC, TWO_D, MIXED, 0>(j, smem + cv.tile, tslot * 12u, FX, FY, FZ, tlen, tslot,
                                                            hacc, nn);
                        float *pp = parts + (j * 6) * maxt + t;
                        pp[0 * maxt] = hacc[0][0] + hacc[1][0];
                        pp[1 * maxt] = hacc[0][1] + hacc[1][1];
                        pp[2 * maxt] = hacc[0][2] + hacc[1][2];
                        pp[3 * maxt] = nn[0];
                        pp[4 * maxt] = nn[1];
                        pp[5 * maxt] = nn[2];
                    }
                }
                __syncthreads();

                // ---- 2. finalize: dE, accept, update --------------------------
                for (int t = tid; t < nt; t += SN_THREADS) {
                    const int pk = (cy * SZ + cz) * maxt + t;
                    const float4 pr = props[pk];
                    if (pr.w < 0.0f) continue;  // vacancy
                    float hx = 0.f, hy = 0.f, hz = 0.f, nx = 0.f, ny = 0.f, nz = 0.f;
#pragma unroll
                    for (int j = 0; j < NS; j++) {
                        const float *pp = parts + (j * 6) * maxt + t;
                        hx += pp[0 * maxt];
                        hy += pp[1 * maxt];
                        hz += pp[2 * maxt];
                        nx += pp[3 * maxt];
                        ny += pp[4 * maxt];
                        nz += pp[5 * maxt];
                    }
                    const int qz = t % nzc, r = t / nzc, qy = r % nyc, qx = r / nyc;
                    const int tslot = (bx0 + qx) * Sx + (by0 + qy) * Sy + bz0 + qz;
                    const int site = psite[pk];
                    float Li, ox, oy, oz;
                    if constexpr (MIXED) {
                        Li = tlen[tslot];
                        ox = gpx[site];
                        oy = gpy[site];
                        oz = gpz[site];
                    } else {
                        Li = Lu;
                        ox = tile[3 * tslot + 0];
                        oy = tile[3 * tslot + 1];
                        oz = tile[3 * tslot + 2];
                    }
                    const float sc = MIXED ? Li : gscale;
                    const float gx = fmaf(sc, hx, fmaf(-C, nx, Ex));
                    const float gy = fmaf(sc, hy, fmaf(-C, ny, Ey));
                    const float gz = fmaf(sc, hz, fmaf(-C, nz, Ez));
                    const float dx = pr.x - ox, dy = pr.y - oy, dz = pr.z - oz;
                    float dE = fmaf(dx, gx, fmaf(dy, gy, dz * gz));
                    if (Kk > 0.0f) dE -= Kk * ((fabsf(pr.x) - fabsf(ox)) + (fabsf(pr.y) - fabsf(oy)));
                    satt++;
                    const bool acc = (dE < 0.0f) || (expf(-beta * dE) > pr.w);
                    if (acc) {
                        tile[3 * tslot + 0] = MIXED ? Li * pr.x : pr.x;
                        tile[3 * tslot + 1] = MIXED ? Li * pr.y : pr.y;
                        tile[3 * tslot + 2] = MIXED ? Li * pr.z : pr.z;
                        gpx[site] = pr.x;
                        gpy[site] = pr.y;
                        gpz[site] = pr.z;
                        sacc++;
                        sdE += (double)dE;
                        sPx += (double)(Li * dx);
                        sPy += (double)(Li * dy);
                        sPz += (double)(Li * dz);
                    }
                }
                __syncthreads();
            }
        }
    }

    // ---- block reduction of the move statistics ---------------------------------
    double v[6] = {sdE, sPx, sPy, sPz, (double)sacc, (double)satt};
#pragma unroll
    for (int k = 0; k < 6; k++) v[k] = warp_sum(v[k]);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 6; k++) red[warp * 16 + k] = v[k];
    }
    __syncthreads();
    if (tid == 0) {
        double t[6] = {0, 0, 0, 0, 0, 0};
        for (int q = 0; q < SN_THREADS / 32; q++)
            for (int k = 0; k < 6; k++) t[k] += red[q * 16 + k];
        SnAccum *A = a.acc + w.rep;
        atomicAdd(&A->dE, t[0]);
        atomicAdd(&A->dP[0], t[1]);
        atomicAdd(&A->dP[1], t[2]);
        atomicAdd(&A->dP[2], t[3]);
        atomicAdd(&A->acc, (unsigned long long)t[4]);
        atomicAdd(&A->att, (unsigned long long)t[5]);
    }
}


// ---------------------------------------------------------------------------
// Full local-field pass (energy recompute, site energies, adjoint).  Same
// tiles and stencil as the sweep, read-only, every block of the replica in
// one launch.  R = float: FP32 local fields, FP64 site products and sums;
// R = double: every operation in FP64.
//   red[rep*red_stride + k]: 0 E_dd = 1/2 sum len_i p_i.H_i   1 sum p_i.nn_i
//                    2 sum p_i.E                       3 sum K term
//                    4..6 sum len_i p_i                7..9 sum p_i
// where H_i = sum_j len_j T_o p_j is the dipole field at site i.
struct SnFieldArgs {
    const SnWork *work;
    const SnReplicaDev *reps;
    const SnTile *geoms;
    float cage;
    float K;
    double *site_e;  // nullable: N doubles
    float *grad;     // nullable: 3N floats (interleaved)
    double *red;     // 10 doubles per replica
    int red_stride;  // doubles between replicas in red (0: all replicas share one slot)
};

template <typename R, int RC, bool TWO_D, bool MIXED>
__global__ void __launch_bounds__(SN_THREADS, 1) field_tiled(const SnFieldArgs a)
{
    using G = Geo<RC, TWO_D>;
    constexpr int S = G::S, H = G::H, HZ = G::HZ, SZ = G::SZ, NF = G::NF, NS = G::NS;
    extern __shared__ __align__(16) unsigned char smem[];

    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const SnWork w = a.work[blockIdx.x];
    const SnReplicaDev &Rp = a.reps[w.rep];
    const SnTile &Gm = a.geoms[Rp.geom];
    const int X = Rp.X, Y = Rp.Y, Z = Rp.Z;
    const float *__restrict__ gpx = Rp.px;
    const float *__restrict__ gpy = Rp.py;
    const float *__restrict__ gpz = Rp.pz;
    const float *__restrict__ glen = Rp.len;
    const int Bx = Gm.B[0], By = Gm.B[1], Bz = Gm.B[2];
    const int Tx = Gm.T[0], Ty = Gm.T[1], Tz = Gm.T[2];
    const int Sy = Gm.Sy, Sx = Gm.Sx, maxt = Gm.maxt;
    const double C = a.cage, Kk = a.K;
    const double Ex = Rp.E[0], Ey = Rp.E[1], Ez = Rp.E[2];
    const R Lu = (R)Rp.length;

    const Carve cv = sn_carve(Gm.slots, maxt, S, SZ, NS, NF, MIXED);
    float *tile = reinterpret_cast<float *>(smem + cv.tile);
    float *tlen = reinterpret_cast<float *>(smem + cv.tlen);
    R *parts = reinterpret_cast<R *>(smem + cv.parts);
    int *ftab = reinterpret_cast<int *>(smem + cv.ftab);
    int *start = reinterpret_cast<int *>(smem + cv.start);
    double *red = reinterpret_cast<double *>(smem + cv.red);

    if (tid < 3 * SN_MAX_S) start[tid] = Gm.start[tid / SN_MAX_S][tid % SN_MAX_S];
    __syncthreads();
    for (int i = tid; i < 3 * S * NF; i += SN_THREADS) {
        const int ax = i / (S * NF), c = (i / NF) % S, o = i % NF - H;
        int v = 0;
        const int Ha = ax == 2 ? HZ : H;
        const int T = Gm.T[ax];
        const int u0 = c + Ha, u = u0 + o;
        if (!(ax == 2 && TWO_D) && u >= 0 && u < T && u0 < T) {
            const int *st = start + ax * SN_MAX_S;
            const int d = sn_pi<S>(st, u) - sn_pi<S>(st, u0);
            const int stride = ax == 0 ? Sx : (ax == 1 ? Sy : 1);
            v = d * stride * 12;
        }
        ftab[i] = v;
    }
    for (int row = warp; row < Tx * Ty; row += SN_THREADS / 32) {
        const int ux = row / Ty, uy = row - (row / Ty) * Ty;
        const int gx = sn_wrap(w.x0 - H + ux, X), gy = sn_wrap(w.y0 - H + uy, Y);
        const int rslot = sn_pi<S>(start, ux) * Sx + sn_pi<S>(start + SN_MAX_S, uy) * Sy;
        const long long gb = ((long long)gx * Y + gy) * Z;
        for (int uz = lane; uz < Tz; uz += 32) {
            const int gz = TWO_D ? 0 : sn_wrap(w.z0 - HZ + uz, Z);
            const long long g = gb + gz;
            const int slot = rslot + (TWO_D ? 0 : sn_pi<S>(start + 2 * SN_MAX_S, uz));
            float x = gpx[g], y = gpy[g], z = gpz[g];
            if constexpr (MIXED) {
                const float L = glen[g];
                tlen[slot] = L;
                x *= L;
                y *= L;
                z *= L;
            }
            tile[3 * slot + 0] = x;
            tile[3 * slot + 1] = y;
            tile[3 * slot + 2] = z;
        }
    }
    __syncthreads();

    double acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int cx = 0; cx < S; cx++) {
        const int nxc = sn_count(Bx, cx, S);
        if (nxc == 0) continue;
        int FX[NF];
#pragma unroll
        for (int o = 0; o < NF; o++) FX[o] = ftab[(0 * S + cx) * NF + o];
        const int bx0 = sn_pi<S>(start, cx + H);
        for (int cy = 0; cy < S; cy++) {
            const int nyc = sn_count(By, cy, S);
            if (nyc == 0) continue;
            int FY[NF];
#pragma unroll
            for (int o = 0; o < NF; o++) FY[o] = ftab[(1 * S + cy) * NF + o];
            const int by0 = sn_pi<S>(start + SN_MAX_S, cy + H);
            for (int cz = 0; cz < SZ; cz++) {
                const int nzc = TWO_D ? 1 : sn_count(Bz, cz, S);
                const int nt = nxc * nyc * nzc;
                if (nt == 0) continue;
                int FZ[NF];
#pragma unroll
                for (int o = 0; o < NF; o++) FZ[o] = TWO_D ? 0 : ftab[(2 * S + cz) * NF + o];
                const int bz0 = TWO_D ? 0 : sn_pi<S>(start + 2 * SN_MAX_S, cz + HZ);
                const int ntp = (nt + 31) & ~31;
                for (int wi = tid; wi < NS * ntp; wi += SN_THREADS) {
                    const int j = wi / ntp, t = wi - j * ntp;
                    if (t < nt) {
                        const int qz = t % nzc, r = t / nzc, qy = r % nyc, qx = r / nyc;
                        const uint32_t tslot = (uint32_t)((bx0 + qx) * Sx + (by0 + qy) * Sy + bz0 + qz);
                        R hacc[2][3] = {{0, 0, 0}, {0, 0, 0}};
                        R nn[3] = {0, 0, 0};
                        dispatch_split<R, RC, TWO_D, MIXED, 0>(j, smem + cv.tile, tslot * 12u, FX, FY, FZ, tlen, tslot,
                                                               hacc, nn);
                        R *pp = parts + (j * 6) * maxt + t;
                        pp[0 * maxt] = hacc[0][0] + hacc[1][0];
                        pp[1 * maxt] = hacc[0][1] + hacc[1][1];
                        pp[2 * maxt] = hacc[0][2] + hacc[1][2];
                        pp[3 * maxt] = nn[0];
                        pp[4 * maxt] = nn[1];
                        pp[5 * maxt] = nn[2];
                    }
                }
                __syncthreads();
                for (int t = tid; t < nt; t += SN_THREADS) {
                    R hx = 0, hy = 0, hz = 0, nx = 0, ny = 0, nz = 0;
#pragma unroll
                    for (int j = 0; j < NS; j++) {
                        const R *pp = parts + (j * 6) * maxt + t;
                        hx += pp[0 * maxt];
                        hy += pp[1 * maxt];
                        hz += pp[2 * maxt];
                        nx += pp[3 * maxt];
                        ny += pp[4 * maxt];
                        nz += pp[5 * maxt];
                    }
                    const int qz = t % nzc, r = t / nzc, qy = r % nyc, qx = r / nyc;
                    const int lx = cx + S * qx, ly = cy + S * qy, lz = TWO_D ? 0 : cz + S * qz;
                    const long long site = ((long long)(w.x0 + lx) * Y + (w.y0 + ly)) * Z + (w.z0 + lz);
                    const double px = gpx[site], py = gpy[site], pz = gpz[site];
                    const double Li = MIXED ? (double)glen[site] : (double)Rp.length;
                    if (Li == 0.0) {
                        if (a.site_e) a.site_e[site] = 0.0;
                        if (a.grad) {
                            a.grad[3 * site + 0] = 0.0f;
                            a.grad[3 * site + 1] = 0.0f;
                            a.grad[3 * site + 2] = 0.0f;
                        }
                        continue;
                    }
                    // H = sum_j len_j T p_j: uniform tiles hold unit p (H = L h)
                    const R sc = MIXED ? R(1) : Lu;
                    const double Hx = (double)(sc * hx), Hy = (double)(sc * hy), Hz = (double)(sc * hz);
                    const double gx = Li * Hx - C * (double)nx + Ex;
                    const double gy = Li * Hy - C * (double)ny + Ey;
                    const double gz = Li * Hz - C * (double)nz + Ez;
                    const double kt = Kk > 0.0 ? -Kk * (fabs(px) + fabs(py)) : 0.0;
                    const double pH = px * Hx + py * Hy + pz * Hz;
                    const double pn = px * (double)nx + py * (double)ny + pz * (double)nz;
                    const double pE = px * Ex + py * Ey + pz * Ez;
                    if (a.site_e) a.site_e[site] = px * gx + py * gy + pz * gz + kt;
                    if (a.grad) {
                        const double sx = Kk > 0.0 ? (px > 0.0 ? 1.0 : (px < 0.0 ? -1.0 : 0.0)) : 0.0;
                        const double sy = Kk > 0.0 ? (py > 0.0 ? 1.0 : (py < 0.0 ? -1.0 : 0.0)) : 0.0;
                        a.grad[3 * site + 0] = (float)(gx - Kk * sx);
                        a.grad[3 * site + 1] = (float)(gy - Kk * sy);
                        a.grad[3 * site + 2] = (float)gz;
                    }
                    acc[0] += 0.5 * Li * pH;
                    acc[1] += pn;
                    acc[2] += pE;
                    acc[3] += kt;
                    acc[4] += Li * px;
                    acc[5] += Li * py;
                    acc[6] += Li * pz;
                    acc[7] += px;
                    acc[8] += py;
                    acc[9] += pz;
                }
                __syncthreads();
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 10; k++) acc[k] = warp_sum(acc[k]);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 10; k++) red[warp * 16 + k] = acc[k];
    }
    __syncthreads();
    if (tid < 10) {
        double t = 0.0;
        for (int q = 0; q < SN_THREADS / 32; q++) t += red[q * 16 + tid];
        atomicAdd(&a.red[a.red_stride * w.rep + tid], t);
    }
}

template <typename R, int RC>
cudaError_t launch_field_rc(bool two_d, bool mixed, const SnFieldArgs &args, int grid, int smem_bytes,
                            cudaStream_t st)
{
    static bool configured[4] = {false, false, false, false};
    const int idx = (two_d ? 2 : 0) + (mixed ? 1 : 0);
    void (*fn)(const SnFieldArgs);
    if (two_d) fn = mixed ? field_tiled<R, RC, true, true> : field_tiled<R, RC, true, false>;
    else fn = mixed ? field_tiled<R, RC, false, true> : field_tiled<R, RC, false, false>;
    if (!configured[idx]) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        if (e != cudaSuccess) return e;
        configured[idx] = true;
    }
    if (grid <= 0) return cudaSuccess;
    fn<<<grid, SN_THREADS, smem_bytes, st>>>(args);
    return cudaGetLastError();
}

template <int RC>
cudaError_t launch_rc(bool two_d, bool mixed, const SnPhaseArgs &args, int grid, int smem_bytes, cudaStream_t st)
{
    static bool configured[4] = {false, false, false, false};
    const int idx = (two_d ? 2 : 0) + (mixed ? 1 : 0);
    void (*fn)(const SnPhaseArgs);
    if (two_d) fn = mixed ? sweep_phase<RC, true, true> : sweep_phase<RC, true, false>;
    else fn = mixed ? sweep_phase<RC, false, true> : sweep_phase<RC, false, false>;
    if (!configured[idx]) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        if (e != cudaSuccess) return e;
        configured[idx] = true;
    }
    if (grid <= 0) return cudaSuccess;
    fn<<<grid, SN_THREADS, smem_bytes, st>>>(args);
    return cudaGetLastError();
}

// Sizes the host needs for planning (must match the kernel's template choices).
template <int RC>
inline void geo_sizes(bool two_d, int &S, int &SZ, int &NS, int &NF)
{
    if (two_d) {
        S = Geo<RC, true>::S;
        SZ = Geo<RC, true>::SZ;
        NS = Geo<RC, true>::NS;
        NF = Geo<RC, true>::NF;
    } else {
        S = Geo<RC, false>::S;
        SZ = Geo<RC, false>::SZ;
        NS = Geo<RC, false>::NS;
        NF = Geo<RC, false>::NF;
    }
}

}  // namespace sn_sweep
