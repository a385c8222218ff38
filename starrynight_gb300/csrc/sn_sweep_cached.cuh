// sn_sweep_cached.cuh -- the cached-field Metropolis sweep of one block.
//
// The energy change of a move at site i is dE = (p' - p).(g_i + E) (+ the K
// term) with the local field g_i = len_i sum_j len_j T_ij p_j - CageStrain
// sum_nn p_j (src/starrynight-montecarlo-core.c:91-134: site_energy's
// dipole, cage-strain and field terms).  g is linear in the neighbours'
// dipoles, so instead of summing the cutoff stencil for every attempted move
// (what sweep_block does), this kernel keeps g of every site in HBM and, when
// a move at site a is accepted, adds the change of every neighbour's field,
// dg_{a+o} = len_{a+o} len_a T_o dp_a - CageStrain [|o| = 1] dp_a, for the
// offsets o of the cutoff sphere.  An attempt then costs one read of g_i; the
// stencil work is spent only on accepted moves.  The result of every move is
// that of the stencil sum up to rounding (the field is the same linear sum).
//
// Fixed point, exactly.  Each neighbour's contribution is rounded to a
// fixed-point grid of 2^-k on its own, Q(c_ij) with c_ij = w (T_o p_j) -
// CageStrain [|o| = 1] p_j, w = len_i len_j (for unit uniform lengths
// c_ij = (T_o - CageStrain [|o| = 1] I) p_j, the cage strain folded into the
// tensor), and g_i is the int32 sum of those integers.  A move of site a
// from p to p' then changes g_n by exactly Q(c(p')) - Q(c(p)), which the
// sweep adds with integer shared-memory atomics or reductions: integer
// addition is associative, so g after any sequence of moves equals, bit for
// bit, the g that the field pass (gfield_tiled) computes from scratch for
// the current lattice -- independent of thread order, schedule, batching or
// a resume from a checkpoint, and free of drift.  k is chosen on the host so
// that |c * 2^k| < 2^22 for every contribution; Q is then one FMA with a
// magic constant (round to nearest even), the same operation everywhere.
//
// Ownership.  A block's tile is the block plus a halo of `cutoff` sites
// (the z halo rounded up to 4 sites for 16-byte rows).  It is loaded when the
// block starts and stored back when the block ends: with every block side
// >= 2 cutoff (a planner condition), the cutoff-wide parts of the tiles of
// blocks that can run at the same time (not adjacent) are disjoint, and
// adjacent blocks run one after the other (block colours; the dataflow
// kernel's dependency waits), so each site's g is held by at most one
// running block.  The store covers the cutoff-wide tile, or the whole tile
// when the z side is at least twice the rounded z halo (whole tiles are then
// disjoint too).
#pragma once

namespace sn_sweep {

// Shared-memory carve-up of the cached sweep, identical on host and device.
struct CCarve {
    uint32_t tile, tlen, props, list, ctab, pairs, cnt, red, total;
};

__host__ __device__ inline CCarve sn_ccarve(int cslots, int tg, int pc, int np, bool mixed, int ng)
{
    CCarve c;
    uint32_t o = 0;
    // the reduction slots and the pair table first: their places must not
    // depend on the replica's tile, because a CTA uses them across the blocks
    // it sweeps (the move statistics are reduced when the replica changes)
    c.red = o;
    o += (SN_CACHED_THREADS / 32) * 16u * 8u;
    c.pairs = o;
    o += sn_align16((uint32_t)np * 48u);
    c.tile = o;
    o += sn_align16(3u * (uint32_t)cslots * 4u);
    c.tlen = o;
    if (mixed) o += sn_align16((uint32_t)cslots * 4u);
    c.props = o;
    o += (uint32_t)(2 * pc * tg) * 32u;  // two chunks of (p', threshold), (p_old, -) per target
    c.list = o;
    o += (uint32_t)((tg + 31) / 32) * 32u * 32u;  // accepted moves of a group: 32 entries per target warp
    c.ctab = o;
    o += sn_align16((uint32_t)ng * 16u);  // per group and merged half: tile-slot and site offsets of its colour
    c.cnt = o;
    // the tile-copy mbarrier (bytes 8..15), its phase parity (16..19), the
    // target warps' accepted-move counts (from byte 32, one int per warp)
    o += 32u + sn_align16(4u * (SN_CACHED_THREADS / 32));
    c.total = o;
    return c;
}

// One stencil pair's constants in shared memory: T_o (xx yy zz xy xz yz),
// the offset, and whether |o| = 1 (cage strain).
struct CPair {
    float t[6];
    int o[3];
    int nn;
    int pad[2];
};
static_assert(sizeof(CPair) == 48, "pair record");

// Q(v * 2^k) for |v * 2^k| < 2^22: adding 1.5 * 2^23 leaves round-to-nearest-
// even(v * 2^k) in the low mantissa bits (the scaling by a power of two is exact).
#define SN_Q_MAGIC 12582912.0f  // 1.5 * 2^23
#define SN_Q_MAGIC_BITS 0x4B400000u
__device__ __forceinline__ uint32_t q_bits(float v, float scale) { return __float_as_uint(fmaf(v, scale, SN_Q_MAGIC)); }

// The contribution c = w (T p) - C [nn] p of one dipole p through offset tensor
// t (xx yy zz xy xz yz), as the raw magic-biased bits of Q(c) per component.
// Every kernel that builds or updates the field cache calls this function, so
// the rounding is the same everywhere.
// W1: w is known to be 1 (uniform lengths of 1), and the multiplication by it,
// which is exact, is skipped.  For w = 1 the cage-strain term is folded into
// the tensor instead (the callers pass t with its diagonal reduced by C,
// rounded once, and NN = false): c = (T - C I) p for |o| = 1.  The field-cache
// pass folds the same way, so both compute the same floats.
template <bool W1 = false>
__device__ __forceinline__ void q_contrib(const float (&t)[6], bool NN, float w, float C, float scale, float px,
                                          float py, float pz, uint32_t &qx, uint32_t &qy, uint32_t &qz)
{
    float vx = fmaf(t[0], px, fmaf(t[3], py, __fmul_rn(t[4], pz)));
    float vy = fmaf(t[3], px, fmaf(t[1], py, __fmul_rn(t[5], pz)));
    float vz = fmaf(t[4], px, fmaf(t[5], py, __fmul_rn(t[2], pz)));
    if (!W1) {
        vx = __fmul_rn(w, vx);
        vy = __fmul_rn(w, vy);
        vz = __fmul_rn(w, vz);
    }
    if (NN) {
        vx = __fsub_rn(vx, __fmul_rn(C, px));
        vy = __fsub_rn(vy, __fmul_rn(C, py));
        vz = __fsub_rn(vz, __fmul_rn(C, pz));
    }
    qx = q_bits(vx, scale);
    qy = q_bits(vy, scale);
    qz = q_bits(vz, scale);
}

template <int RC, int I>
__device__ __forceinline__ void put_pair(CPair *tab)
{
    constexpr sn_stencil::Off o = sn_stencil::pair_offset(RC, false, I);
    CPair p;
#pragma unroll
    for (int e = 0; e < 6; e++) p.t[e] = 0.0f;
    p.t[0] = (float)sn_stencil::tensor_d(o.x, o.y, o.z, 0);
    p.t[1] = (float)sn_stencil::tensor_d(o.x, o.y, o.z, 1);
    p.t[2] = (float)sn_stencil::tensor_d(o.x, o.y, o.z, 2);
    p.t[3] = (float)sn_stencil::tensor_d(o.x, o.y, o.z, 3);
    p.t[4] = (float)sn_stencil::tensor_d(o.x, o.y, o.z, 4);
    p.t[5] = (float)sn_stencil::tensor_d(o.x, o.y, o.z, 5);
    p.o[0] = o.x;
    p.o[1] = o.y;
    p.o[2] = o.z;
    p.nn = (o.x * o.x + o.y * o.y + o.z * o.z == 1) ? 1 : 0;
    p.pad[0] = p.pad[1] = 0;
    tab[I] = p;
}

// Thread k of the CTA writes pairs k, k + nthreads, ... of the table.
template <int RC, int... Is>
__device__ __forceinline__ void fill_pairs(std::integer_sequence<int, Is...>, CPair *tab, int tid, int nthreads)
{
    ((tid == Is % nthreads ? put_pair<RC, Is>(tab) : void()), ...);
}

__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc)
{
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gsrc) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

// v added to the shared-memory word at byte address a (a reduction: no value returned)
__device__ __forceinline__ void red_shared_add(uint32_t a, uint32_t v)
{
    asm volatile("red.shared.add.u32 [%0], %1;\n" ::"r"(a), "r"(v) : "memory");
}

// ---- TMA bulk copies (the tile_copy = 1 load path) ------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// One bulk copy global -> shared of `bytes` (a multiple of 16, both addresses
// 16-byte aligned), completing on `bar`.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Bounded wait for the tile copies of phase `parity`; on time-out records
// bit 1 in *err, then waits once more (bounded) for the copies still in
// flight, so the CTA never leaves with its shared memory being written.
__device__ __forceinline__ void mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t *err)
{
    uint32_t it = 0;
    while (!mbar_try_wait(bar, parity)) {
        if (++it >= SN_BULK_WAIT_LIMIT) {
            if (err) atomicOr(err, 2u);
            for (uint32_t k = 0; k < SN_BULK_WAIT_LIMIT && !mbar_try_wait(bar, parity); k++) __nanosleep(1000);
            return;
        }
    }
}

// The tile of block w (3 field arrays, and the lengths when tlen is set) as
// TMA bulk copies, one per tile row and array (two where the row wraps
// around z), all completing on `bar`.  Thread 0 has announced the byte count
// before any copy is issued.
__device__ __forceinline__ void bulk_load_tile(const SnReplicaDev &R, const SnTile &Gm, const SnWork &w, int *tile,
                                               float *tlen, uint64_t *bar, int tid, int nthreads)
{
    const int X = R.X, Y = R.Y, Z = R.Z;
    const int T1 = Gm.cT[1], T2 = Gm.cT[2];
    const long long N = R.n_sites;
    const int cs = Gm.cslots;
    const int rows = Gm.cT[0] * T1;
    const int narr = tlen ? 4 : 3;
    const int zs = sn_wrap(w.z0 - Gm.cH[2], Z);
    const int n1 = min(T2, Z - zs);  // sites before the z wrap (multiples of 4)
    asm volatile("fence.proxy.async;\n" ::: "memory");
    for (int i = tid; i < rows * narr; i += nthreads) {
        const int arr = i / rows, row = i - arr * rows;
        const int ux = row / T1, uy = row - ux * T1;
        const int gx = sn_wrap(w.x0 - Gm.cH[0] + ux, X), gy = sn_wrap(w.y0 - Gm.cH[1] + uy, Y);
        const long long gr = ((long long)gx * Y + gy) * Z;
        const void *src = arr < 3 ? (const void *)(R.gcache + arr * N + gr) : (const void *)(R.len + gr);
        unsigned char *dst = arr < 3 ? (unsigned char *)(tile + arr * cs + row * T2) : (unsigned char *)(tlen + row * T2);
        bulk_g2s(dst, (const unsigned char *)src + 4ll * zs, 4u * n1, bar);
        if (n1 < T2) bulk_g2s(dst + 4 * n1, src, 4u * (T2 - n1), bar);
    }
}

// Wait until at most N of this thread's committed copy groups are in flight.
template <int N>
__device__ __forceinline__ void cp_async_wait_group()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Copy (store = false) or write back (store = true) the tile of block w:
// cT[0] x cT[1] rows of cT[2] consecutive z sites per array, in 16-byte
// chunks.  Z, the block origin and the z halo are multiples of 4, so a chunk
// never straddles the periodic wrap.  The write-back covers only the sites
// within `hz` (the cutoff) of the block along z: the rounding of the z halo
// to 4 sites adds sites that another block may hold at the same time (the
// disjointness of running tiles holds for the cutoff-wide halo only), so
// chunks at the two ends of a row are written site by site.
template <bool STORE>
__device__ __forceinline__ void move_tile(const SnReplicaDev &R, const SnTile &Gm, const SnWork &w, int *tile,
                                          float *tlen, int tid, int nthreads, int hz = 0)
{
    const int X = R.X, Y = R.Y, Z = R.Z;
    const int T1 = Gm.cT[1], T2 = Gm.cT[2], cpr = T2 >> 2;
    const long long N = R.n_sites;
    const int cs = Gm.cslots;
    const int rows = Gm.cT[0] * T1;
    const int zlo = Gm.cH[2] - hz, zhi = Gm.cH[2] + Gm.B[2] + hz;  // tile z range written back
    // Thread tid moves chunk c of rows r0, r0 + step, ...: the chunk and the
    // global z of a thread never change, the row advances by a fixed step
    // (tracked as (ux, uy) without divisions).
    const int per = nthreads / cpr;  // rows a pass covers
    if (tid >= per * cpr) return;
    const int c = tid % cpr, r0 = tid / cpr;
    const int gz = sn_wrap(w.z0 - Gm.cH[2] + 4 * c, Z);
    const bool full = 4 * c >= zlo && 4 * c + 4 <= zhi;
    const int sx = per / T1, sy = per - (per / T1) * T1;
    int ux = r0 / T1, uy = r0 - (r0 / T1) * T1;
    for (int row = r0; row < rows; row += per) {
        const int gx = sn_wrap(w.x0 - Gm.cH[0] + ux, X), gy = sn_wrap(w.y0 - Gm.cH[1] + uy, Y);
        const long long g = ((long long)gx * Y + gy) * Z + gz;
        const int slot = row * T2 + 4 * c;
        if (STORE) {
            if (full) {
#pragma unroll
                for (int arr = 0; arr < 3; arr++)
                    *reinterpret_cast<int4 *>(R.gcache + arr * N + g) =
                        *reinterpret_cast<const int4 *>(tile + arr * cs + slot);
            } else {
#pragma unroll
                for (int e = 0; e < 4; e++)
                    if (4 * c + e >= zlo && 4 * c + e < zhi) {
#pragma unroll
                        for (int arr = 0; arr < 3; arr++) R.gcache[arr * N + g + e] = tile[arr * cs + slot + e];
                    }
            }
        } else {
#pragma unroll
            for (int arr = 0; arr < 3; arr++) cp_async16(tile + arr * cs + slot, R.gcache + arr * N + g);
            if (tlen) cp_async16(tlen + slot, R.len + g);
        }
        ux += sx;
        uy += sy;
        if (uy >= T1) {
            uy -= T1;
            ux++;
        }
    }
}

// A thread's move statistics: compensated FP32 sums of dE and dP over its
// accepted moves, and its accepted and attempted counts.
struct CStats {
    KahanF dE, Px, Py, Pz;
    unsigned int acc = 0, att = 0;
};

// Adds every thread's statistics into the replica's per-sweep totals A and
// clears them (all threads of the CTA call it; red: (NT / 32) * 16 doubles of
// shared memory).  Within a warp the compensated FP32 sums are combined as
// (sum, error) pairs by error-free additions (Knuth's TwoSum); FP64 (a slow
// pipe on this GPU) is used only to add the warps' results.
__device__ __forceinline__ void flush_cstats(CStats &st, double *red, SnAccum *A)
{
    constexpr int NT = SN_CACHED_THREADS;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float hs[4] = {st.dE.s, st.Px.s, st.Py.s, st.Pz.s}, hc[4] = {-st.dE.c, -st.Px.c, -st.Py.c, -st.Pz.c};
    unsigned int ia = st.acc, it = st.att;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float bs = __shfl_xor_sync(0xffffffffu, hs[k], o), bc = __shfl_xor_sync(0xffffffffu, hc[k], o);
            const float t2 = __fadd_rn(hs[k], bs);
            const float bb = __fsub_rn(t2, hs[k]);
            const float err = __fadd_rn(__fsub_rn(hs[k], __fsub_rn(t2, bb)), __fsub_rn(bs, bb));
            hs[k] = t2;
            hc[k] = __fadd_rn(__fadd_rn(hc[k], bc), err);
        }
        ia += __shfl_xor_sync(0xffffffffu, ia, o);
        it += __shfl_xor_sync(0xffffffffu, it, o);
    }
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 4; k++) red[warp * 16 + k] = (double)hs[k] + (double)hc[k];
        red[warp * 16 + 4] = (double)ia;
        red[warp * 16 + 5] = (double)it;
    }
    __syncthreads();
    if (tid < 6) {
        double v = 0.0;
        for (int q = 0; q < (NT >> 5); q++) v += red[q * 16 + tid];
        if (tid == 0) atomicAdd(&A->dE, v);
        else if (tid < 4) atomicAdd(&A->dP[tid - 1], v);
        else if (tid == 4) atomicAdd(&A->acc, (unsigned long long)v);
        else atomicAdd(&A->att, (unsigned long long)v);
    }
    __syncthreads();  // red is free again
    st = CStats();
}

// fill: write the stencil pair table into shared memory (once per CTA: the
// table depends on the cutoff only).  cst: the calling thread's running move
// statistics for this block's replica, added up by the caller (nullptr: the
// block adds its statistics to the replica's totals itself).
template <int RC, bool MIXED, bool FLOW>
__device__ __forceinline__ void sweep_block_cached(const SnWork w, const SnPhaseArgs &a, unsigned char *smem,
                                                   bool fill, CStats *cst)
{
    using G = Geo<RC, false>;
    constexpr int S = G::S, NP = G::NP;
    constexpr bool MERGE = G::MERGE;
    constexpr int NT = SN_CACHED_THREADS;
    constexpr int PPT = (NP + NT - 1) / NT;     // stencil pairs per thread in the scatter
    constexpr int GRP = NP >= NT ? 1 : NT / NP;  // accepted moves scattered at once

    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const SnReplicaDev &R = a.reps[w.rep];
    const SnTile &Gm = a.geoms[R.geom];
    const int Y = R.Y, Z = R.Z;
    float *__restrict__ gpx = R.px;
    float *__restrict__ gpy = R.py;
    float *__restrict__ gpz = R.pz;
    const int Bx = Gm.B[0], By = Gm.B[1], Bz = Gm.B[2];
    const int T1 = Gm.cT[1], T2 = Gm.cT[2];
    const int tp = Gm.tp, tg = Gm.tg, ng = Gm.ng, pc = Gm.cpc;
    const int nqy = Gm.nq[1], nqz = Gm.nq[2];
    const float Ex = R.E[0], Ey = R.E[1], Ez = R.E[2];
    const float C = a.cage, Kk = a.K;
    const float Lu = R.length;
    const float gscale = R.gscale, ginv = R.ginv;  // 2^k, 2^-k
    const int cs = Gm.cslots;
    const int cH0 = Gm.cH[0], cH1 = Gm.cH[1], cH2 = Gm.cH[2];
    float4 *__restrict__ gprop = R.prop;

    const CCarve cv = sn_ccarve(cs, tg, pc, NP, MIXED, ng);
    int *tile = reinterpret_cast<int *>(smem + cv.tile);
    const uint32_t tile_u32 = smem_u32(tile), cs4 = 4u * (uint32_t)cs;
    float *tlen = MIXED ? reinterpret_cast<float *>(smem + cv.tlen) : nullptr;
    float4 *props = reinterpret_cast<float4 *>(smem + cv.props);
    float4 *list = reinterpret_cast<float4 *>(smem + cv.list);
    const CPair *pairs = reinterpret_cast<const CPair *>(smem + cv.pairs);
    int *cnt = reinterpret_cast<int *>(smem + cv.cnt);
    double *red = reinterpret_cast<double *>(smem + cv.red);

    uint64_t *tbar = reinterpret_cast<uint64_t *>(cnt + 2);  // 8-byte aligned: cnt is 16-byte aligned
    uint32_t tphase = 0;
    if (a.tile_copy) {
        // the tile through TMA bulk copies on an mbarrier (one phase per block)
        if (fill && tid == 0) {
            mbar_init(tbar, 1);
            cnt[4] = 0;  // phase parity of the barrier's next completion
        }
        __syncthreads();
        tphase = (uint32_t)cnt[4];
        if (tid == 0)
            mbar_arrive_expect_tx(tbar, (uint32_t)((MIXED ? 4 : 3) * Gm.cslots) * 4u);
        __syncthreads();
        bulk_load_tile(R, Gm, w, tile, tlen, tbar, tid, NT);
    } else {
        move_tile<false>(R, Gm, w, tile, tlen, tid, NT);
    }
    cp_async_commit();
    int *wc = cnt + 8;  // accepted moves per target warp in the current group
    const int nAw = (tg + 31) >> 5;  // target warps

    // this thread's target role: target tt = tid % tg of every colour group.
    // Threads tid < tg decide the group's moves (phase A).  Proposals are
    // staged by the threads from sb on (thread tid for target tt of groups
    // pj0, pj0 + pstride, ... of a chunk): when tg is a multiple of 32 and
    // the other warps can stage a whole group, only they do, while the
    // target warps run phase A of the chunk's first group (ovl); otherwise
    // every thread stages at the start of the chunk.
    const bool ovl = tg % 32 == 0 && NT - tg >= tg;
    const int sb = ovl ? tg : 0;
    const int tt = tid % tg, pstride = (NT - sb) / tg, pj0 = (tid - sb) / tg;
    const bool stager = tid >= sb && tid - sb < pstride * tg;
    const int hh = tt / tp, t = tt - (tt / tp) * tp;
    const int qz = t % nqz, qy = (t / nqz) % nqy, qx = t / (nqz * nqy);
    const bool tvalid = stager && qx < Gm.nq[0];
    const int trel = (S * qx * T1 + S * qy) * T2 + S * qz;
    const int srel = ((S * qx) * Y + S * qy) * Z + S * qz;
    const int sbase = (w.x0 * Y + w.y0) * Z + w.z0 + srel;  // this thread's target site less its colour offset

    // this thread's scatter role (phase B): stencil pairs q = pq + k * NT of
    // the accepted moves e = pj, pj + GRP, ...; the pair's tensor T_o, whether
    // |o| = 1, and the slot delta of +o in this tile
    const int pj = NP >= NT ? 0 : tid / NP;
    const int pq = NP >= NT ? tid : tid - pj * NP;
    const bool prole = NP >= NT ? true : pj < GRP;
    const float L2 = __fmul_rn(Lu, Lu);
    float Tq[PPT][6];
    int dq[PPT];
    uint32_t dq4[PPT];  // 4 dq: the byte delta of +o
    bool nnp[PPT], qok[PPT];

    CStats own;
    CStats &st = cst ? *cst : own;

    // amask bit g: this thread's target of group g exists (groups >= 64 are tested when staged).
    // Block sides that are multiples of S give every colour the same count: all bits.
    unsigned long long amask = 0ull;
    if (Bx % S == 0 && By % S == 0 && Bz % S == 0) {
        if (tvalid) amask = ng >= 64 ? ~0ull : (1ull << ng) - 1ull;
    } else {
        for (int g = 0; g < ng && g < 64; g++) {
            int cx, cy, cz;
            group_colour<S, S, MERGE>(g, hh, cx, cy, cz);
            if (tvalid && qx < sn_count(Bx, cx, S) && qy < sn_count(By, cy, S) && qz < sn_count(Bz, cz, S))
                amask |= 1ull << g;
        }
    }

    // Proposals arrive in chunks of pc colour groups, copied asynchronously
    // from the sweep's proposal buffer (drawn before the sweep by
    // sweep_proposals_kernel) together with the targets' current dipoles,
    // into two alternating buffers: chunk c + 1 is in flight while chunk c
    // is used.
    const int nchunks = (ng + pc - 1) / pc;
    auto stage = [&](int c) {
        const int g0 = c * pc, nk = min(pc, ng - g0);
        float4 *buf = props + (c & 1) * (2 * pc * tg);
        if (stager) {
            for (int k = pj0; k < nk; k += pstride) {
                int cx, cy, cz;
                group_colour<S, S, MERGE>(g0 + k, hh, cx, cy, cz);
                const bool tgt = (g0 + k < 64) ? ((amask >> (g0 + k)) & 1ull) != 0ull
                                               : (tvalid && qx < sn_count(Bx, cx, S) && qy < sn_count(By, cy, S) &&
                                                  qz < sn_count(Bz, cz, S));
                float4 *slot = buf + 2 * (k * tg + tt);
                if (tgt) {
                    const int site = ((w.x0 + cx) * Y + (w.y0 + cy)) * Z + w.z0 + cz + srel;
                    cp_async16(slot, gprop + site);
                    cp_async4(&slot[1].x, gpx + site);
                    cp_async4(&slot[1].y, gpy + site);
                    cp_async4(&slot[1].z, gpz + site);
                } else {
                    slot[0] = make_float4(0.0f, 0.0f, 0.0f, -2.0f);  // no target here
                }
            }
        }
        cp_async_commit();
    };
    // the colour offsets of every group's two halves: tile slot
    // ((cx + cH0) T1 + cy + cH1) T2 + cz + cH2 and site (cx Y + cy) Z + cz
    // (read by phase A after the first chunk's barrier)
    int2 *ctab = reinterpret_cast<int2 *>(smem + cv.ctab);
    for (int i = tid; i < 2 * ng; i += NT) {
        int cx, cy, cz;
        group_colour<S, S, MERGE>(i >> 1, i & 1, cx, cy, cz);
        ctab[i] = make_int2(((cx + cH0) * T1 + (cy + cH1)) * T2 + cz + cH2, (cx * Y + cy) * Z + cz);
    }
    stage(0);
    const float4 *cur = props;
    int gchunk = 0, c = -1, gnext = 0;  // chunk of the current group, first group of the next chunk
    for (int g = 0; g < ng; g++) {
        if (g == gnext) {
            c++;
            gnext = g + pc;
            if (ovl) {
                cp_async_wait_group<0>();  // the tile and chunk c have landed (chunk c + 1 is staged below)
            } else {
                if (c + 1 < nchunks) stage(c + 1);  // into the buffer chunk c - 1 used (all done with it)
                else cp_async_commit();
                cp_async_wait_group<1>();  // the tile and chunk c have landed (chunk c + 1 may be in flight)
            }
            if (g == 0 && a.tile_copy) mbar_wait_bounded(tbar, tphase, a.err);
            if (g == 0 && fill)
                fill_pairs<RC>(std::make_integer_sequence<int, NP>{}, reinterpret_cast<CPair *>(smem + cv.pairs), tid,
                               NT);
            __syncthreads();
            if (g == 0) {
                // this thread's stencil pairs for the scatter
#pragma unroll
                for (int k = 0; k < PPT; k++) {
                    const int q = pq + k * NT;
                    qok[k] = prole && q < NP;
                    const CPair &P = pairs[qok[k] ? q : 0];
                    dq[k] = (P.o[0] * T1 + P.o[1]) * T2 + P.o[2];
                    dq4[k] = 4u * (uint32_t)dq[k];
                    nnp[k] = P.nn != 0;
#pragma unroll
                    for (int e = 0; e < 6; e++) Tq[k][e] = P.t[e];
                    if (!MIXED && L2 == 1.0f && nnp[k]) {  // unit lengths: cage strain folded into the tensor
                        Tq[k][0] = __fsub_rn(Tq[k][0], C);
                        Tq[k][1] = __fsub_rn(Tq[k][1], C);
                        Tq[k][2] = __fsub_rn(Tq[k][2], C);
                        nnp[k] = false;
                    }
                }
            }
            gchunk = g;
            cur = props + (c & 1) * (2 * pc * tg);
            // the staging warps issue chunk c + 1 (into the buffer chunk c - 1
            // used, read before the barrier above) while phase A runs
            if (ovl && c + 1 < nchunks) stage(c + 1);
        }

        // ---- A. targets of the group: dE from the cached field, accept, record ---------
        // Warp w lists its accepted moves in entries 32 w ... of the group's
        // list and their number in wc[w] (no shared counter to contend for).
        if (warp < nAw) {
            bool acc = false;
            float dx = 0.0f, dy = 0.0f, dz = 0.0f, Li = Lu;
            int tslot = 0;
            float4 pr = make_float4(0.0f, 0.0f, 0.0f, -2.0f), po = pr;
            if (tid < tg) {
                const int2 co = ctab[2 * g + hh];
                pr = cur[2 * ((g - gchunk) * tg + tt)];
                po = cur[2 * ((g - gchunk) * tg + tt) + 1];
                tslot = co.x + trel;
                if (pr.w >= 0.0f) {
                    const float gx = fmaf((float)tile[tslot], ginv, Ex);
                    const float gy = fmaf((float)tile[cs + tslot], ginv, Ey);
                    const float gz = fmaf((float)tile[2 * cs + tslot], ginv, Ez);
                    dx = pr.x - po.x;
                    dy = pr.y - po.y;
                    dz = pr.z - po.z;
                    float dE = fmaf(dx, gx, fmaf(dy, gy, dz * gz));
                    if (Kk > 0.0f) dE -= Kk * ((fabsf(pr.x) - fabsf(po.x)) + (fabsf(pr.y) - fabsf(po.y)));
                    st.att++;
                    if (dE < pr.w) {
                        acc = true;
                        const int site = sbase + co.y;
                        gpx[site] = pr.x;
                        gpy[site] = pr.y;
                        gpz[site] = pr.z;
                        if (MIXED) Li = tlen[tslot];
                        st.acc++;
                        st.dE.add(dE);
                        st.Px.add(Li * dx);
                        st.Py.add(Li * dy);
                        st.Pz.add(Li * dz);
                    }
                }
            }
            // (the list order does not matter: the scatter adds integers)
            const unsigned m = __ballot_sync(0xffffffffu, acc);
            if (acc) {
                const int e = 32 * warp + __popc(m & ((1u << lane) - 1u));
                // the target's tile slot (mixed lengths) or its byte address in shared memory
                list[2 * e] = make_float4(__int_as_float(MIXED ? tslot : (int)(tile_u32 + 4u * (uint32_t)tslot)), pr.x,
                                          pr.y, pr.z);
                list[2 * e + 1] = make_float4(po.x, po.y, po.z, Li);
            }
            if (lane == 0) wc[warp] = __popc(m);
        }
        __syncthreads();

        // ---- B. scatter the accepted moves' field changes into the tile --------------
        // dg_n = Q(c(p')) - Q(c(p)) for n = a +- o (the magic bias cancels).
        // Moves e = pj, pj + GRP, ... of the warps' lists taken in warp order.
        const int c0 = wc[0];
        int n = c0;
        for (int q = 1; q < nAw; q++) n += wc[q];
        if constexpr (MIXED) {
            int lw = 0, lbase = 0, lcnt = c0;  // list region of the current move
            for (int e = pj; e < n && prole; e += GRP) {
                while (e - lbase >= lcnt) {
                    lbase += lcnt;
                    lcnt = wc[++lw];
                }
                const int le = 32 * lw + e - lbase;
                const float4 en = list[2 * le], eo = list[2 * le + 1];
                const int sa = __float_as_int(en.x);
#pragma unroll
                for (int k = 0; k < PPT; k++) {
                    if (!qok[k]) continue;
                    const int sp = sa + dq[k], sm = sa - dq[k];
                    uint32_t nx, ny, nz, ox, oy, oz;
                    const float wp = __fmul_rn(tlen[sp], eo.w), wm = __fmul_rn(tlen[sm], eo.w);
                    q_contrib(Tq[k], nnp[k], wp, C, gscale, en.y, en.z, en.w, nx, ny, nz);
                    q_contrib(Tq[k], nnp[k], wp, C, gscale, eo.x, eo.y, eo.z, ox, oy, oz);
                    atomicAdd(tile + sp, (int)(nx - ox));
                    atomicAdd(tile + cs + sp, (int)(ny - oy));
                    atomicAdd(tile + 2 * cs + sp, (int)(nz - oz));
                    q_contrib(Tq[k], nnp[k], wm, C, gscale, en.y, en.z, en.w, nx, ny, nz);
                    q_contrib(Tq[k], nnp[k], wm, C, gscale, eo.x, eo.y, eo.z, ox, oy, oz);
                    atomicAdd(tile + sm, (int)(nx - ox));
                    atomicAdd(tile + cs + sm, (int)(ny - oy));
                    atomicAdd(tile + 2 * cs + sm, (int)(nz - oz));
                }
            }
        } else if (prole) {
            // uniform lengths: the same contribution for +o and -o, added by
            // shared-memory reductions at byte addresses (tile word s at
            // tile_u32 + 4 s, component c at + c * cs4; a move's list entry
            // carries its target's address)
            auto scatter = [&](auto unit) {
                constexpr bool W1 = decltype(unit)::value;
                int lw = 0, lbase = 0, lcnt = c0;
                for (int e = pj; e < n; e += GRP) {
                    int le;
                    if (nAw <= 2) {
                        le = e < c0 ? e : e + 32 - c0;
                    } else {
                        while (e - lbase >= lcnt) {
                            lbase += lcnt;
                            lcnt = wc[++lw];
                        }
                        le = 32 * lw + e - lbase;
                    }
                    const float4 en = list[2 * le], eo = list[2 * le + 1];
                    const uint32_t at = __float_as_uint(en.x);
#pragma unroll
                    for (int k = 0; k < PPT; k++) {
                        if (!qok[k]) continue;
                        uint32_t nx, ny, nz, ox, oy, oz;
                        // W1: the cage strain is folded into Tq (nnp false)
                        q_contrib<W1>(Tq[k], W1 ? false : nnp[k], L2, C, gscale, en.y, en.z, en.w, nx, ny, nz);
                        q_contrib<W1>(Tq[k], W1 ? false : nnp[k], L2, C, gscale, eo.x, eo.y, eo.z, ox, oy, oz);
                        const uint32_t ix = nx - ox, iy = ny - oy, iz = nz - oz;
                        const uint32_t ap = at + dq4[k], am = at - dq4[k];
                        red_shared_add(ap, ix);
                        red_shared_add(ap + cs4, iy);
                        red_shared_add(ap + 2u * cs4, iz);
                        red_shared_add(am, ix);
                        red_shared_add(am + cs4, iy);
                        red_shared_add(am + 2u * cs4, iz);
                    }
                }
            };
            if (L2 == 1.0f) scatter(std::true_type{});
            else scatter(std::false_type{});
        }
        __syncthreads();
    }

    // ---- the tile's fields back to HBM ---------------------------------------------
    // (the whole rounded z halo when z blocks are at least twice as long as
    // it: tiles of blocks that may run together are then disjoint with it,
    // and every row is written in whole 16-byte chunks)
    move_tile<true>(R, Gm, w, tile, nullptr, tid, NT, Bz >= 2 * Gm.cH[2] ? Gm.cH[2] : RC);

    // ---- the block's final sites to the caller's buffer ---------------------------
    if (float *out = R.out_xyz) {
        // a block row (fixed x, y) is 3*Bz consecutive floats of the interleaved
        // buffer: lanes write consecutive floats, reading the component arrays
        for (int row = warp; row < Bx * By; row += NT >> 5) {
            const int lx = row / By, ly = row - (row / By) * By;
            const long long s0 = (((long long)(w.x0 + lx)) * Y + (w.y0 + ly)) * Z + w.z0;
            for (int e = lane; e < 3 * Bz; e += 32) {
                const int site = e / 3, comp = e - 3 * (e / 3);
                const float *src = comp == 0 ? gpx : (comp == 1 ? gpy : gpz);
                out[3 * s0 + e] = __ldcg(src + s0 + site);
            }
        }
    }

    if (a.tile_copy && tid == 0) cnt[4] = (int)(tphase ^ 1u);  // read by the CTA's next block after its barriers
    if (!cst) flush_cstats(own, red, a.acc + w.rep);
}

// ---------------------------------------------------------------------------
// Field pass of the cache: g_i = sum_o Q(c(i, i+o)) for every site of a block
// from a tile of the dipoles (same tile geometry as the cached sweep), plus
// the replica's energy sums from it.  Each of the 2 NP contributions of a
// site is rounded on its own (q_contrib), so the result is the sweep's
// incremental cache bit for bit.  red[rep*stride + k] as SnFieldArgs, except
// red[0] = 1/2 sum p_i.g_i (dipole + cage-strain energy) and red[1] = 0.

// Rows of block w's tile of float arrays (px, py, pz and, when MIXED, len)
// into shared memory by 16-byte asynchronous copies.
template <bool MIXED>
__device__ __forceinline__ void stage_p_tile(const SnReplicaDev &R, const SnTile &Gm, const SnWork &w, float *tp,
                                             int tid, int nthreads)
{
    const int X = R.X, Y = R.Y, Z = R.Z;
    const int T1 = Gm.cT[1], T2 = Gm.cT[2], cpr = T2 >> 2;
    const int total = Gm.cT[0] * T1 * cpr;
    const int cs = Gm.cslots;
    for (int idx = tid; idx < total * (MIXED ? 4 : 3); idx += nthreads) {
        const int arr = idx / total, rem = idx - arr * total;
        const int row = rem / cpr, c = rem - row * cpr;
        const int ux = row / T1, uy = row - ux * T1;
        const int gx = sn_wrap(w.x0 - Gm.cH[0] + ux, X), gy = sn_wrap(w.y0 - Gm.cH[1] + uy, Y);
        const int gz = sn_wrap(w.z0 - Gm.cH[2] + 4 * c, Z);
        const float *src = arr == 0 ? R.px : (arr == 1 ? R.py : (arr == 2 ? R.pz : R.len));
        cp_async16(tp + arr * cs + row * T2 + 4 * c, src + (((long long)gx * Y + gy) * Z + gz));
    }
}

// Both contributions of stencil pair I to the field of the site in slot `slot`.
// Zero tensor entries are skipped: that changes at most the sign of a zero,
// which Q does not see, so the result equals q_contrib's.
template <int RC, bool MIXED, int I>
__device__ __forceinline__ void q_pair(const float *__restrict__ tp, int cs, int slot, int T1, int T2, float w_u,
                                       float Li, float C, float scale, uint32_t &ax, uint32_t &ay, uint32_t &az)
{
    constexpr sn_stencil::Off o = sn_stencil::pair_offset(RC, false, I);
    constexpr float t0 = (float)sn_stencil::tensor_d(o.x, o.y, o.z, 0);
    constexpr float t1 = (float)sn_stencil::tensor_d(o.x, o.y, o.z, 1);
    constexpr float t2 = (float)sn_stencil::tensor_d(o.x, o.y, o.z, 2);
    constexpr float t3 = (float)sn_stencil::tensor_d(o.x, o.y, o.z, 3);
    constexpr float t4 = (float)sn_stencil::tensor_d(o.x, o.y, o.z, 4);
    constexpr float t5 = (float)sn_stencil::tensor_d(o.x, o.y, o.z, 5);
    constexpr bool NN = o.x * o.x + o.y * o.y + o.z * o.z == 1;
    const int d = (o.x * T1 + o.y) * T2 + o.z;
    // unit uniform lengths: the cage strain folded into the diagonal (as the sweep's scatter does)
    const bool fold = NN && !MIXED && w_u == 1.0f;
    const float m0 = fold ? __fsub_rn(t0, C) : t0, m1 = fold ? __fsub_rn(t1, C) : t1,
                m2 = fold ? __fsub_rn(t2, C) : t2;
#pragma unroll
    for (int side = 0; side < 2; side++) {
        const int sj = side ? slot - d : slot + d;
        const float px = tp[sj], py = tp[cs + sj], pz = tp[2 * cs + sj];
        const float w = MIXED ? __fmul_rn(Li, tp[3 * cs + sj]) : w_u;
        // vx = fmaf(t0, px, fmaf(t3, py, t4 * pz)) and so on, without the zero terms
        float vx = t4 != 0.0f ? __fmul_rn(t4, pz) : 0.0f;
        if (t3 != 0.0f) vx = fmaf(t3, py, vx);
        vx = fmaf(m0, px, vx);
        float vy = t5 != 0.0f ? __fmul_rn(t5, pz) : 0.0f;
        vy = fmaf(m1, py, vy);
        if (t3 != 0.0f) vy = fmaf(t3, px, vy);
        float vz = __fmul_rn(m2, pz);
        if (t5 != 0.0f) vz = fmaf(t5, py, vz);
        if (t4 != 0.0f) vz = fmaf(t4, px, vz);
        if (MIXED || w != 1.0f) {
            vx = __fmul_rn(w, vx);
            vy = __fmul_rn(w, vy);
            vz = __fmul_rn(w, vz);
        }
        if (NN && !fold) {
            vx = __fsub_rn(vx, __fmul_rn(C, px));
            vy = __fsub_rn(vy, __fmul_rn(C, py));
            vz = __fsub_rn(vz, __fmul_rn(C, pz));
        }
        ax += q_bits(vx, scale);
        ay += q_bits(vy, scale);
        az += q_bits(vz, scale);
    }
}

template <int RC, bool MIXED, int... Is>
__device__ __forceinline__ void q_pairs(std::integer_sequence<int, Is...>, const float *tp, int cs, int slot, int T1,
                                        int T2, float w_u, float Li, float C, float scale, uint32_t &ax, uint32_t &ay,
                                        uint32_t &az)
{
    (q_pair<RC, MIXED, Is>(tp, cs, slot, T1, T2, w_u, Li, C, scale, ax, ay, az), ...);
}

// Column form of the pass (cutoffs up to 4): a thread takes 4 consecutive
// z sites of a row; for each column (ox, oy) of the cutoff disk it loads the
// column's dipoles around them with 16-byte loads (z from lz0 - 4 to lz0 + 7)
// and adds every contribution (ox, oy, oz) to each of the 4 sites.  Each
// contribution is q_pair's, with T_{-o} = T_o, so the integers are the same.
struct GCol {
    int x, y, h;  // column offset and the half-height of the cutoff sphere above it
};

constexpr int gcol_count(int rc)
{
    int n = 0;
    for (int x = -rc; x <= rc; x++)
        for (int y = -rc; y <= rc; y++)
            if (x * x + y * y <= rc * rc) n++;
    return n;
}

constexpr GCol gcol_at(int rc, int idx)
{
    int n = 0;
    for (int x = -rc; x <= rc; x++)
        for (int y = -rc; y <= rc; y++)
            if (x * x + y * y <= rc * rc) {
                if (n == idx) {
                    int h = 0;
                    while ((h + 1) * (h + 1) <= rc * rc - x * x - y * y) h++;
                    return GCol{x, y, h};
                }
                n++;
            }
    return GCol{0, 0, 0};
}

// Contribution of offset (OX, OY, OZ) to the 4 sites from the column's
// values v[k] at z = lz0 - 4 + k.
template <bool MIXED, int OX, int OY, int OZ>
__device__ __forceinline__ void gcell(const float (&vx)[12], const float (&vy)[12], const float (&vz)[12],
                                      const float (&vl)[12], const float (&Lt)[4], float w_u, float C, float scale,
                                      uint32_t (&ax)[4], uint32_t (&ay)[4], uint32_t (&az)[4])
{
    if constexpr (OX != 0 || OY != 0 || OZ != 0) {
        constexpr float t0 = (float)sn_stencil::tensor_d(OX, OY, OZ, 0);
        constexpr float t1 = (float)sn_stencil::tensor_d(OX, OY, OZ, 1);
        constexpr float t2 = (float)sn_stencil::tensor_d(OX, OY, OZ, 2);
        constexpr float t3 = (float)sn_stencil::tensor_d(OX, OY, OZ, 3);
        constexpr float t4 = (float)sn_stencil::tensor_d(OX, OY, OZ, 4);
        constexpr float t5 = (float)sn_stencil::tensor_d(OX, OY, OZ, 5);
        constexpr bool NN = OX * OX + OY * OY + OZ * OZ == 1;
        const bool fold = NN && !MIXED && w_u == 1.0f;
        const float m0 = fold ? __fsub_rn(t0, C) : t0, m1 = fold ? __fsub_rn(t1, C) : t1,
                    m2 = fold ? __fsub_rn(t2, C) : t2;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float px = vx[j + OZ + 4], py = vy[j + OZ + 4], pz = vz[j + OZ + 4];
            const float w = MIXED ? __fmul_rn(Lt[j], vl[j + OZ + 4]) : w_u;
            float qx = t4 != 0.0f ? __fmul_rn(t4, pz) : 0.0f;
            if (t3 != 0.0f) qx = fmaf(t3, py, qx);
            qx = fmaf(m0, px, qx);
            float qy = t5 != 0.0f ? __fmul_rn(t5, pz) : 0.0f;
            qy = fmaf(m1, py, qy);
            if (t3 != 0.0f) qy = fmaf(t3, px, qy);
            float qz = __fmul_rn(m2, pz);
            if (t5 != 0.0f) qz = fmaf(t5, py, qz);
            if (t4 != 0.0f) qz = fmaf(t4, px, qz);
            if (MIXED || w != 1.0f) {
                qx = __fmul_rn(w, qx);
                qy = __fmul_rn(w, qy);
                qz = __fmul_rn(w, qz);
            }
            if (NN && !fold) {
                qx = __fsub_rn(qx, __fmul_rn(C, px));
                qy = __fsub_rn(qy, __fmul_rn(C, py));
                qz = __fsub_rn(qz, __fmul_rn(C, pz));
            }
            ax[j] += q_bits(qx, scale);
            ay[j] += q_bits(qy, scale);
            az[j] += q_bits(qz, scale);
        }
    }
}

template <bool MIXED, int OX, int OY, int H, int... Ks>
__device__ __forceinline__ void gcells(std::integer_sequence<int, Ks...>, const float (&vx)[12], const float (&vy)[12],
                                       const float (&vz)[12], const float (&vl)[12], const float (&Lt)[4], float w_u,
                                       float C, float scale, uint32_t (&ax)[4], uint32_t (&ay)[4], uint32_t (&az)[4])
{
    (gcell<MIXED, OX, OY, Ks - H>(vx, vy, vz, vl, Lt, w_u, C, scale, ax, ay, az), ...);
}

__device__ __forceinline__ void lds4(float *dst, const float *src)
{
    const float4 v = *reinterpret_cast<const float4 *>(src);
    dst[0] = v.x;
    dst[1] = v.y;
    dst[2] = v.z;
    dst[3] = v.w;
}

// All contributions of column CI to the 4 sites whose first slot is slot0.
template <int RC, bool MIXED, int CI>
__device__ __forceinline__ void gcolumn(const float *__restrict__ tp, int cs, int slot0, int T1, int T2, float w_u,
                                        const float (&Lt)[4], float C, float scale, uint32_t (&ax)[4],
                                        uint32_t (&ay)[4], uint32_t (&az)[4])
{
    constexpr GCol cl = gcol_at(RC, CI);
    const int base = slot0 + (cl.x * T1 + cl.y) * T2;
    float vx[12], vy[12], vz[12], vl[12];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        if (c != 1 && cl.h == 0) continue;  // a column of one cell per site needs only its own chunk
        lds4(vx + 4 * c, tp + base + 4 * (c - 1));
        lds4(vy + 4 * c, tp + cs + base + 4 * (c - 1));
        lds4(vz + 4 * c, tp + 2 * cs + base + 4 * (c - 1));
        if (MIXED) lds4(vl + 4 * c, tp + 3 * cs + base + 4 * (c - 1));
    }
    gcells<MIXED, cl.x, cl.y, cl.h>(std::make_integer_sequence<int, 2 * cl.h + 1>{}, vx, vy, vz, vl, Lt, w_u, C, scale,
                                    ax, ay, az);
}

template <int RC, bool MIXED, int... Cs>
__device__ __forceinline__ void gcolumns(std::integer_sequence<int, Cs...>, const float *tp, int cs, int slot0, int T1,
                                         int T2, float w_u, const float (&Lt)[4], float C, float scale,
                                         uint32_t (&ax)[4], uint32_t (&ay)[4], uint32_t (&az)[4])
{
    (gcolumn<RC, MIXED, Cs>(tp, cs, slot0, T1, T2, w_u, Lt, C, scale, ax, ay, az), ...);
}

template <int RC, bool MIXED>
__global__ void __launch_bounds__(SN_GFIELD_THREADS, 2) gfield_tiled(const SnFieldArgs a)
{
    using G = Geo<RC, false>;
    constexpr int NP = G::NP, NT = SN_GFIELD_THREADS;
    extern __shared__ __align__(16) unsigned char smem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const SnWork w = a.work[blockIdx.x];
    const SnReplicaDev &R = a.reps[w.rep];
    const SnTile &Gm = a.geoms[R.geom];
    const int Y = R.Y, Z = R.Z;
    const int Bx = Gm.B[0], By = Gm.B[1], Bz = Gm.B[2];
    const int T1 = Gm.cT[1], T2 = Gm.cT[2], cs = Gm.cslots;
    const float C = (float)a.cage, Kk = (float)a.K;
    const float Ex = R.E[0], Ey = R.E[1], Ez = R.E[2];
    const float w_u = __fmul_rn(R.length, R.length);
    const float scale = R.gscale;
    const double ginv = (double)R.ginv;
    const long long N = R.n_sites;
    float *tp = reinterpret_cast<float *>(smem);
    double *red = reinterpret_cast<double *>(smem + sn_align16((MIXED ? 4u : 3u) * (uint32_t)cs * 4u));

    stage_p_tile<MIXED>(R, Gm, w, tp, tid, NT);
    cp_async_wait_all();
    __syncthreads();

    // The energy and polarisation sums of the thread's sites as compensated
    // FP32 sums (FP64 is a slow pipe on this GPU; it is used only to add the
    // warps' results): 0 p.g (in units of 2^-k), 2 p.E, 3 |px| + |py| (K
    // term), 4-6 L p, 7-9 p.
    KahanF acc[10];
    const uint32_t bias = (uint32_t)(2 * NP) * SN_Q_MAGIC_BITS;
    auto site_sums = [&](int slot, long long site, int gx, int gy, int gz) {
        const float px = tp[slot], py = tp[cs + slot], pz = tp[2 * cs + slot];
        const float Li = R.len[site];  // 0 at vacancies, whose dipole is zero
        acc[0].add(fmaf(px, (float)gx, fmaf(py, (float)gy, pz * (float)gz)));
        acc[2].add(fmaf(px, Ex, fmaf(py, Ey, pz * Ez)));
        if (Kk > 0.0f && Li != 0.0f) acc[3].add(fabsf(px) + fabsf(py));
        acc[4].add(Li * px);
        acc[5].add(Li * py);
        acc[6].add(Li * pz);
        acc[7].add(px);
        acc[8].add(py);
        acc[9].add(pz);
    };
    if constexpr (RC <= 4) {
        // column form: 4 consecutive z sites per thread (Bz, Z and the z halo are multiples of 4)
        const int nzb = Bz >> 2, ncol = Bx * By * nzb;
        for (int i = tid; i < ncol; i += NT) {
            const int lz0 = 4 * (i % nzb), ly = (i / nzb) % By, lx = i / (nzb * By);
            const int slot0 = ((lx + Gm.cH[0]) * T1 + ly + Gm.cH[1]) * T2 + lz0 + Gm.cH[2];
            float Lt[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            if (MIXED) lds4(Lt, tp + 3 * cs + slot0);
            uint32_t ax[4] = {0u, 0u, 0u, 0u}, ay[4] = {0u, 0u, 0u, 0u}, az[4] = {0u, 0u, 0u, 0u};
            gcolumns<RC, MIXED>(std::make_integer_sequence<int, gcol_count(RC)>{}, tp, cs, slot0, T1, T2, w_u, Lt, C,
                                scale, ax, ay, az);
            int4 gx, gy, gz;
            gx.x = (int)(ax[0] - bias), gx.y = (int)(ax[1] - bias), gx.z = (int)(ax[2] - bias), gx.w = (int)(ax[3] - bias);
            gy.x = (int)(ay[0] - bias), gy.y = (int)(ay[1] - bias), gy.z = (int)(ay[2] - bias), gy.w = (int)(ay[3] - bias);
            gz.x = (int)(az[0] - bias), gz.y = (int)(az[1] - bias), gz.z = (int)(az[2] - bias), gz.w = (int)(az[3] - bias);
            const long long site0 = ((long long)(w.x0 + lx) * Y + (w.y0 + ly)) * Z + w.z0 + lz0;
            if (a.write_g) {
                *reinterpret_cast<int4 *>(R.gcache + site0) = gx;
                *reinterpret_cast<int4 *>(R.gcache + N + site0) = gy;
                *reinterpret_cast<int4 *>(R.gcache + 2 * N + site0) = gz;
            }
            site_sums(slot0, site0, gx.x, gy.x, gz.x);
            site_sums(slot0 + 1, site0 + 1, gx.y, gy.y, gz.y);
            site_sums(slot0 + 2, site0 + 2, gx.z, gy.z, gz.z);
            site_sums(slot0 + 3, site0 + 3, gx.w, gy.w, gz.w);
        }
    } else {
        const int nsite = Bx * By * Bz;
        for (int i = tid; i < nsite; i += NT) {
            const int lz = i % Bz, ly = (i / Bz) % By, lx = i / (Bz * By);
            const int slot = ((lx + Gm.cH[0]) * T1 + ly + Gm.cH[1]) * T2 + lz + Gm.cH[2];
            const float Lt = MIXED ? tp[3 * cs + slot] : 0.0f;
            uint32_t ax = 0u, ay = 0u, az = 0u;
            q_pairs<RC, MIXED>(std::make_integer_sequence<int, NP>{}, tp, cs, slot, T1, T2, w_u, Lt, C, scale, ax, ay,
                               az);
            const int gx = (int)(ax - bias), gy = (int)(ay - bias), gz = (int)(az - bias);
            const long long site = ((long long)(w.x0 + lx) * Y + (w.y0 + ly)) * Z + w.z0 + lz;
            if (a.write_g) {
                R.gcache[site] = gx;
                R.gcache[N + site] = gy;
                R.gcache[2 * N + site] = gz;
            }
            site_sums(slot, site, gx, gy, gz);
        }
    }
    // warp sums of the (sum, error) pairs by error-free additions (TwoSum)
    float hs[10], hc[10];
#pragma unroll
    for (int k = 0; k < 10; k++) {
        hs[k] = acc[k].s;
        hc[k] = -acc[k].c;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 10; k++) {
            if (k == 1) continue;
            const float bs = __shfl_xor_sync(0xffffffffu, hs[k], o), bc = __shfl_xor_sync(0xffffffffu, hc[k], o);
            const float t2 = __fadd_rn(hs[k], bs);
            const float bb = __fsub_rn(t2, hs[k]);
            const float err = __fadd_rn(__fsub_rn(hs[k], __fsub_rn(t2, bb)), __fsub_rn(bs, bb));
            hs[k] = t2;
            hc[k] = __fadd_rn(__fadd_rn(hc[k], bc), err);
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 10; k++) {
            double v = k == 1 ? 0.0 : (double)hs[k] + (double)hc[k];
            if (k == 0) v *= 0.5 * ginv;
            else if (k == 3) v *= -(double)Kk;
            red[warp * 16 + k] = v;
        }
    }
    __syncthreads();
    if (tid < 10 && a.red) {
        double s = 0.0;
        for (int q = 0; q < (NT >> 5); q++) s += red[q * 16 + tid];
        atomicAdd(&a.red[a.red_stride * w.rep + tid], s);
    }
}

__host__ __device__ inline int sn_gfield_smem(int cslots, bool mixed)
{
    return (int)(sn_align16((mixed ? 4u : 3u) * (uint32_t)cslots * 4u) + (SN_GFIELD_THREADS / 32) * 16u * 8u);
}

}  // namespace sn_sweep
