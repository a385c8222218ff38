// sn_gpu.cu -- host implementation of the C ABI in include/sn_gpu.h.
//
// One handle = one replica table resident in HBM + one CUDA stream.  A sweep
// is captured once as a CUDA graph (one dataflow launch of the sweep kernel
// per kernel variant -- or, with SN_SCHEDULE=phases, 8 block-colour launches
// -- plus the end-of-sweep fold) and replayed; every per-sweep quantity the
// kernels need (sweep index, temperatures, fields) lives in device memory so
// the graph never changes.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/sn_gpu.h"
#include "sn_launch.h"
#include "sn_sweep.cuh"

namespace {

const sn_sweep_launch_fn k_sweep[SN_MAX_CUTOFF + 1] = {nullptr,
                                                        sn_launch_sweep_rc1,
                                                        sn_launch_sweep_rc2,
                                                        sn_launch_sweep_rc3,
                                                        sn_launch_sweep_rc4,
                                                        sn_launch_sweep_rc5,
                                                        sn_launch_sweep_rc6};
const sn_field_launch_fn k_field[SN_MAX_CUTOFF + 1] = {nullptr,
                                                        sn_launch_field_rc1,
                                                        sn_launch_field_rc2,
                                                        sn_launch_field_rc3,
                                                        sn_launch_field_rc4,
                                                        sn_launch_field_rc5,
                                                        sn_launch_field_rc6};
const sn_geo_fn k_geo[SN_MAX_CUTOFF + 1] = {nullptr,     sn_geo_rc1, sn_geo_rc2, sn_geo_rc3,
                                            sn_geo_rc4,  sn_geo_rc5, sn_geo_rc6};
const sn_flow_launch_fn k_flow[SN_MAX_CUTOFF + 1] = {nullptr,
                                                      sn_launch_flow_rc1,
                                                      sn_launch_flow_rc2,
                                                      sn_launch_flow_rc3,
                                                      sn_launch_flow_rc4,
                                                      sn_launch_flow_rc5,
                                                      sn_launch_flow_rc6};

const sn_cached_smem_fn k_cached_smem[SN_MAX_CUTOFF + 1] = {nullptr,            sn_cached_smem_rc1, sn_cached_smem_rc2,
                                                             sn_cached_smem_rc3, sn_cached_smem_rc4, sn_cached_smem_rc5,
                                                             sn_cached_smem_rc6};
const sn_gfield_launch_fn k_gfield[SN_MAX_CUTOFF + 1] = {nullptr,            sn_launch_gfield_rc1, sn_launch_gfield_rc2,
                                                         sn_launch_gfield_rc3, sn_launch_gfield_rc4, sn_launch_gfield_rc5,
                                                         sn_launch_gfield_rc6};

const int kSmemLimit = 227 * 1024;

// Unique key of block (bx, by, bz) of replica rep (block indices < 2^14 per axis: the
// planner's blocks are >= 2 sites and lattice sides < 2^15).  The key must not depend on
// the replica's block counts: replicas of different shapes share one dataflow list.
inline uint64_t block_key(int rep, int bx, int by, int bz)
{
    return ((uint64_t)rep << 42) | ((uint64_t)bx << 28) | ((uint64_t)by << 14) | (uint64_t)bz;
}

// Host-side launch plan of a replica table: per block colour and kernel variant (3D, 2D) the work
// lists of the eight-launch schedule, per replica the list of all its blocks (field passes), and per
// variant the dataflow list -- the blocks in block-colour order, each with the indices of the adjacent
// blocks of earlier colour (the blocks whose sites its halo reads and that must finish first).  Items
// only wait on items earlier in their list, which a running CTA has already taken.
struct SnPlan {
    std::vector<SnWork> work;
    int work_off[16] = {}, work_cnt[16] = {}, work_smem[16] = {}, work_thr[16] = {};
    std::vector<int> fwork_off, fwork_cnt;
    int flow_off[2] = {0, 0}, flow_items[2] = {0, 0};
    std::vector<int> deps;  // SN_MAX_DEPS ints per work entry: count, then list positions
};

int block_colour(const SnTile &t, const int *c) { return (c[0] % t.m[0]) * 4 + (c[1] % t.m[1]) * 2 + (c[2] % t.m[2]); }

// Dynamic shared memory and threads of the sweep kernel that runs replica
// tile t: the cached-field kernel (t.cmode) or the stencil kernel.
int sweep_smem(const SnTile &t) { return t.cmode ? t.csmem : t.smem_bytes; }
int sweep_threads(const SnTile &t) { return t.cmode ? SN_CACHED_THREADS : t.threads; }

bool build_plan(const std::vector<SnTile> &tiles, const sn_replica_desc *replicas, int n, bool flow, SnPlan &pl,
                std::string &why, int ready = 512)
{
    // SN_FLOW_GROUP=W forces groups of W x slabs (-1: plain colour order); see below
    int flow_group = 0;
    if (const char *env = getenv("SN_FLOW_GROUP")) flow_group = atoi(env);
    std::vector<SnWork> &work = pl.work;
    for (int p = 0; p < 8; p++)
        for (int v = 0; v < 2; v++) {
            const int k = p * 2 + v;
            pl.work_off[k] = (int)work.size();
            const int cb[3] = {(p >> 2) & 1, (p >> 1) & 1, p & 1};
            for (int r = 0; r < n; r++) {
                const bool two_d = replicas[r].Z == 1;
                if ((v == 1) != two_d) continue;
                const SnTile &t = tiles[r];
                for (int bx = 0; bx < t.nb[0]; bx++)
                    for (int by = 0; by < t.nb[1]; by++)
                        for (int bz = 0; bz < t.nb[2]; bz++) {
                            if (bx % t.m[0] != cb[0] || by % t.m[1] != cb[1] || bz % t.m[2] != cb[2]) continue;
                            work.push_back(SnWork{r, bx * t.B[0], by * t.B[1], bz * t.B[2]});
                            pl.work_smem[k] = std::max(pl.work_smem[k], sweep_smem(t));
                            pl.work_thr[k] = std::max(pl.work_thr[k], sweep_threads(t));
                        }
            }
            pl.work_cnt[k] = (int)work.size() - pl.work_off[k];
        }
    pl.fwork_off.assign(n, 0);
    pl.fwork_cnt.assign(n, 0);
    for (int r = 0; r < n; r++) {
        const SnTile &t = tiles[r];
        pl.fwork_off[r] = (int)work.size();
        for (int bx = 0; bx < t.nb[0]; bx++)
            for (int by = 0; by < t.nb[1]; by++)
                for (int bz = 0; bz < t.nb[2]; bz++) work.push_back(SnWork{r, bx * t.B[0], by * t.B[1], bz * t.B[2]});
        pl.fwork_cnt[r] = (int)work.size() - pl.fwork_off[r];
    }
    std::vector<int> &deps = pl.deps;
    for (int v = 0; v < 2 && flow; v++) {
        pl.flow_off[v] = (int)work.size();
        std::unordered_map<uint64_t, int> index;  // (replica, block) -> position in this list
        // Queue order.  A replica whose block colours each hold at least
        // `ready` blocks per group of W x slabs (block rows) is queued in such
        // groups: the group's even slabs (block colours 0-3) in colour order,
        // then the previous group's odd slabs (colours 4-7, which wait on even
        // slabs of both groups), then the next group ...; the last group's odd
        // slabs, which wait on slab 0 across the wrap, close its list.  Every
        // block follows the blocks it waits on, enough blocks are ready at any
        // time to fill the GPU, and the blocks in flight cover about two groups,
        // so more halo re-reads hit L2.  Smaller replicas are queued together
        // in plain colour order (colour 0 of all of them, then colour 1 ...).
        // Within a colour: x, y, then z.
        auto push_colour = [&](int r, int p, int bx0, int bx1) {
            const SnTile &t = tiles[r];
            const int cb[3] = {(p >> 2) & 1, (p >> 1) & 1, p & 1};
            for (int bx = bx0; bx < bx1; bx++) {
                if (bx % t.m[0] != cb[0]) continue;
                for (int by = 0; by < t.nb[1]; by++)
                    for (int bz = 0; bz < t.nb[2]; bz++) {
                        if (by % t.m[1] != cb[1] || bz % t.m[2] != cb[2]) continue;
                        index[block_key(r, bx, by, bz)] = (int)work.size() - pl.flow_off[v];
                        work.push_back(SnWork{r, bx * t.B[0], by * t.B[1], bz * t.B[2]});
                    }
            }
        };
        std::vector<int> small, large, width(n, 0);
        for (int r = 0; r < n; r++) {
            if ((replicas[r].Z == 1) != (v == 1)) continue;
            const SnTile &t = tiles[r];
            const int nbx = t.nb[0];
            const long long per_slab = (long long)t.nb[1] * t.nb[2] / (t.m[1] * t.m[2]);  // one colour, one slab
            int W = nbx;
            if (t.m[0] == 2) {
                if (flow_group > 0) {
                    if (flow_group < nbx && nbx % flow_group == 0 && flow_group % 2 == 0) W = flow_group;
                } else if (flow_group == 0) {
                    for (int c = 2; c < nbx; c += 2)
                        if (nbx % c == 0 && (long long)(c / 2) * per_slab >= ready) {
                            W = c;
                            break;
                        }
                }
            }
            width[r] = W;
            (W == nbx ? small : large).push_back(r);
        }
        for (int p = 0; p < 8; p++)
            for (int r : small) push_colour(r, p, 0, tiles[r].nb[0]);
        for (int r : large) {
            const int W = width[r], G = tiles[r].nb[0] / W;
            for (int g = 0; g < G; g++) {
                for (int p = 0; p < 4; p++) push_colour(r, p, g * W, (g + 1) * W);
                if (g > 0)
                    for (int p = 4; p < 8; p++) push_colour(r, p, (g - 1) * W, g * W);
            }
            for (int p = 4; p < 8; p++) push_colour(r, p, (G - 1) * W, G * W);
        }
        pl.flow_items[v] = (int)work.size() - pl.flow_off[v];
        deps.resize((size_t)(pl.flow_off[v] + pl.flow_items[v]) * SN_MAX_DEPS, 0);
        for (int i = 0; i < pl.flow_items[v]; i++) {
            const SnWork w = work[pl.flow_off[v] + i];
            const SnTile &t = tiles[w.rep];
            const int b[3] = {w.x0 / t.B[0], w.y0 / t.B[1], w.z0 / t.B[2]};
            const int own = block_colour(t, b);
            int *dl = &deps[(size_t)(pl.flow_off[v] + i) * SN_MAX_DEPS];
            for (int dx = -1; dx <= 1; dx++)
                for (int dy = -1; dy <= 1; dy++)
                    for (int dz = -1; dz <= 1; dz++) {
                        const int c[3] = {(b[0] + dx + t.nb[0]) % t.nb[0], (b[1] + dy + t.nb[1]) % t.nb[1],
                                          (b[2] + dz + t.nb[2]) % t.nb[2]};
                        if (c[0] == b[0] && c[1] == b[1] && c[2] == b[2]) continue;
                        const int q = block_colour(t, c);
                        if (q == own) {
                            why = "adjacent blocks share a colour";
                            return false;
                        }
                        if (q > own) continue;
                        const auto it = index.find(block_key(w.rep, c[0], c[1], c[2]));
                        if (it == index.end()) {
                            why = "dataflow list misses a block";
                            return false;
                        }
                        const int j = it->second;
                        bool seen = false;
                        for (int u = 1; u <= dl[0]; u++) seen |= dl[u] == j;
                        if (seen) continue;
                        if (dl[0] + 1 >= SN_MAX_DEPS) {
                            why = "too many dependencies";
                            return false;
                        }
                        dl[++dl[0]] = j;
                    }
        }
    }
    if (flow) deps.resize(work.size() * SN_MAX_DEPS, 0);
    return true;
}
// the sweep kernels' static shared memory (the dataflow queue slot) comes on top of the planned tile
const int kSweepStatic = 128;
// per-block shared memory that still lets two blocks share an SM (228 KB per
// SM, 1 KB reserved per block)
const int kSmemTwoPerSm = (228 * 1024 - 2 * 1024) / 2 - kSweepStatic;

thread_local std::string g_last_error;

// ---------------------------------------------------------------------------
// Planner.

int ceil_div(int a, int b) { return (a + b - 1) / b; }

void axis_starts(int T, int S, int *start)
{
    int acc = 0;
    for (int k = 0; k < SN_MAX_S; k++) {
        start[k] = acc;
        if (k < S && k < T) acc += (T - k + S - 1) / S;
    }
}

int pi_host(const int *start, int S, int u) { return start[u % S] + u / S; }

// Sum over site colours and warps of the worst bank multiplicity of the
// targets' slots (32 lanes -> 32 banks is the ideal: cost 1 per warp).  A
// slot is 3 words, so distinct slots mod 32 are distinct banks.
// Lane t of a colour is target (qx,qy,qz) = t unravelled over nq (z
// fastest); lanes beyond the colour's own target count are idle.
long long conflict_cost(const SnTile &t, int S, bool two_d, int Sy, int Sx)
{
    long long cost = 0;
    const int SZ = two_d ? 1 : S;
    const int ntp = t.nq[0] * t.nq[1] * t.nq[2];
    int cnt[32];
    for (int cx = 0; cx < S; cx++)
        for (int cy = 0; cy < S; cy++)
            for (int cz = 0; cz < SZ; cz++) {
                const int nx = cx < t.B[0] ? ceil_div(t.B[0] - cx, S) : 0;
                const int ny = cy < t.B[1] ? ceil_div(t.B[1] - cy, S) : 0;
                const int nz = two_d ? 1 : (cz < t.B[2] ? ceil_div(t.B[2] - cz, S) : 0);
                if (!(nx && ny && nz)) continue;
                const int bx0 = pi_host(t.start[0], S, cx + t.H[0]);
                const int by0 = pi_host(t.start[1], S, cy + t.H[1]);
                const int bz0 = two_d ? 0 : cz + t.H[2];  // z stored plainly
                for (int w0 = 0; w0 < ntp; w0 += 32) {
                    memset(cnt, 0, sizeof(cnt));
                    int worst = 0;
                    for (int q = w0; q < std::min(ntp, w0 + 32); q++) {
                        const int qz = q % t.nq[2], qy = (q / t.nq[2]) % t.nq[1], qx = q / (t.nq[2] * t.nq[1]);
                        if (qx >= nx || qy >= ny || qz >= nz) continue;
                        const long long slot = (long long)(bx0 + qx) * Sx + (long long)(by0 + qy) * Sy + bz0 + S * qz;
                        worst = std::max(worst, ++cnt[(int)(slot & 31)]);
                    }
                    cost += worst;
                }
            }
    return cost;
}

struct AxisChoice {
    std::vector<int> cands;
};

// Candidate block sizes along an axis of length L: L/B even (a 2-colouring
// of the blocks is then consistent across the periodic boundary) and
// B >= cutoff (same-colour blocks are then more than cutoff apart).
std::vector<int> block_candidates(int L, int rc)
{
    std::vector<int> c;
    for (int B = std::max(rc, 1); B <= L / 2; B++)
        if (L % B == 0 && (L / B) % 2 == 0) c.push_back(B);
    return c;
}

// Geometry of the cached-field sweep for t's block shape (t.cmode = 1), or
// false when the shape does not admit it: every block side >= 2 cutoff (tiles
// of blocks that may run together are then disjoint), Z and the z side
// multiples of 4 (16-byte tile rows), at most SN_CACHED_THREADS targets per
// colour group, and a tile that fits `limit` bytes with >= pc_min groups of
// proposals staged.
bool plan_cached(SnTile &t, int Z, int rc, bool mixed, int limit, int pc_min)
{
    if (Z == 1 || Z % 4 || t.B[2] % 4) return false;
    for (int a = 0; a < 3; a++)
        if (t.B[a] < 2 * rc) return false;
    if (t.tg > SN_CACHED_THREADS) return false;
    t.cH[0] = rc;
    t.cH[1] = rc;
    t.cH[2] = (rc + 3) / 4 * 4;
    for (int a = 0; a < 3; a++) t.cT[a] = t.B[a] + 2 * t.cH[a];
    t.cslots = t.cT[0] * t.cT[1] * t.cT[2];
    // proposal chunks (two buffered): up to 8 groups each, as many as fit
    t.cpc = std::min(t.ng, 8);
    while (t.cpc > 1 && k_cached_smem[rc](t.cslots, t.tg, t.cpc, mixed, t.ng) > limit) t.cpc--;
    t.csmem = k_cached_smem[rc](t.cslots, t.tg, t.cpc, mixed, t.ng);
    if (t.csmem > limit || t.cpc < pc_min) return false;
    if (sn_sweep::sn_gfield_smem(t.cslots, mixed) > kSmemLimit) return false;
    t.cmode = 1;
    return true;
}

// Feasible tile plans of an X x Y x Z replica in preference order (at most
// max_out; force = a block shape to use instead of choosing); cached: plans
// for the cached-field sweep only.
bool plan_tiles(int X, int Y, int Z, int rc, bool mixed, std::vector<SnTile> &outs, size_t max_out, std::string &why,
                const int *force_shape = nullptr, bool cached = false)
{
    if (rc < 1 || rc > SN_MAX_CUTOFF) {
        why = "cutoff outside 1.." + std::to_string(SN_MAX_CUTOFF);
        return false;
    }
    const bool two_d = (Z == 1);
    int S, SZ, NS, NF, merge;
    k_geo[rc](two_d, &S, &SZ, &NS, &NF, &merge);
    const int L[3] = {X, Y, Z};
    std::vector<int> cands[3];
    for (int a = 0; a < 3; a++) {
        if (a == 2 && two_d) {
            cands[a] = {1};
            continue;
        }
        cands[a] = block_candidates(L[a], rc);
        if (cands[a].empty()) {
            why = "axis " + std::string(1, "XYZ"[a]) + "=" + std::to_string(L[a]) +
                  " has no even number of blocks of at least cutoff=" + std::to_string(rc) + " sites";
            return false;
        }
    }
    struct Cand {
        int B[3];
        long long vol;
        int balanced;
    };
    std::vector<Cand> all;
    // a forced block shape (the replica's own, else SN_BLOCK="bx,by,bz"); it must be valid
    int force[3] = {0, 0, 0};
    if (force_shape && force_shape[0] > 0) {
        for (int a = 0; a < 3; a++) force[a] = force_shape[a];
    } else if (const char *env = getenv("SN_BLOCK")) {
        if (sscanf(env, "%d,%d,%d", &force[0], &force[1], &force[2]) != 3) force[0] = 0;
    }
    for (int bx : cands[0])
        for (int by : cands[1])
            for (int bz : cands[2]) {
                if (force[0] && (bx != force[0] || by != force[1] || bz != force[2])) continue;
                if (cached && (two_d || bx < 2 * rc || by < 2 * rc || bz < 2 * rc || bz % 4 || Z % 4)) continue;
                Cand c{{bx, by, bz}, (long long)bx * by * bz, 0};
                c.balanced = (bx % S == 0) + (by % S == 0) + (two_d || bz % S == 0);
                all.push_back(c);
            }
    // Largest blocks first, then the smallest tile (least halo per site),
    // balanced colours, and longer z and y extents (contiguous rows).
    auto tile_sites = [&](const Cand &c) {
        return (long long)(c.B[0] + 2 * rc) * (c.B[1] + 2 * rc) * (two_d ? 1 : c.B[2] + 2 * rc);
    };
    std::sort(all.begin(), all.end(), [&](const Cand &a, const Cand &b) {
        if (a.vol != b.vol) return a.vol > b.vol;
        // the cached-field sweep moves whole z rows (16-byte chunks): longer rows first (measured faster)
        if (cached && a.B[2] != b.B[2]) return a.B[2] > b.B[2];
        if (tile_sites(a) != tile_sites(b)) return tile_sites(a) < tile_sites(b);
        if (a.balanced != b.balanced) return a.balanced > b.balanced;
        if (a.B[2] != b.B[2]) return a.B[2] > b.B[2];
        return a.B[1] > b.B[1];
    });
    const int nh = merge ? 2 : 1;
    const int ng = (merge ? S / 2 : S) * S * SZ;
    // Pass 0 looks for shapes that fit two blocks per SM (each block's
    // barriers then overlap the other's work: measured faster at 256^3);
    // pass 1 takes the largest shape that fits one block per SM.
    for (int pass = 0; pass < 2; pass++) {
        const int pass_limit = pass == 0 ? kSmemTwoPerSm : kSmemLimit - kSweepStatic;
        // the stencil tile (sweep and field pass); with the cached sweep only
        // the field pass uses it, which may take a whole SM
        const int limit = cached ? kSmemLimit - kSweepStatic : pass_limit;
        for (const Cand &c : all) {
            SnTile t;
            memset(&t, 0, sizeof(t));
            for (int a = 0; a < 3; a++) {
                t.B[a] = c.B[a];
                t.H[a] = (a == 2 && two_d) ? 0 : rc;
                t.T[a] = (a == 2 && two_d) ? 1 : c.B[a] + 2 * rc;
                t.nb[a] = L[a] / c.B[a];
                t.m[a] = (a == 2 && two_d) ? 1 : 2;
                t.nq[a] = (a == 2 && two_d) ? 1 : ceil_div(c.B[a], S);
                axis_starts(t.T[a], S, t.start[a]);
            }
            t.tp = ceil_div(t.nq[0] * t.nq[1] * t.nq[2], 32) * 32;
            t.tg = nh * t.tp;
            t.threads = NS * t.tg;
            t.ng = ng;
            t.merge = merge;
            if (t.threads > (pass == 0 && !cached ? SN_TWO_PER_SM_THREADS : SN_SWEEP_MAX_THREADS)) continue;
            const int pc_min = pass == 0 && !cached ? std::min(8, ng) : 1;
            // quick lower bound on shared memory with no padding
            if ((int)sn_sweep::sn_carve(t.T[0] * t.T[1] * t.T[2], t.tg, pc_min, NS, S, NF, mixed, 4).total > limit)
                continue;
            long long best = -1;
            int bSy = 0, bSx = 0;
            for (int dy = 0; dy < 32; dy++) {
                const int Sy = t.T[2] + dy;
                for (int dx = 0; dx < 32; dx++) {
                    const int Sx = t.T[1] * Sy + dx;
                    if ((int)sn_sweep::sn_carve(Sx * t.T[0], t.tg, pc_min, NS, S, NF, mixed, 4).total > limit)
                        continue;
                    const long long cost = conflict_cost(t, S, two_d, Sy, Sx);
                    if (best < 0 || cost < best) {
                        best = cost;
                        bSy = Sy;
                        bSx = Sx;
                    }
                }
            }
            if (best < 0) continue;
            t.Sy = bSy;
            t.Sx = bSx;
            t.slots = bSx * t.T[0];
            // stage as many groups' proposals at once as the budget allows
            t.pc = ng;
            while (t.pc > 1 && (int)sn_sweep::sn_carve(t.slots, t.tg, t.pc, NS, S, NF, mixed, 4).total > limit) t.pc--;
            t.smem_bytes = (int)sn_sweep::sn_carve(t.slots, t.tg, t.pc, NS, S, NF, mixed, 4).total;
            t.field_smem = (int)sn_sweep::sn_carve(t.slots, t.tg, 0, NS, S, NF, mixed, 8).total;
            if (t.smem_bytes > limit || t.field_smem > kSmemLimit || t.pc < pc_min) continue;
            // two buffered chunks of >= 2 groups keep the proposal copies ahead of their use
            if (cached && !plan_cached(t, Z, rc, mixed, pass_limit - kSweepStatic, std::min(2, ng)))
                continue;
            bool seen = false;  // pass 1 meets pass 0's shapes again
            for (const SnTile &o : outs) seen |= o.B[0] == t.B[0] && o.B[1] == t.B[1] && o.B[2] == t.B[2];
            if (seen) continue;
            outs.push_back(t);
            if (outs.size() >= max_out) return true;
        }
    }
    if (!outs.empty()) return true;
    if (force[0])
        why = "block shape " + std::to_string(force[0]) + "x" + std::to_string(force[1]) + "x" +
              std::to_string(force[2]) + " does not tile this lattice (even block counts, blocks >= cutoff) or fit "
                                         "in shared memory";
    else
        why = "no block shape fits in shared memory for this lattice and cutoff";
    return false;
}

bool plan_tile(int X, int Y, int Z, int rc, bool mixed, SnTile &out, std::string &why, const int *force = nullptr,
               bool cached = false)
{
    std::vector<SnTile> v;
    if (!plan_tiles(X, Y, Z, rc, mixed, v, 1, why, force, cached)) return false;
    out = v[0];
    return true;
}

// The sweep method a table asks for: sn_params.sweep_method, overridden by
// the environment variable SN_SWEEP=stencil|cached.
int sweep_method(const sn_params &P)
{
    if (const char *env = getenv("SN_SWEEP")) {
        if (!strcmp(env, "stencil")) return SN_SWEEP_STENCIL;
        if (!strcmp(env, "cached")) return SN_SWEEP_CACHED;
    }
    return P.sweep_method;
}

// Tiles of every replica of a table.  The 3D replicas all take the cached-
// field sweep (auto: when every one of them admits it) or all the stencil
// sweep; 2D replicas always take the stencil sweep.  *cached = the choice.
bool plan_table(const sn_params &P, int n, const sn_replica_desc *replicas, bool mixed, std::vector<SnTile> &tiles,
                bool *cached, std::string &why)
{
    const int method = sweep_method(P);
    if (method != SN_SWEEP_AUTO && method != SN_SWEEP_STENCIL && method != SN_SWEEP_CACHED) {
        why = "unknown sweep_method " + std::to_string(method);
        return false;
    }
    tiles.assign(n, SnTile{});
    bool use = method != SN_SWEEP_STENCIL;
    for (int r = 0; r < n && use; r++) {
        const sn_replica_desc &d = replicas[r];
        if (d.Z == 1) continue;
        std::string w;
        if (!plan_tile(d.X, d.Y, d.Z, P.cutoff, mixed, tiles[r], w, d.block, true)) {
            if (method == SN_SWEEP_CACHED) {
                why = "replica " + std::to_string(r) + " (" + std::to_string(d.X) + "x" + std::to_string(d.Y) + "x" +
                      std::to_string(d.Z) + "): no block shape for the cached-field sweep (block sides >= 2 cutoff, "
                      "Z and bz multiples of 4, tile in shared memory)";
                return false;
            }
            use = false;
        }
    }
    for (int r = 0; r < n; r++) {
        const sn_replica_desc &d = replicas[r];
        if (use && d.Z > 1) continue;
        std::string w;
        if (!plan_tile(d.X, d.Y, d.Z, P.cutoff, mixed, tiles[r], w, d.block, false)) {
            why = "replica " + std::to_string(r) + " (" + std::to_string(d.X) + "x" + std::to_string(d.Y) + "x" +
                  std::to_string(d.Z) + "): " + w;
            return false;
        }
    }
    *cached = use && std::any_of(replicas, replicas + n, [](const sn_replica_desc &d) { return d.Z > 1; });
    return true;
}

// Power-of-two scale 2^k of the field cache: every contribution satisfies
// |c| 2^k < 2^22 (the rounding of q_bits) and every field |g| 2^k < 2^30,
// for dipole components |p| <= 1.0001 (checked at upload) and lengths up to
// Lmax.  The bounds take each offset tensor's largest row sum.
int cache_scale(int rc, double Lmax, double C)
{
    double vmax = 0.0, gsum = 0.0;
    for (int x = -rc; x <= rc; x++)
        for (int y = -rc; y <= rc; y++)
            for (int z = -rc; z <= rc; z++) {
                const int r2 = x * x + y * y + z * z;
                if (r2 == 0 || r2 > rc * rc) continue;
                const double d = std::sqrt((double)r2), i3 = 1.0 / (r2 * d), i5 = i3 / r2;
                const int o[3] = {x, y, z};
                double row = 0.0;
                for (int a = 0; a < 3; a++) {
                    double s = 0.0;
                    for (int b = 0; b < 3; b++) s += std::fabs((a == b ? i3 : 0.0) - 3.0 * o[a] * o[b] * i5);
                    row = std::max(row, s);
                }
                const double v = (Lmax * Lmax * row + (r2 == 1 ? std::fabs(C) : 0.0)) * 1.0002;
                vmax = std::max(vmax, v);
                gsum += v;
            }
    int k = 30;
    while (k > 0 && (std::ldexp(vmax, k) >= 4194304.0 || std::ldexp(gsum, k) >= 1073741824.0)) k--;
    return k;
}

void fill_info(const SnTile &t, int rc, sn_schedule_info *o)
{
    o->bx = t.B[0];
    o->by = t.B[1];
    o->bz = t.B[2];
    o->nbx = t.nb[0];
    o->nby = t.nb[1];
    o->nbz = t.nb[2];
    o->mx = t.m[0];
    o->my = t.m[1];
    o->mz = t.m[2];
    o->s = rc + 1;
    o->halo = rc;
    o->tile_slots = t.slots;
    o->smem_bytes = t.smem_bytes;
    o->merge = t.merge;
    o->threads = t.cmode ? SN_CACHED_THREADS : t.threads;
    o->field_cache = t.cmode;
    if (t.cmode) {
        o->tile_slots = t.cslots;
        o->smem_bytes = t.csmem;
    }
}

}  // namespace

// Internal helpers shared with the no-allocation entry point (sn_noalloc.cu).
void sn_internal_set_error(const char *msg) { g_last_error = msg ? msg : ""; }

bool sn_internal_plan(int X, int Y, int Z, int rc, bool mixed, SnTile *out, char *why, size_t why_len)
{
    std::string w;
    const bool ok = plan_tile(X, Y, Z, rc, mixed, *out, w);
    if (!ok && why && why_len) snprintf(why, why_len, "%s", w.c_str());
    return ok;
}

cudaError_t sn_internal_field_launch(int rc, bool fp64, bool two_d, bool mixed, const SnFieldArgsHost &a, int grid,
                                     int threads, int smem, cudaStream_t st)
{
    if (rc < 1 || rc > SN_MAX_CUTOFF) return cudaErrorInvalidValue;
    return k_field[rc](fp64, two_d, mixed, &a, grid, threads, smem, st);
}

// ---------------------------------------------------------------------------
struct sn_handle {
    sn_params params{};
    int nrep = 0;
    bool mixed = false;
    float length = 0.0f;   // uniform length
    float dipole_ref = 0.0f;
    int rc = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;  // host transfers overlapped with work on `stream`
    static constexpr int kSlabs = SN_UPLOAD_SLABS;
    cudaEvent_t slab_ev[kSlabs] = {};
    // upload: the energy pass runs in chunks alternating between two streams,
    // so one chunk's last wave overlaps the next chunk's first
    cudaStream_t field_stream[2] = {};
    cudaEvent_t conv_ev[kSlabs] = {};
    cudaEvent_t fdone_ev[2] = {};
    std::vector<sn_replica_desc> desc;
    std::vector<SnTile> tiles;
    std::vector<SnReplicaDev> reps;
    // device
    SnReplicaDev *d_reps = nullptr;
    SnTile *d_geoms = nullptr;
    SnAccum *d_acc = nullptr;
    SnState *d_state = nullptr;
    uint32_t *d_sweep = nullptr;
    double *d_hist = nullptr;
    double *d_red = nullptr;     // 10 per replica
    double *d_drift = nullptr;   // per replica
    SnExchange *d_ex = nullptr;
    int *d_order = nullptr;
    int *d_flags = nullptr;
    SnWork *d_work = nullptr;
    std::vector<int> work_off, work_cnt, work_smem, work_thr;  // [phase*2 + variant]
    std::vector<int> fwork_off, fwork_cnt;           // per replica, all blocks
    // dataflow sweep (one persistent launch per kernel variant and sweep)
    bool flow = true;
    int flow_items[2] = {0, 0}, flow_off[2] = {0, 0}, flow_grid[2] = {0, 0};
    int *d_deps = nullptr;
    uint32_t *d_done = nullptr;
    size_t done_n = 0;
    uint32_t *d_queue = nullptr;  // 2 counters
    uint32_t *d_err = nullptr;    // timeout flag, stall statistics, poll limit (SnFlowArgs::err)
    std::vector<int> deps_host;   // the dataflow lists as planned (a test hook edits one on the device)
    int stalled_item = -1;        // item whose first dependency points at the spare flag, or -1
    std::vector<float *> lattice_mem;
    // cached-field sweep of the 3D replicas: their field caches (3N int32 each)
    bool cached = false;
    int tile_copy = 0;  // cached sweep tile load: 0 = cp.async, 1 = TMA bulk copies (SN_TILE_COPY=bulk)
    std::vector<int *> gcache_mem;
    std::vector<float4 *> prop_mem;  // the coming sweep's proposals (16 B per site)
    int nsm = 0;
    // scratch (lazy)
    float *d_stage = nullptr;
    size_t stage_floats = 0;
    double *d_site = nullptr;
    size_t site_n = 0;
    float *d_grad = nullptr;
    size_t grad_n = 0;
    double *d_trace = nullptr;
    size_t trace_n = 0;
    SnAnalysisOffset *d_aoff = nullptr;  // analysis stencil table
    size_t aoff_n = 0;
    double *d_abins = nullptr;  // analysis reductions
    size_t abins_n = 0;
    // graph
    cudaGraphExec_t graph = nullptr;
    uint64_t graph_nodes = 0;
    // counters
    uint64_t launches = 0;
    uint64_t sweeps = 0;
    int exchange_every = 0;
    int recompute_every = 0;
    int recompute_prec = SN_ENERGY_FP32;
    int n_checks = 0;
    std::string err;
};

namespace {

sn_status fail(sn_handle *h, sn_status s, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (h) h->err = buf;
    g_last_error = buf;
    return s;
}

#define SN_CK(h, x)                                                                                  \
    do {                                                                                             \
        cudaError_t e_ = (x);                                                                        \
        if (e_ != cudaSuccess) return fail((h), SN_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_)); \
    } while (0)

sn_status check_rep(sn_handle *h, int r)
{
    if (!h) return fail(nullptr, SN_ERR_ARG, "null handle");
    if (r < 0 || r >= h->nrep) return fail(h, SN_ERR_ARG, "replica %d out of range [0,%d)", r, h->nrep);
    return SN_OK;
}

sn_status ensure(sn_handle *h, void **p, size_t *have, size_t need, size_t elem)
{
    if (*have >= need) return SN_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *have = 0;
    cudaError_t e = cudaMalloc(p, need * elem);
    if (e != cudaSuccess) return fail(h, SN_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", need * elem, cudaGetErrorString(e));
    *have = need;
    return SN_OK;
}

SnFieldArgsHost field_args(sn_handle *h, int r, double *site_e, float *grad, double *red, int stride)
{
    SnFieldArgsHost a;
    a.work = h->d_work + h->fwork_off[r];
    a.reps = h->d_reps;
    a.geoms = h->d_geoms;
    a.cage = h->params.cage_strain;
    a.K = h->params.K;
    a.site_e = site_e;
    a.grad = grad;
    a.red = red;
    a.red_stride = stride;
    a.write_g = 0;
    return a;
}

// Field-cache pass (exact fixed-point g and the energy sums) over the blocks
// bx in [b0, b1) of replica r, which must hold a field cache.
sn_status launch_gfield_x(sn_handle *h, int r, const SnFieldArgsHost &base, int b0, int b1, cudaStream_t st)
{
    if (b1 <= b0) return SN_OK;
    const SnTile &t = h->tiles[r];
    SnFieldArgsHost a = base;
    a.write_g = 1;
    a.work = base.work + (size_t)b0 * t.nb[1] * t.nb[2];
    SN_CK(h, k_gfield[h->rc](h->mixed, &a, (b1 - b0) * t.nb[1] * t.nb[2], sn_sweep::sn_gfield_smem(t.cslots, h->mixed),
                             st));
    h->launches++;
    return SN_OK;
}

sn_status launch_field(sn_handle *h, int r, bool fp64, const SnFieldArgsHost &a)
{
    const bool two_d = h->desc[r].Z == 1;
    SN_CK(h, k_field[h->rc](fp64, two_d, h->mixed, &a, h->fwork_cnt[r], h->tiles[r].threads, h->tiles[r].field_smem,
                            h->stream));
    h->launches++;
    return SN_OK;
}

// Field pass over the blocks bx in [b0, b1) of replica r (the replica's block
// list is x-major, so they are contiguous).
sn_status launch_field_x(sn_handle *h, int r, const SnFieldArgsHost &base, int b0, int b1, cudaStream_t st)
{
    if (b1 <= b0) return SN_OK;
    const SnTile &t = h->tiles[r];
    SnFieldArgsHost a = base;
    a.work = base.work + (size_t)b0 * t.nb[1] * t.nb[2];
    SN_CK(h, k_field[h->rc](false, h->desc[r].Z == 1, h->mixed, &a, (b1 - b0) * t.nb[1] * t.nb[2], t.threads,
                            t.field_smem, st));
    h->launches++;
    return SN_OK;
}

// Recompute replica r's running E and P from a full field pass.  A replica
// with a field cache whose dipoles changed outside the sweep (record = 0:
// initialisation, quench, field change) gets its cache rebuilt by the same
// pass; the periodic drift checks (record = 1) leave the cache alone.
sn_status recompute_one(sn_handle *h, int r, int prec, int record)
{
    double *red = h->d_red + 10 * r;
    SN_CK(h, cudaMemsetAsync(red, 0, 10 * sizeof(double), h->stream));
    SnFieldArgsHost a = field_args(h, r, nullptr, nullptr, h->d_red, 10);
    const bool gpass = h->tiles[r].cmode && !record && prec == SN_ENERGY_FP32;
    sn_status s = gpass ? launch_gfield_x(h, r, a, 0, h->tiles[r].nb[0], h->stream)
                        : launch_field(h, r, prec == SN_ENERGY_FP64, a);
    if (s) return s;
    SN_CK(h, sn_launch_recompute_finish(red, h->d_state, h->d_reps, r, h->params.cage_strain, h->d_drift, record,
                                        h->stream));
    h->launches++;
    return SN_OK;
}

// Issue one sweep's kernels on the handle's stream.  With events (2 per
// launch), each block-colour launch is bracketed for timing.
SnPhaseArgs phase_args(const sn_handle *h, int off, int cnt)
{
    SnPhaseArgs a;
    a.work = h->d_work + off;
    a.n_work = cnt;
    a.reps = h->d_reps;
    a.geoms = h->d_geoms;
    a.acc = h->d_acc;
    a.sweep = h->d_sweep;
    a.cage = (float)h->params.cage_strain;
    a.K = (float)h->params.K;
    a.constrain = h->params.constrain_to_x;
    a.dim = h->params.dim;
    a.err = h->d_err;
    a.tile_copy = h->tile_copy;
    return a;
}

cudaError_t issue_sweep(sn_handle *h, uint64_t *nodes, std::vector<cudaEvent_t> *events)
{
    cudaError_t e = cudaSuccess;
    size_t ev = 0;
    if (h->cached) {
        // the cached-field sweep takes its moves from a buffer drawn here
        e = sn_launch_sweep_proposals(h->d_reps, h->nrep, h->d_sweep, h->params.dim, h->params.constrain_to_x, h->nsm,
                                      h->stream);
        if (nodes) (*nodes)++;
        if (e != cudaSuccess) return e;
    }
    if (h->flow) {
        for (int v = 0; v < 2 && e == cudaSuccess; v++) {
            if (!h->flow_items[v]) continue;
            SnFlowArgs f;
            // the phase-ordered items of a variant are contiguous in d_work
            f.base = phase_args(h, h->flow_off[v], h->flow_items[v]);
            f.deps = h->d_deps + (size_t)h->flow_off[v] * SN_MAX_DEPS;
            f.done = h->d_done + h->flow_off[v];
            f.queue = h->d_queue + v;
            f.err = h->d_err;
            int thr = 0, smem = 0;
            for (int p = 0; p < 8; p++) {
                thr = std::max(thr, h->work_thr[p * 2 + v]);
                smem = std::max(smem, h->work_smem[p * 2 + v]);
            }
            if (events && ev + 1 < events->size()) e = cudaEventRecord((*events)[ev++], h->stream);
            if (e == cudaSuccess)
                e = k_flow[h->rc](v == 1, h->mixed, h->cached && v == 0, f, std::min(h->flow_grid[v], h->flow_items[v]),
                                  thr, smem, h->stream, nullptr);
            if (events && ev < events->size() && e == cudaSuccess) e = cudaEventRecord((*events)[ev++], h->stream);
            if (nodes) (*nodes)++;
        }
        if (e == cudaSuccess) {
            e = sn_launch_sweep_end(h->d_acc, h->d_state, h->d_hist, h->d_reps, h->nrep, h->d_sweep, h->d_ex,
                                    h->d_order, h->d_queue, h->stream);
            if (nodes) (*nodes)++;
        }
        return e;
    }
    for (int p = 0; p < 8 && e == cudaSuccess; p++)
        for (int v = 0; v < 2 && e == cudaSuccess; v++) {
            const int k = p * 2 + v;
            if (!h->work_cnt[k]) continue;
            const SnPhaseArgs a = phase_args(h, h->work_off[k], h->work_cnt[k]);
            if (events && ev + 1 < events->size()) e = cudaEventRecord((*events)[ev++], h->stream);
            if (e == cudaSuccess)
                e = k_sweep[h->rc](v == 1, h->mixed, h->cached && v == 0, a, h->work_cnt[k], h->work_thr[k],
                                   h->work_smem[k], h->stream);
            if (events && ev < events->size() && e == cudaSuccess) e = cudaEventRecord((*events)[ev++], h->stream);
            if (nodes) (*nodes)++;
        }
    if (e == cudaSuccess) {
        e = sn_launch_sweep_end(h->d_acc, h->d_state, h->d_hist, h->d_reps, h->nrep, h->d_sweep, h->d_ex, h->d_order,
                                nullptr, h->stream);
        if (nodes) (*nodes)++;
    }
    return e;
}

// Reads (and clears) the dataflow kernel's wait-timeout flag; the stream must be idle or is synchronised here.
sn_status flow_status(sn_handle *h)
{
    if (!h->d_err) return SN_OK;
    uint32_t err = 0;
    SN_CK(h, cudaMemcpyAsync(&err, h->d_err, sizeof(err), cudaMemcpyDeviceToHost, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    if (!err) return SN_OK;
    SN_CK(h, cudaMemsetAsync(h->d_err, 0, sizeof(err), h->stream));
    return fail(h, SN_ERR_TIMEOUT, "a sweep block waited too long for its neighbours (dataflow schedule)");
}

sn_status capture_graph(sn_handle *h)
{
    // configure function attributes (and size the dataflow grid) outside the capture
    for (int v = 0; v < 2; v++) {
        SN_CK(h, k_sweep[h->rc](v == 1, h->mixed, h->cached && v == 0, SnPhaseArgs{}, 0, 0, 0, h->stream));
        if (h->flow && h->flow_items[v]) {
            int thr = 0, smem = 0;
            for (int p = 0; p < 8; p++) {
                thr = std::max(thr, h->work_thr[p * 2 + v]);
                smem = std::max(smem, h->work_smem[p * 2 + v]);
            }
            SN_CK(h, k_flow[h->rc](v == 1, h->mixed, h->cached && v == 0, SnFlowArgs{}, 0, thr, smem, h->stream,
                                   &h->flow_grid[v]));
            if (h->flow_grid[v] < 1) return fail(h, SN_ERR_CUDA, "dataflow kernel cannot be resident");
        }
    }
    cudaGraph_t g;
    SN_CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    uint64_t nodes = 0;
    cudaError_t e = issue_sweep(h, &nodes, nullptr);
    cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
    if (e != cudaSuccess) return fail(h, SN_ERR_CUDA, "sweep capture: %s", cudaGetErrorString(e));
    if (e2 != cudaSuccess) return fail(h, SN_ERR_CUDA, "sweep capture end: %s", cudaGetErrorString(e2));
    e = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(h, SN_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    h->graph_nodes = nodes;
    return SN_OK;
}

void destroy_all(sn_handle *h)
{
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    for (float *p : h->lattice_mem) cudaFree(p);
    for (int *p : h->gcache_mem) cudaFree(p);
    for (float4 *p : h->prop_mem) cudaFree(p);
    void *ptrs[] = {h->d_reps,  h->d_geoms, h->d_acc,   h->d_state, h->d_sweep, h->d_hist, h->d_red,
                    h->d_drift, h->d_ex,    h->d_order, h->d_flags, h->d_work,  h->d_stage, h->d_site,
                    h->d_grad,  h->d_trace, h->d_deps,  h->d_done,  h->d_queue, h->d_err,
                    h->d_aoff,  h->d_abins};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (auto &e : h->slab_ev)
        if (e) cudaEventDestroy(e);
    for (auto &e : h->conv_ev)
        if (e) cudaEventDestroy(e);
    for (auto &e : h->fdone_ev)
        if (e) cudaEventDestroy(e);
    for (auto &f : h->field_stream)
        if (f) cudaStreamDestroy(f);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

}  // namespace

// ===========================================================================
extern "C" {

const char *sn_gpu_status_string(sn_status s)
{
    switch (s) {
    case SN_OK: return "ok";
    case SN_ERR_ARG: return "invalid argument";
    case SN_ERR_CONFIG: return "invalid configuration";
    case SN_ERR_SCHEDULE: return "no conflict-free schedule for this lattice";
    case SN_ERR_CUDA: return "CUDA error";
    case SN_ERR_NOMEM: return "out of memory";
    case SN_ERR_TIMEOUT: return "device wait timed out";
    case SN_ERR_UNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

const char *sn_gpu_last_error(const sn_handle *h)
{
    if (h && !h->err.empty()) return h->err.c_str();
    return g_last_error.c_str();
}

int sn_neighbour_count(int cutoff, int Z)
{
    if (cutoff < 0) return 0;
    int n = 0;
    const int zc = Z == 1 ? 0 : cutoff;
    for (int x = -cutoff; x <= cutoff; x++)
        for (int y = -cutoff; y <= cutoff; y++)
            for (int z = -zc; z <= zc; z++)
                if ((x || y || z) && x * x + y * y + z * z <= cutoff * cutoff) n++;
    return n;
}

sn_status sn_plan_schedule(int X, int Y, int Z, int cutoff, int mixed_lengths, sn_schedule_info *out)
{
    if (!out || X < 1 || Y < 1 || Z < 1) return fail(nullptr, SN_ERR_ARG, "bad lattice size or null output");
    SnTile t;
    std::string why;
    if (cutoff < 1 || cutoff > SN_MAX_CUTOFF)
        return fail(nullptr, SN_ERR_UNSUPPORTED, "cutoff %d outside 1..%d", cutoff, SN_MAX_CUTOFF);
    sn_params P{};
    P.cutoff = cutoff;
    sn_replica_desc d{};
    d.X = X;
    d.Y = Y;
    d.Z = Z;
    std::vector<SnTile> tiles;
    bool cached = false;
    if (!plan_table(P, 1, &d, mixed_lengths != 0, tiles, &cached, why))
        return fail(nullptr, SN_ERR_SCHEDULE, "%s", why.c_str());
    t = tiles[0];
    fill_info(t, cutoff, out);
    return SN_OK;
}

sn_status sn_check_flow(const sn_params *params, int n_replicas, const sn_replica_desc *replicas, uint64_t *stats)
{
    if (!params || !replicas || n_replicas < 1) return fail(nullptr, SN_ERR_ARG, "null argument or no replicas");
    const sn_params &P = *params;
    if (P.cutoff < 1 || P.cutoff > SN_MAX_CUTOFF)
        return fail(nullptr, SN_ERR_UNSUPPORTED, "cutoff %d outside 1..%d", P.cutoff, SN_MAX_CUTOFF);
    float L = 0.0f;
    bool mixed = false;
    for (int i = 0; i < P.n_species && i < SN_MAX_SPECIES; i++)
        if (P.dipoles[i] > 0.0f) {
            if (L == 0.0f) L = P.dipoles[i];
            else if (P.dipoles[i] != L) mixed = true;
        }
    std::vector<SnTile> tiles;
    std::string why;
    bool cached = false;
    if (!plan_table(P, n_replicas, replicas, mixed, tiles, &cached, why))
        return fail(nullptr, SN_ERR_SCHEDULE, "%s", why.c_str());
    SnPlan pl;
    if (!build_plan(tiles, replicas, n_replicas, true, pl, why)) return fail(nullptr, SN_ERR_SCHEDULE, "%s", why.c_str());
    // Independent check of the dataflow lists (direct block grids, not the key map):
    // every block once; dependencies earlier in the list, of the same replica, adjacent
    // (periodically) and of an earlier colour; every such neighbour present.
    uint64_t items = 0, ndeps = 0, maxd = 0;
    for (int v = 0; v < 2; v++) {
        std::vector<std::vector<int>> pos(n_replicas);
        for (int r = 0; r < n_replicas; r++)
            if ((replicas[r].Z == 1) == (v == 1)) pos[r].assign((size_t)tiles[r].nb[0] * tiles[r].nb[1] * tiles[r].nb[2], -1);
        auto cell = [&](int r, const int *c) -> int & {
            const SnTile &t = tiles[r];
            return pos[r][((size_t)c[0] * t.nb[1] + c[1]) * t.nb[2] + c[2]];
        };
        for (int i = 0; i < pl.flow_items[v]; i++) {
            const SnWork &w = pl.work[pl.flow_off[v] + i];
            const SnTile &t = tiles[w.rep];
            const int b[3] = {w.x0 / t.B[0], w.y0 / t.B[1], w.z0 / t.B[2]};
            if (pos[w.rep].empty() || cell(w.rep, b) != -1)
                return fail(nullptr, SN_ERR_SCHEDULE, "block listed twice or in the wrong variant");
            cell(w.rep, b) = i;
        }
        for (int r = 0; r < n_replicas; r++)
            for (int p : pos[r])
                if (p < 0) return fail(nullptr, SN_ERR_SCHEDULE, "replica %d: a block is missing", r);
        for (int i = 0; i < pl.flow_items[v]; i++) {
            const SnWork &w = pl.work[pl.flow_off[v] + i];
            const SnTile &t = tiles[w.rep];
            const int b[3] = {w.x0 / t.B[0], w.y0 / t.B[1], w.z0 / t.B[2]};
            const int own = block_colour(t, b);
            const int *dl = &pl.deps[(size_t)(pl.flow_off[v] + i) * SN_MAX_DEPS];
            std::vector<int> want;
            for (int dx = -1; dx <= 1; dx++)
                for (int dy = -1; dy <= 1; dy++)
                    for (int dz = -1; dz <= 1; dz++) {
                        const int c[3] = {(b[0] + dx + t.nb[0]) % t.nb[0], (b[1] + dy + t.nb[1]) % t.nb[1],
                                          (b[2] + dz + t.nb[2]) % t.nb[2]};
                        if ((c[0] == b[0] && c[1] == b[1] && c[2] == b[2]) || block_colour(t, c) > own) continue;
                        want.push_back(cell(w.rep, c));
                    }
            std::sort(want.begin(), want.end());
            want.erase(std::unique(want.begin(), want.end()), want.end());
            std::vector<int> got;
            got.reserve((size_t)dl[0]);
            for (int k = 1; k <= dl[0]; k++) got.push_back(dl[k]);
            std::sort(got.begin(), got.end());
            if (got != want) return fail(nullptr, SN_ERR_SCHEDULE, "item %d: dependency list differs", i);
            for (int j : got)
                if (j >= i) return fail(nullptr, SN_ERR_SCHEDULE, "item %d waits on a later item", i);
            ndeps += got.size();
            maxd = std::max<uint64_t>(maxd, got.size());
        }
        items += (uint64_t)pl.flow_items[v];
    }
    if (stats) {
        stats[0] = items;
        stats[1] = ndeps;
        stats[2] = maxd;
    }
    return SN_OK;
}

sn_status sn_plan_candidates(int X, int Y, int Z, int cutoff, int mixed_lengths, sn_schedule_info *out,
                             int max_out, int *n_out)
{
    if (!out || !n_out || max_out < 1 || X < 1 || Y < 1 || Z < 1)
        return fail(nullptr, SN_ERR_ARG, "bad lattice size, null output or max_out < 1");
    if (cutoff < 1 || cutoff > SN_MAX_CUTOFF)
        return fail(nullptr, SN_ERR_UNSUPPORTED, "cutoff %d outside 1..%d", cutoff, SN_MAX_CUTOFF);
    std::vector<SnTile> v;
    std::string why;
    *n_out = 0;
    // the default method's candidates: the cached-field sweep's where the lattice admits it
    sn_params P{};
    const bool try_cached = Z > 1 && sweep_method(P) != SN_SWEEP_STENCIL;
    if (!(try_cached && plan_tiles(X, Y, Z, cutoff, mixed_lengths != 0, v, (size_t)max_out, why, nullptr, true))) {
        v.clear();
        if (!plan_tiles(X, Y, Z, cutoff, mixed_lengths != 0, v, (size_t)max_out, why))
            return fail(nullptr, SN_ERR_SCHEDULE, "%s", why.c_str());
    }
    for (size_t i = 0; i < v.size(); i++) fill_info(v[i], cutoff, &out[i]);
    *n_out = (int)v.size();
    return SN_OK;
}

sn_status sn_gpu_autotune(const sn_params *params, const sn_replica_desc *replica, int max_candidates, int sweeps,
                          int block[3], double *ms_per_sweep)
{
    if (!params || !replica || !block || max_candidates < 1 || sweeps < 1)
        return fail(nullptr, SN_ERR_ARG, "null argument, max_candidates < 1 or sweeps < 1");
    bool mixed = false;
    float L = 0.0f;
    for (int i = 0; i < params->n_species && i < SN_MAX_SPECIES; i++) {
        const float d = params->dipoles[i];
        if (d > 0.0f) {
            if (L == 0.0f) L = d;
            else if (d != L) mixed = true;
        }
    }
    std::vector<sn_schedule_info> cands((size_t)max_candidates);
    int n = 0;
    sn_status s = sn_plan_candidates(replica->X, replica->Y, replica->Z, params->cutoff, mixed ? 1 : 0, cands.data(),
                                     max_candidates, &n);
    if (s) return s;
    double best = 0.0;
    int best_shape[3] = {0, 0, 0};
    for (int i = 0; i < n; i++) {
        sn_replica_desc d = *replica;
        d.block[0] = cands[i].bx;
        d.block[1] = cands[i].by;
        d.block[2] = cands[i].bz;
        sn_handle *h = nullptr;
        if ((s = sn_gpu_init(params, 1, &d, &h))) return s;
        double launch_ms = 0.0, ms = 0.0;
        int nl = 0;
        s = sn_gpu_init_lattice(h, 0, SN_LATTICE_RANDOM, 0);
        if (!s) s = sn_gpu_sweep(h, 2, nullptr, nullptr);  // warm-up
        if (!s) s = sn_gpu_phase_times(h, sweeps, &launch_ms, &ms, &nl);
        if (!s) s = flow_status(h);
        if (s) {
            const std::string msg = h->err;
            sn_gpu_destroy(h);
            return fail(nullptr, s, "block %dx%dx%d: %s", d.block[0], d.block[1], d.block[2], msg.c_str());
        }
        sn_gpu_destroy(h);
        if (i == 0 || ms < best) {
            best = ms;
            for (int k = 0; k < 3; k++) best_shape[k] = d.block[k];
        }
    }
    for (int k = 0; k < 3; k++) block[k] = best_shape[k];
    if (ms_per_sweep) *ms_per_sweep = best;
    return SN_OK;
}

int sn_check_schedule(int X, int Y, int Z, int cutoff, const sn_schedule_info *sc)
{
    if (!sc || X < 1 || Y < 1 || Z < 1 || cutoff < 1) return 0;
    const bool two_d = Z == 1;
    if (sc->bx * sc->nbx != X || sc->by * sc->nby != Y || sc->bz * sc->nbz != Z) return 0;
    if (sc->nbx % sc->mx || sc->nby % sc->my || sc->nbz % sc->mz) return 0;
    if (sc->merge && (two_d || sc->s % 2)) return 0;
    // key = (block colour, colour group); a group is one site colour, or the
    // pair c, c + (s/2,s/2,s/2) when merged
    auto key = [&](int x, int y, int z) {
        const int bx = x / sc->bx, by = y / sc->by, bz = z / sc->bz;
        int cx = (x % sc->bx) % sc->s, cy = (y % sc->by) % sc->s, cz = two_d ? 0 : (z % sc->bz) % sc->s;
        if (sc->merge && cx >= sc->s / 2) {
            cx -= sc->s / 2;
            cy = (cy + sc->s / 2) % sc->s;
            cz = (cz + sc->s / 2) % sc->s;
        }
        long long k = ((bx % sc->mx) * sc->my + (by % sc->my)) * (long long)sc->mz + (bz % sc->mz);
        k = ((k * sc->s + cx) * sc->s + cy) * sc->s + cz;
        return k;
    };
    const int zc = two_d ? 0 : cutoff;
    for (int x = 0; x < X; x++)
        for (int y = 0; y < Y; y++)
            for (int z = 0; z < Z; z++) {
                const long long k0 = key(x, y, z);
                for (int dx = -cutoff; dx <= cutoff; dx++)
                    for (int dy = -cutoff; dy <= cutoff; dy++)
                        for (int dz = -zc; dz <= zc; dz++) {
                            if (!(dx || dy || dz) || dx * dx + dy * dy + dz * dz > cutoff * cutoff) continue;
                            const int x2 = ((x + dx) % X + X) % X, y2 = ((y + dy) % Y + Y) % Y,
                                      z2 = ((z + dz) % Z + Z) % Z;
                            if (x2 == x && y2 == y && z2 == z) return 0;  // a site that sees its own image
                            if (key(x2, y2, z2) == k0) return 0;
                        }
            }
    return 1;
}

sn_status sn_gpu_init(const sn_params *params, int n_replicas, const sn_replica_desc *replicas, sn_handle **out)
{
    if (!params || !replicas || !out || n_replicas < 1) return fail(nullptr, SN_ERR_ARG, "null argument or no replicas");
    *out = nullptr;
    const sn_params &P = *params;
    if (P.cutoff < 1 || P.cutoff > SN_MAX_CUTOFF)
        return fail(nullptr, SN_ERR_UNSUPPORTED, "DipoleCutOff=%d: this build has tiled kernels for 1..%d", P.cutoff,
                    SN_MAX_CUTOFF);
    if (P.dim != 2 && P.dim != 3) return fail(nullptr, SN_ERR_CONFIG, "dim must be 2 or 3");
    if (P.n_species < 1 || P.n_species > SN_MAX_SPECIES)
        return fail(nullptr, SN_ERR_CONFIG, "n_species must be 1..%d", SN_MAX_SPECIES);
    float L = 0.0f;
    bool mixed = false;
    for (int i = 0; i < P.n_species; i++) {
        const float d = P.dipoles[i];
        if (!(d >= 0.0f) || std::isinf(d)) return fail(nullptr, SN_ERR_CONFIG, "Dipoles[%d] must be finite and >= 0", i);
        if (!(P.prevalence[i] >= 0.0f)) return fail(nullptr, SN_ERR_CONFIG, "Prevalence[%d] must be >= 0", i);
        if (d > 0.0f) {
            if (L == 0.0f) L = d;
            else if (d != L) mixed = true;
        }
    }
    for (int r = 0; r < n_replicas; r++) {
        const sn_replica_desc &d = replicas[r];
        if (d.X < 1 || d.Y < 1 || d.Z < 1 || d.X >= (1 << 15) || d.Y >= (1 << 15) || d.Z >= (1 << 15))
            return fail(nullptr, SN_ERR_ARG, "replica %d: bad size (each side 1 .. 32767)", r);
        if ((long long)d.X * d.Y * d.Z > 0x7fffffffLL)
            return fail(nullptr, SN_ERR_UNSUPPORTED, "replica %d: more than 2^31-1 sites", r);
        if (!(d.T > 0.0f)) return fail(nullptr, SN_ERR_ARG, "replica %d: temperature must be > 0", r);
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
        return fail(nullptr, SN_ERR_CUDA, "no CUDA device available");

    sn_handle *h = new sn_handle();
    h->params = P;
    h->nrep = n_replicas;
    h->mixed = mixed;
    h->length = L;
    h->dipole_ref = L;
    h->rc = P.cutoff;
    h->desc.assign(replicas, replicas + n_replicas);
    h->tiles.resize(n_replicas);
    h->reps.resize(n_replicas);
    h->work_off.assign(16, 0);
    h->work_cnt.assign(16, 0);
    h->work_smem.assign(16, 0);
    h->work_thr.assign(16, 0);
    h->fwork_off.assign(n_replicas, 0);
    h->fwork_cnt.assign(n_replicas, 0);

    auto bail = [&](sn_status s) {
        std::string msg = h->err;
        destroy_all(h);
        g_last_error = msg;
        return s;
    };
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->field_stream[0], cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->field_stream[1], cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(h, SN_ERR_CUDA, "cudaStreamCreate failed"));
    for (auto *evs : {&h->slab_ev[0], &h->conv_ev[0]})
        for (int k = 0; k < sn_handle::kSlabs; k++)
            if (cudaEventCreateWithFlags(&evs[k], cudaEventDisableTiming) != cudaSuccess)
                return bail(fail(h, SN_ERR_CUDA, "cudaEventCreate failed"));
    for (auto &e : h->fdone_ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
            return bail(fail(h, SN_ERR_CUDA, "cudaEventCreate failed"));

    {
        std::string why;
        if (!plan_table(P, n_replicas, replicas, mixed, h->tiles, &h->cached, why))
            return bail(fail(h, SN_ERR_SCHEDULE, "%s", why.c_str()));
    }
    float Lmax = 0.0f;
    for (int i = 0; i < P.n_species; i++) Lmax = std::max(Lmax, P.dipoles[i]);
    const int gk = h->cached ? cache_scale(P.cutoff, (double)Lmax, P.cage_strain) : 0;
    if (h->cached && gk < 8)
        return bail(fail(h, SN_ERR_CONFIG, "the cached-field sweep's fixed point has too few bits (k = %d) for "
                                           "Dipoles up to %g and CageStrain %g: use SN_SWEEP_STENCIL", gk,
                         (double)Lmax, P.cage_strain));
    for (int r = 0; r < n_replicas; r++) {
        const sn_replica_desc &d = replicas[r];
        const long long N = (long long)d.X * d.Y * d.Z;
        float *mem = nullptr;
        if (cudaMalloc(&mem, 4 * N * sizeof(float)) != cudaSuccess)
            return bail(fail(h, SN_ERR_NOMEM, "replica %d: cannot allocate %lld sites", r, N));
        h->lattice_mem.push_back(mem);
        if (cudaMemsetAsync(mem, 0, 4 * N * sizeof(float), h->stream) != cudaSuccess)
            return bail(fail(h, SN_ERR_CUDA, "cudaMemset failed"));
        SnReplicaDev &R = h->reps[r];
        memset(&R, 0, sizeof(R));
        R.px = mem;
        R.py = mem + N;
        R.pz = mem + 2 * N;
        R.len = mem + 3 * N;
        R.X = d.X;
        R.Y = d.Y;
        R.Z = d.Z;
        R.geom = r;
        R.n_sites = N;
        R.T = d.T;
        R.beta = (float)(300.0 / (double)d.T);
        for (int k = 0; k < 3; k++) R.E[k] = d.has_efield ? d.efield[k] : P.efield[k];
        R.length = L;
        const uint64_t seed = d.seed ? d.seed : P.seed + (uint64_t)r;
        R.seed_lo = (uint32_t)seed;
        R.seed_hi = (uint32_t)(seed >> 32);
        if (h->tiles[r].cmode) {
            int *gc = nullptr;
            if (cudaMalloc(&gc, 3 * (size_t)N * sizeof(int)) != cudaSuccess)
                return bail(fail(h, SN_ERR_NOMEM, "replica %d: cannot allocate the field cache of %lld sites", r, N));
            h->gcache_mem.push_back(gc);
            if (cudaMemsetAsync(gc, 0, 3 * (size_t)N * sizeof(int), h->stream) != cudaSuccess)
                return bail(fail(h, SN_ERR_CUDA, "cudaMemset failed"));
            R.gcache = gc;
            R.gscale = std::ldexp(1.0f, gk);
            R.ginv = std::ldexp(1.0f, -gk);
            float4 *pb = nullptr;
            if (cudaMalloc(&pb, (size_t)N * sizeof(float4)) != cudaSuccess)
                return bail(fail(h, SN_ERR_NOMEM, "replica %d: cannot allocate the proposal buffer of %lld sites", r, N));
            h->prop_mem.push_back(pb);
            R.prop = pb;
        }
    }

    if (const char *env = getenv("SN_SCHEDULE")) h->flow = strcmp(env, "phases") != 0;
    if (const char *env = getenv("SN_TILE_COPY")) h->tile_copy = strcmp(env, "bulk") == 0 ? 1 : 0;
    SnPlan plan;
    {
        std::string why;
        // blocks that must be ready at once to keep every CTA busy: ~1.5 per CTA slot at 2 CTAs per SM
        int dev = 0, nsm = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) !=
                                                      cudaSuccess)
            nsm = 0;
        h->nsm = nsm > 0 ? nsm : 1;
        if (!build_plan(h->tiles, replicas, n_replicas, h->flow, plan, why, nsm > 0 ? 3 * nsm : 512))
            return bail(fail(h, SN_ERR_SCHEDULE, "%s", why.c_str()));
    }
    for (int k = 0; k < 16; k++) {
        h->work_off[k] = plan.work_off[k];
        h->work_cnt[k] = plan.work_cnt[k];
        h->work_smem[k] = plan.work_smem[k];
        h->work_thr[k] = plan.work_thr[k];
    }
    h->fwork_off = plan.fwork_off;
    h->fwork_cnt = plan.fwork_cnt;
    for (int v = 0; v < 2; v++) {
        h->flow_off[v] = plan.flow_off[v];
        h->flow_items[v] = plan.flow_items[v];
    }
    const std::vector<SnWork> &work = plan.work;
    const std::vector<int> &deps = plan.deps;

    // temperature ladder for exchange: replicas sorted by T
    std::vector<int> order(n_replicas);
    for (int r = 0; r < n_replicas; r++) order[r] = r;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return replicas[a].T < replicas[b].T; });

    const size_t nr = (size_t)n_replicas;
#define ALLOC(ptr, bytes)                                                                         \
    if (cudaMalloc((void **)&(ptr), (bytes)) != cudaSuccess ||                                    \
        cudaMemsetAsync((void *)(ptr), 0, (bytes), h->stream) != cudaSuccess)                     \
        return bail(fail(h, SN_ERR_NOMEM, "device allocation of %zu bytes failed", (size_t)(bytes)));
    ALLOC(h->d_reps, nr * sizeof(SnReplicaDev));
    ALLOC(h->d_geoms, nr * sizeof(SnTile));
    ALLOC(h->d_acc, nr * sizeof(SnAccum));
    ALLOC(h->d_state, nr * sizeof(SnState));
    ALLOC(h->d_sweep, sizeof(uint32_t));
    ALLOC(h->d_hist, nr * SN_HIST_CAP * 2 * sizeof(double));
    ALLOC(h->d_red, nr * 10 * sizeof(double));
    ALLOC(h->d_drift, nr * sizeof(double));
    ALLOC(h->d_ex, sizeof(SnExchange));
    ALLOC(h->d_order, nr * sizeof(int));
    ALLOC(h->d_flags, 4 * sizeof(int));
    ALLOC(h->d_work, std::max<size_t>(work.size(), 1) * sizeof(SnWork));
    if (h->flow) {
        ALLOC(h->d_deps, deps.size() * sizeof(int));
        // one spare flag past the last item: never published (sn_gpu_test_stall_block)
        ALLOC(h->d_done, (work.size() + 1) * sizeof(uint32_t));
        h->done_n = work.size();
        ALLOC(h->d_queue, 2 * sizeof(uint32_t));
    }
    ALLOC(h->d_err, 4 * sizeof(uint32_t));
#undef ALLOC
    SnExchange ex;
    memset(&ex, 0, sizeof(ex));
    ex.seed_lo = (uint32_t)(P.seed ^ 0x5A5A5A5Aull);
    ex.seed_hi = (uint32_t)((P.seed >> 32) ^ 0xA5A5A5A5ull);
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->d_reps, h->reps.data(), nr * sizeof(SnReplicaDev), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->d_geoms, h->tiles.data(), nr * sizeof(SnTile), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->d_work, work.data(), work.size() * sizeof(SnWork), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->d_order, order.data(), nr * sizeof(int), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess && h->flow)
        e = cudaMemcpyAsync(h->d_deps, deps.data(), deps.size() * sizeof(int), cudaMemcpyHostToDevice, h->stream);
    const uint32_t wait_limit = SN_WAIT_LIMIT_DEFAULT;
    if (e == cudaSuccess && h->flow)
        e = cudaMemcpyAsync(h->d_err + 3, &wait_limit, sizeof(wait_limit), cudaMemcpyHostToDevice, h->stream);
    if (h->flow) h->deps_host = deps;
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->d_ex, &ex, sizeof(ex), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return bail(fail(h, SN_ERR_CUDA, "init upload: %s", cudaGetErrorString(e)));
    sn_status s = capture_graph(h);
    if (s) return bail(s);
    *out = h;
    return SN_OK;
}

sn_status sn_gpu_destroy(sn_handle *h)
{
    if (!h) return fail(nullptr, SN_ERR_ARG, "null handle");
    destroy_all(h);
    return SN_OK;
}

sn_status sn_gpu_init_lattice(sn_handle *h, int replica, int pattern, uint64_t seed)
{
    sn_status s = check_rep(h, replica);
    if (s) return s;
    if (pattern != SN_LATTICE_RANDOM && pattern != SN_LATTICE_FERROELECTRIC)
        return fail(h, SN_ERR_ARG, "unknown lattice pattern %d", pattern);
    const SnReplicaDev &R = h->reps[replica];
    SnInitArgs a;
    memset(&a, 0, sizeof(a));
    a.px = R.px;
    a.py = R.py;
    a.pz = R.pz;
    a.len = R.len;
    a.n = R.n_sites;
    a.pattern = pattern;
    a.dim = h->params.dim;
    a.n_species = h->params.n_species;
    for (int i = 0; i < h->params.n_species; i++) {
        a.dipoles[i] = h->params.dipoles[i];
        a.prevalence[i] = h->params.prevalence[i];
    }
    if (!seed) seed = ((uint64_t)R.seed_hi << 32) | R.seed_lo;
    a.seed_lo = (uint32_t)seed;
    a.seed_hi = (uint32_t)(seed >> 32);
    SN_CK(h, sn_launch_init_lattice(a, h->stream));
    h->launches++;
    s = recompute_one(h, replica, SN_ENERGY_FP32, 0);
    if (s) return s;
    SN_CK(h, cudaStreamSynchronize(h->stream));
    return SN_OK;
}

sn_status sn_gpu_upload_lattice(sn_handle *h, int replica, const float *xyz, const float *len)
{
    sn_status s = check_rep(h, replica);
    if (s) return s;
    if (!xyz) return fail(h, SN_ERR_ARG, "null xyz buffer");
    const SnReplicaDev &R = h->reps[replica];
    const SnTile &t = h->tiles[replica];
    const size_t N = (size_t)R.n_sites;
    s = ensure(h, (void **)&h->d_stage, &h->stage_floats, 4 * N, sizeof(float));
    if (s) return s;
    // The copy runs in x slabs (whole block rows) on the copy stream; each slab
    // is converted as soon as it lands, and the energy pass of the running
    // total starts on every block whose tile (block + halo) has fully arrived,
    // so the transfer and the recompute overlap.  Those energy chunks
    // alternate between two streams (a chunk reads only converted slabs, and
    // the conversions write slabs no running chunk reads).  Blocks whose halo
    // wraps past x = 0 or X go last.
    const int nb = t.nb[0], Bx = t.B[0], H = h->rc;
    const int Q = std::max(1, std::min(sn_handle::kSlabs, nb));
    const size_t row = (size_t)R.Y * R.Z;
    double *red = h->d_red + 10 * replica;
    SN_CK(h, cudaMemsetAsync(h->d_flags, 0, 4 * sizeof(int), h->stream));
    SN_CK(h, cudaMemsetAsync(red, 0, 10 * sizeof(double), h->stream));
    SN_CK(h, cudaEventRecord(h->slab_ev[0], h->stream));  // the copies must not overtake earlier work
    SN_CK(h, cudaStreamWaitEvent(h->copy_stream, h->slab_ev[0], 0));
    const SnFieldArgsHost fa = field_args(h, replica, nullptr, nullptr, h->d_red, 10);
    int next_b = 1;  // block 0's tile wraps to the end of the lattice
    for (int q = 0; q < Q; q++) {
        const int x0 = (int)((long long)nb * q / Q) * Bx, x1 = (int)((long long)nb * (q + 1) / Q) * Bx;
        const size_t a0 = (size_t)x0 * row, cnt = (size_t)(x1 - x0) * row;
        SN_CK(h, cudaMemcpyAsync(h->d_stage + 3 * a0, xyz + 3 * a0, 3 * cnt * sizeof(float), cudaMemcpyHostToDevice,
                                 h->copy_stream));
        if (len)
            SN_CK(h, cudaMemcpyAsync(h->d_stage + 3 * N + a0, len + a0, cnt * sizeof(float), cudaMemcpyHostToDevice,
                                     h->copy_stream));
        SN_CK(h, cudaEventRecord(h->slab_ev[q], h->copy_stream));
        SN_CK(h, cudaStreamWaitEvent(h->stream, h->slab_ev[q], 0));
        SN_CK(h, sn_launch_upload_convert(h->d_stage + 3 * a0, len ? h->d_stage + 3 * N + a0 : nullptr, R.px + a0,
                                          R.py + a0, R.pz + a0, R.len + a0, (long long)cnt, h->length,
                                          h->mixed ? 1 : 0, h->params.dipoles[0], h->d_flags, h->stream));
        h->launches++;
        SN_CK(h, cudaEventRecord(h->conv_ev[q], h->stream));
        cudaStream_t fs = h->field_stream[SN_UPLOAD_FIELD_STREAMS > 1 ? (q & 1) : 0];
        SN_CK(h, cudaStreamWaitEvent(fs, h->conv_ev[q], 0));
        // blocks whose tile x range [b*Bx - H, (b+1)*Bx + H) lies in [0, x1)
        int last = (x1 - H) / Bx - 1;
        if (q == Q - 1) last = nb - 1;
        if ((s = t.cmode ? launch_gfield_x(h, replica, fa, next_b, last + 1, fs)
                         : launch_field_x(h, replica, fa, next_b, last + 1, fs)))
            return s;
        next_b = std::max(next_b, last + 1);
    }
    for (int k = 0; k < 2; k++) {
        SN_CK(h, cudaEventRecord(h->fdone_ev[k], h->field_stream[k]));
        SN_CK(h, cudaStreamWaitEvent(h->stream, h->fdone_ev[k], 0));
    }
    if ((s = t.cmode ? launch_gfield_x(h, replica, fa, 0, 1, h->stream) : launch_field_x(h, replica, fa, 0, 1, h->stream)))
        return s;
    SN_CK(h, sn_launch_recompute_finish(red, h->d_state, h->d_reps, replica, h->params.cage_strain, h->d_drift, 0,
                                        h->stream));
    h->launches++;
    int flags[4] = {0, 0, 0, 0};
    SN_CK(h, cudaMemcpyAsync(flags, h->d_flags, sizeof(flags), cudaMemcpyDeviceToHost, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    if (flags[2]) return fail(h, SN_ERR_ARG, "negative or non-finite dipole length in upload");
    if (flags[3] && t.cmode)
        return fail(h, SN_ERR_ARG, "upload has a dipole component beyond +-1; the cached-field sweep (SN_SWEEP_CACHED, "
                                   "the default where it applies) needs unit or shorter dipoles: use SN_SWEEP_STENCIL");
    if (flags[0])
        return fail(h, SN_ERR_ARG, "upload has a dipole length other than %g, but the handle was created for a single "
                                   "species length (list every species in sn_params.dipoles)", (double)h->length);
    return SN_OK;
}

sn_status sn_gpu_download_lattice(sn_handle *h, int replica, float *xyz, float *len)
{
    sn_status s = check_rep(h, replica);
    if (s) return s;
    if (!xyz && !len) return fail(h, SN_ERR_ARG, "null output buffers");
    const SnReplicaDev &R = h->reps[replica];
    const size_t N = (size_t)R.n_sites;
    s = ensure(h, (void **)&h->d_stage, &h->stage_floats, 4 * N, sizeof(float));
    if (s) return s;
    SN_CK(h, sn_launch_download_convert(R.px, R.py, R.pz, R.len, h->d_stage, h->d_stage + 3 * N, (long long)N,
                                        h->stream));
    h->launches++;
    if (xyz) SN_CK(h, cudaMemcpyAsync(xyz, h->d_stage, 3 * N * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    if (len) SN_CK(h, cudaMemcpyAsync(len, h->d_stage + 3 * N, N * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    return flow_status(h);
}

namespace {

// Address under which kernels may write a caller's buffer of n floats:
// pinned or registered host memory (mapped) or this device's memory, checked
// at both ends; nullptr for anything else (pageable memory goes through the
// staged download).
float *device_view(float *p, size_t n)
{
    int dev = -1;
    if (!p || n == 0 || cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    cudaPointerAttributes a0, a1;
    if (cudaPointerGetAttributes(&a0, p) != cudaSuccess || cudaPointerGetAttributes(&a1, p + (n - 1)) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    const bool host = a0.type == cudaMemoryTypeHost && a1.type == cudaMemoryTypeHost;
    const bool devm = a0.type == cudaMemoryTypeDevice && a1.type == cudaMemoryTypeDevice && a0.device == dev &&
                      a1.device == dev;
    if (!(host || devm) || !a0.devicePointer || !a1.devicePointer) return nullptr;
    float *d0 = static_cast<float *>(a0.devicePointer), *d1 = static_cast<float *>(a1.devicePointer);
    return d1 == d0 + (n - 1) ? d0 : nullptr;
}

// n sweeps; outs (nrep entries, nullable) are device views that the last
// sweep writes its final sites to.  Every pointer set here is cleared again
// before returning, also on failure.
sn_status run_sweeps(sn_handle *h, int n_sweeps, float *const *outs, uint64_t *accept, uint64_t *reject,
                     cudaEvent_t ev_begin = nullptr, cudaEvent_t ev_end = nullptr)
{
    std::vector<SnState> before;
    if (accept || reject) {
        before.resize(h->nrep);
        SN_CK(h, cudaMemcpyAsync(before.data(), h->d_state, h->nrep * sizeof(SnState), cudaMemcpyDeviceToHost,
                                 h->stream));
    }
    bool armed = false;
    auto disarm = [&]() {
        for (int r = 0; outs && armed && r < h->nrep; r++)
            if (outs[r]) sn_launch_set_out(h->d_reps, r, nullptr, h->stream);
        armed = false;
    };
    if (ev_begin) SN_CK(h, cudaEventRecord(ev_begin, h->stream));
    for (int i = 0; i < n_sweeps; i++) {
        if (outs && i == n_sweeps - 1) {
            armed = true;
            for (int r = 0; r < h->nrep; r++) {
                if (!outs[r]) continue;
                const cudaError_t e = sn_launch_set_out(h->d_reps, r, outs[r], h->stream);
                if (e != cudaSuccess) {
                    disarm();
                    return fail(h, SN_ERR_CUDA, "%s", cudaGetErrorString(e));
                }
                h->launches++;
            }
        }
        const cudaError_t e = cudaGraphLaunch(h->graph, h->stream);
        if (e != cudaSuccess) {
            disarm();
            return fail(h, SN_ERR_CUDA, "%s", cudaGetErrorString(e));
        }
        if (armed) {
            for (int r = 0; r < h->nrep; r++)
                if (outs[r]) h->launches++;
            disarm();
        }
        h->launches += h->graph_nodes;
        h->sweeps++;
        if (h->recompute_every > 0 && h->sweeps % (uint64_t)h->recompute_every == 0) {
            // a drift check of a lattice whose sweep gave up a wait would be meaningless
            sn_status s = flow_status(h);
            if (s) return s;
            for (int r = 0; r < h->nrep; r++) {
                sn_status s = recompute_one(h, r, h->recompute_prec, 1);
                if (s) return s;
            }
            h->n_checks++;
        }
    }
    if (ev_end) SN_CK(h, cudaEventRecord(ev_end, h->stream));
    if (accept || reject) {
        std::vector<SnState> after(h->nrep);
        SN_CK(h, cudaMemcpyAsync(after.data(), h->d_state, h->nrep * sizeof(SnState), cudaMemcpyDeviceToHost, h->stream));
        SN_CK(h, cudaStreamSynchronize(h->stream));
        uint64_t a = 0, t = 0;
        for (int r = 0; r < h->nrep; r++) {
            a += after[r].acc_total - before[r].acc_total;
            t += after[r].att_total - before[r].att_total;
        }
        if (accept) *accept = a;
        if (reject) *reject = t - a;
    }
    // every call reports its own sweeps' waits (this synchronises the stream)
    sn_status s = flow_status(h);
    if (s) return s;
    SN_CK(h, cudaGetLastError());
    return SN_OK;
}

}  // namespace

sn_status sn_gpu_sweep(sn_handle *h, int n_sweeps, uint64_t *accept, uint64_t *reject)
{
    if (!h) return fail(nullptr, SN_ERR_ARG, "null handle");
    if (n_sweeps < 0) return fail(h, SN_ERR_ARG, "negative sweep count");
    return run_sweeps(h, n_sweeps, nullptr, accept, reject);
}

sn_status sn_gpu_sweep_timed(sn_handle *h, int n_sweeps, double *ms)
{
    if (!h || !ms) return fail(h, SN_ERR_ARG, "null handle or output");
    if (n_sweeps < 1) return fail(h, SN_ERR_ARG, "need n_sweeps >= 1");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    SN_CK(h, cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fail(h, SN_ERR_CUDA, "cudaEventCreate failed");
    }
    sn_status s = run_sweeps(h, n_sweeps, nullptr, nullptr, nullptr, e0, e1);
    float t = 0.0f;
    if (!s && cudaEventElapsedTime(&t, e0, e1) != cudaSuccess) s = fail(h, SN_ERR_CUDA, "cudaEventElapsedTime failed");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!s) *ms = t;
    return s;
}

sn_status sn_gpu_set_wait_limit(sn_handle *h, uint32_t polls)
{
    if (!h) return fail(nullptr, SN_ERR_ARG, "null handle");
    if (polls < 1) return fail(h, SN_ERR_ARG, "the poll limit must be >= 1");
    if (!h->flow) return SN_OK;  // the eight-launch schedule never waits
    SN_CK(h, cudaMemcpyAsync(h->d_err + 3, &polls, sizeof(polls), cudaMemcpyHostToDevice, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    return SN_OK;
}

sn_status sn_gpu_field_cache_check(sn_handle *h, int replica, uint64_t *mismatches)
{
    sn_status s = check_rep(h, replica);
    if (s) return s;
    if (!mismatches) return fail(h, SN_ERR_ARG, "null output");
    const SnReplicaDev &R = h->reps[replica];
    if (!R.gcache) return fail(h, SN_ERR_UNSUPPORTED, "replica %d has no field cache (stencil sweep)", replica);
    const size_t n3 = 3 * (size_t)R.n_sites;
    // the cache as the sweeps left it, then a fresh field-cache pass over it, then compare
    s = ensure(h, (void **)&h->d_site, &h->site_n, (n3 + 1) / 2 + 1, sizeof(double));
    if (s) return s;
    int *old = reinterpret_cast<int *>(h->d_site);
    unsigned long long *cnt = reinterpret_cast<unsigned long long *>(h->d_site + (n3 + 1) / 2);
    SN_CK(h, cudaMemcpyAsync(old, R.gcache, n3 * sizeof(int), cudaMemcpyDeviceToDevice, h->stream));
    SN_CK(h, cudaMemsetAsync(cnt, 0, sizeof(*cnt), h->stream));
    SnFieldArgsHost a = field_args(h, replica, nullptr, nullptr, nullptr, 0);
    if ((s = launch_gfield_x(h, replica, a, 0, h->tiles[replica].nb[0], h->stream))) return s;
    SN_CK(h, sn_launch_count_diff(old, R.gcache, (long long)n3, cnt, h->stream));
    h->launches++;
    unsigned long long c = 0;
    SN_CK(h, cudaMemcpyAsync(&c, cnt, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    *mismatches = c;
    return SN_OK;
}

sn_status sn_gpu_test_stall_block(sn_handle *h, int item)
{
    if (!h) return fail(nullptr, SN_ERR_ARG, "null handle");
    if (!h->flow) return fail(h, SN_ERR_UNSUPPORTED, "the eight-launch schedule has no dependency waits");
    const int n3d = h->flow_items[0];
    if (item < -1 || item >= n3d) return fail(h, SN_ERR_ARG, "item %d outside the 3D dataflow list [0,%d)", item, n3d);
    auto put = [&](int k, const int *v) -> sn_status {
        SN_CK(h, cudaMemcpyAsync(h->d_deps + (size_t)(h->flow_off[0] + k) * SN_MAX_DEPS, v, SN_MAX_DEPS * sizeof(int),
                                 cudaMemcpyHostToDevice, h->stream));
        SN_CK(h, cudaStreamSynchronize(h->stream));
        return SN_OK;
    };
    sn_status s = SN_OK;
    if (h->stalled_item >= 0) {  // restore the planned list
        if ((s = put(h->stalled_item, &h->deps_host[(size_t)(h->flow_off[0] + h->stalled_item) * SN_MAX_DEPS])))
            return s;
        h->stalled_item = -1;
    }
    if (item < 0) return SN_OK;
    int dl[SN_MAX_DEPS];
    memcpy(dl, &h->deps_host[(size_t)(h->flow_off[0] + item) * SN_MAX_DEPS], sizeof(dl));
    // the spare flag sits past the last work entry; items index done[] from the variant's offset
    dl[1] = (int)h->done_n - h->flow_off[0];
    if (dl[0] < 1) dl[0] = 1;
    if ((s = put(item, dl))) return s;
    h->stalled_item = item;
    return SN_OK;
}

void *sn_gpu_host_alloc(size_t bytes)
{
    void *p = nullptr;
    if (bytes == 0 || cudaMallocHost(&p, bytes) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void sn_gpu_host_free(void *p)
{
    if (p) cudaFreeHost(p);
}

sn_status sn_gpu_sweep_download(sn_handle *h, int n_sweeps, float *const *xyz, uint64_t *accept, uint64_t *reject)
{
    if (!h) return fail(nullptr, SN_ERR_ARG, "null handle");
    if (n_sweeps < 0) return fail(h, SN_ERR_ARG, "negative sweep count");
    if (!xyz) return fail(h, SN_ERR_ARG, "null buffer table");
    std::vector<float *> outs(h->nrep, nullptr);
    bool any = false;
    for (int r = 0; r < h->nrep; r++) {
        if (!xyz[r]) continue;
        outs[r] = device_view(xyz[r], 3 * (size_t)h->reps[r].n_sites);
        any |= outs[r] != nullptr;
    }
    sn_status s = run_sweeps(h, n_sweeps, (any && n_sweeps > 0) ? outs.data() : nullptr, accept, reject);
    if (s) return s;
    SN_CK(h, cudaStreamSynchronize(h->stream));
    if ((s = flow_status(h))) return s;
    for (int r = 0; r < h->nrep; r++)  // buffers the kernels cannot write (or no sweep ran)
        if (xyz[r] && (!outs[r] || n_sweeps == 0) && (s = sn_gpu_download_lattice(h, r, xyz[r], nullptr))) return s;
    return SN_OK;
}

sn_status sn_gpu_sweep_count(const sn_handle *h, uint64_t *sweeps)
{
    if (!h || !sweeps) return fail(nullptr, SN_ERR_ARG, "null argument");
    *sweeps = h->sweeps;
    return SN_OK;
}

sn_status sn_gpu_set_sweep_count(sn_handle *h, uint64_t sweeps)
{
    if (!h) return fail(nullptr, SN_ERR_ARG, "null handle");
    const uint32_t s32 = (uint32_t)sweeps;  // the device counter keys the random stream modulo 2^32
    SN_CK(h, cudaMemcpyAsync(h->d_sweep, &s32, sizeof(s32), cudaMemcpyHostToDevice, h->stream));
    // the dataflow done flags hold epochs of the old counter
    if (h->d_done) SN_CK(h, cudaMemsetAsync(h->d_done, 0, h->done_n * sizeof(uint32_t), h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    h->sweeps = sweeps;
    return SN_OK;
}

sn_status sn_gpu_energy(sn_handle *h, int replica, int precision, double *E_total, double *site_E)
{
    sn_status s = check_rep(h, replica);
    if (s) return s;
    const size_t N = (size_t)h->reps[replica].n_sites;
    if (site_E) {
        s = ensure(h, (void **)&h->d_site, &h->site_n, N, sizeof(double));
        if (s) return s;
    }
    double *red = h->d_red + 10 * replica;
    SN_CK(h, cudaMemsetAsync(red, 0, 10 * sizeof(double), h->stream));
    SnFieldArgsHost a = field_args(h, replica, site_E ? h->d_site : nullptr, nullptr, h->d_red, 10);
    s = launch_field(h, replica, precision == SN_ENERGY_FP64, a);
    if (s) return s;
    double hr[10];
    SN_CK(h, cudaMemcpyAsync(hr, red, sizeof(hr), cudaMemcpyDeviceToHost, h->stream));
    if (site_E) SN_CK(h, cudaMemcpyAsync(site_E, h->d_site, N * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    if (E_total) *E_total = hr[0] - 0.5 * (double)h->params.cage_strain * hr[1] + hr[2] + hr[3];
    return SN_OK;
}

sn_status sn_gpu_observables(sn_handle *h, double *E_per_site, double *P_abs, double *P_vec)
{
    if (!h) return fail(nullptr, SN_ERR_ARG, "null handle");
    std::vector<SnState> st(h->nrep);
    SN_CK(h, cudaMemcpyAsync(st.data(), h->d_state, h->nrep * sizeof(SnState), cudaMemcpyDeviceToHost, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    sn_status fs = flow_status(h);
    if (fs) return fs;
    for (int r = 0; r < h->nrep; r++) {
        const double N = (double)h->reps[r].n_sites;
        if (E_per_site) E_per_site[r] = st[r].E / N;
        if (P_abs) P_abs[r] = std::sqrt(st[r].P[0] * st[r].P[0] + st[r].P[1] * st[r].P[1] + st[r].P[2] * st[r].P[2]) / N;
        if (P_vec)
            for (int k = 0; k < 3; k++) P_vec[3 * r + k] = st[r].P[k];
    }
    return SN_OK;
}

sn_status sn_gpu_history(sn_handle *h, int replica, int max, double *E_per_site, double *P_abs, int *n_out)
{
    sn_status s = check_rep(h, replica);
    if (s) return s;
    if (max < 0 || !n_out) return fail(h, SN_ERR_ARG, "bad history buffer");
    SnState st;
    SN_CK(h, cudaMemcpyAsync(&st, h->d_state + replica, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
    std::vector<double> ring((size_t)SN_HIST_CAP * 2);
    SN_CK(h, cudaMemcpyAsync(ring.data(), h->d_hist + (size_t)replica * SN_HIST_CAP * 2, ring.size() * sizeof(double),
                             cudaMemcpyDeviceToHost, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    const int have = std::min(st.hist_head, SN_HIST_CAP);
    const int n = std::min(have, max);
    const int first = st.hist_head - n;
    for (int i = 0; i < n; i++) {
        const int k = (first + i) % SN_HIST_CAP;
        if (E_per_site) E_per_site[i] = ring[2 * k];
        if (P_abs) P_abs[i] = ring[2 * k + 1];
    }
    *n_out = n;
    const int zero = 0;
    SN_CK(h, cudaMemcpyAsync(&h->d_state[replica].hist_head, &zero, sizeof(int), cudaMemcpyHostToDevice, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    return SN_OK;
}

sn_status sn_gpu_recompute(sn_handle *h, int precision, double *max_rel_drift)
{
    if (!h) return fail(nullptr, SN_ERR_ARG, "null handle");
    SN_CK(h, cudaMemsetAsync(h->d_drift, 0, h->nrep * sizeof(double), h->stream));
    for (int r = 0; r < h->nrep; r++) {
        sn_status s = recompute_one(h, r, precision, 1);
        if (s) return s;
    }
    std::vector<double> d(h->nrep);
    SN_CK(h, cudaMemcpyAsync(d.data(), h->d_drift, h->nrep * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    if (max_rel_drift) *max_rel_drift = d.empty() ? 0.0 : *std::max_element(d.begin(), d.end());
    SN_CK(h, cudaMemsetAsync(h->d_drift, 0, h->nrep * sizeof(double), h->stream));
    return SN_OK;
}

sn_status sn_gpu_set_recompute(sn_handle *h, int every, int precision)
{
    if (!h) return fail(nullptr, SN_ERR_ARG, "null handle");
    if (every < 0) return fail(h, SN_ERR_ARG, "negative interval");
    h->recompute_every = every;
    h->recompute_prec = precision;
    return SN_OK;
}

sn_status sn_gpu_drift(const sn_handle *h, double *max_rel_drift, int *n_checks)
{
    if (!h) return fail(nullptr, SN_ERR_ARG, "null handle");
    std::vector<double> d(h->nrep);
    cudaError_t e = cudaMemcpyAsync(d.data(), h->d_drift, h->nrep * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return fail(const_cast<sn_handle *>(h), SN_ERR_CUDA, "drift read: %s", cudaGetErrorString(e));
    if (max_rel_drift) *max_rel_drift = *std::max_element(d.begin(), d.end());
    if (n_checks) *n_checks = h->n_checks;
    return SN_OK;
}

sn_status sn_gpu_set_field(sn_handle *h, int replica, const float efield[3])
{
    sn_status s = check_rep(h, replica);
    if (s) return s;
    if (!efield) return fail(h, SN_ERR_ARG, "null field");
    for (int k = 0; k < 3; k++) h->reps[replica].E[k] = efield[k];
    SN_CK(h, cudaMemcpyAsync(&h->d_reps[replica].E, h->reps[replica].E, 3 * sizeof(float), cudaMemcpyHostToDevice,
                             h->stream));
    // the field term changes the running energy: restart it from a recompute
    s = recompute_one(h, replica, SN_ENERGY_FP32, 0);
    if (s) return s;
    SN_CK(h, cudaStreamSynchronize(h->stream));
    return SN_OK;
}

sn_status sn_gpu_set_temperature(sn_handle *h, int replica, float T)
{
    sn_status s = check_rep(h, replica);
    if (s) return s;
    if (!(T > 0.0f)) return fail(h, SN_ERR_ARG, "temperature must be > 0");
    SnReplicaDev cur;
    SN_CK(h, cudaMemcpyAsync(&cur, h->d_reps + replica, sizeof(cur), cudaMemcpyDeviceToHost, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    cur.T = T;
    cur.beta = (float)(300.0 / (double)T);
    h->reps[replica].T = cur.T;
    h->reps[replica].beta = cur.beta;
    SN_CK(h, cudaMemcpyAsync(h->d_reps + replica, &cur, sizeof(cur), cudaMemcpyHostToDevice, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    return SN_OK;
}

sn_status sn_gpu_get_temperature(const sn_handle *h, int replica, float *T)
{
    if (!h || !T) return fail(nullptr, SN_ERR_ARG, "null argument");
    if (replica < 0 || replica >= h->nrep) return fail(const_cast<sn_handle *>(h), SN_ERR_ARG, "replica out of range");
    SnReplicaDev cur;
    cudaError_t e = cudaMemcpyAsync(&cur, h->d_reps + replica, sizeof(cur), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return fail(const_cast<sn_handle *>(h), SN_ERR_CUDA, "%s", cudaGetErrorString(e));
    *T = cur.T;
    return SN_OK;
}

sn_status sn_gpu_set_exchange(sn_handle *h, int every)
{
    if (!h) return fail(nullptr, SN_ERR_ARG, "null handle");
    if (every < 0) return fail(h, SN_ERR_ARG, "negative interval");
    h->exchange_every = every;
    SN_CK(h, cudaMemcpyAsync(&h->d_ex->every, &h->exchange_every, sizeof(int), cudaMemcpyHostToDevice, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    return SN_OK;
}

sn_status sn_gpu_exchange_stats(sn_handle *h, uint64_t *attempted, uint64_t *accepted)
{
    if (!h) return fail(nullptr, SN_ERR_ARG, "null handle");
    SnExchange ex;
    SN_CK(h, cudaMemcpyAsync(&ex, h->d_ex, sizeof(ex), cudaMemcpyDeviceToHost, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    if (attempted) *attempted = ex.attempted;
    if (accepted) *accepted = ex.accepted;
    return SN_OK;
}

sn_status sn_gpu_adjoint(sn_handle *h, int replica, float *dE_dp, double *dE_dparams, double *E_total)
{
    sn_status s = check_rep(h, replica);
    if (s) return s;
    const size_t N = (size_t)h->reps[replica].n_sites;
    if (dE_dp) {
        s = ensure(h, (void **)&h->d_grad, &h->grad_n, 3 * N, sizeof(float));
        if (s) return s;
    }
    double *red = h->d_red + 10 * replica;
    SN_CK(h, cudaMemsetAsync(red, 0, 10 * sizeof(double), h->stream));
    SnFieldArgsHost a = field_args(h, replica, nullptr, dE_dp ? h->d_grad : nullptr, h->d_red, 10);
    s = launch_field(h, replica, false, a);
    if (s) return s;
    double hr[10];
    SN_CK(h, cudaMemcpyAsync(hr, red, sizeof(hr), cudaMemcpyDeviceToHost, h->stream));
    if (dE_dp) SN_CK(h, cudaMemcpyAsync(dE_dp, h->d_grad, 3 * N * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    if (dE_dparams) {
        dE_dparams[0] = h->dipole_ref != 0.0f ? 2.0 * hr[0] / (double)h->dipole_ref : 0.0;
        dE_dparams[1] = -0.5 * hr[1];
        dE_dparams[2] = hr[7];
        dE_dparams[3] = hr[8];
        dE_dparams[4] = hr[9];
    }
    if (E_total) *E_total = hr[0] - 0.5 * (double)h->params.cage_strain * hr[1] + hr[2] + hr[3];
    return SN_OK;
}

sn_status sn_gpu_quench(sn_handle *h, int replica, int n_steps, float step, double *E_trace)
{
    sn_status s = check_rep(h, replica);
    if (s) return s;
    if (n_steps < 0 || !(step > 0.0f)) return fail(h, SN_ERR_ARG, "need n_steps >= 0 and step > 0");
    const SnReplicaDev &R = h->reps[replica];
    const size_t N = (size_t)R.n_sites;
    s = ensure(h, (void **)&h->d_grad, &h->grad_n, 3 * N, sizeof(float));
    if (s) return s;
    s = ensure(h, (void **)&h->d_trace, &h->trace_n, 10 * (size_t)(n_steps + 1), sizeof(double));
    if (s) return s;
    SN_CK(h, cudaMemsetAsync(h->d_trace, 0, 10 * (size_t)(n_steps + 1) * sizeof(double), h->stream));
    for (int k = 0; k <= n_steps; k++) {
        SnFieldArgsHost a = field_args(h, replica, nullptr, k < n_steps ? h->d_grad : nullptr, h->d_trace + 10 * k, 0);
        s = launch_field(h, replica, false, a);
        if (s) return s;
        if (k < n_steps) {
            SN_CK(h, sn_launch_quench_step(R.px, R.py, R.pz, R.len, h->d_grad, (long long)N, step, h->stream));
            h->launches++;
        }
    }
    std::vector<double> tr(10 * (size_t)(n_steps + 1));
    SN_CK(h, cudaMemcpyAsync(tr.data(), h->d_trace, tr.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    s = recompute_one(h, replica, SN_ENERGY_FP32, 0);
    if (s) return s;
    SN_CK(h, cudaStreamSynchronize(h->stream));
    if (E_trace)
        for (int k = 0; k <= n_steps; k++) {
            const double *r = &tr[10 * (size_t)k];
            E_trace[k] = r[0] - 0.5 * (double)h->params.cage_strain * r[1] + r[2] + r[3];
        }
    return SN_OK;
}

sn_status sn_gpu_schedule(const sn_handle *h, int replica, sn_schedule_info *out)
{
    if (!h || !out) return fail(nullptr, SN_ERR_ARG, "null argument");
    if (replica < 0 || replica >= h->nrep) return fail(const_cast<sn_handle *>(h), SN_ERR_ARG, "replica out of range");
    fill_info(h->tiles[replica], h->rc, out);
    return SN_OK;
}

sn_status sn_gpu_launch_count(const sn_handle *h, uint64_t *launches)
{
    if (!h || !launches) return fail(nullptr, SN_ERR_ARG, "null argument");
    *launches = h->launches;
    return SN_OK;
}

void *sn_gpu_stream(const sn_handle *h) { return h ? (void *)h->stream : nullptr; }

sn_status sn_gpu_phase_times(sn_handle *h, int n_sweeps, double *avg_launch_ms, double *avg_sweep_ms,
                             int *launches_per_sweep)
{
    if (!h || n_sweeps < 1) return fail(h, SN_ERR_ARG, "need a handle and n_sweeps >= 1");
    int nl = 0;
    if (h->flow)
        for (int v = 0; v < 2; v++) nl += h->flow_items[v] ? 1 : 0;
    else
        for (int k = 0; k < 16; k++) nl += h->work_cnt[k] ? 1 : 0;
    std::vector<cudaEvent_t> ev(2 * (size_t)nl);
    for (auto &x : ev) SN_CK(h, cudaEventCreate(&x));
    cudaEvent_t s0, s1;
    SN_CK(h, cudaEventCreate(&s0));
    SN_CK(h, cudaEventCreate(&s1));
    double tot_launch = 0.0, tot_sweep = 0.0;
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < n_sweeps && e == cudaSuccess; i++) {
        e = cudaEventRecord(s0, h->stream);
        if (e == cudaSuccess) e = issue_sweep(h, nullptr, &ev);
        if (e == cudaSuccess) e = cudaEventRecord(s1, h->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(s1);
        for (int k = 0; k < nl && e == cudaSuccess; k++) {
            float ms = 0.0f;
            e = cudaEventElapsedTime(&ms, ev[2 * k], ev[2 * k + 1]);
            tot_launch += ms;
        }
        float sw = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&sw, s0, s1);
        tot_sweep += sw;
        h->launches += (uint64_t)nl + 1 + (h->cached ? 1 : 0);
        h->sweeps++;
    }
    for (auto &x : ev) cudaEventDestroy(x);
    cudaEventDestroy(s0);
    cudaEventDestroy(s1);
    if (e != cudaSuccess) return fail(h, SN_ERR_CUDA, "phase timing: %s", cudaGetErrorString(e));
    sn_status s = flow_status(h);
    if (s) return s;
    if (avg_launch_ms) *avg_launch_ms = tot_launch / ((double)n_sweeps * nl);
    if (avg_sweep_ms) *avg_sweep_ms = tot_sweep / n_sweeps;
    if (launches_per_sweep) *launches_per_sweep = nl;
    return SN_OK;
}

sn_status sn_gpu_flow_stats(sn_handle *h, uint64_t *stats)
{
    if (!h || !stats) return fail(h, SN_ERR_ARG, "null argument");
    uint32_t e[4] = {0, 0, 0, 0};
    if (h->flow && h->d_err) {
        SN_CK(h, cudaMemcpyAsync(e, h->d_err, sizeof(e), cudaMemcpyDeviceToHost, h->stream));
        SN_CK(h, cudaMemsetAsync(h->d_err + 1, 0, 2 * sizeof(uint32_t), h->stream));
        SN_CK(h, cudaStreamSynchronize(h->stream));
    }
    stats[0] = h->flow ? 1 : 0;
    stats[1] = (uint64_t)(h->flow ? h->flow_grid[0] : 0);
    stats[2] = e[1];
    stats[3] = e[2];
    return SN_OK;
}

sn_status sn_gpu_fp32_peak(double *tflops, double *sm_clock_mhz)
{
    if (!tflops) return fail(nullptr, SN_ERR_ARG, "null output");
    int dev = 0, nsm = 0, clk = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return fail(nullptr, SN_ERR_CUDA, "no CUDA device");
    cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, dev);
    const int threads = 1024, blocks = nsm * 2, iters = 1 << 16;
    float *d = nullptr;
    if (cudaMalloc(&d, (size_t)blocks * threads * sizeof(float)) != cudaSuccess)
        return fail(nullptr, SN_ERR_NOMEM, "cudaMalloc failed");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaError_t e = sn_launch_fma_peak(d, blocks, threads, iters / 16, 0);  // warm-up
    float best = 1e30f;
    for (int rep = 0; rep < 5 && e == cudaSuccess; rep++) {
        cudaEventRecord(e0, 0);
        e = sn_launch_fma_peak(d, blocks, threads, iters, 0);
        cudaEventRecord(e1, 0);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms > 0.0f && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (e != cudaSuccess) return fail(nullptr, SN_ERR_CUDA, "fma probe: %s", cudaGetErrorString(e));
    *tflops = 2.0 * 8.0 * (double)iters * blocks * threads / (best * 1e-3) / 1e12;
    if (sm_clock_mhz) *sm_clock_mhz = clk / 1000.0;
    return SN_OK;
}

sn_status sn_gpu_philox(const uint32_t *ctr, const uint32_t *key, uint32_t *out, int n)
{
    if (!ctr || !key || !out || n < 0) return fail(nullptr, SN_ERR_ARG, "null buffer or negative count");
    if (n == 0) return SN_OK;
    uint32_t *d = nullptr;
    if (cudaMalloc(&d, (size_t)n * 10 * sizeof(uint32_t)) != cudaSuccess)
        return fail(nullptr, SN_ERR_NOMEM, "cudaMalloc failed");
    cudaError_t e = cudaMemcpy(d, ctr, (size_t)n * 4 * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + 4 * (size_t)n, key, (size_t)n * 2 * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = sn_launch_philox_batch(d, d + 4 * (size_t)n, d + 6 * (size_t)n, n, 0);
    if (e == cudaSuccess) e = cudaMemcpy(out, d + 6 * (size_t)n, (size_t)n * 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return fail(nullptr, SN_ERR_CUDA, "philox batch: %s", cudaGetErrorString(e));
    return SN_OK;
}

sn_status sn_gpu_proposals(const sn_handle *h, int replica, const uint32_t *sites, int n, uint32_t sweep, float *out4)
{
    if (!h || !sites || !out4 || n < 0) return fail(nullptr, SN_ERR_ARG, "null argument");
    if (replica < 0 || replica >= h->nrep) return fail(const_cast<sn_handle *>(h), SN_ERR_ARG, "replica out of range");
    if (n == 0) return SN_OK;
    const SnReplicaDev &R = h->reps[replica];
    void *d = nullptr;
    if (cudaMalloc(&d, (size_t)n * 5 * sizeof(uint32_t)) != cudaSuccess)
        return fail(const_cast<sn_handle *>(h), SN_ERR_NOMEM, "cudaMalloc failed");
    uint32_t *ds = (uint32_t *)d;
    float *dout = (float *)(ds + n);
    cudaError_t e = cudaMemcpyAsync(ds, sites, (size_t)n * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = sn_launch_proposal_batch(ds, sweep, R.seed_lo, R.seed_hi, h->params.dim, h->params.constrain_to_x, dout, n,
                                     h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out4, dout, (size_t)n * 4 * sizeof(float), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(d);
    if (e != cudaSuccess) return fail(const_cast<sn_handle *>(h), SN_ERR_CUDA, "proposal batch: %s", cudaGetErrorString(e));
    return SN_OK;
}

}  // extern "C"

// ---- analysis stencils: host tables and entry points ----
namespace {

// d = sqrt(float expression) stored to float, as the reference writes it
// (src/starrynight-analysis.c:82,337,419,564).
float ref_distance(float s) { return (float)std::sqrt((double)s); }

SnAnalysisOffset make_offset(int dx, int dy, int dz)
{
    SnAnalysisOffset o;
    memset(&o, 0, sizeof(o));
    o.dx = dx;
    o.dy = dy;
    o.dz = dz;
    return o;
}

// dipole_potential (src/starrynight-analysis.c:65-94): the cube |d_i| <= C in
// dx, dy, dz order, without the origin, kept when d <= C; a = r.
std::vector<SnAnalysisOffset> potential_table(int C)
{
    std::vector<SnAnalysisOffset> t;
    for (int dx = -C; dx <= C; dx++)
        for (int dy = -C; dy <= C; dy++)
            for (int dz = -C; dz <= C; dz++) {
                if (dx == 0 && dy == 0 && dz == 0) continue;
                const float rx = (float)dx, ry = (float)dy, rz = (float)dz;
                const float d = ref_distance(rx * rx + ry * ry + rz * rz);
                if (d > (float)C) continue;
                SnAnalysisOffset o = make_offset(dx, dy, dz);
                o.a[0] = rx;
                o.a[1] = ry;
                o.a[2] = rz;
                o.d3 = d * d * d;
                t.push_back(o);
            }
    return t;
}

// dipole_electricfield (:393-450; half = 0) and dipole_electricfieldoffset
// (:310-380; half = 1, displacements dx + 1/2 for dx in [-C-1, C-1], origin
// not excluded): a = n = r/d, b = 3 n, kept when d <= C.
std::vector<SnAnalysisOffset> efield_table(int C, bool half)
{
    std::vector<SnAnalysisOffset> t;
    const int lo = half ? -C - 1 : -C, hi = half ? C - 1 : C;
    for (int dx = lo; dx <= hi; dx++)
        for (int dy = lo; dy <= hi; dy++)
            for (int dz = lo; dz <= hi; dz++) {
                if (!half && dx == 0 && dy == 0 && dz == 0) continue;
                const float rx = half ? (float)((double)(float)dx + 0.5) : (float)dx;
                const float ry = half ? (float)((double)(float)dy + 0.5) : (float)dy;
                const float rz = half ? (float)((double)(float)dz + 0.5) : (float)dz;
                const float d = ref_distance(rx * rx + ry * ry + rz * rz);
                if (d > (float)C) continue;
                SnAnalysisOffset o = make_offset(dx, dy, dz);
                o.a[0] = rx / d;
                o.a[1] = ry / d;
                o.a[2] = rz / d;
                for (int c = 0; c < 3; c++) o.b[c] = 3.0f * o.a[c];
                o.d3 = d * d * d;
                t.push_back(o);
            }
    return t;
}

// radial_order_parameter (:528-598): the ball |r|^2 <= C^2 including the
// origin, binned by |r|^2; a = n = r/d with d = 1 at the origin.  Sorted by
// bin, the reference's dx, dy, dz order kept within a bin.
std::vector<SnAnalysisOffset> radial_table(int C)
{
    std::vector<SnAnalysisOffset> t;
    for (int dx = -C; dx <= C; dx++)
        for (int dy = -C; dy <= C; dy++)
            for (int dz = -C; dz <= C; dz++) {
                const int ds = dx * dx + dy * dy + dz * dz;
                if (ds > C * C) continue;
                float d = ref_distance((float)dx * dx + dy * dy + dz * dz);
                if (d == 0) d = 1;
                SnAnalysisOffset o = make_offset(dx, dy, dz);
                o.bin = ds;
                o.a[0] = (float)dx / d;
                o.a[1] = (float)dy / d;
                o.a[2] = (float)dz / d;
                t.push_back(o);
            }
    std::stable_sort(t.begin(), t.end(),
                     [](const SnAnalysisOffset &a, const SnAnalysisOffset &b) { return a.bin < b.bin; });
    return t;
}

SnLatticeView view_of(const SnReplicaDev &R)
{
    SnLatticeView L;
    L.px = R.px;
    L.py = R.py;
    L.pz = R.pz;
    L.len = R.len;
    L.X = R.X;
    L.Y = R.Y;
    L.Z = R.Z;
    L.n = R.n_sites;
    return L;
}

sn_status upload_table(sn_handle *h, const std::vector<SnAnalysisOffset> &t)
{
    sn_status s = ensure(h, (void **)&h->d_aoff, &h->aoff_n, std::max<size_t>(t.size(), 1), sizeof(SnAnalysisOffset));
    if (s) return s;
    SN_CK(h, cudaMemcpyAsync(h->d_aoff, t.data(), t.size() * sizeof(SnAnalysisOffset), cudaMemcpyHostToDevice,
                             h->stream));
    return SN_OK;
}

const int kAnalysisMaxCutoff = 32;

}  // namespace

extern "C" {

sn_status sn_gpu_potential(sn_handle *h, int replica, int cutoff, double *pot)
{
    sn_status s = check_rep(h, replica);
    if (s) return s;
    if (!pot || cutoff < 1 || cutoff > kAnalysisMaxCutoff)
        return fail(h, SN_ERR_ARG, "potential: need an output buffer and 1 <= cutoff <= %d", kAnalysisMaxCutoff);
    const SnReplicaDev &R = h->reps[replica];
    const std::vector<SnAnalysisOffset> t = potential_table(cutoff);
    if ((s = upload_table(h, t))) return s;
    if ((s = ensure(h, (void **)&h->d_site, &h->site_n, (size_t)R.n_sites, sizeof(double)))) return s;
    SN_CK(h, sn_launch_potential(view_of(R), h->d_aoff, (int)t.size(), h->d_site, h->stream));
    SN_CK(h, cudaMemcpyAsync(pot, h->d_site, (size_t)R.n_sites * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    return SN_OK;
}

sn_status sn_gpu_efield(sn_handle *h, int replica, int cutoff, int half_offset, double *magnitude)
{
    sn_status s = check_rep(h, replica);
    if (s) return s;
    if (!magnitude || cutoff < 1 || cutoff > kAnalysisMaxCutoff)
        return fail(h, SN_ERR_ARG, "efield: need an output buffer and 1 <= cutoff <= %d", kAnalysisMaxCutoff);
    const SnReplicaDev &R = h->reps[replica];
    const std::vector<SnAnalysisOffset> t = efield_table(cutoff, half_offset != 0);
    if ((s = upload_table(h, t))) return s;
    if ((s = ensure(h, (void **)&h->d_site, &h->site_n, (size_t)R.n_sites, sizeof(double)))) return s;
    SN_CK(h, sn_launch_efield(view_of(R), h->d_aoff, (int)t.size(), half_offset ? 0 : 1, h->d_site, h->stream));
    SN_CK(h, cudaMemcpyAsync(magnitude, h->d_site, (size_t)R.n_sites * sizeof(double), cudaMemcpyDeviceToHost,
                             h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    return SN_OK;
}

sn_status sn_gpu_radial_order(sn_handle *h, int replica, int cutoff, double *fe_sum, double *afe_sum,
                              int64_t *count)
{
    sn_status s = check_rep(h, replica);
    if (s) return s;
    if (cutoff < 1 || cutoff > kAnalysisMaxCutoff)
        return fail(h, SN_ERR_ARG, "radial order: 1 <= cutoff <= %d", kAnalysisMaxCutoff);
    const SnReplicaDev &R = h->reps[replica];
    const int n_bins = cutoff * cutoff + 1;
    const std::vector<SnAnalysisOffset> t = radial_table(cutoff);
    if (count) {
        for (int b = 0; b < n_bins; b++) count[b] = 0;
        for (const SnAnalysisOffset &o : t) count[o.bin] += R.n_sites;
    }
    if ((s = upload_table(h, t))) return s;
    if ((s = ensure(h, (void **)&h->d_abins, &h->abins_n, 2 * (size_t)n_bins, sizeof(double)))) return s;
    SN_CK(h, cudaMemsetAsync(h->d_abins, 0, 2 * (size_t)n_bins * sizeof(double), h->stream));
    SN_CK(h, sn_launch_radial(view_of(R), h->d_aoff, (int)t.size(), n_bins, h->d_abins, h->d_abins + n_bins,
                              h->stream));
    std::vector<double> out(2 * (size_t)n_bins);
    SN_CK(h, cudaMemcpyAsync(out.data(), h->d_abins, out.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    for (int b = 0; b < n_bins; b++) {
        if (fe_sum) fe_sum[b] = out[b];
        if (afe_sum) afe_sum[b] = out[n_bins + b];
    }
    return SN_OK;
}

sn_status sn_gpu_order_parameters(sn_handle *h, int replica, double *polarisation_x, double *landau,
                                  double *orientation_sum)
{
    sn_status s = check_rep(h, replica);
    if (s) return s;
    const SnReplicaDev &R = h->reps[replica];
    if ((s = ensure(h, (void **)&h->d_abins, &h->abins_n, 3, sizeof(double)))) return s;
    SN_CK(h, cudaMemsetAsync(h->d_abins, 0, 3 * sizeof(double), h->stream));
    SN_CK(h, sn_launch_orient_sum(view_of(R), h->d_abins, h->stream));
    double o[3];
    SN_CK(h, cudaMemcpyAsync(o, h->d_abins, sizeof(o), cudaMemcpyDeviceToHost, h->stream));
    SN_CK(h, cudaStreamSynchronize(h->stream));
    if (polarisation_x) *polarisation_x = o[0] / (double)R.n_sites;
    if (landau) *landau = o[0] * o[0] + o[1] * o[1] + o[2] * o[2];
    if (orientation_sum)
        for (int c = 0; c < 3; c++) orientation_sum[c] = o[c];
    return SN_OK;
}

}  // extern "C"
