// sn_internal.h -- structures shared by the host side and the kernels.
//
// Device data layout (one replica = one lattice):
//   px, py, pz, len : SoA float arrays of N = X*Y*Z sites, index (x*Y+y)*Z+z
//                     (z fastest, the reference's lattice[x][y][z] order).
//   Vacancies (len == 0) hold the zero vector, so in uniform-length mode the
//   sweep kernel reads only px/py/pz and a zero vector marks a vacancy.
#pragma once

#include <cstdint>

#define SN_MAX_THREADS 512       // largest sweep / field block
// Stencil pairs per thread (sets the number of splits) and the threads of a
// block that shares its SM with a second one (their registers must fit the
// register file twice).  Build-time tuning knobs.
#ifndef SN_PAIRS_PER_SPLIT
#define SN_PAIRS_PER_SPLIT 15
#endif
#ifndef SN_TWO_PER_SM_THREADS
#define SN_TWO_PER_SM_THREADS 256
#endif
#define SN_SWEEP_MIN_BLOCKS (SN_TWO_PER_SM_THREADS > 256 ? 2 : 1)
// Independent local-field accumulator sets that consecutive stencil pairs rotate through.
#ifndef SN_ACC_SETS
#define SN_ACC_SETS 2
#endif
#define SN_SWEEP_MAX_THREADS (SN_TWO_PER_SM_THREADS > 256 ? SN_TWO_PER_SM_THREADS : SN_MAX_THREADS)
// x slabs of a host upload (each converted and fed to the field-cache pass as
// it lands); at 256^3 an upload took 1.86, 1.74, 1.69 and 1.65 ms with 4, 8,
// 16 and 32 slabs.
#ifndef SN_UPLOAD_SLABS
#define SN_UPLOAD_SLABS 32
#endif
// streams the upload's energy-pass chunks alternate between (1 or 2)
#ifndef SN_UPLOAD_FIELD_STREAMS
#define SN_UPLOAD_FIELD_STREAMS 2
#endif
#define SN_MAX_S 8               // site-colour stride bound (cutoff + 1 <= 7)
#ifndef SN_CACHED_THREADS
#define SN_CACHED_THREADS 256  // block size of the cached-field sweep kernel
#endif
#define SN_GFIELD_THREADS 256  // block size of the field-cache pass
#define SN_BULK_WAIT_LIMIT (1u << 24)  // polls of the tile-copy barrier before an error is recorded
#define SN_HIST_CAP 4096         // per-replica per-sweep observable log

// Geometry of one replica's tiles: block dims, tile dims (block + halo),
// and the permutation that stores the x and y axes class-major
// (coordinates u with the same u mod s contiguous).  Slot of tile
// coordinate (ux,uy,uz) = pi_x(ux)*Sx + pi_y(uy)*Sy + uz, with
// pi_a(u) = start[a][u mod s] + u / s; z is stored plainly.
struct SnTile {
    int B[3];        // block dims
    int T[3];        // tile dims = B + 2*halo (z: 1 in 2D)
    int H[3];        // halo per axis
    int nb[3];       // blocks per axis
    int m[3];        // block colours per axis
    int Sy, Sx;      // padded slot strides (z stride is 1)
    int slots;       // Sx * T[0]
    int nq[3];       // targets per axis of the fullest site colour: ceil(B/s)
    int tp;          // targets of one site colour, padded to a warp multiple
    int tg;          // targets of one colour group (1 or 2 colours)
    int ng;          // colour groups per block
    int pc;          // colour groups whose proposals are staged at once
    int threads;     // sweep / field kernel block size (splits * tg)
    int merge;       // 1: colours c and c + (s/2,s/2,s/2) are updated together
    int start[3][SN_MAX_S];
    int smem_bytes;  // dynamic shared memory for the sweep kernel
    int field_smem;  // dynamic shared memory for the field kernel
    // Cached-field sweep (cmode = 1; sn_sweep_cached.cuh).  Its tile is the
    // block + halo with the z halo rounded up to 4 sites (16-byte rows), one
    // int32 array per field component, plain slots (ux*cT[1] + uy)*cT[2] + uz.
    int cmode;
    int cT[3];       // tile dims
    int cH[3];       // halo per axis (z: cutoff rounded up to a multiple of 4)
    int cslots;      // cT[0]*cT[1]*cT[2]
    int cpc;         // colour groups whose proposals are staged at once
    int csmem;       // dynamic shared memory of the cached sweep kernel
};

struct SnReplicaDev {
    float *px, *py, *pz, *len;
    int X, Y, Z;
    int geom;          // index into the SnTile table
    long long n_sites;
    float beta;        // 300 / T
    float T;
    float E[3];        // applied field
    float length;      // uniform dipole length (uniform mode)
    uint32_t seed_lo, seed_hi;
    // Set for one sweep by sn_gpu_sweep_download: a buffer the GPU can write
    // (mapped pinned host memory or device memory) that receives every
    // block's final sites (x, y, z per site, site order) as the block ends.
    float *out_xyz;
    // Local-field cache of the cached-field sweep (null: none): 3 int32
    // arrays of N (x, y, z components), g_i = len_i sum_j len_j T_ij p_j -
    // CageStrain sum_nn p_j in fixed point, value = int * ginv.
    int *gcache;
    float gscale;      // 2^k: float -> fixed point
    float ginv;        // 2^-k
    // Proposals of the coming sweep for the cached-field sweep (null: none),
    // one per site: (p'x, p'y, p'z, threshold -ln(u)/beta), threshold < 0 at
    // vacancies; written by the proposal kernel before each sweep.
    float4 *prop;
};

// Per-replica sweep accumulators (zeroed at the end of every sweep).
struct SnAccum {
    double dE;
    double dP[3];
    unsigned long long acc;
    unsigned long long att;
};

// Per-replica running state.
struct SnState {
    double E;           // running FP64 total energy
    double P[3];        // running FP64 sum_i len_i p_i
    unsigned long long acc_total, att_total;
    int hist_head;      // entries written since the last read (ring)
    int pad;
};

struct SnWork {
    int rep;
    int x0, y0, z0;     // block origin
};

struct SnPhaseArgs {
    const SnWork *work;
    int n_work;
    const SnReplicaDev *reps;
    const SnTile *geoms;
    SnAccum *acc;
    const uint32_t *sweep;   // device sweep counter
    float cage;
    float K;
    int constrain;
    int dim;
    uint32_t *err;   // device error flags (SnFlowArgs::err): bit 1 = a tile copy wait ran out
    int tile_copy;   // cached-field sweep tile load: 0 = 16-byte cp.async, 1 = TMA bulk row copies
};

#define SN_MAX_DEPS 28            // 1 count + up to 26 adjacent blocks (+1 spare)
// Default polls of a dependency flag before a block gives up with
// SN_ERR_TIMEOUT (about 1-4 s); a handle may lower it (sn_gpu_set_wait_limit).
#define SN_WAIT_LIMIT_DEFAULT (1u << 22)

// Dataflow sweep: the work list holds every block of a kernel variant in
// block-colour order; deps[item*SN_MAX_DEPS] = count, then the items of the
// adjacent blocks with an earlier colour; done[item] = last sweep (epoch)
// that finished the block; queue = next item to take (reset every sweep).
// The done array has one spare flag past the last item that no block ever
// publishes (a test hook points a dependency at it to exercise the timeout).
struct SnFlowArgs {
    SnPhaseArgs base;
    const int *deps;
    uint32_t *done;
    uint32_t *queue;
    // [0] a wait timed out, [1] items that waited, [2] polls, [3] poll limit
    // per dependency (set by the host; read by every waiting thread)
    uint32_t *err;
};

// Neighbour offset table for the per-site kernels (energy, adjoint, quench).
struct SnNeighbour {
    int dx, dy, dz, unit;
    double T[6];        // xx yy zz xy xz yz of (I - 3 n n^T) / d^3
    float Tf[6];
    float pad[2];
};
