// sn_noalloc.cu -- total energy of a caller-owned device lattice without any
// device allocation.
//
// Who needs it: callers that may not call cudaMalloc when they want an
// energy -- a plugin whose host framework owns the device memory pool and
// forbids allocations behind its back, a process that has already reserved
// nearly all device memory for its lattices, or a long run that must not
// risk an out-of-memory failure (or the allocator's implicit device
// synchronisation) between sweeps.  The regular path
// (sn_gpu_init + sn_gpu_energy) allocates the replica table and its
// bookkeeping in HBM; this entry point instead keeps every piece of scratch
// (replica descriptor, tile geometry, the list of lattice blocks and the
// FP64 reduction slots) in one file-scope __device__ array of fixed size,
// present on every GPU that loads the library until the process exits.
//
// Limits: the lattice must split into at most SN_NOALLOC_MAX_BLOCKS = 65536
// tiles (512^3 at cutoff 3 needs 32768); the array is then about 1 MiB.
// Larger lattices get SN_ERR_ARG with the numbers in the message.
//
// All calls share the one array and it keeps the last call's contents; the
// reduction slots are cleared on every call.  Calls whose GPU work overlaps
// (several host threads, or several streams without ordering between them)
// race on the array and give wrong energies: order them on one stream.
//
// The first call on each device looks up the array's device address with
// cudaGetSymbolAddress (with that device current) and caches it; make that
// first call before any stream capture begins.  The cache is per process:
// after cudaDeviceReset the module is loaded again and the cached address is
// stale, so a process that resets a device must not call this entry point on
// that device afterwards.
#include <atomic>
#include <cstdio>
#include <cstring>

#include "../../include/sn_gpu.h"
#include "sn_launch.h"

#define SN_NOALLOC_MAX_BLOCKS 65536
#define SN_NOALLOC_MAX_DEVICES 64

namespace {

struct NoallocHeader {
    SnReplicaDev rep;
    SnTile tile;
    double red[16];
};

constexpr size_t kHeaderBytes = (sizeof(NoallocHeader) + 255) & ~(size_t)255;
constexpr size_t kScratchBytes = kHeaderBytes + (size_t)SN_NOALLOC_MAX_BLOCKS * sizeof(SnWork);

static __device__ __align__(256) unsigned char sn_noalloc_scratch[kScratchBytes];

// Device address of sn_noalloc_scratch per device (host-side cache).  In host
// code the symbol's own name is only a host stand-in, never a device address.
// Host threads may race on the first call of a device: both look the address
// up (the same value) and store it atomically.
std::atomic<void *> g_scratch[SN_NOALLOC_MAX_DEVICES];

thread_local char g_err[256];

sn_status nfail(sn_status s, const char *msg)
{
    sn_internal_set_error(msg);
    return s;
}

}  // namespace

extern "C" {

sn_status sn_gpu_energy_noalloc(const float *d_px, const float *d_py, const float *d_pz, const float *d_len, int X,
                                int Y, int Z, const sn_params *params, const float *efield, double *E_total,
                                void *stream)
{
    if (!d_px || !d_py || !d_pz || !d_len || !params || !E_total) return nfail(SN_ERR_ARG, "null argument");
    if (X < 1 || Y < 1 || Z < 1) return nfail(SN_ERR_ARG, "bad lattice size");
    if ((long long)X * Y * Z > 0x7fffffffLL) return nfail(SN_ERR_UNSUPPORTED, "more than 2^31-1 sites");
    const sn_params &P = *params;
    if (P.cutoff < 1 || P.cutoff > SN_MAX_CUTOFF) return nfail(SN_ERR_UNSUPPORTED, "cutoff outside 1..SN_MAX_CUTOFF");
    if (P.n_species < 1 || P.n_species > SN_MAX_SPECIES) return nfail(SN_ERR_CONFIG, "n_species must be 1..10");
    float L = 0.0f;
    bool mixed = false;
    for (int i = 0; i < P.n_species; i++) {
        const float d = P.dipoles[i];
        if (!(d >= 0.0f)) return nfail(SN_ERR_CONFIG, "Dipoles must be >= 0");
        if (d > 0.0f) {
            if (L == 0.0f) L = d;
            else if (d != L) mixed = true;
        }
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nfail(SN_ERR_CUDA, "no CUDA device");
    if (dev < 0 || dev >= SN_NOALLOC_MAX_DEVICES) return nfail(SN_ERR_UNSUPPORTED, "device index too large");
    void *cached = g_scratch[dev].load(std::memory_order_acquire);
    if (!cached) {
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, sn_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            snprintf(g_err, sizeof(g_err), "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            return nfail(SN_ERR_CUDA, g_err);
        }
        g_scratch[dev].store(ptr, std::memory_order_release);
        cached = ptr;
    }
    unsigned char *base = (unsigned char *)cached;

    SnTile tile;
    char why[200];
    if (!sn_internal_plan(X, Y, Z, P.cutoff, mixed, &tile, why, sizeof(why))) return nfail(SN_ERR_SCHEDULE, why);
    const long long nblocks = (long long)tile.nb[0] * tile.nb[1] * tile.nb[2];
    if (nblocks > SN_NOALLOC_MAX_BLOCKS) {
        snprintf(g_err, sizeof(g_err),
                 "lattice %dx%dx%d needs %lld tiles; the no-allocation entry point holds at most %d", X, Y, Z, nblocks,
                 SN_NOALLOC_MAX_BLOCKS);
        return nfail(SN_ERR_ARG, g_err);
    }
    NoallocHeader hdr;
    memset(&hdr, 0, sizeof(hdr));
    hdr.rep.px = const_cast<float *>(d_px);
    hdr.rep.py = const_cast<float *>(d_py);
    hdr.rep.pz = const_cast<float *>(d_pz);
    hdr.rep.len = const_cast<float *>(d_len);
    hdr.rep.X = X;
    hdr.rep.Y = Y;
    hdr.rep.Z = Z;
    hdr.rep.geom = 0;
    hdr.rep.n_sites = (long long)X * Y * Z;
    hdr.rep.T = 300.0f;  // temperature plays no part in the energy
    hdr.rep.beta = 1.0f;
    for (int k = 0; k < 3; k++) hdr.rep.E[k] = efield ? efield[k] : P.efield[k];
    hdr.rep.length = L;
    hdr.tile = tile;
    cudaStream_t st = (cudaStream_t)stream;
    SnWork *d_work = (SnWork *)(base + kHeaderBytes);
    NoallocHeader *d_hdr = (NoallocHeader *)base;
    // the block list goes up in chunks from a stack buffer
    SnWork chunk[512];
    int n = 0;
    long long done = 0;
    cudaError_t e = cudaMemcpyAsync(d_hdr, &hdr, sizeof(hdr), cudaMemcpyHostToDevice, st);
    for (int bx = 0; bx < tile.nb[0] && e == cudaSuccess; bx++)
        for (int by = 0; by < tile.nb[1] && e == cudaSuccess; by++)
            for (int bz = 0; bz < tile.nb[2] && e == cudaSuccess; bz++) {
                chunk[n++] = SnWork{0, bx * tile.B[0], by * tile.B[1], bz * tile.B[2]};
                if (n == 512) {
                    e = cudaMemcpyAsync(d_work + done, chunk, sizeof(chunk), cudaMemcpyHostToDevice, st);
                    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // chunk is reused
                    done += n;
                    n = 0;
                }
            }
    if (e == cudaSuccess && n) {
        e = cudaMemcpyAsync(d_work + done, chunk, n * sizeof(SnWork), cudaMemcpyHostToDevice, st);
        done += n;
    }
    SnFieldArgsHost a;
    memset(&a, 0, sizeof(a));
    a.work = d_work;
    a.reps = &d_hdr->rep;
    a.geoms = &d_hdr->tile;
    a.cage = P.cage_strain;
    a.K = P.K;
    a.red = d_hdr->red;
    a.red_stride = 0;
    if (e == cudaSuccess)
        e = sn_internal_field_launch(P.cutoff, false, Z == 1, mixed, a, (int)nblocks, tile.threads, tile.field_smem, st);
    double red[16];
    if (e == cudaSuccess) e = cudaMemcpyAsync(red, d_hdr->red, sizeof(red), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        snprintf(g_err, sizeof(g_err), "energy pass: %s", cudaGetErrorString(e));
        return nfail(SN_ERR_CUDA, g_err);
    }
    *E_total = red[0] - 0.5 * (double)P.cage_strain * red[1] + red[2] + red[3];
    return SN_OK;
}

}  // extern "C"
